"""Batches: many graphs counted by one CUDA-graph launch (include/trust_tc.h, trust_tc_batch_*).

The reference counts one graph per run; a batch of thousands of small graphs through it is a loop
of runs.  Here the graphs are preprocessed together into one oriented CSR that keeps every graph a
contiguous row range (trust_tc_build_batch_device), and `Batch.run` replays one captured CUDA graph
that returns every graph's count.

`batch_specs` draws the synthetic batch workload: sizes log-uniform in [nmin, nmax] vertices,
alternately Erdos-Renyi (average degree 4..64) and Barabasi-Albert (2..16 edges per vertex), from a
counter-based stream (splitmix64), so the list is the same on every host.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check, load

_M64 = (1 << 64) - 1


def _mix64(x: int) -> int:  # splitmix64 finaliser (Steele, Lea, Flood 2014)
    x &= _M64
    x ^= x >> 30
    x = (x * 0xBF58476D1CE4E5B9) & _M64
    x ^= x >> 27
    x = (x * 0x94D049BB133111EB) & _M64
    x ^= x >> 31
    return x


def _draw(seed: int, i: int, j: int) -> int:
    return _mix64(_mix64(seed ^ 0x243F6A8885A308D3) + (i * 64 + j) * 0x9E3779B97F4A7C15)


@dataclass(frozen=True)
class GraphSpec:
    kind: str   # "er" or "ba"
    n: int      # vertices
    param: int  # er: average degree; ba: edges per vertex
    seed: int

    @property
    def npairs(self) -> int:
        return self.n * self.param // 2 if self.kind == "er" else self.n * self.param


def batch_specs(num_graphs: int = 4096, nmin: int = 50, nmax: int = 50_000, seed: int = 5) -> list[GraphSpec]:
    specs = []
    for i in range(num_graphs):
        u = (_draw(seed, i, 0) >> 11) / float(1 << 53)
        n = max(nmin, min(nmax, int(nmin * math.exp(u * math.log(nmax / nmin)))))
        if i % 2 == 0:
            specs.append(GraphSpec("er", n, 4 + _draw(seed, i, 1) % 61, _draw(seed, i, 2) & 0x7FFFFFFF))
        else:
            specs.append(GraphSpec("ba", n, 2 + _draw(seed, i, 1) % 15, _draw(seed, i, 2) & 0x7FFFFFFF))
    return specs


def gen_batch_pairs(specs: list[GraphSpec]):
    """All graphs' pairs on the GPU in one (P, 2) int32 tensor, graph g's ids offset by the sum of
    the earlier graphs' vertex counts; returns (pairs, graph_vbeg as an int64 numpy array)."""
    import torch
    from . import gen_ba, gen_er
    vbeg = np.zeros(len(specs) + 1, dtype=np.int64)
    vbeg[1:] = np.cumsum([s.n for s in specs])
    offs = np.zeros(len(specs) + 1, dtype=np.int64)
    offs[1:] = np.cumsum([s.npairs for s in specs])
    pairs = torch.empty((int(offs[-1]), 2), dtype=torch.int32, device="cuda")
    for g, s in enumerate(specs):
        p = gen_er(s.n, s.npairs, seed=s.seed) if s.kind == "er" else gen_ba(s.n, s.param, seed=s.seed)
        pairs[int(offs[g]):int(offs[g + 1])] = p + int(vbeg[g])
    return pairs, vbeg


def build_batch(pairs, graph_vbeg: np.ndarray):
    """GPU preprocessing of a batch: (beg int64, adj int32, graph_vbeg of the result)."""
    import torch
    lib = load()
    vin = np.ascontiguousarray(graph_vbeg, dtype=np.int64)
    vout = np.zeros_like(vin)
    pb, pa = C.c_void_p(), C.c_void_p()
    n, m = C.c_int64(), C.c_int64()
    pairs = pairs.contiguous()
    i64p = C.POINTER(C.c_int64)
    check(lib.trust_tc_build_batch_device(None, C.c_void_p(pairs.data_ptr()), pairs.shape[0],
                                          vin.ctypes.data_as(i64p), vin.size - 1, C.byref(pb), C.byref(pa),
                                          C.byref(n), C.byref(m), vout.ctypes.data_as(i64p)),
          "trust_tc_build_batch_device")
    try:
        beg = torch.empty(n.value + 1, dtype=torch.int64, device="cuda")
        adj = torch.empty(max(m.value, 1), dtype=torch.int32, device="cuda")
        check(lib.trust_tc_copy(C.c_void_p(beg.data_ptr()), pb, 8 * (n.value + 1)), "trust_tc_copy")
        check(lib.trust_tc_copy(C.c_void_p(adj.data_ptr()), pa, 4 * m.value), "trust_tc_copy")
    finally:
        lib.trust_tc_free_device(pb)
        lib.trust_tc_free_device(pa)
    return beg, adj[: m.value], vout


def graph_csr(beg, adj, graph_vbeg: np.ndarray, g: int):
    """Graph g of a batch as its own CSR with local ids (device tensors)."""
    lo, hi = int(graph_vbeg[g]), int(graph_vbeg[g + 1])
    b = beg[lo:hi + 1]
    a0 = int(b[0].item()) if hi > lo else 0
    return (b - a0).contiguous(), (adj[a0:int(b[-1].item())] - lo).contiguous() if hi > lo else adj[:0]


class Batch:
    """A captured batch job over a batch CSR (device tensors kept alive by this object)."""

    def __init__(self, beg, adj, graph_vbeg: np.ndarray, ctx=None):
        from . import Context
        self._keep = (beg, adj)
        self.ctx = ctx if ctx is not None else Context()
        self.vbeg = np.ascontiguousarray(graph_vbeg, dtype=np.int64)
        self.num_graphs = self.vbeg.size - 1
        h = C.c_void_p()
        check(load().trust_tc_batch_create(self.ctx.handle, C.c_void_p(beg.data_ptr()), C.c_void_p(adj.data_ptr()),
                                           beg.numel() - 1, adj.numel(), self.vbeg.ctypes.data_as(C.POINTER(C.c_int64)),
                                           self.num_graphs, C.byref(h)), "trust_tc_batch_create")
        self.handle = h

    def close(self) -> None:
        if getattr(self, "handle", None):
            load().trust_tc_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> dict:
        g = (C.c_int64 * _lib.BATCH_CLASSES)()
        v = (C.c_int64 * _lib.BATCH_CLASSES)()
        d = (C.c_int32 * _lib.BATCH_CLASSES)()
        check(load().trust_tc_batch_info(self.handle, g, v, d), "trust_tc_batch_info")
        return {"graphs": list(g), "vertices": list(v), "max_out_degree": list(d)}

    def get_class(self, s: int) -> dict:
        c = _lib.BatchClass()
        check(load().trust_tc_batch_get_class(self.handle, s, C.byref(c)), "trust_tc_batch_get_class")
        return {"threads_per_block": c.threads_per_block, "warp_max_degree": c.warp_max_degree, "chunk": c.chunk}

    def set_class(self, s: int, threads_per_block: int, warp_max_degree: int, chunk: int) -> None:
        c = _lib.BatchClass(threads_per_block, warp_max_degree, chunk)
        check(load().trust_tc_batch_set_class(self.handle, s, C.byref(c)), "trust_tc_batch_set_class")

    def autotune(self, repeats: int = 2) -> float:
        ms = C.c_double()
        check(load().trust_tc_batch_autotune(self.handle, repeats, C.byref(ms)), "trust_tc_batch_autotune")
        return ms.value

    def run(self, stream=None):
        """(per-graph counts as a uint64 numpy array, CountResult of the whole batch)."""
        from . import _result
        counts = np.zeros(self.num_graphs, dtype=np.uint64)
        r = _lib.Result()
        check(load().trust_tc_batch_run(self.handle, stream, counts.ctypes.data_as(C.POINTER(C.c_uint64)),
                                        C.byref(r)), "trust_tc_batch_run")
        return counts, _result(r)
