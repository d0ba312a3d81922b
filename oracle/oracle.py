"""ctypes binding of the C oracle (oracle/tc_oracle.c).  TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs,
always as the checker.  The product path (trust_gb300/) never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
CUDA_LIB_PATH = os.path.join(HERE, "_build", "liboracle_cuda.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_CUBIN = os.path.join(REF_DIR, "tc_ref_w.cubin")

TRUST_EXACT = 0
TRUST_BUCKET_OVERFLOW, TRUST_REPROBE, TRUST_EARLY_EXIT, TRUST_INT32 = 1, 2, 4, 8

_lib = None
_cuda_lib = None
_P = C.c_void_p


def _declare(lib):
    lib.orc_count_forward.restype = C.c_int
    lib.orc_count_forward.argtypes = [_P, _P, C.c_int64, C.c_int, C.c_int, C.POINTER(C.c_uint64)]
    lib.orc_count_forward_sorted_range.restype = C.c_int
    lib.orc_count_forward_sorted_range.argtypes = [_P, _P, C.c_int64, C.c_int64, C.c_int64, C.c_int, C.c_int,
                                                   C.POINTER(C.c_uint64)]
    lib.orc_count_forward_stride.restype = C.c_int
    lib.orc_count_forward_stride.argtypes = [_P, _P, C.c_int64, C.c_int64, C.c_int64, C.c_int, C.c_int,
                                             C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    lib.orc_wedges.restype = C.c_uint64
    lib.orc_wedges.argtypes = [_P, _P, C.c_int64, C.c_int]
    lib.orc_count_tiles.restype = C.c_int
    lib.orc_count_tiles.argtypes = [_P, _P, _P, _P, _P, _P, C.c_int64, C.c_int64, C.POINTER(C.c_uint64)]
    lib.orc_trust_split.restype = C.c_int64
    lib.orc_trust_split.argtypes = [_P, C.c_int64, C.c_int]
    lib.orc_trust_check.restype = C.c_int
    lib.orc_trust_check.argtypes = [_P, _P, C.c_int64, C.POINTER(C.c_int64)]
    lib.orc_build_csr.restype = C.c_int
    lib.orc_build_csr.argtypes = [_P, C.c_int64, C.c_int64, C.POINTER(C.POINTER(C.c_int64)),
                                  C.POINTER(C.POINTER(C.c_int32)), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.orc_ref_undirect.restype = C.c_int
    lib.orc_ref_undirect.argtypes = [_P, C.c_int64, C.POINTER(C.c_int64), _P, C.POINTER(C.c_int64)]
    lib.orc_ref_outdegree_csr.restype = C.c_int
    lib.orc_ref_outdegree_csr.argtypes = [C.c_int64, _P, C.c_int64, _P, _P, C.POINTER(C.c_int64),
                                          C.POINTER(C.c_int64)]
    lib.orc_partition_sizes.restype = C.c_int
    lib.orc_partition_sizes.argtypes = [_P, _P, C.c_int64, C.c_int, _P, _P]
    lib.orc_partition.restype = C.c_int
    lib.orc_partition.argtypes = [_P, _P, C.c_int64, C.c_int, _P, _P]
    lib.orc_gen_rmat.restype = None
    lib.orc_gen_rmat.argtypes = [C.c_int, C.c_int64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, _P]
    lib.orc_gen_weighted.restype = None
    lib.orc_gen_weighted.argtypes = [_P, C.c_int64, C.c_int64, C.c_uint64, _P]
    lib.orc_gen_er.restype = None
    lib.orc_gen_er.argtypes = [C.c_int64, C.c_int64, C.c_uint64, _P]
    lib.orc_gen_ba.restype = None
    lib.orc_gen_ba.argtypes = [C.c_int64, C.c_int, C.c_uint64, _P]
    lib.orc_chung_lu_cdf.restype = C.c_double
    lib.orc_chung_lu_cdf.argtypes = [C.c_int64, C.c_double, C.c_double, C.c_int64, _P]
    lib.free.restype = None
    lib.free.argtypes = [_P]


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} missing: run trust_gb300/build.py")
        lib = C.CDLL(LIB_PATH)
        _declare(lib)
        _lib = lib
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def count_forward(beg, adj, min_deg: int = 2, threads: int = 1) -> int:
    b = np.ascontiguousarray(beg, dtype=np.int64)
    a = np.ascontiguousarray(adj, dtype=np.int32)
    out = C.c_uint64()
    rc = load().orc_count_forward(_p(b), _p(a), b.size - 1, min_deg, threads, C.byref(out))
    assert rc == 0
    return int(out.value)


def count_forward_sorted_range(beg, adj, lo: int, hi: int, min_deg: int = 2, threads: int = 1) -> int:
    """Counted quantity over source vertices [lo, hi) of a CSR whose rows are sorted ascending."""
    out = C.c_uint64()
    rc = load().orc_count_forward_sorted_range(_p(beg), _p(adj), beg.size - 1, lo, hi, min_deg, threads,
                                               C.byref(out))
    assert rc == 0
    return int(out.value)


def count_forward_stride(beg, adj, start: int, stride: int, min_deg: int = 2, threads: int = 1):
    """(count, arcs) over source vertices start, start + stride, ... of a CSR with sorted rows."""
    out, arcs = C.c_uint64(), C.c_uint64()
    rc = load().orc_count_forward_stride(_p(beg), _p(adj), beg.size - 1, start, stride, min_deg, threads,
                                         C.byref(out), C.byref(arcs))
    assert rc == 0
    return int(out.value), int(arcs.value)


def wedges(beg, adj, min_deg: int = 2) -> int:
    b = np.ascontiguousarray(beg, dtype=np.int64)
    a = np.ascontiguousarray(adj, dtype=np.int32)
    return int(load().orc_wedges(_p(b), _p(a), b.size - 1, min_deg))


def count_tiles(A, B, Cc) -> int:
    arrs = [np.ascontiguousarray(x, dtype=t) for pair in (A, B, Cc) for x, t in zip(pair, (np.int64, np.int32))]
    out = C.c_uint64()
    rc = load().orc_count_tiles(*[_p(x) for x in arrs], arrs[0].size - 1, arrs[4].size - 1, C.byref(out))
    assert rc == 0
    return int(out.value)


def trust_split(beg, val: int = 100) -> int:
    b = np.ascontiguousarray(beg, dtype=np.int64)
    return int(load().orc_trust_split(_p(b), b.size - 1, val))


def trust_check(beg, adj):
    """(flags, warpfirstvertex) for the reference kernel on this CSR; flags == 0 means exact."""
    b = np.ascontiguousarray(beg, dtype=np.int64)
    a = np.ascontiguousarray(adj, dtype=np.int32)
    wf = C.c_int64()
    flags = load().orc_trust_check(_p(b), _p(a), b.size - 1, C.byref(wf))
    return int(flags), int(wf.value)


def build_csr(pairs, id_bound: int):
    lib = load()
    p = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1)
    pb, pa = C.POINTER(C.c_int64)(), C.POINTER(C.c_int32)()
    n, m = C.c_int64(), C.c_int64()
    rc = lib.orc_build_csr(_p(p), p.size // 2, id_bound, C.byref(pb), C.byref(pa), C.byref(n), C.byref(m))
    assert rc == 0
    beg = np.ctypeslib.as_array(pb, shape=(n.value + 1,)).copy()
    adj = np.ctypeslib.as_array(pa, shape=(max(m.value, 1),))[: m.value].copy()
    lib.free(C.cast(pb, C.c_void_p))
    lib.free(C.cast(pa, C.c_void_p))
    return beg, adj


def ref_undirect(pairs):
    """Restated Preprocess/fromDirectToUndirect.cpp: (k, 1-based sorted unique (u<=v) edge array)."""
    p = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1)
    out = np.zeros(max(p.size, 2), dtype=np.int32)
    k, m = C.c_int64(), C.c_int64()
    load().orc_ref_undirect(_p(p), p.size // 2, C.byref(k), _p(out), C.byref(m))
    return int(k.value), out[: 2 * m.value].reshape(-1, 2).copy()


def ref_outdegree_csr(k: int, edges):
    """Restated Preprocess/preprocess_outdegree.cpp on 1-based edges: (beg, adj, s2, s3)."""
    e = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1)
    m = e.size // 2
    beg = np.zeros(k + 1, dtype=np.int64)
    adj = np.zeros(max(2 * m, 1), dtype=np.int32)
    s2, s3 = C.c_int64(), C.c_int64()
    load().orc_ref_outdegree_csr(k, _p(e), m, _p(beg), _p(adj), C.byref(s2), C.byref(s3))
    return beg, adj[: beg[-1]].copy(), int(s2.value), int(s3.value)


def partition(beg, adj, p: int):
    """Restated Preprocess/partition.cpp:72-121: dict (i,j) -> (tile_beg, tile_adj)."""
    lib = load()
    b = np.ascontiguousarray(beg, dtype=np.int64)
    a = np.ascontiguousarray(adj, dtype=np.int32)
    n = b.size - 1
    rows = np.zeros(p, dtype=np.int64)
    ents = np.zeros(p * p, dtype=np.int64)
    lib.orc_partition_sizes(_p(b), _p(a), n, p, _p(rows), _p(ents))
    tb = [np.zeros(rows[t // p] + 1, dtype=np.int64) for t in range(p * p)]
    ta = [np.zeros(max(ents[t], 1), dtype=np.int32) for t in range(p * p)]
    pb = (C.c_void_p * (p * p))(*[x.ctypes.data for x in tb])
    pa = (C.c_void_p * (p * p))(*[x.ctypes.data for x in ta])
    lib.orc_partition(_p(b), _p(a), n, p, C.cast(pb, C.c_void_p), C.cast(pa, C.c_void_p))
    return {(t // p, t % p): (tb[t], ta[t][: ents[t]].copy()) for t in range(p * p)}


def rmat_thresholds(a: float, b: float, c: float):
    s32 = 4294967296.0
    return (int(min(a * s32, s32 - 1)), int(min((a + b) * s32, s32 - 1)), int(min((a + b + c) * s32, s32 - 1)))


def gen_rmat(scale: int, npairs: int, a=0.57, b=0.19, c=0.19, seed=1) -> np.ndarray:
    out = np.zeros((npairs, 2), dtype=np.int32)
    ta, tab, tabc = rmat_thresholds(a, b, c)
    load().orc_gen_rmat(scale, npairs, ta, tab, tabc, seed, _p(out))
    return out


def chung_lu_cdf(n: int, gamma: float, w_max: float, target_edges: int) -> np.ndarray:
    cdf = np.zeros(n, dtype=np.uint64)
    load().orc_chung_lu_cdf(n, gamma, w_max, target_edges, _p(cdf))
    return cdf


def gen_weighted(cdf: np.ndarray, npairs: int, seed: int) -> np.ndarray:
    out = np.zeros((npairs, 2), dtype=np.int32)
    c = np.ascontiguousarray(cdf, dtype=np.uint64)
    load().orc_gen_weighted(_p(c), c.size, npairs, seed, _p(out))
    return out


def gen_er(n: int, npairs: int, seed: int) -> np.ndarray:
    out = np.zeros((npairs, 2), dtype=np.int32)
    load().orc_gen_er(n, npairs, seed, _p(out))
    return out


def gen_ba(n: int, d: int, seed: int) -> np.ndarray:
    """Barabasi-Albert pairs, d per vertex (vertex 0's are self loops): tc_oracle.c orc_gen_ba."""
    out = np.zeros((n * d, 2), dtype=np.int32)
    load().orc_gen_ba(n, d, seed, _p(out))
    return out


def batch_graph_pairs(kind: str, n: int, param: int, npairs: int, seed: int) -> np.ndarray:
    """One batch graph's pairs (local ids) from the CPU twin of its generator: Erdos-Renyi with
    `npairs` uniform pairs, or Barabasi-Albert with `param` edges per vertex."""
    return gen_er(n, npairs, seed) if kind == "er" else gen_ba(n, param, seed)


# ---- the reference kernel rebuilt for sm_103a (GPU host only) ------------------------------------

def ref_kernel_available() -> bool:
    return os.path.exists(CUDA_LIB_PATH) and os.path.exists(REF_CUBIN)


def ref_kernel_count(beg, adj, blocks: int = 1024, chunk: int = 1):
    """Run dynamic_assign from Without-graph-partition/TC.cu (cubin built from source) on a CSR the
    caller has certified with trust_check(...)[0] == 0.  Returns (count, kernel_ms)."""
    global _cuda_lib
    flags, _ = trust_check(beg, adj)
    if flags != TRUST_EXACT:
        raise ValueError(f"reference kernel is not exact on this CSR (flags {flags})")
    if _cuda_lib is None:
        lib = C.CDLL(CUDA_LIB_PATH)
        _declare(lib)
        lib.orc_ref_tc_run.restype = C.c_int
        lib.orc_ref_tc_run.argtypes = [C.c_char_p, _P, _P, C.c_int64, C.c_int64, C.c_int, C.c_int, C.c_int,
                                       C.POINTER(C.c_uint64), C.POINTER(C.c_float)]
        lib.orc_ref_tc_error.restype = C.c_char_p
        _cuda_lib = lib
    b = np.ascontiguousarray(beg, dtype=np.int64)
    a = np.ascontiguousarray(adj, dtype=np.int32)
    cnt, ms = C.c_uint64(), C.c_float()
    rc = _cuda_lib.orc_ref_tc_run(REF_CUBIN.encode(), _p(b), _p(a), b.size - 1, a.size, 1024, blocks, chunk,
                                  C.byref(cnt), C.byref(ms))
    if rc != 0:
        raise RuntimeError("reference kernel run failed: " + _cuda_lib.orc_ref_tc_error().decode())
    return int(cnt.value), float(ms.value)


# ---- pure Python, small cases only ----------------------------------------------------------------

def brute_count(beg, adj, min_deg: int = 2) -> int:
    """The counted quantity by definition (multiplicity on both arc sides, set on the table side)."""
    beg = [int(x) for x in beg]
    adj = [int(x) for x in adj]
    total = 0
    for v in range(len(beg) - 1):
        row = adj[beg[v]:beg[v + 1]]
        if len(row) < min_deg:
            continue
        s = set(row)
        for u in row:
            total += sum(1 for w in adj[beg[u]:beg[u + 1]] if w in s)
    return total
