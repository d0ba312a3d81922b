"""trust_gb300 — GB300-native (sm_103a) vertex-centric hash triangle counter.

Python host mirror of TRUST's operator surface over the C ABI of include/trust_tc.h:

  Triangle_count(rank, name, args, total_process, n_threads, n_blocks, chunk_size[, partition_num])
      the reference operator (Without-graph-partition/TC.cu:602-731 and
      With-graph-partition/TC.cu:976-1157), returning the same `arguments` record
      (Without-graph-partition/TC.cuh:2-8)
  count_csr / count_folder / count_partitioned
      the C entry points with numpy (host) or torch CUDA (device) arrays
  gen_rmat / gen_chung_lu / gen_er / build_csr
      deterministic synthetic graphs and the GPU preprocessing into an oriented CSR

Every count runs in libtrust_tc.so on the GPU; a missing library or device raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import (CLASS_NAMES, DEVICE, HOST, SCHED_LEARNED, SCHED_PLAIN, SCHED_TUNED, VALIDATE_FULL, VALIDATE_NONE,
                   VALIDATE_OFFSETS, TrustTcError, check, load)

__all__ = [
    "arguments", "Triangle_count", "Context", "CountResult", "count_csr", "count_folder", "count_partitioned",
    "count_tiles", "autotune",
    "load_folder", "save_folder", "partition_folder", "gen_rmat", "gen_chung_lu", "gen_er", "build_csr",
    "chung_lu_table", "gen_ba", "TrustTcError", "load", "model_floats", "model_init", "model_default", "model_grad",
    "model_train", "model_predict", "vertex_features",
]


@dataclass
class arguments:  # noqa: N801 — the reference's name (Without-graph-partition/TC.cuh:2-8)
    edge_count: int = 0
    count: int = 0
    time: float = 0.0
    degree: int = 0
    vertices: int = 0


@dataclass
class CountResult:
    triangles: int
    kernel_seconds: float
    count_seconds: float
    call_seconds: float
    vertices: int
    edges: int
    max_out_degree: int
    wedges: int = 0
    class_sizes: dict = field(default_factory=dict)
    direction_split: int = 0  # 1 when the reverse-direction pass ran (tile loop: jobs that ran it)
    split_saving_ms: float = 0.0


def _result(r: _lib.Result) -> CountResult:
    return CountResult(int(r.triangles), r.kernel_seconds, r.count_seconds, r.call_seconds, int(r.vertices),
                       int(r.edges), int(r.max_out_degree), int(r.wedges),
                       {k: int(v) for k, v in zip(CLASS_NAMES, r.class_sizes)}, int(r.direction_split),
                       float(r.split_saving_ms))


def _opts(threads=0, blocks=0, chunk=0, ptr_kind=HOST, validate=VALIDATE_FULL, warp_max=0, block_max=0,
          stream=None, device=-1, schedule=SCHED_LEARNED) -> _lib.Opts:
    o = _lib.Opts()
    load().trust_tc_opts_init(C.byref(o))
    o.device = device
    o.threads_per_block = threads
    o.blocks = blocks
    o.chunk = chunk
    o.ptr_kind = ptr_kind
    o.validate = validate
    o.warp_max_degree = warp_max
    o.block_max_degree = block_max
    o.schedule = schedule
    o.stream = stream
    return o


class Context:
    """Reusable device scratch (trust_tc_ctx).  Use as a context manager or call close()."""

    def __init__(self, device: int = -1):
        h = C.c_void_p()
        check(load().trust_tc_ctx_create(C.byref(h), device), "trust_tc_ctx_create")
        self.handle = h

    def close(self) -> None:
        if self.handle:
            load().trust_tc_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _is_torch_cuda(x) -> bool:
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


def count_csr(beg, adj, *, ctx: Context | None = None, threads=0, blocks=0, chunk=0, stream=None,
              validate=VALIDATE_FULL, warp_max=0, block_max=0, schedule=SCHED_LEARNED,
              cycles=None, direction_split=-1, model=None, hub_cluster=0,
              row_range: tuple[int, int] | None = None) -> CountResult:
    """Count over a CSR held in numpy arrays (host) or contiguous torch CUDA tensors (device).

    `stream` is a cudaStream_t value (e.g. torch.cuda.current_stream().cuda_stream).
    `row_range` = (lo, hi): count only the arcs whose source row lies in [lo, hi); the whole graph
    is still validated and probed, so the slices of a graph sum to its count."""
    lib = load()
    if _is_torch_cuda(beg):
        import torch
        assert beg.dtype == torch.int64 and adj.dtype == torch.int32 and beg.is_contiguous() and adj.is_contiguous()
        n, m = beg.numel() - 1, adj.numel()
        pb, pa, kind = C.c_void_p(beg.data_ptr()), C.c_void_p(adj.data_ptr() if m else 0), DEVICE
        keep = (beg, adj)
    else:
        b = np.ascontiguousarray(beg, dtype=np.int64)
        a = np.ascontiguousarray(adj, dtype=np.int32)
        n, m = b.size - 1, a.size
        pb, pa, kind = b.ctypes.data_as(C.c_void_p), a.ctypes.data_as(C.c_void_p), HOST
        keep = (b, a)
    o = _opts(threads, blocks, chunk, kind, validate, warp_max, block_max, stream, schedule=schedule)
    o.direction_split = direction_split
    o.hub_cluster = hub_cluster
    if row_range is not None:
        lo, hi = int(row_range[0]), int(row_range[1])
        if hi <= 0:  # the C field's 0 means "all rows"; an explicit range ends at a positive row
            raise ValueError("row_range end must be positive")
        o.row_begin, o.row_end = lo, hi
    if model is not None:  # host float32 array of model_floats() entries (learned schedule)
        model = np.ascontiguousarray(model, dtype=np.float32)
        o.model = model.ctypes.data_as(C.c_void_p)
    r = _lib.Result()
    if cycles is not None:  # torch CUDA int64 tensor of n entries: per-vertex clock64 cycles
        assert cycles.is_cuda and cycles.numel() >= n
        o.record_cycles = 1
        r.vertex_cycles = C.c_void_p(cycles.data_ptr())
    st = lib.trust_tc_count_csr(ctx.handle if ctx else None, pb, pa, n, m, C.byref(o), C.byref(r))
    del keep
    check(st, "trust_tc_count_csr")
    return _result(r)


def stage_csr(beg: np.ndarray, adj: np.ndarray, ctx: Context) -> None:
    """Start the host-to-device copy of a host CSR on the context's copy stream; the next
    count_csr(beg, adj, ctx=ctx) counts the staged copy.  The arrays (int64 / int32, contiguous,
    ideally pinned) must stay alive and unchanged until that count returns."""
    assert isinstance(beg, np.ndarray) and beg.dtype == np.int64 and beg.flags.c_contiguous
    assert isinstance(adj, np.ndarray) and adj.dtype == np.int32 and adj.flags.c_contiguous
    check(load().trust_tc_stage_csr(ctx.handle, beg.ctypes.data_as(C.c_void_p), adj.ctypes.data_as(C.c_void_p),
                                    beg.size - 1, adj.size), "trust_tc_stage_csr")


def count_folder(folder: str, threads=0, blocks=0, chunk=0) -> CountResult:
    o = _opts(threads, blocks, chunk)
    r = _lib.Result()
    check(load().trust_tc_count_folder(folder.encode(), C.byref(o), C.byref(r)), "trust_tc_count_folder")
    return _result(r)


def count_partitioned(folder: str, parts: int, threads=0, blocks=0, chunk=0, schedule=SCHED_LEARNED,
                      direction_split: int = -1) -> CountResult:
    o = _opts(threads, blocks, chunk, schedule=schedule)
    o.direction_split = direction_split
    r = _lib.Result()
    check(load().trust_tc_count_partitioned(folder.encode(), parts, C.byref(o), C.byref(r)),
          "trust_tc_count_partitioned")
    return _result(r)


def autotune(beg, adj, ctx: Context, repeats: int = 3, schedule=SCHED_LEARNED,
             time_budget_s: float = 0.0) -> tuple[dict, float]:
    """Fastest launch parameters for this device CSR (torch CUDA tensors): (count_csr keyword
    arguments, median call ms).  `time_budget_s` > 0 stops starting new candidates once the calls
    made add up to that much time."""
    o = _opts(ptr_kind=DEVICE, schedule=schedule)
    best = _lib.Opts()
    ms = C.c_double()
    check(load().trust_tc_autotune(ctx.handle, C.c_void_p(beg.data_ptr()), C.c_void_p(adj.data_ptr()), beg.numel() - 1,
                                   adj.numel(), C.byref(o), repeats, float(time_budget_s), C.byref(best),
                                   C.byref(ms)), "trust_tc_autotune")
    return ({"threads": best.threads_per_block, "warp_max": best.warp_max_degree, "chunk": best.chunk,
             "hub_cluster": best.hub_cluster, "schedule": best.schedule}, ms.value)


def count_tiles(beg, adj, parts: int, budget_bytes: int = 0, threads=0, blocks=0, chunk=0,
                schedule=SCHED_LEARNED, direction_split: int = -1) -> CountResult:
    """The n x n tile loop over a device CSR (torch CUDA tensors): GPU partition into pinned host
    tiles, then the (i,j,k) jobs with tiles streamed into a device cache of `budget_bytes`.
    `direction_split`: -1 the schedule decides per job, 0 never, 1 every job whose tiles allow it
    (`CountResult.direction_split` = the jobs that ran it)."""
    o = _opts(threads, blocks, chunk, DEVICE, schedule=schedule)
    o.direction_split = direction_split
    r = _lib.Result()
    check(load().trust_tc_count_tiles_device(C.c_void_p(beg.data_ptr()), C.c_void_p(adj.data_ptr()), beg.numel() - 1,
                                             adj.numel(), parts, budget_bytes, C.byref(o), C.byref(r)),
          "trust_tc_count_tiles_device")
    return _result(r)


def Triangle_count(rank: int, name: str, args: arguments, total_process: int, n_threads: int, n_blocks: int,
                   chunk_size: int, partition_num: int | None = None) -> arguments:  # noqa: N802
    """The reference operator.  One GPU: rank 0 returns the whole count, other ranks 0, so the
    caller's SUM over ranks (Without-graph-partition/mpi_main.cpp:110-112) is unchanged.  Where the
    reference prints and exits on error, this raises TrustTcError."""
    del total_process
    if rank > 0:
        if partition_num is None:
            b, a = load_folder(name)
            return arguments(edge_count=a.size, count=0, time=0.0,
                             degree=(a.size // (b.size - 1)) if b.size > 1 else 0, vertices=b.size - 1)
        return arguments()
    if partition_num is None:
        r = count_folder(name, n_threads, n_blocks, chunk_size)
    else:
        r = count_partitioned(name, partition_num, n_threads, n_blocks, chunk_size)
    return arguments(edge_count=r.edges, count=r.triangles, time=r.kernel_seconds,
                     degree=(r.edges // r.vertices) if r.vertices else 0, vertices=r.vertices)


def load_folder(folder: str):
    lib = load()
    pb, pa = C.POINTER(C.c_int64)(), C.POINTER(C.c_int32)()
    n, m = C.c_int64(), C.c_int64()
    check(lib.trust_tc_load_folder(folder.encode(), C.byref(pb), C.byref(pa), C.byref(n), C.byref(m)),
          "trust_tc_load_folder")
    try:
        beg = np.ctypeslib.as_array(pb, shape=(n.value + 1,)).copy()
        adj = np.ctypeslib.as_array(pa, shape=(max(m.value, 1),))[: m.value].copy()
    finally:
        lib.trust_tc_free_host(C.cast(pb, C.c_void_p))
        lib.trust_tc_free_host(C.cast(pa, C.c_void_p))
    return beg, adj


def save_folder(folder: str, beg, adj) -> None:
    b = np.ascontiguousarray(beg, dtype=np.int64)
    a = np.ascontiguousarray(adj, dtype=np.int32)
    check(load().trust_tc_save_folder(folder.encode(), b.ctypes.data_as(C.c_void_p), a.ctypes.data_as(C.c_void_p),
                                      b.size - 1, a.size), "trust_tc_save_folder")


def partition_folder(folder: str, beg, adj, parts: int) -> None:
    b = np.ascontiguousarray(beg, dtype=np.int64)
    a = np.ascontiguousarray(adj, dtype=np.int32)
    check(load().trust_tc_partition_folder(folder.encode(), b.ctypes.data_as(C.c_void_p),
                                           a.ctypes.data_as(C.c_void_p), b.size - 1, a.size, parts),
          "trust_tc_partition_folder")


def chung_lu_table(n: int, gamma: float, w_max: float, target_edges: int) -> np.ndarray:
    cdf = np.zeros(n, dtype=np.uint64)
    load().trust_tc_chung_lu_table(n, gamma, w_max, target_edges, cdf.ctypes.data_as(C.c_void_p))
    return cdf


def _pairs(npairs: int):
    import torch
    return torch.empty((npairs, 2), dtype=torch.int32, device="cuda")


def gen_rmat(scale: int, edge_factor: int, a=0.57, b=0.19, c=0.19, seed=1, npairs: int | None = None):
    """R-MAT pairs on the GPU: (edge_factor << scale) x 2 int32 tensor."""
    np_ = (edge_factor << scale) if npairs is None else npairs
    out = _pairs(np_)
    check(load().trust_tc_gen_rmat_device(None, scale, np_, a, b, c, seed, C.c_void_p(out.data_ptr())),
          "trust_tc_gen_rmat_device")
    return out


def gen_chung_lu(n: int, gamma: float, w_max: float, target_edges: int, npairs: int, seed=2):
    out = _pairs(npairs)
    check(load().trust_tc_gen_chung_lu_device(None, n, gamma, w_max, target_edges, npairs, seed,
                                              C.c_void_p(out.data_ptr())), "trust_tc_gen_chung_lu_device")
    return out


def gen_ba(n: int, d: int, seed=5):
    """Barabasi-Albert pairs on the GPU: (n * d) x 2 int32 tensor (vertex 0's d pairs are self loops)."""
    out = _pairs(n * d)
    check(load().trust_tc_gen_ba_device(None, n, d, seed, C.c_void_p(out.data_ptr())), "trust_tc_gen_ba_device")
    return out


def gen_er(n: int, npairs: int, seed=5):
    out = _pairs(npairs)
    check(load().trust_tc_gen_er_device(None, n, npairs, seed, C.c_void_p(out.data_ptr())), "trust_tc_gen_er_device")
    return out


def build_csr(pairs, id_bound: int):
    """GPU preprocessing of an (npairs, 2) int32 CUDA tensor into an oriented CSR (beg int64, adj int32)."""
    import torch
    lib = load()
    pb, pa = C.c_void_p(), C.c_void_p()
    n, m = C.c_int64(), C.c_int64()
    pairs = pairs.contiguous()
    check(lib.trust_tc_build_csr_device(None, C.c_void_p(pairs.data_ptr()), pairs.shape[0], id_bound, C.byref(pb),
                                        C.byref(pa), C.byref(n), C.byref(m)), "trust_tc_build_csr_device")
    try:
        beg = torch.empty(n.value + 1, dtype=torch.int64, device="cuda")
        adj = torch.empty(max(m.value, 1), dtype=torch.int32, device="cuda")
        check(lib.trust_tc_copy(C.c_void_p(beg.data_ptr()), pb, 8 * (n.value + 1)), "trust_tc_copy")
        check(lib.trust_tc_copy(C.c_void_p(adj.data_ptr()), pa, 4 * m.value), "trust_tc_copy")
    finally:
        lib.trust_tc_free_device(pb)
        lib.trust_tc_free_device(pa)
    return beg, adj[: m.value]


# ---- the learned schedule's cost model ------------------------------------------------------------

def model_floats() -> int:
    return int(load().trust_tc_model_floats())


def model_init(seed: int = 1) -> np.ndarray:
    m = np.zeros(model_floats(), dtype=np.float32)
    check(load().trust_tc_model_init(m.ctypes.data_as(C.c_void_p), seed), "trust_tc_model_init")
    return m


def model_default():
    """The model compiled into the library, or None before the first training run."""
    m = np.zeros(model_floats(), dtype=np.float32)
    st = load().trust_tc_model_default(m.ctypes.data_as(C.c_void_p))
    return m if st == _lib.OK else None


def model_grad(x, y, model):
    """MSE gradient at `model` over torch CUDA float32 tensors x (N x 8) and y (N)."""
    g = np.zeros(model_floats(), dtype=np.float32)
    loss = C.c_float()
    m = np.ascontiguousarray(model, dtype=np.float32)
    check(load().trust_tc_model_grad(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), x.shape[0],
                                     m.ctypes.data_as(C.c_void_p), g.ctypes.data_as(C.c_void_p), C.byref(loss)),
          "trust_tc_model_grad")
    return g, float(loss.value)


def model_train(x, y, model, epochs=100, batch=4096, lr=1e-3):
    m = np.ascontiguousarray(model, dtype=np.float32).copy()
    loss = C.c_float()
    check(load().trust_tc_model_train(C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), x.shape[0], epochs, batch,
                                      lr, m.ctypes.data_as(C.c_void_p), C.byref(loss)), "trust_tc_model_train")
    return m, float(loss.value)


def model_predict(x, model):
    import torch
    out = torch.empty(x.shape[0], dtype=torch.float32, device="cuda")
    m = np.ascontiguousarray(model, dtype=np.float32)
    check(load().trust_tc_model_predict(C.c_void_p(x.data_ptr()), x.shape[0], m.ctypes.data_as(C.c_void_p),
                                        C.c_void_p(out.data_ptr())), "trust_tc_model_predict")
    return out


def vertex_features(beg, adj, ctx: Context):
    """n x 8 float32 CUDA tensor of per-vertex features (zeros for out-degree < 2)."""
    import torch
    n = beg.numel() - 1
    f = torch.empty((max(n, 1), 8), dtype=torch.float32, device="cuda")
    check(load().trust_tc_vertex_features(ctx.handle, C.c_void_p(beg.data_ptr()), C.c_void_p(adj.data_ptr()), n,
                                          adj.numel(), C.c_void_p(f.data_ptr())), "trust_tc_vertex_features")
    return f[:n]
