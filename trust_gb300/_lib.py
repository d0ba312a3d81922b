"""ctypes binding of include/trust_tc.h (the in-tree libtrust_tc.so).

Loading fails loudly when the library has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libtrust_tc.so")

OK = 0
E_ARG, E_IO, E_FORMAT, E_OFFSETS, E_IDS, E_TOO_LARGE, E_CUDA, E_NOMEM, E_DEVICE, E_UNSUPPORTED, E_NO_DEVICE = range(1, 12)
HOST, DEVICE = 0, 1
SCHED_PLAIN, SCHED_LEARNED, SCHED_TUNED = 0, 1, 2
VALIDATE_NONE, VALIDATE_OFFSETS, VALIDATE_FULL = 0, 1, 2
CLASS_NAMES = ("skip", "g4", "g8", "g16", "g32", "warp", "cta", "huge")


class Opts(C.Structure):
    _fields_ = [
        ("device", C.c_int),
        ("threads_per_block", C.c_int),
        ("blocks", C.c_int),
        ("chunk", C.c_int),
        ("ptr_kind", C.c_int),
        ("schedule", C.c_int),
        ("validate", C.c_int),
        ("warp_max_degree", C.c_int),
        ("block_max_degree", C.c_int),
        ("record_cycles", C.c_int),
        ("stream", C.c_void_p),
        ("model", C.c_void_p),
        ("direction_split", C.c_int),
        ("hub_cluster", C.c_int),
        ("row_begin", C.c_int64),
        ("row_end", C.c_int64),
        ("test_wait_expiry", C.c_int),
    ]


class Result(C.Structure):
    _fields_ = [
        ("triangles", C.c_uint64),
        ("kernel_seconds", C.c_double),
        ("count_seconds", C.c_double),
        ("call_seconds", C.c_double),
        ("vertices", C.c_int64),
        ("edges", C.c_int64),
        ("max_out_degree", C.c_int64),
        ("wedges", C.c_int64),
        ("class_sizes", C.c_int64 * 8),
        ("vertex_cycles", C.c_void_p),
        ("direction_split", C.c_int32),
        ("split_saving_ms", C.c_float),
    ]


class BatchClass(C.Structure):
    _fields_ = [("threads_per_block", C.c_int), ("warp_max_degree", C.c_int), ("chunk", C.c_int)]


BATCH_CLASSES = 4

_P = C.c_void_p
_I64P = C.POINTER(C.c_int64)
_I32P = C.POINTER(C.c_int32)

# name -> (restype, argtypes); every function declared in include/trust_tc.h
SIGNATURES = {
    "trust_tc_opts_init": (None, [C.POINTER(Opts)]),
    "trust_tc_strerror": (C.c_char_p, [C.c_int]),
    "trust_tc_last_cuda_error": (C.c_char_p, []),
    "trust_tc_version": (C.c_char_p, []),
    "trust_tc_readback_bytes": (C.c_size_t, []),
    "trust_tc_kernel_launches": (C.c_uint64, []),
    "trust_tc_ctx_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "trust_tc_ctx_destroy": (C.c_int, [_P]),
    "trust_tc_validate_csr": (C.c_int, [_P, _P, C.c_int64, C.c_int64, _I64P]),
    "trust_tc_count_csr": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, C.POINTER(Opts), C.POINTER(Result)]),
    "trust_tc_count_csr_noalloc": (C.c_int, [_P, _P, C.c_int64, C.c_int64, C.POINTER(Opts), C.POINTER(Result)]),
    "trust_tc_stage_csr": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64]),
    "trust_tc_load_folder": (C.c_int, [C.c_char_p, C.POINTER(_I64P), C.POINTER(_I32P), _I64P, _I64P]),
    "trust_tc_save_folder": (C.c_int, [C.c_char_p, _P, _P, C.c_int64, C.c_int64]),
    "trust_tc_free_host": (None, [_P]),
    "trust_tc_count_folder": (C.c_int, [C.c_char_p, C.POINTER(Opts), C.POINTER(Result)]),
    "trust_tc_count_partitioned": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(Opts), C.POINTER(Result)]),
    "trust_tc_autotune": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, C.POINTER(Opts), C.c_int, C.c_double,
                                    C.POINTER(Opts), C.POINTER(C.c_double)]),
    "trust_tc_count_tiles_device": (C.c_int, [_P, _P, C.c_int64, C.c_int64, C.c_int, C.c_size_t, C.POINTER(Opts),
                                              C.POINTER(Result)]),
    "trust_tc_partition_folder": (C.c_int, [C.c_char_p, _P, _P, C.c_int64, C.c_int64, C.c_int]),
    "trust_tc_build_csr_device": (C.c_int, [_P, _P, C.c_int64, C.c_int64, C.POINTER(C.c_void_p),
                                            C.POINTER(C.c_void_p), _I64P, _I64P]),
    "trust_tc_free_device": (None, [_P]),
    "trust_tc_copy": (C.c_int, [_P, _P, C.c_size_t]),
    "trust_tc_gen_rmat_device": (C.c_int, [_P, C.c_int, C.c_int64, C.c_double, C.c_double, C.c_double,
                                           C.c_uint64, _P]),
    "trust_tc_gen_chung_lu_device": (C.c_int, [_P, C.c_int64, C.c_double, C.c_double, C.c_int64, C.c_int64,
                                               C.c_uint64, _P]),
    "trust_tc_chung_lu_table": (C.c_double, [C.c_int64, C.c_double, C.c_double, C.c_int64, _P]),
    "trust_tc_gen_er_device": (C.c_int, [_P, C.c_int64, C.c_int64, C.c_uint64, _P]),
    "trust_tc_gen_ba_device": (C.c_int, [_P, C.c_int64, C.c_int, C.c_uint64, _P]),
    "trust_tc_batch_create": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, _I64P, C.c_int64, C.POINTER(C.c_void_p)]),
    "trust_tc_batch_destroy": (None, [_P]),
    "trust_tc_batch_info": (C.c_int, [_P, _I64P, _I64P, _I32P]),
    "trust_tc_batch_get_class": (C.c_int, [_P, C.c_int, C.POINTER(BatchClass)]),
    "trust_tc_batch_set_class": (C.c_int, [_P, C.c_int, C.POINTER(BatchClass)]),
    "trust_tc_batch_autotune": (C.c_int, [_P, C.c_int, C.POINTER(C.c_double)]),
    "trust_tc_batch_run": (C.c_int, [_P, _P, C.POINTER(C.c_uint64), C.POINTER(Result)]),
    "trust_tc_build_batch_device": (C.c_int, [_P, _P, C.c_int64, _I64P, C.c_int64, C.POINTER(C.c_void_p),
                                              C.POINTER(C.c_void_p), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                              _I64P]),
    "trust_tc_model_floats": (C.c_int, []),
    "trust_tc_model_init": (C.c_int, [_P, C.c_uint64]),
    "trust_tc_model_grad": (C.c_int, [_P, _P, C.c_int64, _P, _P, C.POINTER(C.c_float)]),
    "trust_tc_model_train": (C.c_int, [_P, _P, C.c_int64, C.c_int, C.c_int, C.c_float, _P, C.POINTER(C.c_float)]),
    "trust_tc_model_predict": (C.c_int, [_P, C.c_int64, _P, _P]),
    "trust_tc_model_default": (C.c_int, [_P]),
    "trust_tc_vertex_features": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, _P]),
}

_lib = None


def load() -> C.CDLL:
    """Load libtrust_tc.so (built by trust_gb300.build / __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()'); there is no CPU fallback")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class TrustTcError(RuntimeError):
    def __init__(self, status: int, where: str = ""):
        lib = load()
        msg = lib.trust_tc_strerror(status).decode()
        cuda = lib.trust_tc_last_cuda_error().decode()
        super().__init__(f"{where}: {msg}" + (f" [{cuda}]" if cuda and status == E_CUDA else ""))
        self.status = status


def check(status: int, where: str = "") -> None:
    if status != OK:
        raise TrustTcError(status, where)
