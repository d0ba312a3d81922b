"""The allocation-free entry point, trust_tc_count_csr_noalloc, through the C ABI.

It serves callers that may not allocate GPU memory while counting (a fixed memory budget owned by
their own pool, or no tolerance for cudaMalloc's implicit synchronisation).  Its output must equal
the regular entry point's, exactly (integer counts), on two calls in a row over the same shared
scratch array.  This file is collected last so a failure here comes after every other test.
"""
import ctypes as C
import os

import numpy as np
import pytest

import trust_gb300 as T
from trust_gb300 import _lib

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _noalloc(beg, adj, **kw):
    o = T._opts(ptr_kind=T.DEVICE, **kw)
    r = _lib.Result()
    rc = T.load().trust_tc_count_csr_noalloc(C.c_void_p(beg.data_ptr()), C.c_void_p(adj.data_ptr()),
                                              beg.numel() - 1, adj.numel(), C.byref(o), C.byref(r))
    return rc, r


def _regular(beg, adj, **kw):
    o = T._opts(ptr_kind=T.DEVICE, **kw)
    r = _lib.Result()
    rc = T.load().trust_tc_count_csr(None, C.c_void_p(beg.data_ptr()), C.c_void_p(adj.data_ptr()),
                                     beg.numel() - 1, adj.numel(), C.byref(o), C.byref(r))
    return rc, r


def _graphs():
    out = []
    for name in ("rmat_s12", "k150", "chung_lu_3000", "toy"):
        z = np.load(os.path.join(GOLD, name + ".npz"))
        out.append((name, torch.from_numpy(z["ref_beg"]).cuda(), torch.from_numpy(z["ref_adj"]).cuda()))
    pairs = T.gen_chung_lu(200_000, 2.5, 300.0, 800_000, 800_000, seed=11)
    b, a = T.build_csr(pairs, 200_000)
    out.append(("chung_lu_200k", b, a))
    return out


def test_noalloc_matches_regular_entry_point_twice():
    for name, beg, adj in _graphs():
        rc, ref = _regular(beg, adj)
        assert rc == _lib.OK, name
        # the allocation-free variant always lists the sub-warp classes; the regular entry point's
        # default may take the plain split on a small skewed graph, so classes are compared with
        # the regular entry point under the tuned schedule
        rc, ref_tuned = _regular(beg, adj, schedule=T.SCHED_TUNED)
        assert rc == _lib.OK, name
        for call in range(2):
            rc, r = _noalloc(beg, adj)
            assert rc == _lib.OK, (name, call, rc)
            assert r.triangles == ref.triangles, (name, call)
            assert r.wedges == ref.wedges and r.max_out_degree == ref.max_out_degree, (name, call)
            assert list(r.class_sizes) == list(ref_tuned.class_sizes), (name, call)


def test_noalloc_rejects_what_it_cannot_hold():
    z = np.load(os.path.join(GOLD, "k150.npz"))
    beg = torch.from_numpy(z["ref_beg"]).cuda()
    adj = torch.from_numpy(z["ref_adj"]).cuda()
    # out-degrees above the CTA table would need a spill table
    rc, _ = _noalloc(beg, adj, warp_max=32, block_max=64)
    assert rc == _lib.E_TOO_LARGE
    # more rows than the scratch lists hold (rejected before any launch)
    big = torch.zeros(4_194_241 + 1, dtype=torch.int64, device="cuda")
    rc, _ = _noalloc(big, adj[:0])
    assert rc == _lib.E_TOO_LARGE
    # host pointers are not accepted
    o = T._opts(ptr_kind=T.HOST)
    r = _lib.Result()
    b = np.ascontiguousarray(z["ref_beg"])
    a = np.ascontiguousarray(z["ref_adj"])
    rc = T.load().trust_tc_count_csr_noalloc(b.ctypes.data_as(C.c_void_p), a.ctypes.data_as(C.c_void_p),
                                              b.size - 1, a.size, C.byref(o), C.byref(r))
    assert rc == _lib.E_UNSUPPORTED
    # per-vertex cycle recording and source-row ranges belong to the regular entry point only
    for field in ("record_cycles", "row_end"):
        o = T._opts(ptr_kind=T.DEVICE)
        setattr(o, field, 1)
        rc = T.load().trust_tc_count_csr_noalloc(C.c_void_p(beg.data_ptr()), C.c_void_p(adj.data_ptr()),
                                                  beg.numel() - 1, adj.numel(), C.byref(o), C.byref(r))
        assert rc == _lib.E_UNSUPPORTED, field
    # and it still counts correctly afterwards
    rc, r = _noalloc(beg, adj)
    assert rc == _lib.OK and r.triangles == int(z["nx_triangles"][0])
