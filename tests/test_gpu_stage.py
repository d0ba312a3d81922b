"""Host CSRs staged ahead of their count (trust_tc_stage_csr): the copy of the next graph runs on
the context's copy stream while the current one is counted; counts stay exact and staged inputs
are consumed oldest-first by the count call given the same host buffers."""
import os

import numpy as np
import pytest

import trust_gb300 as T
from trust_gb300 import _lib

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _pinned(name):
    z = np.load(os.path.join(GOLD, name + ".npz"))
    b = torch.from_numpy(z["ref_beg"].astype(np.int64)).pin_memory()
    a = torch.from_numpy(z["ref_adj"].astype(np.int32)).pin_memory()
    return b, a, int(z["nx_triangles"][0])


def test_stage_then_count():
    b, a, expect = _pinned("rmat_s12")
    with T.Context() as ctx:
        T.stage_csr(b.numpy(), a.numpy(), ctx)
        r = T.count_csr(b.numpy(), a.numpy(), ctx=ctx)
        assert r.triangles == expect
        assert T.count_csr(b.numpy(), a.numpy(), ctx=ctx).triangles == expect  # unstaged: copies itself


def test_two_staged_consumed_in_order_and_a_third_refused():
    b1, a1, e1 = _pinned("rmat_s12")
    b2, a2, e2 = _pinned("chung_lu_3000")
    with T.Context() as ctx:
        T.stage_csr(b1.numpy(), a1.numpy(), ctx)
        T.stage_csr(b2.numpy(), a2.numpy(), ctx)
        with pytest.raises(_lib.TrustTcError):
            T.stage_csr(b1.numpy(), a1.numpy(), ctx)
        assert T.count_csr(b2.numpy(), a2.numpy(), ctx=ctx).triangles == e2
        T.stage_csr(b2.numpy(), a2.numpy(), ctx)  # the freed slot is reused
        assert T.count_csr(b1.numpy(), a1.numpy(), ctx=ctx).triangles == e1
        assert T.count_csr(b2.numpy(), a2.numpy(), ctx=ctx).triangles == e2


def test_unmatched_count_leaves_the_staged_copy():
    b1, a1, e1 = _pinned("k150")
    b2, a2, e2 = _pinned("er_200")
    with T.Context() as ctx:
        T.stage_csr(b1.numpy(), a1.numpy(), ctx)
        assert T.count_csr(b2.numpy(), a2.numpy(), ctx=ctx).triangles == e2
        assert T.count_csr(b1.numpy(), a1.numpy(), ctx=ctx).triangles == e1


def test_pipelined_stream_of_graphs():
    """stage(next) before count(current), as a caller streaming graphs does."""
    gs = [_pinned(n) for n in ("rmat_s12", "chung_lu_3000", "k150", "rmat_s12", "er_200", "toy")]
    with T.Context() as ctx:
        T.stage_csr(gs[0][0].numpy(), gs[0][1].numpy(), ctx)
        for i, (b, a, e) in enumerate(gs):
            if i + 1 < len(gs):
                T.stage_csr(gs[i + 1][0].numpy(), gs[i + 1][1].numpy(), ctx)
            assert T.count_csr(b.numpy(), a.numpy(), ctx=ctx).triangles == e


def test_destroy_with_a_staged_input():
    b, a, _ = _pinned("rmat_s12")
    ctx = T.Context()
    T.stage_csr(b.numpy(), a.numpy(), ctx)
    ctx.close()


def test_staged_bad_ids_are_rejected():
    """A staged input is validated like any host input (ids checked on the device)."""
    b, a, _ = _pinned("toy")
    a2 = a.clone()
    a2[0] = b.numel() + 5  # out of range
    with T.Context() as ctx:
        T.stage_csr(b.numpy(), a2.numpy(), ctx)
        with pytest.raises(_lib.TrustTcError):
            T.count_csr(b.numpy(), a2.numpy(), ctx=ctx)
        b3, a3, e3 = _pinned("k150")  # the context stays usable
        assert T.count_csr(b3.numpy(), a3.numpy(), ctx=ctx).triangles == e3


def test_contexts_on_concurrent_host_threads():
    """Separate contexts used from several host threads at once (the ctypes calls release the
    GIL): launch attributes and occupancy are cached process-wide, counts stay exact."""
    import threading
    names = ["rmat_s12", "chung_lu_3000", "k150", "er_200"]
    gs = [_pinned(n) for n in names]
    errors, results = [], {}

    def work(i):
        try:
            b, a, e = gs[i % len(gs)]
            with T.Context() as ctx:
                for k in range(6):
                    threads = (128, 256, 512, 1024)[k % 4]
                    r = T.count_csr(b.numpy(), a.numpy(), ctx=ctx, threads=threads)
                    if r.triangles != e:
                        errors.append((i, k, r.triangles, e))
            results[i] = True
        except Exception as ex:  # surfaced below
            errors.append((i, repr(ex)))

    ts = [threading.Thread(target=work, args=(i,)) for i in range(8)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors and len(results) == 8
