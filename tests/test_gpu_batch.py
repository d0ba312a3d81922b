"""Batches on the GPU: many graphs, one CUDA-graph launch, per-graph counts.

Parity: every graph's count equals the CPU oracle's forward-intersection count of the same graph
(generated by the oracle's twin generator and preprocessed by the oracle pipeline), and the
count of the same graph counted alone through trust_tc_count_csr; the batch total equals the
count of the union.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import trust_gb300 as T  # noqa: E402
from trust_gb300 import batch as B  # noqa: E402
from oracle import oracle as O  # noqa: E402


@pytest.mark.parametrize("n,d,seed", [(1, 3, 1), (20, 3, 7), (5000, 2, 5), (50_000, 16, 5)])
def test_ba_generator_matches_oracle(n, d, seed):
    assert np.array_equal(T.gen_ba(n, d, seed=seed).cpu().numpy(), O.gen_ba(n, d, seed))


@pytest.fixture(scope="module")
def small_batch():
    specs = B.batch_specs(96, 50, 6000, seed=11)
    pairs, vbeg = B.gen_batch_pairs(specs)
    beg, adj, gv = B.build_batch(pairs, vbeg)
    del pairs
    expect = []
    for s in specs:
        ob, oa = O.build_csr(O.batch_graph_pairs(s.kind, s.n, s.param, s.npairs, s.seed), s.n)
        expect.append(O.count_forward(ob, oa, threads=8))
    return specs, beg, adj, gv, np.array(expect, dtype=np.uint64)


def test_batch_counts_match_oracle(small_batch):
    specs, beg, adj, gv, expect = small_batch
    with T.Context() as ctx:
        b = B.Batch(beg, adj, gv, ctx=ctx)
        info = b.info()
        assert sum(info["graphs"]) == len(specs)
        counts, r = b.run()
        assert np.array_equal(counts, expect)
        assert r.triangles == int(expect.sum())
        assert r.triangles == T.count_csr(beg, adj, ctx=ctx).triangles  # the union, one graph
        counts2, _ = b.run()  # the captured job replays identically
        assert np.array_equal(counts2, expect)
        b.close()


def test_batch_graph_ranges_and_single_calls(small_batch):
    specs, beg, adj, gv, expect = small_batch
    assert gv[0] == 0 and gv[-1] == beg.numel() - 1 and np.all(np.diff(gv) >= 0)
    with T.Context() as ctx:
        for g in list(range(0, len(specs), 7)):
            gb, ga = B.graph_csr(beg, adj, gv, g)
            ob, oa = O.build_csr(O.batch_graph_pairs(specs[g].kind, specs[g].n, specs[g].param, specs[g].npairs, specs[g].seed), specs[g].n)
            assert gb.numel() - 1 == ob.size - 1 and ga.numel() == oa.size  # same vertices and arcs
            if ga.numel():
                r = T.count_csr(gb, ga, ctx=ctx, schedule=T.SCHED_PLAIN)
                assert r.triangles == int(expect[g])


def test_batch_autotune_and_class_settings(small_batch):
    specs, beg, adj, gv, expect = small_batch
    with T.Context() as ctx:
        b = B.Batch(beg, adj, gv, ctx=ctx)
        ms = b.autotune(repeats=1)
        assert ms > 0
        for s in range(4):
            c = b.get_class(s)
            assert c["threads_per_block"] in (128, 256, 512, 1024) and c["chunk"] in (2, 4, 8, 16)
        counts, _ = b.run()
        assert np.array_equal(counts, expect)
        b.set_class(0, 128, 64, 2)
        assert b.get_class(0) == {"threads_per_block": 128, "warp_max_degree": 64, "chunk": 2}
        counts, _ = b.run()
        assert np.array_equal(counts, expect)
        with pytest.raises(T.TrustTcError):
            b.set_class(1, 100, 128, 8)  # not a multiple of 32
        counts, _ = b.run()  # a rejected setting leaves the job as it was
        assert np.array_equal(counts, expect)
        b.close()


def test_batch_rejects_arcs_across_graphs(small_batch):
    specs, beg, adj, gv, expect = small_batch
    bad = gv.copy()
    g = int(np.argmax(np.diff(gv)))  # split the largest graph in two: its arcs now cross
    bad = np.insert(bad, g + 1, (gv[g] + gv[g + 1]) // 2)
    with T.Context() as ctx:
        with pytest.raises(T.TrustTcError) as e:
            B.Batch(beg, adj, bad, ctx=ctx)
        assert e.value.status == T._lib.E_IDS
