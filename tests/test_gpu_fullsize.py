"""Full-size parity on the large workloads: every count against the oracle or an analytic answer.

* 4096-graph batch (4096 graphs, 50..50,000 vertices, ER/BA, seed 5): every per-graph u64 count of
  the one-launch batch equals the oracle's forward-intersection count of the same graph, built by
  the oracle's own generator twin and preprocessing (Without-graph-partition/TC.cu:586-599 is the
  counted quantity; the oracle merges as Without-graph-partition/graph.hpp:133-149).
* 4096 x 4096 triangulated grid (the cost model's held-out mesh): 2 * 4095^2 triangles under the
  learned, tuned and plain schedules; the GPU preprocessing equals the oracle pipeline byte for byte.
* R-MAT scale 26, edge factor 32, seed 3 (2.08e9 arcs): source-row slices counted on the GPU
  (row_range) under the learned schedule (split decided and forced) and the plain schedule equal the
  oracle's count of the same rows of the same CSR.  The slices cover the largest hub rows (hub
  kernel, TMA staging), the hub/CTA, CTA/warp and warp/group class boundaries and rows whose arcs the
  direction split moves; slices that partition the rows sum to the whole count.
"""
from __future__ import annotations

import concurrent.futures as cf
import os

import numpy as np
import pytest

import trust_gb300 as T
from oracle import oracle as O
from tests import graphs
from trust_gb300 import batch as B

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

THREADS = os.cpu_count() or 1


def _oracle_batch_count(spec) -> int:
    pairs = O.batch_graph_pairs(spec.kind, spec.n, spec.param, spec.npairs, spec.seed)
    ob, oa = O.build_csr(pairs, spec.n)
    return O.count_forward_sorted_range(ob, oa, 0, ob.size - 1, 2, 1)


def test_batch4096_every_graph_matches_oracle():
    specs = B.batch_specs(4096, 50, 50_000, 5)
    pairs, vbeg = B.gen_batch_pairs(specs)
    beg, adj, gv = B.build_batch(pairs, vbeg)
    del pairs
    with T.Context() as ctx:
        bt = B.Batch(beg, adj, gv, ctx=ctx)
        counts, r = bt.run()
        bt.autotune(repeats=1)  # a tuned launch must give the same counts
        counts2, _ = bt.run()
        bt.close()
    # the oracle builds and counts every graph on the host (ctypes releases the GIL: one graph per
    # thread)
    with cf.ThreadPoolExecutor(max_workers=THREADS) as ex:
        expect = np.array(list(ex.map(_oracle_batch_count, specs)), dtype=np.uint64)
    assert counts.size == 4096
    bad = np.nonzero(counts != expect)[0]
    assert bad.size == 0, f"graphs {bad[:10].tolist()} differ: {counts[bad[:10]]} vs {expect[bad[:10]]}"
    assert np.array_equal(counts2, expect)
    assert r.triangles == int(expect.sum())
    assert r.edges == adj.numel()


def test_grid4096_known_count_every_schedule():
    k = 4096
    pairs, tri = graphs.grid(k, 1)
    assert tri == 2 * 4095 ** 2 == 33_538_050
    beg, adj = T.build_csr(torch.from_numpy(pairs).cuda(), k * k)
    eb, ea = O.build_csr(pairs, k * k)
    assert np.array_equal(beg.cpu().numpy(), eb) and np.array_equal(adj.cpu().numpy(), ea)
    with T.Context() as ctx:
        for sch in (T.SCHED_LEARNED, T.SCHED_TUNED, T.SCHED_PLAIN):
            assert T.count_csr(beg, adj, ctx=ctx, schedule=sch).triangles == tri, sch
        assert T.count_csr(beg, adj, ctx=ctx, direction_split=1).triangles == tri
        assert T.count_tiles(beg, adj, 2).triangles == tri


@pytest.fixture(scope="module")
def rmat26():
    pairs = T.gen_rmat(26, 32, 0.57, 0.19, 0.19, seed=3)
    beg, adj = T.build_csr(pairs, 1 << 26)
    del pairs
    torch.cuda.empty_cache()
    hb, ha = beg.cpu().numpy(), adj.cpu().numpy()
    yield beg, adj, hb, ha
    del beg, adj
    torch.cuda.empty_cache()


def _slices(hb):
    """Row slices at every schedule boundary of the R-MAT 26 CSR (rows are numbered by out-degree,
    descending), each small enough for the oracle to count in seconds."""
    d = np.diff(hb)
    n = d.size

    def first_below(x):  # first row with out-degree <= x
        return int(np.searchsorted(-d, -x, side="left"))

    out = [(0, 8)]  # the largest hubs: hub kernel, TMA-staged tables
    for bound in (4096, 512, 128, 32, 16, 8, 4):
        r = first_below(bound)
        width = max(8, min(20_000, int(4e8 // max(1, d[max(r - 1, 0)] ** 2 + 1))))
        out.append((max(0, r - width // 2), min(n, r + width // 2)))
    out.append((n // 2, n // 2 + 200_000))  # rows of degree 2..4 in the middle
    out.append((n - 100_000, n))            # the tail (mostly skipped rows)
    return out


def test_rmat26_slices_match_oracle(rmat26):
    beg, adj, hb, ha = rmat26
    slices = _slices(hb)
    with T.Context() as ctx:
        for lo, hi in slices:
            expect = O.count_forward_sorted_range(hb, ha, lo, hi, 2, THREADS)
            got = {
                "learned": T.count_csr(beg, adj, ctx=ctx, row_range=(lo, hi)),
                "learned_split": T.count_csr(beg, adj, ctx=ctx, row_range=(lo, hi), direction_split=1),
                "plain": T.count_csr(beg, adj, ctx=ctx, row_range=(lo, hi), schedule=T.SCHED_PLAIN),
            }
            for name, r in got.items():
                assert r.triangles == expect, (lo, hi, name, r.triangles, expect)
            assert got["learned_split"].direction_split == 1, (lo, hi)


def test_rmat26_whole_count_is_pinned(rmat26):
    """The whole R-MAT 26 count equals the pinned count of the reference kernel itself (TC.cu
    rebuilt for sm_103a) and, where its cubin is built, a fresh run of that kernel on this CSR."""
    import json
    beg, adj, hb, ha = rmat26
    with open(os.path.join(os.path.dirname(__file__), "golden", "pinned_counts.json")) as f:
        pin = json.load(f)["rmat26_ef32"]
    assert (hb.size - 1, ha.size) == (pin["vertices"], pin["edges"])
    with T.Context() as ctx:
        assert T.count_csr(beg, adj, ctx=ctx).triangles == pin["triangles"]
    if O.ref_kernel_available():
        assert O.trust_check(hb, ha)[0] == O.TRUST_EXACT
        ref, _ = O.ref_kernel_count(hb, ha, blocks=1024, chunk=1)
        assert ref == pin["triangles"]


def test_rmat26_slices_sum_to_whole(rmat26):
    beg, adj, hb, _ = rmat26
    n = hb.size - 1
    cuts = [0, 8, 4600, 60_000, 1_000_000, 8_000_000, 30_000_000, n]
    with T.Context() as ctx:
        whole = T.count_csr(beg, adj, ctx=ctx)
        parts = [T.count_csr(beg, adj, ctx=ctx, row_range=(a, b)).triangles for a, b in zip(cuts[:-1], cuts[1:])]
        assert sum(parts) == whole.triangles
        assert T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_PLAIN).triangles == whole.triangles
        assert whole.direction_split == 1  # the learned schedule takes the split on this graph
