"""The oracle, pinned against the reference's own binaries (golden fixtures) and analytic counts.

The reference ships no test suite and no golden vectors (its only checks are `make test` runs on a
hard-coded cluster path, Without-graph-partition/Makefile:41-47), so the fixtures in tests/golden/
were produced by running the reference's preprocessing, built from source, on seeded inputs
(tests/golden/make_golden.py).
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests import graphs

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def _golden(name):
    return np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))


def test_golden_present():
    assert len(GOLDEN) >= 7


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_count_on_reference_csr(path):
    z = np.load(path)
    expect = int(z["nx_triangles"][0])
    assert O.count_forward(z["ref_beg"], z["ref_adj"]) == expect
    assert O.count_forward(z["ref_beg"], z["ref_adj"], threads=4) == expect
    if z["ref_adj"].size < 60000:
        assert O.brute_count(z["ref_beg"], z["ref_adj"]) == expect
    if "fast_beg" in z:
        assert O.count_forward(z["fast_beg"], z["fast_adj"]) == expect


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_undirect_restatement_is_byte_exact(path):
    z = np.load(path)
    k, edges = O.ref_undirect(z["pairs"])
    assert k == z["undirect_header"][0] == z["undirect_header"][1]
    assert len(edges) == z["undirect_header"][2]
    np.testing.assert_array_equal(edges, z["undirect_edges"])


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_outdegree_restatement(path):
    """Same n, m and count as the reference binary; bytes may differ only through std::sort tie order."""
    z = np.load(path)
    k, edges = O.ref_undirect(z["pairs"])
    beg, adj, s2, s3 = O.ref_outdegree_csr(k, edges)
    assert beg.size == z["ref_beg"].size and adj.size == z["ref_adj"].size
    assert O.count_forward(beg, adj) == int(z["nx_triangles"][0])
    d = np.diff(beg)
    assert np.all(d[:s2] > 100) and np.all(d[s2:s3] <= 100) and np.all(d[s3:] < 2)
    assert O.trust_check(beg, adj)[0] == O.TRUST_EXACT


def test_toy_matches_reference_bytes():
    """The toy list (K4, a triangle, a pendant, a duplicate, a self-loop, a comment line) has no
    degree ties that matter, so the restatement reproduces the reference CSR byte for byte."""
    z = _golden("toy")
    np.testing.assert_array_equal(z["ref_beg"], [0, 2, 5, 7, 7, 8, 9, 10, 10, 10])
    np.testing.assert_array_equal(z["ref_adj"], [3, 4, 3, 4, 0, 8, 6, 3, 8, 8])
    k, edges = O.ref_undirect(z["pairs"])
    beg, adj, _, _ = O.ref_outdegree_csr(k, edges)
    np.testing.assert_array_equal(beg, z["ref_beg"])
    np.testing.assert_array_equal(adj, z["ref_adj"])
    assert O.count_forward(beg, adj) == 5


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_partition_restatement_is_byte_exact(path):
    z = np.load(path)
    for p in (2, 3):
        if f"part{p}_0_0_beg" not in z:
            continue
        tiles = O.partition(z["ref_beg"], z["ref_adj"], p)
        for (i, j), (tb, ta) in tiles.items():
            np.testing.assert_array_equal(tb, z[f"part{p}_{i}_{j}_beg"])
            np.testing.assert_array_equal(ta, z[f"part{p}_{i}_{j}_adj"])
        total = sum(O.count_tiles(tiles[(i, j)], tiles[(i, k)], tiles[(k, j)])
                    for i in range(p) for j in range(p) for k in range(p))
        assert total == int(z["nx_triangles"][0])


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_canonical_pipeline(path):
    z = np.load(path)
    pairs = z["pairs"]
    beg, adj = O.build_csr(pairs, int(pairs.max()) + 1)
    d = np.diff(beg)
    assert np.all(d[:-1] >= d[1:]), "renumbered by out-degree descending"
    for v in range(beg.size - 1):
        row = adj[beg[v]:beg[v + 1]]
        assert np.all(row[:-1] < row[1:]), "rows sorted, no duplicates"
        assert not np.any(row == v)
    assert O.count_forward(beg, adj) == int(z["nx_triangles"][0])
    assert O.trust_check(beg, adj)[0] == O.TRUST_EXACT


@pytest.mark.parametrize("name,pairs,tri", graphs.kat_cases(), ids=[c[0] for c in graphs.kat_cases()])
def test_known_answers(name, pairs, tri):
    beg, adj = O.build_csr(pairs, int(pairs.max()) + 1)
    assert O.count_forward(beg, adj) == tri
    assert O.count_forward(beg, adj, threads=3) == tri


def test_formula_on_arbitrary_csr():
    """Unsorted rows, duplicates and self-loops: forward counter == definition."""
    rng = np.random.default_rng(0)
    for trial in range(20):
        beg, adj = graphs.random_csr(rng, int(rng.integers(1, 60)), int(rng.integers(0, 9)))
        for md in (1, 2):
            assert O.count_forward(beg, adj, min_deg=md) == O.brute_count(beg, adj, min_deg=md)


def test_trust_check_flags():
    # a CTA-range vertex whose 101 neighbours share one bucket (ids congruent mod 1024)
    n = 101 * 1024 + 2
    beg = np.zeros(n + 1, dtype=np.int64)
    beg[1:] = 101
    adj = (np.arange(1, 102) * 1024).astype(np.int32)
    assert O.trust_check(beg, adj)[0] & O.TRUST_BUCKET_OVERFLOW
    # a d<2 vertex before a d>=2 vertex in the warp range
    beg = np.array([0, 1, 3, 3, 3], dtype=np.int64)
    adj = np.array([2, 2, 3], dtype=np.int32)
    assert O.trust_check(beg, adj)[0] & O.TRUST_EARLY_EXIT


def test_generators_deterministic():
    a = O.gen_rmat(10, 5000, seed=3)
    b = O.gen_rmat(10, 5000, seed=3)
    np.testing.assert_array_equal(a, b)
    assert a.min() >= 0 and a.max() < 1 << 10
    assert not np.array_equal(a, O.gen_rmat(10, 5000, seed=4))
    e = O.gen_er(777, 3000, seed=1)
    assert e.min() >= 0 and e.max() < 777
    cdf = O.chung_lu_cdf(5000, 2.5, 100.0, 20000)
    assert np.all(np.diff(cdf.astype(np.float64)) >= 0) and int(cdf[-1]) == 1 << 63
    w = O.gen_weighted(cdf, 4000, seed=9)
    assert w.min() >= 0 and w.max() < 5000


def test_ba_oracle_structure():
    """Barabasi-Albert pairs: vertex v's d pairs come from v, and every target is an earlier
    vertex (vertex 0's pairs are the self-loop seed)."""
    n, d = 3000, 5
    p = O.gen_ba(n, d, 9)
    assert p.shape == (n * d, 2)
    assert np.array_equal(p[:, 0], np.repeat(np.arange(n), d))
    assert np.all(p[:d] == 0)
    assert np.all(p[d:, 1] < p[d:, 0])
    deg = np.bincount(p[d:].ravel(), minlength=n)
    assert deg.max() > 10 * d  # preferential attachment grows hubs
    assert np.array_equal(p, O.gen_ba(n, d, 9)) and not np.array_equal(p, O.gen_ba(n, d, 10))


def test_batch_specs_stream():
    """The batch workload's graph list comes from a counter-based stream: pinned values."""
    from trust_gb300.batch import batch_specs
    s = batch_specs()
    assert len(s) == 4096
    assert [(x.kind, x.n, x.param) for x in s[:4]] == [("er", 102, 27), ("ba", 60, 9), ("er", 14261, 27),
                                                        ("ba", 65, 2)]
    ns = np.array([x.n for x in s])
    assert ns.min() >= 50 and ns.max() <= 50_000
    assert sum(x.kind == "er" for x in s) == 2048
    assert all(4 <= x.param <= 64 for x in s if x.kind == "er") and all(2 <= x.param <= 16 for x in s if x.kind == "ba")


def test_strided_sample_counter():
    """The systematic row sample used by the bench's CPU baseline: the strided counts over every
    offset partition the rows, so they sum to the whole count, and the arcs they report too."""
    z = _golden("chung_lu_3000")
    beg = z["ref_beg"]
    adj = np.concatenate([np.sort(z["ref_adj"][beg[v]:beg[v + 1]]) for v in range(beg.size - 1)]).astype(np.int32)
    whole = O.count_forward_sorted_range(beg, adj, 0, beg.size - 1, 2, 1)
    assert whole == int(z["nx_triangles"][0])
    for stride in (1, 3, 7):
        parts = [O.count_forward_stride(beg, adj, s, stride, 2, 4) for s in range(stride)]
        assert sum(c for c, _ in parts) == whole
        d = np.diff(beg)
        assert sum(a for _, a in parts) == int(d[d >= 2].sum())
