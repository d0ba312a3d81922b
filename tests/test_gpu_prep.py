"""GPU generators and GPU preprocessing against their CPU twins in the oracle, byte for byte."""
import glob
import os

import numpy as np
import pytest

import trust_gb300 as T
from oracle import oracle as O
from tests import graphs

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


@pytest.mark.parametrize("scale,npairs,seed", [(4, 1, 1), (8, 1000, 2), (12, 65536 + 7, 3), (16, 1 << 20, 1)])
def test_rmat_generator(scale, npairs, seed):
    g = T.gen_rmat(scale, 0, npairs=npairs, seed=seed).cpu().numpy()
    np.testing.assert_array_equal(g, O.gen_rmat(scale, npairs, seed=seed))


def test_rmat_other_probabilities():
    g = T.gen_rmat(11, 0, a=0.45, b=0.22, c=0.22, npairs=30000, seed=9).cpu().numpy()
    np.testing.assert_array_equal(g, O.gen_rmat(11, 30000, 0.45, 0.22, 0.22, seed=9))


@pytest.mark.parametrize("n,npairs,seed", [(1, 10, 1), (1000, 5000, 2), (123457, 400000, 5)])
def test_er_generator(n, npairs, seed):
    np.testing.assert_array_equal(T.gen_er(n, npairs, seed).cpu().numpy(), O.gen_er(n, npairs, seed))


@pytest.mark.parametrize("n,gamma,wmax,target,npairs", [(5000, 2.5, 100.0, 20000, 20000),
                                                       (200000, 2.1, 800.0, 900000, 900000),
                                                       (100000, 3.0, 300.0, 300000, 300000)])
def test_chung_lu_generator(n, gamma, wmax, target, npairs):
    g = T.gen_chung_lu(n, gamma, wmax, target, npairs, seed=2).cpu().numpy()
    cdf = O.chung_lu_cdf(n, gamma, wmax, target)
    np.testing.assert_array_equal(g, O.gen_weighted(cdf, npairs, seed=2))


def _check_prep(pairs_np, id_bound):
    eb, ea = O.build_csr(pairs_np, id_bound)
    pairs = torch.from_numpy(np.ascontiguousarray(pairs_np, dtype=np.int32)).cuda()
    gb, ga = T.build_csr(pairs, id_bound)
    np.testing.assert_array_equal(gb.cpu().numpy(), eb)
    np.testing.assert_array_equal(ga.cpu().numpy(), ea)
    return eb, ea


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_prep_golden(path):
    z = np.load(path)
    beg, adj = _check_prep(z["pairs"], int(z["pairs"].max()) + 1)
    assert T.count_csr(beg, adj).triangles == int(z["nx_triangles"][0])


@pytest.mark.parametrize("name,pairs,tri", graphs.kat_cases(), ids=[c[0] for c in graphs.kat_cases()])
def test_prep_known_answers(name, pairs, tri):
    beg, adj = _check_prep(pairs, int(pairs.max()) + 1)
    assert T.count_csr(beg, adj).triangles == tri


def test_prep_edge_cases():
    # only self-loops: no edges, no vertices
    b, a = _check_prep(np.array([[3, 3], [5, 5]]), 10)
    assert b.tolist() == [0] and a.size == 0
    # duplicates in both directions and orphans beyond the used ids
    b, a = _check_prep(np.array([[1, 2], [2, 1], [1, 2], [2, 3], [3, 1], [7, 7]]), 100)
    assert b.size - 1 == 3 and a.size == 3
    # a single edge
    _check_prep(np.array([[0, 1]]), 2)


@pytest.mark.parametrize("scale,ef,seed", [(10, 16, 4), (14, 8, 2), (16, 16, 1)])
def test_prep_rmat(scale, ef, seed):
    """Config-1 pipeline (R-MAT scale 16, edge factor 16, seed 1) at full size on the largest case."""
    pairs = T.gen_rmat(scale, ef, seed=seed)
    eb, ea = O.build_csr(pairs.cpu().numpy(), 1 << scale)
    gb, ga = T.build_csr(pairs, 1 << scale)
    np.testing.assert_array_equal(gb.cpu().numpy(), eb)
    np.testing.assert_array_equal(ga.cpu().numpy(), ea)
    expect = O.count_forward(eb, ea, threads=8)
    assert T.count_csr(gb, ga).triangles == expect
    if O.ref_kernel_available() and O.trust_check(eb, ea)[0] == O.TRUST_EXACT:
        assert O.ref_kernel_count(eb, ea, blocks=1024, chunk=1)[0] == expect
