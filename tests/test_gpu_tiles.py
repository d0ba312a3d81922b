"""The one-GPU n x n tile loop (With-graph-partition/TC.cu:976-1157 as a loop over all jobs)."""
import os

import numpy as np
import pytest

import trust_gb300 as T
from oracle import oracle as O

pytestmark = pytest.mark.gpu
pytest.importorskip("torch")

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("name", ["toy", "rmat_s12", "k150", "chung_lu_3000", "er_200"])
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_tile_loop_equals_whole_graph(tmp_path, name, p):
    z = np.load(os.path.join(GOLD, name + ".npz"))
    T.partition_folder(str(tmp_path), z["ref_beg"], z["ref_adj"], p)
    r = T.count_partitioned(str(tmp_path), p)
    assert r.triangles == int(z["nx_triangles"][0])
    assert r.edges == z["ref_adj"].size and r.vertices == z["ref_beg"].size - 1


@pytest.mark.parametrize("name,p", [("rmat_s12", 2), ("rmat_s12", 3), ("k150", 2)])
def test_tile_loop_on_reference_tiles(tmp_path, name, p):
    """Tiles written by the reference's own partition binary (golden) give the same total."""
    z = np.load(os.path.join(GOLD, name + ".npz"))
    if f"part{p}_0_0_beg" not in z:
        pytest.skip("no tiles for this split in the fixture")
    for i in range(p):
        for j in range(p):
            d = tmp_path / f"partition{i}_{j}"
            d.mkdir()
            T.save_folder(str(d), z[f"part{p}_{i}_{j}_beg"], z[f"part{p}_{i}_{j}_adj"])
    assert T.count_partitioned(str(tmp_path), p).triangles == int(z["nx_triangles"][0])


def test_tile_loop_rmat16(tmp_path):
    pairs = T.gen_rmat(16, 16, seed=1)
    beg, adj = T.build_csr(pairs, 1 << 16)
    beg, adj = beg.cpu().numpy(), adj.cpu().numpy()
    expect = O.count_forward(beg, adj, threads=8)
    T.partition_folder(str(tmp_path), beg, adj, 2)
    assert T.count_partitioned(str(tmp_path), 2).triangles == expect


@pytest.mark.parametrize("name", ["toy", "rmat_s12", "k150", "chung_lu_3000", "er_200"])
@pytest.mark.parametrize("p", [1, 2, 3, 5])
def test_device_tile_loop_equals_whole_graph(name, p):
    """The GPU partition of a device CSR and the streamed tile loop give the whole count."""
    import torch
    z = np.load(os.path.join(GOLD, name + ".npz"))
    beg = torch.from_numpy(z["ref_beg"].astype(np.int64)).cuda()
    adj = torch.from_numpy(z["ref_adj"].astype(np.int32)).cuda()
    r = T.count_tiles(beg, adj, p)
    assert r.triangles == int(z["nx_triangles"][0])
    assert r.edges == adj.numel() and r.vertices == beg.numel() - 1


@pytest.mark.parametrize("p,budget", [(2, 1), (2, 0), (4, 1 << 20)])
def test_device_tile_loop_streams_under_a_budget(p, budget):
    """A budget smaller than one job's three tiles evicts on every job: same count as in HBM."""
    pairs = T.gen_rmat(17, 16, seed=4)
    beg, adj = T.build_csr(pairs, 1 << 17)
    whole = T.count_csr(beg, adj)
    r = T.count_tiles(beg, adj, p, budget_bytes=budget)
    assert r.triangles == whole.triangles


def test_device_tile_loop_rejects_bad_ids():
    import torch
    beg = torch.tensor([0, 2, 3, 3], dtype=torch.int64, device="cuda")
    adj = torch.tensor([1, 7, 2], dtype=torch.int32, device="cuda")
    with pytest.raises(T.TrustTcError) as e:
        T.count_tiles(beg, adj, 2)
    assert e.value.status == T._lib.E_IDS


def _sorted_csr(kind):
    """A GPU-built oriented CSR (strictly increasing rows) and its oracle count."""
    if kind == "rmat13":
        pairs, bound = T.gen_rmat(13, 16, 0.7, 0.125, 0.125, seed=4), 1 << 13
    elif kind == "rmat12":
        pairs, bound = T.gen_rmat(12, 16, seed=1), 1 << 12
    else:
        pairs, bound = T.gen_chung_lu(20_000, 2.1, 400.0, 120_000, 120_000, seed=3), 20_000
    beg, adj = T.build_csr(pairs, bound)
    return beg, adj, O.count_forward(beg.cpu().numpy(), adj.cpu().numpy(), threads=8)


@pytest.mark.parametrize("kind", ["rmat13", "rmat12", "chung_lu"])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_tile_loop_direction_split(kind, p):
    """Every tile job counted with the direction split (tables from the probe tile's rows where
    those are longer) gives the whole count, as does the loop without it; the split runs."""
    beg, adj, expect = _sorted_csr(kind)
    on = T.count_tiles(beg, adj, p, direction_split=1)
    off = T.count_tiles(beg, adj, p, direction_split=0)
    assert on.triangles == expect and off.triangles == expect
    assert on.direction_split >= 1 and off.direction_split == 0
    assert on.wedges < off.wedges  # fewer probes, same count


def test_tile_loop_direction_split_streamed():
    """The split with tiles streamed through a small device budget (evictions between jobs)."""
    beg, adj, expect = _sorted_csr("rmat13")
    tile_bytes = 8 * beg.numel() + 4 * adj.numel()
    r = T.count_tiles(beg, adj, 4, budget_bytes=tile_bytes // 5, direction_split=1)
    assert r.triangles == expect and r.direction_split >= 1


@pytest.mark.parametrize("name,p", [("rmat_s12", 2), ("k150", 2)])
def test_tile_split_refused_on_unsorted_tiles(tmp_path, name, p):
    """The reference's own tiles keep its unsorted rows: the split is not applied to a job
    whose tiles are not known duplicate-free, and the count stays exact."""
    z = np.load(os.path.join(GOLD, name + ".npz"))
    if f"part{p}_0_0_beg" not in z:
        pytest.skip("no tiles for this split in the fixture")
    for i in range(p):
        for j in range(p):
            d = tmp_path / f"partition{i}_{j}"
            d.mkdir()
            T.save_folder(str(d), z[f"part{p}_{i}_{j}_beg"], z[f"part{p}_{i}_{j}_adj"])
    r = T.count_partitioned(str(tmp_path), p, direction_split=1)
    assert r.triangles == int(z["nx_triangles"][0])
    unsorted = any(np.any(np.diff(z[f"part{p}_{i}_{j}_adj"][b0:b1]) <= 0)
                   for i in range(p) for j in range(p)
                   for b0, b1 in zip(z[f"part{p}_{i}_{j}_beg"][:-1], z[f"part{p}_{i}_{j}_beg"][1:]))
    if unsorted:
        assert r.direction_split < p ** 3


def test_partitioned_folder_direction_split(tmp_path):
    """The folder tile loop over sorted tiles (written by partition_folder) with the split."""
    beg, adj, expect = _sorted_csr("rmat13")
    b, a = beg.cpu().numpy(), adj.cpu().numpy()
    T.partition_folder(str(tmp_path), b, a, 3)
    r = T.count_partitioned(str(tmp_path), 3, direction_split=1)
    assert r.triangles == expect and r.direction_split >= 1
