"""Parity of the sm_103a counting path with the oracle (bit-exact u64 counts).

Inputs: the golden CSRs produced by the reference preprocess (unsorted rows, class layout),
known-answer graphs, arbitrary CSRs with duplicates and self-loops (the counted quantity of
include/trust_tc.h), and every schedule class forced through small thresholds.  Where the
reference kernel itself (Without-graph-partition/TC.cu rebuilt for sm_103a) is available it is
run on the same certified inputs and must agree too.
"""
import glob
import os

import numpy as np
import pytest

import trust_gb300 as T
from trust_gb300 import _lib
from oracle import oracle as O
from tests import graphs

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def _dev(beg, adj):
    return (torch.from_numpy(np.ascontiguousarray(beg, dtype=np.int64)).cuda(),
            torch.from_numpy(np.ascontiguousarray(adj, dtype=np.int32)).cuda())


@pytest.fixture(scope="module")
def ctx():
    with T.Context() as c:
        yield c


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_golden_host_and_device(ctx, path):
    z = np.load(path)
    expect = int(z["nx_triangles"][0])
    beg, adj = z["ref_beg"], z["ref_adj"]
    assert T.count_csr(beg, adj).triangles == expect
    assert T.count_csr(beg, adj, ctx=ctx).triangles == expect
    db, da = _dev(beg, adj)
    r = T.count_csr(db, da, ctx=ctx)
    assert r.triangles == expect
    assert r.vertices == beg.size - 1 and r.edges == adj.size
    assert r.max_out_degree == int(np.diff(beg).max())
    assert r.wedges == O.wedges(beg, adj)
    if "fast_beg" in z:
        assert T.count_csr(z["fast_beg"], z["fast_adj"], ctx=ctx).triangles == expect


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_reference_kernel_agrees(path):
    if not O.ref_kernel_available():
        pytest.skip("reference kernel cubin not built here (oracle/build_ref.sh needs the reference sources)")
    z = np.load(path)
    beg, adj = z["ref_beg"], z["ref_adj"]
    assert O.trust_check(beg, adj)[0] == O.TRUST_EXACT
    ref, _ = O.ref_kernel_count(beg, adj, blocks=64, chunk=1)
    assert ref == int(z["nx_triangles"][0]) == T.count_csr(beg, adj).triangles


# (warp_max, block_max) pairs that push vertices through every class: g4..g32, warp, CTA, huge
THRESHOLDS = [(128, 4096), (32, 32), (32, 64), (64, 128), (100, 100), (256, 8192)]


@pytest.mark.parametrize("wm,bm", THRESHOLDS)
@pytest.mark.parametrize("name", ["k150", "rmat_s12", "chung_lu_3000", "k60"])
def test_every_class_path(ctx, name, wm, bm):
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    db, da = _dev(z["ref_beg"], z["ref_adj"])
    r = T.count_csr(db, da, ctx=ctx, warp_max=wm, block_max=bm)
    assert r.triangles == int(z["nx_triangles"][0])
    d = np.diff(z["ref_beg"])
    cta_max = 1 << max((2 * bm - 1).bit_length() - 1, 5)  # table of the next power of two >= 2*bm
    assert r.class_sizes["huge"] == int(np.sum(d > cta_max))
    assert r.class_sizes["skip"] == int(np.sum(d < 2))


@pytest.mark.parametrize("hub_cluster", [-1, 0, 1, 2, 4, 8])
@pytest.mark.parametrize("name,bm", [("k150", 32), ("rmat_s12", 32), ("rmat_s12", 64), ("k60", 32)])
def test_hub_rows_on_clusters(ctx, name, bm, hub_cluster):
    """Rows above the CTA table counted in shared memory (one CTA or a thread-block cluster
    whose CTAs share the table), or on per-CTA global tables (-1): the same count."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    db, da = _dev(z["ref_beg"], z["ref_adj"])
    r = T.count_csr(db, da, ctx=ctx, warp_max=32, block_max=bm, hub_cluster=hub_cluster)
    assert r.triangles == int(z["nx_triangles"][0])
    assert r.class_sizes["huge"] > 0


@pytest.mark.parametrize("hub_cluster", [0, 1, 2, 4, 8, -1])
def test_hub_row_larger_than_one_cta(ctx, hub_cluster):
    """One row of 20,000 entries (a 65,536-slot table, 256 KiB: more than one CTA's shared
    memory): the default spreads it over a 4-CTA cluster; a cluster too small for it falls back
    to the global table.  Row 0 = 1..D, row i = {i+1}: the count is D - 1."""
    D = 20_000
    beg = np.concatenate([[0], D + np.arange(0, D + 1)]).astype(np.int64)
    adj = np.concatenate([np.arange(1, D + 1), np.arange(2, D + 2)]).astype(np.int32)
    adj[-1] = 0  # row D points back to 0 (keeps ids in range)
    expect = O.count_forward(beg, adj)
    assert expect == D - 1
    r = T.count_csr(*_dev(beg, adj), ctx=ctx, hub_cluster=hub_cluster)
    assert r.triangles == expect and r.class_sizes["huge"] == 1


def test_hub_row_unaligned_neighbour_array(ctx):
    """Hub rows are staged into shared memory by TMA bulk copies of their 16-byte aligned interior;
    a neighbour array that is not 16-byte aligned (a view one element in) is read directly."""
    import torch
    D = 20_000
    beg = np.concatenate([[0], D + np.arange(0, D + 1)]).astype(np.int64)
    adj = np.concatenate([np.arange(1, D + 1), np.arange(2, D + 2)]).astype(np.int32)
    adj[-1] = 0
    db = torch.from_numpy(beg).cuda()
    big = torch.zeros(adj.size + 1, dtype=torch.int32, device="cuda")
    big[1:] = torch.from_numpy(adj).cuda()
    for hc in (0, 1, 4):
        assert T.count_csr(db, big[1:], ctx=ctx, hub_cluster=hc).triangles == D - 1
        assert T.count_csr(db, big[1:].clone(), ctx=ctx, hub_cluster=hc).triangles == D - 1


def test_autotune(ctx):
    """The autotuner returns valid launch parameters; they change the schedule, never the count."""
    pairs = T.gen_rmat(16, 16, seed=1)
    beg, adj = T.build_csr(pairs, 1 << 16)
    expect = T.count_csr(beg, adj, ctx=ctx).triangles
    cfg, ms = T.autotune(beg, adj, ctx, repeats=2)
    assert ms > 0 and cfg["threads"] in (0, 128, 256, 512, 1024) and cfg["chunk"] in (0, 4, 8, 16)
    assert cfg["schedule"] in (T.SCHED_LEARNED, T.SCHED_TUNED, T.SCHED_PLAIN)
    assert T.count_csr(beg, adj, ctx=ctx, **cfg).triangles == expect
    # a budget spent by the first (base) measurement: no other candidate starts
    cfg0, ms0 = T.autotune(beg, adj, ctx, repeats=1, time_budget_s=1e-9)
    assert ms0 > 0 and cfg0 == {"threads": 0, "warp_max": 0, "chunk": 0, "hub_cluster": 0,
                                "schedule": T.SCHED_LEARNED}
    # a graph with a row above the CTA table: the hub cluster size is tuned too
    import torch
    D = 20_000
    hb = torch.from_numpy(np.concatenate([[0], D + np.arange(0, D + 1)]).astype(np.int64)).cuda()
    ha = np.concatenate([np.arange(1, D + 1), np.arange(2, D + 2)]).astype(np.int32)
    ha[-1] = 0
    ha = torch.from_numpy(ha).cuda()
    cfg, ms = T.autotune(hb, ha, ctx, repeats=1)
    assert cfg["hub_cluster"] in (0, 1, 2, 4, -1)
    assert T.count_csr(hb, ha, ctx=ctx, **cfg).triangles == D - 1


def test_hub_rows_on_clusters_split_and_record(ctx):
    """Hub rows in shared memory in both passes of the direction split and with cycle recording."""
    import torch
    pairs = T.gen_rmat(16, 16, seed=1)
    beg, adj = T.build_csr(pairs, 1 << 16)
    expect = T.count_csr(beg, adj, ctx=ctx, hub_cluster=-1, warp_max=32, block_max=64).triangles
    for hc in (0, 2, 8):
        r = T.count_csr(beg, adj, ctx=ctx, warp_max=32, block_max=64, hub_cluster=hc, direction_split=1)
        assert r.triangles == expect and r.direction_split
        cyc = torch.zeros(beg.numel() - 1, dtype=torch.int64, device="cuda")
        r = T.count_csr(beg, adj, ctx=ctx, warp_max=32, block_max=64, hub_cluster=hc, direction_split=0, cycles=cyc)
        assert r.triangles == expect
        d = np.diff(beg.cpu().numpy())
        assert np.all(cyc.cpu().numpy()[d > 128] > 0)  # hub rows recorded too
    with pytest.raises(T.TrustTcError):
        T.count_csr(beg, adj, ctx=ctx, warp_max=32, block_max=64, hub_cluster=3)


@pytest.mark.parametrize("threads", [64, 128, 256, 512, 1024])
@pytest.mark.parametrize("blocks,chunk", [(0, 0), (1, 1), (7, 3), (300, 16)])
def test_launch_shapes(ctx, threads, blocks, chunk):
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "rmat_s12.npz"))
    db, da = _dev(z["ref_beg"], z["ref_adj"])
    r = T.count_csr(db, da, ctx=ctx, threads=threads, blocks=blocks, chunk=chunk, warp_max=64, block_max=256)
    assert r.triangles == int(z["nx_triangles"][0])


@pytest.mark.parametrize("name,pairs,tri", graphs.kat_cases(), ids=[c[0] for c in graphs.kat_cases()])
def test_known_answers(ctx, name, pairs, tri):
    beg, adj = O.build_csr(pairs, int(pairs.max()) + 1)
    assert T.count_csr(beg, adj, ctx=ctx).triangles == tri
    assert T.count_csr(beg, adj, ctx=ctx, warp_max=32, block_max=32).triangles == tri


def test_arbitrary_csr_formula(ctx):
    """Unsorted rows, duplicate arcs, self-loops: the counted quantity, not just triangles."""
    rng = np.random.default_rng(1)
    for trial in range(40):
        n = int(rng.integers(1, 400))
        beg, adj = graphs.random_csr(rng, n, int(rng.integers(0, 40)))
        expect = O.count_forward(beg, adj)
        db, da = _dev(beg, adj)
        for wm, bm in ((128, 4096), (32, 32)):
            assert T.count_csr(db, da, ctx=ctx, warp_max=wm, block_max=bm).triangles == expect


def test_edge_cases(ctx):
    assert T.count_csr(np.array([0]), np.array([], dtype=np.int32), ctx=ctx).triangles == 0
    assert T.count_csr(np.array([0, 0]), np.array([], dtype=np.int32), ctx=ctx).triangles == 0
    # every out-degree < 2
    beg = np.array([0, 1, 2, 2], dtype=np.int64)
    adj = np.array([1, 2], dtype=np.int32)
    assert T.count_csr(beg, adj, ctx=ctx).triangles == 0
    # a single vertex with a self-loop twice: row {0, 0}; d=2 -> each arc probes row 0 (2 entries, both hit)
    assert T.count_csr(np.array([0, 2]), np.array([0, 0], dtype=np.int32), ctx=ctx).triangles == 4
    db, da = _dev(np.array([0]), np.zeros(0, dtype=np.int32))
    assert T.count_csr(db, da, ctx=ctx).triangles == 0


def test_host_input_validation_errors(ctx):
    beg = np.array([0, 2, 3, 3], dtype=np.int64)
    for adj, code in (([1, 7, 2], _lib.E_IDS), ([1, -1, 2], _lib.E_IDS)):
        with pytest.raises(T.TrustTcError) as e:
            T.count_csr(beg, np.array(adj, dtype=np.int32), ctx=ctx)
        assert e.value.status == code
    for b in ([0, 2, 1, 3], [1, 2, 3, 3], [0, 2, 3, 4]):
        with pytest.raises(T.TrustTcError) as e:
            T.count_csr(np.array(b), np.array([1, 2, 2], dtype=np.int32), ctx=ctx)
        assert e.value.status == _lib.E_OFFSETS


@pytest.mark.parametrize("shift", [0, 1, 2, 3])
def test_id_check_every_position_and_alignment(ctx, shift):
    """The id check reads 16-byte words between scalar head and tail entries: a bad id is found
    wherever it sits, whatever the alignment of the neighbour array (a view at an offset)."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "rmat_s12.npz"))
    beg = np.asarray(z["ref_beg"], dtype=np.int64)
    adj = np.asarray(z["ref_adj"], dtype=np.int32)
    m, n = adj.size, beg.size - 1
    expect = int(z["nx_triangles"][0])
    big = torch.zeros(m + 8, dtype=torch.int32, device="cuda")
    db = torch.from_numpy(beg).cuda()
    for pos in sorted({0, 1, 2, 3, 4, 5, m // 2, m - 4, m - 3, m - 2, m - 1}):
        for bad in (n, -1):
            a = adj.copy()
            a[pos] = bad
            big[shift:shift + m] = torch.from_numpy(a).cuda()
            with pytest.raises(T.TrustTcError) as e:
                T.count_csr(db, big[shift:shift + m], ctx=ctx)
            assert e.value.status == _lib.E_IDS, (pos, bad)
    big[shift:shift + m] = torch.from_numpy(adj).cuda()
    assert T.count_csr(db, big[shift:shift + m], ctx=ctx).triangles == expect


def test_id_check_few_rows_many_arcs(ctx):
    """64 rows of 20,000 entries each (a multigraph): the id check still covers every entry,
    wherever the bad one sits, and the valid input counts like the oracle's brute force on a
    slice-equivalent small copy."""
    rng = np.random.default_rng(5)
    n, d = 64, 20_000
    beg = np.arange(0, n * d + 1, d, dtype=np.int64)
    adj = rng.integers(0, n, size=n * d, dtype=np.int32)
    db = torch.from_numpy(beg).cuda()
    for pos in (0, 7, n * d // 3, n * d - 1):
        a = adj.copy()
        a[pos] = n
        with pytest.raises(T.TrustTcError) as e:
            T.count_csr(db, torch.from_numpy(a).cuda(), ctx=ctx)
        assert e.value.status == _lib.E_IDS, pos
    # the counted quantity on rows with duplicates: every row holds all 64 ids many times, so each
    # probe hits; count = sum over v of sum over u in row v of d(u) = n * d * d
    r = T.count_csr(db, torch.from_numpy(adj).cuda(), ctx=ctx, direction_split=0)
    present = [len(np.unique(adj[beg[v]:beg[v + 1]])) == n for v in range(n)]
    if all(present):
        assert r.triangles == n * d * d


def test_device_validation_errors(ctx):
    db, da = _dev(np.array([0, 2, 3, 3]), np.array([1, 3, 2]))
    with pytest.raises(T.TrustTcError) as e:
        T.count_csr(db, da, ctx=ctx)
    assert e.value.status == _lib.E_IDS
    db, da = _dev(np.array([0, 2, 1, 3]), np.array([1, 2, 2]))
    with pytest.raises(T.TrustTcError) as e:
        T.count_csr(db, da, ctx=ctx)
    assert e.value.status == _lib.E_OFFSETS
    db, da = _dev(np.array([0, 2, 3, 4]), np.array([1, 2, 2]))
    with pytest.raises(T.TrustTcError) as e:
        T.count_csr(db, da, ctx=ctx)
    assert e.value.status == _lib.E_OFFSETS
    # the context is still usable afterwards
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "k60.npz"))
    assert T.count_csr(*_dev(z["ref_beg"], z["ref_adj"]), ctx=ctx).triangles == int(z["nx_triangles"][0])


def test_stream_and_context_reuse(ctx):
    s = torch.cuda.Stream()
    zs = [np.load(p) for p in GOLDEN]
    with torch.cuda.stream(s):
        for z in zs + zs[::-1]:
            db, da = _dev(z["ref_beg"], z["ref_adj"])
            r = T.count_csr(db, da, ctx=ctx, stream=s.cuda_stream)
            assert r.triangles == int(z["nx_triangles"][0])
            assert 0 < r.count_seconds <= r.kernel_seconds <= r.call_seconds


def test_relabelled_input(ctx):
    """Count is invariant under a random vertex relabelling with shuffled rows (no class layout)."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "rmat_s12.npz"))
    beg, adj = z["ref_beg"], z["ref_adj"]
    n = beg.size - 1
    rng = np.random.default_rng(5)
    perm = rng.permutation(n).astype(np.int32)
    rows = [perm[adj[beg[v]:beg[v + 1]]] for v in range(n)]
    new_rows = [None] * n
    for v in range(n):
        r = rows[v].copy()
        rng.shuffle(r)
        new_rows[perm[v]] = r
    nb = np.zeros(n + 1, dtype=np.int64)
    nb[1:] = np.cumsum([len(r) for r in new_rows])
    na = np.concatenate(new_rows).astype(np.int32)
    assert T.count_csr(nb, na, ctx=ctx).triangles == int(z["nx_triangles"][0])


@pytest.mark.parametrize("schedule", [T.SCHED_PLAIN, T.SCHED_TUNED])
@pytest.mark.parametrize("name", ["k150", "rmat_s12", "chung_lu_3000", "er_200"])
def test_schedules_agree(ctx, name, schedule):
    """The schedule changes only which lanes do the work, never the count."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    db, da = _dev(z["ref_beg"], z["ref_adj"])
    r = T.count_csr(db, da, ctx=ctx, schedule=schedule)
    assert r.triangles == int(z["nx_triangles"][0])
    d = np.diff(z["ref_beg"])
    if schedule == T.SCHED_PLAIN:  # the reference's split: warp for 2..100, CTA above
        assert r.class_sizes["g4"] == r.class_sizes["g8"] == r.class_sizes["g16"] == r.class_sizes["g32"] == 0
        assert r.class_sizes["warp"] == int(np.sum((d >= 2) & (d <= 100)))
        assert r.class_sizes["cta"] + r.class_sizes["huge"] == int(np.sum(d > 100))


def test_cycle_recording(ctx):
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "rmat_s12.npz"))
    db, da = _dev(z["ref_beg"], z["ref_adj"])
    n = db.numel() - 1
    for schedule in (T.SCHED_PLAIN, T.SCHED_TUNED):
        cyc = torch.full((n,), -1, dtype=torch.int64, device="cuda")
        r = T.count_csr(db, da, ctx=ctx, cycles=cyc, schedule=schedule, warp_max=64, block_max=256)
        assert r.triangles == int(z["nx_triangles"][0])
        c = cyc.cpu().numpy()
        d = np.diff(z["ref_beg"])
        assert np.all(c[d < 2] == 0)
        assert np.all(c[d >= 2] > 0)


@pytest.mark.parametrize("name", ["k150", "rmat_s12", "chung_lu_3000", "er_200", "k60", "rmat_s9"])
def test_direction_split(ctx, name):
    """Charging arcs with d(u) > d(v) to u's side changes which row is hashed, not the count."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    expect = int(z["nx_triangles"][0])
    beg, adj = O.build_csr(z["pairs"], int(z["pairs"].max()) + 1)  # sorted, duplicate-free rows
    db, da = _dev(beg, adj)
    for schedule in (T.SCHED_TUNED, T.SCHED_PLAIN, T.SCHED_LEARNED):
        r = T.count_csr(db, da, ctx=ctx, schedule=schedule, direction_split=1)
        assert r.triangles == expect
        assert r.direction_split
        d = np.diff(beg)
        src = np.repeat(np.arange(d.size), d)
        sel = d[src] >= 2
        assert r.wedges == int(np.minimum(d[adj], d[src])[sel].sum())  # probes of the split plan
    # unsorted rows (the reference preprocess output): the split is not applied, count unchanged
    r = T.count_csr(*_dev(z["ref_beg"], z["ref_adj"]), ctx=ctx, direction_split=1)
    assert r.triangles == expect
    assert not r.direction_split
    assert r.wedges == O.wedges(z["ref_beg"], z["ref_adj"])


def test_learned_schedule_on_rmat(ctx):
    pairs = T.gen_rmat(16, 16, seed=1)
    beg, adj = T.build_csr(pairs, 1 << 16)
    b, a = beg.cpu().numpy(), adj.cpu().numpy()
    expect = O.count_forward(b, a, threads=8)
    for schedule in (T.SCHED_LEARNED, T.SCHED_TUNED, T.SCHED_PLAIN):
        for split in (-1, 0, 1):
            assert T.count_csr(beg, adj, ctx=ctx, schedule=schedule, direction_split=split).triangles == expect


def test_bounded_wait_runs_out_safely(ctx):
    """Failure detection without a fault: the hub kernel's copy barrier is armed with no copy
    issued (opts.test_wait_expiry), so its bounded wait (a few thousand cycles) runs out with
    nothing in flight.  The call reports TRUST_TC_E_DEVICE, the kernel's plain-load fallback still
    gives the exact count, and the next normal call on the same context is unaffected."""
    import ctypes as C
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "k150.npz"))
    expect = int(z["nx_triangles"][0])
    db, da = _dev(z["ref_beg"], z["ref_adj"])
    o = T._opts(ptr_kind=T.DEVICE, warp_max=32, block_max=64)  # rows above 64 entries: hub kernel
    o.test_wait_expiry = 1
    r = _lib.Result()
    rc = T.load().trust_tc_count_csr(ctx.handle, C.c_void_p(db.data_ptr()), C.c_void_p(da.data_ptr()),
                                     db.numel() - 1, da.numel(), C.byref(o), C.byref(r))
    assert rc == _lib.E_DEVICE
    assert r.triangles == expect and r.class_sizes[7] > 0
    again = T.count_csr(db, da, ctx=ctx, warp_max=32, block_max=64)
    assert again.triangles == expect


def test_row_range_slices(ctx):
    """Source-row slices (opts.row_begin/row_end) count exactly the oracle's rows and sum to the
    whole count under every schedule; bad ranges are refused."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "rmat_s12.npz"))
    pairs = T.gen_rmat(14, 16, seed=4)
    beg, adj = T.build_csr(pairs, 1 << 14)
    hb, ha = beg.cpu().numpy(), adj.cpu().numpy()
    n = hb.size - 1
    cuts = [0, 1, 7, 100, 1000, n // 2, n]
    for sch, split in ((T.SCHED_LEARNED, -1), (T.SCHED_LEARNED, 1), (T.SCHED_TUNED, 0), (T.SCHED_PLAIN, 0)):
        total = 0
        for lo, hi in zip(cuts[:-1], cuts[1:]):
            r = T.count_csr(beg, adj, ctx=ctx, schedule=sch, direction_split=split, row_range=(lo, hi))
            assert r.triangles == O.count_forward_sorted_range(hb, ha, lo, hi, 2, 4), (sch, split, lo, hi)
            total += r.triangles
        assert total == T.count_csr(beg, adj, ctx=ctx, schedule=sch).triangles
    # host input and an empty range
    assert T.count_csr(hb, ha, ctx=ctx, row_range=(5, 5)).triangles == 0
    # a range on the unsorted golden rows (no split possible) with forced hub rows
    zb, za = _dev(z["ref_beg"], z["ref_adj"])
    m = z["ref_beg"].size - 1
    r = T.count_csr(zb, za, ctx=ctx, warp_max=32, block_max=64, row_range=(0, m // 3))
    assert r.triangles == O.count_forward_sorted_range(z["ref_beg"], np.concatenate(
        [np.sort(z["ref_adj"][z["ref_beg"][v]:z["ref_beg"][v + 1]]) for v in range(m)]).astype(np.int32), 0, m // 3, 2, 1)
    for bad in ((-1, 5), (6, 5), (0, n + 1)):
        with pytest.raises(T.TrustTcError):
            T.count_csr(beg, adj, ctx=ctx, row_range=bad)


def test_small_skewed_graphs_take_the_plain_split(ctx):
    """Under the default schedule a graph of fewer than 2^21 arcs with a row of at least 64 entries
    is counted with the plain split (one warp per row up to 100 entries, a CTA above), which is
    faster there; a small graph without long rows keeps the sub-warp classes.  Counts never change."""
    pairs = T.gen_rmat(16, 16, seed=1)
    beg, adj = T.build_csr(pairs, 1 << 16)
    d = np.diff(beg.cpu().numpy())
    default = T.count_csr(beg, adj, ctx=ctx)
    plain = T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_PLAIN)
    assert default.triangles == plain.triangles
    assert default.class_sizes == plain.class_sizes
    assert default.class_sizes["warp"] == int(np.sum((d >= 2) & (d <= 100)))
    tuned = T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_TUNED)
    assert tuned.triangles == default.triangles and tuned.class_sizes["g4"] > 0
    pairs = T.gen_chung_lu(200_000, 2.5, 300.0, 800_000, 800_000, seed=11)
    beg, adj = T.build_csr(pairs, 200_000)
    assert int((beg[1:] - beg[:-1]).max()) < 64
    default = T.count_csr(beg, adj, ctx=ctx)
    assert default.class_sizes == T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_TUNED).class_sizes
