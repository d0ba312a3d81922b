"""The learned schedule's cost model on the GPU: CUDA gradients against the numpy oracle, training,
inference, and that the schedule it drives changes only the schedule (counts stay exact)."""
import os

import numpy as np
import pytest

import trust_gb300 as T
from oracle import mlp
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _data(rng, n):
    X = rng.normal(0, 1, (n, 8)).astype(np.float32)
    Y = (10 + X[:, 0] * 2 - np.abs(X[:, 1]) + 0.5 * X[:, 2] * X[:, 3]).astype(np.float32)
    return X, Y


def test_cuda_gradient_matches_oracle():
    rng = np.random.default_rng(1)
    X, Y = _data(rng, 3000)
    p = T.model_init(seed=7)
    p[mlp.OFF_MEAN:mlp.OFF_MEAN + 8] = X.mean(0)
    p[mlp.OFF_ISCALE:mlp.OFF_ISCALE + 8] = 1 / X.std(0)
    p[mlp.OFF_YMEAN], p[mlp.OFF_YSCALE] = Y.mean(), Y.std()
    g, loss = T.model_grad(torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda(), p)
    g_ref, loss_ref = mlp.grad(p, X, Y)
    assert abs(loss - loss_ref) <= 1e-4 * max(1, loss_ref)
    scale = np.abs(g_ref).max()
    np.testing.assert_allclose(g, g_ref, rtol=1e-3, atol=1e-5 * scale)  # fp32 vs fp64


def test_training_and_prediction():
    rng = np.random.default_rng(2)
    X, Y = _data(rng, 20000)
    dx, dy = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    p0 = T.model_init(seed=3)
    p1, loss = T.model_train(dx, dy, p0, epochs=60, batch=1024, lr=3e-3)
    assert loss < 0.1  # normalised units: the target's variance is 1
    pred = T.model_predict(dx, p1).cpu().numpy()
    np.testing.assert_allclose(pred, mlp.predict(p1, X), rtol=1e-4, atol=1e-3)
    assert np.sqrt(np.mean((pred - Y) ** 2)) < 0.35 * Y.std()


def test_vertex_features():
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "rmat_s12.npz"))
    beg, adj = O.build_csr(z["pairs"], 4096)
    with T.Context() as ctx:
        f = T.vertex_features(torch.from_numpy(beg).cuda(), torch.from_numpy(adj).cuda(), ctx).cpu().numpy()
    d = np.diff(beg)
    src = np.repeat(np.arange(d.size), d)
    W = np.bincount(src, weights=d[adj], minlength=d.size)
    Wmin = np.bincount(src, weights=np.minimum(d[adj], d[src]), minlength=d.size)
    act = d >= 2
    np.testing.assert_allclose(f[act, 0], np.log2(1 + d[act]), rtol=1e-5)
    np.testing.assert_allclose(f[act, 1], np.log2(1 + W[act]), rtol=1e-5)
    np.testing.assert_allclose(f[act, 2], np.log2(1 + Wmin[act]), rtol=1e-5)
    assert np.all(f[~act] == 0)


@pytest.mark.parametrize("seed", [1, 2])
def test_learned_schedule_exact_with_any_model(seed):
    """Promotions, queue order and the split come from the model; counts must not move."""
    pairs = T.gen_rmat(15, 16, seed=seed)
    beg, adj = T.build_csr(pairs, 1 << 15)
    b, a = beg.cpu().numpy(), adj.cpu().numpy()
    expect = O.count_forward(b, a, threads=8)
    def constant_model(log2_cycles):  # zero weights: every row predicted at 2^log2_cycles cycles
        m = np.zeros(mlp.FLOATS, dtype=np.float32)
        m[mlp.OFF_ISCALE:mlp.OFF_ISCALE + 8] = 1.0
        m[mlp.OFF_YMEAN], m[mlp.OFF_YSCALE] = log2_cycles, 1.0
        return m

    models = [T.model_init(seed=seed), constant_model(27.0), constant_model(0.0)]
    d = T.model_default()
    if d is not None:
        models.append(d)
    with T.Context() as ctx:
        for mod in models:
            for split in (-1, 0, 1):
                r = T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_LEARNED, model=mod, direction_split=split)
                assert r.triangles == expect
        deg = np.diff(b)
        # (a graph this small only gets the scheduling pass when the split is forced)
        # predicted 2^27 cycles (above the 2^26 promotion bound): every warp-class row promoted to a CTA
        r = T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_LEARNED, model=models[1], direction_split=1)
        assert r.class_sizes["warp"] == 0 and r.class_sizes["cta"] == int(np.sum((deg > 32) & (deg <= 4096)))
        # predicted 1 cycle: the tuned classes stay
        r = T.count_csr(beg, adj, ctx=ctx, schedule=T.SCHED_LEARNED, model=models[2], direction_split=1)
        assert r.class_sizes["warp"] == int(np.sum((deg > 32) & (deg <= 512)))


def _median_call(beg, adj, ctx, reps=5, **kw):
    import statistics
    ts, r = [], None
    for _ in range(reps):
        r = T.count_csr(beg, adj, ctx=ctx, **kw)
        ts.append(r.call_seconds)
    return statistics.median(ts), r


@pytest.mark.parametrize("scale,ef,a,seed", [(20, 16, 0.57, 3), (24, 16, 0.70, 3)])
def test_learned_schedule_gain_on_skewed_rmat(scale, ef, a, seed):
    """What the trained network buys on a skewed graph (R-MAT 20, and the held-out R-MAT 24 with
    a = 0.70), against three arms: (a) the plain degree-threshold schedule; (b) the same learned
    schedule with a network that predicts nothing (all weights zero: every row at 1 cycle, so no
    predicted saving and no direction split); (c) the gate alone: the tuned classes with the
    split taken whenever the rows allow it, no network.  Same count every time.  Measured on GB300
    (call ms): R-MAT 20 learned 5.66, gate-only 5.91, plain 10.2; R-MAT 24 a = 0.70 learned 169.6
    (promotions off), gate-only 169.4, plain 334.  The network turns the split on where the gate
    would; against the gate alone it is equal within noise on the large graph (asserted: no worse
    than 5 %), and faster on R-MAT 20."""
    b_ = (1.0 - a - 0.05) / 2
    pairs = T.gen_rmat(scale, ef, a, b_, b_, seed=seed)
    beg, adj = T.build_csr(pairs, 1 << scale)
    del pairs
    blind = np.zeros(mlp.FLOATS, dtype=np.float32)
    blind[mlp.OFF_ISCALE:mlp.OFF_ISCALE + 8] = 1.0
    blind[mlp.OFF_YSCALE] = 1.0
    with T.Context() as ctx:
        t_plain, r_plain = _median_call(beg, adj, ctx, schedule=T.SCHED_PLAIN)
        t_learned, r_learned = _median_call(beg, adj, ctx)
        t_blind, r_blind = _median_call(beg, adj, ctx, model=blind)
        t_gate, r_gate = _median_call(beg, adj, ctx, schedule=T.SCHED_TUNED, direction_split=1)
    assert r_learned.triangles == r_plain.triangles == r_blind.triangles == r_gate.triangles
    assert r_learned.direction_split and r_learned.split_saving_ms > 1.0
    assert not r_blind.direction_split and r_blind.split_saving_ms < 0.01
    assert r_gate.direction_split
    assert t_learned < 0.85 * t_plain, (t_learned, t_plain)
    assert t_learned < 0.95 * t_blind, (t_learned, t_blind)
    assert t_learned <= 1.05 * t_gate, (t_learned, t_gate)
