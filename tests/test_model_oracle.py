"""The numpy restatement of the cost model, pinned by finite differences (CPU)."""
import numpy as np

from oracle import mlp


def _random_model(rng):
    p = rng.normal(0, 0.3, mlp.FLOATS)
    p[mlp.OFF_MEAN:mlp.OFF_MEAN + 8] = rng.normal(0, 1, 8)
    p[mlp.OFF_ISCALE:mlp.OFF_ISCALE + 8] = rng.uniform(0.5, 2, 8)
    p[mlp.OFF_YMEAN] = 10.0
    p[mlp.OFF_YSCALE] = 2.0
    return p


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = _random_model(rng)
    X = rng.normal(0, 1, (64, 8))
    Y = rng.normal(10, 2, 64)
    g, _ = mlp.grad(p, X, Y)
    eps = 1e-6
    for i in list(range(mlp.OFF_W1, mlp.OFF_W1 + 20)) + list(range(mlp.OFF_W2, mlp.OFF_W2 + 40, 3)) + \
            list(range(mlp.OFF_W3, mlp.OFF_YMEAN)):
        q = p.copy()
        q[i] += eps
        lp = mlp.grad(q, X, Y)[1]
        q[i] -= 2 * eps
        lm = mlp.grad(q, X, Y)[1]
        assert abs((lp - lm) / (2 * eps) - g[i]) < 1e-5 * max(1, abs(g[i]))
    # normalisation slots are not trained
    assert np.all(g[:mlp.OFF_W1] == 0) and g[mlp.OFF_YMEAN] == 0 and g[mlp.OFF_YSCALE] == 0
