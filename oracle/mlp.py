"""numpy restatement of the cost model (8 -> 32 -> 32 -> 1 MLP, ReLU, MSE).  TEST INFRASTRUCTURE ONLY:
the checker for the library's CUDA forward/backward kernels (same parameter layout as
trust_gb300/csrc/tc_model.h)."""
import numpy as np

F, H = 8, 32
OFF_MEAN, OFF_ISCALE = 0, 8
OFF_W1 = 16
OFF_B1 = OFF_W1 + H * F
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
OFF_YMEAN = OFF_B3 + 1
OFF_YSCALE = OFF_YMEAN + 1
FLOATS = OFF_YSCALE + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return dict(mean=p[OFF_MEAN:OFF_MEAN + F], iscale=p[OFF_ISCALE:OFF_ISCALE + F],
                W1=p[OFF_W1:OFF_B1].reshape(H, F), b1=p[OFF_B1:OFF_W2], W2=p[OFF_W2:OFF_B2].reshape(H, H),
                b2=p[OFF_B2:OFF_W3], w3=p[OFF_W3:OFF_B3], b3=p[OFF_B3], ymean=p[OFF_YMEAN], yscale=p[OFF_YSCALE])


def forward(p, X):
    q = unpack(p)
    x = (np.asarray(X, dtype=np.float64) - q["mean"]) * q["iscale"]
    a1 = x @ q["W1"].T + q["b1"]
    h1 = np.maximum(a1, 0)
    a2 = h1 @ q["W2"].T + q["b2"]
    h2 = np.maximum(a2, 0)
    y = h2 @ q["w3"] + q["b3"]
    return y, (x, a1, h1, a2, h2)


def predict(p, X):
    q = unpack(p)
    return forward(p, X)[0] * q["yscale"] + q["ymean"]


def grad(p, X, Y):
    """Gradient of mean((y - t)^2) in normalised target units, same layout as the model."""
    q = unpack(p)
    y, (x, a1, h1, a2, h2) = forward(p, X)
    t = (np.asarray(Y, dtype=np.float64) - q["ymean"]) / q["yscale"]
    n = len(t)
    dy = 2 * (y - t) / n
    g = np.zeros(FLOATS)
    g[OFF_B3] = dy.sum()
    g[OFF_W3:OFF_B3] = dy @ h2
    dh2 = np.outer(dy, q["w3"]) * (a2 > 0)
    g[OFF_B2:OFF_W3] = dh2.sum(0)
    g[OFF_W2:OFF_B2] = (dh2.T @ h1).ravel()
    dh1 = (dh2 @ q["W2"]) * (a1 > 0)
    g[OFF_B1:OFF_W2] = dh1.sum(0)
    g[OFF_W1:OFF_B1] = (dh1.T @ x).ravel()
    return g, float(((y - t) ** 2).mean())
