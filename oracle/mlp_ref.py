"""CPU oracle of the parameter selector's network.

TEST INFRASTRUCTURE ONLY: the tests use it as the checker of the CUDA
kernels; the selector itself never imports it.

The reference has no learned selector; this is the plain mathematical
definition that the CUDA kernels (fasttools2d_gb300/csrc/mlp.cu) must match:
an 8 -> 64 -> 64 -> 4 perceptron with tanh hidden units, parameters packed as
W1[64x8], b1[64], W2[64x64], b2[64], W3[4x64], b3[4] (row-major, y = W x + b),
loss = (1/n) sum_i w_i |y_i - t_i|^2, its gradient by back-propagation, and
one Adam step (Kingma & Ba 2015).  Computed in FP64.
"""
import numpy as np

IN, H, OUT = 8, 64, 4
SHAPES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (OUT, H)), ("b3", (OUT,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, o = {}, 0
    for name, shape in SHAPES:
        k = int(np.prod(shape))
        out[name] = p[o:o + k].reshape(shape)
        o += k
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def init(seed=0):
    """Glorot-uniform weights, zero biases."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in SHAPES:
        if name.startswith("W"):
            lim = np.sqrt(6.0 / (shape[0] + shape[1]))
            d[name] = rng.uniform(-lim, lim, size=shape)
        else:
            d[name] = np.zeros(shape)
    return pack(d)


def forward(p, X, keep=False):
    w = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    h1 = np.tanh(X @ w["W1"].T + w["b1"])
    h2 = np.tanh(h1 @ w["W2"].T + w["b2"])
    y = h2 @ w["W3"].T + w["b3"]
    return (y, h1, h2) if keep else y


def loss_grad(p, X, T, weights=None):
    w = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    n = X.shape[0]
    s = np.ones(n) if weights is None else np.asarray(weights, dtype=np.float64)
    y, h1, h2 = forward(p, X, keep=True)
    r = y - T
    loss = float(np.sum(s * np.sum(r * r, 1)) / n)
    d3 = 2.0 * (s / n)[:, None] * r
    d2 = (d3 @ w["W3"]) * (1 - h2 * h2)
    d1 = (d2 @ w["W2"]) * (1 - h1 * h1)
    g = {"W3": d3.T @ h2, "b3": d3.sum(0), "W2": d2.T @ h1, "b2": d2.sum(0), "W1": d1.T @ X, "b1": d1.sum(0)}
    return loss, pack(g)


def adam(p, g, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
