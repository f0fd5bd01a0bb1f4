"""NumPy restatement of the cost-model network (16 -> 64 -> 64 -> 1, ReLU,
mean squared error): the CPU reference the GPU kernels' outputs and
gradients are checked against.  Test infrastructure."""
import numpy as np

SHAPES = [("W1", (64, 16)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)), ("W3", (64,)), ("b3", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape).astype(np.float64)
        o += n
    return out


def forward(p, X):
    w = unpack(p)
    h1 = np.maximum(X @ w["W1"].T + w["b1"], 0)
    h2 = np.maximum(h1 @ w["W2"].T + w["b2"], 0)
    return h2 @ w["W3"] + w["b3"][0], (h1, h2)


def grad(p, X, y):
    """Gradient of mean((f(X) - y)^2) in float64, packed like the parameters."""
    w = unpack(p)
    out, (h1, h2) = forward(p, X)
    n = X.shape[0]
    d = 2.0 * (out - y) / n
    g = {"W3": h2.T @ d, "b3": np.array([d.sum()])}
    dh2 = np.outer(d, w["W3"]) * (h2 > 0)
    g["W2"], g["b2"] = dh2.T @ h1, dh2.sum(0)
    dh1 = (dh2 @ w["W2"]) * (h1 > 0)
    g["W1"], g["b1"] = dh1.T @ X, dh1.sum(0)
    return np.concatenate([g[name].ravel() for name, _ in SHAPES]), float(np.mean((out - y) ** 2))
