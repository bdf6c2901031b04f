"""Float64 NumPy restatement of the rank-predictor MLP (test infrastructure only).

Same flat parameter layout and loss as the CUDA kernels (atlasq_gb300/csrc/mlp.cu):
W1[64][5] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[64] b4, ReLU hidden
layers, sigmoid output, L = mean (y - t)^2, AdamW update.  There is no reference
implementation of this predictor (the reference's RankPredictor,
src/atlas_q/tools_qih/ai_rank_predictor.py:14-89, consumes singular values after
the SVD); this oracle is the CPU float64 check of the kernels' gradients.
"""
import numpy as np

IN, H = 5, 64
SIZES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
         ("W4", (H,)), ("b4", (1,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SIZES])


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    d = {"W1": rng.standard_normal((H, IN)) * np.sqrt(2.0 / IN), "b1": np.zeros(H),
         "W2": rng.standard_normal((H, H)) * np.sqrt(2.0 / H), "b2": np.zeros(H),
         "W3": rng.standard_normal((H, H)) * np.sqrt(2.0 / H), "b3": np.zeros(H),
         "W4": rng.standard_normal(H) * np.sqrt(1.0 / H), "b4": np.zeros(1)}
    return pack(d)


def forward(p, X):
    d = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    a1 = X @ d["W1"].T + d["b1"]
    h1 = np.maximum(a1, 0)
    a2 = h1 @ d["W2"].T + d["b2"]
    h2 = np.maximum(a2, 0)
    a3 = h2 @ d["W3"].T + d["b3"]
    h3 = np.maximum(a3, 0)
    z = h3 @ d["W4"] + d["b4"][0]
    y = 1.0 / (1.0 + np.exp(-z))
    return y, (X, a1, h1, a2, h2, a3, h3, z)


def loss_and_grad(p, X, T):
    d = unpack(p)
    y, (X, a1, h1, a2, h2, a3, h3, z) = forward(p, X)
    T = np.asarray(T, dtype=np.float64)
    B = len(T)
    loss = np.mean((y - T) ** 2)
    dz = 2.0 * (y - T) / B * y * (1 - y)
    g = {"W4": h3.T @ dz, "b4": np.array([dz.sum()])}
    d3 = np.outer(dz, d["W4"]) * (a3 > 0)
    g["W3"] = d3.T @ h2
    g["b3"] = d3.sum(0)
    d2 = (d3 @ d["W3"]) * (a2 > 0)
    g["W2"] = d2.T @ h1
    g["b2"] = d2.sum(0)
    d1 = (d2 @ d["W2"]) * (a1 > 0)
    g["W1"] = d1.T @ X
    g["b1"] = d1.sum(0)
    return loss, pack(g)


def adam_step(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8, wd=0.0):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    p = p - lr * (mh / (np.sqrt(vh) + eps) + wd * p)
    return p, m, v
