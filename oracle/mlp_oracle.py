"""FP64 numpy restatement of the layout selector's network -- TEST
INFRASTRUCTURE ONLY: the checker for the CUDA forward, gradient and Adam
kernels (cufinufft_gb300/csrc/mlp.cu) and for the committed selector weights.

The network has no counterpart in the reference (cuFINUFFT v1.3 picks its
method from opts.gpu_method alone, src/cufinufft.cu:103-112 of the reference);
it is checked here against its own mathematical definition:
  features F=14 -> H=32 (ReLU) -> H=32 (ReLU) -> K=12,
  params = [W1[H][F], b1[H], W2[H][H], b2[H], W3[K][H], b3[K]],
  L = sum m (y - t)^2 / sum m.
"""
from __future__ import annotations

import re

import numpy as np

F, H, K = 14, 32, 12
SHAPES = [("W1", (H, F)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (K, H)), ("b3", (K,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, o = {}, 0
    for name, s in SHAPES:
        n = int(np.prod(s))
        out[name] = p[o:o + n].reshape(s)
        o += n
    return out


def forward(p, X):
    w = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    A1 = np.maximum(X @ w["W1"].T + w["b1"], 0)
    A2 = np.maximum(A1 @ w["W2"].T + w["b2"], 0)
    return A2 @ w["W3"].T + w["b3"], (A1, A2)


def loss_and_grad(p, X, T, Mk):
    w = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    Y, (A1, A2) = forward(p, X)
    msum = float(np.sum(Mk))
    d = (Y - T) * Mk
    loss = float(np.sum(d * d) / msum)
    dY = 2 * d / msum
    g = {"W3": dY.T @ A2, "b3": dY.sum(0)}
    dA2 = (dY @ w["W3"]) * (A2 > 0)
    g["W2"], g["b2"] = dA2.T @ A1, dA2.sum(0)
    dA1 = (dA2 @ w["W2"]) * (A1 > 0)
    g["W1"], g["b1"] = dA1.T @ X, dA1.sum(0)
    return loss, np.concatenate([g[name].ravel() for name, _ in SHAPES])


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v


def read_weights_header(path):
    """(trained, mean[F], std[F], params[NPARAM]) from selector_weights.h."""
    text = open(path).read()
    trained = int(re.search(r"constexpr int kSelectorTrained\s*=\s*(\d+);", text).group(1))

    def arr(name):
        body = re.search(name + r"\[[^\]]*\]\s*=\s*\{([^}]*)\}", text).group(1)
        vals = [float(x.rstrip("fF")) for x in re.split(r"[,\s]+", body.strip()) if x]
        return np.array(vals, dtype=np.float32)
    return trained, arr("kSelMean"), arr("kSelStd"), arr("kSelParams")
