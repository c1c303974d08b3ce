"""CPU FP64 oracle of the control-variate MLP kernels.

TEST INFRASTRUCTURE ONLY: used by tests/ to check the tensor-core forward and
backward kernels of myquantlib_gb300 (csrc/cv_mlp.cu); never called by the
engine.

The network g(x) = w4 . silu(W3 silu(W2 silu(W1 x + b1) + b2) + b3) + b4 on
16 input slots, and the control-variate loss of a set of paths
    C_p = sum_j g(x_pj) dM_pj,   r_p = Y_p - C_p - mean(Y - C),   L = mean r_p^2.
`bf16=True` reproduces the kernels' storage precision: x, W1, W2, W3 and the
hidden activations h1, h2 rounded to BF16 (biases, w4 and h3 stay wide); the
derivatives treat the rounding as the identity.
"""
from __future__ import annotations

import numpy as np

NPARAM = 35332
LAYOUT = {"W1": (0, (128, 16)), "b1": (2048, (128,)), "W2": (2176, (128, 128)), "b2": (18560, (128,)),
          "W3": (18688, (128, 128)), "b3": (35072, (128,)), "w4": (35200, (128,)), "b4": (35328, (1,))}


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    a = ((a + 0x7FFF + ((a >> 16) & 1)) >> 16) << 16
    return a.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params: np.ndarray) -> dict:
    p = np.asarray(params, dtype=np.float64)
    return {k: p[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in LAYOUT.items()}


def pack(parts: dict) -> np.ndarray:
    out = np.zeros(NPARAM)
    for k, (o, s) in LAYOUT.items():
        out[o:o + int(np.prod(s))] = np.asarray(parts[k], dtype=np.float64).ravel()
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def _inputs(feats: np.ndarray) -> np.ndarray:
    x = np.zeros((feats.shape[0], 16))
    x[:, :feats.shape[1]] = feats
    return x


def forward(params, feats, bf16_storage: bool = True) -> tuple[np.ndarray, dict]:
    """g for every row of feats ([rows][<=16]); returns (g, intermediates)."""
    P = unpack(params)
    rd = bf16 if bf16_storage else (lambda a: np.asarray(a, dtype=np.float64))
    x = rd(_inputs(feats))
    W1, W2, W3 = rd(P["W1"]), rd(P["W2"]), rd(P["W3"])
    z1 = x @ W1.T + P["b1"]
    h1 = rd(silu(z1))
    z2 = h1 @ W2.T + P["b2"]
    h2 = rd(silu(z2))
    z3 = h2 @ W3.T + P["b3"]
    h3 = silu(z3)
    g = h3 @ P["w4"] + P["b4"][0]
    return g, {"x": x, "W1": W1, "W2": W2, "W3": W3, "z1": z1, "h1": h1, "z2": z2, "h2": h2, "z3": z3, "h3": h3}


def loss_and_grad(params, feats, dM, Y, n_paths: int, n_hedge: int, bf16_storage: bool = True):
    """L and dL/dparams (packed like the parameter blob); rows are p * n_hedge + j."""
    P = unpack(params)
    g, t = forward(params, feats, bf16_storage)
    C = (g * dM).reshape(n_paths, n_hedge).sum(axis=1)
    r = Y - C - np.mean(Y - C)
    L = float(np.mean(r * r))
    coef = -2.0 * r / n_paths
    dg = np.repeat(coef, n_hedge) * dM
    grads = {"w4": t["h3"].T @ dg, "b4": np.array([dg.sum()])}
    dz3 = dg[:, None] * P["w4"][None, :] * silu_grad(t["z3"])
    grads["W3"], grads["b3"] = dz3.T @ t["h2"], dz3.sum(axis=0)
    dz2 = (dz3 @ t["W3"]) * silu_grad(t["z2"])
    grads["W2"], grads["b2"] = dz2.T @ t["h1"], dz2.sum(axis=0)
    dz1 = (dz2 @ t["W2"]) * silu_grad(t["z1"])
    grads["W1"], grads["b1"] = dz1.T @ t["x"], dz1.sum(axis=0)
    return L, pack(grads)


def loss(params, feats, dM, Y, n_paths: int, n_hedge: int) -> float:
    g, _ = forward(params, feats, bf16_storage=False)
    C = (g * dM).reshape(n_paths, n_hedge).sum(axis=1)
    r = Y - C - np.mean(Y - C)
    return float(np.mean(r * r))
