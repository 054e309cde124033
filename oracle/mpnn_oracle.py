"""CPU oracle of the learned warm-start network (test infrastructure only).

A numpy restatement of the message-passing network the GPU trains and runs
with tcgen05 BF16 kernels, used only by tests/ to check the GPU forward pass
and gradients.  It evaluates in FP64; with ``bf16=True`` it rounds to BF16
at exactly the points where the GPU stores BF16 (features, weights, hidden
states, neighbour means, pre-activations, and in the backward pass dZ and the
per-face neighbour-mean gradients), so the remaining difference is the GPU's
FP32 accumulation order.

Network (hidden width H = 64), per face E with neighbour set N(E) (the faces
sharing a cell with E, i.e. the off-diagonal pattern of the face system):
    h1 = relu(x W0 + b0)                                   x: 16 features
    a_l = mean_{E' in N(E)} h_l(E')                        l = 1, 2, 3
    h_{l+1} = relu([h_l, a_l] W_l + b_l) + h_l
    out = h4 . wd + bd
Loss: mean over the training faces of (out - y)^2.
"""
from __future__ import annotations

import numpy as np

H = 64
FIN = 16
LAYERS = 3


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rounding) >> 16) << 16
    out = u.astype(np.uint32).view(np.float32).astype(np.float64)
    nan = np.isnan(f)
    if nan.any():
        out[nan] = np.nan
    return out


def init_params(seed: int = 0) -> dict:
    rng = np.random.default_rng(seed)
    p = {"W0": rng.standard_normal((FIN, H)) * np.sqrt(2.0 / FIN), "b0": np.zeros(H)}
    for l in range(1, LAYERS + 1):
        p[f"W{l}"] = rng.standard_normal((2 * H, H)) * np.sqrt(1.0 / (2 * H))
        p[f"b{l}"] = np.zeros(H)
    p["wd"] = rng.standard_normal(H) * 0.01
    p["bd"] = np.zeros(1)
    return p


def neighbour_mean(h: np.ndarray, nbr: np.ndarray, deg: np.ndarray) -> np.ndarray:
    """nbr [F][W] with padding = own index (excluded via deg)."""
    F, W = nbr.shape
    own = np.arange(F)[:, None]
    valid = nbr != own
    s = np.zeros_like(h)
    for k in range(W):
        m = valid[:, k]
        s[m] += h[nbr[m, k]]
    return s / np.maximum(deg, 1)[:, None]


def neighbour_sum_transpose(v: np.ndarray, nbr: np.ndarray) -> np.ndarray:
    """G(v)_E' = sum over rows E having E' as a neighbour of v_E."""
    F, W = nbr.shape
    own = np.arange(F)[:, None]
    valid = nbr != own
    out = np.zeros_like(v)
    for k in range(W):
        m = valid[:, k]
        np.add.at(out, nbr[m, k], v[m])
    return out


def forward(p: dict, x: np.ndarray, nbr: np.ndarray, deg: np.ndarray, bf: bool = True):
    r = bf16 if bf else (lambda a: np.asarray(a, np.float64))
    cache = {}
    x = r(x)
    z0 = x @ r(p["W0"]) + p["b0"]
    z0s = r(z0)
    h = r(np.maximum(z0, 0))
    cache["x"], cache["z0"], cache["h1"] = x, z0s, h
    for l in range(1, LAYERS + 1):
        a = r(neighbour_mean(h, nbr, deg))
        X = np.concatenate([h, a], axis=1)
        z = X @ r(p[f"W{l}"]) + p[f"b{l}"]
        hn = r(np.maximum(z, 0) + h)
        cache[f"a{l}"], cache[f"z{l}"], cache[f"h{l + 1}"] = a, r(z), hn
        h = hn
    out = h @ p["wd"] + p["bd"][0]
    return out, cache


def loss_and_grads(p: dict, x, nbr, deg, y, mask, bf: bool = True):
    r = bf16 if bf else (lambda a: np.asarray(a, np.float64))
    out, c = forward(p, x, nbr, deg, bf)
    nt = max(int(mask.sum()), 1)
    diff = (out - y) * mask
    loss = float((diff ** 2).sum() / nt)
    dout = 2.0 * diff / nt
    g = {}
    h4 = c[f"h{LAYERS + 1}"]
    g["wd"] = h4.T @ dout
    g["bd"] = np.array([dout.sum()])
    dh = np.outer(dout, p["wd"])
    for l in range(LAYERS, 0, -1):
        z = c[f"z{l}"]
        dz = dh * (z > 0)
        X = np.concatenate([c[f"h{l}"], c[f"a{l}"]], axis=1)
        dzr = r(dz)
        g[f"W{l}"] = X.T @ dzr
        g[f"b{l}"] = dz.sum(axis=0)
        dx = dzr @ r(p[f"W{l}"]).T
        dself, da = dx[:, :H], dx[:, H:]
        dh = dh + dself + neighbour_sum_transpose(r(da / np.maximum(deg, 1)[:, None]), nbr)
    dz0 = dh * (c["z0"] > 0)
    g["W0"] = c["x"].T @ r(dz0)
    g["b0"] = dz0.sum(axis=0)
    return loss, g, out
