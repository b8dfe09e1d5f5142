"""CPU oracle of the warm-start proposer network (test infrastructure only).

numpy restatement of the BF16 tensor-core MLP of the GPU library
(hbtg_mlp_forward / hbtg_mlp_backward): 6 -> 64 -> 64 -> 1, ReLU, sigmoid
output, weighted binary cross-entropy.  The operands the kernels feed to the
tensor cores are rounded to bfloat16 (round to nearest even) at the same
points; sums are in float64 here and in FP32 on the GPU, so results agree to
FP32 accumulation error, not bit for bit.

Weight layout (flat float32, 4673 entries):
  W1[6][64] (in x out), b1[64], W2[64][64] (in x out), b2[64], w3[64], b3

The network has no counterpart in the reference; parity for it is agreement
of the GPU gradients with this oracle, and the oracle's own calculus is
checked against finite differences with the rounding switched off.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID = 6, 64
SIZES = [("W1", N_IN * N_HID), ("b1", N_HID), ("W2", N_HID * N_HID), ("b2", N_HID), ("w3", N_HID), ("b3", 1)]
N_PARAMS = sum(n for _, n in SIZES)


def unpack(w):
    out, k = {}, 0
    for name, n in SIZES:
        out[name] = np.asarray(w[k:k + n], dtype=np.float64)
        k += n
    out["W1"] = out["W1"].reshape(N_IN, N_HID)
    out["W2"] = out["W2"].reshape(N_HID, N_HID)
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SIZES]).astype(np.float32)


def bf16(a):
    """Rounds float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _r(a, rounding):
    return bf16(a) if rounding else np.asarray(a, dtype=np.float64)


def forward(w, x, rounding=True):
    """Returns (prob, cache); x is [n, 6]."""
    P = unpack(w)
    xb = _r(x, rounding)
    h1 = np.maximum(xb @ _r(P["W1"], rounding) + P["b1"], 0.0)
    h1b = _r(h1, rounding)
    h2 = np.maximum(h1b @ _r(P["W2"], rounding) + P["b2"], 0.0)
    h2b = _r(h2, rounding)
    w3b = _r(P["w3"], rounding)
    logit = h2b @ w3b + P["b3"][0]
    prob = 1.0 / (1.0 + np.exp(-logit))
    return prob, dict(P=P, xb=xb, h1=h1, h1b=h1b, h2=h2, w3b=w3b, logit=logit, prob=prob)


def loss_and_grad(w, x, y, sw=None, rounding=True):
    """Summed weighted BCE and its gradient, by the kernels' recipe: FP32
    activations for the output-layer and bias gradients, BF16 operands for the
    three weight-gradient products."""
    prob, c = forward(w, x, rounding)
    P = c["P"]
    y = np.asarray(y, dtype=np.float64)
    sw = np.ones_like(y) if sw is None else np.asarray(sw, dtype=np.float64)
    l = c["logit"]
    loss = float(np.sum(sw * (np.maximum(l, 0) - l * y + np.log1p(np.exp(-np.abs(l))))))
    dl = sw * (prob - y)
    g = {}
    g["w3"] = c["h2"].T @ dl
    g["b3"] = np.array([dl.sum()])
    dz2 = np.outer(dl, c["w3b"]) * (c["h2"] > 0)
    g["b2"] = dz2.sum(0)
    dz2b = _r(dz2, rounding)
    dz1 = (dz2b @ _r(P["W2"], rounding).T) * (c["h1"] > 0)
    g["b1"] = dz1.sum(0)
    g["W2"] = c["h1b"].T @ dz2b
    g["W1"] = c["xb"].T @ _r(dz1, rounding)
    return loss, pack(g).astype(np.float64), prob


def init_weights(seed=0):
    """He-normal weights, zero biases."""
    rng = np.random.default_rng(seed)
    d = dict(W1=rng.standard_normal((N_IN, N_HID)) * np.sqrt(2.0 / N_IN), b1=np.zeros(N_HID),
             W2=rng.standard_normal((N_HID, N_HID)) * np.sqrt(2.0 / N_HID), b2=np.zeros(N_HID),
             w3=rng.standard_normal(N_HID) * np.sqrt(1.0 / N_HID), b3=np.zeros(1))
    return pack(d)
