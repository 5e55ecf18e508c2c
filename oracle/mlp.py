"""float64 numpy restatement of the MLP radiance cache -- TEST INFRASTRUCTURE.

Same padded parameter layout, encoding, network, loss and Adam as
rtcore_cache.h, evaluated in float64 with BF16 rounding applied at exactly
the points where the GPU rounds (encoded inputs, weights, the activations fed
to the next layer, the deltas fed to the backward and weight-gradient MMAs).  The GPU accumulates
in FP32 in an unspecified order, so results are compared with a tolerance.
"""
from __future__ import annotations

import numpy as np

IN = [96, 64, 64, 64, 64, 64]
OUT = [64, 64, 64, 64, 64, 8]
USED_IN, USED_OUT = 81, 3


def offsets():
    w, o = [], 0
    for l in range(6):
        w.append((o, o + OUT[l] * IN[l]))
        o += OUT[l] * IN[l] + OUT[l]
    return w, o


W_OFF, N_PARAMS = offsets()


def unpack(p: np.ndarray):
    out = []
    for l in range(6):
        wo, bo = W_OFF[l]
        out.append((p[wo:bo].reshape(OUT[l], IN[l]).astype(np.float64), p[bo:bo + OUT[l]].astype(np.float64)))
    return out


def bf16(x) -> np.ndarray:
    """Round to bfloat16 (nearest, ties to even); float64 values."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _round(x, exact: bool):
    return np.asarray(x, np.float64) if exact else bf16(x)


def encode(inputs: np.ndarray, lo, hi, exact: bool = False) -> np.ndarray:
    """inputs: structured (pos, dir, normal, albedo) float32 [n, 3] each."""
    f32 = np.float32
    lo = np.asarray(lo, f32)
    hi = np.asarray(hi, f32)
    ext = (hi - lo).astype(f32)
    pn = ((inputs["pos"].astype(f32) - lo) / ext).astype(f32)
    n = len(inputs)
    x = np.zeros((n, 96), np.float64)
    for a in range(3):
        for k in range(12):
            arg = (f32(2 ** k) * pn[:, a]).astype(np.float64)
            x[:, 24 * a + 2 * k] = np.sin(np.pi * arg)
            x[:, 24 * a + 2 * k + 1] = np.cos(np.pi * arg)
    x[:, 72:75] = inputs["dir"]
    x[:, 75:78] = inputs["normal"]
    x[:, 78:81] = inputs["albedo"]
    return _round(x, exact)


def forward(p: np.ndarray, inputs: np.ndarray, lo, hi, keep: bool = False, exact: bool = False):
    """exact=True: no BF16 rounding anywhere (plain float64 network)."""
    layers = unpack(p)
    a = encode(inputs, lo, hi, exact)
    acts = [a]
    for l in range(5):
        w, b = layers[l]
        z = a @ _round(w, exact).T + b
        a = _round(np.maximum(z, 0.0), exact)
        acts.append(a)
    w, b = layers[5]
    y = a @ _round(w, exact).T + b
    return (y, acts) if keep else y


def gradient(p: np.ndarray, inputs: np.ndarray, targets: np.ndarray, lo, hi, exact: bool = False):
    """(grad in the padded layout, mean loss)."""
    layers = unpack(p)
    y, acts = forward(p, inputs, lo, hi, keep=True, exact=exact)
    n = len(inputs)
    t = np.zeros_like(y)
    t[:, :3] = targets[:, :3]
    yc = y if exact else y.astype(np.float32).astype(np.float64)
    diff = yc - t
    den = yc * yc + 0.01
    d = np.zeros_like(y)
    d[:, :3] = 2.0 * diff[:, :3] / den[:, :3] / (3.0 * n)
    loss = float((diff[:, :3] ** 2 / den[:, :3]).sum() / (3.0 * n))
    g = np.zeros(N_PARAMS, np.float64)
    for L in range(5, -1, -1):
        wo, bo = W_OFF[L]
        dr = _round(d, exact)  # the weight-gradient MMAs take delta in BF16
        g[wo:bo] = (dr.T @ acts[L]).reshape(-1)
        g[bo:bo + OUT[L]] = dr.sum(axis=0)
        if L == 0:
            break
        w, _ = layers[L]
        dprev = _round(d, exact) @ _round(w, exact)
        d = dprev * (acts[L] > 0)
    return g, loss


def adam(p, g, m, v, step, lr=1e-3, b1=0.9, b2=0.99, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
