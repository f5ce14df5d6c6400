"""FP64 restatement of the learned-radius MLP (test infrastructure only).

The checker for snch_lbvh_gb300/csrc/mlp.cu: the same features, layers, head
and pinball loss, evaluated in float64 with NumPy, with the BF16 roundings of
the tensor-core path applied at the same places (the GEMM operands: features,
hidden activations, weights and back-propagated dZ) so that forward values and
gradients can be compared closely. The reference library has no learned
radius; this model only seeds the exact queries.

Parameter block (float32, row-major [out x in] weights):
  W1 64x192, b1 64, W2 64x64, b2, W3 64x64, b3, W4 64x64, b4, W5 2x64, b5 2
Feature column 6k + 2a (+1) = sin (cos) of pi * s_k * u_a, s_k = float32(2^(k/4)),
u = (p - centre) * inv_half in float32, centre = 0.5 (lo + hi), inv_half = 2 / (hi - lo).
"""
from __future__ import annotations

import numpy as np

FREQ, IN, HID, OUT = 32, 192, 64, 2
SIZES = [(HID, IN), (HID,), (HID, HID), (HID,), (HID, HID), (HID,), (HID, HID), (HID,), (OUT, HID), (OUT,)]


def unpack(params):
    out, off = [], 0
    for s in SIZES:
        k = int(np.prod(s))
        out.append(np.asarray(params[off:off + k], np.float64).reshape(s))
        off += k
    assert off == len(params)
    return out


def bf16(x):
    """Round to bfloat16 (round to nearest, ties to even) through float32."""
    f = np.ascontiguousarray(x, np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def features(pts, lo, hi):
    lo, hi = np.asarray(lo, np.float32), np.asarray(hi, np.float32)
    centre = np.float32(0.5) * (lo + hi)
    inv_half = np.float32(2.0) / (hi - lo)
    u = (np.asarray(pts, np.float32) - centre) * inv_half
    s = np.exp2(0.25 * np.arange(FREQ)).astype(np.float32)
    arg = (s[None, :, None] * u[:, None, :]).astype(np.float32).astype(np.float64) * np.pi  # n x 32 x 3
    X = np.empty((len(u), FREQ, 3, 2))
    X[..., 0] = np.sin(arg)
    X[..., 1] = np.cos(arg)
    return X.reshape(len(u), IN)


def forward(params, pts, lo, hi, emulate_bf16=True):
    """Returns (outputs n x 2, cache) in float64."""
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3, W4, b4, W5, b5 = unpack(params)
    X = r(features(pts, lo, hi))
    Hs, h = [], X
    for W, b in ((W1, b1), (W2, b2), (W3, b3), (W4, b4)):
        h = r(np.maximum(h @ r(W).T + b, 0.0))
        Hs.append(h)
    o = h @ W5.T + b5
    return o, (X, Hs)


def radius(params, pts, lo, hi, margin, floor, emulate_bf16=True):
    o, _ = forward(params, pts, lo, hi, emulate_bf16)
    return np.exp(o) * margin + floor


def loss_and_grad(params, pts, targets, lo, hi, tau, emulate_bf16=True):
    """Mean (over points) of the summed pinball losses of the two outputs and its
    gradient; NaN targets are left out. Mirrors mlp_forward_backward."""
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3, W4, b4, W5, b5 = unpack(params)
    n = len(pts)
    o, (X, Hs) = forward(params, pts, lo, hi, emulate_bf16)
    y = np.asarray(targets, np.float64)
    res = y - o
    valid = ~np.isnan(y)
    res0 = np.where(valid, res, 0.0)
    loss = np.where(res0 > 0, tau * res0, (tau - 1.0) * res0).sum() / n
    d = np.where(valid, np.where(res0 > 0, -tau, 1.0 - tau), 0.0) / n  # dL/do, n x 2
    g = [None] * 10
    g[8] = d.T @ Hs[3]
    g[9] = d.sum(0)
    Ws = [W1, W2, W3, W4]
    dZ = r((d @ W5) * (Hs[3] > 0))
    g[7] = dZ.sum(0)
    for l in range(3, -1, -1):
        A = X if l == 0 else Hs[l - 1]
        g[2 * l] = dZ.T @ A
        if l == 0:
            break
        dH = dZ @ r(Ws[l])
        gz = dH * (Hs[l - 1] > 0)
        g[2 * l - 1] = gz.sum(0)
        dZ = r(gz)
    return loss, np.concatenate([x.reshape(-1) for x in g])
