"""Float64 NumPy restatement of the ray-map surrogate's arithmetic.

Test infrastructure only: the tests use it to check the GPU's packing,
forward pass, loss gradient and backward pass.  The product never imports
it.

The reference has no learned part, so nothing here follows a reference
file.  The functions restate the network the package defines: 9 inputs,
SiLU hidden layers, 3 outputs, squared error on the position residual,
binary cross-entropy with logits on the vignetting label.  With
``rounding=True`` they round to BF16 at the points where the GPU stores
BF16:

* the packed inputs;
* each pre-activation Z and activation H = silu(Z);
* the loss gradient dY;
* each back-propagated dZ.

Everything else is float64.  The remaining differences from the GPU are its
FP32 accumulation order, plus an occasional BF16 rounding that falls on the
other side of a tie.

Parity pin: with ``rounding=False`` the backward pass is checked against
central finite differences of the forward pass and loss in float64.
"""

from __future__ import annotations

import itertools

import numpy as np


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even), returned as float32."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def features(wl, fx, fy, qx, qy, wl_lo, wl_hi, fxh, fyh, ph) -> np.ndarray:
    """Normalised ray inputs u0..u4 in float32, as the packing kernel forms
    them: IEEE float32 divisions by the half ranges."""
    f32 = np.float32
    wl_mid = f32(0.5) * (f32(wl_lo) + f32(wl_hi))
    wl_half = f32(0.5) * (f32(wl_hi) - f32(wl_lo))
    u = np.stack([np.asarray(fx, f32) / f32(fxh), np.asarray(fy, f32) / f32(fyh),
                  np.asarray(qx, f32) / f32(ph), np.asarray(qy, f32) / f32(ph),
                  (np.asarray(wl, f32) - wl_mid) / wl_half], axis=-1)
    return u.astype(np.float32)


def quadratic_basis(u) -> np.ndarray:
    u = np.asarray(u, dtype=np.float64)
    cols = [np.ones(len(u))] + [u[:, i] for i in range(5)]
    cols += [u[:, i] * u[:, j] for i, j in itertools.combinations_with_replacement(range(5), 2)]
    return np.stack(cols, axis=-1)


def sigmoid(z):
    return 0.5 * (1.0 + np.tanh(0.5 * z))


def silu(z):
    return z * sigmoid(z)


def silu_grad(z):
    s = sigmoid(z)
    return s * (1.0 + z * (1.0 - s))


def forward(x, weights, biases, rounding: bool = True):
    """Outputs y [rows x 3] and the stored Z, H of every hidden layer.

    x: [rows x 9] inputs; weights[l]: [out x in]; biases[l]: [out]."""
    r = bf16 if rounding else (lambda v: np.asarray(v, dtype=np.float64))
    h = np.asarray(x, dtype=np.float64)
    zs, hs = [], [h]
    for l, (w, b) in enumerate(zip(weights, biases)):
        z = h @ np.asarray(w, np.float64).T + np.asarray(b, np.float64)
        if l == len(weights) - 1:
            return z, zs, hs
        zs.append(np.asarray(r(z), np.float64))
        h = np.asarray(r(silu(z)), np.float64)
        hs.append(h)
    raise ValueError("no layers")


def loss(y, t, label, w_pos, w_cls, norm):
    """Squared position error on unvignetted rays plus BCE with logits."""
    e = (y[:, 0] - t[:, 0]) ** 2 + (y[:, 1] - t[:, 1]) ** 2
    s = y[:, 2]
    bce = np.maximum(s, 0.0) - s * label + np.log1p(np.exp(-np.abs(s)))
    return norm * (w_pos * np.sum(label * e) + w_cls * np.sum(bce))


def loss_grad(y, t, label, w_pos, w_cls, norm, rounding: bool = True):
    g = np.zeros_like(y, dtype=np.float64)
    g[:, 0] = 2.0 * w_pos * norm * label * (y[:, 0] - t[:, 0])
    g[:, 1] = 2.0 * w_pos * norm * label * (y[:, 1] - t[:, 1])
    g[:, 2] = w_cls * norm * (sigmoid(y[:, 2]) - label)
    return np.asarray(bf16(g), np.float64) if rounding else g


def backward(dy, weights, zs, hs, rounding: bool = True):
    """Weight and bias gradients of every layer from dL/dy."""
    r = bf16 if rounding else (lambda v: np.asarray(v, dtype=np.float64))
    nl = len(weights)
    gw, gb = [None] * nl, [None] * nl
    dz = np.asarray(dy, np.float64)
    for l in range(nl - 1, -1, -1):
        gw[l] = dz.T @ hs[l]
        gb[l] = dz.sum(axis=0)
        if l == 0:
            break
        dh = dz @ np.asarray(weights[l], np.float64)
        dz = np.asarray(r(dh * silu_grad(zs[l - 1])), np.float64)
    return gw, gb
