"""Host restatement of the batched trace's ray generation (test oracle).

TEST INFRASTRUCTURE.  Philox4x32-10 (Salmon, Moraes, Dror and Shaw, SC
2011) in NumPy, bit-identical to optika_gb300/csrc/philox.cuh, and the
float32 formulas of the device's ``batch_ray`` evaluated with NumPy float32
operations (one rounding each, no fused multiply-add), so the oracle traces
exactly the rays the kernel generated.
"""

from __future__ import annotations

import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0: int, k1: int):
    c0, c1, c2, c3 = (np.asarray(v, dtype=np.uint64) & MASK for v in (c0, c1, c2, c3))
    k0 = np.uint64(k0 & 0xFFFFFFFF)
    k1 = np.uint64(k1 & 0xFFFFFFFF)
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0 = (k0 + np.uint64(W0)) & MASK
        k1 = (k1 + np.uint64(W1)) & MASK
    return c0, c1, c2, c3


def u01(x) -> np.ndarray:
    return (np.asarray(x, dtype=np.uint64) >> np.uint64(8)).astype(np.float32) * np.float32(
        5.9604644775390625e-8
    )


def batch_inputs(seed: int, config: int, n: int, wl_lo: float, wl_hi: float, fxh: float,
                 fyh: float, pupil_half: float) -> dict:
    """float32 inputs of rays 0..n-1 of one configuration."""
    i = np.arange(n, dtype=np.uint64)
    k0, k1 = seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF
    a = philox4x32_10(i & MASK, i >> np.uint64(32), np.uint64(config), np.uint64(0), k0, k1)
    ff = np.uint64(0xFF)
    low = ((a[0] & ff) << np.uint64(24)) | ((a[1] & ff) << np.uint64(16)) | (
        (a[2] & ff) << np.uint64(8))
    f = np.float32
    two, one = f(2), f(1)
    wl = f(wl_lo) + u01(a[0]) * (f(wl_hi) - f(wl_lo))
    fx = f(fxh) * (two * u01(a[1]) - one)
    fy = f(fyh) * (two * u01(a[2]) - one)
    qx = f(pupil_half) * (two * u01(a[3]) - one)
    qy = f(pupil_half) * (two * u01(low) - one)
    return dict(wavelength=wl, field_x=fx, field_y=fy, pupil_x=qx, pupil_y=qy)
