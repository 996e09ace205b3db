"""Float64 restatement of the calibration fits on traced rays (test oracle).

TEST INFRASTRUCTURE: imported only by tests/.  Follows
optika/systems/_sequential.py:1208-1285 (distortion), 1287-1368
(vignetting) and 1370-1512 (area_effective) with the rays traced by this
package's float64 oracle (oracle/trace.py), and restates the polynomial fit
of ``named_arrays.PolynomialFitFunctionArray.from_degree`` (not vendored in
the reference) as a linear least-squares fit of all monomials of total
degree <= degree in the inputs minus their mean.
"""

from __future__ import annotations

import numpy as np

from . import stops as OS
from . import trace as O


def monomial_exponents(n: int, degree: int):
    """All exponent tuples of n variables with total degree <= degree."""
    out = [()]
    for _ in range(n):
        out = [t + (e,) for t in out for e in range(degree + 1)]
    return [t for t in out if sum(t) <= degree]


def polyfit(inputs, outputs, degree, where=True):
    """(predict, center): least squares over the points in ``where``."""
    X = np.stack([np.ravel(np.asarray(v, dtype=np.float64)) for v in inputs], axis=1)
    c = X.mean(axis=0)
    ex = monomial_exponents(X.shape[1], degree)

    def design(Z):
        D = Z - c
        return np.stack([np.prod([D[:, j] ** e[j] for j in range(len(e))], axis=0)
                         for e in ex], axis=1)

    m = np.ravel(np.broadcast_to(np.asarray(where, dtype=bool), np.shape(inputs[0])))
    A = design(X)[m]
    s = np.sqrt((A * A).sum(axis=0))
    s[s == 0] = 1
    Y = np.stack([np.ravel(np.asarray(o, dtype=np.float64)) for o in outputs], axis=1)[m]
    coef = np.linalg.lstsq(A / s, Y, rcond=None)[0] / s[:, None]

    def predict(*z):
        shape = np.broadcast_shapes(*[np.shape(v) for v in z])
        Z = np.stack([np.broadcast_to(np.asarray(v, dtype=np.float64), shape).ravel()
                      for v in z], axis=1)
        y = design(Z) @ coef
        return [y[:, k].reshape(shape) for k in range(y.shape[1])]

    return predict


def grid_rays(system, w, fx, fy, px, py, normalized_field=False, normalized_pupil=False,
              intensity=None):
    """Rays of the product grid at the sensor, shape (nw, nfx, nfy, npx, npy),
    and the (denormalised) field and pupil at every grid point."""
    W, FX, FY, PX, PY = np.meshgrid(w, fx, fy, px, py, indexing="ij")
    if normalized_field or normalized_pupil:
        FX, FY, PX, PY = (a.copy() for a in (FX, FY, PX, PY))
        for k, wk in enumerate(np.asarray(w, dtype=np.float64)):
            (FX[k], FY[k]), (PX[k], PY[k]) = OS.denormalize(
                system, float(wk), (FX[k], FY[k]), (PX[k], PY[k]), normalized_field,
                normalized_pupil)
    r = O.rayfunction(system, W, FX, FY, PX, PY, intensity=intensity)
    return r, W, FX, FY


def distortion(system, w, fx, fy, px, py, degree=2, **kw):
    r, W, FX, FY = grid_rays(system, w, fx, fy, px, py, **kw)
    u = r["unvignetted"]
    where = u.any(axis=(3, 4))
    m = u | ~where[..., None, None]
    mx = (r["px"] * m).sum(axis=(3, 4)) / m.sum(axis=(3, 4))
    my = (r["py"] * m).sum(axis=(3, 4)) / m.sum(axis=(3, 4))
    scene = (W[..., 0, 0], FX[..., 0, 0], FY[..., 0, 0])
    return dict(scene=scene, sensor=(mx, my), where=where,
                fit=polyfit(scene, (mx, my), degree, where))


def vignetting(system, w, fx, fy, px, py, degree=2, **kw):
    r, W, FX, FY = grid_rays(system, w, fx, fy, px, py, **kw)
    u = r["unvignetted"]
    where = u.any(axis=(3, 4))
    illum = u.mean(axis=(3, 4))
    norm = np.array([illum[k][where[k]].mean() for k in range(len(w))])
    illum = illum / norm[:, None, None]
    scene = (W[..., 0, 0], FX[..., 0, 0], FY[..., 0, 0])
    return dict(scene=scene, illumination=illum, where=where,
                fit=polyfit(scene, (illum,), degree, where))


def area_effective_centres(system, w, fx, fy, vx, vy):
    """Physical pupil vertices, rays at the pupil cell centres weighted by
    the cell areas; returns the effective area per wavelength."""
    cx = (np.asarray(vx)[:-1] + np.asarray(vx)[1:]) / 2
    cy = (np.asarray(vy)[:-1] + np.asarray(vy)[1:]) / 2
    area = np.abs(np.diff(vx)[:, None] * np.diff(vy)[None, :])
    W, FX, FY, PX, PY = np.meshgrid(w, fx, fy, cx, cy, indexing="ij")
    A = np.broadcast_to(area, PX.shape)
    r = O.rayfunction(system, W, FX, FY, PX, PY, intensity=A)
    s = np.where(r["unvignetted"], r["intensity"], 0).sum(axis=(3, 4))
    return s.mean(axis=(1, 2))


__all__ = ["monomial_exponents", "polyfit", "grid_rays", "distortion", "vignetting",
           "area_effective_centres"]
