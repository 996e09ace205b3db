"""Calibration fits on traced rays: ``SequentialSystem.distortion``,
``vignetting`` and ``area_effective`` (optika/systems/_sequential.py:
1208-1512).

The grid is a product of 1-D coordinate arrays (wavelength, field x, field
y, pupil x, pupil y, the pupil fastest).  The rays go through the fused
trace, and the masked reductions over the pupil (counts and means of the
unvignetted rays, flux sums) run on the GPU in ``otx_pupil_reduce``; the
small polynomial fits of the models run on the host in float64.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib as L
from .distortion import PolynomialDistortionModel
from .radiometry import InterpolatedEffectiveAreaModel, PolynomialVignettingModel
from .vectors import Cartesian2dVectorArray, SpectralPositionalVectorArray

__all__ = ["pupil_reduce", "distortion", "vignetting", "area_effective"]


def pupil_reduce(rays, groups: int, per_group: int) -> torch.Tensor:
    """[groups, 6] float64 sums of otx_pupil_reduce over rays laid out as
    ``groups`` runs of ``per_group`` consecutive rays."""
    from . import _api

    def flat(t):
        return None if t is None else t.reshape(-1).contiguous()

    b = dict(px=flat(rays.position.x), py=flat(rays.position.y),
             intensity=flat(rays.intensity),
             unvignetted=None if rays.unvignetted is None else flat(rays.unvignetted).to(
                 torch.uint8))
    n = groups * per_group
    sums = torch.empty((groups, 6), dtype=torch.float64, device=_api.device())
    L.check(L.load().otx_pupil_reduce(ctypes.byref(_api._rays_struct(b, n)), groups, per_group,
                                      _api.ptr(sums), _api.stream_handle()), "otx_pupil_reduce")
    return sums


def _axis(v, name: str) -> np.ndarray:
    if isinstance(v, torch.Tensor):
        v = v.detach().double().cpu().numpy()
    a = np.atleast_1d(np.asarray(v, dtype=np.float64))
    if a.ndim != 1:
        raise ValueError(f"{name} must be a 1-D array of grid values")
    return a


def _grid(system, wavelength, field, pupil):
    g = system.grid_input
    if wavelength is None:
        wavelength = None if g is None else g.wavelength
    if field is None:
        field = None if g is None else g.field
    if pupil is None:
        pupil = None if g is None else g.pupil
    if wavelength is None or field is None or pupil is None:
        raise ValueError("the calibration fits need wavelength, field and pupil grids")
    w = _axis(wavelength, "wavelength")
    if w.size < 1:
        raise ValueError("fitting a model requires the wavelength grid to vary along its own "
                         "logical axis.")
    return (w, _axis(field.x, "field x"), _axis(field.y, "field y"), _axis(pupil.x, "pupil x"),
            _axis(pupil.y, "pupil y"))


def _trace(system, w, fx, fy, px, py, normalized_field, normalized_pupil, intensity=None):
    """Rays of the product grid at the sensor, the denormalised inputs and
    the pupil sums [nw, nfx, nfy, 6]."""
    nw, nfx, nfy, npx, npy = len(w), len(fx), len(fy), len(px), len(py)
    shp = lambda a, k: a.reshape([-1 if i == k else 1 for i in range(5)])  # noqa: E731
    res = system.rayfunction(
        intensity=intensity, wavelength=shp(w, 0),
        field=Cartesian2dVectorArray(shp(fx, 1), shp(fy, 2)),
        pupil=Cartesian2dVectorArray(px.reshape(1, 1, 1, -1, 1) if np.ndim(px) == 1 else px,
                                     py.reshape(1, 1, 1, 1, -1) if np.ndim(py) == 1 else py),
        normalized_field=normalized_field, normalized_pupil=normalized_pupil,
        outputs=("px", "py", "intensity", "unvignetted"))
    rays = res.outputs
    full = (nw, nfx, nfy, npx, npy)
    for name in ("x", "y"):
        v = getattr(rays.position, name)
        if tuple(v.shape) != full:
            setattr(rays.position, name, v.expand(full))
    sums = pupil_reduce(rays, nw * nfx * nfy, npx * npy).reshape(nw, nfx, nfy, 6)
    return res.inputs, sums.cpu().numpy()


def _scene(inputs, nw, nfx, nfy) -> SpectralPositionalVectorArray:
    def g(v):
        a = v.detach().double().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(
            v, dtype=np.float64)
        a = a.reshape(a.shape + (1,) * max(0, 5 - a.ndim)) if a.ndim < 5 else a
        return np.broadcast_to(a, np.broadcast_shapes(a.shape, (nw, nfx, nfy, 1, 1)))[..., 0, 0]

    return SpectralPositionalVectorArray(
        wavelength=g(inputs.wavelength),
        position=Cartesian2dVectorArray(g(inputs.field.x), g(inputs.field.y)))


def distortion(system, wavelength=None, field=None, pupil=None, normalized_field=True,
               normalized_pupil=True, degree=2) -> PolynomialDistortionModel:
    """optika/systems/_sequential.py:1208-1285: the mean sensor position of
    the unvignetted rays of each scene point (all its rays where none is
    unvignetted), fitted by a polynomial of ``degree``; points with no
    unvignetted ray are left out of the fit."""
    w, fx, fy, px, py = _grid(system, wavelength, field, pupil)
    inputs, s = _trace(system, w, fx, fy, px, py, normalized_field, normalized_pupil)
    n = s[..., 0]
    where = n > 0
    per = len(px) * len(py)
    with np.errstate(invalid="ignore", divide="ignore"):
        mx = np.where(where, s[..., 1] / n, s[..., 3] / per)
        my = np.where(where, s[..., 2] / n, s[..., 4] / per)
    return PolynomialDistortionModel(
        coordinates_scene=_scene(inputs, len(w), len(fx), len(fy)),
        coordinates_sensor=Cartesian2dVectorArray(mx, my), degree=degree, where=where)


def vignetting(system, wavelength=None, field=None, pupil=None, normalized_field=True,
               normalized_pupil=True, degree=2) -> PolynomialVignettingModel:
    """optika/systems/_sequential.py:1287-1368: the unvignetted fraction of
    each scene point's pupil rays, normalised per wavelength by its mean
    over the field points that have any unvignetted ray, fitted by a
    polynomial of ``degree``."""
    w, fx, fy, px, py = _grid(system, wavelength, field, pupil)
    inputs, s = _trace(system, w, fx, fy, px, py, normalized_field, normalized_pupil)
    where = s[..., 0] > 0
    illum = s[..., 0] / (len(px) * len(py))
    m = np.array([illum[k][where[k]].mean() if where[k].any() else np.nan
                  for k in range(len(w))])
    illum = illum / m[:, None, None]
    return PolynomialVignettingModel(coordinates_scene=_scene(inputs, len(w), len(fx), len(fy)),
                                     illumination=illum, degree=degree, where=where)


def area_effective(system, wavelength=None, field=None, pupil=None, normalized_field=True,
                   normalized_pupil=True, random=True, seed=0) -> InterpolatedEffectiveAreaModel:
    """optika/systems/_sequential.py:1370-1512: ``pupil`` holds cell
    *vertices* (default a normalised 10 x 10 grid of cells); one ray per
    pupil cell at a uniformly drawn point of the cell (its centre when not
    ``random``), weighted by the cell's area; the intensity of the
    unvignetted rays summed over the pupil and averaged over the field."""
    from .stops import extents, extents_many

    g = system.grid_input
    if wavelength is None:
        wavelength = None if g is None else g.wavelength
    if field is None:
        field = None if g is None else g.field
    if pupil is None:
        pupil = Cartesian2dVectorArray(np.linspace(-1, 1, 11), np.linspace(-1, 1, 11))
    w = _axis(wavelength, "wavelength")
    fx, fy = _axis(field.x, "field x"), _axis(field.y, "field y")
    vx, vy = _axis(pupil.x, "pupil x"), _axis(pupil.y, "pupil y")
    nw, npx, npy = len(w), len(vx) - 1, len(vy) - 1
    # pupil vertices at each wavelength (denormalised by the stop solver)
    if normalized_pupil:
        extents_many(system, w)  # all wavelengths in one batched solve
    PX = np.empty((nw, npx + 1))
    PY = np.empty((nw, npy + 1))
    for k in range(nw):
        if normalized_pupil:
            e = extents(system, float(w[k]))
            PX[k] = (e[3][0] - e[2][0]) * (vx + 1) / 2 + e[2][0]
            PY[k] = (e[3][1] - e[2][1]) * (vy + 1) / 2 + e[2][1]
        else:
            PX[k], PY[k] = vx, vy
    area = np.abs(np.diff(PX, axis=1)[:, :, None] * np.diff(PY, axis=1)[:, None, :])
    dev = torch.device("cuda", torch.cuda.current_device())
    shape = (nw, len(fx), len(fy), npx, npy)
    if random:
        gen = torch.Generator(device=dev)
        gen.manual_seed(int(seed))
        ux = torch.rand(shape, generator=gen, device=dev, dtype=torch.float64)
        uy = torch.rand(shape, generator=gen, device=dev, dtype=torch.float64)
    else:
        ux = uy = torch.full(shape, 0.5, device=dev, dtype=torch.float64)
    PXt = torch.as_tensor(PX, device=dev)
    PYt = torch.as_tensor(PY, device=dev)
    lox = PXt[:, :-1].reshape(nw, 1, 1, npx, 1)
    dx = (PXt[:, 1:] - PXt[:, :-1]).reshape(nw, 1, 1, npx, 1)
    loy = PYt[:, :-1].reshape(nw, 1, 1, 1, npy)
    dy = (PYt[:, 1:] - PYt[:, :-1]).reshape(nw, 1, 1, 1, npy)
    qx = (lox + dx * ux).float()
    qy = (loy + dy * uy).float()
    inten = torch.as_tensor(area, device=dev, dtype=torch.float32).reshape(nw, 1, 1, npx, npy)
    res = system.rayfunction(
        intensity=inten, wavelength=w.reshape(-1, 1, 1, 1, 1),
        field=Cartesian2dVectorArray(fx.reshape(1, -1, 1, 1, 1), fy.reshape(1, 1, -1, 1, 1)),
        pupil=Cartesian2dVectorArray(qx, qy), normalized_field=normalized_field,
        normalized_pupil=False, outputs=("px", "py", "intensity", "unvignetted"))
    rays = res.outputs
    full = shape
    for name in ("x", "y"):
        v = getattr(rays.position, name)
        if tuple(v.shape) != full:
            setattr(rays.position, name, v.expand(full))
    s = pupil_reduce(rays, nw * len(fx) * len(fy), npx * npy).reshape(
        nw, len(fx), len(fy), 6).cpu().numpy()
    a = s[..., 5].mean(axis=(1, 2))
    return InterpolatedEffectiveAreaModel(wavelength=w, area=a)
