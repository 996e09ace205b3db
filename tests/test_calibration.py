"""Calibration fits on traced rays: distortion, vignetting, effective area
(optika/systems/_sequential.py:1208-1512, optika/distortion,
optika/radiometry).

CPU: the polynomial fit against the oracle's independent restatement and
against exact polynomials (the reference's distortion docstring example:
a quadratic map is reproduced exactly at degree 2, not at degree 1); the
simple distortion model's exact inverse; interpolation of the effective
area.  GPU: the pupil reduction against NumPy, and distortion, vignetting
and effective area of the Newtonian telescope against the float64 oracle,
with the effective area of the annular pupil against pi (50^2 - 12^2).
"""

import math

import numpy as np
import pytest
import torch

import optika_gb300 as ok
from optika_gb300 import calibration, configs
from optika_gb300._polyfit import PolynomialFit
from optika_gb300.vectors import Cartesian2dVectorArray as V2
from optika_gb300.vectors import SpectralPositionalVectorArray as SP
from oracle import fits as OF

DEG = math.pi / 180


def _docstring_scene():
    w, x, y = np.meshgrid(np.linspace(500, 600, 3), np.linspace(-1, 1, 13),
                          np.linspace(-1, 1, 13), indexing="ij")
    return w, x, y


def test_fit_reproduces_polynomials_and_respects_where():
    w, x, y = _docstring_scene()
    sx = x * 10 + x**2
    sy = y * 10 + y**2 + 0.01 * (w - 550) * x
    m = ok.distortion.PolynomialDistortionModel(SP(w, V2(x, y)), V2(sx, sy), degree=2)
    out = m.distort(SP(w, V2(x, y)))
    assert np.allclose(out.position.x, sx, atol=1e-9)
    assert np.allclose(out.position.y, sy, atol=1e-9)
    lin = ok.distortion.PolynomialDistortionModel(SP(w, V2(x, y)), V2(sx, sy), degree=1)
    assert np.abs(lin.distort(SP(w, V2(x, y))).position.x - sx).max() > 0.1
    # points outside `where` do not move the fit
    bad = sx.copy()
    where = np.ones_like(sx, dtype=bool)
    where[:, :3, :] = False
    bad[~where] = 1e6
    f = PolynomialFit((w, x, y), (bad,), 2, where=where)
    assert np.allclose(f(w, x, y)[0], sx, atol=1e-8)
    # the inverse fit maps back close to the scene
    back = m.undistort(out)
    assert np.abs(back.position.x - x).max() < 0.05


def test_fit_matches_the_oracle_restatement():
    rng = np.random.default_rng(0)
    w, x, y = (rng.uniform(0, 1, 200) * s + o for s, o in ((100, 500), (2, -1), (2, -1)))
    z = np.sin(x) + np.cos(y) * (w - 550) / 50 + rng.normal(0, 0.01, 200)
    where = rng.uniform(size=200) > 0.2
    for degree in (1, 2, 3):
        a = PolynomialFit((w, x, y), (z,), degree, where=where)
        b = OF.polyfit((w, x, y), (z,), degree, where)
        t = rng.uniform(0, 1, (3, 50))
        q = (t[0] * 100 + 500, t[1] * 2 - 1, t[2] * 2 - 1)
        assert np.allclose(a(*q)[0], b(*q)[0], atol=1e-9)


def test_simple_distortion_model_is_exactly_invertible():
    m = ok.distortion.SimpleDistortionModel(plate_scale=0.5, dispersion=2.0, angle=0.3,
                                            reference=SP(550.0, V2(1.0, -2.0)))
    c = SP(np.array([550.0, 560.0, 540.0]), V2(np.array([0.0, 0.4, -1.0]),
                                               np.array([0.0, -0.2, 2.0])))
    d = m.distort(c)
    assert np.allclose([d.position.x[0], d.position.y[0]], [1.0, -2.0])
    u = m.undistort(d)
    assert np.allclose(u.position.x, c.position.x) and np.allclose(u.position.y, c.position.y)
    # 10 nm at 2 nm per length unit moves 5 along the rotated x axis
    assert np.isclose(d.position.x[1] - m.distort(SP(550.0, V2(0.4, -0.2))).position.x, 5.0)


def test_fits_need_grids():
    s = configs.newtonian()
    with pytest.raises(ValueError, match="grids"):
        s.distortion()
    with pytest.raises(ValueError, match="grids"):
        s.vignetting(wavelength=np.array([550.0]))
    with pytest.raises(ValueError, match="1-D"):
        s.distortion(np.ones((2, 2)), V2(np.zeros(3), np.zeros(3)), V2(np.zeros(3), np.zeros(3)))


def test_effective_area_interpolation():
    m = ok.radiometry.InterpolatedEffectiveAreaModel(np.array([10.0, 20.0, 30.0]),
                                                     np.array([1.0, 3.0, 2.0]))
    assert np.allclose(m(np.array([5.0, 15.0, 25.0, 35.0])), [1.0, 2.0, 2.5, 2.0])


def test_oracle_distortion_has_the_paraboloid_plate_scale():
    """The Newtonian's paraboloid (R = -800 mm) has a focal length of 400 mm:
    the mean sensor position of a field point moves 400 mm per radian of
    field angle (to 1 %: the pupil-averaged coma shifts the centroid), odd
    in the angle."""
    s = configs.newtonian()
    f = np.linspace(-0.1, 0.1, 5) * DEG
    p = np.linspace(-40.0, 40.0, 9)
    o = OF.distortion(s, np.array([550.0]), f, f, p, p)
    mx, my = o["sensor"]
    for line in (mx[0, :, 2], my[0, 2, :]):
        slope = np.polyfit(f, line, 1)[0]
        assert abs(abs(slope) / 400.0 - 1) < 0.01
        assert np.allclose(line, -line[::-1], atol=1e-9)


def test_oracle_vignetting_has_unit_mean():
    """optika/systems/_sequential_test.py:344-350: the relative illumination
    averages to one over the field points with unvignetted rays."""
    s = configs.newtonian()
    f = np.linspace(-0.12, 0.12, 5) * DEG
    p = np.linspace(-48.0, 48.0, 9)
    v = OF.vignetting(s, np.array([450.0, 650.0]), f, f, p, p)
    for k in range(2):
        assert abs(v["illumination"][k][v["where"][k]].mean() - 1) < 1e-12


# ---------------------------------------------------------------- GPU


@pytest.mark.gpu
def test_pupil_reduce_matches_numpy(cuda):
    rng = np.random.default_rng(2)
    g, p = 37, 300
    x, y = rng.normal(0, 5, (2, g * p)).astype(np.float32)
    i = rng.uniform(0, 2, g * p).astype(np.float32)
    u = rng.uniform(size=g * p) > 0.3
    rays = ok.rays.RayVectorArray(position=ok.vectors.Cartesian3dVectorArray(
        torch.from_numpy(x).to(cuda), torch.from_numpy(y).to(cuda), 0.0),
        intensity=torch.from_numpy(i).to(cuda), unvignetted=torch.from_numpy(u).to(cuda))
    s = calibration.pupil_reduce(rays, g, p).cpu().numpy()
    X, Y, I, U = (a.astype(np.float64).reshape(g, p) for a in (x, y, i, u))
    ref = np.stack([U.sum(1), (X * U).sum(1), (Y * U).sum(1), X.sum(1), Y.sum(1),
                    (I * U).sum(1)], axis=1)
    assert np.allclose(s, ref, rtol=1e-12, atol=1e-9)


def _newtonian_grid():
    w = np.array([450.0, 550.0, 650.0])
    f = np.linspace(-0.12, 0.12, 5) * DEG
    p = np.linspace(-48.0, 48.0, 17)
    return w, f, f, p, p


@pytest.mark.gpu
def test_distortion_matches_oracle(cuda):
    s = configs.newtonian()
    w, fx, fy, px, py = _newtonian_grid()
    m = s.distortion(w, V2(fx, fy), V2(px, py), normalized_field=False, normalized_pupil=False)
    o = OF.distortion(s, w, fx, fy, px, py)
    assert np.array_equal(m.where, o["where"])
    assert np.abs(m.coordinates_sensor.x - o["sensor"][0]).max() < 2e-4
    assert np.abs(m.coordinates_sensor.y - o["sensor"][1]).max() < 2e-4
    q = SP(np.array([500.0, 600.0]), V2(np.array([0.05, -0.1]) * DEG, np.array([0.0, 0.07]) * DEG))
    a = m.distort(q).position
    b = o["fit"](q.wavelength, q.position.x, q.position.y)
    assert np.abs(a.x - b[0]).max() < 2e-4 and np.abs(a.y - b[1]).max() < 2e-4


@pytest.mark.gpu
def test_vignetting_matches_oracle(cuda):
    s = configs.newtonian()
    w, fx, fy, px, py = _newtonian_grid()
    m = s.vignetting(w, V2(fx, fy), V2(px, py), normalized_field=False, normalized_pupil=False)
    o = OF.vignetting(s, w, fx, fy, px, py)
    assert np.array_equal(m.where, o["where"])
    assert np.abs(m.illumination - o["illumination"]).max() < 2 / (17 * 17)
    for k in range(len(w)):
        assert abs(m.illumination[k][m.where[k]].mean() - 1) < 1e-12
    q = SP(np.array([550.0]), V2(np.array([0.03 * DEG]), np.array([-0.05 * DEG])))
    assert abs(m(q)[0] - o["fit"](q.wavelength, q.position.x, q.position.y)[0][0]) < 1e-2


@pytest.mark.gpu
def test_effective_area_matches_oracle_and_the_annulus(cuda):
    s = configs.newtonian()
    w = np.array([500.0, 600.0])
    f = np.array([0.0])
    v = np.linspace(-50.0, 50.0, 101)
    m = s.area_effective(w, V2(f, f), V2(v, v), normalized_field=False, normalized_pupil=False,
                         random=False)
    ref = OF.area_effective_centres(s, w, f, f, v, v)
    assert np.allclose(m.area, ref, rtol=1e-4)
    annulus = math.pi * (50.0**2 - 12.0**2)
    assert np.all(np.abs(m.area / annulus - 1) < 0.02)
    r = s.area_effective(w, V2(f, f), V2(v, v), normalized_field=False, normalized_pupil=False,
                         random=True, seed=3)
    assert np.all(np.abs(r.area / annulus - 1) < 0.02)
    assert np.allclose(m(550.0), (m.area[0] + m.area[1]) / 2)


@pytest.mark.gpu
def test_normalized_grids_use_the_stops(cuda):
    s = configs.stop_newtonian()
    w = np.array([500.0, 600.0])
    f = np.linspace(-1, 1, 5)
    p = np.linspace(-1, 1, 9)
    m = s.distortion(w, V2(f, f), V2(p, p))
    fmin, fmax = s.field_min, s.field_max
    assert np.allclose(m.coordinates_scene.position.x[0, :, 0],
                       np.linspace(fmin[0], fmax[0], 5), rtol=1e-6, atol=1e-12)
    # the field stop is circular: the corners of the normalised square lie
    # outside it and all their rays are vignetted
    r2 = f[:, None] ** 2 + f[None, :] ** 2
    assert m.where[:, r2 < 0.99].all() and not m.where[:, r2 > 1.01].any()
