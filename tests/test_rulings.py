"""Ruling models: groove efficiencies and effective incidence.

CPU: the float64 oracle pinned to the published thin-grating results the
reference cites (Magnusson and Gaylord 1978, Table 1) and to the
reference's own property tests (optika/rulings/_rulings_test.py:10-74:
efficiency within [0, 1] for its rays and models, incident_effective
changes the rays), plus the lowering of each model.

GPU: the groove efficiency multiplied into the traced intensity, the
``efficiency`` and ``incident_effective`` methods, all against the oracle.
"""

import math

import numpy as np
import pytest
import torch

import optika_gb300 as ok
from optika_gb300 import _lib as L
from optika_gb300._lower import lower_surfaces
from optika_gb300.vectors import Cartesian3dVectorArray as V3
from optika_gb300.vectors import FunctionArray, SpectralDirectionalVectorArray
from oracle import trace as O

SPACING = 1e-3  # 1 um in mm
DEPTH = 1e-5  # 10 nm in mm


def _models(order, depth=DEPTH, spacing=SPACING):
    return {
        "sinusoidal": ok.rulings.SinusoidalRulings(spacing=spacing, depth=depth,
                                                   diffraction_order=order),
        "square": ok.rulings.SquareRulings(spacing=spacing, depth=depth, diffraction_order=order),
        "sawtooth": ok.rulings.SawtoothRulings(spacing=spacing, depth=depth,
                                               diffraction_order=order),
        "triangular": ok.rulings.TriangularRulings(spacing=spacing, depth=depth,
                                                   diffraction_order=order),
        "rectangular": ok.rulings.RectangularRulings(spacing=spacing, depth=depth,
                                                     ratio_duty=0.3, diffraction_order=order),
    }


def _measured(order=1, wl=None, center=0.0, width=1.0):
    """The reference's test measurement (100-300 Angstrom, in nm) or a
    Gaussian of the given center and width over ``wl``."""
    wl = np.linspace(10.0, 30.0, 11) if wl is None else wl
    return ok.rulings.MeasuredRulings(
        spacing=SPACING, diffraction_order=order,
        efficiency_measured=FunctionArray(
            inputs=SpectralDirectionalVectorArray(wavelength=wl, direction=V3(0.0, 0.0, 1.0)),
            outputs=np.exp(-np.square((wl - center) / width) / 2)))


def _normal_incidence(wavelength):
    wavelength = np.atleast_1d(np.asarray(wavelength, dtype=np.float64))
    z = np.zeros_like(wavelength)
    return O.make_rays(wavelength.shape, px=z, py=z, pz=z, dx=z, dy=z, dz=z + 1,
                       wavelength=wavelength)


def _eff(rulings, rays, normal=(0.0, 0.0, -1.0)):
    return O.ruling_efficiency(rulings, rays, *normal)


# ---------------------------------------------------------------- oracle pins


def test_square_known_answers():
    """gamma = 1 (depth = lambda / 4 at normal incidence): first order
    4 / pi^2 = 40.5%, zeroth order cos^2(pi / 2) = 0, even orders 0, third
    order 4 / (9 pi^2)."""
    wl = 500.0
    depth = wl / 4 * 1e-6
    r = _normal_incidence(wl)
    expect = {0: 0.0, 1: 4 / math.pi**2, 2: 0.0, 3: 4 / (9 * math.pi**2), -1: 4 / math.pi**2}
    for m, e in expect.items():
        v = _eff(ok.rulings.SquareRulings(spacing=SPACING, depth=depth, diffraction_order=m), r)
        assert np.allclose(v, e, atol=1e-12), m


def test_rectangular_half_duty_equals_square():
    """A rectangular profile of duty 1/2 is the square profile."""
    rng = np.random.default_rng(1)
    r = _normal_incidence(rng.uniform(100, 900, 50))
    r["dx"] = rng.uniform(-0.2, 0.2, 50)
    for m in (0, 1, 2, 3, -1):
        sq = ok.rulings.SquareRulings(spacing=SPACING, depth=8e-5, diffraction_order=m)
        re = ok.rulings.RectangularRulings(spacing=SPACING, depth=8e-5, ratio_duty=0.5,
                                           diffraction_order=m)
        assert np.allclose(_eff(sq, r), _eff(re, r), atol=1e-12), m


def test_sawtooth_blaze():
    """The blazed (sawtooth) thin grating puts all the light into the order
    m = -gamma: gamma -> 1 for m = -1."""
    wl = 500.0
    depth = wl / 2 * 1e-6 * (1 - 1e-7)  # gamma = 1 - 1e-7
    r = _normal_incidence(wl)
    v = _eff(ok.rulings.SawtoothRulings(spacing=SPACING, depth=depth, diffraction_order=-1), r)
    assert np.allclose(v, 1.0, atol=1e-10)
    v = _eff(ok.rulings.SawtoothRulings(spacing=SPACING, depth=depth, diffraction_order=0), r)
    assert np.allclose(v, 0.0, atol=1e-6)


def test_sinusoidal_returns_bessel_itself():
    """The reference's code returns J_m(2 gamma) (its docstring writes J_m^2):
    at 2 gamma = 1.8412, the first maximum of J_1, that is 0.5819."""
    wl = 400.0
    depth = 1.8412 / 2 * wl / math.pi * 1e-6
    r = _normal_incidence(wl)
    v = _eff(ok.rulings.SinusoidalRulings(spacing=SPACING, depth=depth, diffraction_order=1), r)
    assert np.allclose(v, 0.58187, atol=1e-4)
    v = _eff(ok.rulings.SinusoidalRulings(spacing=SPACING, depth=depth, diffraction_order=-1), r)
    assert np.allclose(v, -0.58187, atol=1e-4)


def test_triangular_zeroth_order_limit():
    """Shallow grooves leave the light in order 0 of every profile; the
    triangular zeroth order is (gamma sin(pi^2 gamma / 4) / (pi gamma / 2)^2)^2
    -> 1 as gamma -> 0."""
    r = _normal_incidence(500.0)
    for name, model in _models(0, depth=1e-9).items():
        v = _eff(model, r)
        assert np.allclose(v, 1.0, atol=1e-4), name


def test_direction_scalar_quirk():
    """cos_theta = -(a - (a . q)).n with the scalar a . q subtracted from
    every component (optika/rulings/_rulings.py:444-446): for the ruling
    normal x on the plane z = 0, q = (0, -1, 0) and cos_theta = a_z + a_y."""
    wl, ay = 500.0, 0.2
    r = _normal_incidence(wl)
    r["dy"] = np.array([ay])
    r["dz"] = np.array([math.sqrt(1 - ay * ay)])
    cos_t = r["dz"][0] + ay
    depth = 2e-4
    g = math.pi * (depth * 1e6 / (math.pi / 4)) / (wl * cos_t)
    v = _eff(ok.rulings.SquareRulings(spacing=SPACING, depth=depth, diffraction_order=0), r)
    assert np.allclose(v, math.cos(math.pi * g / 2) ** 2, atol=1e-12)


def test_measured_interpolates_and_clamps():
    ru = _measured()
    m = ru.efficiency_measured
    r = _normal_incidence(np.concatenate([m.inputs.wavelength, [5.0, 40.0, 15.0]]))
    v = _eff(ru, r)
    out = np.asarray(m.outputs)
    assert np.allclose(v[:11], out)
    assert np.allclose(v[11:13], [out[0], out[-1]])
    assert np.allclose(v[13], (out[2] + out[3]) / 2)


@pytest.mark.parametrize("order", [0, 1, 2])
@pytest.mark.parametrize("name", ["sinusoidal", "square", "sawtooth", "triangular",
                                  "rectangular", "measured", "ideal"])
def test_reference_property_bounds(name, order):
    """optika/rulings/_rulings_test.py:55-74 and its rays
    (optika/rays/_tests/test_ray_vectors.py:11-38), normal (0, 0, -1)."""
    if name == "measured":
        ru = _measured(order)
    elif name == "ideal":
        ru = ok.rulings.Rulings(spacing=SPACING, diffraction_order=order)
    else:
        ru = _models(order)[name]
    n = 11
    ang = np.deg2rad(np.linspace(-1, 1, n))
    rays = [
        O.make_rays((1,), px=0.0, py=1.0, pz=2.0, dx=0.0, dy=0.0, dz=1.0, wavelength=500.0),
        O.make_rays((n,), px=np.linspace(-10, 10, n), py=np.linspace(-10, 10, n),
                    pz=np.linspace(-10, 10, n), dx=np.sin(ang), dy=0.0, dz=np.cos(ang),
                    wavelength=np.linspace(400, 500, n), n=np.linspace(1, 1.5, n)),
    ]
    for r in rays:
        eff = np.broadcast_to(_eff(ru, r), r["px"].shape)
        assert np.all(eff >= 0) and np.all(eff <= 1)
        out = O.incident_effective(r, ru, 0.0, 0.0, -1.0)
        changed = any(not np.array_equal(out[k], r[k]) for k in ("dx", "dy", "dz"))
        assert changed == (order != 0)


# ---------------------------------------------------------------- lowering


def test_lowering_of_models():
    surfaces = [ok.surfaces.Surface(rulings=ru) for ru in _models(1).values()]
    surfaces.append(ok.surfaces.Surface(rulings=_measured()))
    surfaces.append(ok.surfaces.Surface(rulings=ok.rulings.Rulings(spacing=SPACING)))
    lw = lower_surfaces(surfaces, pre=np.eye(4), final=None, input_mode=L.INPUT_RAYS)
    S = lw.sys.surfaces
    tags = [S[k].rule_eff_type for k in range(len(surfaces))]
    assert tags == [L.RULE_EFF_SINUSOIDAL, L.RULE_EFF_SQUARE, L.RULE_EFF_SAWTOOTH,
                    L.RULE_EFF_TRIANGULAR, L.RULE_EFF_RECTANGULAR, L.RULE_EFF_MEASURED,
                    L.RULE_EFF_IDEAL]
    amp = [1.0, math.pi / 4, math.pi / 2, math.pi**2 / 8,
           math.pi / (2 * math.sqrt(2 * (1 - math.cos(2 * math.pi * 0.3))))]
    for k, a in enumerate(amp):
        assert np.isclose(S[k].rule_depth, DEPTH * 1e6 / a, rtol=1e-6)
    assert np.isclose(S[4].rule_duty, 2 * math.pi * 0.3, rtol=1e-6)
    assert S[5].rule_table == 0 and len(lw.table_list) == 1
    assert S[6].rule_efficiency == 1.0


def test_lowering_rejects_what_the_reference_rejects():
    bad = _measured()
    bad.efficiency_measured.inputs.direction = V3(np.zeros(2), np.zeros(2), np.ones(2))
    with pytest.raises(ValueError, match="incidence angles"):
        lower_surfaces([ok.surfaces.Surface(rulings=bad)], pre=np.eye(4), final=None,
                       input_mode=L.INPUT_RAYS)
    bad = _measured()
    bad.efficiency_measured.inputs.wavelength = np.ones((2, 3))
    with pytest.raises(ValueError, match="one dimensional"):
        lower_surfaces([ok.surfaces.Surface(rulings=bad)], pre=np.eye(4), final=None,
                       input_mode=L.INPUT_RAYS)
    half = ok.rulings.SinusoidalRulings(spacing=SPACING, depth=DEPTH, diffraction_order=0.5)
    with pytest.raises(NotImplementedError, match="integer"):
        lower_surfaces([ok.surfaces.Surface(rulings=half)], pre=np.eye(4), final=None,
                       input_mode=L.INPUT_RAYS)


# ---------------------------------------------------------------- GPU parity


def _grating_rays(n=4000, seed=17):
    rng = np.random.default_rng(seed)
    px, py = rng.uniform(-20, 20, (2, n))
    dx, dy, dz = O.direction(rng.uniform(-0.15, 0.15, n), rng.uniform(-0.15, 0.15, n))
    wl = rng.uniform(100, 400, n)  # order 2 stays propagating: 2 lambda / d <= 0.8
    r = O.make_rays((n,), px=px, py=py, pz=np.full(n, -100.0), dx=dx, dy=dy, dz=dz,
                    wavelength=wl)
    for k in ("px", "py", "pz", "dx", "dy", "dz", "wavelength"):
        r[k] = r[k].astype(np.float32).astype(np.float64)
    return r


def _gpu(surfaces, r):
    from optika_gb300 import _api

    rays = ok.rays.RayVectorArray(
        wavelength=r["wavelength"], position=V3(r["px"], r["py"], r["pz"]),
        direction=V3(r["dx"], r["dy"], r["dz"]), intensity=r["intensity"],
        attenuation=r["attenuation"], index_refraction=r["n"], unvignetted=r["unvignetted"])
    out = _api.propagate_rays(surfaces, rays)
    torch.cuda.synchronize()
    return out.numpy()


def _gpu_cases():
    cases = []
    for order in (0, 1, 2, -1):
        for name, ru in _models(order, depth=1.5e-4).items():
            cases.append((f"{name}[{order}]", ru))
    cases.append(("measured[1]", _measured(1, np.linspace(90.0, 410.0, 33), 250.0, 60.0)))
    return cases


@pytest.mark.gpu
@pytest.mark.parametrize("case", _gpu_cases(), ids=lambda c: c[0])
def test_efficiency_in_trace(cuda, case):
    """A ruled concave mirror: the traced intensity carries the groove
    efficiency of the model (float32 against the float64 oracle)."""
    _, ru = case
    grating = ok.surfaces.Surface(sag=ok.sags.SphericalSag(-500.0),
                                  material=ok.materials.Mirror(), rulings=ru)
    det = ok.surfaces.Surface(transformation=ok.transforms.Translation(z=-250.0))
    r = _grating_rays()
    ref = O.propagate_rays([grating, det], r)
    out = _gpu([grating, det], r)
    m = np.isfinite(ref["px"]) & np.isfinite(ref["intensity"])
    assert m.mean() > 0.99
    err = np.abs(out["intensity"][m] - ref["intensity"][m])
    assert (err <= 2e-5 + 1e-4 * np.abs(ref["intensity"][m])).all(), err.max()
    # strongly diffracted rays travel ~300 mm at up to ~55 degrees: FP32
    # direction rounding (~1e-7 relative) scales with the distance
    assert (np.abs(out["px"][m] - ref["px"][m]) <= 2e-4 + 5e-6 * np.abs(ref["px"][m])).all()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sinusoidal", "square", "sawtooth", "triangular",
                                  "rectangular", "measured", "ideal"])
def test_efficiency_and_incident_effective_methods(cuda, name):
    rng = np.random.default_rng(9)
    n = 2000
    if name == "measured":
        ru = _measured(2, np.linspace(20.0, 680.0, 34), 300.0, 150.0)
    elif name == "ideal":
        ru = ok.rulings.Rulings(spacing=ok.rulings.Polynomial1dRulingSpacing({0: 1e-3, 1: 2e-6}),
                                diffraction_order=2)
    else:
        ru = _models(2, depth=1.2e-4)[name]
    px, py = rng.uniform(-20, 20, (2, n))
    pz = np.zeros(n)
    dx, dy, dz = O.direction(rng.uniform(-0.3, 0.3, n), rng.uniform(-0.3, 0.3, n))
    nx, ny, nz = O.direction(rng.uniform(-0.1, 0.1, n), rng.uniform(-0.1, 0.1, n))
    nz = -nz
    wl = rng.uniform(5, 700, n)
    idx = rng.uniform(1.0, 1.5, n)
    f32 = lambda a: a.astype(np.float32).astype(np.float64)  # noqa: E731
    px, py, dx, dy, dz, nx, ny, nz, wl, idx = map(f32, (px, py, dx, dy, dz, nx, ny, nz, wl, idx))
    r = O.make_rays((n,), px=px, py=py, pz=pz, dx=dx, dy=dy, dz=dz, wavelength=wl, n=idx)
    rays = ok.rays.RayVectorArray(wavelength=wl, position=V3(px, py, pz),
                                  direction=V3(dx, dy, dz), index_refraction=idx)
    normal = V3(nx, ny, nz)
    eff = ru.efficiency(rays, normal).cpu().numpy()
    ref = np.broadcast_to(O.ruling_efficiency(ru, r, nx, ny, nz), (n,))
    fin = np.isfinite(ref)
    assert fin.mean() > 0.99
    assert np.array_equal(np.isfinite(eff), fin)
    err = np.abs(eff[fin] - ref[fin])
    assert (err <= 2e-5 + 1e-4 * np.abs(ref[fin])).all(), err.max()
    out = ru.incident_effective(rays, normal)
    o = O.incident_effective(r, ru, nx, ny, nz)
    for k, v in (("dx", out.direction.x), ("dy", out.direction.y), ("dz", out.direction.z)):
        assert np.abs(v.cpu().numpy() - o[k]).max() < 2e-6, k


@pytest.mark.gpu
def test_invalid_measured_table_is_refused(cuda):
    """A measured-efficiency table index outside the pool is refused on the
    host before any launch."""
    from optika_gb300 import _api

    ru = _measured()
    lw = lower_surfaces([ok.surfaces.Surface(rulings=ru)], pre=np.eye(4), final=None,
                        input_mode=L.INPUT_RAYS, device=cuda)
    lw.sys.surfaces[0].rule_table = 99
    n = 4
    z = torch.zeros(n, device=cuda)
    rs = _api._rays_struct(dict(px=z, py=z, pz=z, dx=z, dy=z, dz=z + 1, wavelength=z + 20), n)
    ns = _api._rays_struct(dict(dx=z, dy=z, dz=z - 1), n)
    eff = torch.empty(n, device=cuda)
    lib = L.load()
    import ctypes

    st = lib.otx_rulings_eval(ctypes.byref(lw.sys), 0, ctypes.byref(rs), ctypes.byref(ns),
                              _api.ptr(eff), None, _api.stream_handle())
    assert st == L.ERR_INVALID
