"""The float64 oracle against the reference's golden vectors and identities.

Pins: IMD multilayer files (optika/materials/_tests/test_multilayers.py:
178-287), vector / scalar Snell closed forms (optika/materials/_tests/
test_snells_law.py:29-120), intercept-on-sag and unit normals
(optika/sags/_tests/_abc_test.py:78-102), the grazing hyperboloid
(optika/sags/_tests/_conic_test.py:57-87), the grating deflection of the
reference's grazing spectrograph test (optika/systems/_sequential_test.py:
600-651) and the layout of the Newtonian telescope docstring
(optika/systems/_sequential.py:1850-1912).
"""

import math
import pathlib

import numpy as np
import pytest

import optika_gb300 as ok
from oracle import trace as O

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden" / "multilayer_imd.npz"
CASES = ["Si", "SiO2_50A", "SiO2_100A", "SiC_Cr"]


def golden_case(name):
    z = np.load(GOLDEN)
    wl = z[f"{name}/wavelength"]
    th = z[f"{name}/thickness"]
    nc = int(z[f"{name}/num_chemicals"])
    chems = [ok.chemicals.Chemical(wl, z[f"{name}/n{i}"], z[f"{name}/k{i}"]) for i in range(nc)]
    sigma = float(z[f"{name}/interface_width"])
    prof = (lambda: ok.materials.profiles.ErfInterfaceProfile(sigma)) if sigma > 0 else (
        lambda: None)
    layers = [ok.materials.Layer(chems[i], th[i], interface=prof()) for i in range(len(th))]
    sub = ok.materials.Layer(chems[-1], interface=prof())
    return wl, z[f"{name}/efficiency"], bool(z[f"{name}/is_mirror"]), layers, sub


@pytest.mark.parametrize("name", CASES)
def test_multilayer_vs_imd(name):
    wl, eff_file, is_mirror, layers, sub = golden_case(name)
    Rs, Rp, Ts, Tp = O.multilayer_efficiency(wl, 1.0, 1.0, layers, sub)
    eff = (Rs + Rp) / 2 if is_mirror else (Ts + Tp) / 2
    assert np.allclose(eff, eff_file, rtol=1e-4)


def test_multilayer_energy_bounds():
    rng = np.random.default_rng(0)
    wl = rng.uniform(10, 30, 200)
    cos = np.cos(rng.uniform(0, 1.2, 200))
    A = ok.materials.Layer(1 - 0.03 + 0.004j, 3.0)
    B = ok.materials.Layer(1 - 0.002 + 0.0005j, 5.0)
    stack = ok.materials.PeriodicLayerSequence([A, B], num_periods=20)
    Rs, Rp, Ts, Tp = O.multilayer_efficiency(wl, cos, 1.0, stack, ok.materials.Layer(0.98 + 0.01j))
    for R, T in [(Rs, Ts), (Rp, Tp)]:
        assert np.all(R >= 0) and np.all(R <= 1)
        assert np.all(T >= 0) and np.all(T <= 1)
        assert np.all(R + T <= 1 + 1e-12)


def test_periodic_power_equals_explicit_sequence():
    rng = np.random.default_rng(1)
    wl = rng.uniform(12, 15, 50)
    cos = np.cos(rng.uniform(0, 0.35, 50))
    A = ok.materials.Layer(0.97 + 0.002j, 4.0)
    B = ok.materials.Layer(0.999 + 0.0003j, 6.0)
    sub = ok.materials.Layer(0.95 + 0.01j)
    per = O.multilayer_efficiency(wl, cos, 1.0, ok.materials.PeriodicLayerSequence([A, B], 40), sub)
    seq = O.multilayer_efficiency(wl, cos, 1.0, [A, B] * 40, sub)
    for a, b in zip(per, seq):
        assert np.allclose(a, b, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("cos_incidence", [1.0, np.linspace(-1, 1, 7)])
@pytest.mark.parametrize("n2", [1.5, 1.5 + 0.2j, np.linspace(1, 2, 4)[:, None]])
def test_snells_law_scalar_closed_form(cos_incidence, n2):
    result = O.snells_law_scalar(cos_incidence, 1.0, n2)
    expected = np.cos(np.emath.arcsin(1.0 * np.sin(np.emath.arccos(cos_incidence)) / n2))
    assert np.allclose(result, expected)


@pytest.mark.parametrize("angles", [(0.0, 0.0), (1 * math.pi / 180, 2 * math.pi / 180)])
@pytest.mark.parametrize("n2", [1.5, np.linspace(1, 2, 4)])
@pytest.mark.parametrize("mirror", [False, True])
def test_snells_law_vector_closed_form(angles, n2, mirror):
    ax, ay, az = O.direction(*angles)
    n1 = 1.0
    ux, uy, uz = 0.0, 0.0, -1.0
    bx, by, bz = O.snells_law(ax, ay, az, n1, n2, mirror, ux, uy, uz)
    r = n1 / np.asarray(n2)
    c = -(ax * ux + ay * uy + az * uz)
    m = np.sign(c) * (2 * mirror - 1)
    t = np.sqrt(np.square(1 / r) + np.square(c) - 1.0)
    ex, ey, ez = r * (ax + (c + m * t) * ux), r * (ay + (c + m * t) * uy), r * (az + (c + m * t) * uz)
    assert np.allclose(np.sqrt(bx**2 + by**2 + bz**2), 1)
    assert np.allclose([bx, by, bz], [ex, ey, ez])
    side_in = np.sign(az * uz)
    side_out = np.sign(bz * uz)
    if mirror:
        assert np.all(side_in != side_out)
    else:
        assert np.all(side_in == side_out)


def _sags():
    return [
        ok.sags.SphericalSag(radius=100.0),
        ok.sags.SphericalSag(radius=-100.0),
        ok.sags.ConicSag(radius=-200.0, conic=0.0),
        ok.sags.ConicSag(radius=-200.0, conic=-1.0),
        ok.sags.ConicSag(radius=150.0, conic=-0.5),
        ok.sags.ConicSag(radius=-300.0, conic=0.7),
        ok.sags.ConicSag(radius=-300.0, conic=-1.8),
        ok.sags.ParabolicSag(focal_length=-150.0),
        ok.sags.ToroidalSag(radius=300.0, radius_of_rotation=500.0),
        ok.sags.ToroidalSag(radius=-400.0, radius_of_rotation=250.0),
        ok.sags.CylindricalSag(radius=100.0),
        ok.sags.CylindricalSag(radius=-100.0),
    ]


def _rays(n=500, seed=3):
    rng = np.random.default_rng(seed)
    ox = rng.uniform(-20, 20, n)
    oy = rng.uniform(-20, 20, n)
    oz = rng.uniform(-50, -5, n)
    ax = rng.uniform(-0.1, 0.1, n)
    ay = rng.uniform(-0.1, 0.1, n)
    d = O.direction(ax, ay)
    return (ox, oy, oz), d


@pytest.mark.parametrize("sag", _sags(), ids=lambda s: type(s).__name__)
def test_intercept_lies_on_sag(sag):
    o, u = _rays()
    t = O.sag_intercept(sag, o, u)
    x, y, z = (o[i] + u[i] * t for i in range(3))
    assert np.all(np.isfinite(t))
    assert np.allclose(O.sag_value(sag, x, y), z, atol=1e-9)
    # the closed form picks the root the iterative solver reaches from the
    # vertex plane (optika/sags/_tests/_abc_test.py:90-102)
    t_plane = -o[2] / u[2]
    tt = t_plane.copy()
    for _ in range(50):
        xx, yy, zz = (o[i] + u[i] * tt for i in range(3))
        f = zz - O.sag_value(sag, xx, yy)
        h = 1e-6
        xx2, yy2, zz2 = (o[i] + u[i] * (tt + h) for i in range(3))
        f2 = zz2 - O.sag_value(sag, xx2, yy2)
        tt = tt - f * h / (f2 - f)
    assert np.allclose(t, tt, atol=1e-7)


@pytest.mark.parametrize("sag", _sags() + [ok.sags.NoSag()], ids=lambda s: type(s).__name__)
def test_normals_unit_with_negative_z(sag):
    rng = np.random.default_rng(5)
    x, y = rng.uniform(-20, 20, (2, 300))
    nx, ny, nz = O.sag_normal(sag, x, y)
    assert np.allclose(nx**2 + ny**2 + nz**2, 1)
    assert np.all(nz < 0)


def test_cylinder_known_answers():
    """The cylinder is the sphere's x-z cross-section extruded along y
    (optika/sags/_cylindrical.py:75-160): an axial ray at height x meets it
    at R - sign(R) sqrt(R^2 - x^2), independent of y; a ray that misses the
    cylinder stops at the vertex plane."""
    for R in (80.0, -80.0):
        sag = ok.sags.CylindricalSag(radius=R)
        x = np.linspace(-30, 30, 13)
        y = np.linspace(-50, 50, 13)
        t = O.sag_intercept(sag, (x, y, np.full(13, -10.0)), (0 * x, 0 * x, np.ones(13)))
        z = -10.0 + t
        assert np.allclose(z, R - np.sign(R) * np.sqrt(R * R - x * x), atol=1e-12)
        sph = ok.sags.SphericalSag(radius=R)
        assert np.allclose(O.sag_value(sag, x, y), O.sag_value(sph, x, 0 * y), atol=1e-12)
        nx, ny, nz = O.sag_normal(sag, x, y)
        sx, sy, sz = O.sag_normal(sph, x, 0 * y)
        assert np.allclose((nx, ny, nz), (sx, sy, sz), atol=1e-15)
    # |x| > R: no real root, the vertex-plane intercept (o_z = -10, u_z = 1)
    sag = ok.sags.CylindricalSag(radius=20.0)
    t = O.sag_intercept(sag, (np.array([25.0]), np.array([3.0]), np.array([-10.0])),
                        (np.array([0.0]), np.array([0.0]), np.array([1.0])))
    assert np.allclose(t, 10.0)


@pytest.mark.parametrize("sag", _sags(), ids=lambda s: type(s).__name__)
def test_exact_intercept_keeps_the_reference_root(sag):
    """The exact mode polishes the root the reference's closed form picks:
    the same root to the literal form's rounding, on the sag to float64
    rounding."""
    o, u = _rays()
    t_lit = O.sag_intercept(sag, o, u)
    t_ex = O.sag_intercept(sag, o, u, exact=True)
    assert np.allclose(t_ex, t_lit, rtol=0, atol=1e-7)
    x, y, z = (o[i] + u[i] * t_ex for i in range(3))
    assert np.abs(O.sag_value(sag, x, y) - z).max() < 1e-12


def test_literal_conic_intercept_cancels_for_near_axial_rays():
    """The reference's (-B +- sqrt(B^2 - 4 A C)) / 2A (optika/sags/_conic.py:
    144-162) loses float64 digits when A = c (u_x^2 + u_y^2) is small but
    above the 1e-12 linear-branch threshold: the Newtonian primary
    (R -800 mm, k -1) with field angles of ~3e-5 rad.  The exact mode's
    point lies on the sag; the literal one can be ~1e-4 mm off it."""
    sag = ok.sags.ConicSag(radius=-800.0, conic=-1.0)
    rng = np.random.default_rng(12)
    n = 2000
    ang = rng.uniform(2.9e-5, 4e-5, n)
    phi = rng.uniform(0, 2 * np.pi, n)
    u = O.direction(ang * np.cos(phi), ang * np.sin(phi))
    r = np.sqrt(rng.uniform(12**2, 50**2, n))
    o = (r * np.cos(phi), r * np.sin(phi), np.full(n, -350.0))
    c = 1 / sag.radius
    assert np.all(np.abs(c * (u[0] ** 2 + u[1] ** 2)) > 1e-12)
    res = {}
    for exact in (False, True):
        t = O.sag_intercept(sag, o, u, exact=exact)
        x, y, z = (o[i] + u[i] * t for i in range(3))
        res[exact] = np.abs(O.sag_value(sag, x, y) - z)
    assert res[True].max() < 1e-12
    assert res[False].max() > 1e-6


def test_parabola_equals_conic():
    p = ok.sags.ParabolicSag(focal_length=-120.0)
    c = ok.sags.ConicSag(radius=-240.0, conic=-1.0)
    rng = np.random.default_rng(9)
    x, y = rng.uniform(-30, 30, (2, 100))
    assert np.allclose(O.sag_normal(p, x, y), O.sag_normal(c, x, y))
    o, u = _rays()
    assert np.allclose(O.sag_intercept(p, o, u), O.sag_intercept(c, o, u), rtol=1e-9)


def test_grazing_hyperboloid_vertex_sheet():
    sag = ok.sags.ConicSag(radius=-0.7, conic=-1.0007)
    az = np.linspace(0, 2 * np.pi, 64, endpoint=False)
    o = (68 * np.cos(az), 68 * np.sin(az), np.full(64, -2000.0))
    u = (np.zeros(64), np.zeros(64), np.ones(64))
    t = O.sag_intercept(sag, o, u)
    x, y, z = (o[i] + u[i] * t for i in range(3))
    assert np.allclose(O.sag_value(sag, x, y), z)
    c = 1 / sag.radius
    assert np.all(z * (c * (x * x + y * y) - z) >= 0)


def test_transformation_list_order_matches_reference_layout():
    deg = math.pi / 180
    fold = ok.transforms.TransformationList(
        [ok.transforms.RotationY(135 * deg), ok.transforms.Translation(z=50.0)]
    )
    sensor = ok.transforms.TransformationList(
        [ok.transforms.RotationY(-90 * deg), ok.transforms.Translation(x=-50.0, z=50.0)]
    )
    assert np.allclose(O._mat(fold)[:3, 3], [0, 0, 50])
    assert np.allclose(O._mat(sensor)[:3, 3], [-50, 0, 50])
    # a ray going -z off the fold's normal leaves along -x towards the sensor
    n = O._mat(fold)[:3, :3] @ np.array([0, 0, -1.0])
    b = O.snells_law(0.0, 0.0, -1.0, 1.0, 1.0, True, *n)
    assert np.allclose(b, [-1, 0, 0])


def test_newtonian_on_axis_focus():
    from optika_gb300 import configs

    s = configs.newtonian()
    g = configs.newtonian_grid(num_pupil=500)
    r = O.rayfunction(s, g["wavelength"], g["field_x"], g["field_y"], g["pupil_x"], g["pupil_y"])
    on = slice(12 * 500, 13 * 500)  # the central field point
    m = r["unvignetted"][on]
    assert m.mean() > 0.9
    assert np.abs(r["px"][on][m]).max() < 1e-9
    assert np.abs(r["py"][on][m]).max() < 1e-9
    assert np.allclose(r["opl"][on][m], 800.0, atol=1e-9)


def test_grating_deflection_of_grazing_spectrograph():
    """Transmission grating of the reference's grazing spectrograph test:
    first order lands (z_grating - z_sensor) * tan(asin(lambda / d)) off axis."""
    grating = ok.surfaces.Surface(
        rulings=ok.rulings.Rulings(spacing=0.010, diffraction_order=1),
        transformation=ok.transforms.Translation(z=1000.0),
    )
    sensor = ok.surfaces.Surface(transformation=ok.transforms.Translation(z=480.0))
    n = 10
    rays = O.make_rays((n,), px=np.linspace(-5, 5, n), dz=-1.0, pz=2000.0, wavelength=500.0)
    out = O.propagate_rays([grating, sensor], rays)
    expect = 520.0 * math.tan(math.asin(500e-6 / 0.010))
    assert np.allclose(out["px"] - np.linspace(-5, 5, n), expect)


def test_histogram_semantics_match_numpy():
    rng = np.random.default_rng(2)
    edges = np.linspace(-1, 1, 11)
    v = np.concatenate([rng.uniform(-1.2, 1.2, 1000), edges, [np.nan]])
    idx = O.bin_index(edges, v)
    h = np.bincount(idx[idx >= 0], minlength=10)
    ref, _ = np.histogram(v[np.isfinite(v)], bins=edges)
    assert np.array_equal(h, ref)


def test_aperture_clip_only_removes_rays():
    rng = np.random.default_rng(4)
    x, y = rng.uniform(-30, 30, (2, 1000))
    z = np.zeros_like(x)
    for ap in [ok.apertures.CircularAperture(10.0), ok.apertures.RectangularAperture((5.0, 8.0)),
               ok.apertures.EllipticalAperture((6.0, 3.0)),
               ok.apertures.CircularSectorAperture(20.0, 0.2, 2.0),
               ok.apertures.RegularPolygonalAperture(radius=15.0, num_vertices=6),
               ok.apertures.IsoscelesTrapezoidalAperture(x_left=5.0, x_right=20.0, angle=0.6)]:
        m = O.aperture_mask(ap, x, y, z)
        assert 0 < m.sum() < m.size
        ap.inverted = True
        assert np.array_equal(O.aperture_mask(ap, x, y, z), ~m)
        ap.inverted = False
        ap.active = False
        assert O.aperture_mask(ap, x, y, z).all()
