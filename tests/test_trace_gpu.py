"""Parity of the CUDA trace (through the C-ABI) with the float64 oracle.

Tolerances (FP32 trace against float64, stated here and in the design
notes): sensor-plane positions within 1.5e-4 mm per ray (0.011 px of
13.5 um) and 3e-5 mm RMS; directions within 2e-6; optical path length
within 1e-3 mm; vignetting masks identical except for rays within 1e-5 mm
of an aperture edge; pixel indices identical for rays farther than
EDGE_PX from a pixel edge (the measured per-ray bound of the FP32 trace).
"""

import math

import numpy as np
import pytest
import torch

import optika_gb300 as ok
from optika_gb300 import _api, _lib, configs
from oracle import trace as O

pytestmark = pytest.mark.gpu

V2 = ok.vectors.Cartesian2dVectorArray
V3 = ok.vectors.Cartesian3dVectorArray
PIX = 0.0135
EDGE_PX = 1e-3


def f32(g: dict) -> dict:
    """Inputs rounded to float32, the values the kernel sees; the oracle is
    given the same values so that only arithmetic differs."""
    return {k: np.asarray(v, dtype=np.float32).astype(np.float64) for k, v in g.items()}


def c32(z: complex) -> complex:
    return complex(np.float32(z.real), np.float32(z.imag))


def run_rayfunction(system, g, **kw):
    res = system.rayfunction(
        wavelength=g["wavelength"], field=V2(g["field_x"], g["field_y"]),
        pupil=V2(g["pupil_x"], g["pupil_y"]), normalized_field=False, normalized_pupil=False,
        **kw,
    )
    torch.cuda.synchronize()
    return res


def oracle_rayfunction(system, g):
    return O.rayfunction(system, g["wavelength"], g["field_x"], g["field_y"], g["pupil_x"],
                         g["pupil_y"])


def assert_rays_close(out, ref, pos_tol=1.5e-4, dir_tol=2e-6, opl_tol=1e-3, rms_tol=3e-5):
    m = ref["unvignetted"]
    assert np.array_equal(out["unvignetted"], m)
    e = np.hypot(out["px"][m] - ref["px"][m], out["py"][m] - ref["py"][m])
    assert e.max() < pos_tol, e.max()
    assert np.sqrt(np.mean(e**2)) < rms_tol
    for k in ("dx", "dy", "dz"):
        assert np.abs(out[k][m] - ref[k][m]).max() < dir_tol, k
    assert np.abs(out["opl"][m] - ref["opl"][m]).max() < opl_tol
    assert np.allclose(out["intensity"][m], ref["intensity"][m], rtol=2e-6, atol=1e-7)


def test_newtonian_small_workload(cuda):
    s = configs.newtonian()
    g = f32(configs.newtonian_grid())
    res = run_rayfunction(s, g, image=True)
    out = res.outputs.numpy()
    ref = oracle_rayfunction(s, g)
    assert_rays_close(out, ref)
    counts, flux = (t.cpu().numpy() for t in res.image)
    c_ref, f_ref = O.collect(s.sensor, ref)
    assert counts.sum() == c_ref.sum()
    # per-ray pixel indices agree away from pixel edges
    ex, ey = O.histogram_edges(s.sensor)
    m = ref["unvignetted"]
    fx = (ref["px"][m] - ex[0]) / PIX
    fy = (ref["py"][m] - ey[0]) / PIX
    far = (np.abs(fx - np.round(fx)) > EDGE_PX) & (np.abs(fy - np.round(fy)) > EDGE_PX)
    # the on-axis field point focuses onto the central pixel corner
    assert far.mean() > 0.9
    ix_g = O.bin_index(ex, out["px"][m][far])
    iy_g = O.bin_index(ey, out["py"][m][far])
    ix_r = O.bin_index(ex, ref["px"][m][far])
    iy_r = O.bin_index(ey, ref["py"][m][far])
    assert np.array_equal(ix_g, ix_r) and np.array_equal(iy_g, iy_r)
    # the kernel's own bins equal a float64 histogram of its outputs except
    # for rays on an edge
    c_own, _ = O.collect(s.sensor, out)
    assert np.abs(counts - c_own).sum() <= 2 * np.count_nonzero(~far)
    assert np.allclose(flux.sum(), f_ref.sum(), rtol=1e-5)


def test_accumulate_matches_per_surface(cuda):
    s = configs.newtonian()
    g = f32(configs.newtonian_grid(num_pupil=400))
    res = s.raytrace(wavelength=g["wavelength"], field=V2(g["field_x"], g["field_y"]),
                     pupil=V2(g["pupil_x"], g["pupil_y"]), normalized_field=False,
                     normalized_pupil=False, accumulate=True)
    out = res.outputs.numpy()
    ref = O.raytrace(s, g["wavelength"], g["field_x"], g["field_y"], g["pupil_x"], g["pupil_y"])
    assert out["px"].shape[0] == 5
    for k in range(5):
        m = ref[k]["unvignetted"]
        assert np.array_equal(out["unvignetted"][k], m)
        for c in ("px", "py", "pz"):
            # global-frame coordinates up to ~400 mm: FP32 output rounding
            assert np.abs(out[c][k][m] - ref[k][c][m]).max() < 1e-4 + 2e-7 * np.abs(ref[k][c][m]).max()


def test_precision_workload_error_budget(cuda):
    s = configs.newtonian(coated=True)
    g = f32(configs.precision_grid(200_000))
    out = run_rayfunction(s, g).outputs.numpy()
    ref = oracle_rayfunction(s, g)
    assert_rays_close(out, ref)
    m = ref["unvignetted"]
    assert np.allclose(out["intensity"][m], ref["intensity"][m], rtol=1e-5, atol=1e-6)


def test_rays_input_equals_grid_input(cuda):
    s = configs.newtonian()
    g = f32(configs.newtonian_grid(num_pupil=100))
    a = run_rayfunction(s, g).outputs.numpy()
    rin = O.input_rays(s, g["wavelength"], g["field_x"], g["field_y"], g["pupil_x"], g["pupil_y"])
    rays = ok.rays.RayVectorArray(
        wavelength=rin["wavelength"], position=V3(rin["px"], rin["py"], rin["pz"]),
        direction=V3(rin["dx"], rin["dy"], rin["dz"]))
    out = _api.propagate_rays(s.surfaces_all, rays)
    torch.cuda.synchronize()
    b = out.numpy()
    # propagate_rays returns the parent frame; move to the sensor frame
    ref = O.propagate_rays(s.surfaces_all, rin)
    m = ref["unvignetted"]
    assert np.array_equal(b["unvignetted"], m)
    assert np.abs(b["pz"][m] - ref["pz"][m]).max() < 1e-4
    assert np.array_equal(a["unvignetted"], m)


def _single_surface_rays(n=4000, seed=11, spread=0.15):
    rng = np.random.default_rng(seed)
    px = rng.uniform(-25, 25, n)
    py = rng.uniform(-25, 25, n)
    pz = np.full(n, -100.0)
    dx, dy, dz = O.direction(rng.uniform(-spread, spread, n), rng.uniform(-spread, spread, n))
    wl = rng.uniform(400, 700, n)
    r = O.make_rays((n,), px=px, py=py, pz=pz, dx=dx, dy=dy, dz=dz, wavelength=wl)
    for k in ("px", "py", "pz", "dx", "dy", "dz", "wavelength"):
        r[k] = r[k].astype(np.float32).astype(np.float64)
    return r


def _gpu_propagate(surfaces, r):
    rays = ok.rays.RayVectorArray(
        wavelength=r["wavelength"], position=V3(r["px"], r["py"], r["pz"]),
        direction=V3(r["dx"], r["dy"], r["dz"]), intensity=r["intensity"],
        attenuation=r["attenuation"], index_refraction=r["n"], unvignetted=r["unvignetted"])
    out = _api.propagate_rays(surfaces, rays)
    torch.cuda.synchronize()
    return out.numpy()


SURFACES = {
    "sphere_mirror": ok.surfaces.Surface(sag=ok.sags.SphericalSag(-400.0),
                                         material=ok.materials.Mirror()),
    "convex_sphere": ok.surfaces.Surface(sag=ok.sags.SphericalSag(300.0),
                                         material=ok.materials.Mirror()),
    "conic_hyperbola": ok.surfaces.Surface(sag=ok.sags.ConicSag(-500.0, -1.6),
                                           material=ok.materials.Mirror()),
    "conic_ellipse": ok.surfaces.Surface(sag=ok.sags.ConicSag(400.0, -0.4),
                                         material=ok.materials.Mirror()),
    "parabola": ok.surfaces.Surface(sag=ok.sags.ParabolicSag(-250.0),
                                    material=ok.materials.Mirror()),
    "toroid": ok.surfaces.Surface(sag=ok.sags.ToroidalSag(600.0, 900.0),
                                  material=ok.materials.Mirror()),
    "cylinder_mirror": ok.surfaces.Surface(sag=ok.sags.CylindricalSag(-400.0),
                                           material=ok.materials.Mirror()),
    "cylinder_lens": ok.surfaces.Surface(sag=ok.sags.CylindricalSag(250.0),
                                         material=ok.materials.Glass.n_bk7()),
    "glass_lens": ok.surfaces.Surface(sag=ok.sags.SphericalSag(200.0),
                                      material=ok.materials.Glass.n_bk7()),
    "tilted_flat": ok.surfaces.Surface(
        material=ok.materials.Mirror(),
        transformation=ok.transforms.TransformationList(
            [ok.transforms.RotationX(0.3), ok.transforms.RotationZ(0.5),
             ok.transforms.Translation(x=3.0, y=-2.0, z=40.0)])),
}


@pytest.mark.parametrize("name", sorted(SURFACES))
def test_surface_types(cuda, name):
    surface = SURFACES[name]
    det = ok.surfaces.Surface(transformation=ok.transforms.Translation(z=-300.0))
    r = _single_surface_rays()
    ref = O.propagate_rays([surface, det], r)
    out = _gpu_propagate([surface, det], r)
    m = ref["unvignetted"] & np.isfinite(ref["px"])
    assert m.mean() > 0.9
    assert np.abs(out["px"][m] - ref["px"][m]).max() < 2e-4
    assert np.abs(out["py"][m] - ref["py"][m]).max() < 2e-4
    for k in ("dx", "dy", "dz"):
        assert np.abs(out[k][m] - ref[k][m]).max() < 3e-6, k
    assert np.allclose(out["wavelength"][m], ref["wavelength"][m], rtol=1e-6)


APERTURES = {
    "circular": ok.apertures.CircularAperture(18.0),
    "circular_inverted": ok.apertures.CircularAperture(8.0, inverted=True),
    "inactive": ok.apertures.CircularAperture(1.0, active=False),
    "rectangular": ok.apertures.RectangularAperture((15.0, 9.0)),
    "elliptical": ok.apertures.EllipticalAperture((20.0, 10.0)),
    "sector": ok.apertures.CircularSectorAperture(22.0, -0.5, 2.0),
    "polygon": ok.apertures.PolygonalAperture([(0, 0), (20, 3), (5, 18), (-15, 10)]),
    "octagon": ok.apertures.OctagonalAperture(radius=17.0),
    "trapezoid": ok.apertures.IsoscelesTrapezoidalAperture(x_left=3.0, x_right=20.0, angle=1.0),
    "translated": ok.apertures.CircularAperture(
        10.0, transformation=ok.transforms.Translation(x=5.0, y=-3.0)),
    "direction": ok.apertures.CircularAperture(0.08, dimensionless=True),
}


@pytest.mark.parametrize("name", sorted(APERTURES))
def test_apertures(cuda, name):
    ap = APERTURES[name]
    surface = ok.surfaces.Surface(aperture=ap)
    r = _single_surface_rays(seed=13)
    ref = O.propagate_rays([surface], r)
    out = _gpu_propagate([surface], r)
    diff = out["unvignetted"] != ref["unvignetted"]
    # only rays within ~1e-5 of an edge may differ
    assert diff.sum() <= max(2, int(1e-3 * diff.size))
    assert 0 < ref["unvignetted"].mean() <= 1


@pytest.mark.parametrize("kind", ["constant", "polynomial", "holographic"])
def test_rulings(cuda, kind):
    if kind == "constant":
        spacing = ok.rulings.ConstantRulingSpacing(constant=1 / 1200, normal=(1.0, 0.0, 0.0))
    elif kind == "polynomial":
        d0 = 1 / 2400
        spacing = ok.rulings.Polynomial1dRulingSpacing(
            {0: d0, 1: d0 * 1e-4, 2: d0 * 1e-7}, normal=(1.0, 0.0, 0.0),
            transformation=ok.transforms.Translation(x=2.0))
    else:
        spacing = ok.rulings.HolographicRulingSpacing(
            x1=(-300.0, 0.0, -800.0), x2=(250.0, 10.0, -900.0), wavelength=441.6)
    surface = ok.surfaces.Surface(
        sag=ok.sags.SphericalSag(-1000.0), material=ok.materials.Mirror(),
        rulings=ok.rulings.Rulings(spacing=spacing, diffraction_order=1))
    det = ok.surfaces.Surface(transformation=ok.transforms.Translation(z=-500.0))
    r = _single_surface_rays(seed=17, spread=0.05)
    r["wavelength"] = np.linspace(58, 63, r["px"].size).astype(np.float32).astype(np.float64)
    ref = O.propagate_rays([surface, det], r)
    out = _gpu_propagate([surface, det], r)
    m = ref["unvignetted"] & np.isfinite(ref["px"])
    assert m.mean() > 0.9
    for k in ("dx", "dy", "dz"):
        assert np.abs(out[k][m] - ref[k][m]).max() < 3e-6, k
    assert np.abs(out["px"][m] - ref["px"][m]).max() < 5e-4


@pytest.mark.parametrize("name", ["Si", "SiO2_50A", "SiO2_100A", "SiC_Cr"])
def test_multilayer_vs_imd_golden(cuda, name):
    from tests.test_oracle import golden_case

    wl, eff_file, is_mirror, layers, sub = golden_case(name)
    R, T = ok.multilayer_efficiency(wl, 1.0, 1.0, layers, sub)
    eff = (R.average if is_mirror else T.average).cpu().numpy()
    assert np.allclose(eff, eff_file, rtol=1e-4, atol=1e-8)


def test_multilayer_periodic_vs_oracle(cuda):
    rng = np.random.default_rng(4)
    n = 20000
    wl = rng.uniform(12, 15, n).astype(np.float32).astype(np.float64)
    cos = np.cos(rng.uniform(0, 20 * math.pi / 180, n)).astype(np.float32).astype(np.float64)
    d = 10.0
    A = ok.materials.Layer(c32(1 - 0.02 + 0.004j), 0.4 * d)
    B = ok.materials.Layer(c32(1 - 0.002 + 0.0006j), 0.6 * d)
    stack = ok.materials.PeriodicLayerSequence([A, B], num_periods=40)
    sub = ok.materials.Layer(c32(1 - 0.03 + 0.01j))
    R, T = ok.multilayer_efficiency(wl, cos, 1.0, stack, sub)
    Rs, Rp, Ts, Tp = O.multilayer_efficiency(wl, cos, 1.0, stack, sub)
    assert np.abs(R.s.cpu().numpy() - Rs).max() < 1e-5
    assert np.abs(R.p.cpu().numpy() - Rp).max() < 1e-5
    assert np.abs(T.s.cpu().numpy() - Ts).max() < 1e-5
    assert np.abs(T.p.cpu().numpy() - Tp).max() < 1e-5


def test_multilayer_film_and_table_interp(cuda):
    rng = np.random.default_rng(8)
    n = 5000
    chem = ok.chemicals.Chemical(wavelength=[10.0, 20.0, 35.0, 50.0],
                                 n=np.float32([0.9, 0.95, 0.97, 0.99]),
                                 k=np.float32([0.05, 0.02, 0.01, 0.004]))
    wl = rng.uniform(5, 60, n).astype(np.float32).astype(np.float64)  # includes clamped ends
    cos = np.cos(rng.uniform(0, 1.0, n)).astype(np.float32).astype(np.float64)
    layers = [ok.materials.Layer(chem, 15.0), ok.materials.Layer(c32(0.98 + 0.003j), 7.0)]
    R, T = ok.multilayer_efficiency(wl, cos, 1.0, layers, None)
    Rs, Rp, Ts, Tp = O.multilayer_efficiency(wl, cos, 1.0, layers, None)
    assert np.abs(T.average.cpu().numpy() - (Ts + Tp) / 2).max() < 1e-5
    assert np.abs(R.average.cpu().numpy() - (Rs + Rp) / 2).max() < 1e-5


def test_collect_matches_oracle(cuda):
    s = configs.newtonian()
    g = configs.newtonian_grid(num_pupil=500)
    ref = oracle_rayfunction(s, g)
    rays = ok.rays.RayVectorArray(
        wavelength=ref["wavelength"], position=V3(ref["px"], ref["py"], ref["pz"]),
        direction=V3(ref["dx"], ref["dy"], ref["dz"]), intensity=ref["intensity"],
        unvignetted=ref["unvignetted"])
    counts, flux = s.sensor.collect_counts(rays)
    c_ref, f_ref = O.collect(s.sensor, ref)
    ex, ey = O.histogram_edges(s.sensor)
    fx = (ref["px"] - ex[0]) / PIX
    near = np.abs(fx - np.round(fx)) < 1e-3
    assert np.abs(counts.cpu().numpy() - c_ref).sum() <= 2 * near.sum()
    wbins = (540.0, 560.0, 4)
    cw, fw = s.sensor.collect_counts(rays, wavelength=wbins)
    cw_ref, _ = O.collect(s.sensor, ref, wavelength_bins=wbins)
    assert cw.shape == (4, 1024, 1024)
    assert cw.sum().item() == cw_ref.sum()


def test_collect_image_and_direction(cuda):
    """The reference's (image, direction) pair: intensity image and the
    flux-weighted mean cosine of incidence per pixel (ideal sensor
    material), from otx_collect and from the trace kernel's own binning."""
    s = configs.newtonian()
    g = f32(configs.newtonian_grid(num_pupil=500))
    ref = oracle_rayfunction(s, g)
    rays = ok.rays.RayVectorArray(
        wavelength=ref["wavelength"], position=V3(ref["px"], ref["py"], ref["pz"]),
        direction=V3(ref["dx"], ref["dy"], ref["dz"]), intensity=ref["intensity"],
        unvignetted=ref["unvignetted"])
    image, direction = s.sensor.collect(rays)
    i_ref, d_ref = O.collect_reference(s.sensor, ref)
    image, direction = image.cpu().numpy(), direction.cpu().numpy()
    c, _ = (t.cpu().numpy() for t in s.sensor.collect_counts(rays))
    c_ref, _ = O.collect(s.sensor, ref)
    same = c == c_ref  # pixels whose rays are the same on both sides
    assert same.mean() > 0.999
    assert np.allclose(image[same], i_ref[same], rtol=1e-5, atol=1e-6)
    assert np.allclose(direction[same], d_ref[same], rtol=0, atol=1e-6)
    assert np.all(direction[i_ref == 0][same[i_ref == 0]] == 1.0)
    # the trace kernel's binning fills the same moment image
    V2 = ok.vectors.Cartesian2dVectorArray
    pt = _api.PreparedTrace(s, wavelength=torch.as_tensor(g["wavelength"], device="cuda"),
                            field=V2(torch.as_tensor(g["field_x"], device="cuda"),
                                     torch.as_tensor(g["field_y"], device="cuda")),
                            pupil=V2(torch.as_tensor(g["pupil_x"], device="cuda"),
                                     torch.as_tensor(g["pupil_y"], device="cuda")),
                            image=True)
    mom = torch.zeros_like(pt.flux)
    pt.img.cos_moment = mom.data_ptr()
    pt.run()
    torch.cuda.synchronize()
    m_ref = (i_ref * d_ref)[i_ref > 0].sum()
    assert abs(float(mom.sum()) - m_ref) < 1e-5 * m_ref


def test_sag_api(cuda):
    rng = np.random.default_rng(21)
    x, y = rng.uniform(-20, 20, (2, 1000))
    for sag in [ok.sags.SphericalSag(-200.0), ok.sags.ConicSag(300.0, -0.7),
                ok.sags.ToroidalSag(400.0, 600.0), ok.sags.CylindricalSag(-150.0)]:
        z = sag(V3(x, y, 0.0)).cpu().numpy()
        assert np.allclose(z, O.sag_value(sag, x, y), atol=2e-6)
        n = sag.normal(V3(x, y, 0.0))
        nn = O.sag_normal(sag, x, y)
        for a, b in zip((n.x, n.y, n.z), nn):
            assert np.allclose(a.cpu().numpy(), b, atol=2e-7)
        r = _single_surface_rays(n=500, seed=5, spread=0.05)
        rays = ok.rays.RayVectorArray(wavelength=r["wavelength"],
                                      position=V3(r["px"], r["py"], r["pz"]),
                                      direction=V3(r["dx"], r["dy"], r["dz"]))
        hit = sag.intercept(rays).numpy()
        t = O.sag_intercept(sag, (r["px"], r["py"], r["pz"]), (r["dx"], r["dy"], r["dz"]))
        assert np.abs(hit["px"] - (r["px"] + r["dx"] * t)).max() < 1e-4


def test_edge_cases(cuda):
    s = configs.newtonian()
    # empty input
    empty = {k: np.zeros(0) for k in ("wavelength", "field_x", "field_y", "pupil_x", "pupil_y")}
    res = run_rayfunction(s, empty, image=True)
    assert res.outputs.position.x.numel() == 0
    assert res.image[0].sum().item() == 0
    # NaN inputs propagate to NaN outputs and are never binned
    g = configs.newtonian_grid(num_pupil=20)
    g["pupil_x"][:7] = np.nan
    res = run_rayfunction(s, g, image=True)
    out = res.outputs.numpy()
    ref = oracle_rayfunction(s, g)
    assert np.isnan(out["px"][:7]).all()
    assert np.array_equal(out["unvignetted"], ref["unvignetted"])
    assert res.image[0].sum().item() == int(ref["unvignetted"][np.isfinite(ref["px"])].sum())
    # a sphere the rays miss gives NaN intercepts
    miss = ok.surfaces.Surface(sag=ok.sags.SphericalSag(5.0), material=ok.materials.Mirror())
    r = _single_surface_rays(n=200, seed=2)
    out = _gpu_propagate([miss], r)
    ref = O.propagate_rays([miss], r)
    assert np.array_equal(np.isnan(out["px"]), np.isnan(ref["px"]))
    # a cylinder the rays miss keeps them on its vertex plane, as in the
    # reference (a sphere gives NaN instead)
    cyl = ok.surfaces.Surface(sag=ok.sags.CylindricalSag(5.0), material=ok.materials.Mirror())
    out = _gpu_propagate([cyl], r)
    ref = O.propagate_rays([cyl], r)
    assert np.array_equal(np.isnan(out["px"]), np.isnan(ref["px"]))
    miss_ref = np.abs(ref["px"]) > 5.0
    assert miss_ref.sum() > 50
    ok_ = np.isfinite(ref["px"])
    assert np.abs(out["px"][ok_] - ref["px"][ok_]).max() < 2e-4
    assert np.abs(out["pz"][miss_ref] - ref["pz"][miss_ref]).max() < 1e-4
    # broadcast scalar wavelength and intensity
    g = configs.newtonian_grid(num_pupil=50)
    res = s.rayfunction(wavelength=550.0, field=V2(g["field_x"], g["field_y"]),
                        pupil=V2(g["pupil_x"], g["pupil_y"]), intensity=2.0,
                        normalized_field=False, normalized_pupil=False)
    torch.cuda.synchronize()
    o = res.outputs.numpy()
    assert np.allclose(o["intensity"][o["unvignetted"]], 2.0)


def test_multilayer_periodic_batched_vs_oracle(cuda):
    """The 40-bilayer form: per-config mirrors drawn as in the workload,
    R and T within 1e-5 of complex128."""
    rng = np.random.default_rng(4)
    mirrors = []
    for _ in range(32):
        d = rng.uniform(9.5, 10.5)
        def idx():
            delta = 10 ** rng.uniform(-3, -1)
            beta = 10 ** rng.uniform(-4, -2)
            return c32(1 - delta + 1j * beta)
        mirrors.append(ok.materials.PeriodicMirror(
            a=ok.materials.Layer(idx(), float(np.float32(0.4 * d))),
            b=ok.materials.Layer(idx(), float(np.float32(0.6 * d))),
            num_periods=40, substrate=ok.materials.Layer(idx())))
    n = 4000
    wl = rng.uniform(12, 15, n).astype(np.float32).astype(np.float64)
    cos = np.cos(rng.uniform(0, 20 * math.pi / 180, n)).astype(np.float32).astype(np.float64)
    index = rng.integers(0, len(mirrors), n)
    R, T = ok.materials.multilayer_efficiency_periodic(wl, cos, mirrors, index)
    got = [x.cpu().numpy() for x in (R.s, R.p, T.s, T.p)]
    for k in range(len(mirrors)):
        sel = index == k
        m = mirrors[k]
        ref = O.multilayer_efficiency(wl[sel], cos[sel], 1.0, m.layers, m.substrate)
        for g, r in zip(got, ref):
            assert np.abs(g[sel] - r).max() < 1e-5


def test_attenuation_through_refracting_surface(cuda):
    """Rays in an absorbing medium (attenuation alpha > 0) lose
    I exp(-alpha |delta x|) on the way to the first surface
    (optika/sags/_abc.py:116-120); the glass behind it is clear."""
    rng = np.random.default_rng(31)
    r = _single_surface_rays(n=4000, seed=31)
    r["attenuation"] = rng.uniform(1e-3, 1e-2, r["px"].size).astype(np.float32).astype(np.float64)
    lens = SURFACES["glass_lens"]
    det = ok.surfaces.Surface(transformation=ok.transforms.Translation(z=-300.0))
    ref = O.propagate_rays([lens, det], r)
    out = _gpu_propagate([lens, det], r)
    m = ref["unvignetted"] & np.isfinite(ref["px"])
    assert m.mean() > 0.9
    # the factor is far from 1: exp(-alpha 100 mm) spans 0.37-0.9
    assert ref["intensity"][m].min() < 0.5 and ref["intensity"][m].max() > 0.85
    assert np.allclose(out["intensity"][m], ref["intensity"][m], rtol=2e-6, atol=0)
    assert np.all(out["attenuation"][m] == 0.0)
    assert np.abs(out["px"][m] - ref["px"][m]).max() < 2e-4


def test_attenuation_into_multilayer_mirror(cuda):
    """Rays arriving through an absorbing medium at a multilayer mirror: the
    incident index becomes n + i alpha lambda / (4 pi)
    (optika/materials/_multilayers.py:927-935), the segment loses
    exp(-alpha |delta x|), and the mirror keeps the medium's attenuation."""
    rng = np.random.default_rng(37)
    n = 4000
    r = O.make_rays((n,), px=rng.uniform(-1, 1, n), py=rng.uniform(-1, 1, n),
                    pz=np.full(n, -2e-4))
    dx, dy, dz = O.direction(rng.uniform(-0.2, 0.2, n), rng.uniform(-0.2, 0.2, n))
    r.update(dx=dx, dy=dy, dz=dz, wavelength=rng.uniform(12.5, 14.5, n),
             attenuation=rng.uniform(1000.0, 5000.0, n))
    for k in ("px", "py", "pz", "dx", "dy", "dz", "wavelength", "attenuation"):
        r[k] = r[k].astype(np.float32).astype(np.float64)
    si = ok.materials.Layer(c32(0.999 + 0.0018j), 4.1)
    mo = ok.materials.Layer(c32(0.922 + 0.0064j), 2.8)
    mirror = ok.surfaces.Surface(material=ok.materials.MultilayerMirror(
        layers=ok.materials.PeriodicLayerSequence([si, mo], num_periods=10),
        substrate=ok.materials.Layer(c32(0.999 + 0.0018j))))
    ref = O.propagate_rays([mirror], r)
    out = _gpu_propagate([mirror], r)
    # the imaginary part alpha lambda / 4 pi (1e-3 - 6e-3) changes R: the
    # same mirror seen from a clear medium reflects differently
    clear = dict(r, attenuation=np.zeros(n))
    ref_clear = O.propagate_rays([mirror], clear)
    assert np.abs(ref["intensity"] - ref_clear["intensity"]
                  * np.exp(-r["attenuation"] * 2e-4 / r["dz"])).max() > 1e-3
    # the multilayer tolerance of the single-precision transfer-matrix product
    assert np.abs(out["intensity"] - ref["intensity"]).max() < 1e-5
    assert np.allclose(out["attenuation"], ref["attenuation"], rtol=0, atol=0)


def test_calls_beyond_the_launch_grid_stride(cuda):
    """A call with more rays than the launch grid holds (4096 CTAs of 256
    threads per SM) strides over them: it equals the same rays traced in
    two calls of half the size, bit for bit, sensor image included."""
    dev = torch.device("cuda", torch.cuda.current_device())
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    n = sms * 4096 * 256 + 12345
    gen = torch.Generator(device=dev).manual_seed(17)
    u = lambda lo, hi: lo + (hi - lo) * torch.rand(n, device=dev, generator=gen)  # noqa: E731
    f = configs.FIELD_HALF
    r, t = torch.sqrt(u(12.0**2, 50.0**2)), u(0.0, 2 * math.pi)  # the pupil annulus
    g = dict(wavelength=u(400.0, 700.0), field_x=u(-f, f), field_y=u(-f, f),
             pupil_x=r * torch.cos(t), pupil_y=r * torch.sin(t))
    system = configs.newtonian(coated=True)
    outs = ("px", "py", "unvignetted")
    whole = run_rayfunction(system, g, image=True, outputs=outs)
    h = n // 2
    parts = [run_rayfunction(system, {k: v[a:b] for k, v in g.items()}, image=True, outputs=outs)
             for a, b in ((0, h), (h, n))]
    wo = whole.outputs
    for k in ("x", "y"):
        got = getattr(wo.position, k)
        ref = torch.cat([getattr(p.outputs.position, k) for p in parts])
        assert torch.equal(got, ref), k
    assert torch.equal(wo.unvignetted, torch.cat([p.outputs.unvignetted for p in parts]))
    assert int(wo.unvignetted.sum()) > 0.5 * n
    assert torch.equal(whole.image[0], parts[0].image[0] + parts[1].image[0])
