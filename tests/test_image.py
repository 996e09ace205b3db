"""SequentialSystem.image: cells of a scene, their rays, the photon image and
the exposure (optika/systems/_sequential.py:1002-1206,
optika/sensors/_sensors.py:92-252).

CPU: the host cell tables against the oracle's independent restatement
(solid angles by l'Huilier's theorem against van Oosterom-Strackee, both
published; coordinate-cell limit), the oracle's cell sampling (centres,
points inside their cells), argument checks.  GPU: the photon image of the
cell rays against the float64 oracle tracing the same cells (centres, and
random points from the same Philox draws), chunking, normalised
coordinates, and the exposure's shot and read noise statistics.
"""

import math

import numpy as np
import pytest
import torch

import optika_gb300 as ok
from optika_gb300 import configs, imaging
from optika_gb300.vectors import Cartesian2dVectorArray as V2
from optika_gb300.vectors import FunctionArray, SpectralPositionalVectorArray
from oracle import image as OI

DEG = math.pi / 180


def _scene(nw=2, nf=16, half=0.1 * DEG, radiance=None):
    w = np.linspace(500.0, 600.0, nw + 1)
    f = np.linspace(-half, half, nf + 1)
    rad = np.ones((nw, nf, nf)) if radiance is None else radiance
    return FunctionArray(inputs=SpectralPositionalVectorArray(wavelength=w, position=V2(f, f)),
                         outputs=rad)


def _pupil(n=16, r=50.0):
    v = np.linspace(-r, r, n + 1)
    return V2(v, v)


def test_solid_angles_agree_and_reach_the_coordinate_limit():
    ax = np.linspace(-0.3, 0.2, 7)
    ay = np.linspace(-0.25, 0.4, 9)
    a = imaging.solid_angle_cells(ax, ay)
    b = OI.solid_angle_cells(ax, ay)
    assert np.allclose(a, b, rtol=1e-10, atol=0)
    # small cells: the area element cos(ay) dax day of direction(ax, ay)
    ax = np.linspace(0.1, 0.1 + 1e-3, 2)
    ay = np.linspace(0.3, 0.3 + 1e-3, 2)
    exact = 1e-3 * (math.sin(0.3 + 1e-3) - math.sin(0.3))
    assert abs(imaging.solid_angle_cells(ax, ay)[0, 0] / exact - 1) < 1e-5


def test_solid_angle_total_converges_to_the_coordinate_integral():
    """The cells of the square field [-a, a]^2 of field angles cover
    int cos(ay) dax day = 4 a sin(a); the great-circle cells converge to it
    quadratically."""
    a = 5 * DEG
    exact = 4 * a * math.sin(a)
    errs = [abs(imaging.solid_angle_cells(np.linspace(-a, a, n + 1),
                                          np.linspace(-a, a, n + 1)).sum() / exact - 1)
            for n in (16, 64)]
    assert errs[1] < 1e-6 and errs[0] / errs[1] > 12


def test_image_flux_is_radiance_times_etendue():
    """Every ray of a system without apertures reaches the sensor: the photon
    image holds radiance x wavelength width x field solid angle x pupil
    area, in the oracle's trace of the product's cell tables as in the
    tables themselves."""
    sensor = ok.sensors.ImagingSensor(width_pixel=0.1, num_pixel=(512, 512),
                                      transformation=ok.transforms.Translation(z=100.0))
    s = ok.systems.SequentialSystem(surfaces=[], sensor=sensor)
    a = 0.5 * DEG
    w = np.linspace(500.0, 600.0, 3)
    f = np.linspace(-a, a, 17)
    v = np.linspace(-5.0, 5.0, 9)
    scene = FunctionArray(inputs=SpectralPositionalVectorArray(wavelength=w, position=V2(f, f)),
                          outputs=np.ones((2, 16, 16)))
    t = imaging.cell_tables(s, scene, V2(v, v), False, False)
    tab = OI.cell_tables(s, w, f, f, scene.outputs, v, v, False, False)
    img, _ = OI.photon_image(s, OI.cell_inputs(tab, random=True, seed=3), (500.0, 600.0, 1))
    expect = 100.0 * 4 * a * math.sin(a) * 10.0**2
    assert abs(img.sum() / expect - 1) < 1e-6
    assert abs(t.weight.sum() * t.weight_pupil[0].sum() / expect - 1) < 1e-6


def test_cell_tables_match_the_oracle_in_physical_coordinates():
    s = configs.newtonian()
    rng = np.random.default_rng(3)
    scene = _scene(nw=3, nf=5, radiance=rng.uniform(0.5, 2.0, (3, 5, 5)))
    pupil = _pupil(n=4)
    t = imaging.cell_tables(s, scene, pupil, normalized_field=False, normalized_pupil=False)
    o = OI.cell_tables(s, scene.inputs.wavelength, scene.inputs.position.x,
                       scene.inputs.position.y, scene.outputs, pupil.x, pupil.y, False, False)
    for a, b in zip((t.wavelength, t.field_x, t.field_y, t.pupil_x, t.pupil_y, t.weight,
                     t.weight_pupil), o):
        assert np.allclose(a, b, rtol=1e-10, atol=0)
    assert t.count == 3 * 5 * 5 * 4 * 4


def test_oracle_cell_samples_lie_in_their_cells():
    s = configs.newtonian()
    scene = _scene(nw=2, nf=3)
    pupil = _pupil(n=2)
    tab = OI.cell_tables(s, scene.inputs.wavelength, scene.inputs.position.x,
                         scene.inputs.position.y, scene.outputs, pupil.x, pupil.y, False, False)
    c = OI.cell_inputs(tab, random=False)
    assert np.allclose(c["wavelength"][:: 3 * 3 * 2 * 2], [525.0, 575.0])
    r = OI.cell_inputs(tab, random=True, seed=9)
    n = r["wavelength"].size
    idx = np.arange(n)
    iw = idx // (3 * 3 * 2 * 2)
    w = scene.inputs.wavelength
    assert np.all((r["wavelength"] >= w[iw]) & (r["wavelength"] < w[iw + 1]))
    ifx = (idx // (3 * 2 * 2)) % 3
    f = scene.inputs.position.x
    assert np.all((r["field_x"] >= f[ifx]) & (r["field_x"] <= f[ifx + 1]))
    assert not np.allclose(r["field_x"], c["field_x"])


def test_argument_checks_before_any_device_work():
    s = configs.newtonian()
    no_sensor = ok.systems.SequentialSystem(surfaces=s.surfaces, object=s.object)
    with pytest.raises(ValueError, match="sensor"):
        no_sensor.image(_scene(), pupil=_pupil(), normalized_field=False,
                        normalized_pupil=False)
    one = _scene()
    one.inputs.wavelength = np.array([550.0])
    with pytest.raises(ValueError, match="vertices"):
        s.image(one, pupil=_pupil(), normalized_field=False, normalized_pupil=False)


def test_photons_absorbed_and_uncertainty_of_the_ideal_sensor():
    """optika/sensors/_sensors_test.py:96-134: photons_absorbed inverts
    expose (one electron per photon, divided by the exposure time); the
    uncertainty is sqrt(electrons + read_noise^2)."""
    sensor = ok.sensors.ImagingSensor(width_pixel=0.01, num_pixel=(4, 4),
                                      timedelta_exposure=2.0, read_noise=3.0)
    e = torch.tensor([[0.0, 4.0], [16.0, 100.0]])
    assert torch.equal(sensor.photons_absorbed(e), e / 2.0)
    assert torch.equal(sensor.photons_absorbed(e, timedelta=4.0), e / 4.0)
    assert torch.allclose(sensor.uncertainty(e), torch.sqrt(e + 9.0))


def test_integrate_false_needs_uniform_wavelengths():
    s = configs.newtonian()
    scene = _scene()
    scene.inputs.wavelength = np.array([500.0, 520.0, 600.0])
    with pytest.raises(ValueError, match="uniformly spaced"):
        s.image(scene, pupil=_pupil(), normalized_field=False, normalized_pupil=False,
                integrate=False)


# ---------------------------------------------------------------- GPU


def _gpu_vs_oracle(system, scene, pupil, random, seed=0, chunk=1 << 24, integrate=True):
    res = system.image(scene, pupil=pupil, normalized_field=False, normalized_pupil=False,
                       noise=False, random=random, seed=seed, timedelta=1.0, chunk=chunk,
                       integrate=integrate)
    tab = OI.cell_tables(system, scene.inputs.wavelength, scene.inputs.position.x,
                         scene.inputs.position.y, scene.outputs, pupil.x, pupil.y, False, False)
    inputs = OI.cell_inputs(tab, random=random, seed=seed)
    w = scene.inputs.wavelength
    bins = (w.min(), w.max(), 1) if integrate else (w[0], w[-1], len(w) - 1)
    ref, _ = OI.photon_image(system, inputs, bins)
    return res, ref


@pytest.mark.gpu
@pytest.mark.parametrize("random", [False, True])
def test_photon_image_matches_oracle(cuda, random):
    s = configs.newtonian()
    rng = np.random.default_rng(5)
    scene = _scene(radiance=rng.uniform(0.5, 2.0, (2, 16, 16)))
    res, ref = _gpu_vs_oracle(s, scene, _pupil(), random, seed=11)
    img = res.outputs.cpu().numpy().astype(np.float64)
    assert img.shape == ref.shape == (1, 1024, 1024)
    tot = ref.sum()
    assert tot > 0
    assert abs(img.sum() / tot - 1) < 1e-5
    # a ray near a pixel edge may land in the neighbour: a small share
    assert np.abs(img - ref).sum() / tot < 2e-3
    assert np.allclose(res.inputs.wavelength, [500.0, 600.0])


@pytest.mark.gpu
def test_wavelength_bins_and_chunks(cuda):
    s = configs.newtonian()
    scene = _scene(nw=4, nf=8)
    res, ref = _gpu_vs_oracle(s, scene, _pupil(n=8), True, seed=2, chunk=1000,
                              integrate=False)
    img = res.outputs.cpu().numpy()
    assert img.shape == (4, 1024, 1024)
    per_bin = ref.sum(axis=(1, 2))
    assert np.allclose(img.sum(axis=(1, 2)), per_bin, rtol=1e-5)
    one = s.image(scene, pupil=_pupil(n=8), normalized_field=False, normalized_pupil=False,
                  noise=False, random=True, seed=2, timedelta=1.0, integrate=False)
    assert np.allclose(one.outputs.cpu().numpy(), img, rtol=1e-5, atol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("coated", [False, True])
def test_fused_cell_trace_equals_cell_rays_then_trace(cuda, coated):
    """otx_trace_cells (each cell's ray generated inside the trace kernel)
    bins the same rays as otx_cell_rays into buffers followed by the trace
    of those buffers in chunks: identical counts, flux to FP32 summation."""
    import torch

    from optika_gb300.imaging import ImagePlan

    s = configs.newtonian(coated=coated)
    scene = _scene(nw=3, nf=16)
    kw = dict(normalized_field=False, normalized_pupil=False, integrate=False, random=True,
              seed=9)
    fused = ImagePlan(s, scene, _pupil(n=12), fused=True, **kw)
    split = ImagePlan(s, scene, _pupil(n=12), fused=False, chunk=1000, **kw)
    assert fused.launches == 2 and split.launches > 2
    f_flux, f_mom = (t.clone() for t in fused.photons())
    f_counts = fused.trace.counts.clone()
    s_flux, s_mom = split.photons()
    torch.cuda.synchronize()
    assert f_counts.sum().item() > 0.5 * fused.count
    assert torch.equal(f_counts, split.trace.counts)
    assert torch.allclose(f_flux, s_flux, rtol=1e-5, atol=1e-6 * float(s_flux.max()))
    assert torch.allclose(f_mom, s_mom, rtol=1e-5, atol=1e-6 * float(s_mom.max()))


@pytest.mark.gpu
def test_normalized_scene_fills_the_stops(cuda):
    """Normalised field and pupil vertices are denormalised per wavelength
    vertex by the stop solver: the image equals the one of the physical
    vertices at the stop extents."""
    s = configs.stop_newtonian()
    fmin, fmax = s.field_min, s.field_max
    pmin, pmax = s.pupil_min, s.pupil_max
    nscene = _scene(nw=1, nf=4, half=1.0)
    nscene.inputs.wavelength = np.array([550.0, 550.0 + 1e-3])
    a = s.image(nscene, pupil=V2(np.linspace(-1, 1, 5), np.linspace(-1, 1, 5)),
                noise=False, random=False, timedelta=1.0)
    fx = np.linspace(fmin[0], fmax[0], 5)
    fy = np.linspace(fmin[1], fmax[1], 5)
    pscene = FunctionArray(inputs=SpectralPositionalVectorArray(
        wavelength=nscene.inputs.wavelength, position=V2(fx, fy)), outputs=nscene.outputs)
    b = s.image(pscene, pupil=V2(np.linspace(pmin[0], pmax[0], 5), np.linspace(pmin[1], pmax[1], 5)),
                normalized_field=False, normalized_pupil=False, noise=False, random=False,
                timedelta=1.0)
    assert np.allclose(a.outputs.cpu().numpy(), b.outputs.cpu().numpy(), rtol=1e-4, atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("mean", [0.3, 4.0, 37.0, 2.5e4])
def test_expose_shot_noise_statistics(cuda, mean):
    sensor = ok.sensors.ImagingSensor(width_pixel=0.01, num_pixel=(1000, 1000),
                                      timedelta_exposure=2.0)
    img = torch.full((1, 1000, 1000), mean / 2.0, device=cuda)
    e = sensor.expose(img, seed=4).double()
    n = e.numel()
    assert torch.all(e == torch.round(e))  # integer counts without read noise
    m, v = e.mean().item(), e.var().item()
    assert abs(m - mean) < 5 * math.sqrt(mean / n)
    # variance of the sample variance ~ 2 mean^2 / n (+ mean / n)
    assert abs(v - mean) < 5 * math.sqrt((2 * mean * mean + mean) / n)
    again = sensor.expose(img, seed=4)
    assert torch.equal(again, sensor.expose(img, seed=4))
    assert not torch.equal(again, sensor.expose(img, seed=5))


@pytest.mark.gpu
def test_expose_read_noise_and_noiseless(cuda):
    sensor = ok.sensors.ImagingSensor(width_pixel=0.01, num_pixel=(1000, 1000),
                                      timedelta_exposure=1.0, read_noise=3.0)
    img = torch.zeros((1, 1000, 1000), device=cuda)
    e = sensor.expose(img, seed=1).double()
    assert abs(e.mean().item()) < 5 * 3.0 / 1000
    assert abs(e.std().item() / 3.0 - 1) < 0.01
    img = torch.rand((1, 1000, 1000), device=cuda)
    assert torch.equal(sensor.expose(img, noise=False, timedelta=2.5), img * 2.5)


@pytest.mark.gpu
def test_photons_absorbed_inverts_expose(cuda):
    sensor = ok.sensors.ImagingSensor(width_pixel=0.01, num_pixel=(64, 64),
                                      timedelta_exposure=3.0)
    img = torch.rand((1, 64, 64), device=cuda) * 100
    back = sensor.photons_absorbed(sensor.expose(img, noise=False))
    assert torch.allclose(back, img, rtol=1e-6, atol=0)


@pytest.mark.gpu
def test_measure_is_collect_then_expose(cuda):
    s = configs.newtonian()
    g = configs.newtonian_grid(num_pupil=200)
    r = s.rayfunction(wavelength=g["wavelength"], field=V2(g["field_x"], g["field_y"]),
                      pupil=V2(g["pupil_x"], g["pupil_y"]), normalized_field=False,
                      normalized_pupil=False).outputs
    sensor = s.sensor
    flux, _ = sensor.collect(r)
    e = sensor.measure(r, timedelta=3.0, noise=False)
    assert torch.allclose(e, flux * 3.0)
