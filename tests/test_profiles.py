"""Interface roughness profiles of multilayer stacks (Stearns 1989).

CPU: the host profile methods against the reference's property tests
(optika/materials/_tests/test_profiles.py: profile, transmissivity and
reflectivity within [0, 1]); the oracle pinned to the Debye-Waller factor of
a single rough interface, to the unchanged transmission of a single
interface, and to the IMD file of the rough SiC/Cr mirror (which the
reference itself marks xfail because IMD evaluates the roughness factor with
the vacuum wavelength: agreement to a fraction of a percent, against ~20%
without roughness); the lowering.  GPU: the transfer-matrix kernel and the
trace against the oracle, for every profile on layers, periodic blocks and
substrates.
"""

import math

import numpy as np
import pytest
import torch

import optika_gb300 as ok
from optika_gb300 import _lib as L
from optika_gb300._lower import Lowering
from oracle import trace as O

P = ok.materials.profiles
PROFILES = {
    "erf": P.ErfInterfaceProfile,
    "exponential": P.ExponentialInterfaceProfile,
    "linear": P.LinearInterfaceProfile,
    "sinusoidal": P.SinusoidalInterfaceProfile,
}


@pytest.mark.parametrize("name", sorted(PROFILES))
@pytest.mark.parametrize("width", [0.5, 1.0])
def test_reference_property_bounds(name, width):
    a = PROFILES[name](width)
    for z in (torch.tensor(0.0, dtype=torch.float64), torch.linspace(-1, 1, 11,
                                                                   dtype=torch.float64)):
        v = a(z)
        assert torch.all(v >= 0) and torch.all(v <= 1)
    for wl in (torch.tensor(30.4, dtype=torch.float64),
               torch.linspace(30, 40, 5, dtype=torch.float64)):
        t = a.transmissivity(wl, 1.0, 1.0, 1.0, 1.5)
        assert torch.all(t >= 0) and torch.all(t <= 1)
        for d in (1.0, torch.cos(torch.deg2rad(torch.linspace(-90, 90, 5, dtype=torch.float64)))):
            r = a.reflectivity(wl, d, 1.5)
            assert torch.all(r >= 0) and torch.all(r <= 1 + 1e-15)


@pytest.mark.parametrize("name", sorted(PROFILES))
def test_oracle_factor_equals_host_methods(name):
    a = PROFILES[name](0.8)
    wl = np.linspace(10, 40, 7)
    d = np.cos(np.linspace(0, 1.2, 7)) + 0.01j
    n = 0.97 + 0.02j
    host = a.reflectivity(torch.from_numpy(wl), torch.from_numpy(d), n).numpy()
    assert np.allclose(O.interface_reflectivity(a, wl, d, n), host, rtol=1e-13)


def test_erf_single_interface_is_debye_waller():
    """One rough interface: R = R_smooth exp(-(4 pi sigma n cos / lambda)^2),
    T unchanged (t = 2 q_i / (q_i + q_j) carries no profile factor)."""
    wl = np.linspace(10, 60, 26)
    cos = np.cos(np.deg2rad(15.0))
    sub_rough = ok.materials.Layer(0.95 + 0.03j, interface=P.ErfInterfaceProfile(1.5))
    sub = ok.materials.Layer(0.95 + 0.03j)
    Rs, Rp, Ts, Tp = O.multilayer_efficiency(wl, cos, 1.0, None, sub_rough)
    Rs0, Rp0, Ts0, Tp0 = O.multilayer_efficiency(wl, cos, 1.0, None, sub)
    dw = np.exp(-np.square(4 * np.pi * 1.5 * cos / wl))
    assert np.allclose(Rs, Rs0 * dw, rtol=1e-12)
    assert np.allclose(Rp, Rp0 * dw, rtol=1e-12)
    assert np.allclose(Ts, Ts0, rtol=1e-12) and np.allclose(Tp, Tp0, rtol=1e-12)


def test_rough_mirror_vs_imd_file():
    from tests.test_oracle import golden_case

    wl, eff_file, is_mirror, layers, sub = golden_case("SiC_Cr_Rough")
    Rs, Rp, _, _ = O.multilayer_efficiency(wl, 1.0, 1.0, layers, sub)
    m = eff_file > 1e-3
    rel = np.abs((Rs + Rp)[m] / 2 / eff_file[m] - 1)
    assert np.median(rel) < 0.01
    assert np.abs((Rs + Rp) / 2 - eff_file).max() < 5e-3
    smooth = [ok.materials.Layer(x.chemical, x.thickness) for x in layers]
    Rs0, Rp0, _, _ = O.multilayer_efficiency(wl, 1.0, 1.0, smooth,
                                             ok.materials.Layer(sub.chemical))
    assert np.median(np.abs((Rs0 + Rp0)[m] / 2 / eff_file[m] - 1)) > 0.1


def test_lowering_of_profiles():
    lw = Lowering()
    layers = [ok.materials.Layer(0.9 + 0.01j, 4.0, interface=PROFILES[k](0.3 + i))
              for i, k in enumerate(sorted(PROFILES))]
    k = lw.add_stack(layers, ok.materials.Layer(0.9 + 0.1j, interface=P.ErfInterfaceProfile(0.7)))
    K = lw.sys.stacks[k]
    tags = [lw.sys.layers[K.pre_begin + i].interface_type for i in range(4)]
    assert tags == [L.PROFILE_ERF, L.PROFILE_EXPONENTIAL, L.PROFILE_LINEAR, L.PROFILE_SINUSOIDAL]
    assert [round(lw.sys.layers[K.pre_begin + i].interface_width, 6) for i in range(4)] == [
        0.3, 1.3, 2.3, 3.3]
    assert lw.sys.layers[K.substrate].interface_type == L.PROFILE_ERF
    with pytest.raises(NotImplementedError):
        Lowering().add_stack([ok.materials.Layer(1.0 + 0j, 5.0, interface=object())], None)


def _stack(name, periodic):
    prof = PROFILES[name]
    A = ok.materials.Layer(0.98 + 0.004j, 4.0, interface=prof(0.4))
    B = ok.materials.Layer(0.997 + 0.0006j, 6.0, interface=prof(0.3))
    cap = ok.materials.Layer(0.96 + 0.02j, 2.0, interface=prof(0.5))
    sub = ok.materials.Layer(0.97 + 0.01j, interface=prof(0.6))
    if periodic:
        return [cap, ok.materials.PeriodicLayerSequence([A, B], 20)], sub
    return [cap, A, B], sub


@pytest.mark.gpu
@pytest.mark.parametrize("periodic", [False, True])
@pytest.mark.parametrize("name", sorted(PROFILES))
def test_rough_stacks_vs_oracle(cuda, name, periodic):
    rng = np.random.default_rng(6)
    n = 20000
    wl = rng.uniform(12, 16, n).astype(np.float32).astype(np.float64)
    cos = np.cos(rng.uniform(0, 60 * math.pi / 180, n)).astype(np.float32).astype(np.float64)
    layers, sub = _stack(name, periodic)
    R, T = ok.multilayer_efficiency(wl, cos, 1.0, layers, sub)
    Rs, Rp, Ts, Tp = O.multilayer_efficiency(wl, cos, 1.0, layers, sub)
    for a, b in ((R.s, Rs), (R.p, Rp), (T.s, Ts), (T.p, Tp)):
        assert np.abs(a.cpu().numpy() - b).max() < 2e-5


@pytest.mark.gpu
def test_rough_imd_case_on_gpu(cuda):
    from tests.test_oracle import golden_case

    wl, _, _, layers, sub = golden_case("SiC_Cr_Rough")
    R, _ = ok.multilayer_efficiency(wl, 1.0, 1.0, layers, sub)
    Rs, Rp, _, _ = O.multilayer_efficiency(wl, 1.0, 1.0, layers, sub)
    assert np.allclose(R.average.cpu().numpy(), (Rs + Rp) / 2, rtol=1e-4, atol=1e-7)


@pytest.mark.gpu
@pytest.mark.parametrize("layered", [False, True])
def test_rough_mirrors_in_trace(cuda, layered):
    """A rough bare substrate (the trace's Fresnel kind) and a rough layered
    coating on a concave mirror: the traced intensity against the oracle."""
    from optika_gb300 import _api
    from optika_gb300.vectors import Cartesian3dVectorArray as V3

    if layered:
        layers, sub = _stack("erf", periodic=True)
    else:
        layers, sub = None, ok.materials.Layer(0.97 + 0.01j, interface=P.ErfInterfaceProfile(0.6))
    mirror = ok.surfaces.Surface(sag=ok.sags.SphericalSag(-400.0),
                                 material=ok.materials.MultilayerMirror(layers=layers,
                                                                        substrate=sub))
    det = ok.surfaces.Surface(transformation=ok.transforms.Translation(z=-200.0))
    rng = np.random.default_rng(8)
    n = 4000
    dx, dy, dz = O.direction(rng.uniform(-0.3, 0.3, n), rng.uniform(-0.3, 0.3, n))
    r = O.make_rays((n,), px=rng.uniform(-20, 20, n), py=rng.uniform(-20, 20, n),
                    pz=np.full(n, -50.0), dx=dx, dy=dy, dz=dz,
                    wavelength=rng.uniform(12, 16, n))
    for k in ("px", "py", "pz", "dx", "dy", "dz", "wavelength"):
        r[k] = r[k].astype(np.float32).astype(np.float64)
    ref = O.propagate_rays([mirror, det], r)
    rays = ok.rays.RayVectorArray(wavelength=r["wavelength"],
                                  position=V3(r["px"], r["py"], r["pz"]),
                                  direction=V3(r["dx"], r["dy"], r["dz"]))
    out = _api.propagate_rays([mirror, det], rays)
    torch.cuda.synchronize()
    o = out.numpy()
    assert np.abs(o["intensity"] - ref["intensity"]).max() < 2e-5
