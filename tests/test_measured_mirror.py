"""MeasuredMirror: a reflectivity measured in wavelength, interpolated for
each ray (optika/materials/_materials.py:177-306).

CPU: the oracle on the reference's docstring example (a Gaussian
reflectivity peak at 304 Angstrom, width 10 Angstrom, measured at 11
wavelengths over +-3 widths: interpolation returns the measurements at the
measured wavelengths and the end values outside), the reference's checks of
the measurement, and the lowering.  GPU: the traced intensity against the
oracle.
"""

import numpy as np
import pytest
import torch

import optika_gb300 as ok
from optika_gb300 import _lib as L
from optika_gb300._lower import lower_surfaces
from optika_gb300.vectors import Cartesian3dVectorArray as V3
from optika_gb300.vectors import FunctionArray, SpectralDirectionalVectorArray
from oracle import trace as O


def _mirror(center=30.4, width=1.0, num=11):
    wl = np.linspace(center - 3 * width, center + 3 * width, num)
    return ok.materials.MeasuredMirror(FunctionArray(
        inputs=SpectralDirectionalVectorArray(wavelength=wl, direction=V3(0.0, 0.0, 1.0)),
        outputs=np.exp(-np.square((wl - center) / width) / 2)))


def _flat_rays(wavelength):
    wavelength = np.asarray(wavelength, dtype=np.float64)
    n = wavelength.size
    return O.make_rays((n,), px=np.linspace(-1, 1, n), pz=np.full(n, -10.0), dz=1.0,
                       wavelength=wavelength)


def test_docstring_example_interpolation():
    m = _mirror()
    wl = m.efficiency_measured.inputs.wavelength
    meas = m.efficiency_measured.outputs
    probe = np.concatenate([wl, [20.0, 40.0], (wl[:-1] + wl[1:]) / 2])
    out = O.propagate_rays([ok.surfaces.Surface(material=m)], _flat_rays(probe))
    eff = out["intensity"]
    assert np.allclose(eff[:11], meas, atol=1e-15)
    assert np.allclose(eff[11:13], [meas[0], meas[-1]], atol=1e-15)
    assert np.allclose(eff[13:], (meas[:-1] + meas[1:]) / 2, atol=1e-15)
    # a mirror: n and attenuation unchanged, direction reflected
    assert np.allclose(out["dz"], -1.0) and np.allclose(out["n"], 1.0)


def test_measurement_checks_and_lowering():
    m = _mirror()
    lw = lower_surfaces([ok.surfaces.Surface(material=m), ok.surfaces.Surface(material=m)],
                        pre=np.eye(4), final=None, input_mode=L.INPUT_RAYS)
    s0, s1 = lw.sys.surfaces[0], lw.sys.surfaces[1]
    assert s0.mat_type == L.MAT_MEASURED_MIRROR and s0.mat_is_mirror == 1
    assert s0.mat_table == 0 and s1.mat_table == 1 and len(lw.table_list) == 2
    bad = _mirror()
    bad.efficiency_measured.inputs.direction = V3(np.zeros(3), np.zeros(3), np.ones(3))
    with pytest.raises(ValueError, match="incidence angles"):
        lower_surfaces([ok.surfaces.Surface(material=bad)], pre=np.eye(4), final=None,
                       input_mode=L.INPUT_RAYS)
    assert ok.materials.MeasuredMirror.is_mirror


@pytest.mark.gpu
def test_measured_mirror_in_trace(cuda):
    from optika_gb300 import _api

    rng = np.random.default_rng(4)
    n = 4000
    m = _mirror(center=300.0, width=40.0, num=25)
    mirror = ok.surfaces.Surface(sag=ok.sags.SphericalSag(-400.0), material=m)
    det = ok.surfaces.Surface(transformation=ok.transforms.Translation(z=-200.0))
    dx, dy, dz = O.direction(rng.uniform(-0.1, 0.1, n), rng.uniform(-0.1, 0.1, n))
    r = O.make_rays((n,), px=rng.uniform(-20, 20, n), py=rng.uniform(-20, 20, n),
                    pz=np.full(n, -50.0), dx=dx, dy=dy, dz=dz,
                    wavelength=rng.uniform(150, 450, n))
    for k in ("px", "py", "pz", "dx", "dy", "dz", "wavelength"):
        r[k] = r[k].astype(np.float32).astype(np.float64)
    ref = O.propagate_rays([mirror, det], r)
    rays = ok.rays.RayVectorArray(
        wavelength=r["wavelength"], position=V3(r["px"], r["py"], r["pz"]),
        direction=V3(r["dx"], r["dy"], r["dz"]))
    out = _api.propagate_rays([mirror, det], rays)
    torch.cuda.synchronize()
    o = out.numpy()
    assert np.abs(o["intensity"] - ref["intensity"]).max() < 2e-6
    assert np.abs(o["px"] - ref["px"]).max() < 2e-4
    assert (ref["intensity"] < 0.9).mean() > 0.3  # the table matters
