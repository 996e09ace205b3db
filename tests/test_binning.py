"""Sensor binning inside the trace kernels equals a serial histogram of the
kernel's own output rays.

The kernels bin each unvignetted ray with warp-aggregated shared-memory
atomics (optika/sensors/_sensors.py:140-161 restated: numpy.histogramdd
edges, last edge inclusive).  Here the same rays' float32 sensor-frame
positions are binned serially on the host with the kernel's explicitly
rounded bin formula, and the integer count images must be identical bit for
bit; the intensity and cosine-moment images are float sums whose order the
atomics do not fix, so they agree to FP32 summation error.  Cases: the small
Newtonian workload (25 field points of 4000 rays: a warp's rays land in a
handful of pixels, the contended case the aggregation is for) and 1e6 rays of
the precision workload (rays spread over the sensor).
"""

import numpy as np
import pytest
import torch

import optika_gb300 as ok
from optika_gb300 import _api, configs

pytestmark = pytest.mark.gpu

V2 = ok.vectors.Cartesian2dVectorArray


def _trace(system, g):
    dev = torch.device("cuda", torch.cuda.current_device())
    t = {k: torch.as_tensor(np.asarray(v, np.float32), device=dev) for k, v in g.items()}
    prep = _api.PreparedTrace(system, wavelength=t["wavelength"],
                              field=V2(t["field_x"], t["field_y"]),
                              pupil=V2(t["pupil_x"], t["pupil_y"]), image=True, cos_moment=True,
                              outputs=("px", "py", "dz", "intensity", "unvignetted"))
    prep.run()
    torch.cuda.synchronize()
    out = {k: prep.bufs[k].cpu().numpy() for k in ("px", "py", "dz", "intensity", "unvignetted")}
    images = [x.cpu().numpy()[0] for x in (prep.counts, prep.flux, prep.moment)]
    return prep.lowering.sys.sensor, out, images


def _serial_histogram(S, out):
    """The kernel's bin formula in float32, one ray at a time in order."""
    f = np.float32
    lo_x, lo_y, wx, wy = f(S.lo_x), f(S.lo_y), f(S.width_x), f(S.width_y)
    nx, ny = int(S.num_x), int(S.num_y)
    # upper edges: one fused multiply-add, lo + num w rounded once
    hx = f(np.float64(nx) * np.float64(wx) + np.float64(lo_x))
    hy = f(np.float64(ny) * np.float64(wy) + np.float64(lo_y))
    inv_x, inv_y = f(1) / wx, f(1) / wy
    px, py = out["px"].astype(np.float32), out["py"].astype(np.float32)
    ok_ = (out["unvignetted"] != 0) & (px >= lo_x) & (px <= hx) & (py >= lo_y) & (py <= hy)
    ix = np.floor((px[ok_] - lo_x) * inv_x).astype(np.int64).clip(0, nx - 1)
    iy = np.floor((py[ok_] - lo_y) * inv_y).astype(np.int64).clip(0, ny - 1)
    flat = ix * ny + iy
    counts = np.zeros(nx * ny, np.int64)
    flux = np.zeros(nx * ny, np.float64)
    moment = np.zeros(nx * ny, np.float64)
    w = out["intensity"][ok_].astype(np.float64)
    for arr, val in ((counts, 1), (flux, w), (moment, w * out["dz"][ok_].astype(np.float32))):
        np.add.at(arr, flat, val)
    return counts.reshape(nx, ny), flux.reshape(nx, ny), moment.reshape(nx, ny)


@pytest.mark.parametrize("case", ["newtonian-25-fields", "precision-1e6"])
def test_atomic_image_equals_serial_histogram(cuda, case):
    if case == "newtonian-25-fields":
        system, g = configs.newtonian(), configs.newtonian_grid()
    else:
        system, g = configs.newtonian(coated=True), configs.precision_grid(1_000_000)
    S, out, (counts, flux, moment) = _trace(system, g)
    c_ref, f_ref, m_ref = _serial_histogram(S, out)
    assert c_ref.sum() > 0.9 * len(g["wavelength"])
    assert np.array_equal(counts.astype(np.int64), c_ref)
    assert np.allclose(flux, f_ref, rtol=2e-6, atol=1e-6)
    assert np.allclose(moment, m_ref, rtol=2e-6, atol=1e-6)
    if case == "newtonian-25-fields":
        # the contended case: at most a few hundred pixels take all 1e5 rays
        assert np.count_nonzero(c_ref) < 2000
