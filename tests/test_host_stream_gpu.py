"""The host path (``otx_trace_grid_host``): host arrays in, host arrays out.
Page-locked arrays are read and written in place by the trace kernel
(zero-copy over the host link); pageable arrays are staged through the GPU
in overlapping chunks.  Both run the same kernel as the device path on the
same inputs, so every ray output must be bit-identical to the device
path's; count images are identical and flux images equal up to the order
of the float atomic additions."""

import ctypes

import numpy as np
import pytest
import torch

import optika_gb300 as ok
from optika_gb300 import _api, _lib as L, configs
from oracle import trace as O

pytestmark = pytest.mark.gpu

V2 = ok.vectors.Cartesian2dVectorArray
FIELDS = ("px", "py", "pz", "dx", "dy", "dz", "intensity", "unvignetted", "opl")


def _inputs(g, pin=True):
    t = {k: torch.from_numpy(np.asarray(v, dtype=np.float32)) for k, v in g.items()}
    return {k: (v.pin_memory() if pin else v) for k, v in t.items()}


def _call(system, t, **kw):
    return system.rayfunction(wavelength=t["wavelength"], field=V2(t["field_x"], t["field_y"]),
                              pupil=V2(t["pupil_x"], t["pupil_y"]), normalized_field=False,
                              normalized_pupil=False, **kw)


def test_host_rayfunction_equals_device_path(cuda):
    s = configs.newtonian(coated=True)
    g = configs.precision_grid(1_500_000, seed=31)
    host = _call(s, _inputs(g), image=True)
    assert host.outputs.position.x.device.type == "cpu"
    assert host.image[0].device.type == "cpu"
    dev = _call(s, {k: v.cuda() for k, v in _inputs(g).items()}, image=True)
    torch.cuda.synchronize()
    a, b = host.outputs.numpy(), dev.outputs.numpy()
    for k in FIELDS:
        assert np.array_equal(a[k], b[k], equal_nan=True), k
    assert torch.equal(host.image[0], dev.image[0].cpu())
    assert torch.allclose(host.image[1], dev.image[1].cpu(), rtol=1e-5, atol=1e-5)
    # and the oracle agrees with both (pinned to float64, same tolerance as the device tests)
    sub = slice(0, 20000)
    ref = O.rayfunction(s, *(np.asarray(g[k][sub], np.float32).astype(np.float64)
                             for k in ("wavelength", "field_x", "field_y", "pupil_x", "pupil_y")))
    m = ref["unvignetted"]
    assert np.array_equal(a["unvignetted"][sub], m)
    e = np.hypot(a["px"][sub][m] - ref["px"][m], a["py"][sub][m] - ref["py"][m])
    assert e.max() < 1.5e-4


def test_host_pageable_and_scalar_inputs(cuda):
    s = configs.newtonian()
    g = configs.precision_grid(50_000, seed=32)
    t = _inputs(g, pin=False)
    t["wavelength"] = torch.tensor(550.0)
    host = _call(s, t)
    dt = {k: v.cuda() for k, v in t.items()}
    dev = _call(s, dt)
    torch.cuda.synchronize()
    a, b = host.outputs.numpy(), dev.outputs.numpy()
    for k in FIELDS:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("accumulate", [False, True])
def test_host_path_through_the_c_abi(cuda, accumulate, pinned):
    """Pinned buffers: the zero-copy launch (its workspace is just the
    scalar head).  Pageable buffers: the staged path, with a workspace far
    below the recommended size so that there are many chunks and a ragged
    last one, and every slot of the three-slot ring is reused."""
    s = configs.newtonian(coated=True)
    n = 100_003
    g = configs.precision_grid(n, seed=33)
    t = _inputs(g, pin=pinned)
    surfaces = s.surfaces_all
    from optika_gb300._lower import lower_surfaces
    from optika_gb300.transforms import matrix_of, rigid_inverse

    pre = rigid_inverse(matrix_of(s.transformation)) @ matrix_of(s.object.transformation)
    final = None if accumulate else rigid_inverse(matrix_of(s.sensor.transformation)) @ \
        matrix_of(surfaces[-1].transformation)
    lw = lower_surfaces(surfaces, pre=pre, final=final, input_mode=L.INPUT_GRID_INFINITY,
                        sensor=s.sensor, device=torch.device("cuda", 0))
    grid = L.Grid()
    grid.wavelength, grid.field_x, grid.field_y, grid.pupil_x, grid.pupil_y = (
        t[k].data_ptr() for k in ("wavelength", "field_x", "field_y", "pupil_x", "pupil_y"))
    grid.stride_wavelength = grid.stride_field = grid.stride_pupil = 1
    grid.count = n
    S = len(surfaces) if accumulate else 1
    shape = (S, n) if accumulate else (n,)

    def outs(pin, dev):
        b = {}
        for k in ("px", "py", "pz", "dx", "dy", "dz", "intensity", "unvignetted", "opl"):
            dt = torch.uint8 if k == "unvignetted" else (
                torch.float64 if k == "opl" else torch.float32)
            b[k] = torch.full(shape, 7, dtype=dt, device=dev, pin_memory=pin)
        return b

    hb = outs(pinned, "cpu")
    ho = _api._rays_struct(hb, n, n if accumulate else 0)
    counts = torch.zeros((1, 1024, 1024), dtype=torch.int32, device="cuda")
    img = L.Image()
    img.counts = counts.data_ptr()
    ln = L.Launch()
    ln.accumulate = int(accumulate)
    lib = L.load()
    need = lib.otx_trace_grid_host_workspace(ctypes.byref(grid), ctypes.byref(ho), S)
    if pinned:
        assert need == 256  # zero-copy: only the head of broadcast scalars
        small = need
    else:
        # room for chunks of ~7000 rays: 15 chunks, the last one ragged
        per_ray = need / (3 * min(n, 1 << 20))
        small = int(256 + 3 * 7000 * per_ray) + 3 * 256 * 12
    ws = torch.empty(small, dtype=torch.uint8, device="cuda")
    for _ in range(2):  # twice: the second call reuses the streams and events
        counts.zero_()
        st = lib.otx_trace_grid_host(ctypes.byref(lw.sys), ctypes.byref(grid), ctypes.byref(ho),
                                     ctypes.byref(img), ctypes.byref(ln), ws.data_ptr(), small,
                                     _api.stream_handle())
        assert st == L.OK, lib.otx_status_string(st)
        torch.cuda.synchronize()
    # the same trace on the device in one launch
    dg = L.Grid.from_buffer_copy(grid)
    dt_in = {k: v.cuda() for k, v in t.items()}
    dg.wavelength, dg.field_x, dg.field_y, dg.pupil_x, dg.pupil_y = (
        dt_in[k].data_ptr() for k in ("wavelength", "field_x", "field_y", "pupil_x", "pupil_y"))
    db = outs(False, "cuda")
    do = _api._rays_struct(db, n, n if accumulate else 0)
    c2 = torch.zeros_like(counts)
    img2 = L.Image()
    img2.counts = c2.data_ptr()
    st = lib.otx_trace_grid(ctypes.byref(lw.sys), ctypes.byref(dg), ctypes.byref(do),
                            ctypes.byref(img2), ctypes.byref(ln), _api.stream_handle())
    assert st == L.OK
    torch.cuda.synchronize()
    for k in hb:
        assert torch.equal(hb[k], db[k].cpu()) or torch.allclose(
            hb[k].double(), db[k].cpu().double(), rtol=0, atol=0, equal_nan=True), k
    assert torch.equal(counts, c2)
    assert int(counts.sum()) > 0
