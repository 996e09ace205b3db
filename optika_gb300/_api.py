"""GPU calls behind the host API: tensors in, C-ABI call, tensors out.

Every public entry point of the package that computes something ends here,
in a call through the C-ABI library.  There is no CPU path: without a CUDA
device these functions raise.
"""

from __future__ import annotations

import ctypes
import dataclasses
from typing import Sequence

import numpy as np
import torch

from . import _lib as L
from ._lower import lower_surfaces
from .rays import RayFunctionArray, RayVectorArray
from .transforms import matrix_of, rigid_inverse
from .vectors import Cartesian3dVectorArray, PolarizationVectorArray


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("optika_gb300 needs a CUDA device (GB300, sm_103a); none is available")
    return torch.device("cuda", torch.cuda.current_device())


def stream_handle() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t: torch.Tensor | None) -> int:
    return 0 if t is None else t.data_ptr()


def as_f32(x, dev) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.to(device=dev, dtype=torch.float32)
    return torch.as_tensor(np.asarray(x, dtype=np.float32), device=dev)


class _Field:
    """A flattened float32 device input with its element stride (0 = scalar)."""

    def __init__(self, t: torch.Tensor, n: int):
        if t.numel() == 1:
            self.t = t.reshape(1).contiguous()
            self.stride = 0
        else:
            self.t = t.reshape(-1).contiguous()
            if self.t.numel() != n:
                raise ValueError("input sizes do not broadcast")
            self.stride = 1


def _broadcast_inputs(values: Sequence, dev) -> tuple[list[_Field], tuple[int, ...]]:
    ts = [as_f32(v, dev) for v in values]
    shape = torch.broadcast_shapes(*[t.shape for t in ts])
    n = int(np.prod(shape)) if len(shape) else 1
    out = []
    for t in ts:
        if t.numel() == 1:
            out.append(_Field(t, n))
        else:
            out.append(_Field(t.expand(shape), n))
    return out, tuple(shape)


def _alloc_rays(n: int, dev, shape_prefix: tuple = (), fields=None) -> dict[str, torch.Tensor]:
    full = shape_prefix + (n,)
    names = ("px", "py", "pz", "dx", "dy", "dz", "wavelength", "intensity", "attenuation",
             "index_refraction", "unvignetted", "opl")
    out = {}
    for k in names:
        if fields is not None and k not in fields:
            out[k] = None
        elif k == "unvignetted":
            out[k] = torch.empty(full, dtype=torch.uint8, device=dev)
        elif k == "opl":
            out[k] = torch.empty(full, dtype=torch.float64, device=dev)
        else:
            out[k] = torch.empty(full, dtype=torch.float32, device=dev)
    return out


def _rays_struct(b: dict, n: int, stride: int = 0) -> L.Rays:
    r = L.Rays()
    for k in ("px", "py", "pz", "dx", "dy", "dz", "wavelength", "intensity", "attenuation",
              "index_refraction", "unvignetted", "opl"):
        setattr(r, k, ptr(b.get(k)))
    r.count = n
    r.surface_stride = stride
    return r


def _to_ray_array(b: dict, shape: tuple) -> RayVectorArray:
    def rs(t):
        return t.reshape(t.shape[:-1] + shape)

    return RayVectorArray(
        wavelength=rs(b["wavelength"]),
        position=Cartesian3dVectorArray(rs(b["px"]), rs(b["py"]), rs(b["pz"])),
        direction=Cartesian3dVectorArray(rs(b["dx"]), rs(b["dy"]), rs(b["dz"])),
        intensity=rs(b["intensity"]),
        attenuation=rs(b["attenuation"]),
        index_refraction=rs(b["index_refraction"]),
        unvignetted=rs(b["unvignetted"]).view(torch.bool),  # bytes 0 / 1: a view, no copy
        opl=rs(b["opl"]),
    )


def _image_buffers(sensor, wavelength_bins, dev, cos_moment: bool = False):
    nx, ny = sensor.num_pixel
    nw = 1 if wavelength_bins is None else int(wavelength_bins[2])
    counts = torch.zeros((nw, int(nx), int(ny)), dtype=torch.int32, device=dev)
    flux = torch.zeros((nw, int(nx), int(ny)), dtype=torch.float32, device=dev)
    img = L.Image()
    img.counts = counts.data_ptr()
    img.flux = flux.data_ptr()
    if cos_moment:
        mom = torch.zeros((nw, int(nx), int(ny)), dtype=torch.float32, device=dev)
        img.cos_moment = mom.data_ptr()
        return counts, flux, img, mom
    return counts, flux, img


# ---------------------------------------------------------------- traces


OUTPUT_FIELDS = ("px", "py", "pz", "dx", "dy", "dz", "wavelength", "intensity", "attenuation",
                 "index_refraction", "unvignetted", "opl")


class PreparedTrace:
    """A grid trace with its descriptor and every buffer allocated once.

    ``run()`` enqueues exactly one kernel (plus the image clear when binning)
    on the current stream, so it can be timed, repeated or captured in a
    CUDA graph.  ``outputs`` selects which ray fields are written.
    """

    def __init__(self, system, *, wavelength, field, pupil, intensity=None, accumulate=False,
                 final_local=True, image=False, wavelength_bins=None, launch=None,
                 outputs=OUTPUT_FIELDS, cos_moment=False):
        dev = device()
        self.device = dev
        surfaces = system.surfaces_all
        obj = system.object
        pre = rigid_inverse(matrix_of(system.transformation)) @ (
            matrix_of(obj.transformation) if obj is not None else np.eye(4)
        )
        sensor = system.sensor
        if final_local:
            if sensor is None:
                raise ValueError("rayfunction needs a sensor")
            final = rigid_inverse(matrix_of(sensor.transformation)) @ matrix_of(
                surfaces[-1].transformation
            )
        else:
            final = None
        mode = L.INPUT_GRID_INFINITY if system.object_is_at_infinity else L.INPUT_GRID_FINITE
        self.lowering = lower_surfaces(
            surfaces, pre=pre, final=final, input_mode=mode,
            sensor=sensor if image else None, wavelength_bins=wavelength_bins, device=dev,
        )
        vals = [wavelength, field.x, field.y, pupil.x, pupil.y]
        if intensity is not None:
            vals.append(intensity)
        fields, shape = _broadcast_inputs(vals, dev)
        n = int(np.prod(shape)) if len(shape) else 1
        if fields[1].stride != fields[2].stride or fields[3].stride != fields[4].stride:
            for f in fields[1:5]:
                if f.stride == 0:
                    f.t = f.t.expand(n).contiguous()
                    f.stride = 1
        g = L.Grid()
        g.wavelength, g.field_x, g.field_y, g.pupil_x, g.pupil_y = (ptr(f.t) for f in fields[:5])
        g.stride_wavelength = fields[0].stride
        g.stride_field = fields[1].stride
        g.stride_pupil = fields[3].stride
        if intensity is not None:
            g.intensity = ptr(fields[5].t)
            g.stride_intensity = fields[5].stride
        g.count = n
        self.grid = g
        self.fields = fields
        self.shape = shape
        self.count = n
        self.num_surfaces = len(surfaces)
        self.accumulate = accumulate
        self.bufs = _alloc_rays(n, dev, (self.num_surfaces,) if accumulate else (), outputs)
        self.out = _rays_struct(self.bufs, n, n if accumulate else 0)
        self.img = L.Image()
        self.counts = self.flux = self.moment = None
        if image:
            bufs = _image_buffers(sensor, wavelength_bins, dev, cos_moment=cos_moment)
            self.counts, self.flux, self.img = bufs[:3]
            if cos_moment:
                self.moment = bufs[3]
        self.launch_desc = launch if launch is not None else L.Launch()
        self.launch_desc.accumulate = 1 if accumulate else 0
        self.lib = L.load()

    def run(self, clear: bool = True) -> None:
        """One trace launch; ``clear=False`` adds to the images of earlier
        runs instead of starting from zero."""
        if self.counts is not None and clear:
            self.counts.zero_()
            self.flux.zero_()
            if self.moment is not None:
                self.moment.zero_()
        st = self.lib.otx_trace_grid(
            ctypes.byref(self.lowering.sys), ctypes.byref(self.grid), ctypes.byref(self.out),
            ctypes.byref(self.img), ctypes.byref(self.launch_desc), stream_handle(),
        )
        L.check(st, "otx_trace_grid")

    def result(self) -> RayFunctionArray:
        b = {k: (v if v is not None else None) for k, v in self.bufs.items()}
        rays = _to_ray_array_partial(b, self.shape)
        img = (self.counts, self.flux) if self.counts is not None else None
        return RayFunctionArray(inputs=None, outputs=rays, image=img)


def _to_ray_array_partial(b: dict, shape: tuple) -> RayVectorArray:
    def rs(t):
        return None if t is None else t.reshape(t.shape[:-1] + shape)

    unv = rs(b["unvignetted"])
    return RayVectorArray(
        wavelength=rs(b["wavelength"]),
        position=Cartesian3dVectorArray(rs(b["px"]), rs(b["py"]), rs(b["pz"])),
        direction=Cartesian3dVectorArray(rs(b["dx"]), rs(b["dy"]), rs(b["dz"])),
        intensity=rs(b["intensity"]),
        attenuation=rs(b["attenuation"]),
        index_refraction=rs(b["index_refraction"]),
        unvignetted=None if unv is None else unv.view(torch.bool),
        opl=rs(b["opl"]),
    )


def _is_host(values) -> bool:
    """True when every tensor argument is a CPU torch tensor (and at least one is)."""
    ts = [v for v in values if isinstance(v, torch.Tensor)]
    return bool(ts) and all(t.device.type == "cpu" for t in ts)


def _host_field(x, n: int, shape: tuple) -> tuple[torch.Tensor, int]:
    t = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x, dtype=np.float32))
    t = t.to(torch.float32)
    if t.numel() == 1:
        return t.reshape(1).contiguous(), 0
    t = t.expand(shape).reshape(-1)
    return t.contiguous(), 1


def trace_grid_host(system, *, wavelength, field, pupil, intensity=None, accumulate: bool,
                    final_local: bool, image: bool = False, wavelength_bins=None,
                    launch: L.Launch | None = None, outputs=OUTPUT_FIELDS) -> RayFunctionArray:
    """:func:`trace_grid` for host (CPU tensor) inputs, with host outputs.

    The rays stream through the GPU in chunks (``otx_trace_grid_host``):
    copies in, traces and copies out overlap.  Outputs are page-locked CPU
    tensors, complete on return (the call synchronises the current stream),
    as the reference's NumPy results are; images are copied to the host
    too.  Page-locked inputs (``tensor.pin_memory()``) give full speed."""
    dev = device()
    surfaces = system.surfaces_all
    obj = system.object
    pre = rigid_inverse(matrix_of(system.transformation)) @ (
        matrix_of(obj.transformation) if obj is not None else np.eye(4)
    )
    sensor = system.sensor
    final = None
    if final_local:
        if sensor is None:
            raise ValueError("rayfunction needs a sensor")
        final = rigid_inverse(matrix_of(sensor.transformation)) @ matrix_of(
            surfaces[-1].transformation)
    mode = L.INPUT_GRID_INFINITY if system.object_is_at_infinity else L.INPUT_GRID_FINITE
    lw = lower_surfaces(surfaces, pre=pre, final=final, input_mode=mode,
                        sensor=sensor if image else None, wavelength_bins=wavelength_bins,
                        device=dev)
    vals = [wavelength, field.x, field.y, pupil.x, pupil.y]
    if intensity is not None:
        vals.append(intensity)
    shapes = [tuple(v.shape) if isinstance(v, torch.Tensor) else np.shape(v) for v in vals]
    shape = tuple(torch.broadcast_shapes(*shapes))
    n = int(np.prod(shape)) if len(shape) else 1
    fs = [_host_field(v, n, shape) for v in vals]
    # field x/y share a stride, as do pupil x/y: expand the scalar of a mixed pair
    for a, b in ((1, 2), (3, 4)):
        if fs[a][1] != fs[b][1]:
            fs[a] = (fs[a][0].expand(n).contiguous(), 1) if fs[a][1] == 0 else fs[a]
            fs[b] = (fs[b][0].expand(n).contiguous(), 1) if fs[b][1] == 0 else fs[b]
    g = L.Grid()
    g.wavelength, g.field_x, g.field_y, g.pupil_x, g.pupil_y = (ptr(f[0]) for f in fs[:5])
    g.stride_wavelength, g.stride_field, g.stride_pupil = fs[0][1], fs[1][1], fs[3][1]
    if intensity is not None:
        g.intensity, g.stride_intensity = ptr(fs[5][0]), fs[5][1]
    g.count = n
    S = len(surfaces)
    full = (S, n) if accumulate else (n,)
    bufs = {}
    for k in OUTPUT_FIELDS:
        if k not in outputs:
            bufs[k] = None
            continue
        dt = torch.uint8 if k == "unvignetted" else (torch.float64 if k == "opl" else torch.float32)
        bufs[k] = torch.empty(full, dtype=dt, pin_memory=True)
    out = _rays_struct(bufs, n, n if accumulate else 0)
    counts = flux = None
    img = L.Image()
    if image:
        counts, flux, img = _image_buffers(sensor, wavelength_bins, dev)
    ln = launch if launch is not None else L.Launch()
    ln.accumulate = 1 if accumulate else 0
    lib = L.load()
    need = int(lib.otx_trace_grid_host_workspace(ctypes.byref(g), ctypes.byref(out),
                                                 S if accumulate else 1))
    if need < 0:
        raise ValueError("invalid host trace arguments")
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    st = lib.otx_trace_grid_host(ctypes.byref(lw.sys), ctypes.byref(g), ctypes.byref(out),
                                 ctypes.byref(img), ctypes.byref(ln), ptr(ws), need,
                                 stream_handle())
    L.check(st, "otx_trace_grid_host")
    host_img = None
    if image:
        host_img = (torch.empty(counts.shape, dtype=counts.dtype, pin_memory=True),
                    torch.empty(flux.shape, dtype=flux.dtype, pin_memory=True))
        host_img[0].copy_(counts, non_blocking=True)
        host_img[1].copy_(flux, non_blocking=True)
    torch.cuda.current_stream().synchronize()
    del ws
    rays = _to_ray_array_partial(bufs, shape)
    return RayFunctionArray(inputs=None, outputs=rays, image=host_img)


def trace_grid(system, *, wavelength, field, pupil, intensity=None, accumulate: bool,
               final_local: bool, image: bool = False, wavelength_bins=None,
               launch: L.Launch | None = None, outputs=OUTPUT_FIELDS) -> RayFunctionArray:
    """Input rays from (wavelength, field, pupil), traced through
    ``system.surfaces_all`` (optika/systems/_sequential.py:791-988).

    CPU tensor inputs take the streamed host path (:func:`trace_grid_host`)
    and give CPU outputs; anything else is moved to the GPU and gives GPU
    tensors."""
    bad = set(outputs) - set(OUTPUT_FIELDS)
    if bad:
        raise ValueError(f"unknown ray output fields {sorted(bad)}; known: {OUTPUT_FIELDS}")
    vals = [wavelength, field.x, field.y, pupil.x, pupil.y, intensity]
    if _is_host(vals):
        return trace_grid_host(system, wavelength=wavelength, field=field, pupil=pupil,
                               intensity=intensity, accumulate=accumulate,
                               final_local=final_local, image=image,
                               wavelength_bins=wavelength_bins, launch=launch, outputs=outputs)
    p = PreparedTrace(system, wavelength=wavelength, field=field, pupil=pupil,
                      intensity=intensity, accumulate=accumulate, final_local=final_local,
                      image=image, wavelength_bins=wavelength_bins, launch=launch,
                      outputs=outputs)
    p.run()
    return p.result()


def _rays_inputs(rays: RayVectorArray, dev) -> tuple[dict, tuple, int]:
    comps = dict(
        px=rays.position.x,
        py=rays.position.y,
        pz=rays.position.z,
        dx=rays.direction.x,
        dy=rays.direction.y,
        dz=rays.direction.z,
        wavelength=rays.wavelength if rays.wavelength is not None else 0.0,
        intensity=rays.intensity,
        attenuation=rays.attenuation,
        index_refraction=rays.index_refraction,
    )
    ts = {k: as_f32(v, dev) for k, v in comps.items()}
    unv = rays.unvignetted
    unv_t = (unv.to(dev) if isinstance(unv, torch.Tensor) else torch.as_tensor(np.asarray(unv), device=dev))
    opl = rays.opl
    opl_t = (opl.to(device=dev, dtype=torch.float64) if isinstance(opl, torch.Tensor)
             else torch.as_tensor(np.asarray(opl, dtype=np.float64), device=dev))
    shape = torch.broadcast_shapes(*[t.shape for t in ts.values()], unv_t.shape, opl_t.shape)
    n = int(np.prod(shape)) if len(shape) else 1
    b = {k: t.expand(shape).reshape(-1).contiguous() for k, t in ts.items()}
    b["unvignetted"] = unv_t.expand(shape).reshape(-1).to(torch.uint8).contiguous()
    b["opl"] = opl_t.expand(shape).reshape(-1).contiguous()
    return b, tuple(shape), n


def propagate_rays(surfaces: Sequence, rays: RayVectorArray, accumulate: bool = False,
                   launch: L.Launch | None = None) -> RayVectorArray:
    """optika/propagators.py:19-73 over the given surfaces, on the GPU."""
    dev = device()
    b_in, shape, n = _rays_inputs(rays, dev)
    lw = lower_surfaces(list(surfaces), pre=np.eye(4), final=None, input_mode=L.INPUT_RAYS,
                        device=dev)
    S = len(surfaces)
    bufs = _alloc_rays(n, dev, (S,) if accumulate else ())
    ln = launch if launch is not None else L.Launch()
    ln.accumulate = 1 if accumulate else 0
    lib = L.load()
    st = lib.otx_trace_rays(
        ctypes.byref(lw.sys), ctypes.byref(_rays_struct(b_in, n)),
        ctypes.byref(_rays_struct(bufs, n, n if accumulate else 0)), None, ctypes.byref(ln),
        stream_handle(),
    )
    L.check(st, "otx_trace_rays")
    return _to_ray_array(bufs, shape)


def collect(sensor, rays: RayVectorArray, wavelength=None, where=True, cos_moment=False):
    """optika/sensors/_sensors.py:92-169 on the GPU: (counts, flux) images,
    and with ``cos_moment`` the flux-weighted sum of the cosine of
    incidence as a third image."""
    dev = device()
    b_in, shape, n = _rays_inputs(rays, dev)
    if where is not True:
        w = torch.as_tensor(np.asarray(where) if not isinstance(where, torch.Tensor) else where,
                            device=dev).expand(shape).reshape(-1)
        b_in["unvignetted"] = (b_in["unvignetted"].bool() & w.bool()).to(torch.uint8)
    lw = lower_surfaces([sensor], pre=np.eye(4), final=None, input_mode=L.INPUT_RAYS,
                        sensor=sensor, wavelength_bins=wavelength)
    bufs = _image_buffers(sensor, wavelength, dev, cos_moment=cos_moment)
    img = bufs[2]
    lib = L.load()
    st = lib.otx_collect(ctypes.byref(lw.sys.sensor), ctypes.byref(_rays_struct(b_in, n)),
                         ctypes.byref(img), stream_handle())
    L.check(st, "otx_collect")
    if cos_moment:
        return bufs[0], bufs[1], bufs[3]
    return bufs[0], bufs[1]


def _sag_system(sag) -> L.System:
    from .surfaces import Surface

    return lower_surfaces([Surface(sag=sag)], pre=np.eye(4), final=None,
                          input_mode=L.INPUT_RAYS).sys


def sag_eval(sag, what: str, position):
    dev = device()
    fields, shape = _broadcast_inputs([position.x, position.y], dev)
    n = int(np.prod(shape)) if len(shape) else 1
    x = fields[0].t.expand(n).contiguous() if fields[0].stride == 0 else fields[0].t
    y = fields[1].t.expand(n).contiguous() if fields[1].stride == 0 else fields[1].t
    inp = _rays_struct(dict(px=x, py=y), n)
    lib = L.load()
    sys_ = _sag_system(sag)
    if what == "sag":
        z = torch.empty(n, dtype=torch.float32, device=dev)
        out = _rays_struct(dict(pz=z), n)
        L.check(lib.otx_sag_eval(ctypes.byref(sys_), 0, ctypes.byref(inp), ctypes.byref(out),
                                 stream_handle()), "otx_sag_eval")
        return z.reshape(shape)
    nx, ny, nz = (torch.empty(n, dtype=torch.float32, device=dev) for _ in range(3))
    out = _rays_struct(dict(dx=nx, dy=ny, dz=nz), n)
    L.check(lib.otx_sag_eval(ctypes.byref(sys_), 1, ctypes.byref(inp), ctypes.byref(out),
                             stream_handle()), "otx_sag_eval")
    return Cartesian3dVectorArray(nx.reshape(shape), ny.reshape(shape), nz.reshape(shape))


def sag_intercept(sag, rays: RayVectorArray) -> RayVectorArray:
    dev = device()
    b_in, shape, n = _rays_inputs(rays, dev)
    px, py, pz = (torch.empty(n, dtype=torch.float32, device=dev) for _ in range(3))
    out = _rays_struct(dict(px=px, py=py, pz=pz), n)
    lib = L.load()
    sys_ = _sag_system(sag)
    L.check(lib.otx_sag_eval(ctypes.byref(sys_), 2, ctypes.byref(_rays_struct(b_in, n)),
                             ctypes.byref(out), stream_handle()), "otx_sag_eval")
    res = _to_ray_array({**b_in, "px": px, "py": py, "pz": pz}, shape)
    return res


def rulings_eval(rulings, what: str, rays: RayVectorArray, normal):
    """Groove efficiency (``what="efficiency"``) or the rays with their
    effective incident direction (``"incident_effective"``) of ``rulings``
    for rays at the ruled surface, through otx_rulings_eval."""
    from .surfaces import Surface

    dev = device()
    comps = dict(px=rays.position.x, py=rays.position.y, pz=rays.position.z,
                 dx=rays.direction.x, dy=rays.direction.y, dz=rays.direction.z,
                 wavelength=rays.wavelength, index_refraction=rays.index_refraction,
                 nx=normal.x, ny=normal.y, nz=normal.z)
    ts = {k: as_f32(v, dev) for k, v in comps.items()}
    shape = tuple(torch.broadcast_shapes(*[t.shape for t in ts.values()]))
    n = int(np.prod(shape)) if len(shape) else 1
    b = {k: t.expand(shape).reshape(-1).contiguous() for k, t in ts.items()}
    lw = lower_surfaces([Surface(rulings=rulings)], pre=np.eye(4), final=None,
                        input_mode=L.INPUT_RAYS, device=dev)
    lib = L.load()
    rs = _rays_struct({k: b[k] for k in ("px", "py", "pz", "dx", "dy", "dz", "wavelength",
                                         "index_refraction")}, n)
    ns = _rays_struct(dict(dx=b["nx"], dy=b["ny"], dz=b["nz"]), n)
    if what == "efficiency":
        eff = torch.empty(n, dtype=torch.float32, device=dev)
        L.check(lib.otx_rulings_eval(ctypes.byref(lw.sys), 0, ctypes.byref(rs), ctypes.byref(ns),
                                     ptr(eff), None, stream_handle()), "otx_rulings_eval")
        return eff.reshape(shape)
    dx, dy, dz = (torch.empty(n, dtype=torch.float32, device=dev) for _ in range(3))
    out = _rays_struct(dict(dx=dx, dy=dy, dz=dz), n)
    L.check(lib.otx_rulings_eval(ctypes.byref(lw.sys), 1, ctypes.byref(rs), ctypes.byref(ns),
                                 None, ctypes.byref(out), stream_handle()), "otx_rulings_eval")
    return dataclasses.replace(
        rays, direction=Cartesian3dVectorArray(dx.reshape(shape), dy.reshape(shape),
                                               dz.reshape(shape)))


def multilayer_efficiency_gpu(wavelength, direction, n, layers, substrate):
    dev = device()
    from ._lower import Lowering

    lw = Lowering()
    lw.add_stack(layers, substrate)
    lw.finish_tables(dev)
    n_arr = np.asarray(n) if not isinstance(n, torch.Tensor) else n
    if isinstance(n_arr, torch.Tensor):
        n_re, n_im = n_arr.real if n_arr.is_complex() else n_arr, (
            n_arr.imag if n_arr.is_complex() else torch.zeros_like(n_arr))
    else:
        n_re, n_im = np.real(n_arr), np.imag(n_arr)
    fields, shape = _broadcast_inputs([wavelength, direction, n_re, n_im], dev)
    cnt = int(np.prod(shape)) if len(shape) else 1
    if fields[2].stride != fields[3].stride:
        for f in fields[2:4]:
            if f.stride == 0:
                f.t = f.t.expand(cnt).contiguous()
                f.stride = 1
    outs = [torch.empty(cnt, dtype=torch.float32, device=dev) for _ in range(4)]
    lib = L.load()
    st = lib.otx_multilayer_efficiency(
        ctypes.byref(lw.sys), cnt, ptr(fields[0].t), fields[0].stride, ptr(fields[1].t),
        fields[1].stride, ptr(fields[2].t), ptr(fields[3].t), fields[2].stride, None,
        *(ptr(o) for o in outs), stream_handle(),
    )
    L.check(st, "otx_multilayer_efficiency")
    rs, rp, ts, tp = (o.reshape(shape) for o in outs)
    return PolarizationVectorArray(rs, rp), PolarizationVectorArray(ts, tp)


def periodic_table(mirrors, dev) -> torch.Tensor:
    """Pack PeriodicMirror descriptions into a device otx_periodic_stack array."""
    arr = (L.PeriodicStack * len(mirrors))()
    for i, m in enumerate(mirrors):
        na, nb, ns = (complex(x.chemical) for x in (m.a, m.b, m.substrate))
        d = arr[i]
        d.n_a_re, d.n_a_im = na.real, na.imag
        d.n_b_re, d.n_b_im = nb.real, nb.imag
        d.n_sub_re, d.n_sub_im = ns.real, ns.imag
        d.thickness_a, d.thickness_b = float(m.a.thickness), float(m.b.thickness)
        d.num_periods = int(m.num_periods)
    raw = bytes(arr)
    return torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(dev)


def multilayer_periodic_gpu(wavelength, direction, mirrors, index, n):
    dev = device()
    table = periodic_table(mirrors, dev)
    fields, shape = _broadcast_inputs([wavelength, direction], dev)
    cnt = int(np.prod(shape)) if len(shape) else 1
    idx = None
    if index is not None:
        idx = torch.as_tensor(np.asarray(index) if not isinstance(index, torch.Tensor) else index,
                              device=dev).to(torch.int32).expand(shape).reshape(-1).contiguous()
    outs = [torch.empty(cnt, dtype=torch.float32, device=dev) for _ in range(4)]
    n = complex(n)
    lib = L.load()
    st = lib.otx_multilayer_periodic(
        ptr(table), len(mirrors), cnt, ptr(fields[0].t), fields[0].stride, ptr(fields[1].t),
        fields[1].stride, ptr(idx), n.real, n.imag, *(ptr(o) for o in outs), stream_handle(),
    )
    L.check(st, "otx_multilayer_periodic")
    rs, rp, ts, tp = (o.reshape(shape) for o in outs)
    return PolarizationVectorArray(rs, rp), PolarizationVectorArray(ts, tp)


def cell_rays(cells: L.Cells, first: int, count: int, grid: L.Grid) -> None:
    """Input rays of scene cells [first, first + count) into the grid's
    arrays (otx_cell_rays)."""
    L.check(L.load().otx_cell_rays(ctypes.byref(cells), first, count, ctypes.byref(grid),
                                   stream_handle()), "otx_cell_rays")


def expose(photons: torch.Tensor, scale: float, read_noise: float, noise: bool,
           seed: int) -> torch.Tensor:
    """Electrons of an ideal sensor (otx_expose) from a photon image."""
    p = photons.to(device=device(), dtype=torch.float32).contiguous()
    out = torch.empty_like(p)
    L.check(L.load().otx_expose(ptr(p), ptr(out), p.numel(), float(scale), float(read_noise),
                                1 if noise else 0, int(seed) & (2**64 - 1), stream_handle()),
            "otx_expose")
    return out
