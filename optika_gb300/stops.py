"""The stop solver: rays that strike the edges of the field and pupil stops,
and the normalised field / pupil coordinates they define.

Follows optika/systems/_sequential.py:343-361 (``_anchor_surface``),
363-394 (``_ray_error``), 396-693 (``_calc_rayfunction_stops_only``),
695-754 (``_calc_rayfunction_stops``), 755-799 (``field_min`` ...
``pupil_max``) and 801-850 (``_denormalize_grid``).

For every pair of a point on the first stop's boundary and a point on the
last stop's (21 x 21 pairs), Newton's method finds the free component of
the ray at the first stop (its direction, or its position when the first
stop's aperture is angular) that lands the ray on the target point of the
last stop.  The whole Newton solve runs in one kernel launch
(``otx_stop_newton``): one thread per ray traces it and its two
finite-difference perturbations through the surfaces between the stops in
every iteration and applies the 2 x 2 update, with no host round trip.
The solved rays are then traced back to the object surface (the reversed
surface list, as the reference does).

The trace is FP32, so the convergence test uses the larger of the
reference's 1e-9 (times the target aperture's size) and a floor of 4e-7 of
it, and two further Newton steps polish each ray's root to the trace's
noise (the reference stops when every ray has converged; here each ray
stops on its own);
the extents agree with the float64 restatement to ~1e-6 relative (see the
tests).
"""

from __future__ import annotations

from typing import Sequence

import numpy as np
import torch

from . import transforms
from ._api import device

SAMPLES_STOP = 21
MAX_ITER = 60


def anchor_surface(subsystem: Sequence):
    """The first surface after the start of ``subsystem`` with optical
    power (a mirror, a curved sag or rulings), else the last one
    (optika/systems/_sequential.py:343-361)."""
    for surface in subsystem[1:]:
        mat = surface.material
        if mat is not None and getattr(mat, "is_mirror", False):
            return surface
        if surface.sag is not None and type(surface.sag).__name__ != "NoSag":
            return surface
        if surface.rulings is not None:
            return surface
    return subsystem[-1]


def _matrix(t) -> torch.Tensor:
    return torch.as_tensor(transforms.matrix_of(t), dtype=torch.float64, device=device())


def _apply(M: torch.Tensor, p: torch.Tensor, point: bool = True) -> torch.Tensor:
    """x' = R x (+ t) for p of shape [3, ...] (float64)."""
    out = torch.einsum("ij,j...->i...", M[:3, :3], p)
    if point:
        out = out + M[:3, 3].reshape((3,) + (1,) * (p.dim() - 1))
    return out


def _inverse(M: torch.Tensor) -> torch.Tensor:
    out = torch.eye(4, dtype=M.dtype, device=M.device)
    out[:3, :3] = M[:3, :3].T
    out[:3, 3] = -M[:3, :3].T @ M[:3, 3]
    return out


def _sag(sag, x: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
    """Sag values on the device (the sag kernel, float32)."""
    from .vectors import Cartesian2dVectorArray

    return sag(Cartesian2dVectorArray(x.float(), y.float())).to(torch.float64)


def _api_sag_system(sag):
    from ._api import _sag_system

    return _sag_system(sag)


def _sag_normal(lowered, x: torch.Tensor, y: torch.Tensor):
    """Unit normals (float64 tensors) of a lowered sag at (x, y): the sag
    kernel (otx_sag_eval, float32) with the descriptor made once."""
    import ctypes

    from . import _api
    from . import _lib as L

    n = x.numel()
    xy = torch.stack([x.reshape(-1), y.reshape(-1)]).to(torch.float32)
    nrm = torch.empty((3, n), dtype=torch.float32, device=x.device)
    inp = _api._rays_struct(dict(px=xy[0], py=xy[1]), n)
    out = _api._rays_struct(dict(dx=nrm[0], dy=nrm[1], dz=nrm[2]), n)
    L.check(L.load().otx_sag_eval(ctypes.byref(lowered), 1, ctypes.byref(inp), ctypes.byref(out),
                                  _api.stream_handle()), "otx_sag_eval")
    nrm = nrm.to(torch.float64)
    return nrm[0].reshape(x.shape), nrm[1].reshape(x.shape), nrm[2].reshape(x.shape)


def _lower(surfaces: Sequence):
    """The descriptor of ``surfaces`` for repeated traces within one solve."""
    from . import _lib as L
    from ._lower import lower_surfaces

    return lower_surfaces(list(surfaces), pre=np.eye(4), final=None, input_mode=L.INPUT_RAYS,
                          device=device())


def _cached(system, key, make):
    """A descriptor, or the wavelength-independent setup of a solve, made
    once per system and key: the stop solve of a system repeats for every
    batch of wavelengths, and the extents it gives are cached on the system
    the same way."""
    cache = system.__dict__.setdefault("_stop_lowerings", {})
    key = (str(device()),) + tuple(key)  # descriptors and tensors live on one device
    if key not in cache:
        cache[key] = make()
    return cache[key]


def _trace(surfaces: Sequence, p: torch.Tensor, d: torch.Tensor, wavelength, lowering=None):
    """Rays [3, N] (system frame, float64 on the host side of the kernel
    call) through ``surfaces``: one launch of the trace kernel
    (otx_trace_rays) with only the position, direction and wavelength given
    (the other ray fields take their defaults) and only position and
    direction written.  ``wavelength`` is one value or a tensor [N];
    ``lowering`` is the descriptor from :func:`_lower`, made once per
    solve."""
    import ctypes

    from . import _api
    from . import _lib as L

    n = p.shape[1]
    dev = p.device
    lw = lowering if lowering is not None else _lower(surfaces)
    wl = (wavelength.to(device=dev, dtype=torch.float32).contiguous()
          if isinstance(wavelength, torch.Tensor)
          else torch.full((n,), float(wavelength), device=dev))
    pf = p.to(torch.float32).contiguous()
    df = d.to(torch.float32).contiguous()
    inp = dict(px=pf[0], py=pf[1], pz=pf[2], dx=df[0], dy=df[1], dz=df[2], wavelength=wl)
    out = torch.empty((6, n), dtype=torch.float32, device=dev)
    outs = dict(px=out[0], py=out[1], pz=out[2], dx=out[3], dy=out[4], dz=out[5])
    L.check(L.load().otx_trace_rays(
        ctypes.byref(lw.sys), ctypes.byref(_api._rays_struct(inp, n)),
        ctypes.byref(_api._rays_struct(outs, n)), None, ctypes.byref(L.Launch()),
        _api.stream_handle()), "otx_trace_rays")
    o = out.to(torch.float64)
    return o[:3], o[3:]


def _newton(lowering, first, pos_f, dir_f, wl_f, tx, ty, to_last: list, *, free_position: bool,
            target_direction: bool, step: float, tol: float) -> torch.Tensor:
    """The Newton iterations of every ray on the device (otx_stop_newton):
    ``pos_f`` / ``dir_f`` ([3, n] float64, system frame) are updated in
    place with the solved rays.  One thread per ray: each iteration traces
    the ray and its two finite-difference perturbations and applies the
    2 x 2 update; a ray whose residual drops below ``tol`` takes two more
    steps.  Returns a device flag, true when some ray did not converge:
    the host reads it with the results, so nothing waits for the solve
    before the work that follows it is queued."""
    import ctypes

    from . import _api
    from . import _lib as L

    n = pos_f.shape[1]
    dev = pos_f.device
    f64 = torch.float64
    pos = pos_f.to(f64).contiguous()
    dirn = dir_f.to(f64).contiguous()
    wl = wl_f.to(f64).contiguous()
    txc, tyc = tx.to(f64).contiguous(), ty.to(f64).contiguous()
    status = torch.empty(n, dtype=torch.int32, device=dev)
    sol = L.StopSolve()
    sol.count = n
    sol.free_position = int(free_position)
    sol.target_direction = int(target_direction)
    sol.max_iterations = MAX_ITER
    sol.polish_steps = 2
    sol.step = float(step)
    sol.tolerance = float(tol)
    for k, v in enumerate(to_last):
        sol.to_last[k] = v
    sol.position, sol.direction, sol.wavelength = (_api.ptr(t) for t in (pos, dirn, wl))
    sol.target_x, sol.target_y, sol.status = (_api.ptr(t) for t in (txc, tyc, status))
    L.check(L.load().otx_stop_newton(ctypes.byref(lowering.sys), ctypes.byref(first),
                                     ctypes.byref(sol), _api.stream_handle()), "otx_stop_newton")
    pos_f.copy_(pos)
    dir_f.copy_(dirn)
    return (status < 0).any()


def _seed(sub: Sequence, samples_pupil: int, samples_field: int) -> dict:
    """The wavelength-independent part of a stop solve between the first and
    last surfaces of ``sub``: the boundary grids, the first guesses (aimed
    at the first surface with power, or at the target itself), the targets
    and the tolerances (optika/systems/_sequential.py:396-560).  Made once
    per system and stop pair."""
    dev = device()
    f64 = torch.float64
    s_first, s_last = sub[0], sub[-1]
    gf = torch.as_tensor(s_first.aperture.wire(samples_pupil)[:, :2], dtype=f64, device=dev)
    gl = torch.as_tensor(s_last.aperture.wire(samples_field)[:, :2], dtype=f64, device=dev)
    shape = (gf.shape[0], gl.shape[0])
    gx = gf[:, 0:1].expand(shape)
    gy = gf[:, 1:2].expand(shape)
    if not s_first.aperture.dimensionless:
        pos = torch.stack([gx, gy, _sag(s_first.sag, gx, gy)])
        dirn = torch.stack([torch.zeros(shape, dtype=f64, device=dev),
                            torch.zeros(shape, dtype=f64, device=dev),
                            torch.ones(shape, dtype=f64, device=dev)])
        variable = "direction"
    else:
        dirn = torch.stack([gx, gy, torch.sqrt(1 - (gx * gx + gy * gy))])
        pos = torch.zeros((3,) + shape, dtype=f64, device=dev)
        variable = "position"

    # seed: aim at the first surface with power, or at the target itself
    anchor = anchor_surface(sub)
    if anchor is s_last and not s_last.aperture.dimensionless:
        ax_ = gl[None, :, 0].expand(shape)
        ay_ = gl[None, :, 1].expand(shape)
        aim = torch.stack([ax_, ay_, _sag(s_last.sag, ax_, ay_)])
        aim = _apply(_matrix(s_last.transformation), aim)
    else:
        aim = _apply(_matrix(anchor.transformation),
                     torch.zeros((3,) + shape, dtype=f64, device=dev))
    aim = _apply(_inverse(_matrix(s_first.transformation)), aim)
    if variable == "direction":
        d = aim - pos
        d = d / torch.sqrt((d * d).sum(0))
        flip = torch.sign(d[2])
        where = d[2] != 0
        dirn = torch.stack([torch.where(where, flip * d[0], 0.0),
                            torch.where(where, flip * d[1], 0.0),
                            torch.where(where, flip * d[2], 1.0)])
    else:
        t = aim[2] / dirn[2]
        px, py = aim[0] - dirn[0] * t, aim[1] - dirn[1] * t
        pos = torch.stack([px, py, _sag(s_first.sag, px, py)])
    M = _matrix(s_first.transformation)
    pos = _apply(M, pos)
    dirn = _apply(M, dirn, point=False)
    target = "direction" if s_last.aperture.dimensionless else "position"
    tx = gl[None, :, 0].expand(shape).reshape(-1)
    ty = gl[None, :, 1].expand(shape).reshape(-1)
    scale = max(float(np.ptp(gl[:, 0].cpu().numpy())), float(np.ptp(gl[:, 1].cpu().numpy())))
    unit = max(scale, 1.0)
    tol = max(1e-9 * unit, 4e-7 * unit)
    dx = 1e-4 if variable == "direction" else 1e-4 * unit
    Tl = _inverse(_matrix(s_last.transformation))
    return dict(shape=shape, variable=variable, target=target, pos=pos, dirn=dirn, tx=tx, ty=ty,
                tol=tol, step=dx, to_last=Tl[:3, :4].reshape(-1).cpu().tolist())


def stops_only(system, wavelength, samples_pupil: int = SAMPLES_STOP,
               samples_field: int = SAMPLES_STOP) -> dict:
    """Rays (system frame, [3, first wire, last wire]) from the first stop
    that strike every point of the last stop's boundary
    (optika/systems/_sequential.py:396-693).  ``wavelength`` may be a 1-D
    array: every wavelength is solved in the same Newton iterations (one
    trace launch per iteration for all of them) and the arrays gain a
    wavelength axis after the first, [3, wavelength, first wire, last
    wire].  Raises ValueError when some ray does not converge."""
    out = _stops_only(system, wavelength, samples_pupil, samples_field)
    _check([bool(f) for f in out.pop("failed")], out.pop("stops"))
    return out


def _stops_only(system, wavelength, samples_pupil: int = SAMPLES_STOP,
                samples_field: int = SAMPLES_STOP) -> dict:
    """:func:`stops_only` without reading the convergence flags: ``failed``
    holds one device flag per stop pair and ``stops`` their names."""
    scalar = np.ndim(wavelength) == 0
    wls = np.atleast_1d(np.asarray(wavelength, dtype=np.float64))
    nw = len(wls)
    surfaces = system.surfaces_all
    ip = [i for i, s in enumerate(surfaces) if s.is_pupil_stop]
    jf = [i for i, s in enumerate(surfaces) if s.is_field_stop]
    if not ip:
        raise ValueError("pupil not defined: set is_pupil_stop=True on a surface")
    if not jf:
        raise ValueError("field stop not defined: set is_field_stop=True on a surface")
    dev = device()
    f64 = torch.float64
    out = None
    flags, names = [], []
    while ip and jf:
        first_i, last_i = min(ip[0], jf[0]), max(ip[0], jf[0])
        sub = surfaces[first_i:last_i + 1]
        s_first, s_last = sub[0], sub[-1]
        if s_first.is_pupil_stop:
            ip.pop(0)
        else:
            jf.pop(0)
        plan = _cached(system, ("plan", first_i, last_i, samples_pupil, samples_field),
                       lambda: _seed(sub, samples_pupil, samples_field))
        shape, variable, target = plan["shape"], plan["variable"], plan["target"]
        pos, dirn, tx, ty = plan["pos"], plan["dirn"], plan["tx"], plan["ty"]
        # every wavelength repeats the grid (wavelength-major)
        pos_f = pos.reshape(3, -1).repeat(1, nw)
        dir_f = dirn.reshape(3, -1).repeat(1, nw)
        tx = tx.repeat(nw)
        ty = ty.repeat(nw)
        wl_f = torch.as_tensor(wls, dtype=f64, device=dev).repeat_interleave(shape[0] * shape[1])

        lw_sub = _cached(system, ("sub", first_i, last_i), lambda: _lower(sub[1:]))
        first = _cached(system, ("sag", first_i), lambda: _api_sag_system(s_first.sag))
        failed = _newton(lw_sub, first, pos_f, dir_f, wl_f, tx, ty, plan["to_last"],
                         free_position=variable == "position",
                         target_direction=target == "direction", step=plan["step"],
                         tol=plan["tol"])
        flags.append(failed)
        names.append((s_first.name, s_last.name))
        full = (3,) + ((nw,) if not scalar else ()) + shape
        out = dict(position=pos_f.reshape(full), direction=dir_f.reshape(full),
                   wavelength=wl_f.reshape(full[1:]))
    out.update(failed=flags, stops=names)
    return out


def _check(failed: list, stops: list) -> None:
    """Raise for the first stop pair whose solve did not converge."""
    for f, (a, b) in zip(failed, stops):
        if f:
            raise ValueError(f"could not solve for the rays connecting the stop surfaces "
                             f"{a!r} and {b!r}")


def rayfunction_stops(system, wavelength, samples_pupil: int = SAMPLES_STOP,
                      samples_field: int = SAMPLES_STOP) -> dict:
    """The stop rays traced back to the object surface, directions pointing
    into the system, with the field and pupil grids they give: angles
    (rad) for the side at infinity, positions (mm) for the other
    (optika/systems/_sequential.py:695-754).  A 1-D ``wavelength`` adds a
    leading wavelength axis to every grid.  Raises ValueError when some
    ray of the stop solve does not converge."""
    out = _rayfunction_stops(system, wavelength, samples_pupil, samples_field)
    _check([bool(f) for f in out.pop("failed")], out.pop("stops"))
    return out


def _rayfunction_stops(system, wavelength, samples_pupil: int = SAMPLES_STOP,
                       samples_field: int = SAMPLES_STOP) -> dict:
    """:func:`rayfunction_stops` with the convergence flags left on the
    device (``failed``, ``stops`` as in :func:`_stops_only`)."""
    st = _stops_only(system, wavelength, samples_pupil, samples_field)
    surfaces = system.surfaces_all
    ip = max(i for i, s in enumerate(surfaces) if s.is_pupil_stop)
    jf = max(i for i, s in enumerate(surfaces) if s.is_field_stop)
    sub = surfaces[min(ip, jf)::-1]
    p, d = st["position"], st["direction"]
    shape = p.shape[1:]
    lw_back = _cached(system, ("back", min(ip, jf)), lambda: _lower(sub))
    po, do = _trace(sub, p.reshape(3, -1), d.reshape(3, -1), st["wavelength"].reshape(-1),
                    lw_back)
    obj = sub[-1]
    Mi = _cached(system, ("obj_inverse", min(ip, jf)), lambda: _inverse(_matrix(obj.transformation)))
    pl = _apply(Mi, po)
    dl = _apply(Mi, do, point=False)
    obj_sag = _cached(system, ("object_sag", min(ip, jf)),
                      lambda: _api_sag_system(obj.sag))
    nx, ny, nz = _sag_normal(obj_sag, pl[0], pl[1])
    dot = dl[0] * nx + dl[1] * ny + dl[2] * nz
    do = torch.where(dot > 0, -do, do)
    if system.transformation is not None:
        M = _cached(system, ("system", 0), lambda: _matrix(system.transformation))
        po, do = _apply(M, po), _apply(M, do, point=False)
    ang_x = -torch.atan2(do[0], do[2])
    ang_y = -torch.asin(do[1] / torch.sqrt((do * do).sum(0)))
    if system.object_is_at_infinity:
        field, pupil = (ang_x, ang_y), (po[0], po[1])
    else:
        field, pupil = (po[0], po[1]), (ang_x, ang_y)
    return dict(position=po.reshape((3,) + shape), direction=do.reshape((3,) + shape),
                field=tuple(f.reshape(shape) for f in field),
                pupil=tuple(q.reshape(shape) for q in pupil), failed=st["failed"],
                stops=st["stops"])


def extents(system, wavelength: float) -> tuple:
    """(field_min, field_max, pupil_min, pupil_max), each an (x, y) pair of
    floats, cached on the system per wavelength
    (optika/systems/_sequential.py:755-799)."""
    return extents_many(system, [wavelength])[0]


def extents_many(system, wavelengths) -> list[tuple]:
    """:func:`extents` of several wavelengths; the ones not yet cached are
    solved together (one batched Newton solve, see :func:`stops_only`)."""
    cache = system.__dict__.setdefault("_stop_extents", {})
    keys = [float(w) for w in np.atleast_1d(np.asarray(wavelengths, dtype=np.float64))]
    todo = sorted({k for k in keys if k not in cache})
    if todo:
        st = _rayfunction_stops(system, np.array(todo))
        f, q = st["field"], st["pupil"]
        g = torch.stack([a.reshape(len(todo), -1) for a in (*f, *q)])  # [4, wl, rays]
        lo_hi = torch.stack([g.amin(2), g.amax(2)], 1).reshape(-1)
        flags = torch.stack(st["failed"]).to(lo_hi.dtype)
        host = torch.cat([lo_hi, flags]).cpu().numpy()  # the one read of the solve
        _check(list(host[lo_hi.numel():] != 0), st["stops"])
        lo_hi = host[:lo_hi.numel()].reshape(4, 2, len(todo))
        red = [(lo_hi[i, 0], lo_hi[i, 1]) for i in range(4)]
        for j, k in enumerate(todo):
            (fx0, fx1), (fy0, fy1), (qx0, qx1), (qy0, qy1) = red
            cache[k] = ((float(fx0[j]), float(fy0[j])), (float(fx1[j]), float(fy1[j])),
                        (float(qx0[j]), float(qy0[j])), (float(qx1[j]), float(qy1[j])))
    return [cache[k] for k in keys]


def _values(x):
    if isinstance(x, torch.Tensor):
        return x.detach().reshape(-1).double().cpu().numpy()
    return np.asarray(x, dtype=np.float64).reshape(-1)


def denormalize(system, wavelength, field, pupil, normalized_field: bool,
                normalized_pupil: bool):
    """Physical field and pupil coordinates from normalised ones:
    ``min + ptp (v + 1) / 2`` per component, with the stop extents at each
    ray's wavelength (optika/systems/_sequential.py:801-850).  ``field`` and
    ``pupil`` are (x, y) pairs of arrays or tensors; the results keep their
    kind and device."""
    ws = np.unique(_values(wavelength))
    if len(ws) > 64:
        raise ValueError("normalised coordinates support at most 64 distinct wavelengths")
    ext = extents_many(system, ws)

    def table(which: int, comp: int):
        lo = np.array([e[which][comp] for e in ext])
        hi = np.array([e[which + 1][comp] for e in ext])
        return lo, hi - lo

    def map_one(v, lo, ptp):
        if len(ws) == 1:
            return ptp[0] * (v + 1) / 2 + lo[0]
        if isinstance(v, torch.Tensor):
            w = wavelength if isinstance(wavelength, torch.Tensor) else torch.as_tensor(
                np.asarray(wavelength, dtype=np.float64))
            w = w.to(device=v.device, dtype=torch.float64)
            idx = torch.searchsorted(torch.as_tensor(ws, device=v.device), w)
            lo_t = torch.as_tensor(lo, device=v.device)[idx]
            ptp_t = torch.as_tensor(ptp, device=v.device)[idx]
            return (ptp_t * (v.double() + 1) / 2 + lo_t).to(v.dtype)
        idx = np.searchsorted(ws, np.asarray(wavelength, dtype=np.float64))
        return ptp[idx] * (np.asarray(v) + 1) / 2 + lo[idx]

    fx, fy = field
    qx, qy = pupil
    if normalized_field:
        lo, ptp = table(0, 0)
        fx = map_one(fx, lo, ptp)
        lo, ptp = table(0, 1)
        fy = map_one(fy, lo, ptp)
    if normalized_pupil:
        lo, ptp = table(2, 0)
        qx = map_one(qx, lo, ptp)
        lo, ptp = table(2, 1)
        qy = map_one(qy, lo, ptp)
    return (fx, fy), (qx, qy)


__all__ = ["anchor_surface", "stops_only", "rayfunction_stops", "extents", "extents_many",
           "denormalize"]
