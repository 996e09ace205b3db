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
last stop.  Each Newton iteration evaluates the rays and their two
finite-difference perturbations in ONE launch of the trace kernel
(``otx_trace_rays`` over the surfaces between the stops); the 2 x 2 updates
run on the same device tensors.  The solved rays are then traced back to
the object surface (the reversed surface list, as the reference does).

The trace is FP32, so the convergence test uses the larger of the
reference's 1e-9 (times the target aperture's size) and a floor of 4e-7 of
it, and two further Newton steps polish each root to the trace's noise;
the extents agree with the float64 restatement to ~1e-6 relative (see the
tests).
"""

from __future__ import annotations

from typing import Sequence

import numpy as np
import torch

from . import transforms
from ._api import device, propagate_rays
from .rays import RayVectorArray
from .vectors import Cartesian3dVectorArray

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


def _trace(surfaces: Sequence, p: torch.Tensor, d: torch.Tensor, wavelength: float):
    """Rays [3, N] (system frame, float64 on the host side of the kernel
    call) through ``surfaces``: one launch of the trace kernel."""
    n = p.shape[1]
    dev = p.device
    rays = RayVectorArray(
        wavelength=torch.full((n,), float(wavelength), device=dev),
        position=Cartesian3dVectorArray(*(p[i].float() for i in range(3))),
        direction=Cartesian3dVectorArray(*(d[i].float() for i in range(3))),
        intensity=torch.ones(n, device=dev),
        attenuation=torch.zeros(n, device=dev),
        index_refraction=torch.ones(n, device=dev),
        unvignetted=torch.ones(n, dtype=torch.bool, device=dev),
        opl=torch.zeros(n, dtype=torch.float64, device=dev),
    )
    out = propagate_rays(list(surfaces), rays)
    po = torch.stack([out.position.x, out.position.y, out.position.z]).to(torch.float64)
    do = torch.stack([out.direction.x, out.direction.y, out.direction.z]).to(torch.float64)
    return po, do


def stops_only(system, wavelength: float, samples_pupil: int = SAMPLES_STOP,
               samples_field: int = SAMPLES_STOP) -> dict:
    """Rays (system frame, [3, first wire, last wire]) from the first stop
    that strike every point of the last stop's boundary
    (optika/systems/_sequential.py:396-693)."""
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
    while ip and jf:
        first_i, last_i = min(ip[0], jf[0]), max(ip[0], jf[0])
        sub = surfaces[first_i:last_i + 1]
        s_first, s_last = sub[0], sub[-1]
        gf = torch.as_tensor(s_first.aperture.wire(samples_pupil)[:, :2], dtype=f64, device=dev)
        gl = torch.as_tensor(s_last.aperture.wire(samples_field)[:, :2], dtype=f64, device=dev)
        if s_first.is_pupil_stop:
            ip.pop(0)
        else:
            jf.pop(0)
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

        def zf(x, y):
            if variable == "direction":
                return torch.sqrt(1 - (x * x + y * y))
            return _sag(s_first.sag, x, y)

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
        n = shape[0] * shape[1]
        pos_f = pos.reshape(3, n)
        dir_f = dirn.reshape(3, n)

        def residuals(xs, ys):
            """Residuals of len(xs) / n stacked evaluations in one launch."""
            k = xs.shape[0] // n
            p = pos_f.repeat(1, k)
            d = dir_f.repeat(1, k)
            v = d if variable == "direction" else p
            v[0], v[1], v[2] = xs, ys, zf(xs, ys)
            po, do = _trace(sub[1:], p, d, wavelength)
            if target == "direction":
                c = _apply(Tl, do, point=False)
            else:
                c = _apply(Tl, po)
            return c[0] - tx.repeat(k), c[1] - ty.repeat(k)

        v0 = dir_f if variable == "direction" else pos_f
        x, y = v0[0].clone(), v0[1].clone()
        polish = -1
        for _ in range(MAX_ITER):
            xs = torch.cat([x, x + dx, x])
            ys = torch.cat([y, y, y + dx])
            rx, ry = residuals(xs, ys)
            fx, fy = rx[:n], ry[:n]
            err = torch.maximum(fx.abs(), fy.abs())
            if polish < 0 and bool((err < tol).all()):
                polish = 2
            if polish == 0:
                break
            j11, j21 = (rx[n:2 * n] - fx) / dx, (ry[n:2 * n] - fy) / dx
            j12, j22 = (rx[2 * n:] - fx) / dx, (ry[2 * n:] - fy) / dx
            det = j11 * j22 - j12 * j21
            ok = torch.isfinite(det) & (det != 0)
            sx = torch.where(ok, (j22 * fx - j12 * fy) / det, 0.0)
            sy = torch.where(ok, (-j21 * fx + j11 * fy) / det, 0.0)
            x, y = x - sx, y - sy
            if polish > 0:
                polish -= 1
        else:
            raise ValueError(
                f"could not solve for the rays connecting the stop surfaces "
                f"{s_first.name!r} and {s_last.name!r}")
        v = dir_f if variable == "direction" else pos_f
        v[0], v[1], v[2] = x, y, zf(x, y)
        out = dict(position=pos_f.reshape((3,) + shape), direction=dir_f.reshape((3,) + shape))
    return out


def rayfunction_stops(system, wavelength: float, samples_pupil: int = SAMPLES_STOP,
                      samples_field: int = SAMPLES_STOP) -> dict:
    """The stop rays traced back to the object surface, directions pointing
    into the system, with the field and pupil grids they give: angles
    (rad) for the side at infinity, positions (mm) for the other
    (optika/systems/_sequential.py:695-754)."""
    st = stops_only(system, wavelength, samples_pupil, samples_field)
    surfaces = system.surfaces_all
    ip = max(i for i, s in enumerate(surfaces) if s.is_pupil_stop)
    jf = max(i for i, s in enumerate(surfaces) if s.is_field_stop)
    sub = surfaces[min(ip, jf)::-1]
    p, d = st["position"], st["direction"]
    shape = p.shape[1:]
    po, do = _trace(sub, p.reshape(3, -1), d.reshape(3, -1), wavelength)
    obj = sub[-1]
    Mi = _inverse(_matrix(obj.transformation))
    pl = _apply(Mi, po)
    dl = _apply(Mi, do, point=False)
    from .vectors import Cartesian2dVectorArray

    nrm = obj.sag.normal(Cartesian2dVectorArray(pl[0].float(), pl[1].float()))
    dot = dl[0] * nrm.x.double() + dl[1] * nrm.y.double() + dl[2] * nrm.z.double()
    do = torch.where(dot > 0, -do, do)
    if system.transformation is not None:
        M = _matrix(system.transformation)
        po, do = _apply(M, po), _apply(M, do, point=False)
    ang_x = -torch.atan2(do[0], do[2])
    ang_y = -torch.asin(do[1] / torch.sqrt((do * do).sum(0)))
    if system.object_is_at_infinity:
        field, pupil = (ang_x, ang_y), (po[0], po[1])
    else:
        field, pupil = (po[0], po[1]), (ang_x, ang_y)
    return dict(position=po.reshape((3,) + shape), direction=do.reshape((3,) + shape),
                field=tuple(f.reshape(shape) for f in field),
                pupil=tuple(q.reshape(shape) for q in pupil))


def extents(system, wavelength: float) -> tuple:
    """(field_min, field_max, pupil_min, pupil_max), each an (x, y) pair of
    floats, cached on the system per wavelength
    (optika/systems/_sequential.py:755-799)."""
    cache = system.__dict__.setdefault("_stop_extents", {})
    key = float(wavelength)
    if key not in cache:
        st = rayfunction_stops(system, key)
        f, q = st["field"], st["pupil"]
        cache[key] = ((float(f[0].min()), float(f[1].min())),
                      (float(f[0].max()), float(f[1].max())),
                      (float(q[0].min()), float(q[1].min())),
                      (float(q[0].max()), float(q[1].max())))
    return cache[key]


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
    ext = [extents(system, w) for w in ws]

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


__all__ = ["anchor_surface", "stops_only", "rayfunction_stops", "extents", "denormalize"]
