"""Float64 restatement of optika's stop solver (test oracle).

TEST INFRASTRUCTURE: imported only by tests/.  Follows
optika/systems/_sequential.py:363-394 (``_ray_error``), 396-693
(``_calc_rayfunction_stops_only``), 695-754 (``_calc_rayfunction_stops``),
801-850 (``_denormalize_grid``) and 343-361 (``_anchor_surface``), with the
rays traced by this package's float64 oracle (oracle/trace.py).

``named_arrays`` is not vendored in the reference; what its calls do here:
* ``na.optimize.root_newton``: Newton's method x <- x - J^-1 f(x) on every
  ray of the grid, until max |f| over the components is below
  ``max_abs_error`` for every ray (at most ``max_iter`` steps);
* ``na.jacobian``: forward differences with the step ``dx`` of the
  reference;
* the stop grids broadcast as [first wire, last wire].
"""

from __future__ import annotations

import numpy as np

from . import trace as O


def anchor_surface(subsystem):
    """optika/systems/_sequential.py:343-361."""
    for surface in subsystem[1:]:
        mat = surface.material
        if mat is not None and getattr(mat, "is_mirror", False):
            return surface
        if surface.sag is not None and type(surface.sag).__name__ != "NoSag":
            return surface
        if surface.rulings is not None:
            return surface
    return subsystem[-1]


def _zfunc(variable, surface_first):
    if variable == "direction":
        return lambda x, y: np.sqrt(1 - (x * x + y * y))
    return lambda x, y: O.sag_value(surface_first.sag, x, y)


def stops_only(system, wavelength: float, samples_pupil: int = 21, samples_field: int = 21,
               max_iter: int = 100):
    """optika/systems/_sequential.py:396-693 for one wavelength: rays (in the
    system frame) from the first stop that strike every point of the last
    stop's boundary, as arrays [first wire, last wire]."""
    surfaces = system.surfaces_all
    ip = [i for i, s in enumerate(surfaces) if s.is_pupil_stop]
    jf = [i for i, s in enumerate(surfaces) if s.is_field_stop]
    if not ip:
        raise ValueError("pupil not defined")
    if not jf:
        raise ValueError("field stop not defined")
    out = None
    while ip and jf:
        first_i, last_i = min(ip[0], jf[0]), max(ip[0], jf[0])
        sub = surfaces[first_i:last_i + 1]
        s_first, s_last = sub[0], sub[-1]
        g_first = s_first.aperture.wire(samples_pupil)[:, :2]
        g_last = s_last.aperture.wire(samples_field)[:, :2]
        if s_first.is_pupil_stop:
            ip.pop(0)
        else:
            jf.pop(0)
        n1, n2 = len(g_first), len(g_last)
        shape = (n1, n2)
        gx = np.broadcast_to(g_first[:, 0:1], shape)
        gy = np.broadcast_to(g_first[:, 1:2], shape)
        if not s_first.aperture.dimensionless:
            pos = np.stack([gx, gy, O.sag_value(s_first.sag, gx, gy)])
            dirn = np.stack([np.zeros(shape), np.zeros(shape), np.ones(shape)])
            variable = "direction"
        else:
            dirn = np.stack([gx, gy, np.sqrt(1 - (gx * gx + gy * gy))])
            pos = np.zeros((3,) + shape)
            variable = "position"
        zf = _zfunc(variable, s_first)
        # the seed aims at the first surface with power (or the target itself)
        anchor = anchor_surface(sub)
        if anchor is s_last and not s_last.aperture.dimensionless:
            aim = np.stack([np.broadcast_to(g_last[None, :, 0], shape),
                            np.broadcast_to(g_last[None, :, 1], shape), np.zeros(shape)])
            aim[2] = O.sag_value(s_last.sag, aim[0], aim[1])
            aim = _apply_point(O._mat(s_last.transformation), aim)
        else:
            aim = _apply_point(O._mat(anchor.transformation),
                               np.zeros((3,) + shape))
        aim = _apply_point(O._inv(O._mat(s_first.transformation)), aim)
        if variable == "direction":
            d = aim - pos
            d = d / np.sqrt((d * d).sum(0))
            flip = np.sign(d[2])
            where = d[2] != 0
            dirn = np.stack([np.where(where, flip * d[0], 0), np.where(where, flip * d[1], 0),
                             np.where(where, flip * d[2], 1)])
        else:
            t = aim[2] / dirn[2]
            px, py = aim[0] - dirn[0] * t, aim[1] - dirn[1] * t
            pos = np.stack([px, py, O.sag_value(s_first.sag, px, py)])
        M = O._mat(s_first.transformation)
        pos = _apply_point(M, pos)
        dirn = np.einsum("ij,j...->i...", M[:3, :3], dirn)
        target = "direction" if s_last.aperture.dimensionless else "position"
        tx = np.broadcast_to(g_last[None, :, 0], shape)
        ty = np.broadcast_to(g_last[None, :, 1], shape)
        scale = max(np.ptp(g_last[:, 0]), np.ptp(g_last[:, 1]))
        tol = 1e-9 * max(scale, 1.0)
        dx = 1e-6 if variable == "direction" else 1e-6 * max(scale, 1.0)
        Tl = O._inv(O._mat(s_last.transformation))

        def f(x, y):
            p, d = pos.copy(), dirn.copy()
            v = d if variable == "direction" else p
            v[0], v[1], v[2] = x, y, zf(x, y)
            rays = O.make_rays(shape, px=p[0], py=p[1], pz=p[2], dx=d[0], dy=d[1], dz=d[2],
                               wavelength=wavelength)
            r = O.apply(Tl, O.propagate_rays(sub[1:], rays))
            k = "d" if target == "direction" else "p"
            return r[k + "x"] - tx, r[k + "y"] - ty

        v0 = dirn if variable == "direction" else pos
        x, y = v0[0].copy(), v0[1].copy()
        for _ in range(max_iter):
            fx, fy = f(x, y)
            if np.all(np.maximum(np.abs(fx), np.abs(fy)) < tol):
                break
            ax, ay = f(x + dx, y)
            bx, by = f(x, y + dx)
            j11, j21 = (ax - fx) / dx, (ay - fy) / dx
            j12, j22 = (bx - fx) / dx, (by - fy) / dx
            det = j11 * j22 - j12 * j21
            x = x - (j22 * fx - j12 * fy) / det
            y = y - (-j21 * fx + j11 * fy) / det
        else:
            raise ValueError("stop root-finding did not converge")
        v = dirn if variable == "direction" else pos
        v[0], v[1], v[2] = x, y, zf(x, y)
        out = dict(position=pos, direction=dirn, first_index=first_i, last_index=last_i,
                   first_is_pupil=s_first.is_pupil_stop)
    return out


def _apply_point(M, p):
    return np.einsum("ij,j...->i...", M[:3, :3], p) + M[:3, 3].reshape((3,) + (1,) * (p.ndim - 1))


def rayfunction_stops(system, wavelength: float, samples_pupil: int = 21,
                      samples_field: int = 21):
    """optika/systems/_sequential.py:695-754: the stop rays traced back to the
    object surface, directions pointing into the system, field and pupil
    grids (angles in radians or positions in mm)."""
    st = stops_only(system, wavelength, samples_pupil, samples_field)
    surfaces = system.surfaces_all
    ip = max(i for i, s in enumerate(surfaces) if s.is_pupil_stop)
    jf = max(i for i, s in enumerate(surfaces) if s.is_field_stop)
    index_stop = min(ip, jf)
    sub = surfaces[index_stop::-1]
    p, d = st["position"], st["direction"]
    shape = p.shape[1:]
    rays = O.make_rays(shape, px=p[0], py=p[1], pz=p[2], dx=d[0], dy=d[1], dz=d[2],
                       wavelength=wavelength)
    r = O.propagate_rays(sub, rays)
    obj = sub[-1]
    rl = O.apply(O._inv(O._mat(obj.transformation)), r)
    nx, ny, nz = O.sag_normal(obj.sag, rl["px"], rl["py"])
    flip = rl["dx"] * nx + rl["dy"] * ny + rl["dz"] * nz > 0
    for k in ("dx", "dy", "dz"):
        r[k] = np.where(flip, -r[k], r[k])
    if system.transformation is not None:
        r = O.apply(O._mat(system.transformation), r)
    ang_x = -np.arctan2(r["dx"], r["dz"])
    ang_y = -np.arcsin(r["dy"] / np.sqrt(r["dx"] ** 2 + r["dy"] ** 2 + r["dz"] ** 2))
    if system.object_is_at_infinity:
        field, pupil = (ang_x, ang_y), (r["px"], r["py"])
    else:
        field, pupil = (r["px"], r["py"]), (ang_x, ang_y)
    return dict(rays=r, field=field, pupil=pupil)


def extents(system, wavelength: float):
    """(field_min, field_max, pupil_min, pupil_max), each an (x, y) pair:
    optika/systems/_sequential.py:755-799."""
    st = rayfunction_stops(system, wavelength)
    f, p = st["field"], st["pupil"]
    return ((f[0].min(), f[1].min()), (f[0].max(), f[1].max()),
            (p[0].min(), p[1].min()), (p[0].max(), p[1].max()))


def denormalize(system, wavelength: float, field, pupil, normalized_field=True,
                normalized_pupil=True):
    """optika/systems/_sequential.py:801-850 for one wavelength."""
    fmin, fmax, pmin, pmax = extents(system, wavelength)
    fx, fy = field
    qx, qy = pupil
    if normalized_field:
        fx = (fmax[0] - fmin[0]) * (np.asarray(fx) + 1) / 2 + fmin[0]
        fy = (fmax[1] - fmin[1]) * (np.asarray(fy) + 1) / 2 + fmin[1]
    if normalized_pupil:
        qx = (pmax[0] - pmin[0]) * (np.asarray(qx) + 1) / 2 + pmin[0]
        qy = (pmax[1] - pmin[1]) * (np.asarray(qy) + 1) / 2 + pmin[1]
    return (fx, fy), (qx, qy)


__all__ = ["anchor_surface", "stops_only", "rayfunction_stops", "extents", "denormalize"]
