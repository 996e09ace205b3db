"""Float64 restatement of SequentialSystem.image up to the photon image
(test oracle).

TEST INFRASTRUCTURE: imported only by tests/.  Follows
optika/systems/_sequential.py:1088-1206 (``image``) and :1002-1086
(``_rayfunction_from_vertices``), optika/vectors/_vectors_object.py:42-132
(``cell_area``) and optika/sensors/_sensors.py:92-171 (``collect``), with
the rays traced by this package's float64 oracle (oracle/trace.py).

``named_arrays`` is not vendored in the reference; what its calls do here:
* ``volume_cell`` of a 1-D vertex array: the difference of neighbouring
  vertices; of a rectilinear 2-D grid: the product of those differences;
* ``solid_angle_cell``: the solid angle of the spherical quadrilateral of
  the cell's four corner directions, as two spherical triangles (here by
  l'Huilier's theorem from the great-circle side lengths, an independent
  form of the triangle's solid angle);
* ``cell_centers(axis)``: the mean of the two vertices along each axis;
  with ``random=True`` a uniformly drawn point of the cell, the draws here
  being the same Philox4x32-10 uniforms the device uses (oracle/batch.py:
  one generator call per ray, four uniforms from the top 24 bits of its
  words, the fifth from the low bytes of the first three), one draw per
  axis shared by every coordinate of the ray.
"""

from __future__ import annotations

import numpy as np

from . import stops as OS
from . import trace as O
from .batch import MASK, philox4x32_10, u01


def _direction(ax, ay):
    return np.stack(O.direction(ax, ay))


def _arc(a, b):
    """Great-circle distance of unit vectors."""
    return 2 * np.arcsin(np.clip(np.linalg.norm(a - b, axis=0) / 2, 0, 1))


def _triangle(a, b, c):
    """Spherical excess by l'Huilier's theorem."""
    x, y, z = _arc(b, c), _arc(c, a), _arc(a, b)
    s = (x + y + z) / 2
    t = np.tan(s / 2) * np.tan((s - x) / 2) * np.tan((s - y) / 2) * np.tan((s - z) / 2)
    return 4 * np.arctan(np.sqrt(np.clip(t, 0, None)))


def solid_angle_cells(ax, ay):
    X, Y = np.meshgrid(np.asarray(ax, dtype=np.float64), np.asarray(ay, dtype=np.float64),
                       indexing="ij")
    d = _direction(X, Y)
    d00, d10, d11, d01 = d[:, :-1, :-1], d[:, 1:, :-1], d[:, 1:, 1:], d[:, :-1, 1:]
    return _triangle(d00, d10, d11) + _triangle(d00, d11, d01)


def _area(x, y, angular):
    if angular:
        return solid_angle_cells(x, y)
    return np.abs(np.diff(x)[:, None] * np.diff(y)[None, :])


def cell_tables(system, wavelength, field_x, field_y, radiance, pupil_x=(-1.0, 1.0),
                pupil_y=(-1.0, 1.0), normalized_field=True, normalized_pupil=True):
    """(w, fx, fy, px, py, weight, weight_pupil): vertices at every wavelength
    vertex and the per-cell weights (radiance x wavelength width x field
    area; pupil area), areas averaged over each cell's wavelength vertices."""
    w = np.asarray(wavelength, dtype=np.float64)
    nw = len(w) - 1

    def per(v, normalized, field):
        v = np.asarray(v, dtype=np.float64)
        out = []
        for k in range(nw + 1):
            if normalized:
                f, p = OS.denormalize(system, w[k], (v, v), (v, v), True, True)
                out.append(f[0] if field == "x" else f[1] if field == "y" else
                           p[0] if field == "px" else p[1])
            else:
                out.append(v)
        return np.stack(out)

    fx = per(field_x, normalized_field, "x")
    fy = per(field_y, normalized_field, "y")
    px = per(pupil_x, normalized_pupil, "px")
    py = per(pupil_y, normalized_pupil, "py")
    inf = system.object_is_at_infinity
    af = np.stack([_area(fx[k], fy[k], inf) for k in range(nw + 1)])
    ap = np.stack([_area(px[k], py[k], not inf) for k in range(nw + 1)])
    af = 0.5 * (af[:-1] + af[1:])
    ap = 0.5 * (ap[:-1] + ap[1:])
    rad = np.broadcast_to(np.asarray(radiance, dtype=np.float64), af.shape)
    return w, fx, fy, px, py, rad * np.diff(w)[:, None, None] * af, ap


def cell_inputs(tables, random=True, seed=0, first=0, count=None):
    """Input grid of cells [first, first + count) (all by default; ray order
    wavelength, field x, field y, pupil x, pupil y, the last fastest)."""
    w, fx, fy, px, py, weight, wp = tables
    nw, nfx, nfy = weight.shape
    npx, npy = wp.shape[1:]
    total = nw * nfx * nfy * npx * npy
    n = total - first if count is None else count
    i = np.arange(first, first + n, dtype=np.uint64)
    q = i.astype(np.int64)
    ipy = q % npy
    q //= npy
    ipx = q % npx
    q //= npx
    ify = q % nfy
    q //= nfy
    ifx = q % nfx
    iw = q // nfx
    if random:
        k0, k1 = seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF
        a = philox4x32_10(i & MASK, i >> np.uint64(32), 0x1CE115, 0, k0, k1)
        uw, ufx, ufy, upx = (u01(v).astype(np.float64) for v in a)
        ff = np.uint64(0xFF)
        low = ((a[0] & ff) << np.uint64(24)) | ((a[1] & ff) << np.uint64(16)) | (
            (a[2] & ff) << np.uint64(8))
        upy = u01(low).astype(np.float64)
    else:
        uw = ufx = ufy = upx = upy = np.full(n, 0.5)

    def lerp(t, k, u):
        lo = t[iw, k] + (t[iw, k + 1] - t[iw, k]) * u
        hi = t[iw + 1, k] + (t[iw + 1, k + 1] - t[iw + 1, k]) * u
        return lo + (hi - lo) * uw

    return dict(
        wavelength=w[iw] + (w[iw + 1] - w[iw]) * uw,
        field_x=lerp(fx, ifx, ufx), field_y=lerp(fy, ify, ufy),
        pupil_x=lerp(px, ipx, upx), pupil_y=lerp(py, ipy, upy),
        intensity=weight[iw, ifx, ify] * wp[iw, ipx, ipy],
    )


def photon_image(system, inputs, wavelength_bins):
    """(image, direction) of the traced cell rays, as ``collect`` returns
    them (oracle/trace.py:collect_reference)."""
    r = O.rayfunction(system, inputs["wavelength"], inputs["field_x"], inputs["field_y"],
                      inputs["pupil_x"], inputs["pupil_y"], intensity=inputs["intensity"])
    return O.collect_reference(system.sensor, r, wavelength_bins)


__all__ = ["solid_angle_cells", "cell_tables", "cell_inputs", "photon_image"]
