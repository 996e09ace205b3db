"""Float64 NumPy restatement of optika's sequential raytrace (test oracle).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline.  Every function cites the reference code it
follows (paths within the optika project).  Rays are dicts of float64
arrays: px py pz dx dy dz wavelength intensity attenuation n (index of
refraction) unvignetted opl.  Units: mm, nm, rad, 1/mm.

The description objects (surfaces, sags, ...) are the plain dataclasses of
optika_gb300; this module reads their fields and does all arithmetic itself
(its own 4x4 transform algebra, its own formulas).
"""

from __future__ import annotations

import math

import numpy as np

# ---------------------------------------------------------------- transforms


def _mat(t) -> np.ndarray:
    """4x4 float64 matrix of a transformation description (x' = R x + t),
    TransformationList applied in list order (see optika_gb300.transforms
    for the convention and its derivation from the reference's Newtonian
    telescope docstring, optika/systems/_sequential.py:1850-1912)."""
    if t is None:
        return np.eye(4)
    name = type(t).__name__
    m = np.eye(4)
    if name in ("Translation",):
        m[:3, 3] = [t.x, t.y, t.z]
    elif name in ("RotationX", "RotationY", "RotationZ"):
        c, s = math.cos(t.angle), math.sin(t.angle)
        i, j = {"RotationX": (1, 2), "RotationY": (2, 0), "RotationZ": (0, 1)}[name]
        # rotation in the (i, j) plane: e_i -> c e_i + s e_j
        m[i, i], m[i, j], m[j, i], m[j, j] = c, -s, s, c
    elif name == "TransformationList":
        for sub in t.transformations:
            m = _mat(sub) @ m
    elif name == "AffineTransformation":
        m[:3, :3] = np.asarray(t.matrix_, dtype=np.float64)
        m[:3, 3] = np.asarray(t.vector, dtype=np.float64)
    elif name == "Identity":
        pass
    else:
        raise NotImplementedError(name)
    return m


def _inv(m: np.ndarray) -> np.ndarray:
    out = np.eye(4)
    out[:3, :3] = m[:3, :3].T
    out[:3, 3] = -m[:3, :3].T @ m[:3, 3]
    return out


def apply(m: np.ndarray, rays: dict) -> dict:
    """Transform position (affine) and direction (linear) of rays
    (optika/rays/_ray_vectors.py:105-166)."""
    r = dict(rays)
    R, t = m[:3, :3], m[:3, 3]
    p = np.stack([rays["px"], rays["py"], rays["pz"]])
    d = np.stack([rays["dx"], rays["dy"], rays["dz"]])
    p2 = np.einsum("ij,j...->i...", R, p) + t.reshape((3,) + (1,) * (p.ndim - 1))
    d2 = np.einsum("ij,j...->i...", R, d)
    r["px"], r["py"], r["pz"] = p2
    r["dx"], r["dy"], r["dz"] = d2
    return r


# ---------------------------------------------------------------- sags


def _sag_kind(sag) -> str:
    return type(sag).__name__


def sag_value(sag, x, y):
    """z(x, y): _spherical.py:100-123, _conic.py:31-48, _toroidal.py:38-57."""
    k = _sag_kind(sag)
    if k == "NoSag":
        return np.zeros_like(x)
    if k == "SphericalSag":
        c = 1 / sag.radius
        r2 = x * x + y * y
        return c * r2 / (1 + np.sqrt(1 - c * c * r2))
    if k in ("ConicSag", "ParabolicSag"):
        c = 1 / sag.radius
        r2 = x * x + y * y
        return c * r2 / (1 + np.sqrt(1 - (1 + sag.conic) * c * c * r2))
    if k == "ToroidalSag":
        c = 1 / sag.radius
        r = sag.radius_of_rotation
        zy = c * y * y / (1 + np.sqrt(1 - c * c * y * y))
        return r - np.sqrt(np.square(r - zy) - x * x)
    if k == "CylindricalSag":  # _cylindrical.py:75-91
        c = 1 / sag.radius
        r2 = x * x
        return c * r2 / (1 + np.sqrt(1 - c * c * r2)) + 0 * y
    raise NotImplementedError(k)


def sag_normal(sag, x, y):
    """Unit normal, z < 0: _flat.py:41-45, _spherical.py:125-146,
    _conic.py:50-75, _parabolic.py:40-63, _toroidal.py:59-88."""
    k = _sag_kind(sag)
    if k == "NoSag":
        z = np.zeros_like(x)
        return z, z.copy(), -np.ones_like(x)
    if k == "SphericalSag":
        c = 1 / sag.radius
        nx, ny = c * x, c * y
        return nx, ny, -np.sqrt(1 - nx * nx - ny * ny)
    if k == "CylindricalSag":  # _cylindrical.py:93-113
        nx = x / sag.radius
        return nx, 0 * y, -np.sqrt(1 - nx**2)
    if k == "ParabolicSag":
        r = sag.radius
        s = np.sqrt((x / r) ** 2 + (y / r) ** 2 + 1)
        return x / s / r, y / s / r, -r * np.ones_like(x) / s / r
    if k == "ConicSag":
        c = 1 / sag.radius
        g = np.sqrt(1 - (1 + sag.conic) * c * c * (x * x + y * y))
        gx, gy = c * x / g, c * y / g
    elif k == "ToroidalSag":
        c = 1 / sag.radius
        r = sag.radius_of_rotation
        g = np.sqrt(1 - c * c * y * y)
        zy = c * y * y / (1 + g)
        f = np.sqrt(np.square(r - zy) - x * x)
        gx = x / f
        gy = (r - zy) * (c * y / g) / f
    else:
        raise NotImplementedError(k)
    L = np.sqrt(gx * gx + gy * gy + 1)
    return gx / L, gy / L, -1 / L


def _polish_root(sag, o, u, t, iters=3, reach=1e-3):
    """Float64 Newton steps on f(t) = z(t) - sag(x(t), y(t)) from the
    reference formula's root ``t``: the same root (the same sheet and
    branch), free of the cancellation of that formula.  Only points within
    ``reach`` mm of the sag are moved; others keep ``t``."""
    ox, oy, oz = o
    ux, uy, uz = u
    with np.errstate(all="ignore"):
        x, y, z = ox + ux * t, oy + uy * t, oz + uz * t
        near = np.isfinite(t) & (np.abs(z - sag_value(sag, x, y)) < reach)
        for _ in range(iters):
            x, y, z = ox + ux * t, oy + uy * t, oz + uz * t
            nx, ny, nz = sag_normal(sag, x, y)
            gx, gy = -nx / nz, -ny / nz
            dt = (z - sag_value(sag, x, y)) / (uz - gx * ux - gy * uy)
            t = np.where(near & np.isfinite(dt), t - dt, t)
    return t


def sag_intercept(sag, o, u, newton_tol=1e-12, newton_max=60, exact=False):
    """Line parameter t of the intercept of rays o + t u.

    ``exact=False`` evaluates the reference's closed forms literally, with
    their float64 rounding: the conic's ``(-B +- sqrt(B^2 - 4AC)) / 2A``
    loses up to ~1e-4 mm along a near-axial ray (A ~ 1e-12 / mm), which is
    the reference's own error.  ``exact=True`` keeps the root those forms
    choose and polishes it with float64 Newton steps on the sag equation
    (:func:`_polish_root`): the float64 solution of the same problem.

    flat      _flat.py:47-64
    sphere    _spherical.py:148-191
    conic     _conic.py:77-170 (vertex-sheet root nearest the origin)
    parabola  _parabolic.py:65-158
    toroid    _abc.py:76-107 (iterative root; here Newton from the vertex
              plane intercept, iterated to convergence in float64)
    cylinder  _cylindrical.py:115-160
    """
    t = _sag_intercept_literal(sag, o, u, newton_tol, newton_max)
    if exact and _sag_kind(sag) in ("SphericalSag", "ConicSag", "ParabolicSag",
                                    "CylindricalSag"):
        t = _polish_root(sag, o, u, t)
    return t


def _sag_intercept_literal(sag, o, u, newton_tol, newton_max):
    ox, oy, oz = o
    ux, uy, uz = u
    k = _sag_kind(sag)
    with np.errstate(all="ignore"):
        if k == "NoSag":
            return -oz / uz
        if k == "SphericalSag":
            r = sag.radius
            px, py, pz = ox, oy, oz - r
            b = ux * px + uy * py + uz * pz
            return -b - np.sign(r * uz) * np.sqrt(b * b - (px * px + py * py + pz * pz - r * r))
        if k == "CylindricalSag":
            # line o + d u against the cylinder of radius r about the y axis
            # through (0, 0, r): b = (0, 0, r) - o, a = y
            r = sag.radius
            bx, bz = -ox, r - oz
            cx, cz = -uz, ux  # u x a
            ncs = cx * cx + cz * cz
            negative_b = cx * (-bz) + cz * bx  # (u x a) . (b x a)
            disc = ncs * r * r - np.square(bx * cx + bz * cz)
            sgn = np.sign(r * uz)
            return np.where(disc > 0, (negative_b - sgn * np.sqrt(disc)) / ncs, -oz / uz)
        if k == "ParabolicSag":
            f = sag.focal_length
            a = ux * ux + uy * uy
            D = (
                -((oy * ux) ** 2) - (ox * uy) ** 2 + 2 * oy * uy * (ox * ux - 2 * f * uz)
                + 4 * f * (oz * a - ox * ux * uz + f * uz * uz)
            )
            quad = (-ox * ux - oy * uy + 2 * f * uz - np.sign(f * uz) * np.sqrt(D)) / a
            lin = (ox * ox + oy * oy - 4 * f * oz) / (4 * f * uz)
            return np.where(a > 1e-10, quad, lin)
        if k == "ConicSag":
            c = 1 / sag.radius
            kp1 = 1 + sag.conic
            A = c * (ux * ux + uy * uy + kp1 * uz * uz)
            B = 2 * (c * (ox * ux + oy * uy + kp1 * oz * uz) - uz)
            C = c * (ox * ox + oy * oy + kp1 * oz * oz) - 2 * oz
            disc = B * B - 4 * A * C
            real = disc >= 0
            sq = np.sqrt(np.where(real, disc, 0))
            deg = np.abs(A) < 1e-12
            den = np.where(deg, 1.0, 2 * A)
            tlin = -C / B

            def root(sign):
                t = np.where(deg, tlin, (-B + sign * sq) / den)
                x, y, z = ox + ux * t, oy + uy * t, oz + uz * t
                sheet = (z * (c * (x * x + y * y) - z)) >= 0
                return np.where(real & sheet, t, np.inf)

            ta, tb = root(-1), root(+1)
            return np.where(np.abs(ta) <= np.abs(tb), ta, tb)
        if k == "ToroidalSag":
            t = -oz / uz
            for _ in range(newton_max):
                x, y, z = ox + ux * t, oy + uy * t, oz + uz * t
                c = 1 / sag.radius
                r = sag.radius_of_rotation
                g = np.sqrt(1 - c * c * y * y)
                zy = c * y * y / (1 + g)
                f = np.sqrt(np.square(r - zy) - x * x)
                zs = r - f
                gx = x / f
                gy = (r - zy) * (c * y / g) / f
                dt = (z - zs) / (uz - gx * ux - gy * uy)
                t = t - dt
                if np.all(~np.isfinite(dt) | (np.abs(dt) <= newton_tol * (1 + np.abs(t)))):
                    break
            return t
    raise NotImplementedError(k)


# ---------------------------------------------------------------- Snell


def snells_law(ax, ay, az, n1, n2, is_mirror, ux, uy, uz):
    """optika/materials/_snells_law.py:341-366."""
    a2 = ax * ax + ay * ay + az * az
    r = n1 / n2
    au = ax * ux + ay * uy + az * uz
    sgn = -np.copysign(1.0, au)
    m = 2 * float(is_mirror) - 1
    with np.errstate(invalid="ignore"):
        d = -au + sgn * m * np.sqrt(1 / (r * r) + au * au - a2)
    return r * (ax + d * ux), r * (ay + d * uy), r * (az + d * uz)


def snells_law_scalar(cos_incidence, n1, n2):
    """optika/materials/_snells_law.py:13-38 (numpy.emath square roots)."""
    sin_i = np.emath.sqrt(1 - np.square(cos_incidence))
    sin_t = n1 * sin_i / n2
    return np.emath.sqrt(1 - np.square(sin_t))


# ---------------------------------------------------------------- rulings


def ruling_kappa(spacing, x, y, z, nx, ny, nz):
    """optika/rulings/_spacing.py:69-74, 109-128, 295-328."""
    name = type(spacing).__name__
    if name in ("ConstantRulingSpacing", "_ConstantSpacing"):
        g = np.asarray(spacing.normal, dtype=np.float64)
        d = spacing.constant * np.ones_like(x)
        return d * g[0], d * g[1], d * g[2]
    if name == "Polynomial1dRulingSpacing":
        g = np.asarray(spacing.normal, dtype=np.float64)
        m = _mat(spacing.transformation)
        p = np.stack([x, y, z])
        p = np.einsum("ij,j...->i...", m[:3, :3], p) + m[:3, 3].reshape((3,) + (1,) * (p.ndim - 1))
        xs = p[0] * g[0] + p[1] * g[1] + p[2] * g[2]
        d = 0.0 * xs
        for power, coef in spacing.coefficients.items():
            d = d + coef * xs**power
        return d * g[0], d * g[1], d * g[2]
    if name == "HolographicRulingSpacing":
        d1 = 2 * bool(spacing.is_diverging_1) - 1
        d2 = 2 * bool(spacing.is_diverging_2) - 1
        x1 = np.asarray(spacing.x1, dtype=np.float64)
        x2 = np.asarray(spacing.x2, dtype=np.float64)
        r1 = np.stack([x - x1[0], y - x1[1], z - x1[2]])
        r2 = np.stack([x - x2[0], y - x2[1], z - x2[2]])
        r1 = d1 * r1 / np.sqrt((r1 * r1).sum(0))
        r2 = d2 * r2 / np.sqrt((r2 * r2).sum(0))
        dr = r1 - r2
        n = np.stack([nx, ny, nz])
        aq = np.cross(n, dr, axis=0)
        a = np.sqrt((aq * aq).sum(0))
        q = aq / a
        sp = spacing.wavelength * 1e-6 / a
        k = sp * np.cross(q, n, axis=0)
        return k[0], k[1], k[2]
    raise NotImplementedError(name)


class _ConstantSpacing:
    """A bare number as ruling spacing: constant, ruling normal +x
    (optika/rulings/_rulings.py:157-168)."""

    def __init__(self, constant):
        self.constant = float(constant)
        self.normal = (1.0, 0.0, 0.0)


def spacing_of(rulings):
    s = rulings.spacing
    if isinstance(s, (int, float, np.floating)):
        return _ConstantSpacing(s)
    return s


def incident_effective(rays, rulings, nx, ny, nz):
    """optika/rulings/_rulings.py:124-126 via :170-204."""
    spacing = spacing_of(rulings)
    kx, ky, kz = ruling_kappa(spacing, rays["px"], rays["py"], rays["pz"], nx, ny, nz)
    d = np.sqrt(kx * kx + ky * ky + kz * kz)
    gx, gy, gz = kx / d, ky / d, kz / d
    w = rays["wavelength"] * 1e-6
    an = rays["dx"] * nx + rays["dy"] * ny + rays["dz"] * nz
    f = np.sign(an) * rulings.diffraction_order * w / (rays["n"] * d)
    r = dict(rays)
    r["dx"] = rays["dx"] + f * gx
    r["dy"] = rays["dy"] + f * gy
    r["dz"] = rays["dz"] + f * gz
    return r


def ruling_efficiency(rulings, rays, nx, ny, nz):
    """Groove efficiency of the ruling models on the rays after
    incident_effective (optika/surfaces.py:182-184):
    Rulings :246-251 (1), MeasuredRulings :287-314 (np.interp on wavelength),
    SinusoidalRulings :404-457, SquareRulings :548-614,
    SawtoothRulings :705-758, TriangularRulings :849-911,
    RectangularRulings :1008-1073 of optika/rulings/_rulings.py.  As in the
    reference, the scalar direction . parallel_rulings is subtracted from
    every component of the direction before cos_theta = -direction . normal,
    and the Sinusoidal model returns J_m(2 gamma) itself."""
    import scipy.special

    name = type(rulings).__name__
    if name == "Rulings":
        return 1.0
    if name == "MeasuredRulings":
        m = rulings.efficiency_measured
        return np.interp(rays["wavelength"], np.asarray(m.inputs.wavelength, dtype=np.float64),
                         np.asarray(m.outputs, dtype=np.float64).reshape(-1))
    kx, ky, kz = ruling_kappa(spacing_of(rulings), rays["px"], rays["py"], rays["pz"],
                              nx, ny, nz)
    with np.errstate(all="ignore"):
        kl = np.sqrt(kx * kx + ky * ky + kz * kz)
        kx, ky, kz = kx / kl, ky / kl, kz / kl
        px, py, pz = ny * kz - nz * ky, nz * kx - nx * kz, nx * ky - ny * kx
        pl = np.sqrt(px * px + py * py + pz * pz)
        px, py, pz = px / pl, py / pl, pz / pl
        dx, dy, dz = rays["dx"], rays["dy"], rays["dz"]
        s = dx * px + dy * py + dz * pz
        dx, dy, dz = dx - s, dy - s, dz - s
        cos_theta = -(dx * nx + dy * ny + dz * nz)
        wavelength = rays["wavelength"]
        i = rulings.diffraction_order
        depth = rulings.depth * 1e6  # mm -> nm
        if name == "SinusoidalRulings":
            gamma = np.pi * depth / (wavelength * cos_theta)
            return scipy.special.jv(i, 2 * gamma)
        if name == "SquareRulings":
            gamma = np.pi * (depth / (np.pi / 4)) / (wavelength * cos_theta)
            result = np.where(i % 2 == 0, 0, np.square(2 * np.sin(np.pi * gamma / 2) / (i * np.pi)))
            return np.where(i == 0, np.square(np.cos(np.pi * gamma / 2)), result)
        if name == "SawtoothRulings":
            gamma = np.pi * (depth / (np.pi / 2)) / (wavelength * cos_theta)
            return np.square(np.sin(np.pi * gamma) / (np.pi * (gamma + i)))
        if name == "TriangularRulings":
            gamma = np.pi * (depth / (np.square(np.pi) / 8)) / (wavelength * cos_theta)
            a = gamma / (np.square(np.pi * gamma / 2) + np.square(i))
            return np.where(i % 2 == 0, np.square(a * np.sin(np.square(np.pi) * gamma / 4)),
                            np.square(a * np.cos(np.square(np.pi) * gamma / 4)))
        if name == "RectangularRulings":
            a = 2 * np.pi * rulings.ratio_duty
            amplitude = np.pi / (2 * np.sqrt(2 * (1 - np.cos(a))))
            gamma = np.pi * (depth / amplitude) / (wavelength * cos_theta)
            b = np.square(np.sin(np.pi * gamma / np.sqrt(2 * (1 - np.cos(a)))))
            return np.where(i == 0, 1 - ((2 * a / np.pi) - np.square(a / np.pi)) * b,
                            (2 / np.square(i * np.pi)) * (1 - np.cos(i * a)) * b)
    raise NotImplementedError(name)


# ---------------------------------------------------------------- apertures


def point_in_polygon(x, y, vx, vy):
    """Even-odd crossing test (the documented behaviour of
    named_arrays.geometry.point_in_polygon, used at
    optika/apertures/_apertures.py:752-758)."""
    inside = np.zeros(np.shape(x), dtype=bool)
    n = len(vx)
    j = n - 1
    with np.errstate(all="ignore"):
        for i in range(n):
            cond = ((vy[i] > y) != (vy[j] > y)) & (
                x < (vx[j] - vx[i]) * (y - vy[i]) / (vy[j] - vy[i]) + vx[i]
            )
            inside ^= cond
            j = i
    return inside


def aperture_mask(ap, x, y, z):
    """optika/apertures/_apertures.py: Circular :292-314, Sector :438-480,
    Elliptical :640-663, Polygonal :739-778, Rectangular :941-968."""
    name = type(ap).__name__
    if ap.transformation is not None:
        m = _inv(_mat(ap.transformation))
        p = np.stack([x, y, z])
        p = np.einsum("ij,j...->i...", m[:3, :3], p) + m[:3, 3].reshape((3,) + (1,) * (p.ndim - 1))
        x, y, z = p
    with np.errstate(invalid="ignore"):
        if name == "CircularAperture":
            mask = np.sqrt(x * x + y * y) <= ap.radius
        elif name == "RectangularAperture":
            hx, hy = ap.half_width_xy
            mask = (-hx <= x) & (x <= hx) & (-hy <= y) & (y <= hy)
        elif name == "EllipticalAperture":
            mask = np.square(x / ap.radius[0]) + np.square(y / ap.radius[1]) <= 1
        elif name == "CircularSectorAperture":
            mr = np.sqrt(x * x + y * y) <= ap.radius
            ang = np.arctan2(y, x)
            apos = np.mod(ang, 2 * np.pi)
            aneg = np.mod(ang, -2 * np.pi)
            ma = ((ap.angle_start < apos) & (apos < ap.angle_stop)) | (
                (ap.angle_start < aneg) & (aneg < ap.angle_stop)
            )
            mask = mr & ma
        elif hasattr(ap, "vertex_array"):
            v = ap.vertex_array()
            mask = point_in_polygon(x, y, v[:, 0], v[:, 1])
        else:
            raise NotImplementedError(name)
    mask = np.asarray(mask, dtype=bool)
    if ap.inverted:
        mask = ~mask
    if not ap.active:
        mask = np.ones_like(mask)
    return mask


# ---------------------------------------------------------------- multilayers


def layer_index(chemical, wavelength):
    """Complex index of a layer medium: vacuum, constant, or a table
    interpolated linearly with the ends held (optika/chemicals/_chemicals.py:
    101-144; numpy.interp semantics for na.interp)."""
    w = np.asanyarray(wavelength, dtype=np.float64)
    if chemical is None:
        return np.ones_like(w) + 0j
    if hasattr(chemical, "wavelength"):
        return np.interp(w, chemical.wavelength, chemical.n) + 1j * np.interp(
            w, chemical.wavelength, chemical.k
        )
    return np.full(w.shape, complex(chemical))


def interface_reflectivity(interface, wavelength, direction, n):
    """Factor of an interface profile on r_ij: the Fourier transform of the
    profile's derivative at s = Re(-2 k), k = -2 pi n direction / lambda
    (optika/materials/profiles.py:103-128; transforms :221-223 erf,
    :320-326 exponential, :424-431 linear, :532-541 sinusoidal)."""
    if interface is None:
        return 1.0
    w = interface.width
    k = -2 * np.pi * n * direction / wavelength
    sv = np.real(-2 * k)
    name = type(interface).__name__
    with np.errstate(all="ignore"):
        if name == "ErfInterfaceProfile":
            return np.exp(-np.square(sv * w) / 2)
        if name == "ExponentialInterfaceProfile":
            return 1 / (1 + np.square(sv * w) / 2)
        if name == "LinearInterfaceProfile":
            x = np.sqrt(3) * w * sv
            return np.sin(x) / x
        if name == "SinusoidalInterfaceProfile":
            a = np.pi / (np.square(np.pi) - 8)
            x = a * w * sv
            x1, x2 = x - np.pi / 2, x + np.pi / 2
            return np.pi * (np.sin(x1) / x1 + np.sin(x2) / x2) / 4
    raise NotImplementedError(name)


def _refraction(cos_i, cos_j, n_i, n_j, s, wavelength=None, interface=None):
    """optika/materials/matrices.py:127-161 for one polarisation."""
    ci = cos_i if s else np.conj(cos_i)
    cj = cos_j if s else np.conj(cos_j)
    qi = ci * (n_i if s else 1 / n_i)
    qj = cj * (n_j if s else 1 / n_j)
    a = qi + qj
    r = (qi - qj) / a
    t = 2 * qi / a
    if interface is not None:
        r = r * interface_reflectivity(interface, wavelength, ci, n_i)
    one = np.ones_like(r)
    return np.stack([np.stack([one, r], -1), np.stack([r, one], -1)], -2) / t[..., None, None]


def _propagation(wavelength, cos, thickness, n):
    """optika/materials/matrices.py:241-246."""
    beta = 2 * np.pi * thickness * n * cos / wavelength
    z = np.zeros_like(beta)
    return np.stack(
        [np.stack([np.exp(-1j * beta), z], -1), np.stack([z, np.exp(1j * beta)], -1)], -2
    )


def _layer_transfer(layer_chem, thickness, wavelength, cos, n, s, where, interface=None):
    """optika/materials/_layers.py:229-277."""
    n_int = layer_index(layer_chem, wavelength)
    cos_int = snells_law_scalar(cos, n, n_int)
    W = _refraction(cos, cos_int, n, n_int, s, wavelength, interface)
    eye = np.broadcast_to(np.eye(2, dtype=complex), W.shape)
    W = np.where(where[..., None, None], W, eye)
    with np.errstate(all="ignore"):
        U = _propagation(wavelength, cos_int, 0.0 if thickness is None else thickness, n_int)
        wprop = np.abs(U[..., 0, 0]) < 1e10
        where2 = where & wprop
        T = np.where(where2[..., None, None], W @ U, W)
    return n_int, cos_int, T, where2


def _flatten(layers):
    if layers is None:
        return []
    name = type(layers).__name__
    if name in ("Layer", "PeriodicLayerSequence"):
        return [layers]
    if name == "LayerSequence":
        return _flatten(list(layers.layers))
    out = []
    for x in layers:
        out += _flatten(x)
    return out


def _sequence_transfer(items, wavelength, cos, n, s, where):
    """optika/materials/_layers.py:473-499 and 611-645 (periodic: first
    period times the period matrix to the power num_periods - 1)."""
    M = np.broadcast_to(np.eye(2, dtype=complex), np.shape(cos) + (2, 2)).copy()
    for it in items:
        if type(it).__name__ == "PeriodicLayerSequence":
            inner = _flatten(it.layers)
            n, cos, start, where = _sequence_transfer(inner, wavelength, cos, n, s, where)
            n, cos, per, where = _sequence_transfer(inner, wavelength, cos, n, s, where)
            P = np.linalg.matrix_power(per, int(it.num_periods) - 1)
            M = M @ start @ P
        else:
            n, cos, T, where = _layer_transfer(it.chemical, it.thickness, wavelength, cos, n, s,
                                               where, getattr(it, "interface", None))
            M = M @ T
    return n, cos, M, where


def multilayer_efficiency(wavelength, direction=1.0, n=1.0, layers=None, substrate=None):
    """(R_s, R_p, T_s, T_p), optika/materials/_multilayers.py:33-237 and
    240-532, in complex128."""
    # (subclass-preserving conversions: oracle/flops.py counts this code's
    # arithmetic on a counting array type)
    wavelength, direction, n = np.broadcast_arrays(
        np.asanyarray(wavelength, dtype=np.float64),
        np.asanyarray(direction, dtype=np.complex128),
        np.asanyarray(n, dtype=np.complex128), subok=True,
    )
    items = _flatten(layers)
    sub_chem = None if substrate is None else substrate.chemical
    out = {}
    for s in (True, False):
        where = np.ones(wavelength.shape, dtype=bool)
        n1, c1, M, where = _sequence_transfer(items, wavelength, direction, n, s, where)
        n1, c1, Ms, where = _layer_transfer(sub_chem, 0.0, wavelength, c1, n1, s, where,
                                            getattr(substrate, "interface", None))
        M = M @ Ms
        r = M[..., 1, 0] / M[..., 0, 0]
        t = 1 / M[..., 0, 0]
        t = np.where(where, t, 0)
        n_sub = layer_index(sub_chem, wavelength)
        c_sub = snells_law_scalar(direction, n, n_sub)
        if s:
            q_amb, q_sub = direction * n, c_sub * n_sub
        else:
            q_amb, q_sub = np.conj(direction) / n, np.conj(c_sub) / n_sub
        out[s] = (np.abs(r) ** 2, np.abs(t) ** 2 * np.real(q_sub / q_amb))
    return out[True][0], out[False][0], out[True][1], out[False][1]


# ---------------------------------------------------------------- surfaces


def _material(mat):
    name = type(mat).__name__
    return name


def propagate_surface(surface, rays: dict, exact: bool = False) -> dict:
    """optika/surfaces.py:123-198 with rays in the parent frame (``exact``:
    see :func:`sag_intercept`)."""
    T = _mat(surface.transformation)
    r = apply(_inv(T), rays)
    sag = surface.sag
    o = (r["px"], r["py"], r["pz"])
    u = (r["dx"], r["dy"], r["dz"])
    t = sag_intercept(sag, o, u, exact=exact)
    with np.errstate(all="ignore"):
        px, py, pz = o[0] + u[0] * t, o[1] + u[1] * t, o[2] + u[2] * t
        disp = np.sqrt((px - o[0]) ** 2 + (py - o[1]) ** 2 + (pz - o[2]) ** 2)
        r["intensity"] = r["intensity"] * np.exp(-r["attenuation"] * disp)
        r["opl"] = r["opl"] + r["n"] * t
    r["px"], r["py"], r["pz"] = px, py, pz
    with np.errstate(all="ignore"):
        nx, ny, nz = sag_normal(sag, px, py)
    rulings = getattr(surface, "rulings", None)
    if rulings is not None:
        r = incident_effective(r, rulings, nx, ny, nz)
    mat = surface.material
    name = _material(mat)
    n1 = r["n"]
    eff = 1.0
    mirror = bool(getattr(mat, "is_mirror", False))
    if name in ("Vacuum", "IdealSensorMaterial"):
        n2 = np.ones_like(n1)
        att2 = np.zeros_like(n1)
    elif name == "Glass":
        w2 = (r["wavelength"] * 1e-3) ** 2  # um^2
        n2 = np.sqrt(1 + mat.b1 * w2 / (w2 - mat.c1) + mat.b2 * w2 / (w2 - mat.c2)
                     + mat.b3 * w2 / (w2 - mat.c3))
        att2 = np.zeros_like(n1)
    elif name in ("MultilayerMirror", "MultilayerFilm"):
        n2 = n1
        att2 = r["attenuation"]
        k = r["attenuation"] * (r["wavelength"] * 1e-6) / (4 * np.pi)
        cos0 = -(r["dx"] * nx + r["dy"] * ny + r["dz"] * nz)
        with np.errstate(all="ignore"):
            Rs, Rp, Ts, Tp = multilayer_efficiency(
                r["wavelength"], cos0, n1 + 1j * k, mat.layers,
                mat.substrate if name == "MultilayerMirror" else None,
            )
        eff = (Rs + Rp) / 2 if name == "MultilayerMirror" else (Ts + Tp) / 2
    elif name == "MeasuredMirror":  # _materials.py:279-306
        n2 = n1
        att2 = r["attenuation"]
        m = mat.efficiency_measured
        eff = np.interp(r["wavelength"], np.asarray(m.inputs.wavelength, dtype=np.float64),
                        np.asarray(m.outputs, dtype=np.float64).reshape(-1))
    elif mirror:
        n2 = n1
        att2 = r["attenuation"]
    else:
        raise NotImplementedError(name)
    if rulings is not None:
        eff = eff * ruling_efficiency(rulings, r, nx, ny, nz)
    rr = n1 / n2
    r["wavelength"] = r["wavelength"] / rr
    r["dx"], r["dy"], r["dz"] = snells_law(r["dx"], r["dy"], r["dz"], n1, n2, mirror, nx, ny, nz)
    r["intensity"] = r["intensity"] * eff
    r["attenuation"] = att2
    r["n"] = n2
    ap = surface.aperture
    if ap is not None:
        if ap.dimensionless:
            mask = aperture_mask(ap, r["dx"], r["dy"], r["dz"])
        else:
            mask = aperture_mask(ap, r["px"], r["py"], r["pz"])
        r["unvignetted"] = r["unvignetted"] & mask
    return apply(T, r)


def make_rays(shape, **kw) -> dict:
    z = np.zeros(shape)
    r = dict(px=z.copy(), py=z.copy(), pz=z.copy(), dx=z.copy(), dy=z.copy(), dz=np.ones(shape),
             wavelength=z.copy(), intensity=np.ones(shape), attenuation=z.copy(),
             n=np.ones(shape), unvignetted=np.ones(shape, dtype=bool), opl=z.copy())
    for k, v in kw.items():
        r[k] = np.broadcast_to(np.asarray(v, dtype=r[k].dtype), shape).copy()
    return r


def direction(ax, ay):
    """optika/_util.py:69-73."""
    return -np.cos(ay) * np.sin(ax), -np.sin(ay), np.cos(ay) * np.cos(ax)


def input_rays(system, wavelength, field_x, field_y, pupil_x, pupil_y, intensity=None) -> dict:
    """optika/systems/_sequential.py:791-828 and 906-909."""
    wavelength, field_x, field_y, pupil_x, pupil_y = np.broadcast_arrays(
        *[np.asarray(v, dtype=np.float64) for v in (wavelength, field_x, field_y, pupil_x, pupil_y)]
    )
    shape = wavelength.shape
    if system.object_is_at_infinity:
        px, py = pupil_x, pupil_y
        dx, dy, dz = direction(field_x, field_y)
    else:
        px, py = field_x, field_y
        dx, dy, dz = direction(pupil_x, pupil_y)
    rays = make_rays(shape, px=px, py=py, dx=dx, dy=dy, dz=dz, wavelength=wavelength)
    if intensity is not None:
        rays["intensity"] = np.broadcast_to(np.asarray(intensity, dtype=np.float64), shape).copy()
    if system.object is not None and system.object.transformation is not None:
        rays = apply(_mat(system.object.transformation), rays)
    if system.transformation is not None:
        rays = apply(_inv(_mat(system.transformation)), rays)
    return rays


def raytrace(system, wavelength, field_x, field_y, pupil_x, pupil_y, intensity=None,
             accumulate=True, exact=False):
    """optika/systems/_sequential.py:836-925: list of rays after every
    surface (accumulate) or the last rays, in the system frame."""
    rays = input_rays(system, wavelength, field_x, field_y, pupil_x, pupil_y, intensity)
    out = []
    for s in system.surfaces_all:
        rays = propagate_surface(s, rays, exact=exact)
        out.append(rays)
    return out if accumulate else rays


def rayfunction(system, wavelength, field_x, field_y, pupil_x, pupil_y, intensity=None,
                exact=False):
    """optika/systems/_sequential.py:927-988: last rays in the sensor frame."""
    rays = raytrace(system, wavelength, field_x, field_y, pupil_x, pupil_y, intensity,
                    accumulate=False, exact=exact)
    return apply(_inv(_mat(system.sensor.transformation)), rays)


def propagate_rays(surfaces, rays: dict, accumulate=False, exact=False):
    """optika/propagators.py:19-73."""
    out = []
    for s in surfaces:
        rays = propagate_surface(s, rays, exact=exact)
        out.append(rays)
    return out if accumulate else rays


# ---------------------------------------------------------------- sensor


def histogram_edges(sensor):
    """linspace(bound_lower.xy, bound_upper.xy, num + 1)
    (optika/sensors/_sensors.py:141-149)."""
    wx, wy = sensor.width_pixel_xy
    nx, ny = sensor.num_pixel
    ex = np.linspace(-wx * nx / 2, wx * nx / 2, nx + 1)
    ey = np.linspace(-wy * ny / 2, wy * ny / 2, ny + 1)
    return ex, ey


def bin_index(edges, v):
    """numpy.histogramdd bin of each value: [e_j, e_j+1), last edge
    inclusive, -1 outside (and for NaN)."""
    i = np.searchsorted(edges, v, side="right") - 1
    i = np.where(v == edges[-1], len(edges) - 2, i)
    ok = (v >= edges[0]) & (v <= edges[-1])
    return np.where(ok, i, -1)


def collect(sensor, rays: dict, wavelength_bins=None):
    """(counts, flux) images [num_w, num_x, num_y] of rays in the sensor frame
    weighted by intensity * unvignetted (optika/sensors/_sensors.py:92-161)."""
    ex, ey = histogram_edges(sensor)
    ix = bin_index(ex, rays["px"].ravel())
    iy = bin_index(ey, rays["py"].ravel())
    nx, ny = sensor.num_pixel
    if wavelength_bins is None:
        iw = np.zeros_like(ix)
        nw = 1
    else:
        w0, w1, nw = wavelength_bins
        ew = np.linspace(w0, w1, nw + 1)
        iw = bin_index(ew, rays["wavelength"].ravel())
    ok = rays["unvignetted"].ravel() & (ix >= 0) & (iy >= 0) & (iw >= 0)
    flat = (iw[ok] * nx + ix[ok]) * ny + iy[ok]
    counts = np.bincount(flat, minlength=nw * nx * ny).reshape(nw, nx, ny)
    flux = np.bincount(flat, weights=rays["intensity"].ravel()[ok], minlength=nw * nx * ny)
    return counts, flux.reshape(nw, nx, ny)


def collect_reference(sensor, rays: dict, wavelength_bins=None):
    """(image, direction) of optika/sensors/_sensors.py:92-169 for an ideal
    sensor material: the intensity image and the flux-weighted mean cosine of
    incidence, -direction . normal with the flat sensor's normal (0, 0, -1)
    (optika/sensors/materials/_materials.py:1603-1616), 1 where a pixel is
    empty."""
    _, image = collect(sensor, rays, wavelength_bins)
    r2 = dict(rays)
    r2["intensity"] = rays["intensity"] * rays["dz"]
    _, moment = collect(sensor, r2, wavelength_bins)
    with np.errstate(invalid="ignore", divide="ignore"):
        direction = np.where(image > 0, moment / image, 1.0)
    return image, direction
