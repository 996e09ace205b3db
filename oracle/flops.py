"""Algorithmic operation count of the reference's trace, per ray.

MEASUREMENT INFRASTRUCTURE (like the rest of ``oracle/``): it runs the
oracle's own per-surface code (``oracle/trace.py``, which restates
optika/surfaces.py:123-198 and the sag, Snell, multilayer and aperture code
it calls) on arrays of a counting ``ndarray`` subclass, so the count is the
reference algorithm's arithmetic as written there: both frame changes per
surface (optika/surfaces.py:141-142, 196), both roots of each closed-form
intercept (the vectorised formulation evaluates both), the transfer-matrix
arithmetic of the coatings.  It is not the device code's instruction count
(the device composes frame changes, keeps float-float compensation terms and
skips the unused root).

Only non-trivial real operations count: a product with a factor of 0, 1 or
-1 and a sum with a zero term are free.  The reference's vectorised
formulation multiplies by identity matrices (a bare substrate's
zero-thickness propagation matrix, the empty stack's starting product) and
by rotations whose entries are 0 and 1; those cost nothing here.  Complex
operations are split into their real operations, each tested the same way.

Categories (per ray):

* ``flops``: real additions, subtractions and multiplications;
* ``div``: real divisions (a complex division is |b|^2, the product with
  conj(b) and two divisions);
* ``special``: square roots, exponentials, logarithms, sines, cosines,
  arctangents, powers other than squares (complex ones count 2);
* ``cmp``: comparisons, signs, minima and maxima, finiteness tests.

The bench's FP32 roofline divides ``flops`` per ray by the kernel's time;
divisions and special functions are reported beside it, not added to it.
"""

from __future__ import annotations

import collections

import numpy as np

_SPECIAL = {np.sqrt, np.exp, np.log, np.sin, np.cos, np.tan, np.arctan2, np.arctan, np.arcsin,
            np.arccos, np.hypot, np.cbrt, np.expm1, np.log1p, np.sinh, np.cosh, np.tanh}
_CMP = {np.less, np.less_equal, np.greater, np.greater_equal, np.equal, np.not_equal,
        np.sign, np.copysign, np.maximum, np.minimum, np.fmax, np.fmin, np.isfinite,
        np.isnan, np.isinf, np.logical_and, np.logical_or, np.logical_not, np.floor,
        np.ceil, np.rint, np.signbit}
_FREE = {np.negative, np.positive, np.conjugate, np.bitwise_and, np.bitwise_or,
         np.bitwise_not, np.invert, np.bitwise_xor}


class Counter(collections.Counter):
    """Operation counts; ``per(n)`` divides by a number of rays."""

    def per(self, n: int) -> dict:
        return {k: v / n for k, v in sorted(self.items())}


COUNTS = Counter()


def _plain(x):
    return x.view(np.ndarray) if isinstance(x, Counted) else x


def _parts(x):
    x = np.asarray(x)
    if np.iscomplexobj(x):
        return x.real, x.imag
    return x, np.zeros_like(x, dtype=np.float64)


def _nz(x):
    return np.asarray(x) != 0


def _factor(x):  # a factor that makes a product non-trivial
    x = np.asarray(x)
    return (x != 0) & (x != 1) & (x != -1)


def _n_add(a, b) -> int:
    """Non-trivial real sums a + b (elementwise, broadcast)."""
    return int(np.count_nonzero(_nz(a) & _nz(b)))


def _n_mul(a, b) -> int:
    return int(np.count_nonzero(_factor(a) & _factor(b)))


def _cmul_counts(a, b):
    """Real products and sums of a complex product, and its parts."""
    ar, ai = _parts(a)
    br, bi = _parts(b)
    muls = _n_mul(ar, br) + _n_mul(ai, bi) + _n_mul(ar, bi) + _n_mul(ai, br)
    adds = _n_add(ar * br, ai * bi) + _n_add(ar * bi, ai * br)
    return muls + adds


def _count_ufunc(uf, inputs) -> None:
    cplx = any(np.iscomplexobj(x) for x in inputs)
    if uf in (np.add, np.subtract):
        a, b = inputs
        if cplx:
            ar, ai = _parts(a)
            br, bi = _parts(b)
            COUNTS["flops"] += _n_add(ar, br) + _n_add(ai, bi)
        else:
            COUNTS["flops"] += _n_add(a, b)
    elif uf is np.multiply:
        a, b = inputs
        COUNTS["flops"] += _cmul_counts(a, b) if cplx else _n_mul(a, b)
    elif uf is np.square:
        a, = inputs
        COUNTS["flops"] += _cmul_counts(a, a) if cplx else _n_mul(a, a)
    elif uf is np.power and len(inputs) == 2 and np.all(np.asarray(inputs[1]) == 2):
        a = inputs[0]
        COUNTS["flops"] += _cmul_counts(a, a) if cplx else _n_mul(a, a)
    elif uf in (np.divide, np.true_divide, np.reciprocal):
        a, b = (1.0, inputs[0]) if uf is np.reciprocal else inputs
        if cplx:
            ar, ai = _parts(a)
            br, bi = _parts(b)
            real_b = ~_nz(bi)
            # real denominator: one division per non-zero part of a
            COUNTS["div"] += int(np.count_nonzero(real_b & _factor(br) & _nz(ar)))
            COUNTS["div"] += int(np.count_nonzero(real_b & _factor(br) & _nz(ai)))
            # complex denominator: |b|^2 (3), a conj(b) (6), two divisions
            full = np.broadcast_to(~real_b, np.broadcast(ar, br).shape)
            COUNTS["flops"] += 9 * int(np.count_nonzero(full))
            COUNTS["div"] += 2 * int(np.count_nonzero(full))
        else:
            COUNTS["div"] += int(np.count_nonzero(
                np.broadcast_to(_nz(a) & (np.asarray(b) != 1) & (np.asarray(b) != -1),
                                np.broadcast(a, b).shape)))
    elif uf is np.absolute:
        a, = inputs
        if cplx:
            ar, ai = _parts(a)
            COUNTS["flops"] += _n_mul(ar, ar) + _n_mul(ai, ai) + _n_add(ar, ai)
            COUNTS["special"] += int(np.count_nonzero(_nz(ai)))
    elif uf in _SPECIAL or uf is np.power:
        size = np.broadcast(*inputs).size if len(inputs) > 1 else np.size(inputs[0])
        COUNTS["special"] += size * (2 if cplx else 1)
    elif uf in _CMP:
        size = np.broadcast(*inputs).size if len(inputs) > 1 else np.size(inputs[0])
        COUNTS["cmp"] += size
    elif uf in _FREE:
        pass
    else:
        COUNTS["other:" + uf.__name__] += np.size(inputs[0])


def _count_matmul(a, b) -> None:
    """C = A @ B over the last two axes: each term A_ik B_kj a product,
    each running sum a sum, both tested for triviality."""
    a = np.asarray(a)
    b = np.asarray(b)
    ni, nk = a.shape[-2:]
    nj = b.shape[-1]
    for i in range(ni):
        for j in range(nj):
            terms = []
            for k in range(nk):
                x, y = a[..., i, k], b[..., k, j]
                COUNTS["flops"] += _cmul_counts(x, y)
                terms.append(x * y)
            acc = terms[0]
            for t in terms[1:]:
                ar, ai = _parts(acc)
                tr, ti = _parts(t)
                COUNTS["flops"] += _n_add(ar, tr) + _n_add(ai, ti)
                acc = acc + t


class Counted(np.ndarray):
    """An ndarray whose elementwise arithmetic is tallied in ``COUNTS``."""

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        plain = [_plain(x) for x in inputs]
        if "out" in kwargs:
            kwargs["out"] = tuple(_plain(o) for o in kwargs["out"])
        res = getattr(ufunc, method)(*plain, **kwargs)
        if method == "__call__":
            if ufunc is np.matmul:
                _count_matmul(*plain)
            else:
                _count_ufunc(ufunc, plain)
        elif method == "reduce" and ufunc is np.add:
            COUNTS["flops"] += max(np.size(plain[0]) - 1, 0)
        return _wrap(res)

    def __array_function__(self, func, types, args, kwargs):
        a = [_plain_tree(x) for x in args]
        k = {key: _plain_tree(v) for key, v in kwargs.items()}
        res = func(*a, **k)
        if func is np.einsum:
            # "ij,j...->i...": the matrix's rows on a vector per element
            mat = np.asarray(a[1])
            vec = np.asarray(a[2])
            for i in range(mat.shape[0]):
                terms = [mat[i, j] * vec[j] for j in range(mat.shape[1])]
                COUNTS["flops"] += sum(_n_mul(mat[i, j], vec[j]) for j in range(mat.shape[1]))
                acc = terms[0]
                for t in terms[1:]:
                    COUNTS["flops"] += _n_add(acc, t)
                    acc = acc + t
        elif func is np.linalg.matrix_power:
            # binary powering of 2 x 2 complex matrices: squarings plus the
            # products of the set bits, 4 x (4 x 2 + 2 x 2 + 2) real
            # operations each (complex entries, none trivial in general)
            e = int(a[1])
            mults = max(e.bit_length() - 1, 0) + max(bin(e).count("1") - 1, 0)
            mats = np.size(a[0]) // 4
            COUNTS["flops"] += 56 * mults * mats
        elif func is np.interp:
            # (x - x0) / (x1 - x0) (y1 - y0) + y0 per element
            COUNTS["flops"] += 4 * np.size(res)
            COUNTS["div"] += np.size(res)
        return _wrap(res)


def _plain_tree(x):
    if isinstance(x, Counted):
        return x.view(np.ndarray)
    if isinstance(x, (list, tuple)):
        return type(x)(_plain_tree(v) for v in x)
    return x


def _wrap(res):
    if isinstance(res, tuple):
        return tuple(_wrap(r) for r in res)
    if isinstance(res, np.ndarray) and not isinstance(res, Counted):
        return res.view(Counted)
    return res


def count_rayfunction(system, grid: dict) -> dict:
    """Per-ray operation counts of ``oracle.trace.rayfunction`` (the literal
    reference arithmetic) on ``grid`` (wavelength, field_x, field_y,
    pupil_x, pupil_y).  The input rays (direction cosines from the field
    angles, optika/_util.py:69-73) and the sensor frame change are
    included; the histogram is not."""
    from oracle import trace as O

    n = len(grid["wavelength"])
    COUNTS.clear()
    g = {k: np.asarray(v, dtype=np.float64).view(Counted) for k, v in grid.items()}
    # input rays: the object at infinity takes direction(field), position pupil
    if system.object_is_at_infinity:
        d = O.direction(g["field_x"], g["field_y"])
    else:
        d = O.direction(g["pupil_x"], g["pupil_y"])
    plain = {k: np.asarray(v).view(np.ndarray) for k, v in grid.items()}
    rays = O.input_rays(system, plain["wavelength"], plain["field_x"], plain["field_y"],
                        plain["pupil_x"], plain["pupil_y"])
    rays["dx"], rays["dy"], rays["dz"] = (np.asarray(c).view(Counted) for c in d)
    rays = {k: (v.view(Counted) if isinstance(v, np.ndarray) and v.dtype != bool else v)
            for k, v in rays.items()}
    for s in system.surfaces_all:
        rays = O.propagate_surface(s, rays)
    O.apply(O._inv(O._mat(system.sensor.transformation)), rays)
    out = COUNTS.per(n)
    COUNTS.clear()
    return out


def count_multilayer(layers, substrate, wavelength, cos_incidence, n=1.0) -> dict:
    """Per-sample operation counts of ``oracle.trace.multilayer_efficiency``
    (R and T for s and p; the reference's periodic block as its first
    period times the period matrix to the power num_periods - 1, by binary
    powering, optika/materials/_layers.py:611-645)."""
    from oracle import trace as O

    m = len(np.atleast_1d(wavelength))
    COUNTS.clear()
    O.multilayer_efficiency(np.asarray(wavelength, dtype=np.float64).view(Counted),
                            np.asarray(cos_incidence, dtype=np.float64).view(Counted), n,
                            layers, substrate)
    out = COUNTS.per(m)
    COUNTS.clear()
    return out
