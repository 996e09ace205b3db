"""Least-squares polynomial fits of several variables, the role
``named_arrays.PolynomialFitFunctionArray.from_degree`` plays in the
reference's calibration models (optika/distortion/_distortion.py:315-344,
optika/radiometry/_vignetting.py:147-158).

The polynomial has every monomial of total degree <= ``degree`` in the
inputs minus ``center``; each output component is fitted independently by
linear least squares over the points selected by ``where`` (columns scaled
to unit norm for conditioning; rank-deficient designs, such as a single
wavelength, take the minimum-norm solution).  These fits are small host
computations on a few hundred calibration points.
"""

from __future__ import annotations

import itertools

import numpy as np


def exponents(num_inputs: int, degree: int) -> np.ndarray:
    """Exponent rows of the monomials, by increasing total degree."""
    rows = []
    for d in range(degree + 1):
        for combo in itertools.combinations_with_replacement(range(num_inputs), d):
            e = np.zeros(num_inputs, dtype=np.int64)
            for k in combo:
                e[k] += 1
            rows.append(e)
    return np.array(rows)


class PolynomialFit:
    """outputs ~ sum_k c_k prod_j (x_j - center_j)^e_kj."""

    def __init__(self, inputs, outputs, degree: int, center=None, where=True):
        x = np.stack([np.asarray(v, dtype=np.float64) for v in np.broadcast_arrays(*inputs)],
                     axis=-1).reshape(-1, len(inputs))
        ys = [np.broadcast_to(np.asarray(o, dtype=np.float64),
                              np.broadcast_shapes(*[np.shape(v) for v in inputs])).reshape(-1)
              for o in outputs]
        self.center = x.mean(axis=0) if center is None else np.asarray(center, dtype=np.float64)
        self.exponents = exponents(len(inputs), degree)
        m = np.broadcast_to(np.asarray(where, dtype=bool),
                            np.broadcast_shapes(*[np.shape(v) for v in inputs])).reshape(-1)
        A = self._design(x)[m]
        scale = np.linalg.norm(A, axis=0)
        scale[scale == 0] = 1.0
        Y = np.stack(ys, axis=-1)[m]
        coef, *_ = np.linalg.lstsq(A / scale, Y, rcond=None)
        self.coefficients = coef / scale[:, None]  # [num_terms, num_outputs]

    def _design(self, x: np.ndarray) -> np.ndarray:
        d = x - self.center
        return np.prod(d[:, None, :] ** self.exponents[None, :, :], axis=-1)

    def __call__(self, *inputs) -> list[np.ndarray]:
        shape = np.broadcast_shapes(*[np.shape(v) for v in inputs])
        x = np.stack([np.broadcast_to(np.asarray(v, dtype=np.float64), shape).reshape(-1)
                      for v in inputs], axis=-1)
        y = self._design(x) @ self.coefficients
        return [y[:, k].reshape(shape) for k in range(y.shape[1])]
