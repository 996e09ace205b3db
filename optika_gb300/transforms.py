"""Rigid coordinate transformations (host side, float64).

Restates the subset of ``named_arrays.transformations`` used by optika's
trace (every ``transformation(...)`` / ``transformation.inverse(...)``, e.g.
optika/surfaces.py:141-142, 195-196): translations, rotations about the
Cartesian axes, explicit affine maps and lists of them.

Conventions (named_arrays is not vendored in the reference, so they are
fixed here and checked against the layout of the Newtonian telescope in the
docstring of optika/systems/_sequential.py:1850-1912, where the fold mirror
``TransformationList([RotationY(135 deg), Translation(z=50 mm)])`` must sit
at z = 50 mm and the sensor ``[RotationY(-90 deg), Translation(x=-50, z=50)]``
at x = -50 mm):

* a transformation maps local coordinates to its parent's: ``x' = R x + t``;
* ``TransformationList([A, B, ...])`` applies ``A`` first, then ``B``;
* rotations are right-handed, ``RotationY(a) @ (0, 0, 1) = (sin a, 0, cos a)``.

Angles are radians (multiply degrees by :data:`optika_gb300.deg`), lengths mm.
"""

from __future__ import annotations

import dataclasses
import math
from typing import Sequence

import numpy as np

__all__ = [
    "AbstractTransformation",
    "Identity",
    "Translation",
    "RotationX",
    "RotationY",
    "RotationZ",
    "AffineTransformation",
    "TransformationList",
    "Cartesian3dTranslation",
    "Cartesian3dRotationX",
    "Cartesian3dRotationY",
    "Cartesian3dRotationZ",
    "matrix_of",
]


class AbstractTransformation:
    """A rigid map ``x' = R x + t`` represented by a 4x4 float64 matrix."""

    def matrix(self) -> np.ndarray:
        raise NotImplementedError

    def inverse_matrix(self) -> np.ndarray:
        return rigid_inverse(self.matrix())

    @property
    def inverse(self) -> "AffineTransformation":
        m = self.inverse_matrix()
        return AffineTransformation(m[:3, :3], m[:3, 3])

    def __call__(self, points: np.ndarray) -> np.ndarray:
        """Apply to an array of points with trailing dimension 3."""
        m = self.matrix()
        p = np.asarray(points, dtype=np.float64)
        return p @ m[:3, :3].T + m[:3, 3]

    def __matmul__(self, other: "AbstractTransformation") -> "AffineTransformation":
        m = self.matrix() @ other.matrix()
        return AffineTransformation(m[:3, :3], m[:3, 3])


def rigid_inverse(m: np.ndarray) -> np.ndarray:
    r = m[:3, :3]
    t = m[:3, 3]
    out = np.eye(4)
    out[:3, :3] = r.T
    out[:3, 3] = -r.T @ t
    return out


@dataclasses.dataclass(eq=False)
class Identity(AbstractTransformation):
    def matrix(self) -> np.ndarray:
        return np.eye(4)


@dataclasses.dataclass(eq=False)
class Translation(AbstractTransformation):
    """``x' = x + (x, y, z)`` (mm)."""

    x: float = 0.0
    y: float = 0.0
    z: float = 0.0

    def matrix(self) -> np.ndarray:
        m = np.eye(4)
        m[:3, 3] = [float(self.x), float(self.y), float(self.z)]
        return m


@dataclasses.dataclass(eq=False)
class RotationX(AbstractTransformation):
    angle: float = 0.0

    def matrix(self) -> np.ndarray:
        c, s = math.cos(self.angle), math.sin(self.angle)
        m = np.eye(4)
        m[1, 1], m[1, 2], m[2, 1], m[2, 2] = c, -s, s, c
        return m


@dataclasses.dataclass(eq=False)
class RotationY(AbstractTransformation):
    angle: float = 0.0

    def matrix(self) -> np.ndarray:
        c, s = math.cos(self.angle), math.sin(self.angle)
        m = np.eye(4)
        m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, s, -s, c
        return m


@dataclasses.dataclass(eq=False)
class RotationZ(AbstractTransformation):
    angle: float = 0.0

    def matrix(self) -> np.ndarray:
        c, s = math.cos(self.angle), math.sin(self.angle)
        m = np.eye(4)
        m[0, 0], m[0, 1], m[1, 0], m[1, 1] = c, -s, s, c
        return m


@dataclasses.dataclass(eq=False)
class AffineTransformation(AbstractTransformation):
    """Explicit ``x' = matrix @ x + vector`` with an orthonormal ``matrix``."""

    matrix_: np.ndarray = dataclasses.field(default_factory=lambda: np.eye(3))
    vector: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(3))

    def matrix(self) -> np.ndarray:
        m = np.eye(4)
        m[:3, :3] = np.asarray(self.matrix_, dtype=np.float64)
        m[:3, 3] = np.asarray(self.vector, dtype=np.float64)
        return m


@dataclasses.dataclass(eq=False)
class TransformationList(AbstractTransformation):
    """Apply ``transformations[0]`` first, then ``transformations[1]``, ..."""

    transformations: Sequence[AbstractTransformation] = ()

    def matrix(self) -> np.ndarray:
        m = np.eye(4)
        for t in self.transformations:
            m = matrix_of(t) @ m
        return m


Cartesian3dTranslation = Translation
Cartesian3dRotationX = RotationX
Cartesian3dRotationY = RotationY
Cartesian3dRotationZ = RotationZ


def matrix_of(t: None | AbstractTransformation) -> np.ndarray:
    """4x4 float64 matrix of a transformation (identity for ``None``)."""
    if t is None:
        return np.eye(4)
    return t.matrix()
