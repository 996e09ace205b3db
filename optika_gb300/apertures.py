"""Apertures and obscurations, mirroring optika/apertures/_apertures.py.

The mask test runs on the GPU inside the trace.  As in the reference
(``clip_rays``, :82-102) an aperture with length units tests the ray
position, a dimensionless one (``dimensionless=True`` here, e.g. an angular
field stop of radius ``sin(theta)``) tests the ray direction.  Edges are
inclusive, ``inverted`` turns an aperture into an obscuration and
``active=False`` passes every ray.
"""

from __future__ import annotations

import dataclasses
import math
from typing import Sequence

import numpy as np

from . import transforms

__all__ = [
    "AbstractAperture",
    "CircularAperture",
    "CircularSectorAperture",
    "EllipticalAperture",
    "PolygonalAperture",
    "RectangularAperture",
    "RegularPolygonalAperture",
    "OctagonalAperture",
    "IsoscelesTrapezoidalAperture",
]


def _linspace_wire(num: int, endpoint: bool) -> np.ndarray:
    return np.linspace(0.0, 1.0, num, endpoint=endpoint)


def _polygon_wire(vertices: np.ndarray, num: int) -> np.ndarray:
    """Points along the sides of a polygon, ``num / sides`` per side, the
    last side closing the loop on the first vertex
    (optika/apertures/_apertures.py:794-840)."""
    nv = len(vertices)
    per_side = num / nv
    out = []
    cum = 0
    for v in range(nv):
        num_v = int((v + 1) * per_side - cum)
        cum += num_v
        t = _linspace_wire(num_v, endpoint=cum == num)[:, None]
        left, right = vertices[v], vertices[(v + 1) % nv]
        out.append(left + (right - left) * t)
    return np.concatenate(out, axis=0)


@dataclasses.dataclass(eq=False)
class AbstractAperture:
    active: bool = dataclasses.field(default=True, kw_only=True)
    inverted: bool = dataclasses.field(default=False, kw_only=True)
    transformation: None | transforms.AbstractTransformation = dataclasses.field(
        default=None, kw_only=True
    )
    dimensionless: bool = dataclasses.field(default=False, kw_only=True)

    samples_wire: int = dataclasses.field(default=101, kw_only=True)

    def _wire_local(self, num: int) -> np.ndarray:
        raise NotImplementedError(f"{type(self).__name__} has no wire")

    def wire(self, num: None | int = None) -> np.ndarray:
        """``num`` points (float64, ``[num, 3]``) along the boundary of this
        aperture in surface coordinates, its transformation applied
        (optika/apertures/_apertures.py:121-130 and the overrides)."""
        num = self.samples_wire if num is None else int(num)
        xy = self._wire_local(num)
        pts = np.concatenate([xy, np.zeros((len(xy), 1))], axis=1)
        if self.transformation is not None:
            m = transforms.matrix_of(self.transformation)
            pts = pts @ m[:3, :3].T + m[:3, 3]
        return pts


@dataclasses.dataclass(eq=False)
class CircularAperture(AbstractAperture):
    """``|xy| <= radius`` (optika/apertures/_apertures.py:292-314)."""

    radius: float = 0.0

    def _wire_local(self, num: int) -> np.ndarray:
        # optika/apertures/_apertures.py:338-355 (both ends of 0..360 deg)
        az = np.linspace(0.0, 2 * math.pi, num)
        return np.stack([self.radius * np.cos(az), self.radius * np.sin(az)], axis=-1)


@dataclasses.dataclass(eq=False)
class CircularSectorAperture(AbstractAperture):
    """Circle of ``radius`` between two angles in radians
    (optika/apertures/_apertures.py:438-480)."""

    radius: float = 0.0
    angle_start: float = 0.0
    angle_stop: float = 0.0

    def _wire_local(self, num: int) -> np.ndarray:
        # optika/apertures/_apertures.py:548-594: the two radial arms and the arc
        per = num / 3
        out = []
        cum = 0
        for seg in range(3):
            num_s = int((seg + 1) * per - cum)
            cum += num_s
            t = _linspace_wire(num_s, endpoint=cum == num)
            if seg == 0:
                r, a = self.radius * t, np.full_like(t, self.angle_start)
            elif seg == 1:
                r = np.full_like(t, self.radius)
                a = self.angle_start + (self.angle_stop - self.angle_start) * t
            else:
                r, a = self.radius * (1 - t), np.full_like(t, self.angle_stop)
            out.append(np.stack([r * np.cos(a), r * np.sin(a)], axis=-1))
        return np.concatenate(out, axis=0)


@dataclasses.dataclass(eq=False)
class EllipticalAperture(AbstractAperture):
    """``(x/rx)^2 + (y/ry)^2 <= 1`` (optika/apertures/_apertures.py:640-663)."""

    radius: tuple[float, float] = (0.0, 0.0)

    def _wire_local(self, num: int) -> np.ndarray:
        # optika/apertures/_apertures.py:704-720
        az = np.linspace(0.0, 2 * math.pi, num)
        rx, ry = self.radius
        return np.stack([rx * np.cos(az), ry * np.sin(az)], axis=-1)


@dataclasses.dataclass(eq=False)
class RectangularAperture(AbstractAperture):
    """``|x| <= hx and |y| <= hy`` (optika/apertures/_apertures.py:941-968).
    ``half_width`` is a scalar or an ``(hx, hy)`` pair."""

    half_width: float | tuple[float, float] = 0.0

    @property
    def half_width_xy(self) -> tuple[float, float]:
        hw = self.half_width
        if np.ndim(hw) == 0:
            return float(hw), float(hw)
        hx, hy = hw
        return float(hx), float(hy)

    @property
    def vertices(self) -> np.ndarray:
        hx, hy = self.half_width_xy
        return np.array([[hx, hy], [-hx, hy], [-hx, -hy], [hx, -hy]], dtype=np.float64)

    def _wire_local(self, num: int) -> np.ndarray:
        return _polygon_wire(self.vertices, num)


@dataclasses.dataclass(eq=False)
class PolygonalAperture(AbstractAperture):
    """Even-odd point-in-polygon test over ``vertices`` (N x 2, local xy)
    (optika/apertures/_apertures.py:739-778)."""

    vertices: Sequence[Sequence[float]] = ()

    def vertex_array(self) -> np.ndarray:
        v = np.asarray(self.vertices, dtype=np.float64)
        return v[:, :2]

    def _wire_local(self, num: int) -> np.ndarray:
        return _polygon_wire(self.vertex_array(), num)


@dataclasses.dataclass(eq=False)
class RegularPolygonalAperture(PolygonalAperture):
    """Regular polygon with vertices at ``radius``, the first on +x
    (optika/apertures/_apertures.py:1000-1040)."""

    radius: float = 0.0
    num_vertices: int = 0

    def vertex_array(self) -> np.ndarray:
        a = np.arange(self.num_vertices) * (2 * math.pi / self.num_vertices)
        return np.stack([self.radius * np.cos(a), self.radius * np.sin(a)], axis=-1)


@dataclasses.dataclass(eq=False)
class OctagonalAperture(RegularPolygonalAperture):
    """Regular octagon (optika/apertures/_apertures.py:1043-1075)."""

    num_vertices: int = 8


@dataclasses.dataclass(eq=False)
class IsoscelesTrapezoidalAperture(PolygonalAperture):
    """Trapezoid between ``x_left`` and ``x_right`` with legs at
    +-``angle``/2 (optika/apertures/_apertures.py:1078-1193)."""

    x_left: float = 0.0
    x_right: float = 0.0
    angle: float = 0.0

    def vertex_array(self) -> np.ndarray:
        m = math.tan(self.angle / 2)
        upper = [[self.x_left, m * self.x_left], [self.x_right, m * self.x_right]]
        lower = [[x, -y] for x, y in reversed(upper)]
        return np.array(upper + lower, dtype=np.float64)
