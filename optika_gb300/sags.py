"""Sag profiles (surface shapes), mirroring optika/sags.

Each class describes one shape; the arithmetic runs on the GPU, either fused
into the trace or through :func:`optika_gb300.sags.AbstractSag.__call__`,
:meth:`normal` and :meth:`intercept`, which launch the same device functions
as the trace.  Lengths are mm.  Normals follow the reference's z < 0
convention (optika/sags/_tests/_abc_test.py:78-88).
"""

from __future__ import annotations

import dataclasses
import math

from . import transforms

__all__ = [
    "AbstractSag",
    "NoSag",
    "SphericalSag",
    "AbstractConicSag",
    "ConicSag",
    "ParabolicSag",
    "ToroidalSag",
    "CylindricalSag",
]


@dataclasses.dataclass(eq=False)
class AbstractSag:
    """Base of all sag profiles (optika/sags/_abc.py:14-122)."""

    transformation: None | transforms.AbstractTransformation = dataclasses.field(
        default=None, kw_only=True
    )

    def __call__(self, position):
        """Sag z(x, y) at each position (``Cartesian3dVectorArray``)."""
        from ._api import sag_eval

        return sag_eval(self, "sag", position)

    def normal(self, position):
        """Unit normal (z < 0) at each position."""
        from ._api import sag_eval

        return sag_eval(self, "normal", position)

    def intercept(self, rays):
        """Rays moved along their direction onto this sag."""
        from ._api import sag_intercept

        return sag_intercept(self, rays)


@dataclasses.dataclass(eq=False)
class NoSag(AbstractSag):
    """A flat sag profile (optika/sags/_flat.py:13-64)."""


@dataclasses.dataclass(eq=False)
class SphericalSag(AbstractSag):
    """``z = c r^2 / (1 + sqrt(1 - c^2 r^2))`` (optika/sags/_spherical.py:40-191)."""

    radius: float = math.inf

    @property
    def curvature(self) -> float:
        return 1.0 / self.radius


@dataclasses.dataclass(eq=False)
class AbstractConicSag(AbstractSag):
    """Conic of revolution (optika/sags/_conic.py:16-170)."""

    @property
    def radius(self) -> float:  # pragma: no cover - abstract
        raise NotImplementedError

    @property
    def conic(self) -> float:  # pragma: no cover - abstract
        raise NotImplementedError


@dataclasses.dataclass(eq=False)
class ConicSag(AbstractConicSag):
    """``z = c r^2 / (1 + sqrt(1 - (1 + k) c^2 r^2))`` (optika/sags/_conic.py:173-252)."""

    radius: float = math.inf
    conic: float = 0.0


@dataclasses.dataclass(eq=False)
class ParabolicSag(AbstractConicSag):
    """Paraboloid of focal length f: radius 2 f, conic -1
    (optika/sags/_parabolic.py:14-158)."""

    focal_length: float = math.inf

    @property
    def radius(self) -> float:
        return 2.0 * self.focal_length

    @property
    def conic(self) -> float:
        return -1.0


@dataclasses.dataclass(eq=False)
class ToroidalSag(AbstractSag):
    """``z = r - sqrt((r - z_y)^2 - x^2)``, ``z_y`` the circle of ``radius`` in y
    (optika/sags/_toroidal.py:14-88).  ``radius`` is the minor radius and
    ``radius_of_rotation`` the major radius; as in the reference the vertex
    is at the origin only for ``radius_of_rotation >= 0``."""

    radius: float = math.inf
    radius_of_rotation: float = 0.0


@dataclasses.dataclass(eq=False)
class CylindricalSag(AbstractSag):
    """``z = c x^2 / (1 + sqrt(1 - c^2 x^2))``: a cylinder of ``radius`` whose
    axis is parallel to the local y axis (optika/sags/_cylindrical.py:14-160).
    Rays that miss the cylinder stop at the vertex plane z = 0, as in the
    reference."""

    radius: float = math.inf

    @property
    def curvature(self) -> float:
        return 1.0 / self.radius
