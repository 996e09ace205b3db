"""Small vector containers of the host API.

Components are anything array-like (floats, numpy arrays, torch tensors);
they are broadcast and moved to the device when a trace is launched.
Mirrors optika/vectors (ObjectVectorArray ``_vectors_object.py:136-160``,
PolarizationVectorArray ``_vectors_polarization.py:36-37``).
"""

from __future__ import annotations

import dataclasses
from typing import Any

__all__ = [
    "Cartesian2dVectorArray",
    "Cartesian3dVectorArray",
    "ObjectVectorArray",
    "PolarizationVectorArray",
]


@dataclasses.dataclass
class Cartesian2dVectorArray:
    x: Any = 0.0
    y: Any = 0.0


@dataclasses.dataclass
class Cartesian3dVectorArray:
    x: Any = 0.0
    y: Any = 0.0
    z: Any = 0.0

    @property
    def xy(self) -> Cartesian2dVectorArray:
        return Cartesian2dVectorArray(self.x, self.y)


@dataclasses.dataclass
class ObjectVectorArray:
    """Input grid of a sequential system: vacuum wavelength (nm), field and
    pupil coordinates.  For an object at infinity the field is a pair of
    angles (radians) and the pupil a position (mm); for a finite object the
    field is a position and the pupil a pair of angles."""

    wavelength: Any = 550.0
    field: Cartesian2dVectorArray = dataclasses.field(default_factory=Cartesian2dVectorArray)
    pupil: Cartesian2dVectorArray = dataclasses.field(default_factory=Cartesian2dVectorArray)


@dataclasses.dataclass
class PolarizationVectorArray:
    """A quantity for s and p polarisation; ``average`` is ``(s + p) / 2``."""

    s: Any = 0.0
    p: Any = 0.0

    @property
    def average(self) -> Any:
        return (self.s + self.p) / 2
