"""Small vector containers of the host API.

Components are anything array-like (floats, numpy arrays, torch tensors);
they are broadcast and moved to the device when a trace is launched.
Mirrors optika/vectors (ObjectVectorArray ``_vectors_object.py:136-160``,
PolarizationVectorArray ``_vectors_polarization.py:36-37``) and the two
named_arrays containers a measured ruling efficiency is given in
(``SpectralDirectionalVectorArray`` inputs of a ``FunctionArray``).
"""

from __future__ import annotations

import dataclasses
from typing import Any

import numpy as np

__all__ = [
    "Cartesian2dVectorArray",
    "Cartesian3dVectorArray",
    "ObjectVectorArray",
    "PolarizationVectorArray",
    "SpectralDirectionalVectorArray",
    "SpectralPositionalVectorArray",
    "FunctionArray",
    "spectral_table",
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


@dataclasses.dataclass
class SpectralDirectionalVectorArray:
    """A wavelength (nm) and a propagation direction."""

    wavelength: Any = 550.0
    direction: Any = None


@dataclasses.dataclass
class SpectralPositionalVectorArray:
    """A wavelength (nm) and a position (a Cartesian2dVectorArray)."""

    wavelength: Any = 550.0
    position: Any = None


@dataclasses.dataclass
class FunctionArray:
    """Sampled function: ``outputs`` at ``inputs``."""

    inputs: Any = None
    outputs: Any = None


def spectral_table(measurement: FunctionArray) -> tuple[np.ndarray, np.ndarray]:
    """(wavelength, value) of a measurement taken at one incidence
    direction, checked as the reference checks its measured mirrors and
    rulings (optika/materials/_materials.py:285-301,
    optika/rulings/_rulings.py:293-307)."""
    wavelength = np.asarray(measurement.inputs.wavelength, dtype=np.float64)
    direction = measurement.inputs.direction
    size = 1 if direction is None else np.asarray(getattr(direction, "x", direction)).size
    if size != 1:
        raise ValueError("Interpolating over different incidence angles is not supported.")
    if wavelength.ndim != 1:
        raise ValueError(f"wavelength must be one dimensional, got shape {wavelength.shape}")
    value = np.asarray(measurement.outputs, dtype=np.float64).reshape(-1)
    if value.shape != wavelength.shape:
        raise ValueError("one measured value per wavelength is needed")
    if wavelength.size < 1:
        raise ValueError("the measurement has no wavelengths")
    return wavelength, value
