"""Radiometric calibration models, mirroring optika/radiometry: relative
illumination (vignetting) and effective area."""

from __future__ import annotations

import dataclasses

import numpy as np

from ._polyfit import PolynomialFit
from .vectors import SpectralPositionalVectorArray

__all__ = ["PolynomialVignettingModel", "InterpolatedEffectiveAreaModel"]


@dataclasses.dataclass(eq=False)
class PolynomialVignettingModel:
    """Polynomial fit of the relative illumination over the scene coordinates
    (optika/radiometry/_vignetting.py:99-160); ``inverse`` is ``1 / I``
    (:43-58)."""

    coordinates_scene: SpectralPositionalVectorArray = None
    illumination: object = None
    axis_wavelength: str = "wavelength"
    axis_field: tuple[str, str] = ("field_x", "field_y")
    degree: int = 1
    where: object = True

    @property
    def fit(self) -> PolynomialFit:
        if "_fit" not in self.__dict__:
            s = self.coordinates_scene
            self.__dict__["_fit"] = PolynomialFit(
                (s.wavelength, s.position.x, s.position.y), (self.illumination,), self.degree,
                where=self.where)
        return self.__dict__["_fit"]

    def __call__(self, coordinates):
        return self.fit(coordinates.wavelength, coordinates.position.x,
                        coordinates.position.y)[0]

    def inverse(self, coordinates):
        return 1 / self(coordinates)


@dataclasses.dataclass(eq=False)
class InterpolatedEffectiveAreaModel:
    """Effective area linearly interpolated in wavelength
    (optika/radiometry/_effective_area.py:33-95; numpy.interp semantics for
    na.interp: the end values outside the calibration range)."""

    wavelength: object = None
    area: object = None
    axis_wavelength: str = "wavelength"

    def __call__(self, wavelength):
        return np.interp(np.asarray(wavelength, dtype=np.float64),
                         np.asarray(self.wavelength, dtype=np.float64),
                         np.asarray(self.area, dtype=np.float64))
