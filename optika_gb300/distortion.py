"""Distortion models, mirroring optika/distortion/_distortion.py: maps of
scene coordinates (wavelength, field position) to sensor positions and
back.  Coordinates are :class:`~optika_gb300.vectors.SpectralPositionalVectorArray`
of numpy arrays (wavelength nm; field in radians or mm as the system's
object gives it; sensor positions mm)."""

from __future__ import annotations

import dataclasses

import numpy as np

from ._polyfit import PolynomialFit
from .vectors import Cartesian2dVectorArray, SpectralPositionalVectorArray

__all__ = ["AbstractDistortionModel", "SimpleDistortionModel", "PolynomialDistortionModel"]


class AbstractDistortionModel:
    """optika/distortion/_distortion.py:25-66."""

    def distort(self, coordinates):  # pragma: no cover - abstract
        raise NotImplementedError

    def undistort(self, coordinates):  # pragma: no cover - abstract
        raise NotImplementedError


@dataclasses.dataclass(eq=False)
class SimpleDistortionModel(AbstractDistortionModel):
    """Rotation by ``angle``, isotropic ``plate_scale`` (field per sensor
    length) and linear ``dispersion`` (wavelength per sensor length) along
    the rotated x axis, about ``reference`` (a SpectralPositionalVectorArray:
    the wavelength and the sensor position of the field centre);
    optika/distortion/_distortion.py:116-235.  ``undistort`` is the exact
    inverse."""

    plate_scale: float = 1.0
    dispersion: float = 1.0
    angle: float = 0.0
    reference: SpectralPositionalVectorArray = None

    def distort(self, coordinates):
        c, s = np.cos(self.angle), np.sin(self.angle)
        w = np.asarray(coordinates.wavelength, dtype=np.float64)
        x = np.asarray(coordinates.position.x, dtype=np.float64)
        y = np.asarray(coordinates.position.y, dtype=np.float64)
        dw = w - self.reference.wavelength
        sx = (c * x - s * y) / self.plate_scale + dw / self.dispersion + self.reference.position.x
        sy = (s * x + c * y) / self.plate_scale + self.reference.position.y
        return SpectralPositionalVectorArray(wavelength=w, position=Cartesian2dVectorArray(sx, sy))

    def undistort(self, coordinates):
        c, s = np.cos(self.angle), np.sin(self.angle)
        w = np.asarray(coordinates.wavelength, dtype=np.float64)
        dw = w - self.reference.wavelength
        u = (np.asarray(coordinates.position.x) - self.reference.position.x
             - dw / self.dispersion) * self.plate_scale
        v = (np.asarray(coordinates.position.y) - self.reference.position.y) * self.plate_scale
        return SpectralPositionalVectorArray(
            wavelength=w, position=Cartesian2dVectorArray(c * u + s * v, -s * u + c * v))


@dataclasses.dataclass(eq=False)
class PolynomialDistortionModel(AbstractDistortionModel):
    """Polynomial fits scene -> sensor (``distort``) and sensor -> scene
    (``undistort``), each of total degree ``degree`` about the mean of the
    calibration points, over the points selected by ``where``
    (optika/distortion/_distortion.py:276-366)."""

    coordinates_scene: SpectralPositionalVectorArray = None
    coordinates_sensor: Cartesian2dVectorArray = None
    axis_wavelength: str = "wavelength"
    axis_field: tuple[str, str] = ("field_x", "field_y")
    degree: int = 1
    where: object = True

    def _scene(self):
        s = self.coordinates_scene
        return (np.asarray(s.wavelength, dtype=np.float64),
                np.asarray(s.position.x, dtype=np.float64),
                np.asarray(s.position.y, dtype=np.float64))

    @property
    def fit(self) -> PolynomialFit:
        if "_fit" not in self.__dict__:
            w, x, y = self._scene()
            self.__dict__["_fit"] = PolynomialFit(
                (w, x, y), (self.coordinates_sensor.x, self.coordinates_sensor.y),
                self.degree, where=self.where)
        return self.__dict__["_fit"]

    @property
    def fit_inverse(self) -> PolynomialFit:
        if "_fit_inverse" not in self.__dict__:
            w, x, y = self._scene()
            self.__dict__["_fit_inverse"] = PolynomialFit(
                (w, self.coordinates_sensor.x, self.coordinates_sensor.y), (x, y), self.degree,
                where=self.where)
        return self.__dict__["_fit_inverse"]

    def distort(self, coordinates):
        sx, sy = self.fit(coordinates.wavelength, coordinates.position.x, coordinates.position.y)
        return SpectralPositionalVectorArray(wavelength=coordinates.wavelength,
                                             position=Cartesian2dVectorArray(sx, sy))

    def undistort(self, coordinates):
        x, y = self.fit_inverse(coordinates.wavelength, coordinates.position.x,
                                coordinates.position.y)
        return SpectralPositionalVectorArray(wavelength=coordinates.wavelength,
                                             position=Cartesian2dVectorArray(x, y))
