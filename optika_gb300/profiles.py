"""Interface profiles between the layers of a multilayer stack (Stearns
1989), mirroring optika/materials/profiles.py.

A profile on a :class:`~optika_gb300.materials.Layer` describes the
interface on the layer's left side; the trace multiplies that interface's
reflection amplitude by the Fourier transform of the profile's derivative,
evaluated on the GPU inside the multilayer transfer-matrix product.  The
methods here (``__call__``, ``reflectivity``, ``transmissivity``) evaluate
the same closed forms with torch on the device of their inputs, for
inspection and plotting; widths and wavelengths are nm.
"""

from __future__ import annotations

import dataclasses
import math

import torch

__all__ = [
    "AbstractInterfaceProfile",
    "ErfInterfaceProfile",
    "ExponentialInterfaceProfile",
    "LinearInterfaceProfile",
    "SinusoidalInterfaceProfile",
]


def _t(x) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x if x.is_floating_point() or x.is_complex() else x.double()
    return torch.as_tensor(x, dtype=torch.complex128 if isinstance(x, complex) else
                           torch.float64)


@dataclasses.dataclass(eq=False)
class AbstractInterfaceProfile:
    """Base of the profiles (optika/materials/profiles.py:21-128)."""

    width: float = 0.0
    """Characteristic length of the profile (nm)."""

    tag = 0

    def _derivative_fourier_transform(self, s: torch.Tensor) -> torch.Tensor:
        raise NotImplementedError  # pragma: no cover

    def transmissivity(self, wavelength, direction_before, direction_after, n_before, n_after):
        """Specular transmission factor, Stearns (1989) eq. 42
        (optika/materials/profiles.py:67-101)."""
        k_before = -2 * math.pi * _t(n_before) * _t(direction_before) / _t(wavelength)
        k_after = -2 * math.pi * _t(n_after) * _t(direction_after) / _t(wavelength)
        s = torch.real(k_after - k_before) if (k_after - k_before).is_complex() else (
            k_after - k_before)
        return self._derivative_fourier_transform(s)

    def reflectivity(self, wavelength, direction, n):
        """Factor on the reflection amplitude (optika/materials/profiles.py:
        103-128): the transform at s = Re(4 pi n direction / lambda)."""
        k = -2 * math.pi * _t(n) * _t(direction) / _t(wavelength)
        s = -2 * k
        s = torch.real(s) if s.is_complex() else s
        return self._derivative_fourier_transform(s)


@dataclasses.dataclass(eq=False)
class ErfInterfaceProfile(AbstractInterfaceProfile):
    """Error-function profile (optika/materials/profiles.py:130-223)."""

    tag = 1

    def __call__(self, z):
        return (1 + torch.special.erf(_t(z) / (math.sqrt(2) * self.width))) / 2

    def _derivative_fourier_transform(self, s):
        return torch.exp(-torch.square(s * self.width) / 2)


@dataclasses.dataclass(eq=False)
class ExponentialInterfaceProfile(AbstractInterfaceProfile):
    """Exponential profile (optika/materials/profiles.py:226-326)."""

    tag = 2

    def __call__(self, z):
        z = _t(z)
        sgn = torch.sign(z)
        return (1 + sgn - sgn * torch.exp(-sgn * math.sqrt(2) * z / self.width)) / 2

    def _derivative_fourier_transform(self, s):
        return 1 / (1 + torch.square(s * self.width) / 2)


@dataclasses.dataclass(eq=False)
class LinearInterfaceProfile(AbstractInterfaceProfile):
    """Linear profile (optika/materials/profiles.py:328-431)."""

    tag = 3

    def __call__(self, z):
        r = 0.5 + _t(z) / (2 * math.sqrt(3) * self.width)
        return torch.clamp(r, 0, 1)

    def _derivative_fourier_transform(self, s):
        x = math.sqrt(3) * self.width * s
        return torch.sin(x) / x


@dataclasses.dataclass(eq=False)
class SinusoidalInterfaceProfile(AbstractInterfaceProfile):
    """Sinusoidal profile, a = pi / (pi^2 - 8)
    (optika/materials/profiles.py:434-541)."""

    tag = 4

    def __call__(self, z):
        a = math.pi / (math.pi**2 - 8)
        z = torch.clamp(_t(z), -a * self.width, a * self.width)
        return 0.5 + torch.sin(math.pi * z / (2 * a * self.width)) / 2

    def _derivative_fourier_transform(self, s):
        a = math.pi / (math.pi**2 - 8)
        x = a * self.width * s
        x1 = x - math.pi / 2
        x2 = x + math.pi / 2
        return math.pi * (torch.sin(x1) / x1 + torch.sin(x2) / x2) / 4
