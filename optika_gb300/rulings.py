"""Grating rulings, mirroring optika/rulings.

Ruling spacings (optika/rulings/_spacing.py): constant, 1-D polynomial
(variable line spacing ``d(x) = sum c_k x^k`` with ``x`` the projection of
the (optionally transformed) position on the ruling normal) and holographic
(two recording point sources).

Ruling models (optika/rulings/_rulings.py) differ in their groove
efficiency: :class:`Rulings` is ideal (efficiency 1), :class:`MeasuredRulings`
interpolates a measured efficiency in wavelength, and the thin-grating
models of Magnusson and Gaylord (1978), Table 1 -- :class:`SinusoidalRulings`,
:class:`SquareRulings`, :class:`SawtoothRulings`, :class:`TriangularRulings`
and :class:`RectangularRulings` -- evaluate the efficiency of the groove
profile for each ray inside the trace.  Lengths (spacings, groove depths)
are mm; wavelengths are nm.
"""

from __future__ import annotations

import dataclasses
import math
from typing import Mapping

import numpy as np

from . import transforms
from .vectors import spectral_table

__all__ = [
    "AbstractRulingSpacing",
    "ConstantRulingSpacing",
    "Polynomial1dRulingSpacing",
    "HolographicRulingSpacing",
    "AbstractRulings",
    "Rulings",
    "MeasuredRulings",
    "SinusoidalRulings",
    "SquareRulings",
    "SawtoothRulings",
    "TriangularRulings",
    "RectangularRulings",
]


class AbstractRulingSpacing:
    pass


@dataclasses.dataclass(eq=False)
class ConstantRulingSpacing(AbstractRulingSpacing):
    constant: float = 0.0
    normal: tuple[float, float, float] = (1.0, 0.0, 0.0)


@dataclasses.dataclass(eq=False)
class Polynomial1dRulingSpacing(AbstractRulingSpacing):
    coefficients: Mapping[int, float] = dataclasses.field(default_factory=dict)
    normal: tuple[float, float, float] = (1.0, 0.0, 0.0)
    transformation: None | transforms.AbstractTransformation = None


@dataclasses.dataclass(eq=False)
class HolographicRulingSpacing(AbstractRulingSpacing):
    x1: tuple[float, float, float] = (0.0, 0.0, 0.0)
    x2: tuple[float, float, float] = (0.0, 0.0, 0.0)
    wavelength: float = 0.0
    is_diverging_1: bool = True
    is_diverging_2: bool = False
    transformation: None | transforms.AbstractTransformation = None


class AbstractRulings:
    """Base of the ruling models (optika/rulings/_rulings.py:132-222)."""

    diffraction_order: float = 1.0

    @property
    def spacing_(self) -> AbstractRulingSpacing:
        """``spacing`` as a spacing object: a bare number is a constant
        spacing with ruling normal +x (optika/rulings/_rulings.py:157-168)."""
        s = self.spacing
        if isinstance(s, AbstractRulingSpacing):
            return s
        return ConstantRulingSpacing(constant=float(s), normal=(1.0, 0.0, 0.0))

    def incident_effective(self, rays, normal):
        """Rays with the effective incident direction of this diffraction
        order (optika/rulings/_rulings.py:170-204), on the GPU.  ``rays``
        are at the ruled surface, in its frame; ``normal`` is the sag normal
        there (a ``Cartesian3dVectorArray``)."""
        from ._api import rulings_eval

        return rulings_eval(self, "incident_effective", rays, normal)

    def efficiency(self, rays, normal):
        """Fraction of the light diffracted into ``diffraction_order``
        (optika/rulings/_rulings.py:207-222), on the GPU: the same device
        function the trace multiplies into each ray's intensity."""
        from ._api import rulings_eval

        return rulings_eval(self, "efficiency", rays, normal)


@dataclasses.dataclass(eq=False)
class Rulings(AbstractRulings):
    """Ideal rulings: efficiency 1 in every order
    (optika/rulings/_rulings.py:225-251)."""

    spacing: float | AbstractRulingSpacing = 0.0
    diffraction_order: float = 1.0


@dataclasses.dataclass(eq=False)
class MeasuredRulings(AbstractRulings):
    """Rulings whose efficiency was measured at a set of wavelengths for one
    incidence direction (optika/rulings/_rulings.py:255-314): linear
    interpolation in wavelength, clamped to the end values outside the
    measured range.

    ``efficiency_measured`` is a :class:`~optika_gb300.vectors.FunctionArray`
    whose ``inputs`` is a
    :class:`~optika_gb300.vectors.SpectralDirectionalVectorArray` (one
    increasing wavelength axis in nm, a single direction) and whose
    ``outputs`` are the efficiencies at those wavelengths."""

    spacing: float | AbstractRulingSpacing = 0.0
    diffraction_order: float = 1.0
    efficiency_measured: object = None

    def table(self) -> tuple[np.ndarray, np.ndarray]:
        """(wavelength, efficiency) of the measurement."""
        return spectral_table(self.efficiency_measured)


@dataclasses.dataclass(eq=False)
class SinusoidalRulings(AbstractRulings):
    """Sinusoidal grooves of the given ``depth`` (mm): efficiency
    ``J_m(2 gamma)``, ``gamma = pi depth / (lambda cos theta)``
    (optika/rulings/_rulings.py:317-457; the reference returns the Bessel
    function itself, not its square).  Integer diffraction orders."""

    spacing: float | AbstractRulingSpacing = 0.0
    depth: float = 0.0
    diffraction_order: float = 1.0

    amplitude = 1.0


@dataclasses.dataclass(eq=False)
class SquareRulings(AbstractRulings):
    """Square-wave grooves of the given ``depth`` (mm), amplitude pi / 4
    (optika/rulings/_rulings.py:461-614)."""

    spacing: float | AbstractRulingSpacing = 0.0
    depth: float = 0.0
    diffraction_order: float = 1.0

    amplitude = math.pi / 4


@dataclasses.dataclass(eq=False)
class SawtoothRulings(AbstractRulings):
    """Sawtooth (blazed) grooves of the given ``depth`` (mm), amplitude
    pi / 2 (optika/rulings/_rulings.py:618-758)."""

    spacing: float | AbstractRulingSpacing = 0.0
    depth: float = 0.0
    diffraction_order: float = 1.0

    amplitude = math.pi / 2


@dataclasses.dataclass(eq=False)
class TriangularRulings(AbstractRulings):
    """Symmetric triangular grooves of the given ``depth`` (mm), amplitude
    pi^2 / 8 (optika/rulings/_rulings.py:762-911)."""

    spacing: float | AbstractRulingSpacing = 0.0
    depth: float = 0.0
    diffraction_order: float = 1.0

    amplitude = math.pi**2 / 8


@dataclasses.dataclass(eq=False)
class RectangularRulings(AbstractRulings):
    """Rectangular grooves of the given ``depth`` (mm) and duty cycle
    ``ratio_duty`` (a = 2 pi ratio_duty, amplitude
    pi / (2 sqrt(2 (1 - cos a)))), optika/rulings/_rulings.py:915-1073."""

    spacing: float | AbstractRulingSpacing = 0.0
    depth: float = 0.0
    ratio_duty: float = 0.5
    diffraction_order: float = 1.0

    @property
    def amplitude(self) -> float:
        a = 2 * math.pi * float(self.ratio_duty)
        return math.pi / (2 * math.sqrt(2 * (1 - math.cos(a))))
