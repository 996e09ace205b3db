"""Optical materials and multilayer stacks, mirroring optika/materials.

* :class:`Vacuum`, :class:`Mirror`, :class:`Glass` (optika/materials/_materials.py:82-455)
* :class:`Layer`, :class:`LayerSequence`, :class:`PeriodicLayerSequence`
  (optika/materials/_layers.py)
* :class:`MultilayerMirror`, :class:`MultilayerFilm` and
  :func:`multilayer_efficiency` (optika/materials/_multilayers.py)

Units: wavelengths and thicknesses in nm, Sellmeier C terms in um^2 (as in
the reference), attenuation in 1/mm.
"""

from __future__ import annotations

import dataclasses
from typing import Sequence, Union

from . import profiles  # noqa: F401  (optika.materials.profiles)
from .chemicals import Chemical
from .vectors import PolarizationVectorArray

__all__ = [
    "AbstractMaterial",
    "Vacuum",
    "AbstractMirror",
    "Mirror",
    "MeasuredMirror",
    "Glass",
    "Layer",
    "LayerSequence",
    "PeriodicLayerSequence",
    "MultilayerMirror",
    "MultilayerFilm",
    "multilayer_efficiency",
    "PeriodicMirror",
    "multilayer_efficiency_periodic",
]


class AbstractMaterial:
    is_mirror: bool = False


@dataclasses.dataclass(eq=False)
class Vacuum(AbstractMaterial):
    """n = 1, no attenuation, transmits (optika/materials/_materials.py:82-116)."""

    is_mirror = False


class AbstractMirror(AbstractMaterial):
    is_mirror = True


@dataclasses.dataclass(eq=False)
class Mirror(AbstractMirror):
    """A perfect mirror, efficiency 1 (optika/materials/_materials.py:161-173)."""

    substrate: None | "Layer" = None


@dataclasses.dataclass(eq=False)
class MeasuredMirror(AbstractMirror):
    """A mirror whose reflectivity was measured at a set of wavelengths for
    one incidence direction (optika/materials/_materials.py:177-306): linear
    interpolation in the wavelength of the incident rays, clamped to the end
    values outside the measured range.  ``efficiency_measured`` is a
    :class:`~optika_gb300.vectors.FunctionArray` of reflectivities over a
    :class:`~optika_gb300.vectors.SpectralDirectionalVectorArray` (one
    increasing wavelength axis in nm, a single direction)."""

    efficiency_measured: object = None
    substrate: None | "Layer" = None
    serial_number: None | str = None

    def table(self):
        """(wavelength, reflectivity) of the measurement."""
        from .vectors import spectral_table

        return spectral_table(self.efficiency_measured)


@dataclasses.dataclass(eq=False)
class Glass(AbstractMaterial):
    """Three-term Sellmeier glass (optika/materials/_materials.py:309-455).
    ``c1..c3`` in um^2."""

    b1: float = 0.0
    b2: float = 0.0
    b3: float = 0.0
    c1: float = 0.0
    c2: float = 0.0
    c3: float = 0.0

    @classmethod
    def n_bk7(cls) -> "Glass":
        """SCHOTT N-BK7 (catalogue Sellmeier coefficients)."""
        return cls(1.03961212, 0.231792344, 1.01046945, 0.00600069867, 0.0200179144, 103.560653)

    @classmethod
    def f2(cls) -> "Glass":
        """SCHOTT F2 (catalogue Sellmeier coefficients)."""
        return cls(1.34533359, 0.209073176, 0.937357162, 0.00997743871, 0.0470450767, 111.886764)


IndexSource = Union[None, complex, float, Chemical]


@dataclasses.dataclass(eq=False)
class Layer:
    """One homogeneous layer (optika/materials/_layers.py:150-277).
    ``chemical`` is ``None`` (vacuum), a constant complex index or a
    :class:`~optika_gb300.chemicals.Chemical` table; ``thickness`` in nm."""

    chemical: IndexSource = None
    thickness: None | float = None
    interface: None | object = None


@dataclasses.dataclass(eq=False)
class LayerSequence:
    layers: Sequence[Layer] = ()


@dataclasses.dataclass(eq=False)
class PeriodicLayerSequence:
    """``layers`` repeated ``num_periods`` times; evaluated as the first
    period times the period matrix to the power ``num_periods - 1``
    (optika/materials/_layers.py:611-645)."""

    layers: Sequence[Layer] = ()
    num_periods: int = 1


LayersLike = Union[None, Layer, LayerSequence, PeriodicLayerSequence, Sequence]


@dataclasses.dataclass(eq=False)
class MultilayerMirror(AbstractMirror):
    """Mirror whose efficiency is the multilayer reflectivity averaged over
    s and p (optika/materials/_multilayers.py:908-935)."""

    layers: LayersLike = None
    substrate: None | Layer = None


@dataclasses.dataclass(eq=False)
class MultilayerFilm(AbstractMaterial):
    """Thin film whose efficiency is the multilayer transmissivity averaged
    over s and p (optika/materials/_multilayers.py:839-866)."""

    layers: LayersLike = None
    is_mirror = False


def multilayer_efficiency(
    wavelength,
    direction=1.0,
    n=1.0,
    layers: LayersLike = None,
    substrate: None | Layer = None,
) -> tuple[PolarizationVectorArray, PolarizationVectorArray]:
    """Reflectivity and transmissivity (s, p) of a multilayer stack on the GPU.

    Mirrors optika/materials/_multilayers.py:240-532.  ``wavelength`` is the
    vacuum wavelength in nm, ``direction`` the cosine of the incidence angle
    in the ambient medium and ``n`` its complex index; each is a scalar or an
    array (numpy or torch), broadcast together.  Returns two
    :class:`~optika_gb300.vectors.PolarizationVectorArray` of float32 CUDA
    tensors.
    """
    from ._api import multilayer_efficiency_gpu

    return multilayer_efficiency_gpu(wavelength, direction, n, layers, substrate)


@dataclasses.dataclass(eq=False)
class PeriodicMirror:
    """A periodic bilayer mirror ``[a, b] x num_periods`` on ``substrate``,
    every medium of constant complex index (optika/materials/_layers.py:
    571-645 with two layers)."""

    a: Layer
    b: Layer
    num_periods: int
    substrate: Layer

    @property
    def layers(self) -> PeriodicLayerSequence:
        return PeriodicLayerSequence([self.a, self.b], self.num_periods)


def multilayer_efficiency_periodic(wavelength, direction, mirrors, index=None, n=1.0):
    """Batched :func:`multilayer_efficiency` over periodic bilayer mirrors.

    ``mirrors`` is a sequence of :class:`PeriodicMirror`; ``index`` (int
    array, or ``None`` for mirror 0) picks each sample's mirror.  Returns
    ``(R, T)`` as :class:`~optika_gb300.vectors.PolarizationVectorArray` of
    float32 CUDA tensors.  Transfer matrices are float-float.
    """
    from ._api import multilayer_periodic_gpu

    return multilayer_periodic_gpu(wavelength, direction, mirrors, index, n)
