"""Grating rulings, mirroring optika/rulings.

Ruling spacings (optika/rulings/_spacing.py): constant, 1-D polynomial
(variable line spacing ``d(x) = sum c_k x^k`` with ``x`` the projection of
the (optionally transformed) position on the ruling normal) and holographic
(two recording point sources).  :class:`Rulings` is the ideal ruling of
efficiency 1 (optika/rulings/_rulings.py:225-251).  Lengths are mm; the
holographic recording wavelength is nm.
"""

from __future__ import annotations

import dataclasses
from typing import Mapping

from . import transforms

__all__ = [
    "AbstractRulingSpacing",
    "ConstantRulingSpacing",
    "Polynomial1dRulingSpacing",
    "HolographicRulingSpacing",
    "AbstractRulings",
    "Rulings",
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
    diffraction_order: float = 1.0

    @property
    def spacing_(self) -> AbstractRulingSpacing:
        """``spacing`` as a spacing object: a bare number is a constant
        spacing with ruling normal +x (optika/rulings/_rulings.py:157-168)."""
        s = self.spacing
        if isinstance(s, AbstractRulingSpacing):
            return s
        return ConstantRulingSpacing(constant=float(s), normal=(1.0, 0.0, 0.0))


@dataclasses.dataclass(eq=False)
class Rulings(AbstractRulings):
    """Ideal rulings: efficiency 1 in every order."""

    spacing: float | AbstractRulingSpacing = 0.0
    diffraction_order: float = 1.0

    efficiency = 1.0
