"""Optical surfaces, mirroring optika/surfaces.py.

A :class:`Surface` composes a sag, a material, an aperture and optional
rulings at a position given by ``transformation``.  Its
:meth:`propagate_rays` traces rays through this one surface on the GPU with
the same fused kernel that traces whole systems
(optika/surfaces.py:123-198).
"""

from __future__ import annotations

import dataclasses

from . import apertures as _apertures
from . import materials as _materials
from . import rulings as _rulings
from . import sags as _sags
from . import transforms

__all__ = ["AbstractSurface", "Surface"]


class AbstractSurface:
    def propagate_rays(self, rays):
        """Refract, reflect and/or diffract ``rays`` (in the parent frame)
        off this surface; returns new rays in the parent frame."""
        from ._api import propagate_rays

        return propagate_rays([self], rays)


@dataclasses.dataclass(eq=False)
class Surface(AbstractSurface):
    name: None | str = None
    sag: None | _sags.AbstractSag = None
    material: None | _materials.AbstractMaterial = None
    aperture: None | _apertures.AbstractAperture = None
    aperture_mechanical: None | _apertures.AbstractAperture = None
    rulings: None | _rulings.AbstractRulings = None
    is_field_stop: bool = False
    is_pupil_stop: bool = False
    transformation: None | transforms.AbstractTransformation = None

    def __post_init__(self):
        if self.sag is None:
            self.sag = _sags.NoSag()
        if self.material is None:
            self.material = _materials.Vacuum()
