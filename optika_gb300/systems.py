"""Sequential optical systems, mirroring optika/systems/_sequential.py.

:meth:`SequentialSystem.raytrace` and :meth:`SequentialSystem.rayfunction`
build the input rays from a (wavelength, field, pupil) grid and trace them
through ``[object] + surfaces + [sensor]`` in one fused GPU launch
(optika/systems/_sequential.py:791-988).  Field and pupil coordinates must
be physical (``normalized_field=False, normalized_pupil=False``): the stop
solve behind normalised coordinates (:396-789) is not part of this build.
"""

from __future__ import annotations

import dataclasses
from typing import Sequence

from . import _lib as L
from . import transforms
from .rays import RayFunctionArray
from .surfaces import AbstractSurface
from .vectors import ObjectVectorArray

__all__ = ["SequentialSystem"]


@dataclasses.dataclass(eq=False)
class SequentialSystem:
    surfaces: Sequence[AbstractSurface] = ()
    object: None | AbstractSurface = None
    sensor: None | AbstractSurface = None
    grid_input: None | ObjectVectorArray = None
    transformation: None | transforms.AbstractTransformation = None
    axis_surface: str = "surface"

    @property
    def object_is_at_infinity(self) -> bool:
        """No object aperture, or a dimensionless one, means the object is at
        infinity (optika/systems/_sequential.py:44-63)."""
        obj = self.object
        if obj is None or obj.aperture is None:
            return True
        return bool(obj.aperture.dimensionless)

    @property
    def surfaces_all(self) -> list[AbstractSurface]:
        """``[object] + surfaces + [sensor]`` (optika/systems/_sequential.py:92-112)."""
        out = [] if self.object is None else [self.object]
        out += list(self.surfaces)
        if self.sensor is not None:
            out.append(self.sensor)
        return out

    def _grid(self, wavelength, field, pupil, normalized_field, normalized_pupil):
        if normalized_field or normalized_pupil:
            raise NotImplementedError(
                "normalized field/pupil coordinates need the stop solver, which this build "
                "does not provide; pass physical coordinates with "
                "normalized_field=False, normalized_pupil=False"
            )
        g = self.grid_input if self.grid_input is not None else ObjectVectorArray()
        return (
            g.wavelength if wavelength is None else wavelength,
            g.field if field is None else field,
            g.pupil if pupil is None else pupil,
        )

    def raytrace(
        self,
        intensity=None,
        wavelength=None,
        field=None,
        pupil=None,
        axis: None | str = None,
        normalized_field: bool = True,
        normalized_pupil: bool = True,
        accumulate: bool = True,
        image: bool = False,
        wavelength_bins=None,
        launch: None | L.Launch = None,
        outputs: None | Sequence[str] = None,
    ) -> RayFunctionArray:
        """Trace input rays through every surface; outputs in the system's
        frame, stacked over surfaces (leading axis) when ``accumulate``
        (optika/systems/_sequential.py:836-925).  ``image=True`` also bins
        the rays on the sensor (``result.image = (counts, flux)``).
        ``outputs`` names the ray fields to return (``px py pz dx dy dz
        wavelength intensity attenuation index_refraction unvignetted
        opl``; default all); the others are ``None``.  CPU tensor inputs
        give CPU outputs."""
        from ._api import OUTPUT_FIELDS, trace_grid

        wl, fld, pup = self._grid(wavelength, field, pupil, normalized_field, normalized_pupil)
        res = trace_grid(
            self, wavelength=wl, field=fld, pupil=pup, intensity=intensity,
            accumulate=accumulate, final_local=False, image=image,
            wavelength_bins=wavelength_bins, launch=launch,
            outputs=OUTPUT_FIELDS if outputs is None else tuple(outputs),
        )
        res.inputs = ObjectVectorArray(wavelength=wl, field=fld, pupil=pup)
        return res

    def rayfunction(
        self,
        intensity=None,
        wavelength=None,
        field=None,
        pupil=None,
        normalized_field: bool = True,
        normalized_pupil: bool = True,
        image: bool = False,
        wavelength_bins=None,
        launch: None | L.Launch = None,
        outputs: None | Sequence[str] = None,
    ) -> RayFunctionArray:
        """Rays at the last surface in the sensor's local frame
        (optika/systems/_sequential.py:927-988).  ``outputs`` as in
        :meth:`raytrace`."""
        from ._api import OUTPUT_FIELDS, trace_grid

        wl, fld, pup = self._grid(wavelength, field, pupil, normalized_field, normalized_pupil)
        res = trace_grid(
            self, wavelength=wl, field=fld, pupil=pup, intensity=intensity,
            accumulate=False, final_local=True, image=image,
            wavelength_bins=wavelength_bins, launch=launch,
            outputs=OUTPUT_FIELDS if outputs is None else tuple(outputs),
        )
        res.inputs = ObjectVectorArray(wavelength=wl, field=fld, pupil=pup)
        return res
