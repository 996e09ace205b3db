"""Sequential optical systems, mirroring optika/systems/_sequential.py.

:meth:`SequentialSystem.raytrace` and :meth:`SequentialSystem.rayfunction`
build the input rays from a (wavelength, field, pupil) grid and trace them
through ``[object] + surfaces + [sensor]`` in one fused GPU launch
(optika/systems/_sequential.py:791-988).  Normalised field and pupil
coordinates (the default, as in the reference) are mapped to physical ones
through the extents of the field and pupil stops, which the stop solver
(:mod:`optika_gb300.stops`) finds on the GPU (:396-850).
"""

from __future__ import annotations

import dataclasses
import functools
from typing import Sequence

import numpy as np

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

    # ---- stops (optika/systems/_sequential.py:262-341, 755-799)

    @property
    def index_field_stop(self) -> int:
        idx = [i for i, s in enumerate(self.surfaces_all) if s.is_field_stop]
        if not idx:
            raise ValueError("field stop is not defined for this system; set "
                             "`is_field_stop=True` for at least one surface")
        return idx[-1]

    @property
    def index_pupil_stop(self) -> int:
        idx = [i for i, s in enumerate(self.surfaces_all) if s.is_pupil_stop]
        if not idx:
            raise ValueError("pupil stop is not defined for this system; set "
                             "`is_pupil_stop=True` for at least one surface")
        return idx[-1]

    @property
    def field_stop(self) -> AbstractSurface:
        return self.surfaces_all[self.index_field_stop]

    @property
    def pupil_stop(self) -> AbstractSurface:
        return self.surfaces_all[self.index_pupil_stop]

    def _wavelength_input(self) -> float:
        g = self.grid_input if self.grid_input is not None else ObjectVectorArray()
        w = np.unique(np.asarray(g.wavelength, dtype=np.float64))
        if len(w) != 1:
            raise ValueError("field_min/max and pupil_min/max need a single input wavelength")
        return float(w[0])

    def rayfunction_stops(self, wavelength: None | float = None) -> dict:
        """Rays from the object that strike the edges of both stops, with
        the field and pupil grids they give (torch tensors [first stop
        wire, last stop wire], 21 x 21)."""
        from .stops import rayfunction_stops

        w = self._wavelength_input() if wavelength is None else float(wavelength)
        return rayfunction_stops(self, w)

    @property
    def field_min(self) -> tuple[float, float]:
        """Lower corner of the field of view (rad at infinity, else mm)."""
        from .stops import extents

        return extents(self, self._wavelength_input())[0]

    @property
    def field_max(self) -> tuple[float, float]:
        from .stops import extents

        return extents(self, self._wavelength_input())[1]

    @property
    def pupil_min(self) -> tuple[float, float]:
        """Lower corner of the entrance pupil (mm at infinity, else rad)."""
        from .stops import extents

        return extents(self, self._wavelength_input())[2]

    @property
    def pupil_max(self) -> tuple[float, float]:
        from .stops import extents

        return extents(self, self._wavelength_input())[3]

    def _grid(self, wavelength, field, pupil, normalized_field, normalized_pupil):
        g = self.grid_input if self.grid_input is not None else ObjectVectorArray()
        wl = g.wavelength if wavelength is None else wavelength
        fld = g.field if field is None else field
        pup = g.pupil if pupil is None else pupil
        if normalized_field or normalized_pupil:
            from .stops import denormalize
            from .vectors import Cartesian2dVectorArray

            (fx, fy), (qx, qy) = denormalize(self, wl, (fld.x, fld.y), (pup.x, pup.y),
                                             normalized_field, normalized_pupil)
            fld = Cartesian2dVectorArray(fx, fy)
            pup = Cartesian2dVectorArray(qx, qy)
        return wl, fld, pup

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

    @functools.cached_property
    def rayfunction_default(self) -> RayFunctionArray:
        """:meth:`rayfunction` of :attr:`grid_input`, cached
        (optika/systems/_sequential.py:990-1000); ``del
        system.rayfunction_default`` recomputes it."""
        return self.rayfunction()

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

    def image(
        self,
        scene,
        pupil=None,
        normalized_field: bool = True,
        normalized_pupil: bool = True,
        integrate: bool = True,
        noise: bool = True,
        random: bool = True,
        seed: int = 0,
        timedelta=None,
        chunk: int = 1 << 24,
    ):
        """Forward model: detector electrons of a scene of spectral radiance
        given on cell vertices (optika/systems/_sequential.py:1088-1206).

        ``scene`` is a :class:`~optika_gb300.vectors.FunctionArray` whose
        inputs are a :class:`~optika_gb300.vectors.SpectralPositionalVectorArray`
        of wavelength vertices (nm) and field vertices (a
        ``Cartesian2dVectorArray`` of 1-D x and y vertices) and whose outputs
        are the radiance of each cell ``[nw, nfx, nfy]``; ``pupil`` holds
        pupil vertices (default one normalised cell ``[-1, 1]^2``).  The
        reference decides from units whether coordinates are normalised;
        here ``normalized_field`` / ``normalized_pupil`` say so.  Returns a
        ``FunctionArray`` of wavelength bin edges and pixel edges to
        electrons ``[num_w, num_pixel_x, num_pixel_y]`` (one wavelength bin
        when ``integrate``).  See :mod:`optika_gb300.imaging`."""
        from .imaging import image

        return image(self, scene, pupil=pupil, normalized_field=normalized_field,
                     normalized_pupil=normalized_pupil, integrate=integrate, noise=noise,
                     random=random, seed=seed, timedelta=timedelta, chunk=chunk)

    # ---- calibration fits (optika/systems/_sequential.py:1208-1512)

    def distortion(self, wavelength=None, field=None, pupil=None, normalized_field: bool = True,
                   normalized_pupil: bool = True, degree: int = 2):
        """Polynomial distortion model fitted to traced rays; grids are 1-D
        arrays per coordinate (see :mod:`optika_gb300.calibration`)."""
        from .calibration import distortion

        return distortion(self, wavelength, field, pupil, normalized_field, normalized_pupil,
                          degree)

    def vignetting(self, wavelength=None, field=None, pupil=None, normalized_field: bool = True,
                   normalized_pupil: bool = True, degree: int = 2):
        """Polynomial vignetting model fitted to traced rays."""
        from .calibration import vignetting

        return vignetting(self, wavelength, field, pupil, normalized_field, normalized_pupil,
                          degree)

    def area_effective(self, wavelength=None, field=None, pupil=None,
                       normalized_field: bool = True, normalized_pupil: bool = True,
                       random: bool = True, seed: int = 0):
        """Effective area versus wavelength from traced rays (pupil given on
        cell vertices)."""
        from .calibration import area_effective

        return area_effective(self, wavelength, field, pupil, normalized_field,
                              normalized_pupil, random, seed)
