"""Ray ensembles held on the device as structure-of-arrays float32 tensors.

Mirrors optika/rays/_ray_vectors.py:240-294 (RayVectorArray) with one extra
field, the optical path length ``opl`` (float64, mm), which the reference
does not carry.  Defaults follow the reference: intensity 1, attenuation 0,
index of refraction 1, unvignetted True.
"""

from __future__ import annotations

import dataclasses
from typing import Any

import numpy as np
import torch

from .vectors import Cartesian3dVectorArray

__all__ = ["RayVectorArray", "RayFunctionArray"]


@dataclasses.dataclass
class RayVectorArray:
    wavelength: Any = None  # nm
    position: Cartesian3dVectorArray = dataclasses.field(default_factory=Cartesian3dVectorArray)
    direction: Cartesian3dVectorArray = dataclasses.field(
        default_factory=lambda: Cartesian3dVectorArray(0.0, 0.0, 1.0)
    )
    intensity: Any = 1.0
    attenuation: Any = 0.0  # 1/mm
    index_refraction: Any = 1.0
    unvignetted: Any = True
    opl: Any = 0.0  # mm

    @property
    def n(self):
        """Complex index n + i alpha lambda / (4 pi) (_ray_vectors.py:74-87)."""
        k = self.attenuation * (self.wavelength * 1e-6) / (4 * np.pi)
        return self.index_refraction + 1j * k

    def numpy(self) -> dict[str, np.ndarray]:
        """Host copy of every field as float64 / bool numpy arrays."""

        def h(v):
            if isinstance(v, torch.Tensor):
                return v.detach().cpu().numpy()
            return np.asarray(v)

        return dict(
            wavelength=h(self.wavelength),
            px=h(self.position.x),
            py=h(self.position.y),
            pz=h(self.position.z),
            dx=h(self.direction.x),
            dy=h(self.direction.y),
            dz=h(self.direction.z),
            intensity=h(self.intensity),
            attenuation=h(self.attenuation),
            index_refraction=h(self.index_refraction),
            unvignetted=h(self.unvignetted),
            opl=h(self.opl),
        )

    def __getitem__(self, item) -> "RayVectorArray":
        def g(v):
            return v[item] if isinstance(v, torch.Tensor) and v.ndim > 0 else v

        return RayVectorArray(
            wavelength=g(self.wavelength),
            position=Cartesian3dVectorArray(g(self.position.x), g(self.position.y), g(self.position.z)),
            direction=Cartesian3dVectorArray(
                g(self.direction.x), g(self.direction.y), g(self.direction.z)
            ),
            intensity=g(self.intensity),
            attenuation=g(self.attenuation),
            index_refraction=g(self.index_refraction),
            unvignetted=g(self.unvignetted),
            opl=g(self.opl),
        )


@dataclasses.dataclass
class RayFunctionArray:
    """Inputs (the object grid) and outputs (the traced rays) of a trace
    (optika/rays/_ray_functions.py:25-32).  ``image`` holds the sensor
    counts / flux images when binning was requested."""

    inputs: Any = None
    outputs: RayVectorArray | None = None
    image: Any = None
