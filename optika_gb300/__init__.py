"""optika_gb300: a GB300-native sequential raytracer with optika's API.

The host API (this package) mirrors the classes and call signatures of
optika's hot path; every per-ray computation (traces, sags, rulings,
multilayers, binning, cell sampling, exposure, pupil reductions) runs in
hand-written sm_103a CUDA kernels behind the C-ABI declared in
``include/optika_gb300.h``.  Only small setup work stays on the host: the
descriptor packing, the scene's cell tables and the calibration models'
least-squares fits.  Units:
lengths mm, vacuum wavelengths nm, angles radians (multiply degrees by
:data:`deg`), attenuation 1/mm.
"""

import math

from . import (
    apertures,
    chemicals,
    distortion,
    materials,
    profiles,
    radiometry,
    rays,
    rulings,
    sags,
    sensors,
    surfaces,
    systems,
    transforms,
    vectors,
)
from .materials import multilayer_efficiency

deg = math.pi / 180.0
"""Radians per degree."""

__all__ = [
    "apertures",
    "chemicals",
    "distortion",
    "materials",
    "profiles",
    "radiometry",
    "rays",
    "rulings",
    "sags",
    "sensors",
    "surfaces",
    "systems",
    "transforms",
    "vectors",
    "multilayer_efficiency",
    "deg",
]
