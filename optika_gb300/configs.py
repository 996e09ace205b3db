"""Canonical workloads: the systems and seeded synthetic inputs that the
benchmark and the parity tests run.

* :func:`newtonian` -- parabolic primary (radius -800 mm, conic -1, 50 mm
  clear radius) behind a 12 mm central obscuration, a flat 45 degree fold
  mirror (radius 15 mm) 350 mm in front of it, and a 1024 x 1024 sensor of
  13.5 um pixels at focus (the reference's Newtonian layout,
  optika/systems/_sequential.py:1850-1912, at these dimensions).
* :func:`newtonian_grid` -- the small workload: a 5 x 5 field grid over
  +-0.15 deg, 4000 pupil points per field uniform on the 12-50 mm annulus,
  550 nm (1e5 rays, seed 1).
* :func:`precision_grid` -- the precision workload: the same telescope with
  both mirrors coated by a single aluminium layer (substrate-only Fresnel
  reflection, complex index from a seeded 3-point table at 400/550/700 nm),
  field uniform in the +-0.15 deg square, 400-700 nm (seed 2).

All inputs are synthetic (numpy ``default_rng(seed)``); there is no dataset.
"""

from __future__ import annotations

import math

import numpy as np

from . import apertures, materials, sags, sensors, surfaces, systems, transforms
from .chemicals import Chemical

DEG = math.pi / 180.0
FIELD_HALF = 0.15 * DEG


def aluminium_table(seed: int = 2) -> Chemical:
    """Seeded 3-point complex index table (400, 550, 700 nm) of aluminium-like
    values: n in [0.4, 1.6], k in [4.5, 8.5]."""
    rng = np.random.default_rng(seed)
    wl = np.array([400.0, 550.0, 700.0])
    n = rng.uniform(0.4, 1.6, 3)
    k = rng.uniform(4.5, 8.5, 3)
    return Chemical(wavelength=wl, n=n, k=k, name="Al-synthetic")


def newtonian(coated: bool = False, seed: int = 2) -> systems.SequentialSystem:
    if coated:
        al = materials.Layer(aluminium_table(seed))
        mirror = lambda: materials.MultilayerMirror(layers=None, substrate=al)  # noqa: E731
    else:
        mirror = materials.Mirror
    obscuration = surfaces.Surface(
        name="obscuration",
        aperture=apertures.CircularAperture(12.0, inverted=True),
        transformation=transforms.Translation(z=50.0),
    )
    primary = surfaces.Surface(
        name="primary",
        sag=sags.ConicSag(radius=-800.0, conic=-1.0),
        material=mirror(),
        aperture=apertures.CircularAperture(50.0),
        is_pupil_stop=True,
        transformation=transforms.Translation(z=400.0),
    )
    fold = surfaces.Surface(
        name="fold",
        material=mirror(),
        aperture=apertures.CircularAperture(15.0),
        transformation=transforms.TransformationList(
            [transforms.RotationY(135 * DEG), transforms.Translation(z=50.0)]
        ),
    )
    sensor = sensors.ImagingSensor(
        name="sensor",
        width_pixel=0.0135,
        num_pixel=(1024, 1024),
        transformation=transforms.TransformationList(
            [transforms.RotationY(-90 * DEG), transforms.Translation(x=-50.0, z=50.0)]
        ),
    )
    return systems.SequentialSystem(
        object=surfaces.Surface(name="object"),
        surfaces=[obscuration, primary, fold],
        sensor=sensor,
    )


def annulus(rng, n: int, r0: float = 12.0, r1: float = 50.0):
    r = np.sqrt(rng.uniform(r0 * r0, r1 * r1, n))
    t = rng.uniform(0, 2 * np.pi, n)
    return r * np.cos(t), r * np.sin(t)


def newtonian_grid(num_pupil: int = 4000, seed: int = 1) -> dict:
    """Small workload inputs (float64 numpy), rays ordered field-major."""
    rng = np.random.default_rng(seed)
    f = np.linspace(-FIELD_HALF, FIELD_HALF, 5)
    fx, fy = np.meshgrid(f, f, indexing="ij")
    fx = np.repeat(fx.ravel(), num_pupil)
    fy = np.repeat(fy.ravel(), num_pupil)
    px, py = annulus(rng, fx.size)
    return dict(
        wavelength=np.full(fx.size, 550.0),
        field_x=fx,
        field_y=fy,
        pupil_x=px,
        pupil_y=py,
    )


def precision_grid(n: int, seed: int = 2) -> dict:
    """Precision workload inputs (float64 numpy) of ``n`` rays."""
    rng = np.random.default_rng(seed + 1000)
    fx = rng.uniform(-FIELD_HALF, FIELD_HALF, n)
    fy = rng.uniform(-FIELD_HALF, FIELD_HALF, n)
    px, py = annulus(rng, n)
    wl = rng.uniform(400.0, 700.0, n)
    return dict(wavelength=wl, field_x=fx, field_y=fy, pupil_x=px, pupil_y=py)
