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


# ---------------------------------------------------------------- spectrograph

# Geometry of the batched EUV imaging spectrograph, fixed once: a spherical
# primary (R -1600 mm, 40 mm aperture) at z = 1000 mm focuses the beam back
# towards -z; a toroidal VLS grating 600 mm in front of it (concave to the
# returning beam: minor radius 1150 mm, radius of rotation 1200 mm in its
# own frame, light arriving along -z) re-images the spectrum onto a
# 2048 x 1024 sensor of 13.5 um pixels at the grating's first-order focus
# for 60.5 nm and 2400 lines/mm (147.5 mm along the 8.378 deg diffracted
# chief ray, found with the float64 oracle).  The reference's toroid places
# its vertex at the origin only for a non-negative radius of rotation
# (z = r - sqrt((r - z_y)^2 - x^2)), hence the positive radii facing the
# returning beam.
SPEC_PRIMARY_Z = 1000.0
SPEC_GRATING_Z = 400.0
SPEC_SENSOR_X = 21.4613817
SPEC_SENSOR_Z = 545.943704
SPEC_SENSOR_ANGLE = 8.377987233014737 * DEG
SPEC_FIELD_HALF = (0.01 * DEG, 0.05 * DEG)
SPEC_PUPIL_HALF = 40.0
SPEC_WAVELENGTH = (58.0, 63.0)


def spectrograph(d0: float = 1 / 2400, a1: float = 0.0, a2: float = 0.0,
                 tilt: float = 0.0) -> systems.SequentialSystem:
    """One configuration: ruling spacing d(x) = d0 (1 + a1 x + a2 x^2) (mm)
    along x, grating tilt (rad) about y, diffraction order +1."""
    from . import rulings

    primary = surfaces.Surface(
        name="primary",
        sag=sags.SphericalSag(-1600.0),
        material=materials.Mirror(),
        aperture=apertures.CircularAperture(40.0),
        is_pupil_stop=True,
        transformation=transforms.Translation(z=SPEC_PRIMARY_Z),
    )
    grating = surfaces.Surface(
        name="grating",
        sag=sags.ToroidalSag(radius=1150.0, radius_of_rotation=1200.0),
        material=materials.Mirror(),
        rulings=rulings.Rulings(
            spacing=rulings.Polynomial1dRulingSpacing(
                {0: d0, 1: d0 * a1, 2: d0 * a2}, normal=(1.0, 0.0, 0.0)
            ),
            diffraction_order=1,
        ),
        transformation=transforms.TransformationList(
            [transforms.RotationY(tilt), transforms.Translation(z=SPEC_GRATING_Z)]
        ),
    )
    sensor = sensors.ImagingSensor(
        name="sensor",
        width_pixel=0.0135,
        num_pixel=(2048, 1024),
        transformation=transforms.TransformationList(
            [transforms.RotationY(SPEC_SENSOR_ANGLE),
             transforms.Translation(x=SPEC_SENSOR_X, z=SPEC_SENSOR_Z)]
        ),
    )
    return systems.SequentialSystem(
        object=surfaces.Surface(name="object"), surfaces=[primary, grating], sensor=sensor
    )


def spectrograph_batch(num_configs: int = 4096, seed: int = 3, min_rays: int = 1000,
                       max_rays: int = 1_000_000) -> tuple[list, np.ndarray, np.ndarray]:
    """Seeded configurations: 1/d0 ~ U(2200, 2600) lines/mm, a1 ~ N(0, 1e-4),
    a2 ~ N(0, 1e-7), tilt ~ U(-2, 2) deg; ray counts log-uniform in
    [min_rays, max_rays].  Returns (systems, ray counts, parameters[c, 4])."""
    rng = np.random.default_rng(seed)
    d0 = 1.0 / rng.uniform(2200.0, 2600.0, num_configs)
    a1 = rng.normal(0.0, 1e-4, num_configs)
    a2 = rng.normal(0.0, 1e-7, num_configs)
    tilt = rng.uniform(-2.0, 2.0, num_configs) * DEG
    counts = np.floor(10 ** rng.uniform(np.log10(min_rays), np.log10(max_rays), num_configs))
    params = np.stack([d0, a1, a2, tilt], axis=-1)
    systems_ = [spectrograph(*p) for p in params]
    return systems_, counts.astype(np.int64), params


# -------------------------------------------------- systems with stops
# The two stop-solver systems of the reference's tests
# (optika/systems/_sequential_test.py:536-575 and 599-646), in mm and rad.

STOP_NEWTONIAN_FIELD = 0.05 * DEG
STOP_GRAZING_FIELD = 0.25 * DEG


def stop_newtonian() -> systems.SequentialSystem:
    """Spherical primary (R -2000 mm, r 50 mm) at z = 500 mm, the pupil stop
    (r 10 mm) downstream at z = 250 mm, the sensor (128^2 x 15 um) at
    z = -500 mm; the object is the field stop, an angular aperture of
    radius sin(0.05 deg)."""
    obj = surfaces.Surface(
        name="source",
        aperture=apertures.CircularAperture(math.sin(STOP_NEWTONIAN_FIELD), dimensionless=True),
        is_field_stop=True,
    )
    primary = surfaces.Surface(
        name="primary", sag=sags.SphericalSag(-2000.0), material=materials.Mirror(),
        aperture=apertures.CircularAperture(50.0),
        transformation=transforms.Translation(z=500.0),
    )
    stop = surfaces.Surface(
        name="aperture", aperture=apertures.CircularAperture(10.0), is_pupil_stop=True,
        transformation=transforms.Translation(z=250.0),
    )
    sensor = sensors.ImagingSensor(
        name="sensor", width_pixel=0.015, num_pixel=(128, 128),
        transformation=transforms.Translation(z=-500.0),
    )
    return systems.SequentialSystem(object=obj, surfaces=[primary, stop], sensor=sensor)


def stop_grazing() -> systems.SequentialSystem:
    """Parabolic primary (f -2000 mm, r 260 mm, the pupil stop) at
    z = 2500 mm, a transmission grating (10 um spacing, order +1, 60 mm
    square) at z = 1000 mm, the sensor (2048 x 1024 x 15 um) at x = 26,
    z = 480 mm; the object is the field stop, an angular aperture of radius
    sin(0.25 deg)."""
    from . import rulings

    obj = surfaces.Surface(
        name="source",
        aperture=apertures.CircularAperture(math.sin(STOP_GRAZING_FIELD), dimensionless=True),
        is_field_stop=True,
    )
    primary = surfaces.Surface(
        name="paraboloid", sag=sags.ParabolicSag(focal_length=-2000.0),
        material=materials.Mirror(), aperture=apertures.CircularAperture(260.0),
        is_pupil_stop=True, transformation=transforms.Translation(z=2500.0),
    )
    grating = surfaces.Surface(
        name="grating", rulings=rulings.Rulings(spacing=0.010, diffraction_order=1),
        aperture=apertures.RectangularAperture(half_width=60.0),
        transformation=transforms.Translation(z=1000.0),
    )
    sensor = sensors.ImagingSensor(
        name="sensor", width_pixel=0.015, num_pixel=(2048, 1024),
        transformation=transforms.Translation(x=26.0, z=480.0),
    )
    return systems.SequentialSystem(object=obj, surfaces=[primary, grating], sensor=sensor)
