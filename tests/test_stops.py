"""The stop solver: aperture wires, the anchor rule, the float64 oracle
pinned to the reference's known answers, and the GPU solver (trace kernel
per Newton iteration) against the oracle on the reference's two stop
systems.

Tolerances: field extents within 2e-8 rad (1e-6 deg, the reference's own
bound on its known answers), pupil extents within 2e-6 of their size
(FP32 trace against float64)."""

import math

import numpy as np
import pytest

import optika_gb300 as ok
from optika_gb300 import configs
from oracle import stops as OS

DEG = math.pi / 180


def test_circular_wire_closes_on_itself():
    w = ok.apertures.CircularAperture(10.0).wire(21)
    assert w.shape == (21, 3)
    assert np.allclose(w[0], w[-1]) and np.allclose(np.hypot(w[:, 0], w[:, 1]), 10.0)


def test_polygon_wire_follows_the_sides():
    w = ok.apertures.RectangularAperture(half_width=(60.0, 30.0)).wire(21)
    assert w.shape == (21, 3)
    # 5, 5, 5, 6 points per side, the last side ending on the first vertex
    assert np.allclose(w[0, :2], [60, 30]) and np.allclose(w[5, :2], [-60, 30])
    assert np.allclose(w[10, :2], [-60, -30]) and np.allclose(w[15, :2], [60, -30])
    assert np.allclose(w[-1, :2], [60, 30])
    on_edge = np.isclose(np.abs(w[:, 0]), 60) | np.isclose(np.abs(w[:, 1]), 30)
    assert on_edge.all()


def test_sector_and_transformed_wires():
    s = ok.apertures.CircularSectorAperture(radius=5.0, angle_start=0.2, angle_stop=1.2).wire(30)
    r = np.hypot(s[:, 0], s[:, 1])
    assert s.shape == (30, 3) and r.max() <= 5.0 + 1e-12 and np.isclose(r.min(), 0.0)
    t = ok.apertures.CircularAperture(
        2.0, transformation=ok.transforms.Translation(x=3.0, y=-1.0)).wire(9)
    assert np.allclose(np.hypot(t[:, 0] - 3.0, t[:, 1] + 1.0), 2.0)


def test_anchor_rule():
    # optika/systems/_sequential_test.py:512-533, re-expressed
    S = ok.surfaces.Surface
    first, last = S(name="first"), S(name="last")
    mirror = S(name="mirror", material=ok.materials.Mirror())
    curved = S(name="curved", sag=ok.sags.SphericalSag(-100.0))
    grating = S(name="grating", rulings=ok.rulings.Rulings(spacing=1e-3, diffraction_order=1))
    flat = S(name="flat")
    a = OS.anchor_surface
    from optika_gb300.stops import anchor_surface as b

    for f in (a, b):
        assert f([first, flat, mirror, last]) is mirror
        assert f([first, curved, last]) is curved
        assert f([first, grating, last]) is grating
        assert f([first, flat, last]) is last


@pytest.mark.parametrize("make,radius", [(configs.stop_newtonian, configs.STOP_NEWTONIAN_FIELD),
                                         (configs.stop_grazing, configs.STOP_GRAZING_FIELD)])
def test_oracle_known_answers(make, radius):
    """The reference's own known answers: field_max equals the source's
    angular aperture to 1e-6 deg (optika/systems/_sequential_test.py:591-597,
    665-671); the field and pupil are symmetric."""
    fmin, fmax, pmin, pmax = OS.extents(make(), 500.0)
    assert abs(fmax[0] - radius) < 1e-6 * DEG and abs(fmax[1] - radius) < 1e-6 * DEG
    assert abs(fmin[0] + radius) < 1e-6 * DEG and abs(fmin[1] + radius) < 1e-6 * DEG
    assert np.allclose(pmin, [-pmax[0], -pmax[1]], rtol=1e-9)


def test_oracle_stop_rays_hit_the_stop_edges():
    """The solved rays strike the pupil stop's wire points."""
    from oracle import trace as O

    s = configs.stop_newtonian()
    st = OS.stops_only(s, 500.0)
    p, d = st["position"], st["direction"]
    rays = O.make_rays(p.shape[1:], px=p[0], py=p[1], pz=p[2], dx=d[0], dy=d[1], dz=d[2],
                       wavelength=500.0)
    surf = s.surfaces_all
    r = O.apply(O._inv(O._mat(surf[2].transformation)), O.propagate_rays(surf[1:3], rays))
    w = surf[2].aperture.wire(21)
    assert np.abs(r["px"] - w[None, :, 0]).max() < 1e-8
    assert np.abs(r["py"] - w[None, :, 1]).max() < 1e-8


# --------------------------------------------------------------------------- GPU


@pytest.mark.gpu
@pytest.mark.parametrize("make", [configs.stop_newtonian, configs.stop_grazing])
def test_gpu_stop_extents_match_oracle(cuda, make):
    from optika_gb300.stops import extents

    s = make()
    got = extents(s, 500.0)
    ref = OS.extents(make(), 500.0)
    for (gx, gy), (rx, ry) in zip(got[:2], ref[:2]):
        assert abs(gx - rx) < 2e-8 and abs(gy - ry) < 2e-8
    size = max(ref[3][0] - ref[2][0], ref[3][1] - ref[2][1])
    for (gx, gy), (rx, ry) in zip(got[2:], ref[2:]):
        assert abs(gx - rx) < 2e-6 * size and abs(gy - ry) < 2e-6 * size, (got, ref)


@pytest.mark.gpu
def test_gpu_normalized_raytrace(cuda):
    """rayfunction with normalised coordinates equals rayfunction with the
    physical coordinates the oracle's extents give."""
    import torch

    s = configs.stop_newtonian()
    V2 = ok.vectors.Cartesian2dVectorArray
    u = np.linspace(-1, 1, 5)
    fx, fy, qx, qy = (a.ravel() for a in np.meshgrid(u, u, u, u, indexing="ij"))
    a = s.rayfunction(wavelength=500.0, field=V2(fx, fy), pupil=V2(qx, qy))
    (pfx, pfy), (pqx, pqy) = OS.denormalize(configs.stop_newtonian(), 500.0, (fx, fy), (qx, qy))
    b = s.rayfunction(wavelength=500.0, field=V2(pfx, pfy), pupil=V2(pqx, pqy),
                      normalized_field=False, normalized_pupil=False)
    torch.cuda.synchronize()
    oa, ob = a.outputs.numpy(), b.outputs.numpy()
    # normalised pupil coordinates of +-1 put a ray on the stop's edge by
    # construction (the solved extents are where rays graze it): the two
    # sides' extents differ by FP32 rounding, so only rays strictly inside
    # have a defined mask; every ray unvignetted on both sides must land alike
    inside = (np.abs(qx) < 1) & (np.abs(qy) < 1)
    assert np.array_equal(oa["unvignetted"][inside], ob["unvignetted"][inside])
    m = ob["unvignetted"] & oa["unvignetted"]
    assert np.abs(oa["px"][m] - ob["px"][m]).max() < 1e-4
    assert np.abs(oa["py"][m] - ob["py"][m]).max() < 1e-4
    # the pupil corners reach the stop's edge: some rays are vignetted, not all
    assert 0 < m.sum() < m.size


@pytest.mark.gpu
def test_gpu_stop_solve_reports_rays_that_do_not_converge(cuda, monkeypatch):
    """A solve whose rays stop short of the tolerance (here: one Newton
    iteration allowed) raises, through the public calls and through the
    batched extents, whose single read of the results carries the flag."""
    from optika_gb300 import stops

    monkeypatch.setattr(stops, "MAX_ITER", 1)
    for call in (lambda s: stops.rayfunction_stops(s, 500.0),
                 lambda s: stops.stops_only(s, 500.0),
                 lambda s: stops.extents_many(s, [500.0, 550.0])):
        with pytest.raises(ValueError, match="could not solve"):
            call(configs.stop_grazing())
    # the full iteration count solves the same system
    monkeypatch.setattr(stops, "MAX_ITER", 60)
    assert len(stops.extents_many(configs.stop_grazing(), [500.0, 550.0])) == 2
