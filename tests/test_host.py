"""Host-side logic: descriptor lowering, transform composition, errors for
unsupported plugins, sharding, and the multi-process (gloo) image reduction."""

import math
import os

import numpy as np
import pytest
import torch

import optika_gb300 as ok
from optika_gb300 import _lib as L
from optika_gb300 import configs, distributed
from optika_gb300._lower import Lowering, lower_surfaces, split_f64
from oracle import trace as O


def _affine(a: L.Affine) -> np.ndarray:
    m = np.eye(4)
    m[:3, :3] = np.array(a.m[:]).reshape(3, 3)
    m[:3, 3] = np.array(a.t_hi[:], dtype=np.float64) + np.array(a.t_lo[:], dtype=np.float64)
    return m


def test_split_f64_is_exact_to_float_float():
    for v in [0.0, 350.0, -1234.56789, 1e-3, math.pi * 1000]:
        hi, lo = split_f64(v)
        assert np.float32(hi) == hi and np.float32(lo) == lo
        assert abs((hi + lo) - v) <= 1e-13 * max(1.0, abs(v))


def test_frame_chain_composes_to_sensor_frame():
    s = configs.newtonian()
    surfaces = s.surfaces_all
    lw = lower_surfaces(surfaces, pre=np.eye(4), final=None, input_mode=L.INPUT_GRID_INFINITY)
    chain = np.eye(4)
    for k in range(len(surfaces)):
        chain = _affine(lw.sys.surfaces[k].to_local) @ chain
    expect = O._inv(O._mat(s.sensor.transformation))
    assert np.allclose(chain, expect, atol=1e-5)
    for k, surf in enumerate(surfaces):
        assert np.allclose(_affine(lw.sys.surfaces[k].to_output), O._mat(surf.transformation),
                           atol=1e-5)


def test_lowering_types_and_pools():
    sysm = configs.newtonian(coated=True)
    lw = lower_surfaces(sysm.surfaces_all, pre=np.eye(4), final=np.eye(4),
                        input_mode=L.INPUT_GRID_INFINITY, sensor=sysm.sensor)
    S = lw.sys
    kinds = [S.surfaces[k].sag_type for k in range(5)]
    assert kinds == [L.SAG_FLAT, L.SAG_FLAT, L.SAG_CONIC, L.SAG_FLAT, L.SAG_FLAT]
    assert S.surfaces[2].mat_type == L.MAT_MULTILAYER_MIRROR
    assert S.surfaces[1].aper_flags & L.APER_FLAG_INVERTED
    assert S.surfaces[4].aper_type == L.APER_RECTANGULAR
    assert S.surfaces[4].is_sensor == 1
    assert S.sensor.num_x == 1024 and abs(S.sensor.lo_x + 6.912) < 1e-6
    assert S.flags & L.SYS_FLAG_FINAL_IDENTITY
    assert len(lw.table_list) == 1  # one Al table shared by both mirrors


def test_periodic_stack_lowering():
    lw = Lowering()
    A = ok.materials.Layer(0.9 + 0.01j, 4.0)
    B = ok.materials.Layer(0.99 + 0.001j, 6.0)
    cap = ok.materials.Layer(0.95 + 0.02j, 2.0)
    k = lw.add_stack([cap, ok.materials.PeriodicLayerSequence([A, B], 40)],
                     ok.materials.Layer(0.9 + 0.1j))
    K = lw.sys.stacks[k]
    assert (K.pre_count, K.per_count, K.num_periods, K.post_count) == (1, 2, 40, 0)
    assert K.substrate == 3 and lw.sys.layers[K.substrate].thickness == 0.0


@pytest.mark.parametrize(
    "surface",
    [
        ok.surfaces.Surface(sag=ok.sags.SphericalSag(100.0, transformation=ok.transforms.Translation(z=1.0))),
        ok.surfaces.Surface(material=ok.materials.MultilayerMirror(
            layers=[ok.materials.Layer("Si", 5.0)])),
        ok.surfaces.Surface(material=ok.materials.MultilayerMirror(
            layers=[ok.materials.Layer(1.0 + 0j, 5.0, interface=object())])),
        ok.surfaces.Surface(material=object()),
        ok.surfaces.Surface(aperture=object()),
    ],
)
def test_unsupported_plugins_raise(surface):
    with pytest.raises((NotImplementedError, AttributeError)):
        lower_surfaces([surface], pre=np.eye(4), final=None, input_mode=L.INPUT_RAYS)


def test_polynomial_power_limit():
    r = ok.rulings.Rulings(spacing=ok.rulings.Polynomial1dRulingSpacing({9: 1.0}), diffraction_order=1)
    with pytest.raises(ValueError):
        lower_surfaces([ok.surfaces.Surface(rulings=r)], pre=np.eye(4), final=None,
                       input_mode=L.INPUT_RAYS)


def test_normalized_coordinates_need_stops():
    """Normalised coordinates (the default) need a field and a pupil stop;
    without them the stop solver refuses before any device work."""
    s = configs.newtonian()
    with pytest.raises(ValueError, match="not defined"):
        s.raytrace()


def test_rayfunction_default_is_cached_and_needs_stops():
    s = configs.newtonian()
    with pytest.raises(ValueError, match="not defined"):
        s.rayfunction_default
    assert "rayfunction_default" not in s.__dict__  # nothing cached after a failure


def test_configs_are_seeded():
    a = configs.precision_grid(1000)
    b = configs.precision_grid(1000)
    for k in a:
        assert np.array_equal(a[k], b[k])
    g = configs.newtonian_grid()
    assert g["field_x"].size == 100_000


def test_shard_covers_range():
    for n in [0, 1, 7, 100, 101]:
        for world in [1, 2, 3, 8]:
            idx = np.concatenate([np.arange(n)[distributed.shard(n, r, world)] for r in range(world)])
            assert np.array_equal(idx, np.arange(n))


def _gloo_worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s = configs.newtonian()
    g = configs.newtonian_grid(num_pupil=200)
    sl = distributed.shard(g["field_x"].size, rank, world)
    r = O.rayfunction(s, *(g[k][sl] for k in ("wavelength", "field_x", "field_y", "pupil_x",
                                                 "pupil_y")))
    counts, flux = O.collect(s.sensor, r)
    c = torch.from_numpy(counts.astype(np.int64))
    f = torch.from_numpy(flux)
    distributed.reduce_image(c, f)
    if rank == 0:
        q.put((c.numpy(), f.numpy()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_image_reduction_equals_single_process():
    import multiprocessing as mp
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_gloo_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    c, f = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    s = configs.newtonian()
    g = configs.newtonian_grid(num_pupil=200)
    r = O.rayfunction(s, g["wavelength"], g["field_x"], g["field_y"], g["pupil_x"], g["pupil_y"])
    c1, f1 = O.collect(s.sensor, r)
    assert np.array_equal(c, c1)
    assert np.allclose(f, f1)


def test_affine_flags_select_the_device_frame_change():
    """The lowering flags the frames the device changes by a cheaper form:
    the identity rotation (plus the identity map when the translation is 0)
    and rotations about y, which mix x and z only; any other rotation takes
    the full 3 x 3 form.  Values are split exactly into hi + lo pairs."""
    from optika_gb300 import _lib as L
    from optika_gb300._lower import set_affine

    def flags(m):
        a = L.Affine()
        set_affine(a, m)
        return a.flags, a

    m = np.eye(4)
    assert flags(m)[0] == L.AFFINE_ROT_IDENTITY | L.AFFINE_IDENTITY
    m[:3, 3] = [0.0, 0.0, 123.456]
    f, a = flags(m)
    assert f == L.AFFINE_ROT_IDENTITY
    assert float(np.float32(a.t_hi[2])) + float(a.t_lo[2]) == pytest.approx(123.456, abs=1e-12)
    c, s = np.cos(0.3), np.sin(0.3)
    ry = np.eye(4)
    ry[0, 0], ry[0, 2], ry[2, 0], ry[2, 2] = c, s, -s, c
    assert flags(ry)[0] == L.AFFINE_ROT_Y
    rx = np.eye(4)
    rx[1, 1], rx[1, 2], rx[2, 1], rx[2, 2] = c, -s, s, c
    assert flags(rx)[0] == 0
    # the hi + lo split of every entry reproduces the float64 value to ~2^-48
    f, a = flags(ry)
    for i in range(9):
        assert abs(float(a.m[i]) + float(a.m_lo[i]) - ry[:3, :3].flat[i]) < 1e-14
