"""Batched spectrograph trace: Philox generation pinned by the Random123
known-answer vectors, per-configuration parity with the float64 oracle,
the fixed-shape and generic kernels agreeing, the autotuner and a CUDA
graph replay."""

import math

import numpy as np
import pytest

from oracle import batch as OB
from oracle import trace as O


@pytest.mark.parametrize(
    "counter,key,expected",
    [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ],
)
def test_philox_known_answers(counter, key, expected):
    out = OB.philox4x32_10(*[np.uint64(c) for c in counter], key[0], key[1])
    assert tuple(int(v) for v in out) == expected


def test_batch_inputs_ranges():
    g = OB.batch_inputs(seed=3, config=7, n=10000, wl_lo=58.0, wl_hi=63.0, fxh=1e-3, fyh=2e-3,
                        pupil_half=40.0)
    assert g["wavelength"].dtype == np.float32
    assert 58.0 <= g["wavelength"].min() and g["wavelength"].max() < 63.0
    assert np.abs(g["pupil_x"]).max() <= 40.0 and np.abs(g["field_y"]).max() <= 2e-3
    # configs draw independent streams
    h = OB.batch_inputs(seed=3, config=8, n=10000, wl_lo=58.0, wl_hi=63.0, fxh=1e-3, fyh=2e-3,
                        pupil_half=40.0)
    assert not np.array_equal(g["pupil_x"], h["pupil_x"])


def test_spectrograph_oracle_focus():
    from optika_gb300 import configs

    s = configs.spectrograph()
    g = OB.batch_inputs(seed=1, config=0, n=3000, wl_lo=60.5, wl_hi=60.5, fxh=0.0, fyh=0.0,
                        pupil_half=40.0)
    r = O.rayfunction(s, *(g[k].astype(np.float64) for k in ("wavelength", "field_x", "field_y",
                                                             "pupil_x", "pupil_y")))
    m = r["unvignetted"]
    assert 0.7 < m.mean() < 0.85  # the square pupil overfills the 40 mm primary
    assert abs(r["px"][m].mean()) < 0.05 and abs(r["py"][m].mean()) < 0.05
    assert r["px"][m].std() < 0.1


def _batch(num_configs=12, seed=3, image=False):
    from optika_gb300 import batch, configs

    systems, counts, params = configs.spectrograph_batch(num_configs, seed=seed, min_rays=500,
                                                          max_rays=4000)
    bt = batch.BatchedTrace(
        systems, overrides=[2, 3], ray_counts=counts, seed=seed,
        wavelength=configs.SPEC_WAVELENGTH, field_half=configs.SPEC_FIELD_HALF,
        pupil_half=configs.SPEC_PUPIL_HALF, image=image, tile_size=1024,
        outputs=("px", "py", "dx", "dy", "dz", "unvignetted", "opl"))
    return bt, systems, counts


@pytest.mark.gpu
def test_batch_matches_oracle_per_config(cuda):
    import torch
    from optika_gb300 import configs

    bt, systems, counts = _batch(image=True)
    bt.run()
    torch.cuda.synchronize()
    out = {k: v.cpu().numpy() for k, v in bt.bufs.items() if v is not None}
    images = bt.images.cpu().numpy()
    for c, s in enumerate(systems):
        sl = bt.config_slice(c)
        g = OB.batch_inputs(bt.seed, c, int(counts[c]), *configs.SPEC_WAVELENGTH,
                            *configs.SPEC_FIELD_HALF, configs.SPEC_PUPIL_HALF)
        ref = O.rayfunction(s, *(g[k].astype(np.float64) for k in (
            "wavelength", "field_x", "field_y", "pupil_x", "pupil_y")))
        m = ref["unvignetted"]
        assert np.array_equal(out["unvignetted"][sl].astype(bool), m)
        e = np.hypot(out["px"][sl][m] - ref["px"][m], out["py"][sl][m] - ref["py"][m])
        assert e.max() < 1.5e-4, (c, e.max())
        for k in ("dx", "dy", "dz"):
            assert np.abs(out[k][sl][m] - ref[k][m]).max() < 3e-6
        assert np.abs(out["opl"][sl][m] - ref["opl"][m]).max() < 1e-3
        c_ref, _ = O.collect(s.sensor, ref)
        assert abs(int(images[c].sum()) - int(c_ref.sum())) <= max(2, int(1e-3 * m.sum()))


@pytest.mark.gpu
def test_batch_fixed_equals_generic_and_graph(cuda):
    import torch

    bt, _, _ = _batch(num_configs=8, seed=5)
    bt.run()
    torch.cuda.synchronize()
    a = {k: v.clone() for k, v in bt.bufs.items() if v is not None}
    bt.launch.generic_only = 1
    bt.run()
    torch.cuda.synchronize()
    # the two kernels are compiled differently (FMA contraction may differ
    # in the last bit): equal masks away from edges, positions to 1e-5 mm
    m = a["unvignetted"].bool() & bt.bufs["unvignetted"].bool()
    assert (a["unvignetted"] != bt.bufs["unvignetted"]).float().mean().item() < 1e-3
    for k in ("px", "py"):
        assert torch.allclose(a[k][m], bt.bufs[k][m], atol=1e-5, rtol=0), k
    bt.launch.generic_only = 0
    choice = bt.tune(candidates=((256, 1), (1024, 2)), repeats=1)
    assert choice in ((256, 1), (1024, 2))
    for v in bt.bufs.values():
        if v is not None:
            v.zero_()
    g = bt.graph()
    g.replay()
    torch.cuda.synchronize()
    for k in a:
        assert torch.equal(a[k], bt.bufs[k]), k
