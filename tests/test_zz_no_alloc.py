"""The allocation-free batched trace (otx_trace_batch_noalloc).

Some callers cannot allocate GPU memory where they call the library: a host
application that embeds it and owns all device memory through its own
allocator, or code that must not allocate because allocation synchronises
the device.  They pass only inputs and outputs; the work counter and tile
list live in a device array of the library.  This test calls that entry
point through the C-ABI twice in a row and checks both results against the
regular entry point's (which takes caller-allocated scratch), within the
tolerances of the batch parity tests.  It runs last so that a failure here
leaves every other test already run.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _outputs(bt, torch):
    n = bt.total
    dev = bt.ray_offset.device
    bufs = {
        "px": torch.empty(n, dtype=torch.float32, device=dev),
        "py": torch.empty(n, dtype=torch.float32, device=dev),
        "unvignetted": torch.empty(n, dtype=torch.uint8, device=dev),
    }
    from optika_gb300._api import _rays_struct

    return bufs, _rays_struct(bufs, n)


def test_noalloc_batch_matches_regular_entry(cuda):
    import torch

    from optika_gb300 import _lib as L
    from optika_gb300 import batch, configs
    from optika_gb300._api import stream_handle

    systems, counts, _ = configs.spectrograph_batch(16, seed=11, min_rays=300, max_rays=5000)
    bt = batch.BatchedTrace(
        systems, overrides=[2, 3], ray_counts=counts, seed=11,
        wavelength=configs.SPEC_WAVELENGTH, field_half=configs.SPEC_FIELD_HALF,
        pupil_half=configs.SPEC_PUPIL_HALF, image=True, tile_size=512,
        outputs=("px", "py", "unvignetted"))
    lib = L.load()
    # regular entry point: caller-allocated counter and tile list
    bt.run()
    torch.cuda.synchronize()
    ref = {k: v.clone() for k, v in bt.bufs.items() if v is not None}
    ref_img = bt.images.clone()
    assert ref_img.sum().item() > 0

    # the same batch through the allocation-free entry point, twice in a row
    b = L.Batch()
    ctypes.memmove(ctypes.byref(b), ctypes.byref(bt.batch), ctypes.sizeof(L.Batch))
    b.tiles = 0
    b.counter = 0
    for _ in range(2):
        bufs, out = _outputs(bt, torch)
        images = torch.zeros_like(bt.images)
        img = L.Image()
        img.counts = images.data_ptr()
        st = lib.otx_trace_batch_noalloc(ctypes.byref(bt.lowering.sys), ctypes.byref(b),
                                         ctypes.byref(out), ctypes.byref(img),
                                         ctypes.byref(bt.launch), stream_handle())
        assert st == L.OK, lib.otx_status_string(st)
        torch.cuda.synchronize()
        assert torch.equal(bufs["unvignetted"], ref["unvignetted"])
        m = ref["unvignetted"].bool()
        for k in ("px", "py"):
            assert torch.allclose(bufs[k][m], ref[k][m], atol=1e-6, rtol=0), k
        assert torch.equal(images, ref_img)

    # the library counts the tiles itself: a caller's count that is too
    # large or too small (but within the array) traces the same rays
    for num_tiles in (b.num_tiles + 100, 1):
        b2 = L.Batch()
        ctypes.memmove(ctypes.byref(b2), ctypes.byref(b), ctypes.sizeof(L.Batch))
        b2.num_tiles = num_tiles
        bufs, out = _outputs(bt, torch)
        images = torch.zeros_like(bt.images)
        img = L.Image()
        img.counts = images.data_ptr()
        st = lib.otx_trace_batch_noalloc(ctypes.byref(bt.lowering.sys), ctypes.byref(b2),
                                         ctypes.byref(out), ctypes.byref(img),
                                         ctypes.byref(bt.launch), stream_handle())
        assert st == L.OK, lib.otx_status_string(st)
        torch.cuda.synchronize()
        assert torch.equal(bufs["unvignetted"], ref["unvignetted"])
        assert torch.equal(images, ref_img)

    # sizes beyond the scratch array are rejected, before any GPU work
    big = L.Batch()
    ctypes.memmove(ctypes.byref(big), ctypes.byref(b), ctypes.sizeof(L.Batch))
    big.num_tiles = L.NOALLOC_MAX_TILES + 1
    st = lib.otx_trace_batch_noalloc(ctypes.byref(bt.lowering.sys), ctypes.byref(big),
                                     ctypes.byref(out), ctypes.byref(img),
                                     ctypes.byref(bt.launch), stream_handle())
    assert st == L.ERR_SIZE
