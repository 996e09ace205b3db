"""Batched trace of many configurations of one system shape.

The reference batches configurations by broadcasting named axes through
every component of a ``SequentialSystem`` (optika/_util.py:21-38).  Here a
batch is a base system plus, per configuration, replacement descriptors of
the surfaces that vary; all configurations run in one persistent launch
(``otx_trace_batch``) that generates each configuration's rays on the
device (Philox4x32-10), so ragged ray counts (1e3 .. 1e6 per configuration)
cost no host traffic.  :meth:`BatchedTrace.tune` picks the tile size and
rays per thread by timing; :meth:`BatchedTrace.graph` captures a step in a
CUDA graph.
"""

from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np
import torch

from . import _lib as L
from ._api import device, ptr, stream_handle, _alloc_rays, _rays_struct
from ._lower import Lowering, lower_surfaces, set_affine
from .transforms import matrix_of, rigid_inverse

_TUNED: dict = {}


def _kind(lw_sys: L.System, k: int) -> tuple:
    s = lw_sys.surfaces[k]
    return (s.sag_type, s.mat_type, s.aper_type, s.rule_type)


class BatchedTrace:
    """All configurations of a batch, traced to the sensor's local frame.

    ``systems`` share one shape (same surface kinds); surfaces that differ
    between them (by transformation or parameters) are listed in
    ``overrides`` (surface indices into ``system.surfaces_all``).
    """

    def __init__(self, systems: Sequence, overrides: Sequence[int], ray_counts, *, seed: int,
                 wavelength: tuple[float, float], field_half: tuple[float, float],
                 pupil_half: float, image: bool = False, tile_size: int = 8192,
                 rays_per_thread: int = 1, outputs=("px", "py", "unvignetted")):
        dev = device()
        if len(systems) < 1:
            raise ValueError("a batch needs at least one configuration")
        if len(overrides) > 4:
            raise ValueError("at most 4 surfaces may vary between configurations")
        base = systems[0]
        if not base.object_is_at_infinity:
            raise NotImplementedError("batched traces generate objects at infinity")
        surfaces0 = base.surfaces_all
        if surfaces0[-1] is base.sensor:
            final = np.eye(4)  # exactly: the last surface is the sensor
        else:
            final = rigid_inverse(matrix_of(base.sensor.transformation)) @ matrix_of(
                surfaces0[-1].transformation)
        pre = rigid_inverse(matrix_of(base.transformation)) @ matrix_of(base.object.transformation)
        self.lowering = lower_surfaces(surfaces0, pre=pre, final=final,
                                       input_mode=L.INPUT_GRID_INFINITY,
                                       sensor=base.sensor if image else None, device=dev)
        n_cfg = len(systems)
        n_ov = len(overrides)
        table = (L.Surface * max(1, n_cfg * n_ov))()
        for c, system in enumerate(systems):
            surfs = system.surfaces_all
            if len(surfs) != len(surfaces0):
                raise ValueError("every configuration must have the base system's surfaces")
            for j, k in enumerate(overrides):
                prev = pre if k == 0 else matrix_of(surfs[k - 1].transformation)
                T = matrix_of(surfs[k].transformation)
                lw = Lowering()
                lw.surface(0, surfs[k], rigid_inverse(T) @ prev, T)
                if lw.n_vertices or lw.n_layers or lw.n_stacks:
                    raise NotImplementedError(
                        "varying surfaces may not carry polygon apertures or multilayers")
                d = lw.sys.surfaces[0]
                if (d.sag_type, d.mat_type, d.aper_type, d.rule_type) != _kind(self.lowering.sys, k):
                    raise ValueError("a varying surface must keep the kinds of the base surface")
                d.is_sensor = self.lowering.sys.surfaces[k].is_sensor
                ctypes.memmove(ctypes.byref(table, (c * n_ov + j) * ctypes.sizeof(L.Surface)),
                               ctypes.byref(d), ctypes.sizeof(L.Surface))
        self.overrides = torch.frombuffer(bytearray(bytes(table)), dtype=torch.uint8).to(dev)
        counts = np.asarray(ray_counts, dtype=np.int64)
        if counts.shape != (n_cfg,) or np.any(counts < 0):
            raise ValueError("ray_counts must give one non-negative count per configuration")
        if np.any(counts > np.iinfo(np.int32).max):
            # a work item stores its first ray as int32 (otx_batch.tiles)
            raise ValueError("a configuration may hold at most 2**31 - 1 rays")
        offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        self.counts = counts
        self.ray_offset_host = offs
        self.ray_offset = torch.from_numpy(offs).to(dev)
        self.total = int(offs[-1])
        self.counter = torch.zeros(1, dtype=torch.int32, device=dev)  # scratch work counter
        self.bufs = _alloc_rays(self.total, dev, (), outputs)
        self.out = _rays_struct(self.bufs, self.total)
        self.img = L.Image()
        self.images = None
        if image:
            nx, ny = base.sensor.num_pixel
            self.images = torch.zeros((n_cfg, 1, int(nx), int(ny)), dtype=torch.int32, device=dev)
            self.img.counts = self.images.data_ptr()
        b = L.Batch()
        b.num_configs = n_cfg
        b.num_overrides = n_ov
        for j, k in enumerate(overrides):
            b.override_index[j] = int(k)
        b.overrides = ptr(self.overrides)
        b.ray_offset = ptr(self.ray_offset)
        b.counter = ptr(self.counter)
        b.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        b.wl_lo, b.wl_hi = float(wavelength[0]), float(wavelength[1])
        b.field_x_half, b.field_y_half = float(field_half[0]), float(field_half[1])
        b.pupil_half = float(pupil_half)
        if image:
            nx, ny = base.sensor.num_pixel
            b.image_stride = int(nx) * int(ny)
        self.batch = b
        self.launch = L.Launch()
        self.seed = int(seed)
        self.shape_key = (tuple(_kind(self.lowering.sys, k) for k in range(len(surfaces0))),
                          n_cfg, self.total)
        self.set_schedule(tile_size, rays_per_thread)
        self.lib = L.load()

    def set_schedule(self, tile_size: int, rays_per_thread: int = 1, block_size: int = 256):
        dev = self.ray_offset.device
        tiles = []
        for c, n in enumerate(self.counts):
            for start in range(0, int(n), tile_size):
                tiles.append((c, start))
        arr = np.asarray(tiles, dtype=np.int32).reshape(-1, 2)
        self.tiles = torch.from_numpy(arr).to(dev)
        self.batch.tiles = ptr(self.tiles)
        self.batch.num_tiles = len(tiles)
        self.batch.tile_size = int(tile_size)
        self.launch.rays_per_thread = int(rays_per_thread)
        self.launch.block_size = int(block_size)
        self.schedule = (int(tile_size), int(rays_per_thread), int(block_size))

    def run(self) -> None:
        if self.images is not None:
            self.images.zero_()
        st = self.lib.otx_trace_batch(
            ctypes.byref(self.lowering.sys), ctypes.byref(self.batch), ctypes.byref(self.out),
            ctypes.byref(self.img), ctypes.byref(self.launch), stream_handle())
        L.check(st, "otx_trace_batch")

    def config_slice(self, c: int) -> slice:
        return slice(int(self.ray_offset_host[c]), int(self.ray_offset_host[c + 1]))

    def tune(self, candidates=((512, 1), (1024, 1), (2048, 1), (8192, 1), (32768, 1), (8192, 2),
                               (32768, 2)),
             repeats: int = 3) -> tuple:
        """Time each (tile size, rays per thread) and keep the fastest; the
        choice is cached per shape, configuration count and ray total."""
        if self.shape_key in _TUNED:
            self.set_schedule(*_TUNED[self.shape_key])
            return _TUNED[self.shape_key]
        best = None
        for tile, rpt in candidates:
            self.set_schedule(tile, rpt)
            self.run()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(repeats):
                self.run()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / repeats
            if best is None or ms < best[0]:
                best = (ms, tile, rpt)
        self.set_schedule(best[1], best[2])
        _TUNED[self.shape_key] = (best[1], best[2])
        return _TUNED[self.shape_key]

    def graph(self) -> torch.cuda.CUDAGraph:
        """Capture one step (image clear, counter clear, kernel) in a CUDA graph."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.run()  # warm
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run()
        return g
