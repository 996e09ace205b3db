"""The forward model: a scene's spectral radiance to detector electrons.

Mirrors ``SequentialSystem.image`` (optika/systems/_sequential.py:1088-1206)
and the steps it composes:

* ``_rayfunction_from_vertices`` (:1002-1086): the scene is given on cell
  *vertices* in wavelength, field and pupil; each cell sends one ray from a
  uniformly drawn point of the cell (the reference's ``cell_centers(...,
  random=True)``), carrying the cell's flux = radiance x cell area
  (``ObjectVectorArray.cell_area``, optika/vectors/_vectors_object.py:42-132:
  wavelength width x field area x pupil area, where an area is a solid
  angle for angular coordinates, and the field and pupil areas are averaged
  over the cell's wavelength vertices);
* ``rayfunction`` with the sensor binning of ``ImagingSensor.collect``
  (optika/sensors/_sensors.py:92-171): photon image and flux-weighted
  cosine of incidence;
* ``ImagingSensor.expose`` (:173-252) with the ideal sensor material:
  Poisson shot noise and Gaussian read noise.

The per-cell tables (a few thousand numbers) are made on the host in
float64; the rays are generated, traced, binned and exposed on the GPU
(``otx_cell_rays``, ``otx_trace_grid``, ``otx_expose``), in chunks of
``chunk`` rays so that any number of cells fits in memory.  Grids are
rectilinear: vertices are 1-D arrays per coordinate.
"""

from __future__ import annotations

import dataclasses

import numpy as np
import torch

from . import _lib as L
from .vectors import (Cartesian2dVectorArray, FunctionArray, SpectralPositionalVectorArray)

__all__ = ["CellTables", "ImagePlan", "cell_tables", "image", "solid_angle_cells"]


def _direction(ax, ay):
    """Unit propagation direction of field angles (optika/_util.py:69-73)."""
    return np.stack([-np.cos(ay) * np.sin(ax), -np.sin(ay), np.cos(ay) * np.cos(ax)])


def _triangle_solid_angle(a, b, c):
    """Solid angle of the spherical triangle of unit vectors a, b, c (van
    Oosterom and Strackee 1983): tan(O / 2) = |a.(b x c)| / (1 + a.b + b.c + c.a)."""
    num = np.abs(np.einsum("i...,i...->...", a, np.cross(b, c, axis=0)))
    den = 1 + np.einsum("i...,i...->...", a, b) + np.einsum("i...,i...->...", b, c) + \
        np.einsum("i...,i...->...", c, a)
    return 2 * np.arctan2(num, den)


def solid_angle_cells(ax: np.ndarray, ay: np.ndarray) -> np.ndarray:
    """Solid angles [nx, ny] of the cells of a rectilinear grid of field
    angles with vertices ``ax`` [nx + 1] and ``ay`` [ny + 1] (radians): each
    cell is the spherical quadrilateral of its corner directions, split into
    two triangles."""
    X, Y = np.meshgrid(np.asarray(ax, dtype=np.float64), np.asarray(ay, dtype=np.float64),
                       indexing="ij")
    d = _direction(X, Y)
    d00, d10 = d[:, :-1, :-1], d[:, 1:, :-1]
    d11, d01 = d[:, 1:, 1:], d[:, :-1, 1:]
    return _triangle_solid_angle(d00, d10, d11) + _triangle_solid_angle(d00, d11, d01)


def _areas(x: np.ndarray, y: np.ndarray, angular: bool) -> np.ndarray:
    if angular:
        return solid_angle_cells(x, y)
    return np.abs(np.outer(np.diff(x), np.diff(y)))


@dataclasses.dataclass
class CellTables:
    """Vertex tables at every wavelength vertex and per-cell weights."""

    wavelength: np.ndarray  # [nw + 1]
    field_x: np.ndarray  # [nw + 1, nfx + 1]
    field_y: np.ndarray  # [nw + 1, nfy + 1]
    pupil_x: np.ndarray  # [nw + 1, npx + 1]
    pupil_y: np.ndarray  # [nw + 1, npy + 1]
    weight: np.ndarray  # [nw, nfx, nfy] radiance x wavelength width x field area
    weight_pupil: np.ndarray  # [nw, npx, npy]

    @property
    def shape(self) -> tuple[int, int, int, int, int]:
        return (len(self.wavelength) - 1, self.field_x.shape[1] - 1, self.field_y.shape[1] - 1,
                self.pupil_x.shape[1] - 1, self.pupil_y.shape[1] - 1)

    @property
    def count(self) -> int:
        return int(np.prod(self.shape))


def _vertices(v, name: str) -> np.ndarray:
    if isinstance(v, torch.Tensor):
        v = v.detach().double().cpu().numpy()
    a = np.asarray(v, dtype=np.float64)
    if a.ndim != 1 or a.size < 2:
        raise ValueError(f"{name} vertices must be a 1-D array of at least two values")
    return a


def cell_tables(system, scene: FunctionArray, pupil=None, normalized_field: bool = True,
                normalized_pupil: bool = True) -> CellTables:
    """Tables of the scene's cells (host, float64)."""
    from .stops import extents, extents_many

    w = _vertices(scene.inputs.wavelength, "wavelength")
    fxn = _vertices(scene.inputs.position.x, "field x")
    fyn = _vertices(scene.inputs.position.y, "field y")
    if pupil is None:
        pupil = Cartesian2dVectorArray(np.array([-1.0, 1.0]), np.array([-1.0, 1.0]))
        normalized_pupil = True
    pxn = _vertices(pupil.x, "pupil x")
    pyn = _vertices(pupil.y, "pupil y")
    nw, nfx, nfy = len(w) - 1, len(fxn) - 1, len(fyn) - 1
    rad = scene.outputs
    if isinstance(rad, torch.Tensor):
        rad = rad.detach().double().cpu().numpy()
    rad = np.broadcast_to(np.asarray(rad, dtype=np.float64), (nw, nfx, nfy))

    if normalized_field or normalized_pupil:
        extents_many(system, w)  # every wavelength vertex in one batched solve

    def per_wavelength(v: np.ndarray, which: int, comp: int, normalized: bool) -> np.ndarray:
        out = np.empty((nw + 1, len(v)))
        for k in range(nw + 1):
            if normalized:
                e = extents(system, float(w[k]))
                lo, hi = e[which][comp], e[which + 1][comp]
                out[k] = (hi - lo) * (v + 1) / 2 + lo
            else:
                out[k] = v
        return out

    fx = per_wavelength(fxn, 0, 0, normalized_field)
    fy = per_wavelength(fyn, 0, 1, normalized_field)
    px = per_wavelength(pxn, 2, 0, normalized_pupil)
    py = per_wavelength(pyn, 2, 1, normalized_pupil)
    infinity = system.object_is_at_infinity
    memo: dict = {}

    def areas(x: np.ndarray, y: np.ndarray, angular: bool) -> np.ndarray:
        # physical grids repeat at every wavelength vertex: compute each once
        key = (x.tobytes(), y.tobytes(), angular)
        if key not in memo:
            memo[key] = _areas(x, y, angular)
        return memo[key]

    area_f = np.stack([areas(fx[k], fy[k], infinity) for k in range(nw + 1)])
    area_p = np.stack([areas(px[k], py[k], not infinity) for k in range(nw + 1)])
    # cell_centers along the wavelength axis: mean of the two vertices
    area_f = (area_f[:-1] + area_f[1:]) / 2
    area_p = (area_p[:-1] + area_p[1:]) / 2
    weight = rad * np.diff(w)[:, None, None] * area_f
    return CellTables(w, fx, fy, px, py, weight, area_p)


class ImagePlan:
    """An image simulation with its tables and device buffers made once:
    :meth:`run` enqueues the trace of every cell with sensor binning and the
    exposure on the current stream and returns the electrons.

    ``fused`` (default): one launch generates each cell's ray inside the
    trace kernel (otx_trace_cells), so no ray is written to memory.
    ``fused=False``: chunks of ``chunk`` cells, each a cell-ray launch into
    device buffers (otx_cell_rays) and a trace of those buffers."""

    def __init__(self, system, scene: FunctionArray, pupil=None, normalized_field: bool = True,
                 normalized_pupil: bool = True, integrate: bool = True, random: bool = True,
                 seed: int = 0, chunk: int = 1 << 24, fused: bool = True):
        from . import _api

        sensor = system.sensor
        if sensor is None:
            raise ValueError("image needs a sensor")
        self.system = system
        self.sensor = sensor
        t = cell_tables(system, scene, pupil, normalized_field, normalized_pupil)
        self.tables = t
        nw, nfx, nfy, npx, npy = t.shape
        w = t.wavelength
        if integrate:
            self.edges = np.array([w.min(), w.max()])
            bins = (float(self.edges[0]), float(self.edges[1]), 1)
        else:
            if not np.allclose(np.diff(w), (w[-1] - w[0]) / nw, rtol=1e-6, atol=0):
                raise ValueError("integrate=False needs uniformly spaced wavelength vertices")
            self.edges = w
            bins = (float(w[0]), float(w[-1]), nw)
        dev = _api.device()

        def dev_table(a: np.ndarray) -> torch.Tensor:
            return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32), device=dev)

        self._tabs = [dev_table(a) for a in (t.wavelength, t.field_x, t.field_y, t.pupil_x,
                                             t.pupil_y, t.weight, t.weight_pupil)]
        cells = L.Cells()
        (cells.wavelength, cells.field_x, cells.field_y, cells.pupil_x, cells.pupil_y,
         cells.weight, cells.weight_pupil) = (_api.ptr(x) for x in self._tabs)
        cells.nw, cells.nfx, cells.nfy, cells.npx, cells.npy = nw, nfx, nfy, npx, npy
        cells.random = 1 if random else 0
        cells.seed = int(seed) & (2**64 - 1)
        self.cells = cells
        self.seed = int(seed)
        self.count = t.count
        self.chunk = max(1, min(int(chunk), self.count))
        self.fused = bool(fused)
        nbuf = 1 if self.fused else self.chunk  # the fused trace reads no buffers
        self._buf = [torch.empty(nbuf, dtype=torch.float32, device=dev) for _ in range(6)]
        b = self._buf
        self.trace = _api.PreparedTrace(
            system, wavelength=b[0], field=Cartesian2dVectorArray(b[1], b[2]),
            pupil=Cartesian2dVectorArray(b[3], b[4]), intensity=b[5], final_local=True,
            image=True, wavelength_bins=bins, outputs=(), cos_moment=True)

    @property
    def launches(self) -> int:
        """Kernels per :meth:`run`: the trace (fused) or, per chunk, the cell
        rays and the trace; then the exposure."""
        if self.fused:
            return 2
        return 2 * ((self.count + self.chunk - 1) // self.chunk) + 1

    def photons(self) -> tuple[torch.Tensor, torch.Tensor]:
        """Photon image and flux-weighted cosine moment of the cells."""
        import ctypes

        from . import _api

        if self.fused:
            t = self.trace
            t.counts.zero_()
            t.flux.zero_()
            t.moment.zero_()
            L.check(L.load().otx_trace_cells(
                ctypes.byref(t.lowering.sys), ctypes.byref(self.cells), 0, self.count,
                ctypes.byref(t.img), ctypes.byref(t.launch_desc), _api.stream_handle()),
                "otx_trace_cells")
            return t.flux, t.moment
        for first in range(0, self.count, self.chunk):
            n = min(self.chunk, self.count - first)
            self.trace.grid.count = n
            _api.cell_rays(self.cells, first, n, self.trace.grid)
            self.trace.run(clear=first == 0)
        return self.trace.flux, self.trace.moment

    def run(self, noise: bool = True, timedelta=None, photons: bool = True) -> torch.Tensor:
        flux, mom = self.photons()
        direction = torch.where(flux > 0, mom / torch.where(flux > 0, flux, 1), 1)
        return self.sensor.expose(flux, direction=direction, timedelta=timedelta, noise=noise,
                                  seed=self.seed + 1, photons=photons, wavelength=self.edges)

    def result(self, electrons: torch.Tensor) -> FunctionArray:
        wx, wy = self.sensor.width_pixel_xy
        nx, ny = self.sensor.num_pixel
        pix = Cartesian2dVectorArray(np.linspace(-wx * nx / 2, wx * nx / 2, nx + 1),
                                     np.linspace(-wy * ny / 2, wy * ny / 2, ny + 1))
        return FunctionArray(
            inputs=SpectralPositionalVectorArray(wavelength=self.edges, position=pix),
            outputs=electrons)


def image(system, scene: FunctionArray, pupil=None, normalized_field: bool = True,
          normalized_pupil: bool = True, integrate: bool = True, noise: bool = True,
          random: bool = True, seed: int = 0, timedelta=None, chunk: int = 1 << 24,
          photons: bool = True) -> FunctionArray:
    """Detector electrons of the scene (optika/systems/_sequential.py:
    1088-1206) as a :class:`FunctionArray` whose inputs are the wavelength
    bin edges and the pixel edges and whose outputs are
    ``[num_wavelength, num_pixel_x, num_pixel_y]``.  See the module
    docstring; ``random=False`` traces the cell centres (deterministic),
    ``seed`` keys the cell draws and the noise."""
    plan = ImagePlan(system, scene, pupil, normalized_field, normalized_pupil, integrate,
                     random, seed, chunk)
    return plan.result(plan.run(noise=noise, timedelta=timedelta, photons=photons))
