"""Lowering of host description objects to the packed ``otx_system``.

Transforms are composed in float64: each surface receives the map from the
previous surface's frame to its own (``to_local``), so rays never visit the
global frame between surfaces, and the map back to the output frame
(``to_output``).  Translations are split into a float-float pair.
Unsupported plugin types raise ``NotImplementedError`` here; there is no
CPU fallback.
"""

from __future__ import annotations

import dataclasses
import math
from typing import Sequence

import numpy as np

from . import _lib as L
from . import apertures as ap
from . import materials as mt
from . import profiles as pr
from . import rulings as ru
from . import sags as sg
from .chemicals import Chemical
from .transforms import matrix_of, rigid_inverse


def split_f64(v: float) -> tuple[float, float]:
    hi = float(np.float32(v))
    lo = float(np.float32(v - hi))
    return hi, lo


def set_affine(dst: L.Affine, m: np.ndarray) -> None:
    r = m[:3, :3]
    t = m[:3, 3]
    for i in range(9):
        hi, lo = split_f64(float(r.flat[i]))
        dst.m[i] = hi
        dst.m_lo[i] = lo
    for i in range(3):
        hi, lo = split_f64(float(t[i]))
        dst.t_hi[i] = hi
        dst.t_lo[i] = lo
    if np.array_equal(r, np.eye(3)):
        dst.flags = L.AFFINE_ROT_IDENTITY
        if not np.any(t):
            dst.flags |= L.AFFINE_IDENTITY
    elif r[1, 1] == 1.0 and r[0, 1] == r[2, 1] == r[1, 0] == r[1, 2] == 0.0:
        dst.flags = L.AFFINE_ROT_Y  # a rotation in the x-z plane
    else:
        dst.flags = 0


@dataclasses.dataclass(eq=False)
class _Table:
    """A measured efficiency in the table pool's [x, y, -] column layout."""

    wavelength: np.ndarray
    n: np.ndarray

    @property
    def k(self) -> np.ndarray:
        return np.zeros_like(self.n)


class Lowering:
    """Accumulates the pools (vertices, layers, stacks, tables) of one system."""

    def __init__(self):
        self.sys = L.System()
        self.sys.abi_version = L.ABI_VERSION
        self.n_vertices = 0
        self.n_layers = 0
        self.n_stacks = 0
        self.table_list: list[Chemical] = []
        self.table_data = None  # torch tensor kept alive with the descriptor
        for k in range(L.MAX_LAYERS):
            self.sys.layers[k].table = -1
        for k in range(L.MAX_STACKS):
            self.sys.stacks[k].substrate = -1

    # ------------------------------------------------------------ layers
    def _add_table(self, table) -> int:
        for i, c in enumerate(self.table_list):
            if c is table:
                return i
        if len(self.table_list) >= L.MAX_STACKS * 4:
            raise ValueError("too many tables (chemicals, measured efficiencies) in one system")
        self.table_list.append(table)
        return len(self.table_list) - 1

    def _index_source(self, lay: L.Layer, chemical) -> None:
        lay.table = -1
        if chemical is None:
            lay.n_re, lay.n_im = 1.0, 0.0
        elif isinstance(chemical, Chemical):
            lay.table = self._add_table(chemical)
        elif isinstance(chemical, str):
            raise NotImplementedError(
                "chemical formulas need an explicit table: pass "
                "optika_gb300.chemicals.Chemical(wavelength, n, k)"
            )
        else:
            c = complex(chemical)
            lay.n_re, lay.n_im = c.real, c.imag

    def _add_layer(self, layer: mt.Layer, substrate: bool = False) -> int:
        if self.n_layers >= L.MAX_LAYERS:
            raise ValueError(f"more than {L.MAX_LAYERS} layers in one system")
        k = self.n_layers
        self.n_layers += 1
        lay = self.sys.layers[k]
        iface = getattr(layer, "interface", None)
        lay.interface_type = L.PROFILE_NONE
        lay.interface_width = 0.0
        if iface is not None:
            if not isinstance(iface, pr.AbstractInterfaceProfile) or not 1 <= iface.tag <= 4:
                raise NotImplementedError(
                    f"interface profile {type(iface).__name__} is not supported on the GPU path")
            lay.interface_type = iface.tag
            lay.interface_width = float(iface.width)
        self._index_source(lay, layer.chemical)
        th = 0.0 if substrate or layer.thickness is None else float(layer.thickness)
        lay.thickness = th
        return k

    def add_stack(self, layers, substrate) -> int:
        if self.n_stacks >= L.MAX_STACKS:
            raise ValueError(f"more than {L.MAX_STACKS} multilayer stacks in one system")
        items = _flatten_layers(layers)
        pre, per, post, periods = [], [], [], 0
        seen_periodic = False
        for it in items:
            if isinstance(it, mt.PeriodicLayerSequence):
                if seen_periodic:
                    raise NotImplementedError("at most one periodic block per stack")
                seen_periodic = True
                per = list(_flatten_layers(it.layers))
                if any(not isinstance(x, mt.Layer) for x in per):
                    raise NotImplementedError("nested periodic blocks are not supported")
                periods = int(it.num_periods)
            elif seen_periodic:
                post.append(it)
            else:
                pre.append(it)
        k = self.n_stacks
        self.n_stacks += 1
        K = self.sys.stacks[k]
        K.pre_begin = self.n_layers
        for x in pre:
            self._add_layer(x)
        K.pre_count = len(pre)
        K.per_begin = self.n_layers
        for x in per:
            self._add_layer(x)
        K.per_count = len(per)
        K.num_periods = periods
        K.post_begin = self.n_layers
        for x in post:
            self._add_layer(x)
        K.post_count = len(post)
        K.substrate = -1 if substrate is None else self._add_layer(substrate, substrate=True)
        return k

    def finish_tables(self, device) -> None:
        if not self.table_list:
            return
        import torch

        data = []
        off = 0
        for i, c in enumerate(self.table_list):
            self.sys.tables[i].offset = off
            self.sys.tables[i].count = len(c.wavelength)
            data += [c.wavelength, c.n, c.k]
            off += 3 * len(c.wavelength)
        arr = np.concatenate(data).astype(np.float32)
        self.table_data = torch.from_numpy(arr).to(device)
        self.sys.table_data = self.table_data.data_ptr()

    # ------------------------------------------------------------ surface
    def surface(self, k: int, s, to_local: np.ndarray, to_output: np.ndarray) -> None:
        d = self.sys.surfaces[k]
        set_affine(d.to_local, to_local)
        set_affine(d.to_output, to_output)
        set_affine(d.aper_to_local, np.eye(4))
        set_affine(d.rule_xform, np.eye(4))
        self._sag(d, s.sag)
        self._material(d, s.material)
        self._aperture(d, s.aperture)
        self._rulings(d, getattr(s, "rulings", None))

    def _sag(self, d: L.Surface, sag) -> None:
        if sag is None:
            sag = sg.NoSag()
        if getattr(sag, "transformation", None) is not None:
            raise NotImplementedError("sag transformations are not supported on the GPU path")
        if isinstance(sag, sg.NoSag):
            d.sag_type = L.SAG_FLAT
        elif isinstance(sag, sg.SphericalSag):
            d.sag_type = L.SAG_SPHERE
            d.sag_radius = float(sag.radius)
            d.sag_curvature = 1.0 / float(sag.radius)
        elif isinstance(sag, sg.ParabolicSag):
            d.sag_type = L.SAG_PARABOLA
            d.sag_focal_length = float(sag.focal_length)
            d.sag_radius = 2.0 * float(sag.focal_length)
            d.sag_curvature = 1.0 / d.sag_radius if d.sag_radius != 0 else math.inf
            d.sag_conic = -1.0
        elif isinstance(sag, sg.AbstractConicSag):
            d.sag_type = L.SAG_CONIC
            d.sag_radius = float(sag.radius)
            d.sag_curvature = 1.0 / float(sag.radius)
            d.sag_conic = float(sag.conic)
        elif isinstance(sag, sg.CylindricalSag):
            r = float(sag.radius)
            if math.isinf(r):  # the reference's formulas reduce to the plane
                d.sag_type = L.SAG_FLAT
            else:
                d.sag_type = L.SAG_CYLINDER
                d.sag_radius = r
                d.sag_curvature = 1.0 / r
        elif isinstance(sag, sg.ToroidalSag):
            d.sag_type = L.SAG_TOROID
            d.sag_radius = float(sag.radius)
            d.sag_curvature = 1.0 / float(sag.radius)
            d.sag_radius_of_rotation = float(sag.radius_of_rotation)
        else:
            raise NotImplementedError(f"sag type {type(sag).__name__} is not supported on the GPU path")

    def _material(self, d: L.Surface, m) -> None:
        if m is None:
            m = mt.Vacuum()
        if isinstance(m, mt.MultilayerMirror):
            d.mat_type = L.MAT_MULTILAYER_MIRROR
            d.mat_is_mirror = 1
            d.mat_stack = self.add_stack(m.layers, m.substrate)
        elif isinstance(m, mt.MultilayerFilm):
            d.mat_type = L.MAT_MULTILAYER_FILM
            d.mat_stack = self.add_stack(m.layers, None)
        elif isinstance(m, mt.MeasuredMirror):
            wavelength, reflectivity = m.table()
            d.mat_type = L.MAT_MEASURED_MIRROR
            d.mat_is_mirror = 1
            d.mat_table = self._add_table(_Table(wavelength, reflectivity))
        elif isinstance(m, mt.AbstractMirror):
            d.mat_type = L.MAT_MIRROR
            d.mat_is_mirror = 1
        elif isinstance(m, mt.Glass):
            d.mat_type = L.MAT_GLASS
            for i, (b, c) in enumerate([(m.b1, m.c1), (m.b2, m.c2), (m.b3, m.c3)]):
                d.sellmeier_b[i] = float(b)
                d.sellmeier_c[i] = float(c) * 1e6  # um^2 -> nm^2
        elif isinstance(m, mt.Vacuum):
            d.mat_type = L.MAT_VACUUM
        else:
            raise NotImplementedError(f"material {type(m).__name__} is not supported on the GPU path")

    def _aperture(self, d: L.Surface, a) -> None:
        if a is None:
            d.aper_type = L.APER_NONE
            return
        flags = 0
        if a.active:
            flags |= L.APER_FLAG_ACTIVE
        if a.inverted:
            flags |= L.APER_FLAG_INVERTED
        if a.dimensionless:
            flags |= L.APER_FLAG_DIRECTION
        if a.transformation is not None:
            flags |= L.APER_FLAG_TRANSFORM
            set_affine(d.aper_to_local, rigid_inverse(matrix_of(a.transformation)))
        d.aper_flags = flags
        if isinstance(a, ap.CircularAperture):
            d.aper_type = L.APER_CIRCULAR
            d.aper_p[0] = float(a.radius)
        elif isinstance(a, ap.RectangularAperture):
            d.aper_type = L.APER_RECTANGULAR
            hx, hy = a.half_width_xy
            d.aper_p[0], d.aper_p[1] = hx, hy
        elif isinstance(a, ap.EllipticalAperture):
            d.aper_type = L.APER_ELLIPTICAL
            d.aper_p[0], d.aper_p[1] = float(a.radius[0]), float(a.radius[1])
        elif isinstance(a, ap.CircularSectorAperture):
            d.aper_type = L.APER_SECTOR
            d.aper_p[0] = float(a.radius)
            d.aper_p[1] = float(a.angle_start)
            d.aper_p[2] = float(a.angle_stop)
        elif isinstance(a, ap.PolygonalAperture):
            v = a.vertex_array()
            if len(v) < 3:
                raise ValueError("a polygonal aperture needs at least 3 vertices")
            if self.n_vertices + len(v) > L.MAX_VERTICES:
                raise ValueError(f"more than {L.MAX_VERTICES} polygon vertices in one system")
            d.aper_type = L.APER_POLYGON
            d.aper_vertex_begin = self.n_vertices
            d.aper_vertex_count = len(v)
            for i, (x, y) in enumerate(v):
                self.sys.vertices[2 * (self.n_vertices + i)] = float(x)
                self.sys.vertices[2 * (self.n_vertices + i) + 1] = float(y)
            self.n_vertices += len(v)
        else:
            raise NotImplementedError(f"aperture {type(a).__name__} is not supported on the GPU path")

    def _rulings(self, d: L.Surface, r) -> None:
        if r is None:
            d.rule_type = L.RULE_NONE
            return
        if not isinstance(r, ru.AbstractRulings):
            raise NotImplementedError(f"rulings {type(r).__name__} are not supported on the GPU path")
        d.rule_order = float(r.diffraction_order)
        d.rule_efficiency = 1.0
        d.rule_eff_type = L.RULE_EFF_IDEAL
        if isinstance(r, ru.MeasuredRulings):
            wavelength, efficiency = r.table()
            d.rule_eff_type = L.RULE_EFF_MEASURED
            d.rule_table = self._add_table(_Table(wavelength, efficiency))
        elif not isinstance(r, ru.Rulings):
            models = {
                ru.SinusoidalRulings: L.RULE_EFF_SINUSOIDAL,
                ru.SquareRulings: L.RULE_EFF_SQUARE,
                ru.SawtoothRulings: L.RULE_EFF_SAWTOOTH,
                ru.TriangularRulings: L.RULE_EFF_TRIANGULAR,
                ru.RectangularRulings: L.RULE_EFF_RECTANGULAR,
            }
            if type(r) not in models:
                raise NotImplementedError(
                    f"rulings {type(r).__name__} are not supported on the GPU path")
            d.rule_eff_type = models[type(r)]
            if d.rule_eff_type == L.RULE_EFF_SINUSOIDAL and (
                    float(r.diffraction_order) != int(r.diffraction_order)):
                raise NotImplementedError("sinusoidal rulings need an integer diffraction order")
            # groove depth (mm) over the model's amplitude, in nm like the
            # wavelengths it is divided by
            d.rule_depth = float(r.depth) / float(r.amplitude) * 1e6
            if isinstance(r, ru.RectangularRulings):
                d.rule_duty = 2 * math.pi * float(r.ratio_duty)
        s = r.spacing_
        if isinstance(s, ru.ConstantRulingSpacing):
            d.rule_type = L.RULE_CONSTANT
            d.rule_coef[0] = float(s.constant)
            for i in range(3):
                d.rule_normal[i] = float(s.normal[i])
        elif isinstance(s, ru.Polynomial1dRulingSpacing):
            d.rule_type = L.RULE_POLY1D
            powers = [int(p) for p in s.coefficients]
            if any(p < 0 for p in powers) or (powers and max(powers) >= L.MAX_POLY_TERMS):
                raise ValueError(f"polynomial ruling powers must be in [0, {L.MAX_POLY_TERMS})")
            n = (max(powers) + 1) if powers else 0
            d.rule_num_terms = n
            for p, c in s.coefficients.items():
                d.rule_coef[int(p)] = float(c)
            for i in range(3):
                d.rule_normal[i] = float(s.normal[i])
            set_affine(d.rule_xform, matrix_of(s.transformation))
        elif isinstance(s, ru.HolographicRulingSpacing):
            d.rule_type = L.RULE_HOLOGRAPHIC
            for i in range(3):
                d.holo_x1[i] = float(s.x1[i])
                d.holo_x2[i] = float(s.x2[i])
            d.holo_wavelength = float(s.wavelength) * 1e-6
            d.holo_d1 = 2.0 * bool(s.is_diverging_1) - 1.0
            d.holo_d2 = 2.0 * bool(s.is_diverging_2) - 1.0
        else:
            raise NotImplementedError(f"ruling spacing {type(s).__name__} is not supported")


def _flatten_layers(layers) -> list:
    if layers is None:
        return []
    if isinstance(layers, (mt.Layer, mt.PeriodicLayerSequence)):
        return [layers]
    if isinstance(layers, mt.LayerSequence):
        return _flatten_layers(list(layers.layers))
    out = []
    for x in layers:
        out += _flatten_layers(x)
    return out


def lower_surfaces(
    surfaces: Sequence,
    *,
    pre: np.ndarray,
    final: np.ndarray | None,
    input_mode: int,
    sensor=None,
    wavelength_bins=None,
    device=None,
    newton_iterations: int = 0,
) -> Lowering:
    """Pack ``surfaces`` into an ``otx_system``.

    ``pre`` maps the input frame to the frame the surfaces' transformations
    are relative to; ``final`` maps the last surface's local frame to the
    output frame of the final rays (``None``: back to that parent frame).
    """
    if len(surfaces) < 1:
        raise ValueError("a system needs at least one surface")
    if len(surfaces) > L.MAX_SURFACES:
        raise ValueError(f"at most {L.MAX_SURFACES} surfaces per system")
    lw = Lowering()
    S = lw.sys
    S.num_surfaces = len(surfaces)
    S.input_mode = input_mode
    S.newton_iterations = int(newton_iterations)
    prev = pre
    for k, s in enumerate(surfaces):
        T = matrix_of(s.transformation)
        lw.surface(k, s, rigid_inverse(T) @ prev, T)
        prev = T
    fin = prev if final is None else final
    set_affine(S.final_to_output, fin)
    if np.array_equal(fin, np.eye(4)):
        S.flags |= L.SYS_FLAG_FINAL_IDENTITY
    if sensor is not None:
        S.surfaces[len(surfaces) - 1].is_sensor = 1
        wx, wy = sensor.width_pixel_xy
        nx, ny = sensor.num_pixel
        S.sensor.num_x, S.sensor.num_y = int(nx), int(ny)
        S.sensor.width_x, S.sensor.width_y = wx, wy
        S.sensor.lo_x, S.sensor.lo_y = -wx * nx / 2, -wy * ny / 2
        S.sensor.inv_width_x, S.sensor.inv_width_y = 1.0 / wx, 1.0 / wy
        if wavelength_bins is None:
            S.sensor.num_w = 1
            S.sensor.w_lo, S.sensor.w_hi = 0.0, 0.0
        else:
            w0, w1, nw = wavelength_bins
            S.sensor.num_w = int(nw)
            S.sensor.w_lo, S.sensor.w_hi = float(w0), float(w1)
            S.sensor.inv_width_w = float(nw) / (float(w1) - float(w0))
    if device is not None:
        lw.finish_tables(device)
    return lw
