"""ctypes binding of the C-ABI in ``include/optika_gb300.h``.

The structures below mirror the header field for field; ``check_layout``
compares their sizes with ``otx_sizeof`` exported by the library.  Loading
fails loudly when the library has not been built: there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import pathlib

ABI_VERSION = 3
MAX_SURFACES = 16
MAX_POLY_TERMS = 8
MAX_VERTICES = 64
MAX_LAYERS = 64
MAX_STACKS = 4
NOALLOC_MAX_TILES = 131000

OK = 0
ERR_INVALID = 1
ERR_UNSUPPORTED = 2
ERR_CUDA = 3
ERR_SIZE = 4
ERR_TIMEOUT = 5

SAG_FLAT, SAG_SPHERE, SAG_CONIC, SAG_PARABOLA, SAG_TOROID, SAG_CYLINDER = range(6)
(MAT_VACUUM, MAT_MIRROR, MAT_GLASS, MAT_MULTILAYER_MIRROR, MAT_MULTILAYER_FILM,
 MAT_MEASURED_MIRROR) = range(6)
APER_NONE, APER_CIRCULAR, APER_RECTANGULAR, APER_ELLIPTICAL, APER_SECTOR, APER_POLYGON = range(6)
APER_FLAG_INVERTED = 1
APER_FLAG_ACTIVE = 2
APER_FLAG_DIRECTION = 4
APER_FLAG_TRANSFORM = 8
RULE_NONE, RULE_CONSTANT, RULE_POLY1D, RULE_HOLOGRAPHIC = range(4)
(RULE_EFF_IDEAL, RULE_EFF_MEASURED, RULE_EFF_SINUSOIDAL, RULE_EFF_SQUARE, RULE_EFF_SAWTOOTH,
 RULE_EFF_TRIANGULAR, RULE_EFF_RECTANGULAR) = range(7)
INPUT_RAYS, INPUT_GRID_INFINITY, INPUT_GRID_FINITE = range(3)
EPI_SILU_BF16, EPI_BIAS_F32, EPI_F32, EPI_DSILU_BF16, EPI_F32_ATOMIC = range(5)
SYS_FLAG_FINAL_IDENTITY = 1
PROFILE_NONE, PROFILE_ERF, PROFILE_EXPONENTIAL, PROFILE_LINEAR, PROFILE_SINUSOIDAL = range(5)

f32 = ctypes.c_float
i32 = ctypes.c_int32
i64 = ctypes.c_int64
u64 = ctypes.c_uint64


AFFINE_ROT_IDENTITY = 1
AFFINE_ROT_Y = 2
AFFINE_IDENTITY = 4


class Affine(ctypes.Structure):
    _fields_ = [
        ("m", f32 * 9),
        ("m_lo", f32 * 9),
        ("t_hi", f32 * 3),
        ("t_lo", f32 * 3),
        ("flags", i32),
        ("pad_", i32),
    ]


class Layer(ctypes.Structure):
    _fields_ = [("n_re", f32), ("n_im", f32), ("thickness", f32), ("table", i32),
                ("interface_type", i32), ("interface_width", f32)]


class Stack(ctypes.Structure):
    _fields_ = [
        ("pre_begin", i32),
        ("pre_count", i32),
        ("per_begin", i32),
        ("per_count", i32),
        ("num_periods", i32),
        ("post_begin", i32),
        ("post_count", i32),
        ("substrate", i32),
    ]


class PeriodicStack(ctypes.Structure):
    _fields_ = [
        ("n_a_re", f32),
        ("n_a_im", f32),
        ("n_b_re", f32),
        ("n_b_im", f32),
        ("n_sub_re", f32),
        ("n_sub_im", f32),
        ("thickness_a", f32),
        ("thickness_b", f32),
        ("num_periods", i32),
        ("pad_", i32),
    ]


class Table(ctypes.Structure):
    _fields_ = [("offset", i32), ("count", i32)]


class Surface(ctypes.Structure):
    _fields_ = [
        ("to_local", Affine),
        ("to_output", Affine),
        ("aper_to_local", Affine),
        ("rule_xform", Affine),
        ("sag_type", i32),
        ("sag_radius", f32),
        ("sag_curvature", f32),
        ("sag_conic", f32),
        ("sag_radius_of_rotation", f32),
        ("sag_focal_length", f32),
        ("mat_type", i32),
        ("mat_is_mirror", i32),
        ("mat_stack", i32),
        ("mat_table", i32),
        ("sellmeier_b", f32 * 3),
        ("sellmeier_c", f32 * 3),
        ("aper_type", i32),
        ("aper_flags", i32),
        ("aper_p", f32 * 4),
        ("aper_vertex_begin", i32),
        ("aper_vertex_count", i32),
        ("rule_type", i32),
        ("rule_num_terms", i32),
        ("rule_order", f32),
        ("rule_efficiency", f32),
        ("rule_normal", f32 * 3),
        ("rule_coef", f32 * MAX_POLY_TERMS),
        ("holo_x1", f32 * 3),
        ("holo_x2", f32 * 3),
        ("holo_wavelength", f32),
        ("holo_d1", f32),
        ("holo_d2", f32),
        ("rule_eff_type", i32),
        ("rule_table", i32),
        ("rule_depth", f32),
        ("rule_duty", f32),
        ("is_sensor", i32),
        ("pad_", i32),
    ]


class Sensor(ctypes.Structure):
    _fields_ = [
        ("num_x", i32),
        ("num_y", i32),
        ("num_w", i32),
        ("pad_", i32),
        ("lo_x", f32),
        ("lo_y", f32),
        ("width_x", f32),
        ("width_y", f32),
        ("w_lo", f32),
        ("w_hi", f32),
        ("inv_width_x", f32),
        ("inv_width_y", f32),
        ("inv_width_w", f32),
        ("pad2_", i32),
    ]


class System(ctypes.Structure):
    _fields_ = [
        ("abi_version", i32),
        ("num_surfaces", i32),
        ("input_mode", i32),
        ("newton_iterations", i32),
        ("flags", i32),
        ("pad_", i32),
        ("final_to_output", Affine),
        ("sensor", Sensor),
        ("surfaces", Surface * MAX_SURFACES),
        ("vertices", f32 * (2 * MAX_VERTICES)),
        ("layers", Layer * MAX_LAYERS),
        ("stacks", Stack * MAX_STACKS),
        ("tables", Table * (MAX_STACKS * 4)),
        ("table_data", u64),
    ]


class Rays(ctypes.Structure):
    _fields_ = [
        ("px", u64),
        ("py", u64),
        ("pz", u64),
        ("dx", u64),
        ("dy", u64),
        ("dz", u64),
        ("wavelength", u64),
        ("intensity", u64),
        ("attenuation", u64),
        ("index_refraction", u64),
        ("unvignetted", u64),
        ("opl", u64),
        ("count", i64),
        ("surface_stride", i64),
    ]


class Grid(ctypes.Structure):
    _fields_ = [
        ("wavelength", u64),
        ("field_x", u64),
        ("field_y", u64),
        ("pupil_x", u64),
        ("pupil_y", u64),
        ("intensity", u64),
        ("stride_wavelength", i64),
        ("stride_field", i64),
        ("stride_pupil", i64),
        ("stride_intensity", i64),
        ("count", i64),
    ]


class Image(ctypes.Structure):
    _fields_ = [("counts", u64), ("flux", u64), ("cos_moment", u64)]


class StopSolve(ctypes.Structure):
    _fields_ = [
        ("count", i64),
        ("free_position", i32),
        ("target_direction", i32),
        ("max_iterations", i32),
        ("polish_steps", i32),
        ("step", ctypes.c_double),
        ("tolerance", ctypes.c_double),
        ("to_last", ctypes.c_double * 12),
        ("position", u64),
        ("direction", u64),
        ("wavelength", u64),
        ("target_x", u64),
        ("target_y", u64),
        ("status", u64),
    ]


class Batch(ctypes.Structure):
    _fields_ = [
        ("num_configs", i32),
        ("num_overrides", i32),
        ("override_index", i32 * 4),
        ("tile_size", i32),
        ("pad_", i32),
        ("overrides", u64),
        ("ray_offset", u64),
        ("tiles", u64),
        ("num_tiles", i64),
        ("counter", u64),
        ("seed", u64),
        ("wl_lo", f32),
        ("wl_hi", f32),
        ("field_x_half", f32),
        ("field_y_half", f32),
        ("pupil_half", f32),
        ("image_stride", i32),
    ]


SURROGATE_NIN = 9
SURROGATE_LDX = 16
SURROGATE_NBASE = 21


class Surrogate(ctypes.Structure):
    _fields_ = [
        ("num_configs", i32),
        ("pad_", i32),
        ("config_inputs", u64),
        ("baseline", u64),
        ("trusted", u64),
        ("out_scale", f32),
        ("logit_band", f32),
        ("pad2_", f32 * 2),
    ]


MLP_MAX_HIDDEN = 6


class Mlp(ctypes.Structure):
    _fields_ = [
        ("num_inputs", i32),
        ("num_hidden", i32),
        ("width", i32),
        ("num_outputs", i32),
        ("w", u64 * (MLP_MAX_HIDDEN + 1)),
        ("ld", i32 * (MLP_MAX_HIDDEN + 1)),
        ("pad_", i32),
        ("b", u64 * (MLP_MAX_HIDDEN + 1)),
    ]


class Launch(ctypes.Structure):
    _fields_ = [
        ("rays_per_thread", i32),
        ("block_size", i32),
        ("accumulate", i32),
        ("generic_only", i32),
    ]


class Cells(ctypes.Structure):
    _fields_ = [
        ("wavelength", u64),
        ("field_x", u64),
        ("field_y", u64),
        ("pupil_x", u64),
        ("pupil_y", u64),
        ("weight", u64),
        ("weight_pupil", u64),
        ("nw", i32),
        ("nfx", i32),
        ("nfy", i32),
        ("npx", i32),
        ("npy", i32),
        ("random", i32),
        ("seed", u64),
    ]


LAYOUT = {
    0: System,
    1: Surface,
    2: Rays,
    3: Grid,
    4: Image,
    5: Launch,
    6: Affine,
    7: Sensor,
    8: Layer,
    9: Stack,
    10: PeriodicStack,
    11: Batch,
    12: Surrogate,
    13: Mlp,
    14: Cells,
    15: StopSolve,
}

LIB_PATH = pathlib.Path(__file__).resolve().parent / "_lib" / "liboptika_gb300.so"

_lib = None


class OtxError(RuntimeError):
    """A non-zero ``otx_status`` returned by the library."""

    def __init__(self, status: int, where: str):
        self.status = status
        msg = _status_string(status)
        super().__init__(f"{where} failed with status {status} ({msg})")


def _status_string(status: int) -> str:
    if _lib is None:
        return "library not loaded"
    return _lib.otx_status_string(status).decode()


def _declare(lib: ctypes.CDLL) -> None:
    P = ctypes.POINTER
    v = ctypes.c_void_p
    lib.otx_sizeof.argtypes = [i32]
    lib.otx_sizeof.restype = i64
    lib.otx_abi_version.argtypes = []
    lib.otx_abi_version.restype = i32
    lib.otx_status_string.argtypes = [i32]
    lib.otx_status_string.restype = ctypes.c_char_p
    lib.otx_trace_rays.argtypes = [P(System), P(Rays), P(Rays), P(Image), P(Launch), v]
    lib.otx_trace_rays.restype = i32
    lib.otx_trace_grid.argtypes = [P(System), P(Grid), P(Rays), P(Image), P(Launch), v]
    lib.otx_trace_grid.restype = i32
    lib.otx_trace_grid_host.argtypes = [P(System), P(Grid), P(Rays), P(Image), P(Launch), v, i64,
                                        v]
    lib.otx_trace_grid_host.restype = i32
    lib.otx_trace_grid_host_workspace.argtypes = [P(Grid), P(Rays), i32]
    lib.otx_trace_grid_host_workspace.restype = i64
    lib.otx_multilayer_efficiency.argtypes = [
        P(System), i64, v, i64, v, i64, v, v, i64, v, v, v, v, v, v,
    ]
    lib.otx_multilayer_efficiency.restype = i32
    lib.otx_multilayer_periodic.argtypes = [
        v, i32, i64, v, i64, v, i64, v, f32, f32, v, v, v, v, v,
    ]
    lib.otx_multilayer_periodic.restype = i32
    lib.otx_trace_batch.argtypes = [P(System), P(Batch), P(Rays), P(Image), P(Launch), v]
    lib.otx_trace_batch.restype = i32
    lib.otx_trace_batch_noalloc.argtypes = [P(System), P(Batch), P(Rays), P(Image), P(Launch), v]
    lib.otx_trace_batch_noalloc.restype = i32
    lib.otx_stop_newton.argtypes = [P(System), P(System), P(StopSolve), v]
    lib.otx_stop_newton.restype = i32
    lib.otx_trace_cells.argtypes = [P(System), P(Cells), i64, i64, P(Image), P(Launch), v]
    lib.otx_trace_cells.restype = i32
    lib.otx_gemm_bf16.argtypes = [v, i32, v, i32, i32, i32, i32, v, i32, v, i32, v, v, i32, v, v]
    lib.otx_gemm_bf16.restype = i32
    lib.otx_silu_backward.argtypes = [v, v, v, i64, v]
    lib.otx_silu_backward.restype = i32
    lib.otx_transpose_bf16.argtypes = [v, i32, i32, i32, v, i32, v]
    lib.otx_transpose_bf16.restype = i32
    lib.otx_colsum_bf16.argtypes = [v, i32, i32, i32, v, v]
    lib.otx_colsum_bf16.restype = i32
    lib.otx_adam.argtypes = [v, v, v, v, i32, i32, f32, f32, f32, f32, i32, v, i32, v, i32, v]
    lib.otx_adam.restype = i32
    lib.otx_surrogate_pack.argtypes = [P(Batch), P(Surrogate), i64, i64, v, v, v, v, v, v, i32,
                                       v, v, v]
    lib.otx_surrogate_pack.restype = i32
    lib.otx_surrogate_loss.argtypes = [v, i32, v, i64, f32, f32, f32, v, v, i32, v, v]
    lib.otx_surrogate_loss.restype = i32
    lib.otx_surrogate_image.argtypes = [P(System), P(Batch), P(Surrogate), i64, i64, v, i32, v,
                                        P(Image), v, v]
    lib.otx_surrogate_image.restype = i32
    lib.otx_surrogate_image_fused.argtypes = [P(System), P(Batch), P(Surrogate), P(Mlp), i64, i64,
                                              P(Image), v, v, i64, v, v, v]
    lib.otx_surrogate_image_fused.restype = i32
    lib.otx_surrogate_image_fused_workspace.argtypes = [P(Batch), P(Mlp), i64]
    lib.otx_surrogate_image_fused_workspace.restype = i64
    lib.otx_collect.argtypes = [P(Sensor), P(Rays), P(Image), v]
    lib.otx_collect.restype = i32
    lib.otx_sag_eval.argtypes = [P(System), i32, P(Rays), P(Rays), v]
    lib.otx_sag_eval.restype = i32
    lib.otx_rulings_eval.argtypes = [P(System), i32, P(Rays), P(Rays), v, P(Rays), v]
    lib.otx_rulings_eval.restype = i32
    lib.otx_pupil_reduce.argtypes = [P(Rays), i64, i64, v, v]
    lib.otx_pupil_reduce.restype = i32
    lib.otx_cell_rays.argtypes = [P(Cells), i64, i64, P(Grid), v]
    lib.otx_cell_rays.restype = i32
    lib.otx_expose.argtypes = [v, v, i64, f32, f32, i32, u64, v]
    lib.otx_expose.restype = i32


def load() -> ctypes.CDLL:
    """Load the C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"optika_gb300 native library not found at {LIB_PATH}; "
                "run `python -c 'import __graft_entry__ as g; g.build()'` "
                "or `python -m optika_gb300.build` first"
            )
        lib = ctypes.CDLL(str(LIB_PATH))
        _declare(lib)
        if lib.otx_abi_version() != ABI_VERSION:
            raise RuntimeError("optika_gb300 library ABI version mismatch; rebuild it")
        _lib = lib
        check_layout()
    return _lib


def check_layout() -> None:
    """Compare every ctypes structure size with the C compiler's."""
    lib = _lib if _lib is not None else load()
    for which, cls in LAYOUT.items():
        n = lib.otx_sizeof(which)
        if n != ctypes.sizeof(cls):
            raise RuntimeError(
                f"ABI layout mismatch for {cls.__name__}: C {n} bytes, ctypes {ctypes.sizeof(cls)}"
            )


def check(status: int, where: str) -> None:
    if status != OK:
        raise OtxError(status, where)
