"""The C-ABI library: builds, loads, exports every declared symbol, matches
the ctypes layouts, and rejects bad descriptors on the host (no GPU work)."""

import ctypes
import pathlib
import re

import pytest

from optika_gb300 import _lib as L

ROOT = pathlib.Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(otx_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported(built_library):
    names = declared_symbols()
    assert "otx_trace_grid" in names and "otx_trace_rays" in names
    for n in names:
        assert hasattr(built_library, n), f"{n} declared in include/ but not exported"


def test_layouts_match(built_library):
    L.check_layout()
    for which, cls in L.LAYOUT.items():
        assert built_library.otx_sizeof(which) == ctypes.sizeof(cls)
    assert built_library.otx_sizeof(99) == -1
    # the system descriptor is passed as a kernel parameter (<= 32 KB)
    assert ctypes.sizeof(L.System) < 32 * 1024


def test_status_strings(built_library):
    for s in range(6):
        assert built_library.otx_status_string(s)


def _system(n=1):
    s = L.System()
    s.abi_version = L.ABI_VERSION
    s.num_surfaces = n
    s.input_mode = L.INPUT_GRID_INFINITY
    for k in range(L.MAX_LAYERS):
        s.layers[k].table = -1
    for k in range(L.MAX_STACKS):
        s.stacks[k].substrate = -1
    return s


def _call_rays(lib, sys_, count=0):
    rin = L.Rays()
    rin.count = count
    rout = L.Rays()
    return lib.otx_trace_rays(ctypes.byref(sys_), ctypes.byref(rin), ctypes.byref(rout), None,
                              None, None)


@pytest.mark.parametrize(
    "mutate,expected",
    [
        (lambda s: setattr(s, "abi_version", 0), L.ERR_INVALID),
        (lambda s: setattr(s, "num_surfaces", 0), L.ERR_SIZE),
        (lambda s: setattr(s, "num_surfaces", L.MAX_SURFACES + 1), L.ERR_SIZE),
        (lambda s: setattr(s.surfaces[0], "sag_type", 99), L.ERR_UNSUPPORTED),
        (lambda s: setattr(s.surfaces[0], "mat_type", 99), L.ERR_UNSUPPORTED),
        (lambda s: setattr(s.surfaces[0], "aper_type", 99), L.ERR_UNSUPPORTED),
        (lambda s: setattr(s.surfaces[0], "rule_type", 99), L.ERR_UNSUPPORTED),
        (lambda s: (setattr(s.surfaces[0], "mat_type", L.MAT_MULTILAYER_MIRROR),
                    setattr(s.surfaces[0], "mat_stack", 7)), L.ERR_INVALID),
        (lambda s: (setattr(s.surfaces[0], "aper_type", L.APER_POLYGON),
                    setattr(s.surfaces[0], "aper_vertex_count", 2)), L.ERR_INVALID),
        (lambda s: (setattr(s.surfaces[0], "rule_type", L.RULE_POLY1D),
                    setattr(s.surfaces[0], "rule_num_terms", 9)), L.ERR_SIZE),
        (lambda s: setattr(s.layers[0], "table", 3), L.ERR_INVALID),
        (lambda s: setattr(s.surfaces[0], "sag_type", L.SAG_CYLINDER + 1), L.ERR_UNSUPPORTED),
        (lambda s: setattr(s.surfaces[0], "mat_type", L.MAT_MEASURED_MIRROR + 1),
         L.ERR_UNSUPPORTED),
        (lambda s: (setattr(s.surfaces[0], "mat_type", L.MAT_MEASURED_MIRROR),
                    setattr(s.surfaces[0], "mat_table", 16)), L.ERR_INVALID),
        (lambda s: (setattr(s.surfaces[0], "mat_type", L.MAT_MEASURED_MIRROR),
                    setattr(s.surfaces[0], "mat_table", 0)), L.ERR_INVALID),  # empty table
        (lambda s: (setattr(s.surfaces[0], "rule_type", L.RULE_CONSTANT),
                    setattr(s.surfaces[0], "rule_eff_type", 7)), L.ERR_UNSUPPORTED),
        (lambda s: (setattr(s.surfaces[0], "rule_type", L.RULE_CONSTANT),
                    setattr(s.surfaces[0], "rule_eff_type", L.RULE_EFF_MEASURED),
                    setattr(s.surfaces[0], "rule_table", -1)), L.ERR_INVALID),
        (lambda s: (setattr(s.stacks[0], "pre_count", 5),
                    setattr(s.stacks[0], "pre_begin", L.MAX_LAYERS - 2)), L.ERR_INVALID),
    ],
)
def test_bad_descriptors_rejected(built_library, mutate, expected):
    s = _system()
    mutate(s)
    assert _call_rays(built_library, s) == expected


def test_empty_input_is_ok_without_launch(built_library):
    assert _call_rays(built_library, _system(), count=0) == L.OK


def test_missing_pointers_rejected(built_library):
    assert _call_rays(built_library, _system(), count=10) == L.ERR_INVALID
    g = L.Grid()
    g.count = 5
    out = L.Rays()
    s = _system()
    assert built_library.otx_trace_grid(ctypes.byref(s), ctypes.byref(g), ctypes.byref(out),
                                        None, None, None) == L.ERR_INVALID
    s.input_mode = L.INPUT_RAYS
    g.count = 0
    assert built_library.otx_trace_grid(ctypes.byref(s), ctypes.byref(g), ctypes.byref(out),
                                        None, None, None) == L.ERR_INVALID


def test_bad_launch_and_image(built_library):
    s = _system()
    rin = L.Rays()
    rin.count = 0
    out = L.Rays()
    img = L.Image()
    img.counts = 1  # non-null: the sensor must then be valid
    assert built_library.otx_trace_rays(ctypes.byref(s), ctypes.byref(rin), ctypes.byref(out),
                                        ctypes.byref(img), None, None) == L.ERR_INVALID
    ln = L.Launch()
    ln.rays_per_thread = 3
    assert built_library.otx_trace_rays(ctypes.byref(s), ctypes.byref(rin), ctypes.byref(out),
                                        None, ctypes.byref(ln), None) in (L.OK, L.ERR_INVALID)


def test_collect_and_sag_validation(built_library):
    sen = L.Sensor()
    r = L.Rays()
    img = L.Image()
    assert built_library.otx_collect(ctypes.byref(sen), ctypes.byref(r), ctypes.byref(img),
                                     None) == L.ERR_INVALID
    s = _system()
    assert built_library.otx_sag_eval(ctypes.byref(s), 5, ctypes.byref(r), ctypes.byref(r),
                                      None) == L.ERR_INVALID
    s.surfaces[0].sag_type = 42
    assert built_library.otx_sag_eval(ctypes.byref(s), 0, ctypes.byref(r), ctypes.byref(r),
                                      None) == L.ERR_UNSUPPORTED


def test_host_trace_validation(built_library):
    """otx_trace_grid_host rejects bad arguments before any device work."""
    lib = built_library
    s = _system()
    x = (ctypes.c_float * 8)()
    g = L.Grid()
    g.count = 8
    for k in ("wavelength", "field_x", "field_y", "pupil_x", "pupil_y"):
        setattr(g, k, ctypes.addressof(x))
    g.stride_wavelength = g.stride_field = g.stride_pupil = 1
    out = L.Rays()
    need = lib.otx_trace_grid_host_workspace(ctypes.byref(g), ctypes.byref(out), 1)
    assert need > 0
    assert lib.otx_trace_grid_host_workspace(ctypes.byref(g), ctypes.byref(out), 0) == -1

    def call(grid, ws, nbytes, sys_=s, ln=None):
        return lib.otx_trace_grid_host(ctypes.byref(sys_), ctypes.byref(grid), ctypes.byref(out),
                                       None, ln, ws, nbytes, None)

    # host input strides other than 0 and 1
    g.stride_pupil = 2
    assert call(g, 256, need) == L.ERR_INVALID
    g.stride_pupil = 1
    # no workspace, unaligned workspace, a workspace too small for one ray
    assert call(g, None, need) == L.ERR_INVALID
    assert call(g, 257, need) == L.ERR_INVALID
    assert call(g, 256, 64) == L.ERR_SIZE
    # a rays-input system, bad launch shape
    s2 = _system()
    s2.input_mode = L.INPUT_RAYS
    assert call(g, 256, need, sys_=s2) == L.ERR_INVALID
    ln = L.Launch()
    ln.rays_per_thread = 3
    assert call(g, 256, need, ln=ctypes.byref(ln)) == L.ERR_INVALID
    # empty input: nothing to do, no device call
    g.count = 0
    assert call(g, None, 0) == L.OK


def test_fused_surrogate_validation(built_library):
    """otx_surrogate_image_fused rejects bad arguments before any device work."""
    lib = built_library
    s = _system(4)
    s.flags = L.SYS_FLAG_FINAL_IDENTITY
    b = L.Batch()
    b.num_configs = 2
    b.ray_offset = 256
    sg = L.Surrogate()
    sg.num_configs = 2
    sg.config_inputs = sg.baseline = 256
    sg.out_scale = 0.005
    net = L.Mlp()
    net.num_inputs, net.num_hidden, net.width, net.num_outputs = 9, 4, 256, 3
    for l in range(5):
        net.w[l] = 4096 * (l + 1)
        net.b[l] = 4096 * (l + 9)
        net.ld[l] = 16 if l == 0 else 256
    need = lib.otx_surrogate_image_fused_workspace(ctypes.byref(b), ctypes.byref(net), 1000)
    assert need >= 4000 and need % 256 == 0
    assert lib.otx_surrogate_image_fused_workspace(None, ctypes.byref(net), 10) == -1

    def call(count=1000, ws=256, nbytes=need, net_=net, sys_=s):
        return lib.otx_surrogate_image_fused(ctypes.byref(sys_), ctypes.byref(b), ctypes.byref(sg),
                                             ctypes.byref(net_), 0, count, None, None, ws, nbytes,
                                             256, 256, None)

    assert call(count=0) == L.OK  # nothing to do, no device call
    assert call(ws=None) == L.ERR_INVALID
    assert call(ws=257) == L.ERR_INVALID
    assert call(nbytes=need - 1) == L.ERR_INVALID
    net2 = L.Mlp.from_buffer_copy(net)
    net2.width = 128
    assert call(net_=net2) == L.ERR_UNSUPPORTED
    net2 = L.Mlp.from_buffer_copy(net)
    net2.ld[1] = 100
    assert call(net_=net2) == L.ERR_INVALID
    s2 = _system(4)
    assert call(sys_=s2) == L.ERR_UNSUPPORTED  # outputs must be in the sensor frame
    # more configurations than the fallback grid's y dimension holds
    b.num_configs = sg.num_configs = 65536
    assert call() == L.ERR_SIZE
    b.num_configs = sg.num_configs = 2


def test_rulings_cells_expose_reduce_validation(built_library):
    """The entry points added for the rulings, the forward model and the
    calibration fits reject bad arguments on the host."""
    lib = built_library
    s = _system()
    r = L.Rays()
    # rulings: no rulings on the surface, bad mode
    assert lib.otx_rulings_eval(ctypes.byref(s), 0, ctypes.byref(r), ctypes.byref(r), None,
                                None, None) == L.ERR_INVALID
    s.surfaces[0].rule_type = L.RULE_CONSTANT
    assert lib.otx_rulings_eval(ctypes.byref(s), 2, ctypes.byref(r), ctypes.byref(r), None,
                                None, None) == L.ERR_INVALID
    assert lib.otx_rulings_eval(ctypes.byref(s), 0, ctypes.byref(r), ctypes.byref(r), None,
                                None, None) == L.OK  # empty input, no launch
    r.count = 4
    assert lib.otx_rulings_eval(ctypes.byref(s), 0, ctypes.byref(r), ctypes.byref(r), None,
                                None, None) == L.ERR_INVALID  # missing pointers
    # cells: bad dimensions, range past the end, missing tables
    c = L.Cells()
    g = L.Grid()
    assert lib.otx_cell_rays(ctypes.byref(c), 0, 1, ctypes.byref(g), None) == L.ERR_INVALID
    c.nw = c.nfx = c.nfy = c.npx = c.npy = 2
    assert lib.otx_cell_rays(ctypes.byref(c), 30, 3, ctypes.byref(g), None) == L.ERR_SIZE
    assert lib.otx_cell_rays(ctypes.byref(c), 0, 0, ctypes.byref(g), None) == L.OK
    assert lib.otx_cell_rays(ctypes.byref(c), 0, 8, ctypes.byref(g), None) == L.ERR_INVALID
    assert lib.otx_cell_rays(ctypes.byref(c), -1, 8, ctypes.byref(g), None) == L.ERR_INVALID
    # exposure
    assert lib.otx_expose(None, None, -1, 1.0, 0.0, 1, 0, None) == L.ERR_INVALID
    assert lib.otx_expose(None, None, 0, 1.0, 0.0, 1, 0, None) == L.OK
    assert lib.otx_expose(None, None, 5, 1.0, 0.0, 1, 0, None) == L.ERR_INVALID
    # pupil reduction: count must be groups x per_group, pointers present
    rr = L.Rays()
    rr.count = 10
    assert lib.otx_pupil_reduce(ctypes.byref(rr), 2, 5, None, None) == L.ERR_INVALID
    assert lib.otx_pupil_reduce(ctypes.byref(rr), 0, 5, None, None) == L.OK
    assert lib.otx_pupil_reduce(ctypes.byref(rr), 2, 0, None, None) == L.ERR_INVALID


def test_stop_newton_and_trace_cells_validation(built_library):
    """The device stop solve and the fused cell trace reject bad arguments
    on the host and return at once on empty inputs."""
    lib = built_library
    s = _system(2)
    first = _system(1)
    sol = L.StopSolve()
    sol.max_iterations, sol.polish_steps, sol.step, sol.tolerance = 60, 2, 1e-4, 1e-9
    call = lambda: lib.otx_stop_newton(ctypes.byref(s), ctypes.byref(first),  # noqa: E731
                                       ctypes.byref(sol), None)
    assert call() == L.OK  # count 0: no device work
    assert lib.otx_stop_newton(None, ctypes.byref(first), ctypes.byref(sol), None) == L.ERR_INVALID
    sol.count = 10
    assert call() == L.ERR_INVALID  # arrays missing
    for k in ("position", "direction", "wavelength", "target_x", "target_y", "status"):
        setattr(sol, k, 256)
    sol.tolerance = 0.0
    assert call() == L.ERR_INVALID
    sol.tolerance, sol.max_iterations = 1e-9, 0
    assert call() == L.ERR_INVALID
    # fused cell trace: the image is its output; cells checked as otx_cell_rays
    c = L.Cells()
    c.nw = c.nfx = c.nfy = c.npx = c.npy = 2
    img = L.Image()
    launch = L.Launch()
    fn = lambda first_, count, image: lib.otx_trace_cells(  # noqa: E731
        ctypes.byref(s), ctypes.byref(c), first_, count, image, ctypes.byref(launch), None)
    assert fn(0, 4, ctypes.byref(img)) == L.ERR_INVALID  # no image buffer
    img.counts = 256
    s.sensor.num_x = s.sensor.num_y = s.sensor.num_w = 4
    s.sensor.width_x = s.sensor.width_y = 0.01
    assert fn(0, 0, ctypes.byref(img)) == L.OK  # empty: no device work
    assert fn(30, 3, ctypes.byref(img)) == L.ERR_SIZE  # past the last cell
    assert fn(0, 8, ctypes.byref(img)) == L.ERR_INVALID  # tables missing
    s.input_mode = L.INPUT_RAYS
    assert fn(0, 0, ctypes.byref(img)) == L.ERR_INVALID  # grid systems only
