"""Host-side logic of the C-ABI that runs before any device call (no GPU): parameter defaults,
argument validation of every session entry point, grid checks of fia_create, error strings."""
import ctypes
import os
import shutil

import pytest

pytestmark = pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                                reason="nvcc not available")

fia = pytest.importorskip("fia")


@pytest.fixture(scope="module")
def lib():
    fia.build()
    return fia.load()


def test_default_advect_params_match_the_python_defaults(lib):
    c = fia.AdvectParams()
    lib.fia_default_advect_params(ctypes.byref(c))
    py = fia.advect_params()
    for name, _ in fia.AdvectParams._fields_:
        assert getattr(c, name) == getattr(py, name), name
    # the benchmark's settings: WENO6, cell-face-aligned split, k = 3, y-integral, zero-velocity
    # correction, no MacCormack, no volume correction, no triangulation
    assert (c.interpolation_method, c.split_method, c.num_gauss_quadrature_point_for_integrate_density) == (0, 0, 3)
    assert (c.use_integral, c.enable_eliminate_zero_velocity_false_diffusion) == (1, 1)
    assert (c.use_MacCormack_scheme, c.enable_cell_volume_correction, c.minimal_area) == (0, 0, 1.0)


def test_default_solver_params_match_the_python_defaults(lib):
    c = fia.SolverParams()
    lib.fia_default_solver_params(ctypes.byref(c))
    py = fia.solver_params()
    for name, _ in fia.SolverParams._fields_:
        assert getattr(c, name) == getattr(py, name), name


def test_null_session_is_rejected_by_every_entry_point(lib):
    p = fia.advect_params()
    sp = fia.solver_params()
    rep = fia.SolverReport()
    step = fia.step_params()
    srep = fia.StepReport()
    d = ctypes.c_double(0.0)
    buf = (ctypes.c_double * 8)()
    u64 = (ctypes.c_ulonglong * 5)()
    n = ctypes.c_ulonglong(0)
    calls = {
        "fia_move_substances_3D": lambda: lib.fia_move_substances_3D(None, 0.01, ctypes.byref(p)),
        "fia_advect_velocity_xyz": lambda: lib.fia_advect_velocity_xyz(None, 0.01, ctypes.byref(p)),
        "fia_calc_pressure_3D": lambda: lib.fia_calc_pressure_3D(None, ctypes.byref(sp), ctypes.byref(rep)),
        "fia_calc_pressure_gradient_term_3D": lambda: lib.fia_calc_pressure_gradient_term_3D(
            None, ctypes.byref(sp), ctypes.byref(rep)),
        "fia_max_abs_velocity": lambda: lib.fia_max_abs_velocity(None, ctypes.byref(d)),
        "fia_step": lambda: lib.fia_step(None, ctypes.byref(step), ctypes.byref(srep)),
        "fia_set_field": lambda: lib.fia_set_field(None, 0, buf, fia.FIA_HOST_F64),
        "fia_get_field": lambda: lib.fia_get_field(None, 0, buf, fia.FIA_HOST_F64),
        "fia_pass_counters": lambda: lib.fia_pass_counters(None, u64),
        "fia_total_momentum": lambda: lib.fia_total_momentum(None, buf),
        "fia_write_density_frame": lambda: lib.fia_write_density_frame(None, b"/nonexistent/frame.fia", 0),
        "fia_append_totals": lambda: lib.fia_append_totals(None, b"/nonexistent/run_", 0.0),
        "fia_debug_clip_fast": lambda: lib.fia_debug_clip_fast(None, 1, ctypes.byref(n)),
        "fia_debug_full_weno": lambda: lib.fia_debug_full_weno(None, 1),
        "fia_debug_piece_pipeline": lambda: lib.fia_debug_piece_pipeline(None, 1),
        "fia_debug_vertex_jitter": lambda: lib.fia_debug_vertex_jitter(None, 1e-7),
    }
    for name, call in calls.items():
        assert call() == fia.FIA_ERR_INVALID, name
    lib.fia_destroy(None)   # a no-op


@pytest.mark.parametrize("args", [(1, 8, 8, 0.1, 0), (8, 8, 0, 0.1, 1), (8, 8, 8, 0.0, 0), (8, 8, 8, -1.0, 1),
                                  (8, 8, 8, 0.1, 7), (2048, 2048, 1024, 1e-3, 1)])
def test_create_rejects_bad_grids_before_touching_the_device(lib, args):
    nx, ny, nz, h, prec = args
    assert not lib.fia_create(nx, ny, nz, ctypes.c_double(h), prec)
    msg = lib.fia_error_string(fia.FIA_ERR_CUDA).decode()
    assert msg.startswith("fia_create:")


def test_error_strings(lib):
    for code in (fia.FIA_OK, fia.FIA_ERR_INVALID, fia.FIA_ERR_UNSUPPORTED, fia.FIA_ERR_NOMEM, 5, -99):
        assert lib.fia_error_string(code)
    assert lib.fia_error_string(fia.FIA_ERR_INVALID).decode() == "invalid argument"


def test_noalloc_entry_point_validates_before_the_device(lib):
    """fia_move_substances_3D_noalloc checks sizes, buffers and flags before it looks up its
    scratch; host addresses stand in for device buffers here, none is dereferenced."""
    f = lib.fia_move_substances_3D_noalloc
    f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] + [ctypes.c_void_p] * 5 + \
        [ctypes.c_double, ctypes.POINTER(fia.AdvectParams), ctypes.c_void_p]
    lib.fia_noalloc_error_string.restype = ctypes.c_char_p
    a, b, u, v, w = (ctypes.addressof(x) for x in [(ctypes.c_double * 1)() for _ in range(5)])
    p = fia.advect_params()

    def call(n=(16, 16, 16), h=1.0 / 16, rho_in=a, rho_out=b, vel=(u, v, w), dt=0.01, params=p):
        return f(*n, h, rho_in, rho_out, *vel, dt, ctypes.byref(params), None)

    cases = [
        (dict(n=(1, 16, 16)), fia.FIA_ERR_INVALID, b"bad grid"),
        (dict(h=0.0), fia.FIA_ERR_INVALID, b"bad grid"),
        (dict(dt=-1.0), fia.FIA_ERR_INVALID, b"time step"),
        (dict(n=(65, 16, 16)), fia.FIA_ERR_INVALID, b"64 cells per axis"),
        (dict(rho_in=None), fia.FIA_ERR_INVALID, b"null buffer"),
        (dict(vel=(u, None, w)), fia.FIA_ERR_INVALID, b"null buffer"),
        (dict(rho_out=a), fia.FIA_ERR_INVALID, b"alias"),
        (dict(params=fia.advect_params(use_MacCormack_scheme=True)), fia.FIA_ERR_UNSUPPORTED, b"MacCormack"),
        (dict(params=fia.advect_params(enable_cell_volume_correction=True)), fia.FIA_ERR_UNSUPPORTED, b"cell-volume"),
        (dict(params=fia.advect_params(num_gauss_quadrature_point_for_integrate_density=2)), fia.FIA_ERR_INVALID,
         b"invalid advection parameters"),
        (dict(params=fia.advect_params(minimal_area=0.0)), fia.FIA_ERR_INVALID, b"invalid advection parameters"),
    ]
    for kw, code, why in cases:
        assert call(**kw) == code, kw
        assert why in lib.fia_noalloc_error_string(), kw


@pytest.mark.parametrize("k", [1, 3, 5, 7, 9, 11, 13, 15])
def test_gauss_rule_is_gauss_legendre_in_the_reference_order(lib, k):
    """The one Gauss rule of the library (the session passes and the allocation-free entry
    point both use it): Gauss-Legendre nodes and weights (numpy's leggauss, weights halved to
    sum 1), ordered centre first then -/+ pairs by increasing |x|, and the oracle's rule."""
    np = pytest.importorskip("numpy")
    x, w = fia.gauss_rule(k)
    lx, lw = np.polynomial.legendre.leggauss(k)
    order = sorted(range(k), key=lambda i: (abs(lx[i]) if abs(lx[i]) > 1e-15 else 0.0, lx[i]))
    np.testing.assert_allclose(x, lx[order], rtol=0, atol=1e-14)
    np.testing.assert_allclose(w, lw[order] / 2.0, rtol=1e-13, atol=0)
    assert abs(w.sum() - 1.0) < 1e-14
    from oracle import Oracle
    ox, ow = Oracle().gauss(k)
    np.testing.assert_allclose(x, ox, rtol=0, atol=1e-15)
    np.testing.assert_allclose(w, ow, rtol=1e-14, atol=0)


@pytest.mark.parametrize("k", [0, 2, 16, 17, -1])
def test_gauss_rule_rejects_even_and_out_of_range_counts(lib, k):
    import numpy as np
    x = np.zeros(20); w = np.zeros(20)
    assert lib.fia_gauss_rule(k, x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                              w.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == fia.FIA_ERR_INVALID


def test_precision_report_arm_specs():
    """The arm grammar of precision_report.py: NAME:PRECISION:TOL[:SOLVER[:DRHO[:DU]]]."""
    import precision_report as pr
    a = pr.parse_arm("p64:fp64:1e-6", 1e-8)
    assert (a["name"], a["precision"], a["tol"], a["solver"], a["drho"], a["du"]) == ("p64", "fp64", 1e-6, "pcg", 0.0, 0.0)
    a = pr.parse_arm("j:fp64:1e-6:pcg:1e-7:6e-8", 1e-8)
    assert (a["drho"], a["du"], a["dv"]) == (1e-7, 6e-8, 0.0)
    a = pr.parse_arm("v:fp64:1e-6:pcg:0:0:1e-7", 1e-8)
    assert (a["drho"], a["du"], a["dv"]) == (0.0, 0.0, 1e-7)
    a = pr.parse_arm("c:fp32c::learned", 1e-8)
    assert (a["tol"], a["solver"]) == (1e-8, "learned")
    for bad in ("x", "x:fp16:1e-6", "x:fp64:1e-6:learned", "x:fp32c:1e-6:amg", "x:fp32c:1e-6:pcg:0:0:1e-7"):
        with pytest.raises(SystemExit):
            pr.parse_arm(bad, 1e-8)
