"""fia_move_substances_3D_noalloc: the density step for callers that cannot allocate device
memory (a host application that owns all device memory, or a real-time loop that must not
allocate).  It runs on the caller's device buffers with its scratch in a static device array.

Checked through the C ABI against the session entry point (fia_move_substances_3D) on two
calls in a row, the second advecting the first's output, within the FP64 parity tolerance
of the other GPU tests (1e-10 relative L2): with the default flags, and for each flag the
allocation-free path handles on its own (interpolation, split method, y-integral, the
zero-velocity passes, the Gauss point count) on cubic and non-cubic grids.  This file is
collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import scenes

fia = pytest.importorskip("fia")

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def noalloc_lib():
    lib = fia.load()
    lib.fia_move_substances_3D_noalloc.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] + [ctypes.c_void_p] * 5 + \
        [ctypes.c_double, ctypes.POINTER(fia.AdvectParams), ctypes.c_void_p]
    lib.fia_noalloc_error_string.restype = ctypes.c_char_p
    return lib


def scene(nx, ny, nz, seed):
    """Fourier velocity (cubic generator, cropped to the grid's faces) and Gaussian blobs."""
    m = max(nx, ny, nz)
    u, v, w = scenes.fourier_velocity(m, seed=seed)
    rho = scenes.gaussian_blobs(m, seed=seed + 1)
    u = u.reshape(m + 1, m, m)[:nx + 1, :ny, :nz]
    v = v.reshape(m, m + 1, m)[:nx, :ny + 1, :nz]
    w = w.reshape(m, m, m + 1)[:nx, :ny, :nz + 1]
    rho = rho.reshape(m, m, m)[:nx, :ny, :nz]
    return [np.ascontiguousarray(a).ravel() for a in (rho, u, v, w)]


def run_both(N, p, seed, dt_cells=2.0):
    """Two chained steps through the session entry point and through the allocation-free one."""
    nx, ny, nz = N
    h = 1.0 / max(N)
    rho, u, v, w = scene(nx, ny, nz, seed)
    dt = dt_cells * h / max(np.abs(u).max(), np.abs(v).max(), np.abs(w).max())
    lib = noalloc_lib()

    ref = fia.Grid3D(nx, ny, nz, h)
    for name, a in (("density", rho), ("u", u), ("v", v), ("w", w)):
        ref.set(name, a)
    ref.move_substances_3D(dt, p)
    first = ref.get("density")
    ref.move_substances_3D(dt, p)
    second = ref.get("density")
    ref.close()

    # the caller's device buffers: the fields of another session (density in, pressure out)
    g = fia.Grid3D(nx, ny, nz, h)
    for name, a in (("density", rho), ("u", u), ("v", v), ("w", w)):
        g.set(name, a)
    g.set("pressure", np.zeros(nx * ny * nz))
    d_rho, d_out = g.device_ptr("density"), g.device_ptr("pressure")
    d_u, d_v, d_w = g.device_ptr("u"), g.device_ptr("v"), g.device_ptr("w")
    stream = g.stream()
    st = lib.fia_move_substances_3D_noalloc(nx, ny, nz, h, d_rho, d_out, d_u, d_v, d_w, dt, ctypes.byref(p), stream)
    assert st == 0, lib.fia_noalloc_error_string()
    got1 = g.get("pressure")
    st = lib.fia_move_substances_3D_noalloc(nx, ny, nz, h, d_out, d_rho, d_u, d_v, d_w, dt, ctypes.byref(p), stream)
    assert st == 0, lib.fia_noalloc_error_string()
    got2 = g.get("density")
    g.close()
    return got1, first, got2, second


def test_noalloc_matches_session_entry_point_twice():
    n = 24
    h = 1.0 / n
    p = fia.advect_params()
    got1, first, got2, second = run_both((n, n, n), p, seed=21)
    assert rel(got1, first) < 1e-10
    assert rel(got2, second) < 1e-10

    # limits are reported, not run
    lib = noalloc_lib()
    g = fia.Grid3D(n, n, n, h)
    d = [g.device_ptr(x) for x in ("density", "pressure", "u", "v", "w")]
    too_big = lib.fia_move_substances_3D_noalloc(65, n, n, h, d[0], d[1], d[2], d[3], d[4], 0.01, ctypes.byref(p),
                                                 g.stream())
    assert too_big == fia.FIA_ERR_INVALID
    assert b"64 cells per axis" in lib.fia_noalloc_error_string()
    alias = lib.fia_move_substances_3D_noalloc(n, n, n, h, d[0], d[0], d[2], d[3], d[4], 0.01, ctypes.byref(p),
                                               g.stream())
    assert alias == fia.FIA_ERR_INVALID
    mac = fia.advect_params(use_MacCormack_scheme=True)
    assert lib.fia_move_substances_3D_noalloc(n, n, n, h, d[0], d[1], d[2], d[3], d[4], 0.01, ctypes.byref(mac),
                                              g.stream()) == fia.FIA_ERR_UNSUPPORTED
    g.close()


CASES = [
    ("linear", (24, 24, 24), dict(interpolation_method="linear", enable_eliminate_zero_velocity_false_diffusion=False)),
    ("xz-AxisAligned", (24, 24, 24), dict(split_method="xz-AxisAligned")),
    ("x-CellFace_z-Axis", (20, 16, 24), dict(split_method="x-CellFaceAligned_z-AxisAligned")),
    ("x-Axis_z-CellFace", (16, 24, 20), dict(split_method="x-AxisAligned_z-CellFaceAligned")),
    ("no_integral", (24, 24, 24), dict(use_integral=False)),
    ("no_zero_velocity_passes", (24, 24, 24), dict(enable_eliminate_zero_velocity_false_diffusion=False)),
    ("k1", (18, 22, 20), dict(num_gauss_quadrature_point_for_integrate_density=1)),
    ("k5", (24, 24, 24), dict(num_gauss_quadrature_point_for_integrate_density=5)),
    ("largest_grid", (64, 64, 64), dict()),
]


@pytest.mark.parametrize("name,N,kw", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_session_entry_point_for_each_flag(name, N, kw):
    p = fia.advect_params(**kw)
    got1, first, got2, second = run_both(N, p, seed=31 + len(name))
    assert rel(got1, first) < 1e-10, name
    assert rel(got2, second) < 1e-10, name
