"""fia_move_substances_3D_noalloc: the density step for callers that cannot allocate device
memory (a host application that owns all device memory, or a real-time loop that must not
allocate).  It runs on the caller's device buffers with its scratch in a static device array.

Checked through the C ABI against the session entry point (fia_move_substances_3D) on two
calls in a row, the second advecting the first's output, within the FP64 parity tolerance
of the other GPU tests (1e-10 relative L2).  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import scenes

fia = pytest.importorskip("fia")

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_noalloc_matches_session_entry_point_twice():
    n = 24
    h = 1.0 / n
    u, v, w = scenes.fourier_velocity(n, seed=21)
    rho = scenes.gaussian_blobs(n, seed=22)
    dt = 2.0 * h
    p = fia.advect_params()
    lib = fia.load()
    lib.fia_move_substances_3D_noalloc.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] + [ctypes.c_void_p] * 5 + \
        [ctypes.c_double, ctypes.POINTER(fia.AdvectParams), ctypes.c_void_p]
    lib.fia_noalloc_error_string.restype = ctypes.c_char_p

    # reference: the session entry point, twice
    ref = fia.Grid3D(n, n, n, h)
    for name, a in (("density", rho), ("u", u), ("v", v), ("w", w)):
        ref.set(name, a)
    ref.move_substances_3D(dt, p)
    first = ref.get("density")
    ref.move_substances_3D(dt, p)
    second = ref.get("density")
    ref.close()

    # the caller's device buffers: the fields of another session (density in, pressure out)
    g = fia.Grid3D(n, n, n, h)
    for name, a in (("density", rho), ("u", u), ("v", v), ("w", w)):
        g.set(name, a)
    g.set("pressure", np.zeros(n ** 3))
    d_rho, d_out = g.device_ptr("density"), g.device_ptr("pressure")
    d_u, d_v, d_w = g.device_ptr("u"), g.device_ptr("v"), g.device_ptr("w")
    stream = g.stream()
    st = lib.fia_move_substances_3D_noalloc(n, n, n, h, d_rho, d_out, d_u, d_v, d_w, dt, ctypes.byref(p), stream)
    assert st == 0, lib.fia_noalloc_error_string()
    got1 = g.get("pressure")
    st = lib.fia_move_substances_3D_noalloc(n, n, n, h, d_out, d_rho, d_u, d_v, d_w, dt, ctypes.byref(p), stream)
    assert st == 0, lib.fia_noalloc_error_string()
    got2 = g.get("density")

    # limits are reported, not run
    too_big = lib.fia_move_substances_3D_noalloc(65, n, n, h, d_rho, d_out, d_u, d_v, d_w, dt, ctypes.byref(p),
                                                 stream)
    assert too_big == fia.FIA_ERR_INVALID
    assert b"64 cells per axis" in lib.fia_noalloc_error_string()
    g.close()

    assert rel(got1, first) < 1e-10
    assert rel(got2, second) < 1e-10
