"""GPU (libfia, FP64 plain form) against the CPU oracle, through the C ABI.

Bar: 1e-10 relative L2 for the flux passes and entry points (the plain form's parity
target), 1e-12 for psi and the backtraced vertex positions.
"""
import os

import numpy as np
import pytest

import scenes
from oracle import Oracle

fia = pytest.importorskip("fia")

pytestmark = pytest.mark.gpu

O = Oracle()


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def make(nx, ny, nz, seed=1, cfl=2.0):
    n = max(nx, ny, nz)
    h = 1.0 / n
    # velocity on the cube of the largest side, cropped to the grid (still a valid MAC field)
    u, v, w = scenes.fourier_velocity(n, seed=seed)
    u = u.reshape(n + 1, n, n)[:nx + 1, :ny, :nz].ravel()
    v = v.reshape(n, n + 1, n)[:nx, :ny + 1, :nz].ravel()
    w = w.reshape(n, n, n + 1)[:nx, :ny, :nz + 1].ravel()
    rho = scenes.gaussian_blobs(n, seed=seed + 1).reshape(n, n, n)[:nx, :ny, :nz].ravel()
    dt = cfl * h
    g = fia.Grid3D(nx, ny, nz, h)
    for name, a in (("density", rho), ("u", u), ("v", v), ("w", w)):
        g.set(name, a)
    return g, h, u, v, w, rho, dt


@pytest.fixture(scope="module")
def cube16():
    g, h, u, v, w, rho, dt = make(16, 16, 16)
    yield g, h, u, v, w, rho, dt
    g.close()


def field_of(comp, rho, u, v, w):
    return rho if comp < 0 else (u, v, w)[comp]


def offsets(comp):
    return (0.5, 0.5, 0.5) if comp < 0 else tuple(0.0 if d == comp else 0.5 for d in range(3))


@pytest.mark.parametrize("comp", [-1, 0, 1, 2])
@pytest.mark.parametrize("mode,k", [(0, 1), (1, 3), (1, 1), (2, 1)])
def test_psi(cube16, comp, mode, k):
    g, h, u, v, w, rho, dt = cube16
    f = field_of(comp, rho, u, v, w)
    M = [16 + (d == comp) for d in range(3)]
    ref = O.psi(f, M, offsets(comp), h, mode, k)
    got = g.debug_psi(comp, f, mode, k)
    assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("comp", [-1, 0, 1, 2])
@pytest.mark.parametrize("interp", [0, 1, 2])
def test_backtrace_vertices(cube16, comp, interp):
    g, h, u, v, w, rho, dt = cube16
    ref = O.backtrace_vertices((16, 16, 16), h, u, v, w, dt, comp, interp)
    got = g.debug_backtrace(comp, dt, interp)
    assert np.abs(got - ref).max() <= 1e-13


PASSES = {  # interp, psi_mode, use_integral, zero_velocity, colour offsets
    "weno6_integral": (0, 1, 1, 0, (0.5, 0.5)),
    "weno6_zero_velocity": (0, 0, 0, 1, (0.5, 0.5)),
    "error_1dy_linear": (2, 0, 0, 0, (0.0, 0.0)),
    "linear_integral": (1, 2, 1, 0, (0.5, 0.5)),
    "weno6_axis_split": (0, 1, 1, 0, (0.0, 0.5)),
}


@pytest.mark.parametrize("name", sorted(PASSES))
@pytest.mark.parametrize("comp", [-1, 0, 1, 2])
def test_flux_pass(cube16, name, comp):
    g, h, u, v, w, rho, dt = cube16
    interp, psi_mode, integ, zv, co = PASSES[name]
    f = field_of(comp, rho, u, v, w)
    ref, ost, nf, npoly = O.flux_pass((16, 16, 16), h, u, v, w, comp, f, dt, interp, psi_mode, integ, zv, co, 3)
    got, st = g.debug_flux_pass(comp, f, dt, interp, psi_mode, integ, zv, co, 3)
    assert st == ost == 0
    assert rel(got, ref) < 1e-10


@pytest.mark.parametrize("interp,k,corr", [("WENO6", 3, True), ("WENO6", 1, False), ("linear", 3, True),
                                           ("WENO6", 5, True)])
def test_move_substances(interp, k, corr):
    g, h, u, v, w, rho, dt = make(16, 16, 16, seed=5)
    p = fia.advect_params(interpolation_method=interp, num_gauss_quadrature_point_for_integrate_density=k,
                          enable_eliminate_zero_velocity_false_diffusion=corr)
    st = g.move_substances_3D(dt, p)
    got = g.get("density")
    ref, ost = O.move_substances_3D((16, 16, 16), h, u, v, w, rho, dt, interp=fia.INTERP[interp], k=k,
                                    correction=int(corr))
    g.close()
    assert st == 0 and ost == 0
    assert rel(got, ref) < 1e-10


@pytest.mark.parametrize("shape", [(12, 10, 8), (7, 9, 6), (24, 16, 20)])
def test_move_substances_ragged_grids(shape):
    g, h, u, v, w, rho, dt = make(*shape, seed=7)
    g.move_substances_3D(dt, fia.advect_params())
    got = g.get("density")
    ref, _ = O.move_substances_3D(shape, h, u, v, w, rho, dt)
    g.close()
    assert rel(got, ref) < 1e-10


def test_move_substances_cfl4_long_faces():
    g, h, u, v, w, rho, dt = make(16, 16, 16, seed=9, cfl=4.0)
    g.move_substances_3D(dt, fia.advect_params())
    got = g.get("density")
    faces, pieces, both_sides, evals, launches = g.pass_counters()
    ref, _ = O.move_substances_3D((16, 16, 16), h, u, v, w, rho, dt)
    g.close()
    assert rel(got, ref) < 1e-10
    assert pieces > faces  # long faces are split


def test_zero_velocity_keeps_interior_constant():
    n = 12
    g = fia.Grid3D(n, n, n, 1.0 / n)
    rho = np.full(n ** 3, 0.7)
    g.set("density", rho)
    for c, s in (("u", (n + 1) * n * n), ("v", n * (n + 1) * n), ("w", n * n * (n + 1))):
        g.set(c, np.zeros(s))
    g.move_substances_3D(0.01, fia.advect_params())
    got = g.get("density")
    z = np.zeros
    ref, _ = O.move_substances_3D((n, n, n), 1.0 / n, z((n + 1) * n * n), z(n * (n + 1) * n), z(n * n * (n + 1)),
                                  rho, 0.01)
    g.close()
    assert rel(got, ref) < 1e-12
    assert np.abs(got - 0.7).max() < 1e-12


def test_advect_velocity():
    g, h, u, v, w, rho, dt = make(12, 12, 12, seed=11, cfl=1.5)
    g.advect_velocity_xyz_flux_advection_3D(dt, fia.advect_params())
    got = [g.get(c) for c in "uvw"]
    ou, ov, ow, _ = O.advect_velocity_3D((12, 12, 12), h, u, v, w, dt)
    g.close()
    for a, b in zip(got, (ou, ov, ow)):
        assert rel(a, b) < 1e-10


def test_advect_velocity_linear_no_correction():
    g, h, u, v, w, rho, dt = make(12, 12, 12, seed=13, cfl=1.5)
    p = fia.advect_params(interpolation_method="linear", enable_eliminate_zero_velocity_false_diffusion=False)
    g.advect_velocity_xyz_flux_advection_3D(dt, p)
    got = [g.get(c) for c in "uvw"]
    ou, ov, ow, _ = O.advect_velocity_3D((12, 12, 12), h, u, v, w, dt, interp=1, correction=0)
    g.close()
    for a, b in zip(got, (ou, ov, ow)):
        assert rel(a, b) < 1e-10


def test_pressure_projection():
    n = 16
    h = 1.0 / n
    rng = np.random.default_rng(3)
    u = rng.normal(size=(n + 1) * n * n); v = rng.normal(size=n * (n + 1) * n); w = rng.normal(size=n * n * (n + 1))
    # closed walls: zero normal velocity on the boundary faces
    u.reshape(n + 1, n, n)[[0, -1]] = 0; v.reshape(n, n + 1, n)[:, [0, -1]] = 0; w.reshape(n, n, n + 1)[:, :, [0, -1]] = 0
    g = fia.Grid3D(n, n, n, h)
    for name, a in (("u", u), ("v", v), ("w", w)):
        g.set(name, a)
    rep = g.calc_pressure_gradient_term_3D(fia.solver_params(tol=1e-12, max_iter=5000))
    p = g.get("pressure")
    b = O.pressure_rhs((n, n, n), h, u, v, w)
    pref, it, rr = O.pressure_solve((n, n, n), b, tol=1e-13)
    assert rep.rel_residual <= 1e-12
    assert rel(p, pref) < 1e-9
    uu, vv, ww = O.subtract_gradient((n, n, n), h, pref, u, v, w)
    for name, ref in (("u", uu), ("v", vv), ("w", ww)):
        assert rel(g.get(name), ref) < 1e-9
    div = scenes.divergence(n, g.get("u"), g.get("v"), g.get("w"))
    assert np.abs(div).max() < 1e-9
    g.close()


def test_cfl_reduction_and_mass():
    g, h, u, v, w, rho, dt = make(10, 12, 14, seed=17)
    assert g.max_abs_velocity() == pytest.approx(O.max_abs_velocity((10, 12, 14), u, v, w), rel=0, abs=0)
    assert g.total_mass() == pytest.approx(rho.sum() * h ** 3, rel=1e-13)
    g.close()


@pytest.mark.parametrize("interp,corr,shape", [("WENO6", True, (16, 16, 16)), ("WENO6", False, (16, 16, 16)),
                                               ("linear", True, (16, 16, 16)), ("WENO6", True, (7, 9, 6))])
def test_move_substances_maccormack(interp, corr, shape):
    """The flux MacCormack scheme (faces at rest, backtraced and traced back, weights 0.5, 1,
    -0.5) against the oracle, which follows the reference's branch and is pinned against the
    reference's own code (tests/test_oracle_golden.py)."""
    g, h, u, v, w, rho, dt = make(*shape, seed=5)
    p = fia.advect_params(interpolation_method=interp, enable_eliminate_zero_velocity_false_diffusion=corr,
                          use_MacCormack_scheme=True)
    st = g.move_substances_3D(dt, p)
    got = g.get("density")
    g.close()
    ref, ost = O.move_substances_3D(shape, h, u, v, w, rho, dt, interp=fia.INTERP[interp], k=3,
                                    correction=int(corr), maccormack=1)
    plain, _ = O.move_substances_3D(shape, h, u, v, w, rho, dt, interp=fia.INTERP[interp], k=3,
                                    correction=int(corr))
    assert st == 0 and ost == 0
    assert rel(got, ref) < 1e-10
    assert rel(got, plain) > 1e-3      # the scheme is in effect


def test_advect_velocity_maccormack():
    g, h, u, v, w, rho, dt = make(12, 12, 12, seed=11, cfl=1.5)
    g.advect_velocity_xyz_flux_advection_3D(dt, fia.advect_params(use_MacCormack_scheme=True))
    got = [g.get(c) for c in "uvw"]
    g.close()
    ou, ov, ow, _ = O.advect_velocity_3D((12, 12, 12), h, u, v, w, dt, maccormack=1)
    for a, b in zip(got, (ou, ov, ow)):
        assert rel(a, b) < 1e-10


@pytest.mark.parametrize("mc", [False, True])
def test_move_substances_volume_correction(mc):
    """the cell-volume correction (move_substances_3d.cpp:243-493) against the oracle; both solve
    the volume Poisson problem to a tight tolerance (the reference stops its AMG-CG at 0.1)"""
    g, h, u, v, w, rho, dt = make(16, 16, 16, seed=5)
    st = g.move_substances_3D(dt, fia.advect_params(enable_cell_volume_correction=True, use_MacCormack_scheme=mc))
    got = g.get("density")
    mass = g.total_mass()
    g.close()
    ref, ost = O.move_substances_3D((16, 16, 16), h, u, v, w, rho, dt, maccormack=int(mc), volume_correction=1)
    plain, _ = O.move_substances_3D((16, 16, 16), h, u, v, w, rho, dt, maccormack=int(mc))
    assert st == 0 and ost == 0
    assert rel(got, ref) < 1e-10
    assert rel(got, plain) > 1e-2
    assert abs(mass - plain.sum() * h ** 3) < 1e-12 * mass


def test_invalid_arguments_fail_loudly():
    g = fia.Grid3D(8, 8, 8, 1.0 / 8)
    with pytest.raises(fia.FiaError):
        g.move_substances_3D(0.01, fia.advect_params(minimal_area=0.0))
    with pytest.raises(fia.FiaError):
        g.move_substances_3D(0.01, fia.advect_params(num_gauss_quadrature_point_for_integrate_density=2))
    with pytest.raises(fia.FiaError):
        g.set("u", np.zeros(5))
    g.close()


def test_fp64_weno_collapse_matches_full_evaluation():
    """The plain form collapses WENO6 along the axes on which a point lies on a node plane
    (vertices at rest, psi points, faces at rest); the full evaluation gives the same steps to
    rounding (the collapse is exact in real arithmetic)."""
    outs = []
    for full in (1, 0):
        g, h, u, v, w, rho, dt = make(20, 16, 18, seed=9)
        assert g.debug_full_weno(full) == full
        g.move_substances_3D(dt, fia.advect_params())
        g.advect_velocity_xyz_flux_advection_3D(dt, fia.advect_params())
        outs.append([g.get(c) for c in ("density", "u", "v", "w")])
        g.close()
    for a, b in zip(*outs):
        assert rel(a, b) < 1e-13


PIPE_CASES = [
    ("default", dict(), 2.0),
    ("maccormack_volumes", dict(use_MacCormack_scheme=True, enable_cell_volume_correction=True), 2.0),
    ("triangulated_k5_cfl4", dict(minimal_area=0.05, num_gauss_quadrature_point_for_integrate_density=5), 4.0),
    ("linear_no_integral", dict(interpolation_method="linear", use_integral=False), 2.0),
]


@pytest.mark.parametrize("name,kw,cfl", PIPE_CASES, ids=[c[0] for c in PIPE_CASES])
def test_fp64_piece_pipeline_matches_per_face_kernel(name, kw, cfl):
    """The plain form's piece pipeline (clip and store, a thread per piece, ordered face sums)
    against one thread per face evaluating each piece as it is clipped: the same pieces, the
    same per-piece arithmetic and the same order of every sum, so the same steps to rounding
    (triangulated polygons are summed flat instead of per polygon); with a store too small
    for the pass, the pipeline grows it and clips again."""
    p = fia.advect_params(**kw)
    outs, counts, stats = [], [], []
    for pipe in (0, 1, 1):
        g, h, u, v, w, rho, dt = make(20, 16, 18, seed=11, cfl=cfl)
        assert g.debug_piece_pipeline(pipe) == pipe
        if pipe and len(outs) == 2:
            g.debug_set_piece_capacity(100)      # far too small: grown by the first pass
        c0 = g.pass_counters()
        stats.append(g.move_substances_3D(dt, p))
        c1 = g.pass_counters()
        g.advect_velocity_xyz_flux_advection_3D(dt, p)
        outs.append([g.get(c) for c in ("density", "u", "v", "w")])
        counts.append([c1[i] - c0[i] for i in range(3)])
        if pipe and len(outs) == 3:
            assert g.debug_piece_capacity() > 100, name   # grown
        g.close()
    for a, b, c in zip(*outs):
        assert rel(b, a) < 1e-14, name
        assert np.array_equal(b, c), name
    assert counts[0] == counts[1], name            # faces, pieces, faces clipped twice
    assert stats[0] == stats[1] == stats[2], name


def test_fp64_vertex_jitter_is_a_small_perturbation():
    """The sensitivity hook of the plain form: backtraced vertices jittered by 1e-7 cells change
    a density step by a small nonzero amount; switched off, the step is the plain one."""
    outs = []
    for amp in (0.0, 1e-7, 0.0):
        g, h, u, v, w, rho, dt = make(16, 16, 16, seed=13)
        if amp:
            g.debug_vertex_jitter(amp)
        g.move_substances_3D(dt, fia.advect_params())
        outs.append(g.get("density"))
        g.close()
    assert np.array_equal(outs[0], outs[2])
    assert 0.0 < rel(outs[1], outs[0]) < 1e-4
    with pytest.raises(fia.FiaError):
        g32 = fia.Grid3D(8, 8, 8, 1.0 / 8, precision=fia.FIA_FP32C)
        try:
            g32.debug_vertex_jitter(1e-7)
        finally:
            g32.close()


@pytest.mark.parametrize("cfl", [2.0, 4.0])
@pytest.mark.parametrize("name,interp,psi_mode,integ,co", [("main", 0, 1, 1, (0.5, 0.5)),
                                                          ("error", 2, 0, 0, (0.0, 0.0))])
def test_fp64_triangulated_passes_match_oracle(cfl, name, interp, psi_mode, integ, co):
    """minimal_area 0.05: pieces triangulated by longest-edge bisection (facecutter.h:255-324).
    The plain form against the oracle on a developed flow.  The library clips each face once,
    in the lower cell's vertex order, the oracle from both cells; where two edges are equally
    long the first one is bisected, and the first depends on the vertex order, so a few cells
    differ (measured 5e-9 to 9e-6 relative L2 over the grid); everywhere else 1e-14."""
    n = 24
    h = 1.0 / n
    u, v, w = scenes.fourier_velocity(n, seed=7)
    rho = scenes.gaussian_blobs(n, seed=8)
    dt = cfl * h
    ref, ost, _, _ = O.flux_pass((n, n, n), h, u, v, w, -1, rho, dt, interp, psi_mode, integ, 0, co, 3,
                                 minimal_area=0.05, nthreads=os.cpu_count() or 1)
    g = fia.Grid3D(n, n, n, h)
    for nm, a in (("density", rho), ("u", u), ("v", v), ("w", w)):
        g.set(nm, a)
    got, st = g.debug_flux_pass(-1, rho, dt, interp, psi_mode, integ, 0, co, 3, minimal_area=0.05)
    g.close()
    assert st == 0 and ost == 0
    d = np.abs(got - ref)
    keep = np.argsort(d)[:-8]
    assert np.linalg.norm((got - ref)[keep]) / np.linalg.norm(ref) < 1e-12
    assert rel(got, ref) < 5e-5
