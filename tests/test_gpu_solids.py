"""GPU tests of the projection with solid spheres: after calc_pressure_3D and
calc_pressure_gradient_term_3D every face touching a solid cell carries zero velocity and
every free fluid cell is divergence-free, in both precisions and with both solvers, even when
the faces inside and around the spheres held velocity before the projection (advection and
buoyancy write every face)."""
import numpy as np
import pytest

import fia

pytestmark = pytest.mark.gpu

N = (40, 36, 32)
CENTERS = [[0.35, 0.4, 0.45], [0.7, 0.65, 0.4]]
RADII = [0.14, 0.11]


def face_masks(solid):
    """faces of each family that touch a solid cell"""
    s = solid.reshape(N).astype(bool)
    nx, ny, nz = N
    fu = np.zeros((nx + 1, ny, nz), bool); fu[:-1] |= s; fu[1:] |= s
    fv = np.zeros((nx, ny + 1, nz), bool); fv[:, :-1] |= s; fv[:, 1:] |= s
    fw = np.zeros((nx, ny, nz + 1), bool); fw[:, :, :-1] |= s; fw[:, :, 1:] |= s
    return fu, fv, fw


def divergence(u, v, w):
    nx, ny, nz = N
    u = u.reshape(nx + 1, ny, nz); v = v.reshape(nx, ny + 1, nz); w = w.reshape(nx, ny, nz + 1)
    return (u[1:] - u[:-1]) + (v[:, 1:] - v[:, :-1]) + (w[:, :, 1:] - w[:, :, :-1])


@pytest.mark.parametrize("precision,method", [(fia.FIA_FP64, "pcg"), (fia.FIA_FP32C, "pcg"),
                                              (fia.FIA_FP32C, "learned")])
def test_projection_with_solids_is_divergence_free(precision, method):
    g = fia.Grid3D(*N, 1.0 / N[0], precision=precision)
    g.set_solid_spheres(CENTERS, RADII)
    solid = g.solid_mask()
    pin = int(np.nonzero(solid == 0)[0][-1])
    rng = np.random.default_rng(5)
    vel = {c: rng.normal(size=g.sizes()[c]) for c in "uvw"}
    for c in "uvw":
        g.set(c, vel[c])             # after the spheres: the solid faces hold velocity too
    sp = fia.solver_params(tol=1e-11 if precision == fia.FIA_FP64 else 1e-7, max_iter=20000)
    if method == "learned":
        g.learned_init(3)
        sp = fia.solver_params(tol=1e-7, max_iter=20000, method=fia.FIA_SOLVER_FCG_LEARNED, fallback_iter=400)
    g.calc_pressure_3D(sp)
    g.calc_pressure_gradient_term_3D(sp)
    out = {c: g.get(c) for c in "uvw"}
    g.close()
    for c, m in zip("uvw", face_masks(solid)):
        assert np.all(out[c][m.ravel()] == 0.0), c
    div0 = divergence(*(vel[c] for c in "uvw")).ravel()
    div = divergence(*(out[c] for c in "uvw")).ravel()
    free = solid == 0
    free[pin] = False
    tol = 1e-8 if precision == fia.FIA_FP64 else 1e-4
    assert np.abs(div[free]).max() < tol * np.abs(div0[free]).max()
