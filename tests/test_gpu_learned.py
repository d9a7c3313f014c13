"""GPU tests of the learned pressure preconditioner against its CPU oracle
(oracle/unet_oracle.py): network forward, parameter gradients, the two-level
preconditioner, the energy-norm loss, one Adam step, and flexible CG with the fallback."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import fia  # noqa: E402
import unet_oracle as U  # noqa: E402

pytestmark = pytest.mark.gpu

FINE = (24, 20, 22)


def rel(a, b):
    a = np.asarray(a, dtype=np.float64).ravel(); b = np.asarray(b, dtype=np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def session(fine=FINE, seed=7):
    g = fia.Grid3D(*fine, 1.0 / fine[0], precision=fia.FIA_FP32C)
    g.learned_init(seed)
    return g


def test_level_dims():
    g = session()
    assert [g.learned_level_dims(l) for l in range(4)] == U.level_dims(FINE)
    assert fia.num_learned_parameters() == U.num_parameters()
    g.close()


def test_unet_forward_matches_oracle():
    g = session()
    w = g.learned_get_weights().astype(np.float64)
    dims = U.level_dims(FINE)
    x0 = np.random.default_rng(1).normal(size=dims[0]).astype(np.float32)
    y = g.debug_unet_forward(x0)
    yo = U.UNet(w, FINE, rounding=True).forward(x0)
    g.close()
    assert np.all(np.isfinite(y))
    assert rel(y, yo) < 5e-3


@pytest.mark.parametrize("fine", [(160, 144, 136), (320, 256, 128)])
def test_tensor_core_convolutions_match_mma_path(fine):
    """The tcgen05 convolutions against the mma.sync kernel (checked against the oracle above)
    on the same weights and input.  The two sizes cover one and two x-planes per CTA, weight
    chunks of 27, 14, 9, 3 and 1 taps, plain, pooled and upsampled-concatenated inputs, 16 to 48
    output channels and the single FP32 output channel, and ragged tiles in y and z."""
    g = fia.Grid3D(*fine, 1.0 / fine[0], precision=fia.FIA_FP32C)
    g.learned_init(5)
    dims = tuple(g.learned_level_dims(0))
    x0 = np.random.default_rng(4).normal(size=dims).astype(np.float32)
    assert g.debug_learned_tc(1) == 0
    y_tc = g.debug_unet_forward(x0)
    st = g.debug_learned_tc(0)
    y_ref = g.debug_unet_forward(x0)
    g.close()
    assert st == 0
    assert np.all(np.isfinite(y_tc))
    assert rel(y_tc, y_ref) < 1e-2


def test_unet_gradients_match_oracle():
    g = session(seed=11)
    w = g.learned_get_weights().astype(np.float64)
    dims = U.level_dims(FINE)
    rng = np.random.default_rng(2)
    x0 = rng.normal(size=dims[0]).astype(np.float32)
    gy = rng.normal(size=dims[0]).astype(np.float32)
    gp = g.debug_unet_backward(x0, gy)
    net = U.UNet(w, FINE, rounding=True)
    net.forward(x0)
    go = net.backward(gy)
    g.close()
    o = 0
    for i, (lev, cin, cout, *_r) in enumerate(U.LAYERS):
        n = 27 * cin * cout
        assert rel(gp[o:o + n], go[o:o + n]) < 2e-2, "layer %d" % i
        o += n


def solid_session(fine=FINE):
    g = session(fine)
    h = 1.0 / fine[0]
    g.set_solid_spheres([[0.4, 0.45, 0.5], [0.75, 0.3, 0.3]], [0.15, 0.12])
    m = g.solid_mask()
    pin = int(np.nonzero(m == 0)[0][-1])
    return g, m, pin, h


def test_precondition_matches_oracle():
    g, m, pin, _ = solid_session()
    w = g.learned_get_weights().astype(np.float64)
    r = np.random.default_rng(3).normal(size=FINE).astype(np.float32)
    r.reshape(-1)[m.astype(bool)] = 0.0
    r.reshape(-1)[pin] = 0.0
    z = g.debug_precondition(r.ravel())
    zo = U.precondition(w, r, FINE, pin, m, rounding=True)
    g.close()
    assert rel(z, zo) < 5e-3


def pair(fine, pin, m, seed):
    """a smooth pressure (white noise filtered at 3 cells) and its right-hand side: the BF16
    network's gradient is well conditioned for it (for white-noise pressures the layer
    gradients move by several percent with the FP32 summation order alone)"""
    ndimage = pytest.importorskip("scipy.ndimage")
    rng = np.random.default_rng(seed)
    p = ndimage.gaussian_filter(rng.normal(size=fine), 3.0)
    p[U.excluded_mask(fine, pin, m)] = 0.0
    r = U.apply_B(p, fine, pin, m)
    return r, p


def test_loss_gradient_and_adam_step_match_oracle():
    g, m, pin, _ = solid_session()
    w0 = g.learned_get_weights().astype(np.float64)
    r, p = pair(FINE, pin, m, 5)
    g.learned_add_pair(r.ravel(), p.ravel())
    loss = g.learned_loss(0)
    rn, pn = U.normalise_pair(r, p, FINE, pin, m)
    lo, go = U.loss_and_grad(w0, rn, pn, FINE, pin, m, rounding=True)
    assert abs(loss - lo) < 2e-3 * lo
    gp, l2 = g.debug_learned_grad(0)
    assert abs(l2 - lo) < 2e-3 * lo
    # the BF16 network's layer gradients move by a few percent with the summation order alone
    # (FP32 against FP64 sums in the oracle: up to 1.3% for this pair; 4.5% seen on GB300)
    o = 0
    for i, (lev, cin, cout, *_r) in enumerate(U.LAYERS):
        n = 27 * cin * cout
        assert rel(gp[o:o + n], go[o:o + n]) < 6e-2, "layer %d" % i
        o += n
    assert abs(gp[-1] - go[-1]) < 1e-2 * abs(go[-1])     # omega
    lr = 1e-4
    losses = g.learned_train_step([0], lr)
    assert abs(losses[0] - lo) < 2e-3 * lo
    w1 = g.learned_get_weights().astype(np.float64)
    g.close()
    # first Adam step: w1 - w0 = -lr g / (|g| + eps), i.e. -lr sign(g) of the GPU's own gradient
    big = np.abs(gp) > 1e-2 * np.abs(gp).max()
    step = (w1 - w0)[big]
    assert np.all(np.sign(step) == -np.sign(gp[big]))
    assert np.allclose(np.abs(step), lr, rtol=0.02, atol=0)


def random_velocity(n, seed):
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(n + 1) * n * n); v = rng.normal(size=n * (n + 1) * n); w = rng.normal(size=n * n * (n + 1))
    # closed walls
    u.reshape(n + 1, n, n)[[0, n]] = 0.0
    v.reshape(n, n + 1, n)[:, [0, n]] = 0.0
    w.reshape(n, n, n + 1)[:, :, [0, n]] = 0.0
    return u, v, w


def divergence(u, v, w, n):
    U3 = u.reshape(n + 1, n, n); V3 = v.reshape(n, n + 1, n); W3 = w.reshape(n, n, n + 1)
    return (U3[1:] - U3[:-1]) + (V3[:, 1:] - V3[:, :-1]) + (W3[:, :, 1:] - W3[:, :, :-1])


@pytest.mark.parametrize("fallback", [400, 3])
def test_fcg_learned_projection(fallback):
    n = 32
    g = fia.Grid3D(n, n, n, 1.0 / n, precision=fia.FIA_FP32C)
    g.learned_init(3)
    # output layer zeroed: z = omega D^-1 r, so flexible CG must converge like Jacobi-PCG
    wts = g.learned_get_weights()
    o = sum(27 * l[1] * l[2] for l in U.LAYERS[:-1])
    wts[o:o + 27 * 16] = 0.0
    g.learned_set_weights(wts)
    u, v, w = random_velocity(n, 9)
    d0 = np.linalg.norm(divergence(u, v, w, n))
    for name, a in (("u", u), ("v", v), ("w", w)):
        g.set(name, a)
    sp = fia.solver_params(tol=1e-6, max_iter=5000, method=fia.FIA_SOLVER_FCG_LEARNED, fallback_iter=fallback)
    rep = g.calc_pressure_gradient_term_3D(sp)
    u2, v2, w2 = g.get("u"), g.get("v"), g.get("w")
    g.close()
    assert rep.rel_residual <= 1e-6
    if fallback == 3:
        # the first solve stops after 3 iterations; the FP64 residual refinement that follows
        # solves its corrections the same way
        assert rep.status & fia.FIA_STATUS_SOLVER_FALLBACK and rep.fcg_iterations >= 3
    else:
        # Jacobi inside FCG(4): it may stall and hand over to Jacobi-PCG, but must converge
        assert rep.fcg_iterations >= 100
    div = divergence(u2, v2, w2, n).ravel()
    div[-1] = 0.0      # the pinned cell's equation is dropped
    assert np.linalg.norm(div) < 1e-5 * d0


WEIGHTS = os.path.join(ROOT, "flux-interpolated-advection_gb300", "weights", "unet_precond.f32")


def multiscale_rhs(n, seed):
    """pressure of white noise filtered at 1.5, 6 and 24 cells; its right-hand side"""
    ndimage = pytest.importorskip("scipy.ndimage")
    rng = np.random.default_rng(seed)
    p = sum(ndimage.gaussian_filter(rng.normal(size=(n, n, n)), s) * s ** 1.5 for s in (1.5, 6.0, 24.0))
    p.reshape(-1)[-1] = 0.0
    return U.apply_B(p, (n, n, n), n ** 3 - 1), p


@pytest.mark.parametrize("n", [64, 128])
def test_trained_preconditioner_gain(n):
    """The committed network against the method without it (Jacobi-PCG) on the same
    problem: flexible CG must converge without the fallback in a small fraction of the
    iterations, and to the same solution."""
    g = fia.Grid3D(n, n, n, 1.0 / n, precision=fia.FIA_FP32C)
    g.learned_set_weights(np.fromfile(WEIGHTS, dtype="<f4"))
    r, p = multiscale_rhs(n, 21)
    xp, rp = g.debug_solve_rhs(r.ravel(), fia.solver_params(tol=1e-6, max_iter=20000))
    xl, rl = g.debug_solve_rhs(r.ravel(), fia.solver_params(tol=1e-6, max_iter=20000,
                                                             method=fia.FIA_SOLVER_FCG_LEARNED, fallback_iter=400))
    g.close()
    assert rp.rel_residual <= 1e-6 and rl.rel_residual <= 1e-6
    assert not rl.status & fia.FIA_STATUS_SOLVER_FALLBACK
    assert rl.fcg_iterations == rl.iterations
    assert rl.iterations * 8 <= rp.iterations, (rl.iterations, rp.iterations)
    # residual 1e-6 leaves an error of about kappa 1e-6 in the solution
    assert rel(xl, p) < 1e-2 and rel(xp, p) < 1e-2


def test_grid_transfers_match_oracle():
    g, m, pin, _ = solid_session()
    dims = U.level_dims(FINE)
    rng = np.random.default_rng(8)
    f = rng.normal(size=FINE).astype(np.float32)
    c = rng.normal(size=dims[0]).astype(np.float32)
    r0 = g.debug_grid_op(0, f)
    p1 = g.debug_grid_op(1, c)
    a2 = g.debug_grid_op(2, f)
    g.close()
    ex = U.excluded_mask(FINE, pin, m)
    pref = U.prolong(c, FINE)
    pref[ex] = 0.0
    assert rel(r0, U.restrict(f, FINE, dims[0])) < 1e-6
    assert rel(p1, pref) < 1e-6
    assert rel(a2, U.prolong_adjoint(f, dims[0])) < 1e-6
