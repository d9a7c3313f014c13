"""CPU checks of the learned-preconditioner oracle: its adjoints and gradients against
finite differences (rounding off), on grids small enough to run in seconds."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import unet_oracle as U  # noqa: E402


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, 3.0e-8, -2.5], dtype=np.float32)
    r = U.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: round to even (1.0); 1.005859375 rounds up
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.0078125) and r[4] == -2.5


@pytest.mark.parametrize("fine,coarse", [((8, 6, 7), (4, 3, 4)), ((5, 4, 3), (3, 2, 2))])
def test_adjoints(fine, coarse):
    rng = np.random.default_rng(0)
    x = rng.normal(size=fine + (3,)); g = rng.normal(size=coarse + (3,))
    assert np.isclose((U.pool(x, coarse) * g).sum(), (x * U.pool_adjoint(g, fine)).sum())
    xc = rng.normal(size=coarse + (3,)); gf = rng.normal(size=fine + (3,))
    assert np.isclose((U.up(xc, fine) * gf).sum(), (xc * U.up_adjoint(gf, coarse)).sum())
    y = rng.normal(size=coarse); gz = rng.normal(size=fine)
    assert np.isclose((U.prolong(y, fine) * gz).sum(), (y * U.prolong_adjoint(gz, coarse)).sum())
    # prolongation reproduces constants
    assert np.allclose(U.prolong(np.ones(coarse), fine), 1.0)


def test_conv_backward_fd():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(4, 3, 5, 2)); W = rng.normal(size=(27, 2, 3)); g = rng.normal(size=(4, 3, 5, 3))
    dx, dW = U.conv_backward(x, W, g)
    vx = rng.normal(size=x.shape); vW = rng.normal(size=W.shape)
    e = 1e-6
    fx = ((U.conv(x + e * vx, W) - U.conv(x - e * vx, W)) * g).sum() / (2 * e)
    fW = ((U.conv(x, W + e * vW) - U.conv(x, W - e * vW)) * g).sum() / (2 * e)
    assert np.isclose(fx, (dx * vx).sum(), rtol=1e-6)
    assert np.isclose(fW, (dW * vW).sum(), rtol=1e-6)


def test_B_is_symmetric_positive_with_solids():
    fine = (5, 4, 6)
    n = int(np.prod(fine))
    solid = np.zeros(n, dtype=np.uint8); solid[[7, 8, 30]] = 1
    pin = n - 1
    M = np.stack([U.apply_B(np.eye(n)[i], fine, pin, solid).ravel() for i in range(n)], axis=1)
    assert np.allclose(M, M.T)
    free = ~U.excluded_mask(fine, pin, solid).ravel()
    ev = np.linalg.eigvalsh(M[np.ix_(free, free)])
    assert ev.min() > 1e-8


def test_network_gradient_fd():
    fine = (10, 8, 9)
    p = U.init_params(3).astype(np.float64)
    dims = U.level_dims(fine)
    rng = np.random.default_rng(2)
    x0 = rng.normal(size=dims[0]); gy = rng.normal(size=dims[0])
    net = U.UNet(p, fine, rounding=False)
    net.forward(x0)
    gp = net.backward(gy)
    v = rng.normal(size=p.size); v[-1] = 0.0
    e = 1e-6
    fp = (U.UNet(p + e * v, fine, False).forward(x0) * gy).sum()
    fm = (U.UNet(p - e * v, fine, False).forward(x0) * gy).sum()
    assert np.isclose((fp - fm) / (2 * e), (gp * v).sum(), rtol=1e-5)


def test_loss_gradient_fd():
    fine = (8, 8, 8)
    n = 512
    pin = n - 1
    solid = np.zeros(n, dtype=np.uint8); solid[[100, 101, 109]] = 1
    rng = np.random.default_rng(4)
    ptrue = rng.normal(size=fine)
    ptrue[U.excluded_mask(fine, pin, solid)] = 0.0
    r = U.apply_B(ptrue, fine, pin, solid)
    r, ptrue = U.normalise_pair(r, ptrue, fine, pin, solid)
    prm = U.init_params(5).astype(np.float64)
    loss, gp = U.loss_and_grad(prm, r, ptrue, fine, pin, solid, rounding=False)
    assert loss > 0
    v = rng.normal(size=prm.size)
    e = 1e-6
    lp, _ = U.loss_and_grad(prm + e * v, r, ptrue, fine, pin, solid, rounding=False)
    lm, _ = U.loss_and_grad(prm - e * v, r, ptrue, fine, pin, solid, rounding=False)
    assert np.isclose((lp - lm) / (2 * e), (gp * v).sum(), rtol=1e-5)
