"""Seeded synthetic scenes for the flux-advection step (host-side input generation).

No public dataset is involved: every scene is produced by one
numpy.random.Generator(PCG64(seed)), and the seed is part of the returned record.

  * fourier_velocity  -- divergence-free MAC velocity, u = curl A, with A a sum of
                         seeded Fourier modes (integer wavenumbers |n| in [1, 8], Gaussian
                         amplitudes) times a window that vanishes on the walls, taken as a
                         discrete curl on cell edges so that the discrete divergence is zero
                         up to round-off and the normal velocity on every wall is zero;
  * gaussian_blobs    -- density as a sum of isotropic Gaussian blobs;
  * plume_density     -- density 1 inside a sphere (the plume source), 0 elsewhere.

Array layout is the reference's Grid_3D layout (grid_3d.h:35-54): z fastest, x slowest;
u is (N+1)xNxN, v is Nx(N+1)xN, w is NxNx(N+1), density is NxNxN.
"""
import numpy as np


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def fourier_velocity(n, seed=1, n_modes=16, kmin=1, kmax=8, target_max=1.0):
    """Return (u, v, w) flattened float64 arrays with max |face velocity| = target_max."""
    rng = _rng(seed)
    h = 1.0 / n
    modes = []
    while len(modes) < n_modes:
        k = rng.integers(-kmax, kmax + 1, size=3)
        kn = float(np.sqrt((k * k).sum()))
        if kn < kmin or kn > kmax:
            continue
        amp = rng.normal(0.0, 1.0, size=3) / kn
        phase = rng.uniform(0.0, 2.0 * np.pi, size=3)
        modes.append((k.astype(np.float64), amp, phase))

    def potential(comp, x, y, z):
        a = np.zeros(np.broadcast(x, y, z).shape)
        for k, amp, phase in modes:
            a += amp[comp] * np.sin(2.0 * np.pi * (k[0] * x + k[1] * y + k[2] * z) + phase[comp])
        return a * np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z)

    i = np.arange(n + 1) * h
    c = (np.arange(n) + 0.5) * h
    # edge-centred potentials: A_x on x-edges (c, i, i), A_y on (i, c, i), A_z on (i, i, c)
    Ax = potential(0, c[:, None, None], i[None, :, None], i[None, None, :])
    Ay = potential(1, i[:, None, None], c[None, :, None], i[None, None, :])
    Az = potential(2, i[:, None, None], i[None, :, None], c[None, None, :])
    u = (Az[:, 1:, :] - Az[:, :-1, :]) / h - (Ay[:, :, 1:] - Ay[:, :, :-1]) / h      # (n+1, n, n)
    v = (Ax[:, :, 1:] - Ax[:, :, :-1]) / h - (Az[1:, :, :] - Az[:-1, :, :]) / h      # (n, n+1, n)
    w = (Ay[1:, :, :] - Ay[:-1, :, :]) / h - (Ax[:, 1:, :] - Ax[:, :-1, :]) / h      # (n, n, n+1)
    m = max(np.abs(u).max(), np.abs(v).max(), np.abs(w).max())
    s = target_max / m
    return (np.ascontiguousarray(u * s).ravel(), np.ascontiguousarray(v * s).ravel(),
            np.ascontiguousarray(w * s).ravel())


def gaussian_blobs(n, seed=2, n_blobs=32, sigma=(0.02, 0.08), amp=(0.5, 1.0)):
    rng = _rng(seed)
    h = 1.0 / n
    c = (np.arange(n) + 0.5) * h
    rho = np.zeros((n, n, n))
    for _ in range(n_blobs):
        ctr = rng.uniform(0.15, 0.85, size=3)
        s = rng.uniform(*sigma)
        a = rng.uniform(*amp)
        gx = np.exp(-0.5 * ((c - ctr[0]) / s) ** 2)
        gy = np.exp(-0.5 * ((c - ctr[1]) / s) ** 2)
        gz = np.exp(-0.5 * ((c - ctr[2]) / s) ** 2)
        rho += a * gx[:, None, None] * gy[None, :, None] * gz[None, None, :]
    return rho.ravel()


def plume_density(n, center=(0.5, 0.15, 0.5), radius=0.1):
    h = 1.0 / n
    c = (np.arange(n) + 0.5) * h
    d2 = ((c[:, None, None] - center[0]) ** 2 + (c[None, :, None] - center[1]) ** 2
          + (c[None, None, :] - center[2]) ** 2)
    return (d2 <= radius * radius).astype(np.float64).ravel()


def divergence(n, u, v, w):
    """Cell divergence times h (the pressure right-hand side of calc_pressure_3d.cpp:111-131)."""
    u = u.reshape(n + 1, n, n); v = v.reshape(n, n + 1, n); w = w.reshape(n, n, n + 1)
    return ((u[1:] - u[:-1]) + (v[:, 1:] - v[:, :-1]) + (w[:, :, 1:] - w[:, :, :-1])).ravel()
