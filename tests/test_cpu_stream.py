"""The streaming-tile CPU baseline (oracle/cpu_stream.inl: the presort-and-stream design of the
reference's sginterp3::interpolate, sginterp3.cpp:204-385, in plain C++ threads around a density
step with unique vertices and faces) against the oracle's move_substances_3D.  No GPU.

Bar: 1e-12 relative L2 (both FP64; the baseline evaluates WENO6 in the difference form and
collapsed on node planes, and sums each face's pieces on its own, all equal in exact
arithmetic), and slab-by-slab evaluation equal to the whole step bit for bit."""
import numpy as np
import pytest

import scenes
from oracle import Oracle

O = Oracle()


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("kw", [dict(), dict(interp=1), dict(use_integral=0), dict(correction=0), dict(k=1),
                                dict(k=5), dict(split_off=(0.0, 0.5)), dict(split_off=(0.0, 0.0))],
                         ids=["default", "linear", "no_integral", "no_correction", "k1", "k5", "x_axis_split",
                              "axis_split"])
def test_streaming_baseline_matches_oracle(kw):
    n = 20
    h = 1.0 / n
    u, v, w = scenes.fourier_velocity(n, seed=5)
    rho = scenes.gaussian_blobs(n, seed=6)
    dt = 2.0 * h
    ref, st = O.move_substances_3D((n, n, n), h, u, v, w, rho, dt, nthreads=4, **kw)
    got, st2, faces = O.stream_move_substances_slab((n, n, n), h, u, v, w, rho, dt, 0, n, 3, nthreads=4, **kw)
    assert st == st2 == 0
    assert faces == 3 * n * n * (n + 1)
    assert rel(got, ref) < 1e-12


def test_streaming_baseline_slabs_equal_the_whole_step_and_the_oracle_slabs():
    n = 24
    h = 1.0 / n
    u, v, w = scenes.fourier_velocity(n, seed=7)
    rho = scenes.gaussian_blobs(n, seed=8)
    dt = 2.5 * h
    margin = int(np.ceil(dt * max(np.abs(u).max(), np.abs(v).max(), np.abs(w).max()) / h)) + 1
    whole, _, _ = O.stream_move_substances_slab((n, n, n), h, u, v, w, rho, dt, 0, n, margin, nthreads=3)
    by_slab, by_oracle_slab = np.zeros(n ** 3), np.zeros(n ** 3)
    for x0 in range(0, n, 5):
        x1 = min(n, x0 + 5)
        O.stream_move_substances_slab((n, n, n), h, u, v, w, rho, dt, x0, x1, margin, nthreads=2, out=by_slab)
        O.move_substances_slab((n, n, n), h, u, v, w, rho, dt, x0, x1, margin, nthreads=2, out=by_oracle_slab)
    assert np.array_equal(by_slab, whole)
    ref, _ = O.move_substances_3D((n, n, n), h, u, v, w, rho, dt, nthreads=4)
    assert np.array_equal(by_oracle_slab, ref)
    assert rel(whole, ref) < 1e-12
