"""GPU tests of the frame output of the reference's main loop (main.cpp:515-654): the dense
density frame that stands in for its OpenVDB export, and the per-frame mass / momentum logs."""
import os

import numpy as np
import pytest

import fia

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [fia.FIA_FP64, fia.FIA_FP32C])
def test_density_frame_and_totals(tmp_path, precision):
    N = (12, 10, 8)
    h = 1.0 / 12
    rng = np.random.default_rng(4)
    rho = rng.uniform(0.0, 1.0, size=N)
    u = rng.normal(size=(N[0] + 1) * N[1] * N[2])
    v = rng.normal(size=N[0] * (N[1] + 1) * N[2])
    w = rng.normal(size=N[0] * N[1] * (N[2] + 1))
    g = fia.Grid3D(*N, h, precision=precision)
    g.set("density", rho)
    for c, a in zip("uvw", (u, v, w)):
        g.set(c, a)
    path = str(tmp_path / "substance_density_0003.fia")
    g.write_density_frame(path, 3)
    data, hd = fia.read_density_frame(path)
    assert data.shape == N and data.dtype == np.float32
    assert np.array_equal(data, g.get("density").reshape(N).astype(np.float32))
    assert hd["frame"] == 3
    assert hd["origin"] == pytest.approx(tuple(-0.5 * h * n for n in N), abs=0)
    assert hd["voxel_size"] == h
    assert os.path.getsize(path) == 64 + 4 * N[0] * N[1] * N[2]
    # totals: mass and momenta (sum * cell volume), the wall losses of the projections
    V = h ** 3
    tol = 1e-13 if precision == fia.FIA_FP64 else 1e-6
    mom = g.total_momentum()
    for got, a in zip(mom, (g.get("u"), g.get("v"), g.get("w"))):
        assert got == pytest.approx(a.sum() * V, rel=tol, abs=tol * np.abs(a).sum() * V)
    g.calc_pressure_gradient_term_3D(fia.solver_params(tol=1e-8))
    prefix = str(tmp_path / "run_")
    g.append_totals(prefix, 0.0)
    g.append_totals(prefix, 0.25)
    mass = g.total_mass()
    mom = g.total_momentum()
    loss = g.wall_momentum_loss()
    g.close()
    lines = open(prefix + "total_mass.dat").read().splitlines()
    assert len(lines) == 2
    t, m = (float(x) for x in lines[1].split())
    assert t == 0.25 and m == pytest.approx(mass, rel=1e-15)
    for c, ax in enumerate("xyz"):
        vals = {}
        for name in ("total_momentum_%s.dat", "total_loss_of_momentum_%s.dat",
                     "momentum_%s_plus_total_loss_of_momentum_%s.dat"):
            fn = prefix + (name % ((ax,) * name.count("%s")))
            row = open(fn).read().splitlines()[-1].split()
            vals[name] = float(row[1])
        assert vals["total_momentum_%s.dat"] == pytest.approx(mom[c], rel=1e-15)
        assert vals["total_loss_of_momentum_%s.dat"] == pytest.approx(loss[c], rel=1e-15)
        assert vals["momentum_%s_plus_total_loss_of_momentum_%s.dat"] == pytest.approx(mom[c] + loss[c], rel=1e-15)


def test_bad_frame_path_fails_loudly(tmp_path):
    g = fia.Grid3D(8, 8, 8, 1.0 / 8)
    with pytest.raises(fia.FiaError):
        g.write_density_frame(str(tmp_path / "no_such_dir" / "f.fia"), 0)
    g.close()
