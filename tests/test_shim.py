"""The reference-signature shim (flux-interpolated-advection_gb300/shim/): the reference's 3D
entry points (move_substances_3D, advect_velocity_xyz_flux_advection_3D_std_thread,
update_fluid_velocity_3D, calc_pressure_3D, calc_pressure_gradient_term_3D) and the CFL step,
called on a grid the way the reference's main loop calls them (tests/shim_driver.cpp).

* Where the reference checkout exists (no GPU needed): fia_shim_reference.cpp compiles against
  the reference's own headers, with MY_FLOAT_TYPE float (as shipped) and double, defines the
  reference's symbols, and links with the reference's own translation units (Grid_3D and the
  rest, oracle/_ref) and libfia into the reference-grid driver.  Without a GPU that driver must
  stop with the library's error (the shim's error convention); with one it runs.
* On the GPU: the driver over a stand-in grid (float and double), plain and chosen forms,
  checked call by call against the oracle (advection) and against the library's session API
  (projection, wall totals, the CFL reduction).
"""
import glob
import os
import shutil
import subprocess

import numpy as np
import pytest

import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "flux-interpolated-advection_gb300", "shim")
DRIVER = os.path.join(ROOT, "tests", "shim_driver.cpp")
REF_OBJ = os.path.join(ROOT, "oracle", "_ref")


def reference_dir():
    return os.environ.get("FIA_REFERENCE_DIR", os.path.join(os.path.dirname(ROOT), "reference"))


def have_nvcc():
    return shutil.which("nvcc") is not None or os.path.exists("/usr/local/cuda/bin/nvcc")


def write_input(path, n, h, dt, rho, u, v, w):
    with open(path, "wb") as f:
        np.array([n], dtype="<i4").tofile(f)
        np.array([h, dt], dtype="<f8").tofile(f)
        for a in (rho, u, v, w):
            np.asarray(a, dtype="<f8").tofile(f)


def read_output(path, n):
    raw = np.fromfile(path, dtype="<f8")
    sizes = {"c": n ** 3, "u": (n + 1) * n * n, "v": n * (n + 1) * n, "w": n * n * (n + 1)}
    out, pos = {}, 0

    def take(key, m):
        nonlocal pos
        out[key] = raw[pos:pos + m]
        pos += m
    take("density", sizes["c"])
    for c in "uvw":
        take("adv_" + c, sizes[c])
    for c in "uvw":
        take("proj_" + c, sizes[c])
    take("proj_p", sizes["c"])
    take("loss", 3)
    take("p_only", sizes["c"])
    for c in "uvw":
        take("upd_" + c, sizes[c])
    take("cfl", 2)
    assert pos == raw.size, (pos, raw.size)
    return out


# ----------------------------------------------------------------------------------------
# the maintainer's build: reference headers, reference translation units, libfia
# ----------------------------------------------------------------------------------------
@pytest.mark.skipif(not have_nvcc(), reason="nvcc not available")
@pytest.mark.parametrize("precision", ["float", "double"])
def test_shim_builds_into_the_reference_program(precision, tmp_path):
    ref = reference_dir()
    objs = sorted(glob.glob(os.path.join(REF_OBJ, "obj_%s" % precision, "*.o")))
    if not os.path.isdir(os.path.join(ref, "include")) or not objs:
        pytest.skip("no reference checkout (or oracle/_ref not built): the maintainer's build is checked where "
                    "the reference is")
    import fia
    lib = fia.build()
    if precision == "float":
        inc = ["-I" + os.path.join(ROOT, "oracle", "ref_shim"), "-I" + os.path.join(ref, "include")]
    else:
        inc = ["-I" + os.path.join(ROOT, "oracle", "ref_shim"), "-I" + os.path.join(REF_OBJ, "include_double")]
    inc += ["-I" + os.path.join(ref, "src"), "-I" + os.path.join(ROOT, "include"), "-I" + SHIM]
    flags = ["-std=c++17", "-O1", "-w"]
    shim_o = str(tmp_path / "fia_shim_reference.o")
    drv_o = str(tmp_path / "shim_driver.o")
    subprocess.check_call(["g++"] + flags + inc + ["-c", os.path.join(SHIM, "fia_shim_reference.cpp"), "-o", shim_o])
    subprocess.check_call(["g++"] + flags + inc + ["-DFIA_REFERENCE_GRID", "-c", DRIVER, "-o", drv_o])
    # the shim defines the reference's entry points with the reference's own signatures
    syms = subprocess.run(["nm", "-C", shim_o], capture_output=True, text=True, check=True).stdout
    real = "double" if precision == "double" else "float"
    for sig in ("smoke_simulation::move_substances_3D(smoke_simulation::Grid_3D&, int, %s," % real,
                "smoke_simulation::advect_velocity_xyz_flux_advection_3D_std_thread(smoke_simulation::Grid_3D&, %s,"
                % real,
                "smoke_simulation::update_fluid_velocity_3D(smoke_simulation::Grid_3D&, int, %s," % real,
                "smoke_simulation::calc_pressure_3D(smoke_simulation::Grid_3D&)",
                "smoke_simulation::calc_pressure_gradient_term_3D(smoke_simulation::Grid_3D&)"):
        assert (" T " + sig) in syms, sig
    # linked with the reference's translation units (not its harness) and libfia
    objs = [o for o in objs if not o.endswith("ref_harness.o")]
    exe = str(tmp_path / "shim_driver_ref")
    subprocess.check_call(["g++", "-o", exe, drv_o, shim_o] + objs +
                          [lib, "-Wl,-rpath," + os.path.dirname(lib), "-lpthread"])
    n = 8
    h = 1.0 / n
    u, v, w = scenes.fourier_velocity(n, seed=3)
    write_input(str(tmp_path / "in.bin"), n, h, h, scenes.gaussian_blobs(n, seed=4), u, v, w)
    r = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True,
                       timeout=600)
    # no GPU: the first call stops with the library's message (the reference's void signature
    # cannot return it); with a GPU the driver runs through
    assert r.returncode == 0 or (r.returncode == 1 and "fia_create" in r.stderr), (r.returncode, r.stderr)


# ----------------------------------------------------------------------------------------
# on the GPU: the stand-in grid
# ----------------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def drivers(tmp_path_factory):
    import fia
    lib = fia.build()
    d = tmp_path_factory.mktemp("shim")
    out = {}
    for real in ("double", "float"):
        exe = str(d / ("shim_driver_" + real))
        subprocess.check_call(["g++", "-std=c++17", "-O1", "-DFIA_GRID_REAL=" + real, "-I" + os.path.join(ROOT, "include"),
                               "-I" + SHIM, DRIVER, "-o", exe, lib, "-Wl,-rpath," + os.path.dirname(lib)])
        out[real] = exe
    return out


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.gpu
@pytest.mark.parametrize("real,precision", [("double", "fp64"), ("float", "fp64"), ("double", "fp32c")])
def test_shim_calls_match_the_oracle_and_the_session_api(drivers, real, precision, tmp_path):
    import fia
    from oracle import Oracle
    n = 16
    h = 1.0 / n
    u, v, w = scenes.fourier_velocity(n, seed=5)
    rho = scenes.gaussian_blobs(n, seed=6)
    dt = 2.0 * h
    if real == "float":     # the grid holds floats: compare with the same rounded inputs
        u, v, w, rho = (a.astype(np.float32).astype(np.float64) for a in (u, v, w, rho))
    write_input(str(tmp_path / "in.bin"), n, h, dt, rho, u, v, w)
    env = dict(os.environ, FIA_SHIM_PRECISION=precision, FIA_SHIM_SOLVER="pcg", FIA_SHIM_TOL="1e-8")
    r = subprocess.run([drivers[real], str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True,
                       text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr
    got = read_output(str(tmp_path / "out.bin"), n)
    # tolerance: FP64 form on double grids at the parity bound; float grids add the rounding
    # of the copies to and from float; the chosen form at its per-step bound
    tol = {("double", "fp64"): 1e-10, ("float", "fp64"): 2e-7, ("double", "fp32c"): 2e-5}[(real, precision)]
    O = Oracle()
    N = (n, n, n)
    ref_rho, _ = O.move_substances_3D(N, h, u, v, w, rho, dt)
    assert rel(got["density"], ref_rho) < tol
    ou, ov, ow, _ = O.advect_velocity_3D(N, h, u, v, w, dt)
    for c, ref in zip("uvw", (ou, ov, ow)):
        assert rel(got["adv_" + c], ref) < tol, c

    # projection, pressure, wall totals and the frame-1 velocity update against the session API
    # of the same library on the shim's own inputs
    prec = fia.FIA_FP64 if precision == "fp64" else fia.FIA_FP32C
    g = fia.Grid3D(n, n, n, h, precision=prec)
    for c in "uvw":
        g.set(c, got["adv_" + c])
    sp = fia.solver_params(tol=1e-8, max_iter=100000)
    g.calc_pressure_gradient_term_3D(sp)
    ptol = 1e-12 if (real, precision) == ("double", "fp64") else tol
    for c in "uvw":
        assert rel(got["proj_" + c], g.get(c)) < ptol, c
    assert rel(got["proj_p"], g.get("pressure")) < ptol
    np.testing.assert_allclose(got["loss"], g.wall_momentum_loss(), rtol=max(ptol, 1e-12), atol=1e-14)
    div = scenes.divergence(n, got["proj_u"], got["proj_v"], got["proj_w"])
    assert np.abs(np.delete(div, n ** 3 - 1)).max() < (1e-6 if real == "double" else 1e-4)
    # calc_pressure_3D of the projected velocity leaves the velocity alone; its pressure is the
    # pressure of a (nearly) divergence-free field
    assert np.abs(got["p_only"]).max() < 1e-3 * max(np.abs(got["proj_p"]).max(), 1e-30)
    # update_fluid_velocity_3D at frame 1: advect, then project
    g.advect_velocity_xyz_flux_advection_3D(dt)
    g.calc_pressure_gradient_term_3D(sp)
    for c in "uvw":
        assert rel(got["upd_" + c], g.get(c)) < ptol, c
    # the CFL step: 2 h / max|u| (or the time to the next movie frame at 60 fps)
    umax = max(np.abs(got["upd_" + c]).max() for c in "uvw")
    expect = min(2.0 * h / umax, 1.0 / 60.0)
    assert abs(got["cfl"][0] - expect) <= 1e-6 * expect
    assert got["cfl"][1] == (1.0 if 2.0 * h / umax > 1.0 / 60.0 else 0.0)
    g.close()
