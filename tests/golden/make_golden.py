"""Writes the golden fixtures of tests/golden/ from the reference's own code.

Runs the reference translation units, built from the reference checkout by
oracle/build_ref.sh into oracle/_ref/ (float as shipped and the double variant), on
small seeded inputs and stores inputs and outputs.  The oracle is pinned against these
files by tests/test_oracle_golden.py; the GPU library is then checked against the oracle.

    python tests/golden/make_golden.py          (needs the reference checkout)
    python tests/golden/make_golden.py maccormack   (the MacCormack fixtures only)
    python tests/golden/make_golden.py volumes      (the cell-volume fixtures only)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "flux-interpolated-advection_gb300"))

import oracle as orc  # noqa: E402
import scenes  # noqa: E402


def main():
    if not os.path.exists(os.path.join(orc.REF_DIR, "libfia_ref_double.so")):
        orc.build_reference()
    refs = {p: orc.Reference(p) for p in ("double", "float")}
    rng = np.random.Generator(np.random.PCG64(20240601))

    # --- point interpolation (WENO6 / linear / 1Dy variants) on a 10x9x8 grid ---
    N = (10, 9, 8); h = 1.0 / 10
    sizes = {"c": N[0] * N[1] * N[2], "x": (N[0] + 1) * N[1] * N[2], "y": N[0] * (N[1] + 1) * N[2],
             "z": N[0] * N[1] * (N[2] + 1)}
    arrays = {k: rng.normal(size=n) for k, n in sizes.items()}
    pts = rng.uniform(-0.15, 1.15, size=(300, 3)) * np.array(N) * h
    out = {"N": np.array(N), "h": h, "pts": pts}
    for k, v in arrays.items():
        out["a_" + k] = v
    kinds = {0: "c", 1: "x", 2: "y", 3: "z", 4: "c", 5: "x", 6: "y", 7: "z", 8: "c", 9: "x", 10: "y", 11: "z"}
    for kind, arr in kinds.items():
        for p, R in refs.items():
            out["interp_%d_%s" % (kind, p)] = R.interp(kind, arrays[arr], N, h, pts)
    np.savez_compressed(os.path.join(HERE, "interp.npz"), **out)

    # --- psi_y of a density field ---
    N = (8, 12, 6); h = 1.0 / 8
    rho = rng.uniform(0.0, 1.0, size=N[0] * N[1] * N[2])
    out = {"N": np.array(N), "h": h, "rho": rho}
    for interp, k, integ in ((0, 3, 1), (0, 1, 1), (1, 1, 1), (3, 1, 0)):
        for p, R in refs.items():
            out["psi_%d_%d_%d_%s" % (interp, k, integ, p)] = R.psi_density(rho, N, h, interp, k, integ)
    np.savez_compressed(os.path.join(HERE, "psi.npz"), **out)

    # --- face clipping: 400 random backtraced faces x 4 split methods ---
    h = 1.0 / 16
    faces = []
    for t in range(400):
        base = np.array([[0, 0, 0], [0, 1, 0], [1, 1, 0], [1, 0, 0]], float) * h + 5 * h
        base = base[:, rng.permutation(3)]
        scale = [0.1, 0.5, 1.5][t % 3]
        faces.append(base + rng.normal(0, 1.0, base.shape) * h * scale)
    faces = np.array(faces)
    out = {"h": h, "faces": faces}
    for split in range(4):
        for p, R in refs.items():
            tot = []
            npieces = []
            for f in faces:
                pc = R.split_face(f, h, split)
                npieces.append(len(pc))
                tot.append(np.concatenate([pc[:, 3:].sum(0), (pc[:, :3] * pc[:, 4:5]).sum(0)]) if len(pc) else np.zeros(6))
            out["split_%d_%s_totals" % (split, p)] = np.array(tot)
            out["split_%d_%s_count" % (split, p)] = np.array(npieces)
    np.savez_compressed(os.path.join(HERE, "split.npz"), **out)

    # --- density passes and move_substances_3D on a 16^3 Fourier/blob scene (CFL 2) ---
    n = 16; N = (n, n, n); h = 1.0 / n
    u, v, w = scenes.fourier_velocity(n, seed=1)
    rho = scenes.gaussian_blobs(n, seed=2)
    dt = 2.0 * h
    out = {"N": np.array(N), "h": h, "u": u, "v": v, "w": w, "rho": rho, "dt": dt}
    passes = {  # name: (interp, psi, use_integral, zero_velocity, split)
        "weno6_integral": (0, 0, 1, 0, 0),
        "weno6_zero_velocity": (0, 0, 0, 1, 0),
        "error_1dy_linear": (2, 3, 0, 0, 1),
        "linear_integral": (1, 1, 1, 0, 0),
    }
    for name, (interp, psi, integ, zv, split) in passes.items():
        for p, R in refs.items():
            out["pass_%s_%s" % (name, p)] = R.density_pass(N, h, u, v, w, rho, dt, interp, psi, integ, zv, split, 3)
    for p, R in refs.items():
        out["move_substances_%s" % p] = R.move_substances_3D(N, h, u, v, w, rho, dt, interp=0, split=0, k=3,
                                                             correction=1, use_integral=1)
    np.savez_compressed(os.path.join(HERE, "density.npz"), **out)

    # --- velocity passes in the reference's defined (linear) form, 12^3 ---
    n = 12; N = (n, n, n); h = 1.0 / n
    u, v, w = scenes.fourier_velocity(n, seed=3)
    dt = 1.5 * h
    out = {"N": np.array(N), "h": h, "u": u, "v": v, "w": w, "dt": dt}
    for dim in range(3):
        for p, R in refs.items():
            out["vel_%d_%s" % (dim, p)] = R.velocity_pass_linear(N, h, u, v, w, dim, dt, 3)
    np.savez_compressed(os.path.join(HERE, "velocity.npz"), **out)
    maccormack(refs)
    volumes(refs)
    print("golden fixtures written to", HERE)


def volumes(refs):
    """advected cell volumes of the density main pass of the 16^3 scene (the volume points of the
    cell-volume correction), plain and with the flux MacCormack scheme"""
    n = 16; N = (n, n, n); h = 1.0 / n
    u, v, w = scenes.fourier_velocity(n, seed=1)
    dt = 2.0 * h
    out = {"N": np.array(N), "h": h, "u": u, "v": v, "w": w, "dt": dt}
    for mc in (0, 1):
        for p, R in refs.items():
            out["vol_mc%d_%s" % (mc, p)] = R.cell_volumes(N, h, u, v, w, dt, maccormack=mc)
    np.savez_compressed(os.path.join(HERE, "volumes.npz"), **out)


def maccormack(refs):
    """the flux MacCormack branch (backtrace_..._for_integrate_density.cpp:146-234): the density
    passes and move_substances_3D of the 16^3 scene with use_MacCormack_scheme on"""
    n = 16; N = (n, n, n); h = 1.0 / n
    u, v, w = scenes.fourier_velocity(n, seed=1)
    rho = scenes.gaussian_blobs(n, seed=2)
    dt = 2.0 * h
    out = {"N": np.array(N), "h": h, "u": u, "v": v, "w": w, "rho": rho, "dt": dt}
    passes = {  # name: (interp, psi, use_integral, zero_velocity, split)
        "weno6_integral": (0, 0, 1, 0, 0),
        "weno6_zero_velocity": (0, 0, 0, 1, 0),
        "error_1dy_linear": (2, 3, 0, 0, 1),
        "linear_integral": (1, 1, 1, 0, 0),
    }
    for name, (interp, psi, integ, zv, split) in passes.items():
        for p, R in refs.items():
            out["pass_%s_%s" % (name, p)] = R.density_pass(N, h, u, v, w, rho, dt, interp, psi, integ, zv, split, 3,
                                                           maccormack=1)
    for p, R in refs.items():
        out["move_substances_%s" % p] = R.move_substances_3D(N, h, u, v, w, rho, dt, interp=0, split=0, k=3,
                                                             correction=1, use_integral=1, maccormack=1)
    np.savez_compressed(os.path.join(HERE, "maccormack.npz"), **out)


if __name__ == "__main__":
    if sys.argv[1:] in (["maccormack"], ["volumes"]):
        if not os.path.exists(os.path.join(orc.REF_DIR, "libfia_ref_double.so")):
            orc.build_reference()
        {"maccormack": maccormack, "volumes": volumes}[sys.argv[1]]({p: orc.Reference(p) for p in ("double", "float")})
    else:
        main()
