#!/usr/bin/env python3
"""Precision and sensitivity of the plume: several runs ("arms") of the same scene in lockstep,
with relative L2 differences of density and velocity between every pair of arms after given
numbers of steps ("a|b": |a - b| / |b|), and each arm's mass drift.

    python precision_report.py [--grid 64] [--steps 25,50,100] [--cfl 2]
                               [--arm NAME:PRECISION:TOL[:SOLVER[:DRHO[:DU[:DV]]]]] ...

PRECISION is fp64 (plain form) or fp32c (chosen form); TOL the pressure tolerance (FP64
residual in both forms); SOLVER pcg (Jacobi-PCG) or learned (flexible CG with the committed
preconditioner, fp32c only); DRHO a relative perturbation of the initial density: the
source sphere holds 1 + DRHO * xi with xi seeded uniform in [0, 1) per cell (the source
re-injects max(density, 1), so the perturbation is kept); DU a relative jitter of the velocity
after every step: each face velocity times 1 + DU * xi, xi seeded uniform in [-1, 1) (DU of
about 6e-8 is the size of FP32 rounding, so an FP64 arm with it measures how far the scheme
carries FP32-sized perturbations made at every step); DV (fp64 only) moves every backtraced
vertex by up to DV cells per axis, independently per vertex, axis and pass (the rounding of
FP32 vertex positions is about 1e-7 cells).  Without --arm the chosen form (fp32c,
Jacobi-PCG) is compared with the plain form at --tol.

Every arm starts from the plume density (sphere r = 0.1 at (0.5, 0.15, 0.5)) at rest, with
the source re-injected every step, buoyancy 1 and CFL --cfl.  Prints one JSON line.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import fia  # noqa: E402
import scenes  # noqa: E402


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def parse_arm(spec, default_tol):
    f = spec.split(":")
    if len(f) < 2 or f[1] not in ("fp64", "fp32c"):
        raise SystemExit("bad --arm %r (NAME:PRECISION:TOL[:SOLVER[:DRHO[:DU[:DV]]]])" % spec)
    arm = {"name": f[0], "precision": f[1], "tol": float(f[2]) if len(f) > 2 and f[2] else default_tol,
           "solver": f[3] if len(f) > 3 and f[3] else "pcg", "drho": float(f[4]) if len(f) > 4 and f[4] else 0.0,
           "du": float(f[5]) if len(f) > 5 and f[5] else 0.0, "dv": float(f[6]) if len(f) > 6 and f[6] else 0.0}
    if arm["solver"] not in ("pcg", "learned") or (arm["solver"] == "learned" and arm["precision"] != "fp32c"):
        raise SystemExit("bad solver in --arm %r" % spec)
    if arm["dv"] and arm["precision"] != "fp64":
        raise SystemExit("vertex jitter is an fp64 arm option: %r" % spec)
    return arm


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=64)
    ap.add_argument("--steps", default="25,50,100")
    ap.add_argument("--cfl", type=float, default=2.0)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--arm", action="append", default=[])
    ap.add_argument("--weights", default=os.path.join(HERE, "weights", "unet_precond.f32"))
    ap.add_argument("--seed", type=int, default=7, help="seed of the density perturbation")
    args = ap.parse_args()
    n = args.grid
    checkpoints = sorted(int(x) for x in args.steps.split(","))
    specs = args.arm or ["fp64:fp64:%g" % args.tol, "fp32c:fp32c:%g" % args.tol]
    arms = [parse_arm(s, args.tol) for s in specs]
    rho0 = scenes.plume_density(n)
    for arm in arms:
        prec = fia.FIA_FP64 if arm["precision"] == "fp64" else fia.FIA_FP32C
        g = fia.Grid3D(n, n, n, 1.0 / n, precision=prec)
        rho = rho0.copy()
        if arm["drho"]:
            xi = np.random.Generator(np.random.PCG64(args.seed)).uniform(0.0, 1.0, size=rho.size)
            rho = rho * (1.0 + arm["drho"] * xi)
        g.set("density", rho)
        if arm["dv"]:
            g.debug_vertex_jitter(arm["dv"])
        for c, m in (("u", (n + 1) * n * n), ("v", n * (n + 1) * n), ("w", n * n * (n + 1))):
            g.set(c, np.zeros(m))
        solver = {"tol": arm["tol"], "max_iter": 50000}
        if arm["solver"] == "learned":
            g.learned_set_weights(np.fromfile(args.weights, dtype="<f4"))
            solver.update(method=fia.FIA_SOLVER_FCG_LEARNED, fallback_iter=200)
        arm.update(grid=g, params=fia.step_params(cfl=args.cfl, solver=solver), masses=[], seconds=0.0,
                   status=0, rng=np.random.Generator(np.random.PCG64(args.seed + 1)))
    out = {"grid": n, "cfl": args.cfl,
           "arms": [{k: a[k] for k in ("name", "precision", "tol", "solver", "drho", "du", "dv")} for a in arms],
           "checkpoints": []}
    step = 0
    for cp in checkpoints:
        while step < cp:
            for arm in arms:
                t0 = time.time()
                arm["params"].frame = step
                rep = arm["grid"].step(arm["params"])
                arm["seconds"] += time.time() - t0
                arm["status"] |= rep.status
                arm["masses"].append((rep.mass_before_advection, rep.mass_after_advection, rep.mass_after))
                if arm["du"]:
                    for c in "uvw":
                        a = arm["grid"].get(c)
                        arm["grid"].set(c, a * (1.0 + arm["du"] * arm["rng"].uniform(-1.0, 1.0, size=a.size)))
            step += 1
        fields = [{c: arm["grid"].get(c) for c in ("density", "u", "v", "w")} for arm in arms]
        row = {"step": step, "density": {}, "velocity": {}}
        for i, a in enumerate(arms):
            for j, b in enumerate(arms):
                if j >= i:
                    continue
                key = "%s|%s" % (a["name"], b["name"])
                row["density"][key] = rel(fields[i]["density"], fields[j]["density"])
                va = np.concatenate([fields[i][c] for c in "uvw"])
                vb = np.concatenate([fields[j][c] for c in "uvw"])
                row["velocity"][key] = rel(va, vb)
        out["checkpoints"].append(row)
        print(json.dumps(row), file=sys.stderr, flush=True)
    out["per_arm"] = {}
    for arm in arms:
        m = np.array(arm["masses"])
        out["per_arm"][arm["name"]] = {
            "mass_max_rel_change_by_advection": float(np.max(np.abs(m[:, 1] - m[:, 0]) / m[:, 0])),
            "mass_max_rel_change_after_correction": float(np.max(np.abs(m[:, 2] - m[:, 0]) / m[:, 0])),
            "seconds": arm["seconds"], "status_bits": arm["status"]}
        arm["grid"].close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
