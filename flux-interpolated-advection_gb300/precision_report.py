#!/usr/bin/env python3
"""Chosen form against the plain form on the plume: relative L2 differences of density and
velocity after given numbers of steps, and the mass drift of each form.

    python precision_report.py [--grid 64] [--steps 25,50,100] [--cfl 2] [--tol 1e-6] [--solver pcg|learned]

Both forms start from the plume density (sphere r = 0.1 at (0.5, 0.15, 0.5)) at rest, with the
source re-injected every step, buoyancy 1 and the pressure solved to --tol (FP64 residual in
both forms).  Prints one JSON line.
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=64)
    ap.add_argument("--steps", default="25,50,100")
    ap.add_argument("--cfl", type=float, default=2.0)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--solver", default="pcg", choices=["pcg", "learned"])
    ap.add_argument("--weights", default=os.path.join(HERE, "weights", "unet_precond.f32"))
    args = ap.parse_args()
    n = args.grid
    checkpoints = sorted(int(x) for x in args.steps.split(","))
    sessions = {}
    for name, prec in (("fp64", fia.FIA_FP64), ("fp32c", fia.FIA_FP32C)):
        g = fia.Grid3D(n, n, n, 1.0 / n, precision=prec)
        g.set("density", scenes.plume_density(n))
        for c, m in (("u", (n + 1) * n * n), ("v", n * (n + 1) * n), ("w", n * n * (n + 1))):
            g.set(c, np.zeros(m))
        solver = {"tol": args.tol, "max_iter": 50000}
        if name == "fp32c" and args.solver == "learned":
            g.learned_set_weights(np.fromfile(args.weights, dtype="<f4"))
            solver.update(method=fia.FIA_SOLVER_FCG_LEARNED, fallback_iter=200)
        sessions[name] = (g, fia.step_params(cfl=args.cfl, solver=solver), [])
    out = {"grid": n, "cfl": args.cfl, "tol": args.tol, "solver_fp32c": args.solver, "checkpoints": []}
    t0 = time.time()
    step = 0
    for cp in checkpoints:
        while step < cp:
            for name, (g, sp, masses) in sessions.items():
                sp.frame = step
                rep = g.step(sp)
                masses.append((rep.mass_before_advection, rep.mass_after_advection, rep.mass_after))
            step += 1
        g64, g32 = sessions["fp64"][0], sessions["fp32c"][0]
        row = {"step": step, "density": rel(g32.get("density"), g64.get("density"))}
        for c in "uvw":
            row[c] = rel(g32.get(c), g64.get(c))
        out["checkpoints"].append(row)
        print(json.dumps(row), file=sys.stderr, flush=True)
    for name, (g, sp, masses) in sessions.items():
        m = np.array(masses)
        out["mass_" + name] = {"max_rel_change_by_advection": float(np.max(np.abs(m[:, 1] - m[:, 0]) / m[:, 0])),
                               "max_rel_change_after_correction": float(np.max(np.abs(m[:, 2] - m[:, 0]) / m[:, 0]))}
        g.close()
    out["seconds"] = time.time() - t0
    print(json.dumps(out))


if __name__ == "__main__":
    main()
