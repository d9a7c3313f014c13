#!/usr/bin/env python3
"""Timing of the pressure solvers on one GPU: one application of the learned preconditioner,
one Jacobi-PCG iteration, and a projection solved by Jacobi-PCG and by flexible CG with the
learned preconditioner (same right-hand side, tolerance 1e-6 in the FP64 residual).

    python solver_bench.py [--grid 256] [--reps 5] [--weights weights/unet_precond.f32]

The right-hand side is B p for a pressure of white noise filtered at 1.5, 6 and 24 cells
(closed box, no solids).  Prints one JSON line.
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
from train_preconditioner import apply_B, multiscale_field  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=256)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--weights", default=os.path.join(HERE, "weights", "unet_precond.f32"))
    args = ap.parse_args()
    n = args.grid
    g = fia.Grid3D(n, n, n, 1.0 / n, precision=fia.FIA_FP32C)
    g.learned_set_weights(np.fromfile(args.weights, dtype="<f4"))
    rng = np.random.default_rng(0)
    out = {"grid": n}
    # one preconditioner application (host round trip of r and z included in the wall time;
    # the device time of the network is reported by the FCG below)
    r = rng.normal(size=n ** 3).astype(np.float32)
    t = []
    for _ in range(args.reps):
        g.synchronize()
        t0 = time.perf_counter()
        g.debug_precondition(r)
        t.append(time.perf_counter() - t0)
    out["precondition_wall_s"] = min(t)
    p = multiscale_field(n, rng)
    p.reshape(-1)[-1] = 0.0
    rhs = apply_B(p, np.zeros((n, n, n), dtype=bool), n ** 3 - 1).ravel()
    for name, method in (("pcg", fia.FIA_SOLVER_PCG_JACOBI), ("learned_fcg", fia.FIA_SOLVER_FCG_LEARNED)):
        sp = fia.solver_params(tol=1e-6, max_iter=20000, method=method, fallback_iter=400)
        g.synchronize()
        t0 = time.perf_counter()
        x, rep = g.debug_solve_rhs(rhs, sp)
        dt = time.perf_counter() - t0
        out[name] = {"iterations": rep.iterations, "fcg_iterations": rep.fcg_iterations, "wall_s": dt,
                     "rel_residual": rep.rel_residual, "status": rep.status, "precond_ms": rep.precond_ms,
                     "solution_rel_error": float(np.linalg.norm(x - p.ravel()) / np.linalg.norm(p))}
    if out["learned_fcg"]["fcg_iterations"]:
        out["precond_ms_per_application"] = out["learned_fcg"]["precond_ms"] / out["learned_fcg"]["fcg_iterations"]
    print(json.dumps(out))
    g.close()


if __name__ == "__main__":
    main()
