#!/usr/bin/env python3
"""The C0 configuration on one GPU: the 64^3 plume (source r = 0.1 at (0.5, 0.15, 0.5)
re-injected every step, buoyancy 1, closed box, at rest initially), CFL 1, WENO6, k = 3,
pressure to 1e-8, 50 steps (the reference's main loop, main.cpp:600-721), in the plain FP64
form and the chosen form.

Per form: steps/s over the whole run (fia_step, device time between CUDA events on the
session stream), and the time of each phase of one step measured on the state after the run
(the step's own calls one by one, each between events, 5 repetitions from the same state,
median): density advection (move_substances_3D), velocity advection
(advect_velocity_xyz_flux_advection_3D) and the projection (calc_pressure_gradient_term_3D).
The projection of the last state can take more iterations than the run's average step, so the
phases need not add up to the mean step.  Also the chosen form's density and velocity error
against the plain form after the run, and both forms' mass change after the correction step.

    python c0_report.py [--grid 64] [--steps 50] [--cfl 1] [--tol 1e-8] [--reps 5]

Prints one JSON line.
"""
import argparse
import json
import os
import statistics
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import fia  # noqa: E402
import scenes  # noqa: E402


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run_form(n, precision, args, torch):
    g = fia.Grid3D(n, n, n, 1.0 / n, precision=precision)
    g.set("density", scenes.plume_density(n))
    for c, m in (("u", (n + 1) * n * n), ("v", n * (n + 1) * n), ("w", n * n * (n + 1))):
        g.set(c, np.zeros(m))
    g.set("pressure", np.zeros(n ** 3))
    solver = {"tol": args.tol, "max_iter": 100000}
    sp = fia.step_params(cfl=args.cfl, solver=solver)
    stream = torch.cuda.ExternalStream(g.stream())
    ev = lambda: torch.cuda.Event(enable_timing=True)   # noqa: E731
    e0, e1 = ev(), ev()
    torch.cuda.synchronize()
    e0.record(stream)
    reps, iters = [], []
    for f in range(args.steps):
        sp.frame = f
        r = g.step(sp)
        reps.append(r)
        iters.append(r.solver_iterations)
    e1.record(stream)
    torch.cuda.synchronize()
    run_ms = e0.elapsed_time(e1)
    last = reps[-1]
    state = {c: g.get(c) for c in ("density", "u", "v", "w", "pressure")}
    p = fia.advect_params()
    solver_p = fia.solver_params(tol=args.tol, max_iter=100000)

    def timed(call):
        out = []
        for _ in range(args.reps):
            for c, a in state.items():
                g.set(c, a)
            torch.cuda.synchronize()
            a0, a1 = ev(), ev()
            a0.record(stream)
            call()
            a1.record(stream)
            torch.cuda.synchronize()
            out.append(a0.elapsed_time(a1))
        return statistics.median(out)

    phases = {
        "density_advection_ms": timed(lambda: g.move_substances_3D(last.dt, p)),
        "velocity_advection_ms": timed(lambda: g.advect_velocity_xyz_flux_advection_3D(last.dt, p)),
        "projection_ms": timed(lambda: g.calc_pressure_gradient_term_3D(solver_p)),
    }
    for c, a in state.items():
        g.set(c, a)
    g.close()
    ms_step = run_ms / args.steps
    phases["sum_ms"] = sum(phases.values())
    masses = [(r.mass_before_advection, r.mass_after) for r in reps]
    return state, {
        "steps_per_s": 1e3 / ms_step, "ms_per_step": ms_step, "phases_last_state": phases,
        "pressure_iterations_first_last_max": [iters[0], iters[-1], max(iters)],
        "max_velocity_last": last.max_velocity, "dt_last": last.dt,
        "mass_max_rel_change_after_correction": max(abs(a - b) / b for b, a in masses),
        "status_bits": int(np.bitwise_or.reduce([r.status for r in reps])),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=64)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--cfl", type=float, default=1.0)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args()
    import torch
    n = args.grid
    out = {"config": "C0", "grid": n, "steps": args.steps, "cfl": args.cfl, "tol": args.tol,
           "data": "synthetic plume (sphere source re-injected every step)"}
    s64, out["fp64"] = run_form(n, fia.FIA_FP64, args, torch)
    s32, out["fp32c"] = run_form(n, fia.FIA_FP32C, args, torch)
    out["fp32c_against_fp64"] = {
        "density_rel_l2": rel(s32["density"], s64["density"]),
        "velocity_rel_l2": rel(np.concatenate([s32[c] for c in "uvw"]), np.concatenate([s64[c] for c in "uvw"])),
    }
    out["speedup_steps_per_s"] = out["fp32c"]["steps_per_s"] / out["fp64"]["steps_per_s"]
    print(json.dumps(out))


if __name__ == "__main__":
    main()
