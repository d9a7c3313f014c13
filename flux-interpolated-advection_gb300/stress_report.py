#!/usr/bin/env python3
"""The chosen form under stress: the plume with seeded solid spheres at a high CFL number.

    python stress_report.py [--grid 384] [--spheres 8] [--cfl 4] [--steps 10] [--warmup 2] \
        [--fallback-iter 200] [--compare-grid 64] [--compare-steps 20]

Runs --warmup + --steps steps of the plume (source r = 0.1 at (0.5, 0.15, 0.5), buoyancy 1)
in the developed flow of bench.py scaled to the given CFL, with --spheres solid spheres of
radius U[0.04, 0.1] (seed 7, kept clear of the source), FP32 advection and flexible CG with
the learned preconditioner (Jacobi-PCG after --fallback-iter iterations; by default the
weights trained with solid-heavy CFL-4 runs, weights/unet_precond_solids.f32).  Reports
steps/s (device time), pieces per face, pressure iterations and fallbacks, the largest
velocity and the mass.  The plain FP64 form is too slow to run many steps at this size, so the
difference between the forms is measured on --compare-grid with the same settings.  Prints
one JSON line.
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

MAX_DT = 1.0 / 60.0


def spheres(count, seed=7):
    rng = np.random.default_rng(seed)
    src = np.array([0.5, 0.15, 0.5])
    centers, radii = [], []
    while len(radii) < count:
        r = rng.uniform(0.04, 0.1)
        c = rng.uniform(r + 0.02, 1.0 - r - 0.02, size=3)
        if np.linalg.norm(c - src) < r + 0.15:
            continue
        if any(np.linalg.norm(c - c2) < r + r2 for c2, r2 in zip(centers, radii)):
            continue
        centers.append(c); radii.append(r)
    return centers, radii


def session(n, precision, args, learned):
    g = fia.Grid3D(n, n, n, 1.0 / n, precision=precision)
    g.set("density", scenes.plume_density(n))
    u, v, w = scenes.fourier_velocity(n, seed=1, target_max=args.cfl * (1.0 / n) / MAX_DT)
    for name, a in (("u", u), ("v", v), ("w", w)):
        g.set(name, a)
    c, r = spheres(args.spheres)
    g.set_solid_spheres(c, r)
    solver = {"tol": args.tol, "max_iter": 50000}
    if learned:
        g.learned_set_weights(np.fromfile(args.weights, dtype="<f4"))
        solver.update(method=fia.FIA_SOLVER_FCG_LEARNED, fallback_iter=args.fallback_iter)
    return g, fia.step_params(cfl=args.cfl, max_dt=MAX_DT, solver=solver)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=384)
    ap.add_argument("--spheres", type=int, default=8)
    ap.add_argument("--cfl", type=float, default=4.0)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--fallback-iter", type=int, default=200)
    ap.add_argument("--compare-grid", type=int, default=64)
    ap.add_argument("--compare-steps", type=int, default=20)
    ap.add_argument("--weights", default=os.path.join(HERE, "weights", "unet_precond_solids.f32"))
    args = ap.parse_args()
    import torch
    n = args.grid
    out = {"grid": n, "spheres": args.spheres, "cfl": args.cfl, "tol": args.tol, "fallback_iter": args.fallback_iter}
    g, sp = session(n, fia.FIA_FP32C, args, True)
    u0 = g.max_abs_velocity()
    for i in range(args.warmup):
        sp.frame = i
        g.step(sp)
    c0 = g.pass_counters()
    stream = torch.cuda.ExternalStream(g.stream())
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    reps = []
    for i in range(args.steps):
        sp.frame = args.warmup + i
        reps.append(g.step(sp))
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    c1 = g.pass_counters()
    out.update({
        "steps_per_s": 1e3 / ms, "ms_per_step": ms,
        "pieces_per_face": (c1[1] - c0[1]) / max(c1[0] - c0[0], 1),
        "faces_per_s": (c1[0] - c0[0]) / (ms * args.steps / 1e3),
        "pressure_iterations": [r.solver_iterations for r in reps],
        "pressure_fcg_iterations": [r.solver_fcg_iterations for r in reps],
        "fallbacks": sum(1 for r in reps if r.status & fia.FIA_STATUS_SOLVER_FALLBACK),
        "pressure_rel_residual_max": max(r.solver_rel_residual for r in reps),
        "max_velocity_initial": u0, "max_velocity": [r.max_velocity for r in reps], "dt_last": reps[-1].dt,
        "mass_rel_change_max": max(abs(r.mass_after - r.mass_before_advection) / r.mass_before_advection
                                   for r in reps if r.mass_before_advection > 0),
        "status_bits": int(np.bitwise_or.reduce([r.status for r in reps])),
    })
    g.close()
    # chosen form against the plain form on the comparison grid
    m = args.compare_grid
    if m > 0:
        t0 = time.time()
        sessions = [session(m, fia.FIA_FP64, args, False), session(m, fia.FIA_FP32C, args, True)]
        for i in range(args.compare_steps):
            for gg, ss in sessions:
                ss.frame = i
                gg.step(ss)
        (g64, _), (g32, _) = sessions
        rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))  # noqa: E731
        out["compare"] = {"grid": m, "steps": args.compare_steps,
                          "density_rel_l2": rel(g32.get("density"), g64.get("density")),
                          "velocity_rel_l2": [rel(g32.get(c), g64.get(c)) for c in "uvw"],
                          "max_velocity": [g64.max_abs_velocity(), g32.max_abs_velocity()],
                          "seconds": time.time() - t0}
        for gg, _ in sessions:
            gg.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
