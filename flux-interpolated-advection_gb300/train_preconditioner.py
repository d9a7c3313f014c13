#!/usr/bin/env python3
"""Trains the learned pressure preconditioner on the GPU with the library's own kernels.

Training pairs B p = r (B = -A) come from four sources:
 * the simulator itself: plume runs on an n^3 grid (default 128^3), each with a seeded source
   position in [0.3,0.7] x [0.1,0.2] x [0.3,0.7] and 0-4 seeded solid spheres of radius
   U[0.05,0.15]; every step, before the projection, the projection is solved with Jacobi-PCG
   to a recursive residual of 1e-10 and the pair (r = -div(u) h, pressure) is kept on the
   device (fia_step capture_pair);
 * multi-scale pairs on each run's solids: p = a sum of smoothed white-noise fields over
   scales of 0.7 to 24 cells, r = B p exactly.  Inside flexible CG the preconditioner sees
   residuals, whose spectrum is much rougher than a divergence field's; a network trained on
   divergences alone maps rough residuals to large smooth corrections orthogonal to them and
   the iteration stalls;
 * stress runs (--stress-runs): the plume in a developed flow at CFL 4 (16 seeded Fourier
   modes) with eight small solid spheres of radius U[0.04, 0.1], the configuration under which
   flexible CG used to stall near the solids, each with its pairs captured like the plume runs'
   and multi-scale pairs on its solids;
 * on-policy pairs: residual and error (r_k, e_k = p - x_k) after k flexible-CG iterations with
   the network of the first training phase, on multi-scale problems without solids and, with
   --onpolicy-stress, with the stress runs' solids (where the residual concentrates beside the
   spheres).
The network (fia_unet.cu) is trained with Adam on the energy-norm loss
(z - p)^T B (z - p) / p^T B p of the whole two-level preconditioner, the last run's pairs held
out for validation.  Finally flexible CG with the trained network is compared with Jacobi-PCG
on a fresh plume state.

    python train_preconditioner.py [--grid 128] [--runs 6] [--steps 30] [--iters 6000] \
        [--batch 4] [--lr 1e-3] [--onpolicy 120] [--onpolicy-share 0.25] [--seed 1] \
        [--stress-runs 2] [--stress-steps 20] [--onpolicy-stress 60] \
        [--eval-grids 128,256] [--out weights/unet_precond.f32]

Writes the FP32 parameter vector (fia_learned_num_parameters() floats, little endian) to
--out and the training record (losses, iteration counts) next to it as JSON.
"""
import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import fia  # noqa: E402

DEFAULT_OUT = os.path.join(HERE, "weights", "unet_precond.f32")


def scene(rng):
    """source centre and solid spheres of one training run"""
    src = np.array([rng.uniform(0.3, 0.7), rng.uniform(0.1, 0.2), rng.uniform(0.3, 0.7)])
    centers, radii = [], []
    for _ in range(int(rng.integers(0, 5))):
        for _try in range(100):
            r = rng.uniform(0.05, 0.15)
            c = rng.uniform(r + 0.02, 1.0 - r - 0.02, size=3)
            if np.linalg.norm(c - src) < r + 0.1 + 0.05:
                continue
            if any(np.linalg.norm(c - c2) < r + r2 for c2, r2 in zip(centers, radii)):
                continue
            centers.append(c); radii.append(r)
            break
    return src, centers, radii


def stress_scene(rng, count=8):
    """eight solid spheres of radius U[0.04, 0.1] kept clear of the plume source (the stress
    configuration's solids, drawn from the training seed)"""
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
    return src, centers, radii


def apply_B(p, solid, pin):
    """B p for the 7-point operator with walls and solids as zero-flux faces, p = 0 on the
    pinned cell (the operator of fia_pressure.cu)"""
    n = p.shape[0]
    fluid = ~solid
    ex = solid.copy()
    ex.reshape(-1)[pin] = True
    pv = np.where(ex, 0.0, p)
    out = np.zeros_like(pv)
    for ax in range(3):
        for sh in (1, -1):
            f = np.roll(fluid, sh, axis=ax)
            v = np.roll(pv, sh, axis=ax)
            edge = [slice(None)] * 3
            edge[ax] = 0 if sh == 1 else n - 1
            f[tuple(edge)] = False
            v[tuple(edge)] = 0.0
            out += f * pv - v
    out[ex] = 0.0
    return out


_K2 = {}


def multiscale_field(n, rng):
    """white noise filtered by a random mix of Gaussians of widths 0.7 to 24 cells (each
    normalised to unit variance), applied in Fourier space"""
    if n not in _K2:
        k = np.fft.fftfreq(n) * 2.0 * np.pi
        kz = np.fft.rfftfreq(n) * 2.0 * np.pi
        _K2[n] = k[:, None, None] ** 2 + k[None, :, None] ** 2 + kz[None, None, :] ** 2
    K2 = _K2[n]
    scales = [0.7, 1.5, 3.0, 6.0, 12.0, 24.0]
    weights = rng.uniform(0.0, 1.0, size=len(scales)) ** 3
    weights[rng.integers(len(scales))] = 1.0
    filt = np.zeros_like(K2)
    for s, wgt in zip(scales, weights):
        G = np.exp(-0.5 * s * s * K2)
        filt += wgt * G / np.sqrt(np.mean(G * G))
    p = np.fft.irfftn(np.fft.rfftn(rng.normal(size=(n, n, n))) * filt, s=(n, n, n))
    return p / max(p.std(), 1e-30)


def add_multiscale_pairs(g, n, rng, count):
    solid = g.solid_mask().reshape(n, n, n).astype(bool)
    pin = int(np.nonzero(~solid.reshape(-1))[0][-1])
    for _ in range(count):
        p = multiscale_field(n, rng)
        p[solid] = 0.0
        p.reshape(-1)[pin] = 0.0
        g.learned_add_pair(apply_B(p, solid, pin).ravel(), p.ravel())
    return solid, pin


def add_onpolicy_pairs(g, n, rng, count, iters=(2, 4, 8, 16), solids=None):
    """(r_k, e_k) after k flexible-CG iterations with the current network, on multi-scale
    problems without solids, or with the given solid spheres (centres, radii)"""
    if solids:
        g.set_solid_spheres(*solids)
        solid = g.solid_mask().reshape(n, n, n).astype(bool)
        pin = int(np.nonzero(~solid.reshape(-1))[0][-1])
    else:
        solid = np.zeros((n, n, n), dtype=bool)
        pin = n ** 3 - 1
    added = 0
    while added < count:
        p = multiscale_field(n, rng)
        p[solid] = 0.0
        p.reshape(-1)[pin] = 0.0
        r = apply_B(p, solid, pin)
        k = int(rng.choice(iters))
        x, _ = g.debug_solve_rhs(r.ravel(), fia.solver_params(tol=1e-12, max_iter=k, method=fia.FIA_SOLVER_FCG_LEARNED,
                                                              fallback_iter=k))
        e = p - x.reshape(n, n, n).astype(np.float64)
        e.reshape(-1)[pin] = 0.0
        e[solid] = 0.0
        g.learned_add_pair(apply_B(e, solid, pin).ravel(), e.ravel())
        added += 1
    if solids:
        g.set_solid_spheres([], [])


def reset(g, n):
    z = np.zeros
    g.set("density", z(n ** 3)); g.set("pressure", z(n ** 3))
    g.set("u", z((n + 1) * n * n)); g.set("v", z(n * (n + 1) * n)); g.set("w", z(n * n * (n + 1)))


def capture_runs(g, n, rng, runs, steps, log, synthetic):
    bounds = []
    for run in range(runs):
        src, centers, radii = scene(rng)
        reset(g, n)
        g.set_solid_spheres(centers, radii)
        first = g.learned_num_pairs()
        t0 = time.time()
        for i in range(steps):
            sp = fia.step_params(source_center=tuple(src), capture_pair=1, capture_tol=1e-10, frame=i)
            g.step(sp)
        add_multiscale_pairs(g, n, rng, synthetic)
        bounds.append((first, g.learned_num_pairs()))
        log.append({"run": run, "source": src.tolist(), "spheres": len(radii), "pairs": bounds[-1][1] - first,
                    "seconds": time.time() - t0})
        print("run %d: source %s, %d spheres, %d pairs, %.1f s" % (run, np.round(src, 3), len(radii),
                                                                   bounds[-1][1] - first, time.time() - t0),
              flush=True)
    g.set_solid_spheres([], [])
    return bounds


def capture_stress_runs(g, n, rng, runs, steps, log, synthetic, cfl=4.0):
    """the plume in a developed flow at CFL `cfl` with eight small spheres; returns the pair
    ranges and the solids of each run"""
    import scenes
    bounds, solids = [], []
    for run in range(runs):
        src, centers, radii = stress_scene(rng)
        reset(g, n)
        g.set("density", scenes.plume_density(n))
        u, v, w = scenes.fourier_velocity(n, seed=int(rng.integers(1 << 30)), target_max=cfl * (1.0 / n) * 60.0)
        for name, a in (("u", u), ("v", v), ("w", w)):
            g.set(name, a)
        g.set_solid_spheres(centers, radii)
        first = g.learned_num_pairs()
        t0 = time.time()
        for i in range(steps):
            g.step(fia.step_params(cfl=cfl, source_center=tuple(src), capture_pair=1, capture_tol=1e-10, frame=i))
        add_multiscale_pairs(g, n, rng, synthetic)
        bounds.append((first, g.learned_num_pairs()))
        solids.append((centers, radii))
        log.append({"stress_run": run, "spheres": len(radii), "cfl": cfl, "pairs": bounds[-1][1] - first,
                    "seconds": time.time() - t0})
        print("stress run %d: %d spheres, CFL %g, %d pairs, %.1f s" % (run, len(radii), cfl, bounds[-1][1] - first,
                                                                       time.time() - t0), flush=True)
    g.set_solid_spheres([], [])
    return bounds, solids


def compare_solvers(g, n, seed, steps=12):
    """plume state after `steps` steps; then the same projection by Jacobi-PCG and by FCG"""
    rng = np.random.default_rng(seed)
    src, centers, radii = scene(rng)
    reset(g, n)
    g.set_solid_spheres(centers, radii)
    for i in range(steps):
        g.step(fia.step_params(source_center=tuple(src), frame=i))
    # one more advection without projection gives a divergent velocity to project
    out = {}
    u0 = {k: g.get(k) for k in ("u", "v", "w")}
    for name, method in (("pcg", fia.FIA_SOLVER_PCG_JACOBI), ("fcg_learned", fia.FIA_SOLVER_FCG_LEARNED)):
        for k, a in u0.items():
            g.set(k, a)
        g.advect_velocity_xyz_flux_advection_3D(1.0 / 60.0)
        t0 = time.time()
        rep = g.calc_pressure_3D(fia.solver_params(tol=1e-6, max_iter=20000, method=method, fallback_iter=400))
        g.synchronize()
        out[name] = {"iterations": rep.iterations, "fcg_iterations": rep.fcg_iterations,
                     "rel_residual": rep.rel_residual, "status": rep.status, "seconds": time.time() - t0,
                     "precond_ms": rep.precond_ms}
    g.set_solid_spheres([], [])
    p = multiscale_field(n, rng)
    p.reshape(-1)[-1] = 0.0
    r = apply_B(p, np.zeros((n, n, n), dtype=bool), n ** 3 - 1)
    for name, method in (("pcg_multiscale", fia.FIA_SOLVER_PCG_JACOBI), ("fcg_learned_multiscale", fia.FIA_SOLVER_FCG_LEARNED)):
        _, rep = g.debug_solve_rhs(r.ravel(), fia.solver_params(tol=1e-6, max_iter=20000, method=method,
                                                                 fallback_iter=400))
        out[name] = {"iterations": rep.iterations, "fcg_iterations": rep.fcg_iterations,
                     "rel_residual": rep.rel_residual, "status": rep.status}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--runs", type=int, default=6)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--iters", type=int, default=6000)
    ap.add_argument("--synthetic", type=int, default=25, help="multi-scale pairs per run")
    ap.add_argument("--onpolicy", type=int, default=120, help="flexible-CG residual pairs after phase 1")
    ap.add_argument("--onpolicy-share", type=float, default=0.25,
                    help="fraction of each batch drawn from the on-policy pairs once they exist")
    ap.add_argument("--stress-runs", type=int, default=2, help="plume runs at CFL 4 with eight small spheres")
    ap.add_argument("--stress-steps", type=int, default=20)
    ap.add_argument("--onpolicy-stress", type=int, default=60,
                    help="flexible-CG residual pairs with the stress runs' solids after phase 1")
    ap.add_argument("--eval-grids", default="128", help="grids of the final solver comparison")
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--init", default=None, help="start from these weights instead of a random init")
    args = ap.parse_args()
    n = args.grid
    rng = np.random.default_rng(args.seed)
    g = fia.Grid3D(n, n, n, 1.0 / n, precision=fia.FIA_FP32C)
    g.learned_init(args.seed)
    record = {"grid": n, "runs": [], "args": vars(args)}
    t0 = time.time()
    bounds = capture_runs(g, n, rng, args.runs, args.steps, record["runs"], args.synthetic)
    stress_bounds, stress_solids = capture_stress_runs(g, n, rng, args.stress_runs, args.stress_steps,
                                                       record["runs"], args.synthetic)
    record["capture_seconds"] = time.time() - t0
    train = [i for b in bounds[:-1] + stress_bounds for i in range(b[0], b[1])]
    val = list(range(bounds[-1][0], bounds[-1][1]))
    if args.init:
        g.learned_set_weights(np.fromfile(args.init, dtype=np.float32))
    else:
        g.learned_calibrate(train[len(train) // 2])
    vloss = lambda: float(np.mean([g.learned_loss(i) for i in val]))   # noqa: E731
    record["val_loss_init"] = vloss()
    print("pairs: %d train, %d validation; initial validation loss %.4f" % (len(train), len(val),
                                                                         record["val_loss_init"]), flush=True)
    curve = []
    t0 = time.time()
    phase1 = args.iters // 3
    onpol = []
    for it in range(args.iters):
        if it == phase1 and args.onpolicy > 0:
            first = g.learned_num_pairs()
            t1 = time.time()
            add_onpolicy_pairs(g, n, rng, args.onpolicy)
            for k, sol in enumerate(stress_solids):
                share = args.onpolicy_stress * (k + 1) // len(stress_solids) - args.onpolicy_stress * k // len(stress_solids)
                add_onpolicy_pairs(g, n, rng, share, solids=sol)
            onpol = list(range(first, g.learned_num_pairs()))
            record["onpolicy_seconds"] = time.time() - t1
            print("added %d on-policy pairs (%.1f s)" % (len(onpol), time.time() - t1), flush=True)
        lr = args.lr * 0.5 * (1.0 + math.cos(math.pi * it / args.iters))
        k_on = int(round(args.batch * args.onpolicy_share)) if onpol else 0
        batch = list(rng.choice(train, size=args.batch - k_on, replace=False))
        if k_on:
            batch += list(rng.choice(onpol, size=k_on, replace=False))
        losses = g.learned_train_step(batch, lr)
        curve.append(float(np.mean(losses)))
        if (it + 1) % 250 == 0 or it == 0:
            print("iter %5d  lr %.2e  train loss %.4f (mean of last 250 %.4f)" %
                  (it + 1, lr, curve[-1], float(np.mean(curve[-250:]))), flush=True)
    record["train_seconds"] = time.time() - t0
    record["train_curve_every_10"] = curve[::10]
    record["val_loss_final"] = vloss()
    print("validation loss %.4f -> %.4f" % (record["val_loss_init"], record["val_loss_final"]), flush=True)
    w = g.learned_get_weights()
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    w.astype("<f4").tofile(args.out)
    record["solvers"] = compare_solvers(g, n, args.seed + 1000)
    print(json.dumps(record["solvers"]), flush=True)
    for m in [int(x) for x in args.eval_grids.split(",") if x and int(x) != n]:
        ge = fia.Grid3D(m, m, m, 1.0 / m, precision=fia.FIA_FP32C)
        ge.learned_set_weights(w)
        record["solvers_%d" % m] = compare_solvers(ge, m, args.seed + 1000, steps=6)
        print(m, json.dumps(record["solvers_%d" % m]), flush=True)
        ge.close()
    with open(os.path.splitext(args.out)[0] + ".json", "w") as f:
        json.dump(record, f, indent=1)
    g.close()


if __name__ == "__main__":
    main()
