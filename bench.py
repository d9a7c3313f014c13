#!/usr/bin/env python3
"""Benchmark: steps/s of the 256^3 smoke plume step on GB300 (flux-interpolated advection
of density and velocity, WENO6 with 3 Gauss points per half cell, pressure to 1e-6 relative
residual), in the chosen form (FP32 advection with compensated sums, FP64 reductions).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One JSON line on stdout (rank 0).  For N > 1 (torchrun) every rank runs an independent
replica of the plume on its own GPU ("replicas only": the path is not sharded), ranks meet
at a barrier around the timed region, and the time is the max over ranks.

--impl reference times the CPU implementation of the same step (the oracle, a restatement
of the reference's 3D path; the reference itself needs Eigen, amgcl, OpenVDB and GL and is
not built on the GPU host) on the host cores, on a bounded sample of the workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "flux-interpolated-advection_gb300")
for p in (PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "steps/s at 256^3 smoke step (flux advection of density and velocity + pressure to 1e-6)"
UNIT = "steps/s"
# FP32 operation count of one 1D WENO6 evaluation as implemented in fia_device.cuh
# (weno6_eval, FP32 form: differences 12, three cubic candidates 18, three smoothness
# indicators in Horner form 42, nonlinear weights and the weighted sum 26; an FMA counted as
# two).  The face kernel counts the 1D evaluations it executes.
WENO1D_FLOP = 98
FP32_LANES_PER_SM = 128
SMS = 152


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def traffic_from_profile():
    """dram bytes per k_quad32 launch at 256^3 from the committed ncu summary (measured on a
    smaller plume and scaled by the pieces processed), if present."""
    path = os.path.join(ROOT, "profiles", "k_quad32_plume128.md")
    try:
        for line in open(path):
            if line.strip().startswith("traffic_bytes_per_launch_256:"):
                return float(line.split(":")[1])
    except Exception:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        try:
            import torch
            if not torch.cuda.is_available():
                backend = "gloo"
            else:
                torch.cuda.set_device(local)
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
        return world, rank, local, dist
    return 1, 0, local, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(x, dist):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


MAX_DT = 1.0 / 60.0   # fia_default_step_params: one step per movie frame at 60 fps


def plume_state(n, cfl):
    """The plume density (sphere r=0.1 at (0.5,0.15,0.5)) in a developed flow: a seeded
    divergence-free velocity (curl of 16 Fourier modes, wavenumbers 1-8) scaled so that the
    frame-length step runs at the requested CFL number (max|u| = cfl h / dt)."""
    import scenes
    rho = scenes.plume_density(n)
    u, v, w = scenes.fourier_velocity(n, seed=1, target_max=cfl * (1.0 / n) / MAX_DT)
    return rho, u, v, w


# ------------------------------------------------------------------------------------
# CPU baseline: the oracle's step on a bounded sample, extrapolated to the full grid
# ------------------------------------------------------------------------------------
def cpu_step_sample(n_sample, n_full, cfl, threads, steps=1):
    """Time one full oracle step (velocity + density advection with all three passes,
    pressure CG to 1e-6) on an n_sample^3 plume carrying a developed (Fourier) velocity at
    the same CFL, and extrapolate to n_full^3: advection work per cell is the same at the
    same CFL, so it scales with the cell count; Jacobi-CG iterations grow with n, so the
    pressure time scales with n^4.  Returns (seconds per full-size step, details)."""
    import scenes
    from oracle import Oracle
    O = Oracle()
    n = n_sample
    h = 1.0 / n
    u, v, w = scenes.fourier_velocity(n, seed=1)
    rho = scenes.plume_density(n)
    dt = cfl * h / max(np.abs(u).max(), np.abs(v).max(), np.abs(w).max())
    t_adv, t_p = [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        u2, v2, w2, _ = O.advect_velocity_3D((n, n, n), h, u, v, w, dt, nthreads=threads)
        r2, _ = O.move_substances_3D((n, n, n), h, u2, v2, w2, rho, dt, nthreads=threads)
        t1 = time.perf_counter()
        b = O.pressure_rhs((n, n, n), h, u2, v2, w2)
        p, it, rr = O.pressure_solve((n, n, n), b, tol=1e-6, maxit=100000)
        t2 = time.perf_counter()
        t_adv.append(t1 - t0); t_p.append(t2 - t1)
    ta, tp = min(t_adv), min(t_p)
    scale = (n_full / n) ** 3
    full = ta * scale + tp * scale * (n_full / n)
    return full, {"sample_grid": n, "advection_s": ta, "pressure_s": tp, "pressure_iters": it}


def run_reference(args, world, rank, dist):
    """--impl reference: the CPU oracle on the host cores (rank 0 only)."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n_sample = args.cpu_sample_grid
    for _ in range(args.warmup):
        cpu_step_sample(n_sample, args.grid, args.cfl, threads)
    per = []
    for _ in range(args.steps):
        s, det = cpu_step_sample(n_sample, args.grid, args.cfl, threads)
        per.append(s)
    sec = statistics.median(per)
    value = 1.0 / sec
    sample = ("one full step of the CPU oracle (restated reference path, %d threads) on a %d^3 plume with a "
              "developed Fourier velocity at CFL %g, extrapolated to %d^3 by cell count (advection) and "
              "cell count x n (Jacobi-CG pressure)" % (threads, n_sample, args.cfl, args.grid))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(args, reference=True),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_of(args, reference=False):
    return {"workload": "smoke plume %d^3 (sphere source r=0.1 at (0.5,0.15,0.5), buoyancy 1.0, closed box) "
                        "in a developed divergence-free flow (16 seeded Fourier modes) at CFL %g, flux advection of density and velocity (WENO6, k=3, zero-velocity "
                        "correction), pressure solved to %g relative residual" % (args.grid, args.cfl, args.tol),
            "grid": args.grid, "cfl": args.cfl, "interpolation": "WENO6", "gauss_points": 3,
            "pressure_tol": args.tol,
            "pressure_solver": ("flexible CG with the learned two-level preconditioner (BF16 U-Net), Jacobi-PCG "
                                "fallback after %d iterations" % args.fallback_iter
                                if (args.solver == "learned" and args.precision == "fp32c" and not reference)
                                else "Jacobi-PCG (FP64 dot products)"),
            "precision": "fp64 oracle" if reference else args.precision,
            "l2": "inputs larger than L2 (fields of %d^3, working set above 1 GB)" % args.grid,
            "parallelism": "replicas"}


# ------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------
def compare_projection(g, args):
    """One projection of the current (advected, divergent) velocity by Jacobi-PCG and by the
    learned FCG, each from p = 0 to the bench tolerance (FP64 residual), device-timed."""
    import torch
    import fia
    u0 = {k: g.get(k) for k in ("u", "v", "w")}
    g.advect_velocity_xyz_flux_advection_3D(MAX_DT)
    u1 = {k: g.get(k) for k in ("u", "v", "w")}
    out = {}
    stream = torch.cuda.ExternalStream(g.stream())
    for name, method in (("pcg", fia.FIA_SOLVER_PCG_JACOBI), ("learned_fcg", fia.FIA_SOLVER_FCG_LEARNED)):
        for k, a in u1.items():
            g.set(k, a)
        sp = fia.solver_params(tol=args.tol, max_iter=20000, method=method, fallback_iter=args.fallback_iter)
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        rep = g.calc_pressure_3D(sp)
        e1.record(stream)
        torch.cuda.synchronize()
        out[name] = {"iterations": rep.iterations, "fcg_iterations": rep.fcg_iterations, "ms": e0.elapsed_time(e1),
                     "rel_residual": rep.rel_residual, "status": rep.status, "precond_ms": rep.precond_ms}
    for k, a in u0.items():
        g.set(k, a)
    out["time_ratio_pcg_over_learned"] = out["pcg"]["ms"] / out["learned_fcg"]["ms"]
    return out


def fp64_plain_arm(args):
    """The plain form (FP64 throughout, Jacobi-PCG) on the same initial plume: one untimed
    step, then args.fp64_steps timed steps (device events)."""
    import torch
    import fia
    n = args.grid
    g = fia.Grid3D(n, n, n, 1.0 / n, precision=fia.FIA_FP64)
    rho, u, v, w = plume_state(n, args.cfl)
    for name, a in (("density", rho), ("u", u), ("v", v), ("w", w)):
        g.set(name, a)
    sp = fia.step_params(cfl=args.cfl, max_dt=MAX_DT, solver={"tol": args.tol, "max_iter": 20000})
    sp.frame = 0
    g.step(sp)
    stream = torch.cuda.ExternalStream(g.stream())
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    reps = []
    for i in range(args.fp64_steps):
        sp.frame = 1 + i
        reps.append(g.step(sp))
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.fp64_steps
    g.close()
    return {"steps_per_s": 1e3 / ms, "ms_per_step": ms, "steps": args.fp64_steps,
            "pressure_iterations": reps[-1].solver_iterations,
            "pressure_rel_residual": reps[-1].solver_rel_residual}

def run_gpu(args, world, rank, local, dist):
    import torch
    import fia
    torch.cuda.set_device(local)
    prec = fia.FIA_FP32C if args.precision == "fp32c" else fia.FIA_FP64
    n = args.grid
    g = fia.Grid3D(n, n, n, 1.0 / n, precision=prec)
    rho, u, v, w = plume_state(n, args.cfl)
    for name, a in (("density", rho), ("u", u), ("v", v), ("w", w)):
        g.set(name, a)
    solver = {"tol": args.tol, "max_iter": 20000}
    weights_used = None
    if args.solver == "learned" and prec == fia.FIA_FP32C:
        g.learned_set_weights(np.fromfile(args.weights, dtype="<f4"))
        solver.update(method=fia.FIA_SOLVER_FCG_LEARNED, fallback_iter=args.fallback_iter)
        weights_used = os.path.relpath(args.weights, ROOT)
    sp = fia.step_params(cfl=args.cfl, max_dt=MAX_DT, solver=solver)
    stream = torch.cuda.ExternalStream(g.stream())
    frame = 0
    for _ in range(args.warmup):
        sp.frame = frame
        r = g.step(sp)
        if args.verbose:
            print("warmup frame %d: dt %.3e umax %.3e mass %.6e -> %.6e (corrected %.6e) CG %d it rel %.2e status %d"
                  % (frame, r.dt, r.max_velocity, r.mass_before_advection, r.mass_after_advection, r.mass_after,
                     r.solver_iterations, r.solver_rel_residual, r.status), file=sys.stderr, flush=True)
        frame += 1
    g.synchronize()
    c0 = g.pass_counters()
    g.profile_faces(64 * args.steps)
    sampler = ClockSampler(local)
    sampler.start()
    barrier(dist)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    reps = []
    for _ in range(args.steps):
        sp.frame = frame
        reps.append(g.step(sp))
        frame += 1
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(dist)
    clocks = sampler.stop()
    t_ms = e0.elapsed_time(e1)
    face_ms, face_launches = g.read_face_profile()
    c1 = g.pass_counters()
    t_max = max_over_ranks(t_ms, dist)
    value = world * args.steps / (t_max / 1e3)

    # ---- end-to-end through the public API with host buffers (pinned), every step:
    #      H2D of density,u,v,w; the step; D2H of density,u,v,w
    e2e = None
    if args.e2e_steps > 0:
        host = {}
        for name in ("density", "u", "v", "w"):
            a = g.get(name).astype(np.float32)
            t = torch.empty(a.size, dtype=torch.float32, pin_memory=True)
            t.numpy()[:] = a
            host[name] = t
        lib = g.lib
        field = fia.FIELD
        torch.cuda.synchronize()
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            for name, t in host.items():
                fia._check(lib.fia_set_field(g.s, field[name], t.data_ptr(), fia.FIA_HOST_F32), "set")
            sp.frame = frame
            g.step(sp)
            frame += 1
            for name, t in host.items():
                fia._check(lib.fia_get_field(g.s, field[name], t.data_ptr(), fia.FIA_HOST_F32), "get")
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        barrier(dist)
        te = max_over_ranks(t1 - t0, dist)
        nbytes = sum(t.numel() * 4 for t in host.values())
        e2e = {"value": world * args.e2e_steps / te, "unit": UNIT, "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes, "steps": args.e2e_steps,
               "path": "fia_set_field x4 (pinned FP32 host) + fia_step + fia_get_field x4"}

    # ---- roofline of the dominant kernel (k_quad32: per-piece quadrature + WENO6)
    evals = c1[3] - c0[3]
    flops = evals * WENO1D_FLOP
    faces = c1[0] - c0[0]
    pieces = c1[1] - c0[1]
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    peak_tf = SMS * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    achieved_tf = flops / (face_ms / 1e3) / 1e12 if face_ms > 0 else 0.0
    traffic = traffic_from_profile()
    peaks = read_peaks()
    # algorithmic bytes of one k_quad32 launch (one pass, all three face families): per piece
    # its record (16 B) and face tag (4 B) read and its flux (4 B) written, plus the advected
    # field (4 B per node) and psi (8 B per node) read once
    launches = max(face_launches, 1)
    alg_bytes = (24.0 * pieces + 12.0 * n ** 3 * launches) / launches
    roofline = {
        "bound": "fp32-simt",
        "kernel": "k_quad32",
        "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s", "frac": achieved_tf / peak_tf if peak_tf else None,
        "peak_source": "152 SMs x 128 FP32 lanes x 2 FLOP x median SM clock sampled in the run (%.0f MHz); "
                       "no FP32-SIMT figure in MEASURED_PEAKS.json" % sm_mhz,
        "algorithmic_flop": "1D WENO6 evaluations executed, counted on the device, x %d FLOP" % WENO1D_FLOP,
        "launches": face_launches, "avg_launch_ms": face_ms / launches,
        "flop_per_launch": flops / launches,
        "share_of_step": (face_ms / t_ms) if t_ms > 0 else None,
        "traffic": traffic,
        "hbm": {"achieved": alg_bytes / (face_ms / launches / 1e3) / 1e9 if face_ms > 0 else None,
                "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                "bytes_per_launch": alg_bytes},
    }
    # ---- CPU baseline (rank 0, N=1 only)
    cpu = None
    if rank == 0 and world == 1 and args.cpu_sample_grid > 0:
        threads = os.cpu_count() or 1
        sec, det = cpu_step_sample(args.cpu_sample_grid, n, args.cfl, threads)
        cpu = {"value": 1.0 / sec, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "one oracle step on a %d^3 plume with a developed velocity at CFL %g (advection %.2f s, "
                         "pressure %.2f s, %d CG iterations), extrapolated to %d^3 by cell count "
                         "(x n for the pressure)" % (det["sample_grid"], args.cfl, det["advection_s"],
                                                     det["pressure_s"], det["pressure_iters"], n)}
    last = reps[-1]
    fp64 = fp64_plain_arm(args) if (rank == 0 and args.fp64_steps > 0 and prec == fia.FIA_FP32C) else None
    solvers = compare_projection(g, args) if (rank == 0 and weights_used) else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if prec == fia.FIA_FP32C else "f64", "data": "synthetic", "config": config_of(args),
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": c1[4] - c0[4],
        "clocks": clocks,
        "details": {"faces_per_s": faces / (t_ms / 1e3), "cells_per_s": n ** 3 * args.steps / (t_ms / 1e3),
                    "pieces_per_face": pieces / max(faces, 1), "faces_clipped_both_sides": c1[2] - c0[2],
                    "weno6_1d_evaluations": evals, "face_kernel_ms": face_ms,
                    "last_dt": last.dt, "last_max_velocity": last.max_velocity,
                    "last_pressure_iterations": last.solver_iterations,
                    "last_pressure_rel_residual": last.solver_rel_residual,
                    "mass_after_correction": last.mass_after, "frames_run": frame,
                    "pressure_fcg_iterations": last.solver_fcg_iterations,
                    "precond_ms_last_step": last.precond_ms,
                    "pressure_status_bits": last.status & 48,
                    "weights": weights_used,
                    "fp64_plain": fp64,
                    "projection_pcg_vs_learned": solvers,
                    "speedup_vs_fp64_plain": (value / fp64["steps_per_s"]) if fp64 else None},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    g.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--grid", type=int, default=256)
    ap.add_argument("--cfl", type=float, default=2.0)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--precision", default="fp32c", choices=["fp32c", "fp64"])
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-sample-grid", type=int, default=24)
    ap.add_argument("--verbose", action="store_true", help="per-step reports of the warm-up on stderr")
    ap.add_argument("--solver", default="learned", choices=["learned", "pcg"],
                    help="pressure solver of the FP32 form: flexible CG with the learned preconditioner "
                         "(Jacobi-PCG fallback) or Jacobi-PCG")
    ap.add_argument("--weights", default=os.path.join(PKG, "weights", "unet_precond.f32"))
    ap.add_argument("--fallback-iter", type=int, default=200)
    ap.add_argument("--fp64-steps", type=int, default=1,
                    help="steps of the plain FP64 form on the same state, timed after the main arm")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.solver == "learned" and not os.path.exists(args.weights):
        print("bench: no preconditioner weights at %s; using Jacobi-PCG" % args.weights, file=sys.stderr)
        args.solver = "pcg"
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, dist)
    else:
        run_gpu(args, world, rank, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
