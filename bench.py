#!/usr/bin/env python3
"""Benchmark of the flux-interpolated advection step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Headline workload (the isolated advection operator of the benchmark configurations): one
density flux-advection step (move_substances_3D: the main pass, the zero-velocity pass and the
error-advection pass; WENO6, 3 Gauss points per half cell, y-integral quadrature,
xz-CellFaceAligned split) on a 128^3 grid, the velocity the curl of 16 seeded Fourier modes
(wavenumbers 1-8) scaled to a maximum CFL number of 2, the density 32 seeded Gaussian blobs.
The metric is unique faces per second (3 N^2 (N+1) faces per step).

* gb300 (default): the chosen form (FP32 advection with compensated sums) with the fields
  resident on the device; `e2e` the same step through the host-buffer C entry point
  (fia_move_substances_3D_host) from pinned host memory; `cpu_baseline` the streaming-tile
  CPU port (oracle/cpu_stream.inl) on the whole step, all host threads; details: the plain FP64 form at the same configuration, the chosen form's
  error against it, and the 256^3 smoke step of the target (chosen form with the learned
  preconditioner against the plain FP64 form from the same state, and the solver's share).
* reference: the CPU oracle (a restatement of the reference's 3D path with its structure:
  per-cell faces, std::thread over cells), all host threads, on the same configuration.  Each
  step is one x-slab of the grid; successive steps walk through the slabs, so the timed steps
  compute the whole step's faces slab by slab.  The reference itself needs Eigen, amgcl,
  OpenVDB and GL and is not built on the GPU host.

One JSON line on stdout (rank 0).  For N > 1 (torchrun) every rank runs an independent
replica on its own GPU ("replicas only": the path is not sharded), ranks meet at a barrier
around the timed region, and the time is the max over ranks.
"""
import argparse
import ctypes
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

METRIC = ("unique faces/s of one density flux-advection step at %d^3 (move_substances_3D, three passes, "
          "Fourier velocity at CFL 2, 32 Gaussian blobs)")
UNIT = "faces/s"
VELOCITY_SEED, DENSITY_SEED = 101, 102
CFL = 2.0
# FP32 operation count of one 1D WENO6 evaluation as implemented in fia_device.cuh
# (weno6_eval, FP32 form: differences 12, three cubic candidates 18, three smoothness
# indicators in Horner form with eps as the start of each chain 45, nonlinear weights by
# reciprocals 9, the weighted sum and its normalisation 9; an FMA counted as two, a
# reciprocal as one).  The face kernel counts the 1D evaluations it executes.
WENO1D_FLOP = 93
FP32_LANES_PER_SM = 128
SMS = 152
L2_BYTES = 129 * 2 ** 20
MAX_DT = 1.0 / 60.0   # fia_default_step_params: one step per movie frame at 60 fps


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def traffic_from_profile():
    """DRAM bytes per k_quad32 launch of this workload from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "k_quad32_c1_128.md")
    try:
        for line in open(path):
            if line.strip().startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except Exception:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 50 ms while the GPU is loaded."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "50"],
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


# ------------------------------------------------------------------------------------
# the workload
# ------------------------------------------------------------------------------------
def c1_state(n):
    """The isolated-operator configuration: divergence-free Fourier velocity (max |u| = 1) and
    Gaussian blobs; dt puts the fastest face at CFL 2."""
    import scenes
    u, v, w = scenes.fourier_velocity(n, seed=VELOCITY_SEED)
    rho = scenes.gaussian_blobs(n, seed=DENSITY_SEED)
    dt = CFL * (1.0 / n) / max(np.abs(u).max(), np.abs(v).max(), np.abs(w).max())
    return rho, u, v, w, dt


def unique_faces(n):
    return 3 * n * n * (n + 1)


def config_of(args):
    """Identical for both arms (the implementation is in `impl` and `dtype`)."""
    return {"workload": "isolated density flux-advection step (move_substances_3D: main, zero-velocity and "
                        "error-advection passes) on %d^3, velocity = curl of 16 seeded Fourier modes (wavenumbers "
                        "1-8) at max CFL %g, density = 32 seeded Gaussian blobs" % (args.grid, CFL),
            "grid": args.grid, "cfl": CFL, "interpolation": "WENO6", "gauss_points": 3, "split": "xz-CellFaceAligned",
            "velocity_seed": VELOCITY_SEED, "density_seed": DENSITY_SEED,
            "l2": "flushed between timed steps (a 256 MB write outside the timed events)",
            "parallelism": "replicas"}


# ------------------------------------------------------------------------------------
# CPU: the oracle, slab by slab
# ------------------------------------------------------------------------------------
def slab_margin(u, v, w, dt, h):
    """cells the error pass reads beyond a slab: the largest backtrace displacement, rounded up, + 1"""
    disp = dt * max(np.abs(u).max(), np.abs(v).max(), np.abs(w).max()) / h
    return int(np.ceil(disp)) + 1


class OracleSlabs:
    """The oracle's density step on x-slabs of the grid; slab i of the sequence is i mod count."""

    def __init__(self, n, slab, threads):
        from oracle import Oracle
        self.O = Oracle()
        self.n = n
        self.h = 1.0 / n
        self.rho, self.u, self.v, self.w, self.dt = c1_state(n)
        self.margin = slab_margin(self.u, self.v, self.w, self.dt, self.h)
        self.slabs = [(x0, min(n, x0 + slab)) for x0 in range(0, n, slab)]
        self.threads = threads
        self.out = np.zeros(n ** 3)
        self.i = 0

    def step(self):
        x0, x1 = self.slabs[self.i % len(self.slabs)]
        self.i += 1
        t0 = time.perf_counter()
        _, st, _ = self.O.move_substances_slab((self.n,) * 3, self.h, self.u, self.v, self.w, self.rho, self.dt, x0, x1,
                                               self.margin, nthreads=self.threads, out=self.out)
        t1 = time.perf_counter()
        return t1 - t0, unique_faces(self.n) * (x1 - x0) / self.n, st


def run_reference(args, world, rank, dist):
    """--impl reference: the CPU oracle on the host cores (rank 0 only)."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    S = OracleSlabs(args.grid, args.ref_slab, threads)
    for _ in range(args.warmup):
        S.step()
    secs, faces = [], 0.0
    for _ in range(args.steps):
        s, f, _ = S.step()
        secs.append(s)
        faces += f
    total = sum(secs)
    value = faces / total
    sample = ("the oracle's density step (per-cell faces, as the reference) on x-slabs of %d planes of the %d^3 grid, "
              "%d threads; step i is slab i mod %d, so the %d timed steps cover %.2f full steps; each slab also "
              "recomputes the zero-velocity pass on %d planes either side, which the error pass reads"
              % (args.ref_slab, args.grid, threads, len(S.slabs), args.steps, args.steps / len(S.slabs), S.margin))
    line = {
        "impl": "reference", "metric": METRIC % args.grid, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(args),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "details": {"slab_seconds": secs, "slabs_per_full_step": len(S.slabs),
                    "full_step_seconds_estimate": total / args.steps * len(S.slabs)},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(args):
    """The streaming-tile CPU baseline (oracle/cpu_stream.inl: the presort-and-stream design of
    the reference's sginterp3 interpolator, unique vertices and faces, std::thread) on the whole
    step of the same workload, all host threads: faces/s measured, no sampling."""
    from oracle import Oracle
    threads = os.cpu_count() or 1
    n = args.grid
    h = 1.0 / n
    rho, u, v, w, dt = c1_state(n)
    O = Oracle()
    t0 = time.perf_counter()
    _, st, faces = O.stream_move_substances_slab((n,) * 3, h, u, v, w, rho, dt, 0, n, slab_margin(u, v, w, dt, h),
                                                 nthreads=threads)
    secs = time.perf_counter() - t0
    return {"value": unique_faces(n) / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "the whole step (%d unique faces, %.1f s) by the streaming-tile CPU port (FP64; the "
                      "presort-and-stream design of the reference's sginterp3 interpolator without ISPC, unique "
                      "vertices and faces, %d threads)" % (unique_faces(n), secs, threads)}


# ------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------
def c1_session(fia, n, precision, state):
    rho, u, v, w, dt = state
    g = fia.Grid3D(n, n, n, 1.0 / n, precision=precision)
    for name, a in (("density", rho), ("u", u), ("v", v), ("w", w)):
        g.set(name, a)
    return g


def timed_steps(g, stream, steps, dt, params, flush):
    """device time of `steps` density steps, each bracketed by events on the session stream,
    with the L2 flushed between them (outside the events)"""
    import torch
    evs = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.add_(1)
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.move_substances_3D(dt, params)
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in evs)


def fp64_same_config(fia, args, state, flush, stream_of):
    """The plain FP64 form on the same configuration: faces/s, and the chosen form's error
    against it after one step from the same state."""
    n = args.grid
    g64 = c1_session(fia, n, fia.FIA_FP64, state)
    g32 = c1_session(fia, n, fia.FIA_FP32C, state)
    p = fia.advect_params()
    dt = state[4]
    g64.move_substances_3D(dt, p)
    g32.move_substances_3D(dt, p)
    a, b = g32.get("density"), g64.get("density")
    err = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    ms = timed_steps(g64, stream_of(g64), args.fp64_steps, dt, p, flush)
    g64.close(); g32.close()
    return {"faces_per_s": unique_faces(n) * args.fp64_steps / (ms / 1e3), "ms_per_step": ms / args.fp64_steps,
            "steps": args.fp64_steps, "chosen_form_rel_l2_after_one_step": err,
            "note": "the plain form matches the CPU oracle to 1e-10 at this size (tests/test_gpu_configs.py)"}


def plume_state(n, cfl):
    """The 256^3 smoke of the target: the plume density (sphere r = 0.1 at (0.5, 0.15, 0.5)) in
    a developed flow (16 seeded Fourier modes) scaled so that the frame-length step runs at
    CFL `cfl`."""
    import scenes
    rho = scenes.plume_density(n)
    u, v, w = scenes.fourier_velocity(n, seed=1, target_max=cfl * (1.0 / n) / MAX_DT)
    return rho, u, v, w


def north_star(fia, args):
    """The 256^3 smoke step of the target: flux advection of density and velocity, pressure to
    1e-6 (FP64 residual in both forms).  The chosen form (FP32 advection, learned-preconditioned
    FCG) is timed over args.ns_steps steps after args.ns_warmup; the plain FP64 form (Jacobi-PCG)
    and the chosen form's advection with Jacobi-PCG are timed over args.ns_fp64_steps steps from
    the state the chosen form's timed steps started from (same frame)."""
    import torch
    n = args.ns_grid
    weights = args.weights
    tol = 1e-6

    def session(prec, state):
        g = fia.Grid3D(n, n, n, 1.0 / n, precision=prec)
        for name, a in zip(("density", "u", "v", "w"), state):
            g.set(name, a)
        return g

    def run(g, sp, frame0, steps):
        stream = torch.cuda.ExternalStream(g.stream())
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        reps = []
        for i in range(steps):
            sp.frame = frame0 + i
            reps.append(g.step(sp))
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, reps

    g = session(fia.FIA_FP32C, plume_state(n, args.ns_cfl))
    g.learned_set_weights(np.fromfile(weights, dtype="<f4"))
    sp = fia.step_params(cfl=args.ns_cfl, max_dt=MAX_DT,
                         solver={"tol": tol, "max_iter": 20000, "method": fia.FIA_SOLVER_FCG_LEARNED,
                                 "fallback_iter": 200})
    for f in range(args.ns_warmup):
        sp.frame = f
        g.step(sp)
    g.synchronize()
    start = tuple(g.get(c) for c in ("density", "u", "v", "w"))
    ms_chosen, reps = run(g, sp, args.ns_warmup, args.ns_steps)
    g.close()
    out = {"grid": n, "cfl": args.ns_cfl, "pressure_tol": tol,
           "chosen": {"steps_per_s": 1e3 / ms_chosen, "ms_per_step": ms_chosen, "steps": args.ns_steps,
                      "fcg_iterations": [r.solver_fcg_iterations for r in reps],
                      "pressure_iterations": [r.solver_iterations for r in reps],
                      "rel_residual": [r.solver_rel_residual for r in reps],
                      "fallback_steps": sum(1 for r in reps if r.status & fia.FIA_STATUS_SOLVER_FALLBACK)}}
    if args.ns_fp64_steps > 0:
        pcg = {"tol": tol, "max_iter": 20000}
        g = session(fia.FIA_FP32C, start)
        ms32, reps32 = run(g, fia.step_params(cfl=args.ns_cfl, max_dt=MAX_DT, solver=pcg), args.ns_warmup,
                           args.ns_fp64_steps)
        g.close()
        g = session(fia.FIA_FP64, start)
        ms64, reps64 = run(g, fia.step_params(cfl=args.ns_cfl, max_dt=MAX_DT, solver=pcg), args.ns_warmup,
                           args.ns_fp64_steps)
        g.close()
        out["fp32c_jacobi_pcg"] = {"steps_per_s": 1e3 / ms32, "ms_per_step": ms32, "steps": args.ns_fp64_steps,
                                   "pressure_iterations": [r.solver_iterations for r in reps32]}
        out["fp64_plain"] = {"steps_per_s": 1e3 / ms64, "ms_per_step": ms64, "steps": args.ns_fp64_steps,
                             "pressure_iterations": [r.solver_iterations for r in reps64],
                             "rel_residual": [r.solver_rel_residual for r in reps64]}
        out["speedup_chosen_vs_fp64_plain"] = ms64 / ms_chosen
        out["speedup_split"] = {"precision_and_advection_kernels (fp32c+pcg vs fp64+pcg)": ms64 / ms32,
                                "learned_preconditioner (chosen vs fp32c+pcg)": ms32 / ms_chosen}
    return out


def run_gpu(args, world, rank, local, dist):
    import torch
    import fia
    torch.cuda.set_device(local)
    n = args.grid
    state = c1_state(n)
    dt = state[4]
    params = fia.advect_params()
    g = c1_session(fia, n, fia.FIA_FP32C, state)
    stream = torch.cuda.ExternalStream(g.stream())
    flush = torch.zeros(256 * 2 ** 20 // 4, dtype=torch.float32, device="cuda")
    sampler = ClockSampler(local)
    sampler.start()
    for _ in range(args.warmup):
        g.move_substances_3D(dt, params)
    g.synchronize()
    c0 = g.pass_counters()
    g.profile_faces(64 * args.steps)
    barrier(dist)
    torch.cuda.synchronize()
    t_ms = timed_steps(g, stream, args.steps, dt, params, flush)
    barrier(dist)
    clocks = sampler.stop()
    face_ms, face_launches = g.read_face_profile()
    c1 = g.pass_counters()
    t_max = max_over_ranks(t_ms, dist)
    faces_step = unique_faces(n)
    value = world * faces_step * args.steps / (t_max / 1e3)

    # ---- end to end through the host-buffer C entry point, every step: density, u, v, w from
    #      pinned host memory, the step, density back
    e2e = None
    if args.e2e_steps > 0:
        host = {}
        for name in ("density", "u", "v", "w"):
            a = g.get(name).astype(np.float32)
            t = torch.empty(a.size, dtype=torch.float32, pin_memory=True)
            t.numpy()[:] = a
            host[name] = t
        lib = g.lib
        torch.cuda.synchronize()
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            fia._check(lib.fia_move_substances_3D_host(g.s, fia.FIA_HOST_F32, host["density"].data_ptr(),
                                                       host["u"].data_ptr(), host["v"].data_ptr(),
                                                       host["w"].data_ptr(), dt, ctypes.byref(params)), "e2e step")
        t1 = time.perf_counter()
        barrier(dist)
        te = max_over_ranks(t1 - t0, dist)
        h2d = sum(t.numel() * 4 for t in host.values())
        e2e = {"value": world * faces_step * args.e2e_steps / te, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": host["density"].numel() * 4, "steps": args.e2e_steps,
               "path": "fia_move_substances_3D_host (FP32 host buffers, pinned): density, u, v, w in, density out"}

    # ---- roofline of the dominant kernel (k_quad32: per-piece quadrature + WENO6)
    evals = c1[3] - c0[3]
    flops = evals * WENO1D_FLOP
    pieces = c1[1] - c0[1]
    faces_visited = c1[0] - c0[0]
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    peak_tf = SMS * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    achieved_tf = flops / (face_ms / 1e3) / 1e12 if face_ms > 0 else 0.0
    peaks = read_peaks()
    launches = max(face_launches, 1)
    # algorithmic bytes of one k_quad32 launch: per piece its record (16 B) and face tag (4 B)
    # read and its flux (4 B) written, plus the advected field (4 B per node) and psi (8 B per
    # node) read once
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
        "traffic": traffic_from_profile(),
        "hbm": {"achieved": alg_bytes / (face_ms / launches / 1e3) / 1e9 if face_ms > 0 else None,
                "peak": peaks.get("hbm_gbs"), "unit": "GB/s", "bytes_per_launch": alg_bytes},
    }
    stream_of = lambda s: torch.cuda.ExternalStream(s.stream())  # noqa: E731
    details = {"steps_per_s": args.steps / (t_ms / 1e3), "ms_per_step": t_ms / args.steps,
               "cells_per_s": n ** 3 * args.steps / (t_ms / 1e3),
               "pieces_per_face": pieces / max(faces_visited, 1), "weno6_1d_evaluations": evals,
               "face_kernel_ms": face_ms, "dt": dt}
    g.close()
    cpu = None
    if rank == 0 and world == 1:
        if args.fp64_steps > 0:
            details["fp64_plain_same_config"] = fp64_same_config(fia, args, state, flush, stream_of)
        if args.cpu_baseline:
            cpu = cpu_baseline_sample(args)
        if args.north_star:
            details["north_star_256"] = north_star(fia, args)
    line = {
        "metric": METRIC % n, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic", "config": config_of(args),
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": c1[4] - c0[4],
        "clocks": clocks, "details": details,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--fp64-steps", type=int, default=3, help="steps of the plain FP64 form at the same configuration")
    ap.add_argument("--ref-slab", type=int, default=16, help="x-planes per step of the CPU oracle")
    ap.add_argument("--cpu-baseline", action=argparse.BooleanOptionalAction, default=True,
                    help="time the streaming-tile CPU port on the whole step (cpu_baseline)")
    ap.add_argument("--north-star", action=argparse.BooleanOptionalAction, default=True,
                    help="also time the 256^3 smoke step of the target (chosen form against the plain FP64 form)")
    ap.add_argument("--ns-grid", type=int, default=256)
    ap.add_argument("--ns-cfl", type=float, default=2.0)
    ap.add_argument("--ns-warmup", type=int, default=3)
    ap.add_argument("--ns-steps", type=int, default=5)
    ap.add_argument("--ns-fp64-steps", type=int, default=3)
    ap.add_argument("--weights", default=os.path.join(PKG, "weights", "unet_precond.f32"),
                    help="learned preconditioner of the 256^3 target step")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, dist)
    else:
        run_gpu(args, world, rank, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
