"""Benchmark: cell-updates/s of the smoke step on the 256^3 workload.

Workload (one "step" = one full simulation step of one 256^3 grid): FP32 fields, 5% Bernoulli
solids (seed 1) plus two r=24 spheres, four seeded sphere emitters, dt = 0.02, pressure-form
red-black SOR warm-started from the last pressure extrapolated along its last change, to
max|residual| <= 0.995e-4 (so that max|div u| <= 1e-4 after the face updates' rounding) checked
every 6 sweeps, capped at 200 sweeps, 50 steps.
Synthetic inputs from smoke_simulation_gb300.scenes (the reference publishes no dataset).  The
K timed steps are the 50-step workload run from its initial fields K/50 times (the fields are
written back between runs, outside the timed events), so every timed step is a step of the
configured workload rather than of an ever longer simulation.

  value   cell-updates/s with the state resident in HBM (CUDA events on the step stream)
  e2e     the same metric through smk_simulate (the reference's simulate(): step plus a
          blocking copy of the density into pinned host memory), host wall clock
  roofline  the sweep phase (red-black passes + residual checks), algorithmic bytes (each sweep
          reads P, b and the flag byte and writes P: 13 B per cell), over its event-timed
          duration in the timed steps
  cpu_baseline  the reference's own step built for the host (OpenMP, all cores) on a bounded
          sample of the same workload
  forms   the chosen forms beside the plain step: 64 uneven grids in the grouped batch form
          (FP32 and BF16 velocities), the 512^3 mixed-precision step, and the Poisson serving
          stream with p50/p99 step latency, each against the plain FP32 form (one grid at a
          time, pressure restarted from zero every step) on the same grids

Multi-GPU: the path does not shard (one grid per simulation); under torchrun every rank runs an
independent replica ("replicas only") and value is the sum over ranks with max-over-ranks time.

--impl reference times the reference's own CPU step (oracle/_ref; the restatement if the
reference build is absent) on the same workload and prints the same JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s"
UNIT = "cell-updates/s"
N_DEFAULT = 256
# Sweeps the reference step is given in the CPU baseline and the reference arm: the
# reference's projection has no convergence test, so it runs the sweep count that this
# workload's tolerance rule takes on the GPU from a zero pressure (mean over the workload's steps).
REF_SWEEPS_DEFAULT = 167
# Algorithmic bytes per cell: one red+black sweep reads P, b, flags and writes P.
SWEEP_BYTES_PER_CELL = 13.0
CHECK_BYTES_PER_CELL = 9.0


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.strip()]
        self.file.close()
        os.unlink(self.file.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for name, val in zip(names, r[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                   "reasons": sorted(reasons), "samples": len(sm)}
        return out


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return ws, rank, local


def dist_max(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def dist_barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def workload(n: int, warm_start: int = 1):
    """The 256^3 workload.  The headline solve warm-starts the pressure from the previous step
    and over-relaxes the warm-started solves with 1.75 from the third step on (same red-black
    SOR, same tolerance rule, so the same max|div| <= 1e-4 guarantee; scenes.large_workload)."""
    from smoke_simulation_gb300 import scenes as S
    return S.large_workload(n=n, steps=50, warm_start=warm_start)


def cpu_reference_rate(n: int, sweeps: int, steps: int, threads: int = 0):
    """Time the reference's own step (host build) or, without it, the restatement, on the
    workload at `n`^3 with `sweeps` fixed iterations.  Returns (rate, kind, cores, seconds)."""
    from oracle import oracle as O
    sc = workload(n)
    sc.scheme = 0
    sc.iterations = sweeps
    sc.tol = 0.0
    cores = threads or os.cpu_count() or 1
    if O.reference_available():
        sim = O.RefHostSim(sc, threads=cores)
        kind = "reference"
        cores = sim.lib.ref_max_threads()
    else:
        sim = O.OracleSim(sc)
        kind = "port"
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.step()
    dt = time.perf_counter() - t0
    if kind == "reference":
        sim.close()
    return sc.cells * steps / dt, kind, cores, dt


def max_div_reference(u, v, w, s) -> float:
    """max |div u| over the cells the reference's projection updates (interior, fluid, at least
    one fluid neighbour; project/smokeSimulation.cu:356-394), on face arrays (z, y, x) of shape
    (nz+1, ny+1, nx+1) and a cell mask (nz, ny, nx)."""
    s = np.asarray(s) != 0
    nz, ny, nx = s.shape
    div = ((u[:nz, :ny, 1:nx + 1].astype(np.float64) - u[:nz, :ny, :nx])
           + (v[:nz, 1:ny + 1, :nx].astype(np.float64) - v[:nz, :ny, :nx])
           + (w[1:nz + 1, :ny, :nx].astype(np.float64) - w[:nz, :ny, :nx]))
    inner = np.zeros_like(s)
    inner[1:-1, 1:-1, 1:-1] = True
    nb = np.zeros(s.shape, np.int32)
    nb[:, :, 1:] += s[:, :, :-1]
    nb[:, :, :-1] += s[:, :, 1:]
    nb[:, 1:, :] += s[:, :-1, :]
    nb[:, :-1, :] += s[:, 1:, :]
    nb[1:, :, :] += s[:-1, :, :]
    nb[:-1, :, :] += s[1:, :, :]
    proj = inner & s & (nb > 0)
    return float(np.abs(div[proj]).max()) if proj.any() else 0.0


def run_reference_arm(args, ws, rank):
    """The reference's own step (host build, OpenMP over every host core) on the same workload,
    timing exactly --steps steps after --warmup untimed ones, like the library's arm.  The
    reference's projection has no convergence test: it runs --ref-sweeps fixed red-black
    iterations (the sweeps a zero-pressure start needs for max|div| <= 1e-4 on this workload),
    and the line reports the max|div u| its projected velocity reaches."""
    if rank != 0:
        return 0
    steps = max(1, args.steps)
    warm = max(0, args.warmup)
    from oracle import oracle as O
    sc = workload(args.side)
    sc.scheme, sc.iterations, sc.tol = 0, args.ref_sweeps, 0.0
    cores = os.cpu_count() or 1
    if O.reference_available():
        sim = O.RefHostSim(sc, threads=cores)
        kind = "reference"
        cores = sim.lib.ref_max_threads()
    else:
        sim = O.OracleSim(sc)
        kind = "port"
    for _ in range(warm):
        sim.step()
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.step()
    dt = time.perf_counter() - t0
    rate = sc.cells * steps / dt
    if kind == "reference":
        st = sim.state()
        now = st["index_now"]
        div = max_div_reference(st["u"][now], st["v"][now], st["w"][now], st["s"])
        sim.close()
    else:
        now = sim.index_now
        div = max_div_reference(sim.u[now], sim.v[now], sim.w[now], sim.s)
    sample = ("%d timed step(s) after %d warm-up step(s) of the %d^3 workload, reference step with "
              "%d fixed red-black iterations, OpenMP over %d threads" % (steps, warm, args.side,
                                                                        args.ref_sweeps, cores))
    line = {
        "metric": METRIC, "value": rate, "unit": UNIT, "impl": "reference", "n_gpus": ws,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * dt / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "smoke step %d^3 FP32, 5%% random solids + 2 spheres r=24, 4 "
                               "emitters, dt=0.02, red-black SOR %d sweeps" % (args.side, args.ref_sweeps),
                   "cells": sc.cells, "l2": "inputs larger than L2 (CPU run)",
                   "ref_sweeps": args.ref_sweeps,
                   "max_div_post_projection": div,
                   "pressure_start": "zero every step (the reference's projection)"},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--side", type=int, default=N_DEFAULT, help="grid cells per side of the workload")
    ap.add_argument("--ref-sweeps", type=int, default=REF_SWEEPS_DEFAULT)
    ap.add_argument("--cpu-steps", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=0, help="0: same as --steps")
    ap.add_argument("--cold-steps", type=int, default=50,
                    help="timed steps of the zero-pressure-start form (0: skip)")
    ap.add_argument("--forms-steps", type=int, default=10, help="timed steps of the batched/mixed forms")
    ap.add_argument("--mixed-n", type=int, default=512, help="mixed-precision grid side (0: skip)")
    ap.add_argument("--mixed-steps", type=int, default=20, help="steps of the mixed-precision form")
    ap.add_argument("--serve-requests", type=int, default=200, help="serving stream length (0: skip)")
    ap.add_argument("--serve-tight-requests", type=int, default=60,
                    help="requests of the serving run under a binding memory budget (0: skip)")
    ap.add_argument("--serve-tight-gb", type=float, default=1.5, help="that run's device-memory budget (GB)")
    ap.add_argument("--render-frames", type=int, default=20, help="timed frames of the render form (0: skip)")
    ap.add_argument("--dropin-steps", type=int, default=20, help="timed steps of the drop-in form (0: skip)")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched/mixed/serving forms")
    ap.add_argument("--sweep-kernel", default="", help="D,Z[,R]: blocked sweep depth, z-chunk and patch "
                    "rows instead of the autotuner's choice (to profile the configuration a timed run chose)")
    ap.add_argument("--batch-schedule", default="", help="C,Z,W: grouped projection schedule instead of "
                    "the autotuner's choice")
    args = ap.parse_args()
    assert args.warmup >= 0 and args.steps >= 1

    ws, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference_arm(args, ws, rank)

    import torch
    import smoke_simulation_gb300 as smk
    from smoke_simulation_gb300 import build
    if not os.path.exists(smk.LIB_PATH):
        build.build()
    torch.cuda.set_device(local)

    sc = workload(args.side)
    # the timed steps run with the library defaults (no divergence diagnostic); the statistics
    # pass below re-runs the same steps with max|div u| measured after every projection
    sim = smk.from_scene(sc, report_div=0)
    initial = sim.read_state()  # the workload's initial fields; every timed segment starts here
    seg = sc.steps              # the workload is sc.steps (50) steps long
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    if args.sweep_kernel:
        parts = [int(x) for x in args.sweep_kernel.split(",")]
        depth, zchunk = parts[0], parts[1]
        sim.set_sweep_kernel(depth, zchunk, rows=parts[2] if len(parts) > 2 else 2)
        tuned_us = None
    else:
        depth, zchunk, tuned_us = sim.autotune()
    rows = sim.sweep_shape()[1]
    if rows & smk.SWEEP_YCLUSTER:
        ncl = (rows >> 9) & 0xF
        kname = "k_sweep_tb_ycl<%d> (%s)" % (depth, "clusters of %d" % ncl if ncl else "one cluster spanning y")
    else:
        kname = "k_sweep_tb<%d, %d>" % (depth, rows)

    # warm-up steps (graph capture, caches); the timed segments restart from the initial state
    for _ in range(max(args.warmup, 0)):
        sim.step(sc.dt, sh)
    torch.cuda.synchronize()

    def segments(total):
        """Lengths of the timed segments: the workload's steps from its initial state, repeated."""
        out = []
        while total > 0:
            out.append(min(seg, total))
            total -= out[-1]
        return out

    # ---- device-timed region: K steps (segments of the 50-step workload), state in HBM --------
    # before each segment the initial fields are written back (outside the timed events; this
    # also restarts the pressure history, as a new simulation has none)
    launches = 0
    elapsed = 0.0
    # clocks are sampled from here until the last timed region of the plain workload (the
    # device-timed steps, the e2e steps and the zero-pressure-start steps) has ended
    clocks = ClockSampler(local)
    clocks.start()
    t_clk0 = time.perf_counter()
    for n in segments(args.steps):
        sim.write_state(initial)
        launches0 = sim.launch_count()
        dist_barrier(ws)
        torch.cuda.synchronize()
        elapsed += _timed_steps(lambda: sim.step(sc.dt, sh), stream, n, torch)
        launches += sim.launch_count() - launches0
    dist_barrier(ws)

    # per-step statistics and stage times: one more pass over the workload's steps with a sync
    # after each (outside the timed region) to read the solver status and the sweep phase timed
    # by CUDA events on the step stream (these steps launch directly, not as a graph)
    sweeps, divs, conv, sweep_ms = [], [], [], []
    sim.write_state(initial)
    sim.set_params(report_div=1)
    sim.set_timing(True)
    for _ in range(seg):
        sim.step(sc.dt, sh)
        st = sim.stats()
        t = sim.stage_times()
        sweeps.append(st.sweeps)
        divs.append(st.div_max)
        conv.append(st.converged)
        sweep_ms.append(float(t[5]))
    sim.set_timing(False)
    sim.set_params(report_div=0)
    elapsed_max = dist_max(elapsed, ws)
    cells_all = dist_sum(float(sc.cells * args.steps), ws)
    value = cells_all / elapsed_max

    # ---- roofline of the dominant kernel (the blocked sweep, per launch) ---------------------
    # algorithmic bytes per launch = cells x 13 B x (depth/2 sweeps); the launch duration is the
    # event-timed sweep phase of the measured steps divided by the launches that ran in it
    # (the residual check is fused into the first launch of each group: no extra bytes).  A
    # solve that the tolerance rule ends also ran the check launch whose passes it dropped (the
    # solve ends on that launch's input): one launch more than its sweeps count
    peak, peak_kind = load_peaks()
    mean_sweeps = float(np.mean(sweeps))
    sweeps_per_launch = depth / 2.0 if depth > 0 else 0.5
    launches_run = mean_sweeps / sweeps_per_launch + (float(np.mean(conv)) if depth > 0 and sc.tol > 0 else 0.0)
    bytes_per_launch = sc.cells * SWEEP_BYTES_PER_CELL * sweeps_per_launch
    launch_seconds = float(np.mean(sweep_ms)) / 1e3 / launches_run
    achieved = bytes_per_launch / launch_seconds / 1e9 if launch_seconds > 0 else None
    # beside it: the launches without check code, timed in the step on a fixed-sweep solve of
    # the same workload (tolerance rule off, 6 full launches), the sweep phase over 6
    full_launch_seconds = None
    if depth > 0:
        n_fix = 6
        sim.set_params(tol=0.0, max_sweeps=int(n_fix * sweeps_per_launch))
        sim.set_timing(True)
        fix_ms = []
        for _ in range(5):
            sim.step(sc.dt, sh)
            fix_ms.append(float(sim.stage_times()[5]))
        sim.set_timing(False)
        sim.set_params(tol=sc.tol, max_sweeps=sc.iterations)
        full_launch_seconds = float(np.median(fix_ms[1:])) / 1e3 / n_fix
    traffic = None
    tf = os.path.join(ROOT, "profiles", "sweep_traffic.json")
    if os.path.exists(tf) and depth > 0:
        with open(tf) as f:
            tr = json.load(f)
        if tr.get("kernel") == kname and tr.get("zchunk") == zchunk:
            traffic = tr["bytes_per_cell_per_sweep"] * sweeps_per_launch * sc.cells

    # ---- e2e through the public API with host buffers ----------------------------------------
    e2e_steps = args.e2e_steps or args.steps
    out = torch.empty(sc.cell_shape, dtype=torch.float32, pin_memory=True).numpy()

    def e2e_run(slabs):
        # smk_simulate with the density copied out in `slabs` slabs during the advection (0: the
        # copy after the step); warm-up calls capture the graph for this output buffer, and the
        # timed segments restart from the initial state
        sim.set_readback_slabs(slabs)
        for _ in range(max(args.warmup, 1)):
            sim.simulate(out, sc.dt)
        dt_sum = 0.0
        for n in segments(e2e_steps):
            sim.write_state(initial)
            dist_barrier(ws)
            t0 = time.perf_counter()
            for _ in range(n):
                # the step's input: the emitter positions (launch parameters); result: the density
                sim.simulate(out, sc.dt)
            dt_sum += time.perf_counter() - t0
        return dist_sum(float(sc.cells * e2e_steps), ws) / dist_max(dt_sum, ws)

    e2e_copy_after = e2e_run(0)
    e2e_value = e2e_run(-1)  # the default: the slab count chosen from the grid size
    readback_slabs = sim.readback_slabs()

    # ---- the same solve from a zero pressure every step (the reference's iteration) ---------
    cold = None
    if args.cold_steps > 0:
        sim.set_params(warm_start=0)
        cold_s = 0.0
        for n in segments(args.cold_steps):
            sim.write_state(initial)
            cold_s += _timed_steps(lambda: sim.step(sc.dt, sh), stream, n, torch)
        sim.write_state(initial)
        cold_sweeps, cold_conv = [], []
        for _ in range(min(seg, args.cold_steps)):
            sim.step(sc.dt, sh)
            st = sim.stats()
            cold_sweeps.append(st.sweeps)
            cold_conv.append(st.converged)
        cold = {"value": dist_sum(float(sc.cells * args.cold_steps), ws) / dist_max(cold_s, ws),
                "ms_per_step": 1e3 * cold_s / args.cold_steps,
                "mean_sweeps": float(np.mean(cold_sweeps)), "converged_frac": float(np.mean(cold_conv)),
                "steps": args.cold_steps,
                "note": "pressure restarted from zero every step, as the reference's projection "
                        "does; same tolerance rule; the first steps of the workload"}
    # ---- the same warm-started solve with omega 1.9 throughout (no over-relaxation schedule) --
    fixed = None
    if args.cold_steps > 0 and sc.warm_start and getattr(sc, "omega_warm", 0.0) > 0.0:
        sim.set_params(warm_start=1, omega_warm=0.0)
        fixed_s = 0.0
        for n in segments(args.cold_steps):
            sim.write_state(initial)
            fixed_s += _timed_steps(lambda: sim.step(sc.dt, sh), stream, n, torch)
        sim.write_state(initial)
        fixed_sweeps, fixed_conv = [], []
        for _ in range(min(seg, args.cold_steps)):
            sim.step(sc.dt, sh)
            st = sim.stats()
            fixed_sweeps.append(st.sweeps)
            fixed_conv.append(st.converged)
        sim.set_params(omega_warm=sc.omega_warm)
        fixed = {"value": dist_sum(float(sc.cells * args.cold_steps), ws) / dist_max(fixed_s, ws),
                 "ms_per_step": 1e3 * fixed_s / args.cold_steps,
                 "mean_sweeps": float(np.mean(fixed_sweeps)), "converged_frac": float(np.mean(fixed_conv)),
                 "steps": args.cold_steps,
                 "note": "warm-started pressure, over-relaxation 1.9 in every step (the reference's "
                         "constant); same tolerance rule"}
    # ---- the same warm-started solve from the last pressure (no extrapolated start) ---------
    noext = None
    if args.cold_steps > 0 and sc.warm_start and getattr(sc, "warm_extrapolate", 0.0) > 0.0:
        sim.set_params(warm_start=1, warm_extrapolate=0.0)
        noext_s = 0.0
        for n in segments(args.cold_steps):
            sim.write_state(initial)
            noext_s += _timed_steps(lambda: sim.step(sc.dt, sh), stream, n, torch)
        sim.write_state(initial)
        noext_sweeps = []
        for _ in range(min(seg, args.cold_steps)):
            sim.step(sc.dt, sh)
            noext_sweeps.append(sim.stats().sweeps)
        sim.set_params(warm_extrapolate=sc.warm_extrapolate)
        noext = {"value": dist_sum(float(sc.cells * args.cold_steps), ws) / dist_max(noext_s, ws),
                 "ms_per_step": 1e3 * noext_s / args.cold_steps,
                 "mean_sweeps": float(np.mean(noext_sweeps)), "steps": args.cold_steps,
                 "note": "warm-started from the last pressure (smk_params.warm_extrapolate 0), the "
                         "over-relaxation schedule kept; same tolerance rule"}
    clk = clocks.stop()
    clk["window_s"] = time.perf_counter() - t_clk0
    clk["window"] = "device-timed, e2e and zero-pressure-start steps of the plain workload"

    # ---- CPU baseline (rank 0, N=1 only) -------------------------------------------------------
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        # the reference step has no tolerance test and no stored pressure: it needs the sweeps
        # a zero-pressure start takes to reach the tolerance (the cold form's count)
        ref_sweeps = int(round(cold["mean_sweeps"])) if cold else REF_SWEEPS_DEFAULT
        rate, kind, cores, secs = cpu_reference_rate(args.side, ref_sweeps, args.cpu_steps)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": kind,
               "sample": "%d step(s) of the %d^3 workload with %d fixed red-black iterations "
                         "(the sweeps a zero-pressure start needs for max|div| <= 1e-4, measured "
                         "on the GPU in this run), %.1f s" % (args.cpu_steps, args.side, ref_sweeps,
                                                             secs)}

    # errors of this workload's fields against the FP64 oracle, as measured by the headline parity
    # test (tests/test_gpu_headline.py: the GPU fields are bit-exact with the FP32 oracle there)
    err_keys = {}
    ef = os.path.join(ROOT, "profiles", "err_vs_fp64.json")
    if os.path.exists(ef) and args.side == 256:
        with open(ef) as f:
            worst = json.load(f)["large256"]["worst_vs_fp64"]
        err_keys = {"err_rho_max_abs_vs_fp64": worst["rho"]["max_abs"],
                    "err_rho_rel_l2_vs_fp64": worst["rho"]["rel_l2"],
                    "err_vel_max_abs_vs_fp64": max(worst[k]["max_abs"] for k in "uvw"),
                    "err_vel_rel_l2_vs_fp64": max(worst[k]["rel_l2"] for k in "uvw"),
                    "err_source": "tests/test_gpu_headline.py, first 5 steps, bit-exact with the FP32 oracle"}

    forms = None
    if rank == 0 and ws == 1 and not args.no_forms:
        sim.close()
        sim = None
        forms = run_forms(args, smk, torch)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed_max / args.steps,
            "sim_steps_per_s": args.steps / elapsed_max,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "smoke step %d^3 FP32, 5%% random solids + 2 spheres r=24, 4 "
                                   "emitters, dt=0.02, warm-started pressure red-black SOR to "
                                   "max|div|<=1e-4 (residual rule at 0.995e-4, "
                                   "checked every 6 sweeps, cap 200)" % args.side,
                       "cells": sc.cells, "parallelism": "replicas" if ws > 1 else "single",
                       "timed_steps": "%d steps: the %d-step workload from its initial fields, "
                                      "%d time(s) (fields written back between segments, outside "
                                      "the timed events)" % (args.steps, seg, len(segments(args.steps))),
                       "l2": "inputs larger than L2 (%.0f MB resident state)" % (
                           sim_bytes(sc) / 1e6),
                       "mean_sweeps": mean_sweeps, "converged_frac": float(np.mean(conv)),
                       "sweep_kernel": {"depth": depth, "rows": rows, "zchunk": zchunk, "tuned_us_per_sweep": tuned_us},
                       "max_div_post_projection": float(np.max(divs)),
                       "max_div_measured": "after every projection of the workload's steps, in a "
                                           "separate pass (the timed steps run without the diagnostic)",
                       "pressure_start": "warm: the previous step's pressure, extrapolated along its last "
                                         "change by %.2f once two solves exist (smk_params."
                                         "warm_extrapolate); over-relaxation 1.9 in the first 2 steps of "
                                         "the history, 1.75 after (smk_params.omega_warm)"
                                         % getattr(sc, "warm_extrapolate", 0.0),
                       # the same workload with the pressure restarted from zero every step (the
                       # reference's projection): the like-for-like comparison with the
                       # reference arm; value / cold_value is what warm starting contributes
                       "cold_value": cold["value"] if cold else None,
                       "cold_ms_per_step": cold["ms_per_step"] if cold else None,
                       "cold_mean_sweeps": cold["mean_sweeps"] if cold else None,
                       "warm_start_gain": (value / cold["value"]) if cold else None,
                       # the same warm-started workload with 1.9 throughout: value / omega_fixed_value
                       # is what the over-relaxation schedule contributes
                       "omega_fixed_value": fixed["value"] if fixed else None,
                       "omega_fixed_mean_sweeps": fixed["mean_sweeps"] if fixed else None,
                       "omega_schedule_gain": (value / fixed["value"]) if fixed else None,
                       # the same workload started from the last pressure: value / that is what
                       # the extrapolated start contributes
                       "no_extrapolation_value": noext["value"] if noext else None,
                       "no_extrapolation_mean_sweeps": noext["mean_sweeps"] if noext else None,
                       "extrapolation_gain": (value / noext["value"]) if noext else None,
                       **err_keys,
                       "cold_start_form": cold,
                       "omega_fixed_form": fixed,
                       "no_extrapolation_form": noext},
            "roofline": {"bound": "hbm", "kernel": "%s (z-chunk %d)" % (kname, zchunk),
                         "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                         "peak_kind": peak_kind, "bytes_per_launch": bytes_per_launch,
                         "launch_us": launch_seconds * 1e6,
                         "no_check_launch_us": full_launch_seconds * 1e6 if full_launch_seconds else None,
                         "no_check_frac": (bytes_per_launch / full_launch_seconds / 1e9 / peak)
                                          if full_launch_seconds else None,
                         "note": "achieved = algorithmic bytes per launch / mean launch duration over "
                                 "the launches of the tolerance-ruled solve (check launches and the "
                                 "dropped one included); no_check_*: the launches without check code, "
                                 "timed on a fixed-sweep solve of the same step; temporal blocking "
                                 "applies depth/2 sweeps per HBM pass, so achieved can exceed the "
                                 "single-pass roofline"},
            "clocks": clk,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 16 * len(sc.spheres),
                    "d2h_bytes_per_step": 4 * sc.cells,
                    "api": "smk_simulate (pinned host out; the density copied in %d z-slabs while the "
                           "advection computes)" % readback_slabs,
                    "copy_after_step_value": e2e_copy_after},
            "gpu_launches": int(launches),
            "cpu_baseline": cpu,
            "forms": forms,
        }
        print(json.dumps(line))
    if sim is not None:
        sim.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def _timed_steps(step, stream, steps, torch):
    """CUDA-event time (s) of `steps` calls of step() on `stream`."""
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3


def _rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run_forms(args, smk, torch):
    """The chosen forms next to the plain one (rank 0, one GPU): a batch of 64 uneven grids in the
    grouped form, the 512^3 mixed-precision step, and the Poisson serving stream.  "Plain" is
    the FP32 step of one grid at a time with the pressure restarted from zero every step (the
    reference's projection), on the same grids; every form solves to max|div u| <= 1e-4."""
    from smoke_simulation_gb300 import scenes as S
    from smoke_simulation_gb300 import serving as SV
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    forms = {}

    # ---- batched: 64 grids, side log-uniform 32..128 (seed 2) --------------------------------
    scs = S.config_batched(count=64, steps=args.forms_steps)
    for sc in scs:
        sc.tol, sc.check_every, sc.iterations, sc.warm_start = 1e-4, 6, 200, 1
        # warm-started solves over-relaxed with 1.75 from the third step and started from the
        # extrapolated pressure, as in the headline
        sc.omega_warm, sc.omega_warm_after = 1.75, 2
        sc.warm_extrapolate = 0.5
    cells = float(sum(sc.cells for sc in scs))
    batched = {}
    dens = {}
    for name, storage in (("f32", smk.STORAGE_F32), ("bf16", smk.STORAGE_BF16_VEL)):
        sims = [smk.from_scene(sc, report_div=1, storage=storage) for sc in scs]
        b = smk.Batch(sims, mode=smk.BATCH_GROUPED)
        b.step(scs[0].dt, sh)
        torch.cuda.synchronize()
        if args.batch_schedule:
            b.set_schedule(*(int(x) for x in args.batch_schedule.split(",")))
            sched_us = None
        else:
            sched_us = b.autotune()[1]
        for _ in range(args.warmup):
            b.step(scs[0].dt, sh)
        _, l0 = b.info()
        secs = _timed_steps(lambda: b.step(scs[0].dt, sh), stream, args.forms_steps, torch)
        _, l1 = b.info()
        st = [s.stats() for s in sims]
        batched[name] = {"value": cells * args.forms_steps / secs, "ms_per_step": 1e3 * secs / args.forms_steps,
                         "mean_sweeps": float(np.mean([x.sweeps for x in st])),
                         "max_div_post_projection": float(max(x.div_max for x in st)),
                         "launches_per_step": (l1 - l0) / args.forms_steps,
                         "schedule": {"ctas_per_sm_zslab_wavebytes": b.schedule(),
                                      "blocked_zchunk": b.blocked(),
                                      "tuned_us_per_sweep": sched_us}}
        dens[name] = [s.read_density() for s in sims]
        b.close()
        for s in sims:
            s.close()
    batched["bf16"]["density_rel_l2_vs_f32_max"] = max(_rel_l2(a, r) for a, r in zip(dens["bf16"], dens["f32"]))
    # plain: the same grids one at a time, FP32, pressure from zero each step
    sims = [smk.from_scene(sc, warm_start=0) for sc in scs]
    for s in sims:
        s.autotune()
    for _ in range(args.warmup):
        for s, sc in zip(sims, scs):
            s.step(sc.dt, sh)
    secs = _timed_steps(lambda: [s.step(sc.dt, sh) for s, sc in zip(sims, scs)], stream, args.forms_steps, torch)
    plain = {"value": cells * args.forms_steps / secs, "ms_per_step": 1e3 * secs / args.forms_steps,
             "mean_sweeps": float(np.mean([s.stats().sweeps for s in sims]))}
    for s in sims:
        s.close()
    # plain_warm: the same grids one at a time, FP32, with the warm-started pressure the grouped
    # form also uses: the ratio against it is what batching itself contributes
    sims = [smk.from_scene(sc, warm_start=1) for sc in scs]
    for s in sims:
        s.autotune()
    for _ in range(args.warmup):
        for s, sc in zip(sims, scs):
            s.step(sc.dt, sh)
    secs = _timed_steps(lambda: [s.step(sc.dt, sh) for s, sc in zip(sims, scs)], stream, args.forms_steps, torch)
    plain_warm = {"value": cells * args.forms_steps / secs, "ms_per_step": 1e3 * secs / args.forms_steps,
                  "mean_sweeps": float(np.mean([s.stats().sweeps for s in sims]))}
    for s in sims:
        s.close()
    forms["batched"] = {"workload": "64 grids, cube side log-uniform 32..128 (seed 2), sphere solid + box "
                                    "emitter each, dt=0.05, warm-started pressure (extrapolated by 0.5, "
                                    "over-relaxation 1.9, 1.75 from the third step) to max|div|<=1e-4; "
                                    "one persistent launch per stage over all grids (grouped form; the "
                                    "solve as cooperative colour passes or blocked launches over every "
                                    "grid's tiles, whichever the autotuner finds faster), CUDA-graph "
                                    "replay",
                        "cells": cells, "steps": args.forms_steps, "grouped": batched, "plain": plain,
                        "plain_warm": plain_warm,
                        "grouped_bf16_vs_plain": batched["bf16"]["value"] / plain["value"],
                        "grouped_f32_vs_plain": batched["f32"]["value"] / plain["value"],
                        "grouped_bf16_vs_plain_warm": batched["bf16"]["value"] / plain_warm["value"],
                        "grouped_f32_vs_plain_warm": batched["f32"]["value"] / plain_warm["value"]}

    # ---- the drop-in path: the reference's simulate() on the REFERENCE scheme -----------------
    if args.dropin_steps > 0:
        dropin = {}
        for name, sc, iters in (("256", S.config_large(256, steps=args.dropin_steps), 30),
                                ("80", S.config_ref80(steps=args.dropin_steps), 40)):
            # the reference's projection: in-place velocity red-black SOR, fixed iterations (30 is
            # the reference's own count, 40 the 80^3 configuration's); bit-exact with the reference
            sc.scheme, sc.iterations, sc.tol, sc.warm_start = 0, iters, 0.0, 0
            sim = smk.from_scene(sc)
            kernel = sim.autotune()[:2]
            out = torch.empty(sc.cell_shape, dtype=torch.float32, pin_memory=True).numpy()
            for _ in range(max(args.warmup, 2)):
                sim.simulate(out, sc.dt)
            t0 = time.perf_counter()
            for _ in range(args.dropin_steps):
                sim.simulate(out, sc.dt)
            e2e_s = (time.perf_counter() - t0) / args.dropin_steps
            dev_s = _timed_steps(lambda: sim.step(sc.dt, sh), stream, args.dropin_steps, torch) / args.dropin_steps
            dropin[name] = {"iterations": iters, "velocity_sweep": list(kernel),
                            "device_ms_per_step": 1e3 * dev_s, "simulate_ms_per_step": 1e3 * e2e_s,
                            "value": sc.cells / dev_s, "simulate_value": sc.cells / e2e_s}
            sim.close()
        forms["dropin"] = {"workload": "smk_simulate / simulate() on the REFERENCE scheme (the reference's "
                                       "in-place velocity SOR, bit-exact with the reference): the 256^3 workload "
                                       "at the reference's 30 iterations and the 80^3 configuration at 40; "
                                       "velocity-sweep kernel from the autotuner (depth, z-chunk); the "
                                       "reference's own kernels on the same GPU: oracle/time_reference_gpu.py, "
                                       "profiles/reference_gpu_step_large256.md",
                           **dropin}

    # ---- mixed precision at 512^3 -------------------------------------------------------------
    if args.mixed_n > 0:
        sc = S.config_mixed(args.mixed_n, steps=args.mixed_steps)
        sc.warm_start = 1
        msteps = max(2, args.mixed_steps)
        mixed = {}
        rho = {}
        for name, storage, extra in (("f32", smk.STORAGE_F32, {}), ("bf16_vel", smk.STORAGE_BF16_VEL, {}),
                                     ("bf16_all", smk.STORAGE_BF16, {}),
                                     # the configuration as specified: FP32 weighted Jacobi (weight 1)
                                     ("bf16_all_jacobi", smk.STORAGE_BF16,
                                      {"solver": smk.SOLVER_JACOBI, "omega": 1.0})):
            # FP32 pressure solve with the FP64-checked refinement (2 rounds of 10 sweeps at most)
            # the SOR forms over-relax warm-started solves with 1.75 from the third step, as the
            # headline workload does; the Jacobi form keeps its weight
            # (started from the last pressure: the extrapolated start helps the FP32 form, 10.21
            # against 10.08 G, and costs the BF16 forms, 9.84 / 9.90 against 10.03 / 10.09 G)
            kw = dict(report_div=1, storage=storage, refine=2, refine_sweeps=10,
                      omega_warm=0.0 if extra else 1.75, omega_warm_after=2, **extra)
            sim = smk.from_scene(sc, **kw)
            sim.autotune()
            sim.step(sc.dt, sh)  # mask upload step (direct launches)
            secs = _timed_steps(lambda: sim.step(sc.dt, sh), stream, msteps - 1, torch)
            st = sim.stats()
            mixed[name] = {"value": float(sc.cells) * (msteps - 1) / secs,
                           "ms_per_step": 1e3 * secs / (msteps - 1), "sweeps_last": st.sweeps,
                           "converged_last": st.converged,
                           "max_div_post_projection": st.div_max, "max_div_fp64": st.div64_max,
                           "refine_rounds_last": st.refine_rounds}
            rho[name] = sim.read_density()
            sim.close()
            if not extra:
                # the same steps again, untimed, for their sweep counts (the runs are deterministic)
                sim = smk.from_scene(sc, **kw)
                sim.autotune()
                sweeps = []
                for _ in range(msteps):
                    sim.step(sc.dt, sh)
                    sweeps.append(sim.stats().sweeps)
                sim.close()
                mixed[name]["mean_sweeps"] = float(np.mean(sweeps[1:]))
        for name in ("bf16_vel", "bf16_all", "bf16_all_jacobi"):
            mixed[name]["density_rel_l2_vs_f32"] = _rel_l2(rho[name], rho["f32"])
        forms["mixed"] = {"workload": "%d^3, 2%% random solids (seed 3), one 32x8x32 emitter, dt=0.02, "
                                      "warm-started FP32 pressure red-black SOR (from the last pressure, "
                                      "over-relaxation 1.9, 1.75 from the third step) to max|div|<=1e-4 "
                                      "(checked every "
                                      "6 sweeps), then max|div| measured with FP64 accumulation and "
                                      "corrected by up to 2 refinement rounds while above 1e-4, %d steps (the "
                                      "first, a mask upload, untimed); bf16_vel = u,v,w in BF16 + density FP32, bf16_all = "
                                      "density too; bf16_all_jacobi = all-BF16 with the FP32 weighted-Jacobi solve (weight 1) "
                                      "and the same refinement; mean_sweeps over the timed steps; errors vs the FP64 "
                                      "oracle: tests/test_gpu_headline.py (512^3, 2 steps)"
                                      % (args.mixed_n, msteps),
                          "cells": float(sc.cells), **mixed}

    # ---- headless rendering: the reference application's frame ---------------------------------
    if args.render_frames > 0:
        sc = S.config_ref80(steps=50, scheme=1)
        sc.tol, sc.check_every, sc.iterations, sc.warm_start = 1e-4, 6, 200, 1
        sim = smk.from_scene(sc)
        sim.autotune()
        for _ in range(sc.steps):
            sim.step(sc.dt, sh)
        rp = smk.default_render_params()
        eye = torch.empty((rp.height, rp.width, 4), dtype=torch.float32, device="cuda")
        comp = torch.empty((rp.height, rp.width, 3), dtype=torch.float32, device="cuda")
        frame = lambda: sim.render_into(eye.data_ptr(), comp.data_ptr(), rp, sh)
        for _ in range(3):
            frame()
        f_s = _timed_steps(frame, stream, args.render_frames, torch)
        both = lambda: (sim.step(sc.dt, sh), frame())
        for _ in range(3):
            both()
        b_s = _timed_steps(both, stream, args.render_frames, torch)
        forms["render"] = {"workload": "the reference application's frame: 80^3 scene after 50 steps, "
                                       "%dx%d eye buffer, %d^2 light buffer, %d half-angle planes, "
                                       "RGBA16F buffers (smk_render, 2 kernels per frame); the reference's "
                                       "OpenGL path and its 110 fps (RTX 3070) are unavailable on this box"
                                       % (rp.width, rp.height, rp.light_res, rp.planes),
                           "ms_per_frame": 1e3 * f_s / args.render_frames,
                           "frames_per_s": args.render_frames / f_s,
                           "step_plus_frame_per_s": args.render_frames / b_s,
                           "covered_pixels": float((eye[..., 3] > 0.01).float().mean().item())}
        sim.close()

    # ---- serving: Poisson stream, continuous admission ----------------------------------------
    if args.serve_requests > 0:
        arr = SV.poisson_stream(args.serve_requests)

        def serve_run(arrivals, budget, slots, mode=SV.SERVE_STREAMS, **kw):
            srv = SV.Server(budget_bytes=budget, max_active=slots, mode=mode)
            wall, _ = SV.drive(srv, arrivals, **kw)
            st = srv.stats()
            srv.close()
            return {"value": st.cell_updates / wall, "wall_s": wall, "requests": st.requests_completed,
                    "steps": st.steps_completed, "p50_step_ms": st.p50_step_ms, "p99_step_ms": st.p99_step_ms,
                    "max_step_ms": st.max_step_ms, "p50_queue_ms": st.p50_queue_ms,
                    "p99_queue_ms": st.p99_queue_ms, "max_queue_ms": st.max_queue_ms,
                    "peak_active": st.peak_active, "peak_queued": st.peak_queued,
                    "peak_gb": st.peak_bytes / 1e9, "budget_gb": budget / 1e9}

        # warm-started solves over-relaxed with 1.75 from each request's third step and started
        # from the extrapolated pressure
        ow = dict(omega_warm=1.75, omega_warm_after=2, warm_extrapolate=0.5)
        serve = serve_run(arr, 120 * 10**9, 64, storage=smk.STORAGE_BF16_VEL, **ow)
        # the same kind of stream under a budget that binds: admission waits on device memory
        tight = serve_run(arr[:args.serve_tight_requests], int(args.serve_tight_gb * 1e9), 64,
                          storage=smk.STORAGE_BF16_VEL, **ow) if args.serve_tight_requests > 0 else None
        # the grouped form (one persistent launch per stage over every active request; the solve
        # blocked, its default) on the first requests of the stream
        grouped = streams_head = None
        if args.serve_tight_requests > 0:
            head = arr[:args.serve_tight_requests]
            grouped = serve_run(head, 120 * 10**9, 64, mode=SV.SERVE_GROUPED, storage=smk.STORAGE_BF16_VEL, **ow)
            streams_head = serve_run(head, 120 * 10**9, 64, storage=smk.STORAGE_BF16_VEL, **ow)
        # one request at a time in plain FP32, on every 12th request of the stream (a sample that
        # spans its sizes and step counts): pressure from zero each step, and warm-started
        sample = arr[::12]
        plain1 = serve_run(sample, 120 * 10**9, 1, warm_start=0)
        plain_warm1 = serve_run(sample, 120 * 10**9, 1, **ow)
        forms["serving"] = {"workload": "%d requests, Poisson 200/s (seed 4), cube side log-uniform 48..192, "
                                        "50..500 steps, sphere solid + box emitter, tol 1e-4; served with "
                                        "u,v,w in BF16 (density FP32), warm-started pressure (extrapolated by "
                                        "0.5, over-relaxation 1.75 from a request's third step), up to 64 "
                                        "resident (120 GB budget), each request's step on its own stream; "
                                        "tight = the first %d requests under a %.1f GB budget; grouped = "
                                        "the same requests in the grouped form (one launch per stage over "
                                        "every active request, blocked solve), streams_head = those requests "
                                        "in the default form; plain = every "
                                        "12th request of the stream one at a time, FP32, pressure from zero "
                                        "each step (plain_warm: warm-started); cell-updates/s over host wall "
                                        "time; queue = submission to admission"
                                        % (args.serve_requests, args.serve_tight_requests, args.serve_tight_gb),
                            "served": serve, "served_tight_budget": tight, "served_grouped": grouped,
                            "served_streams_head": streams_head,
                            "grouped_vs_streams": grouped["value"] / streams_head["value"] if grouped else None,
                            "plain_one_at_a_time": plain1, "plain_warm_one_at_a_time": plain_warm1,
                            "served_vs_plain": serve["value"] / plain1["value"],
                            "served_vs_plain_warm": serve["value"] / plain_warm1["value"]}
    return forms


def sim_bytes(sc) -> float:
    X = (sc.nx + 1 + 15) // 16 * 16
    elems = X * (sc.ny + 1) * (sc.nz + 1)
    return elems * (10 * 4 + 2)


if __name__ == "__main__":
    sys.exit(main())
