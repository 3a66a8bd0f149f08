"""GPU reference baseline -- TEST INFRASTRUCTURE ONLY (a measurement of the reference).

Times the reference's own kernels (project/smokeSimulation.cu built for sm_103a by
oracle/build_oracle.py, "oracle A") on the 256^3 single-grid workload, stage by stage, next to
the library's stages on the same GPU, workload and initial state:

  reference: simulate()'s launches (smokeSimulation.cu:774-819) with CUDA events between the
             stage groups (oracle/ref_gpu_tail.inc), at the reference's own 30 red-black
             iterations per step (:797) and at the iteration count that a zero-pressure start
             needs for max|div u| <= 1e-4 on this workload (167, measured by the library's
             tolerance rule); plus simulate() itself end to end (blocking density read-back).
  library:   the PRESSURE-scheme step with per-stage CUDA events (direct launches), warm-started
             pressure, the solve stopped by the tolerance rule; mean over the workload's 50
             steps from its initial fields;
  drop-in:   the library's REFERENCE-scheme step (what the reference's own simulate() symbol
             runs, bit-exact with the reference) at the same iteration counts as the reference,
             per stage, and smk_simulate end to end.

Usage (on a machine with a GPU; the reference's generated source must be in oracle/_ref/):
    python -m oracle.time_reference_gpu [--side 256] [--steps 4] [--json OUT.json]
Prints one JSON object.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import build_oracle  # noqa: E402

_F = C.POINTER(C.c_float)
STAGES = ["objects", "forcing", "projection", "advection", "readback"]


def load_reference_gpu() -> C.CDLL:
    path = build_oracle.build_reference_gpu()
    if path is None:
        raise RuntimeError("oracle/_ref/ref_step_gpu.cu is absent (generated where the reference "
                           "checkout is present)")
    L = C.CDLL(path)
    L.refg_init.argtypes = [_F, C.c_uint, C.c_uint, C.c_uint, C.c_int]
    L.refg_set_iterations.argtypes = [C.c_int]
    L.refg_set_physics.argtypes = [C.c_float, C.c_float]
    L.refg_add_source.argtypes = [C.c_float] * 4
    L.refg_add_source.restype = C.c_int
    L.refg_add_obstacle.argtypes = [C.c_float] * 7
    L.refg_add_obstacle.restype = C.c_int
    L.refg_set_state.argtypes = [C.c_void_p] * 4
    L.refg_set_state.restype = C.c_int
    L.refg_simulate.argtypes = [_F, C.c_float]
    L.refg_simulate.restype = C.c_int
    L.refg_step_timed.argtypes = [_F, C.c_float, _F]
    L.refg_step_timed.restype = C.c_int
    return L


def time_reference(L, sc, iterations: int, steps: int, warmup: int) -> dict:
    """Stage times (ms, mean over `steps` steps after `warmup`) of the reference's GPU step."""
    rho = np.ascontiguousarray(sc.initial_density().astype(np.float32))
    L.refg_init(rho.ctypes.data_as(_F), sc.nx, sc.ny, sc.nz,
                max(3, len(sc.spheres), len(sc.obstacles)))
    L.refg_set_physics(sc.gravity, sc.buoyancy)
    L.refg_set_iterations(iterations)
    for (x, y, z, r) in sc.spheres:
        L.refg_add_source(x, y, z, r)
    for ob in sc.obstacles:
        L.refg_add_obstacle(*ob)
    mask = np.ascontiguousarray(sc.initial_mask().astype(np.uint8))
    vel = [None if getattr(sc, k + "0") is None else
           np.ascontiguousarray(getattr(sc, k + "0").astype(np.float32)) for k in "uvw"]
    rc = L.refg_set_state(mask.ctypes.data, *[None if a is None else a.ctypes.data for a in vel])
    if rc:
        raise RuntimeError("refg_set_state: CUDA error %d" % rc)
    out = np.zeros(sc.cell_shape, np.float32)
    ms = (C.c_float * 5)()
    rows = []
    for k in range(warmup + steps):
        rc = L.refg_step_timed(out.ctypes.data_as(_F), C.c_float(sc.dt), ms)
        if rc:
            raise RuntimeError("refg_step_timed: CUDA error %d" % rc)
        if k >= warmup:
            rows.append(list(ms))
    t = np.mean(np.array(rows), axis=0)
    # simulate() itself, end to end (host clock around the blocking call)
    t0 = time.perf_counter()
    for _ in range(steps):
        rc = L.refg_simulate(out.ctypes.data_as(_F), C.c_float(sc.dt))
        if rc:
            raise RuntimeError("refg_simulate: CUDA error %d" % rc)
    e2e = (time.perf_counter() - t0) / steps * 1e3
    L.refg_delete()
    res = {k: float(v) for k, v in zip(STAGES, t)}
    res["device_step_ms"] = float(sum(t[:4]))
    res["per_iteration_ms"] = float(t[2] / iterations) if iterations else None
    res["simulate_e2e_ms"] = e2e
    res["iterations"] = iterations
    res["density_finite"] = bool(np.isfinite(out).all())
    return res


def time_library(sc, warmup: int) -> dict:
    """Stage times (ms) of the library's step, mean over the workload's steps (sc.steps, from its
    initial fields, after `warmup` steps that are then undone by writing the fields back)."""
    import copy
    import torch
    import smoke_simulation_gb300 as smk
    sc = copy.copy(sc)
    sc.warm_start = 1  # the benchmark's headline form
    sim = smk.from_scene(sc, report_div=0)
    initial = sim.read_state()
    depth, zchunk, _ = sim.autotune()
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    sim.set_timing(True)
    for _ in range(warmup):
        sim.step(sc.dt, sh)
    sim.write_state(initial)
    rows, sweeps = [], []
    for _ in range(sc.steps):
        sim.step(sc.dt, sh)
        t = sim.stage_times()
        rows.append([float(x) for x in t[:6]])
        sweeps.append(sim.stats().sweeps)
    sim.set_timing(False)
    t = np.mean(np.array(rows), axis=0)
    return {"objects": float(t[0]), "forcing": float(t[1]), "projection": float(t[2]),
            "advection": float(t[3]), "device_step_ms": float(t[4]), "sweep_phase": float(t[5]),
            "mean_sweeps": float(np.mean(sweeps)),
            "per_sweep_ms": float(t[5] / np.mean(sweeps)) if np.mean(sweeps) else None,
            "sweep_kernel": [depth, zchunk],
            "note": "direct launches with per-stage events (the graph-replayed step is faster); "
                    "warm-started pressure, solve stopped by the tolerance rule"}


def time_library_dropin(sc, iterations: int, steps: int, warmup: int) -> dict:
    """Stage times (ms) of the library's drop-in path: the REFERENCE projection scheme (the
    reference's in-place velocity red-black SOR, bit-exact with it) at `iterations` fixed
    iterations from the workload's initial fields, direct launches with per-stage events; plus
    smk_simulate (the reference's simulate(): step and blocking density read-back) end to end."""
    import copy
    import torch
    import smoke_simulation_gb300 as smk
    sc = copy.copy(sc)
    sc.scheme, sc.iterations, sc.tol, sc.warm_start = 0, iterations, 0.0, 0
    sim = smk.from_scene(sc, report_div=0)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    sim.set_timing(True)
    rows = []
    for k in range(warmup + steps):
        sim.step(sc.dt, sh)
        if k >= warmup:
            rows.append([float(x) for x in sim.stage_times()[:5]])
    sim.set_timing(False)
    t = np.mean(np.array(rows), axis=0)
    out = torch.empty(sc.cell_shape, dtype=torch.float32, pin_memory=True).numpy()
    for _ in range(warmup):
        sim.simulate(out, sc.dt)
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.simulate(out, sc.dt)
    e2e = (time.perf_counter() - t0) / steps * 1e3
    sim.close()
    return {"objects": float(t[0]), "forcing": float(t[1]), "projection": float(t[2]),
            "advection": float(t[3]), "device_step_ms": float(t[4]),
            "per_iteration_ms": float(t[2] / iterations) if iterations else None,
            "simulate_e2e_ms": e2e, "iterations": iterations}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--side", type=int, default=256)
    ap.add_argument("--scene", default="large", choices=["large", "ref80"],
                    help="large: the single-large-grid workload at --side; ref80: the 80^3 "
                         "reference-step configuration (sphere obstacle, box emitter, noise)")
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--iterations", default="30,167")
    ap.add_argument("--json", default="")
    args = ap.parse_args()
    import torch
    torch.cuda.init()
    torch.zeros(1, device="cuda")
    from smoke_simulation_gb300 import scenes as S
    sc = S.config_large(args.side) if args.scene == "large" else S.config_ref80(steps=50)
    L = load_reference_gpu()
    ref = {}
    for it in (int(x) for x in args.iterations.split(",")):
        ref[str(it)] = time_reference(L, sc, it, args.steps, args.warmup)
    ours = time_library(sc, args.warmup) if args.scene == "large" else None
    dropin = {str(it): time_library_dropin(sc, it, args.steps, args.warmup)
              for it in (int(x) for x in args.iterations.split(","))}
    res = {"workload": sc.name, "cells": sc.cells, "gpu": torch.cuda.get_device_name(0),
           "reference_gpu": ref, "library": ours, "library_dropin": dropin}
    txt = json.dumps(res)
    print(txt)
    if args.json:
        with open(args.json, "w") as f:
            f.write(txt + "\n")


if __name__ == "__main__":
    main()
