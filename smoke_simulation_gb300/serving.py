"""Serving front end: the continuous-batching server of libsmoke_gb300 (smk_server_*) and the
seeded Poisson request stream used to exercise it.

The server keeps requests resident on the GPU, admits new ones between ticks as memory and
slots free up, and overlaps the steps of different requests (separate streams, or one grouped
step per tick); this module only binds it (ctypes) and drives it in real time from an arrival
schedule.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
import time
from typing import List, Optional

import numpy as np

from . import Params, _check, lib, params_for_scene
from . import scenes as S

REQ_QUEUED, REQ_ACTIVE, REQ_DONE, REQ_FAILED, REQ_CANCELLED = 0, 1, 2, 3, 4

_F = C.POINTER(C.c_float)


class RequestDesc(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("steps", C.c_int),
                ("dt", C.c_float), ("params", C.POINTER(Params)), ("mask", C.c_void_p),
                ("spheres", _F), ("n_spheres", C.c_int), ("boxes", _F), ("n_boxes", C.c_int),
                ("obstacles", _F), ("n_obstacles", C.c_int), ("out_density", C.c_void_p),
                ("out_on_device", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("steps_completed", C.c_longlong), ("requests_completed", C.c_int),
                ("active", C.c_int), ("queued", C.c_int), ("cell_updates", C.c_double),
                ("bytes_in_use", C.c_size_t), ("p50_step_ms", C.c_float),
                ("p99_step_ms", C.c_float), ("max_step_ms", C.c_float),
                ("p50_queue_ms", C.c_float), ("p99_queue_ms", C.c_float), ("max_queue_ms", C.c_float),
                ("peak_active", C.c_int), ("peak_queued", C.c_int), ("peak_bytes", C.c_size_t)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_bound = False


def _bind():
    global _bound
    if _bound:
        return lib()
    L = lib()
    vp, i = C.c_void_p, C.c_int
    for name, res, args in (
            ("smk_server_create", i, [C.c_size_t, i, C.POINTER(vp)]),
            ("smk_server_submit", i, [vp, C.POINTER(RequestDesc), C.POINTER(i)]),
            ("smk_server_tick", i, [vp, C.POINTER(i), C.POINTER(i)]),
            ("smk_server_request_status", i, [vp, i, C.POINTER(i), C.POINTER(i), C.POINTER(i)]),
            ("smk_server_get_stats", i, [vp, C.POINTER(ServerStats)]),
            ("smk_server_destroy", i, [vp]),
            ("smk_server_set_mode", i, [vp, i]),
            ("smk_server_cancel", i, [vp, i]),
            ("smk_server_set_graph_loops", i, [vp, i]),
            ("smk_server_set_blocked", i, [vp, i]),
            ("smk_server_last_error", C.c_char_p, [])):
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _bound = True
    return L


def _srv_check(rc: int):
    if rc != 0:
        from . import SmokeError
        raise SmokeError(rc, _bind().smk_server_last_error().decode())


SERVE_STREAMS, SERVE_GROUPED = 0, 1


class Server:
    """Resident simulations with continuous admission (see smk_server_tick).  mode: STREAMS
    (each request's own kernels on its own stream) or GROUPED (one grouped step per tick)."""

    def __init__(self, budget_bytes: int = 120 * 10**9, max_active: int = 64, mode: int = SERVE_STREAMS):
        L = _bind()
        self.h = C.c_void_p()
        _srv_check(L.smk_server_create(budget_bytes, max_active, C.byref(self.h)))
        if mode != SERVE_STREAMS:
            _srv_check(L.smk_server_set_mode(self.h, int(mode)))
        self._keep = {}
        self.outputs = {}

    def set_graph_loops(self, enable: bool):
        """Device-side group loops in the requests' step graphs (default off)."""
        _srv_check(_bind().smk_server_set_graph_loops(self.h, 1 if enable else 0))

    def set_blocked(self, zchunk: int):
        """GROUPED form: blocked solve with z-chunks of `zchunk` planes (default 137; 0: colour passes)."""
        _srv_check(_bind().smk_server_set_blocked(self.h, int(zchunk)))

    def submit(self, scene, steps: Optional[int] = None, params: Optional[Params] = None,
               keep_output: bool = True, out_device=None, **param_overrides) -> int:
        """Queue `scene` (a scenes.Scene) for `steps` steps; returns the request id.  The final
        density goes to a host array (self.outputs[id]) or, with `out_device` (a CUDA tensor
        of the cell shape, float32), to device memory by a stream-ordered copy."""
        p = params if params is not None else params_for_scene(scene, **param_overrides)
        keep = [p]
        d = RequestDesc()
        d.nx, d.ny, d.nz = scene.nx, scene.ny, scene.nz
        d.steps = int(scene.steps if steps is None else steps)
        d.dt = scene.dt
        d.params = C.pointer(p)
        if scene.mask is not None:
            m = np.ascontiguousarray(scene.mask, np.uint8)
            keep.append(m)
            d.mask = m.ctypes.data
        for attr, width, field in (("spheres", 4, "spheres"), ("boxes", 9, "boxes"),
                                   ("obstacles", 7, "obstacles")):
            rows = getattr(scene, attr)
            if rows:
                a = np.ascontiguousarray(np.array(rows, np.float32).reshape(len(rows), width))
                keep.append(a)
                setattr(d, field, a.ctypes.data_as(_F))
                setattr(d, "n_" + field, len(rows))
        out = None
        if out_device is not None:
            assert tuple(out_device.shape) == tuple(scene.cell_shape) and out_device.is_cuda
            keep.append(out_device)
            d.out_density = out_device.data_ptr()
            d.out_on_device = 1
        elif keep_output:
            out = np.zeros(scene.cell_shape, np.float32)
            keep.append(out)
            d.out_density = out.ctypes.data
        rid = C.c_int()
        _srv_check(_bind().smk_server_submit(self.h, C.byref(d), C.byref(rid)))
        self._keep[rid.value] = keep
        if out is not None:
            self.outputs[rid.value] = out
        return rid.value

    def cancel(self, rid: int):
        _srv_check(_bind().smk_server_cancel(self.h, int(rid)))

    def tick(self):
        a, q = C.c_int(), C.c_int()
        _srv_check(_bind().smk_server_tick(self.h, C.byref(a), C.byref(q)))
        return a.value, q.value

    def status(self, rid: int):
        st, done, err = C.c_int(), C.c_int(), C.c_int()
        _srv_check(_bind().smk_server_request_status(self.h, rid, C.byref(st), C.byref(done),
                                                     C.byref(err)))
        return st.value, done.value, err.value

    def stats(self) -> ServerStats:
        s = ServerStats()
        _srv_check(_bind().smk_server_get_stats(self.h, C.byref(s)))
        return s

    def run_until_idle(self, max_ticks: int = 10**7):
        for _ in range(max_ticks):
            a, q = self.tick()
            if a == 0 and q == 0:
                return
        raise RuntimeError("server did not drain")

    def close(self):
        if self.h:
            _bind().smk_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclasses.dataclass
class Arrival:
    t: float
    scene: S.Scene
    steps: int


def poisson_stream(count: int, rate: float = 200.0, seed: int = 4, lo: int = 48, hi: int = 192,
                   steps_lo: int = 50, steps_hi: int = 500) -> List[Arrival]:
    """The serving workload: Poisson arrivals (rate per second, seeded), cube side log-uniform
    in [lo, hi], step count uniform in [steps_lo, steps_hi], each with a seeded sphere solid and
    a box emitter, dt = 0.05."""
    rng = S.SplitMix64(seed, lane=6)
    gaps = -np.log1p(-rng.uniform(count)) / rate
    times = np.cumsum(gaps)
    sides = np.round(np.exp(rng.uniform(count, math.log(lo), math.log(hi)))).astype(int)
    steps = rng.integers(count, steps_lo, steps_hi + 1)
    out = []
    for i in range(count):
        n = int(sides[i])
        sc = S.Scene("req%03d_%d" % (i, n), n, n, n, dt=0.05, steps=int(steps[i]), scheme=1,
                     iterations=200, tol=1e-4, check_every=6, warm_start=1)
        r = max(2, n // 8)
        cx, cy, cz = (int(v) for v in rng.integers(3, r + 2, n - r - 2))
        sc.mask = S.sphere_mask(n, n, n, [(float(cx), float(cy), float(cz), float(r))],
                                S.reference_initial_mask(n, n, n))
        b = max(2, n // 8)
        ex = int(rng.integers(1, b + 1, n - b - 1)[0])
        ez = int(rng.integers(1, b + 1, n - b - 1)[0])
        sc.boxes = [(ex - b // 2, 1, ez - b // 2, ex - b // 2 + b, 1 + max(2, b // 2),
                     ez - b // 2 + b, 1.0, 0.0, 0.0)]
        out.append(Arrival(float(times[i]), sc, int(steps[i])))
    return out


def drive(server: Server, arrivals: List[Arrival], keep_output: bool = False, **overrides):
    """Submit each arrival when the wall clock reaches its time and tick until everything is
    done.  Returns (wall seconds, request ids)."""
    t0 = time.perf_counter()
    ids = []
    k = 0
    while True:
        now = time.perf_counter() - t0
        while k < len(arrivals) and arrivals[k].t <= now:
            a = arrivals[k]
            ids.append(server.submit(a.scene, a.steps, keep_output=keep_output, **overrides))
            k += 1
        active, queued = server.tick()
        if k == len(arrivals) and active == 0 and queued == 0:
            break
        if active == 0 and queued == 0 and k < len(arrivals):
            time.sleep(max(0.0, min(0.001, arrivals[k].t - now)))
    return time.perf_counter() - t0, ids
