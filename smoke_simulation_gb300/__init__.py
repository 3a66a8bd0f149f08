"""smoke_simulation_gb300 -- GB300-native semi-Lagrangian smoke step (Python front end).

The simulation runs in libsmoke_gb300.so (hand-written sm_103a CUDA kernels behind the C ABI
in include/smoke_gb300.h).  This module is a thin ctypes binding of that ABI for tests,
benchmarks and Python callers; it adds no compute of its own and has no CPU fallback: if the
library is missing, importing `lib()` raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsmoke_gb300.so")

SMK_OK = 0
PROJECT_REFERENCE = 0
PROJECT_PRESSURE = 1
SOLVER_RBSOR, SOLVER_JACOBI = 0, 1
SWEEP_YCLUSTER = 0x100  # smk_set_sweep_shape rows flag: y-column clusters exchanging boundary rows


def SWEEP_YCLUSTER_N(n: int) -> int:
    """rows field of a y-cluster shape with clusters of n (2 or 4) CTAs along y."""
    return n << 9
CLAMP_REFERENCE, CLAMP_MAGNITUDE, CLAMP_NONE = 0, 1, 2
STORAGE_F32, STORAGE_BF16, STORAGE_BF16_VEL = 0, 1, 2


ERR_INVALID, ERR_CUDA, ERR_OOM, ERR_STATE, ERR_TIMEOUT = 1, 2, 3, 4, 5


class SmokeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("smoke_gb300 error %d: %s" % (code, msg))
        self.code = code


class Params(C.Structure):
    _fields_ = [
        ("gravity", C.c_float), ("buoyancy", C.c_float), ("clamp_const", C.c_float),
        ("clamp_mode", C.c_int), ("projection", C.c_int), ("max_sweeps", C.c_int),
        ("omega", C.c_double), ("tol", C.c_float), ("check_every", C.c_int),
        ("warm_start", C.c_int), ("report_div", C.c_int), ("storage", C.c_int),
        ("refine", C.c_int), ("refine_sweeps", C.c_int), ("obstacle_velocity", C.c_int),
        ("solver", C.c_int), ("omega_warm", C.c_double), ("omega_warm_after", C.c_int),
        ("warm_extrapolate", C.c_float),
    ]


class Stats(C.Structure):
    _fields_ = [("sweeps", C.c_int), ("converged", C.c_int), ("resid_max", C.c_float),
                ("div_max", C.c_float), ("step_index", C.c_int), ("refine_rounds", C.c_int),
                ("div64_max", C.c_float), ("subtract_fused", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class HostState(C.Structure):
    _fields_ = [("rho", C.c_void_p * 2), ("u", C.c_void_p * 2), ("v", C.c_void_p * 2),
                ("w", C.c_void_p * 2), ("s", C.c_void_p), ("index_now", C.c_int)]


class RenderParams(C.Structure):
    """smk_render_params: the headless renderer's camera, light and buffers."""
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("light_res", C.c_int), ("planes", C.c_int),
                ("camera_pos", C.c_float * 3), ("camera_dir", C.c_float * 3), ("up", C.c_float * 3),
                ("fovy_deg", C.c_float), ("znear", C.c_float), ("zfar", C.c_float),
                ("light_pos", C.c_float * 3), ("light_fovy_deg", C.c_float), ("light_znear", C.c_float),
                ("light_zfar", C.c_float), ("light_color", C.c_float * 3), ("box_pos", C.c_float * 3),
                ("cell_size", C.c_float), ("bg_color", C.c_float * 3)]


_lib = None


def lib() -> C.CDLL:
    """Load the in-tree CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libsmoke_gb300.so is not built; run smoke_simulation_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    vp, i, f = C.c_void_p, C.c_int, C.c_float
    sig = {
        "smk_default_params": (None, [C.POINTER(Params)]),
        "smk_error_string": (C.c_char_p, [i]),
        "smk_last_error": (C.c_char_p, []),
        "smk_create": (i, [i, i, i, C.POINTER(Params), C.POINTER(vp)]),
        "smk_destroy": (i, [vp]),
        "smk_set_params": (i, [vp, C.POINTER(Params)]),
        "smk_get_params": (i, [vp, C.POINTER(Params)]),
        "smk_set_density": (i, [vp, vp]),
        "smk_set_solid_mask": (i, [vp, vp]),
        "smk_add_obstacle": (i, [vp, f, f, f, f, f, f, f, C.POINTER(i)]),
        "smk_add_smoke_source": (i, [vp, f, f, f, f, C.POINTER(i)]),
        "smk_add_box_emitter": (i, [vp, i, i, i, i, i, i, f, f, i, C.POINTER(i)]),
        "smk_update_object_pos": (i, [vp, i, f, f, f]),
        "smk_clear_objects": (i, [vp]),
        "smk_step": (i, [vp, f, vp]),
        "smk_simulate": (i, [vp, vp, f]),
        "smk_read_density": (i, [vp, vp, i, vp]),
        "smk_sync": (i, [vp, vp]),
        "smk_read_state": (i, [vp, C.POINTER(HostState)]),
        "smk_write_state": (i, [vp, C.POINTER(HostState)]),
        "smk_get_stats": (i, [vp, C.POINTER(Stats)]),
        "smk_set_timing": (i, [vp, i]),
        "smk_get_stage_times": (i, [vp, C.POINTER(C.c_float), i]),
        "smk_launch_count": (C.c_longlong, [vp]),
        "smk_set_sweep_kernel": (i, [vp, i, i]),
        "smk_get_sweep_kernel": (i, [vp, C.POINTER(i), C.POINTER(i)]),
        "smk_set_sweep_shape": (i, [vp, i, i, i]),
        "smk_set_velocity_sweep": (i, [vp, i, i]),
        "smk_get_velocity_sweep": (i, [vp, C.POINTER(i), C.POINTER(i)]),
        "smk_get_sweep_shape": (i, [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i)]),
        "smk_project_noalloc": (i, [vp, vp, vp, vp, i, i, i, C.POINTER(Params),
                                    C.POINTER(Stats), vp]),
        "smk_project_noalloc_max_elems": (C.c_longlong, []),
        "smk_autotune": (i, [vp, C.POINTER(i), C.POINTER(i), C.POINTER(f)]),
        "smk_set_graphs": (i, [vp, i]),
        "smk_set_graph_loops": (i, [vp, i]),
        "smk_set_vector_stages": (i, [vp, i]),
        "smk_set_fused_subtract": (i, [vp, i]),
        "smk_set_readback_slabs": (i, [vp, i]),
        "smk_get_readback_slabs": (i, [vp, C.POINTER(i)]),
        "smk_default_render_params": (None, [C.c_void_p]),
        "smk_render": (i, [vp, C.c_void_p, vp, vp, vp]),
        "smk_batch_create": (i, [i, C.POINTER(vp), C.POINTER(vp)]),
        "smk_batch_step": (i, [vp, C.POINTER(f), f, vp]),
        "smk_batch_destroy": (i, [vp]),
        "smk_batch_set_mode": (i, [vp, i]),
        "smk_batch_set_graphs": (i, [vp, i]),
        "smk_batch_get_info": (i, [vp, C.POINTER(i), C.POINTER(C.c_longlong)]),
        "smk_batch_autotune": (i, [vp, C.POINTER(i), C.POINTER(f)]),
        "smk_batch_get_schedule": (i, [vp, C.POINTER(i), C.POINTER(i), C.POINTER(C.c_longlong)]),
        "smk_batch_set_schedule": (i, [vp, i, i, C.c_longlong]),
        "smk_batch_set_blocked": (i, [vp, i]),
        "smk_batch_get_blocked": (i, [vp, C.POINTER(i)]),
        "smk_project_noalloc_last_error": (C.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(rc: int):
    if rc != SMK_OK:
        L = lib()
        raise SmokeError(rc, "%s: %s" % (L.smk_error_string(rc).decode(),
                                         L.smk_last_error().decode()))


def default_params(**kw) -> Params:
    p = Params()
    lib().smk_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


class Simulation:
    """One resident grid: the reference's implicit module state as an object."""

    def __init__(self, nx: int, ny: int, nz: int, params: Optional[Params] = None):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.h = C.c_void_p()
        _check(lib().smk_create(nx, ny, nz, C.byref(params) if params is not None else None,
                                C.byref(self.h)))

    # -- lifecycle ---------------------------------------------------------------------------
    def close(self):
        if self.h:
            lib().smk_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def cell_shape(self):
        return (self.nz, self.ny, self.nx)

    @property
    def face_shape(self):
        return (self.nz + 1, self.ny + 1, self.nx + 1)

    # -- configuration -----------------------------------------------------------------------
    def params(self) -> Params:
        p = Params()
        _check(lib().smk_get_params(self.h, C.byref(p)))
        return p

    def set_params(self, p: Params = None, **kw):
        p = p or self.params()
        for k, v in kw.items():
            setattr(p, k, v)
        _check(lib().smk_set_params(self.h, C.byref(p)))

    def set_density(self, rho: np.ndarray):
        a = np.ascontiguousarray(rho, np.float32)
        assert a.size == self.nx * self.ny * self.nz
        _check(lib().smk_set_density(self.h, _ptr(a)))

    def set_mask(self, s: np.ndarray):
        a = np.ascontiguousarray(s, np.uint8)
        assert a.size == self.nx * self.ny * self.nz
        _check(lib().smk_set_solid_mask(self.h, _ptr(a)))

    def add_obstacle(self, x, y, z, vx=0.0, vy=0.0, vz=0.0, r=1.0) -> int:
        i = C.c_int()
        _check(lib().smk_add_obstacle(self.h, x, y, z, vx, vy, vz, r, C.byref(i)))
        return i.value

    def add_smoke_source(self, x, y, z, r) -> int:
        i = C.c_int()
        _check(lib().smk_add_smoke_source(self.h, x, y, z, r, C.byref(i)))
        return i.value

    def add_box_emitter(self, x0, y0, z0, x1, y1, z1, density=1.0, vy=0.0, set_vy=False) -> int:
        i = C.c_int()
        _check(lib().smk_add_box_emitter(self.h, int(x0), int(y0), int(z0), int(x1), int(y1),
                                         int(z1), density, vy, int(bool(set_vy)), C.byref(i)))
        return i.value

    def update_object_pos(self, oid: int, x, y, z):
        _check(lib().smk_update_object_pos(self.h, oid, x, y, z))

    def clear_objects(self):
        _check(lib().smk_clear_objects(self.h))

    # -- stepping ----------------------------------------------------------------------------
    def step(self, dt: float, stream: int = 0):
        _check(lib().smk_step(self.h, dt, stream))

    def simulate(self, out: np.ndarray, dt: float):
        assert out.dtype == np.float32 and out.flags["C_CONTIGUOUS"]
        _check(lib().smk_simulate(self.h, _ptr(out), dt))
        return out

    def read_density(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        out = np.empty(self.cell_shape, np.float32) if out is None else out
        _check(lib().smk_read_density(self.h, _ptr(out), 0, None))
        _check(lib().smk_sync(self.h, None))
        return out

    def render(self, params: Optional["RenderParams"] = None, **overrides):
        """Render the current density with the headless half-angle slice renderer; returns
        (eye RGBA [height, width, 4], composite RGB [height, width, 3]) as numpy arrays, rows
        bottom-up."""
        import torch
        rp = params if params is not None else default_render_params()
        for k, v in overrides.items():
            setattr(rp, k, v)
        eye = torch.empty((rp.height, rp.width, 4), dtype=torch.float32, device="cuda")
        comp = torch.empty((rp.height, rp.width, 3), dtype=torch.float32, device="cuda")
        _check(lib().smk_render(self.h, C.byref(rp), eye.data_ptr(), comp.data_ptr(), None))
        _check(lib().smk_sync(self.h, None))
        return eye.cpu().numpy(), comp.cpu().numpy()

    def render_into(self, eye_ptr: int, comp_ptr: int, params: "RenderParams", stream: int = 0):
        """Stream-ordered smk_render into caller-owned device buffers (no synchronisation)."""
        _check(lib().smk_render(self.h, C.byref(params), eye_ptr, comp_ptr or None, stream))

    def read_density_device(self, dev_ptr: int, stream: int = 0):
        _check(lib().smk_read_density(self.h, dev_ptr, 1, stream))

    def sync(self, stream: int = 0):
        _check(lib().smk_sync(self.h, stream))

    def read_state(self) -> dict:
        cs, fs = self.cell_shape, self.face_shape
        st = {"rho": [np.zeros(cs, np.float32) for _ in range(2)],
              "u": [np.zeros(fs, np.float32) for _ in range(2)],
              "v": [np.zeros(fs, np.float32) for _ in range(2)],
              "w": [np.zeros(fs, np.float32) for _ in range(2)],
              "s": np.zeros(cs, np.uint8)}
        hs = HostState()
        for k in ("rho", "u", "v", "w"):
            arr = getattr(hs, k)
            for j in range(2):
                arr[j] = _ptr(st[k][j])
        hs.s = _ptr(st["s"])
        _check(lib().smk_read_state(self.h, C.byref(hs)))
        st["index_now"] = hs.index_now
        return st

    def write_state(self, st: dict):
        keep = []
        hs = HostState()
        for k in ("rho", "u", "v", "w"):
            arr = getattr(hs, k)
            for j in range(2):
                if st.get(k) is None or st[k][j] is None:
                    arr[j] = None
                    continue
                a = np.ascontiguousarray(st[k][j], np.float32)
                keep.append(a)
                arr[j] = _ptr(a)
        if st.get("s") is not None:
            s = np.ascontiguousarray(st["s"], np.uint8)
            keep.append(s)
            hs.s = _ptr(s)
        hs.index_now = int(st.get("index_now", 1))
        _check(lib().smk_write_state(self.h, C.byref(hs)))

    def stats(self) -> Stats:
        s = Stats()
        _check(lib().smk_get_stats(self.h, C.byref(s)))
        return s

    def set_timing(self, on: bool = True):
        _check(lib().smk_set_timing(self.h, int(on)))

    def stage_times(self) -> np.ndarray:
        t = (C.c_float * 6)()
        _check(lib().smk_get_stage_times(self.h, t, 6))
        return np.array(t[:], np.float64)

    def launch_count(self) -> int:
        return int(lib().smk_launch_count(self.h))

    def set_graph_loops(self, enable: bool):
        _check(lib().smk_set_graph_loops(self.h, 1 if enable else 0))

    def set_vector_stages(self, enable: bool):
        """Forcing, rhs and subtract / BF16 projection with four x per thread (default) or one
        cell per thread; results are identical."""
        _check(lib().smk_set_vector_stages(self.h, 1 if enable else 0))

    def set_fused_subtract(self, enable: bool):
        """PRESSURE, FP32, blocked sweeps: the gradient subtract inside the solve's last sweep
        launch (default off); results are identical."""
        _check(lib().smk_set_fused_subtract(self.h, 1 if enable else 0))

    def set_readback_slabs(self, slabs: int):
        """simulate() into page-locked memory: the advection in `slabs` z-slabs, each slab's
        density copied to the host while the next computes (-1, the default: one slab per
        16 MiB of density, 1 to 8; 0: the copy after the step); results are identical."""
        _check(lib().smk_set_readback_slabs(self.h, int(slabs)))

    def readback_slabs(self) -> int:
        """The slab count simulate() uses on this grid."""
        n = C.c_int(0)
        _check(lib().smk_get_readback_slabs(self.h, C.byref(n)))
        return n.value

    def set_sweep_kernel(self, depth: int, zchunk: int = 32, rows: int = 2):
        """Blocked sweep kernel shape: `depth` colour passes per launch, z-chunks of `zchunk`
        planes, patches of `rows` cell rows per thread (2, or 4 with depth 4), or with depth 6
        2 | SWEEP_YCLUSTER [| SWEEP_YCLUSTER_N(2 or 4)]: thread-block clusters along y."""
        _check(lib().smk_set_sweep_shape(self.h, depth, rows, zchunk))

    def set_velocity_sweep(self, depth: int, zchunk: int = 0):
        """REFERENCE-scheme projection kernel: depth 0 = one colour pass per launch, 2 or 4 =
        temporally blocked (depth passes per pass over HBM, z-chunks of zchunk planes, 0 = from
        the grid); results are identical."""
        _check(lib().smk_set_velocity_sweep(self.h, depth, zchunk))

    def velocity_sweep(self):
        d, z = C.c_int(), C.c_int()
        _check(lib().smk_get_velocity_sweep(self.h, C.byref(d), C.byref(z)))
        return d.value, z.value

    def autotune(self):
        """Pick the fastest sweep kernel shape for this grid; returns (depth, zchunk, us/sweep)."""
        d, z, t = C.c_int(), C.c_int(), C.c_float()
        _check(lib().smk_autotune(self.h, C.byref(d), C.byref(z), C.byref(t)))
        return d.value, z.value, t.value

    def set_graphs(self, on: bool = True):
        _check(lib().smk_set_graphs(self.h, int(on)))

    def sweep_kernel(self):
        d, z = C.c_int(), C.c_int()
        _check(lib().smk_get_sweep_kernel(self.h, C.byref(d), C.byref(z)))
        return d.value, z.value

    def sweep_shape(self):
        """(depth, patch rows, zchunk) of the blocked sweep kernel."""
        d, r, z = C.c_int(), C.c_int(), C.c_int()
        _check(lib().smk_get_sweep_shape(self.h, C.byref(d), C.byref(r), C.byref(z)))
        return d.value, r.value, z.value


BATCH_AUTO, BATCH_GROUPED, BATCH_BRANCHES = 0, 1, 2


class Batch:
    """Many independent grids of any sizes stepped together (smk_batch_*): GROUPED runs one
    persistent launch per stage over every member, BRANCHES one graph branch per member; AUTO
    takes GROUPED when every member uses the PRESSURE projection.  The batch does not own its
    members; keep the Simulation objects alive while the batch is in use."""

    def __init__(self, sims, mode: int = BATCH_AUTO):
        self.sims = list(sims)
        arr = (C.c_void_p * len(self.sims))(*[s.h.value for s in self.sims])
        self.h = C.c_void_p()
        _check(lib().smk_batch_create(len(self.sims), arr, C.byref(self.h)))
        if mode != BATCH_AUTO:
            self.set_mode(mode)

    def set_mode(self, mode: int):
        _check(lib().smk_batch_set_mode(self.h, int(mode)))

    def set_graphs(self, enable: bool):
        _check(lib().smk_batch_set_graphs(self.h, 1 if enable else 0))

    def info(self) -> tuple[int, int]:
        """(form of the last step: BATCH_GROUPED / BATCH_BRANCHES, kernels launched so far)."""
        m, n = C.c_int(), C.c_longlong()
        _check(lib().smk_batch_get_info(self.h, C.byref(m), C.byref(n)))
        return m.value, n.value

    def autotune(self) -> tuple[int, float]:
        """Tune the grouped projection's schedule; returns (ctas_per_sm, us_per_sweep)."""
        c, us = C.c_int(), C.c_float()
        _check(lib().smk_batch_autotune(self.h, C.byref(c), C.byref(us)))
        return c.value, us.value

    def schedule(self) -> tuple[int, int, int]:
        """(cooperative CTAs per SM (0 = all resident), z planes per tile, solve-wave bytes)."""
        c, z, w = C.c_int(), C.c_int(), C.c_longlong()
        _check(lib().smk_batch_get_schedule(self.h, C.byref(c), C.byref(z), C.byref(w)))
        return c.value, z.value, w.value

    def set_schedule(self, ctas_per_sm: int, zslab: int, wave_bytes: int):
        _check(lib().smk_batch_set_schedule(self.h, int(ctas_per_sm), int(zslab), int(wave_bytes)))

    def set_blocked(self, zchunk: int):
        """Blocked grouped solve with z-chunks of `zchunk` planes (0: cooperative colour passes)."""
        _check(lib().smk_batch_set_blocked(self.h, int(zchunk)))

    def blocked(self) -> int:
        z = C.c_int()
        _check(lib().smk_batch_get_blocked(self.h, C.byref(z)))
        return z.value

    def step(self, dt, stream: int = 0):
        """dt: one float for every member, or a sequence with one dt per member."""
        if isinstance(dt, (list, tuple, np.ndarray)):
            dts = (C.c_float * len(self.sims))(*[float(x) for x in dt])
            _check(lib().smk_batch_step(self.h, dts, 0.0, stream))
        else:
            _check(lib().smk_batch_step(self.h, None, float(dt), stream))

    def close(self):
        if self.h:
            lib().smk_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def proxy_planes(view_origin, view_dir, box_pos, dims, planes: int):
    """Proxy-plane polygons on the device (smk_proxy_planes): (vertices [planes, 7, 3], counts
    [planes], triangles [planes, 6, 3]) as numpy arrays."""
    import torch
    f3 = lambda v: (C.c_float * 3)(*[float(x) for x in v])
    verts = torch.zeros((planes, 7, 3), dtype=torch.float32, device="cuda")
    counts = torch.zeros(planes, dtype=torch.int32, device="cuda")
    tris = torch.zeros((planes, 6, 3), dtype=torch.int32, device="cuda")
    L = lib()
    L.smk_proxy_planes.argtypes = [C.c_void_p] * 4 + [C.c_int] + [C.c_void_p] * 4
    _check(L.smk_proxy_planes(f3(view_origin), f3(view_dir), f3(box_pos), f3(dims), planes, verts.data_ptr(),
                              counts.data_ptr(), tris.data_ptr(), None))
    torch.cuda.synchronize()
    return verts.cpu().numpy(), counts.cpu().numpy(), tris.cpu().numpy()


def default_render_params(**overrides) -> RenderParams:
    rp = RenderParams()
    lib().smk_default_render_params(C.byref(rp))
    for k, v in overrides.items():
        setattr(rp, k, v)
    return rp


def params_for_scene(scene, **overrides) -> Params:
    p = default_params()
    p.gravity, p.buoyancy = scene.gravity, scene.buoyancy
    p.clamp_const, p.clamp_mode = scene.clamp_const, scene.clamp_mode
    p.projection, p.max_sweeps, p.omega = scene.scheme, scene.iterations, scene.omega
    p.tol, p.check_every, p.warm_start = scene.tol, scene.check_every, scene.warm_start
    p.refine, p.refine_sweeps = scene.refine, scene.refine_sweeps
    p.obstacle_velocity = scene.obstacle_velocity
    p.solver = scene.solver
    p.omega_warm, p.omega_warm_after = scene.omega_warm, scene.omega_warm_after
    p.warm_extrapolate = scene.warm_extrapolate
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def from_scene(scene, **overrides) -> Simulation:
    """A Simulation holding `scene`'s initial state and objects (buffer [0] = initial fields,
    buffer [1] = 0, as after the reference's initializeVolume plus the scene's writes)."""
    sim = Simulation(scene.nx, scene.ny, scene.nz, params_for_scene(scene, **overrides))
    sim.set_density(scene.initial_density())
    if scene.mask is not None:
        sim.set_mask(scene.mask)
    if scene.u0 is not None or scene.v0 is not None or scene.w0 is not None:
        sim.write_state({"u": [scene.initial_velocity("u"), None],
                         "v": [scene.initial_velocity("v"), None],
                         "w": [scene.initial_velocity("w"), None], "index_now": 1})
    for bx in scene.boxes:
        sim.add_box_emitter(*bx[:6], density=bx[6], vy=bx[7], set_vy=bool(bx[8]))
    for (x, y, z, r) in scene.spheres:
        sim.add_smoke_source(x, y, z, r)
    for ob in scene.obstacles:
        sim.add_obstacle(*ob)
    return sim
