"""ctypes front end of the oracles -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs may import
this module, and only as the checker.  The product (smoke_simulation_gb300 and its CUDA
library) never imports it.

Two oracles, both in the reference's memory layout:
  OracleSim   -- the restatement (smoke_oracle.cpp), float32 or float64, velocity or pressure
                 projection scheme.
  RefHostSim  -- the reference's own smokeSimulation.cu built for the host (oracle/_ref),
                 driven through its own public functions.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import build_oracle

_F = C.POINTER(C.c_float)


class OrcParams(C.Structure):
    _fields_ = [
        ("gravity", C.c_float), ("buoyancy", C.c_float), ("clamp_const", C.c_float),
        ("clamp_mode", C.c_int), ("scheme", C.c_int), ("iterations", C.c_int),
        ("omega", C.c_double), ("tol", C.c_float), ("check_every", C.c_int),
        ("warm_start", C.c_int),
        ("spheres", _F), ("n_spheres", C.c_int),
        ("boxes", _F), ("n_boxes", C.c_int),
        ("obstacles", _F), ("n_obstacles", C.c_int),
        ("refine", C.c_int), ("refine_sweeps", C.c_int), ("obstacle_velocity", C.c_int),
        ("solver", C.c_int),
    ]


class OrcState(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("rho", C.c_void_p * 2), ("u", C.c_void_p * 2), ("v", C.c_void_p * 2),
        ("w", C.c_void_p * 2), ("s", C.POINTER(C.c_uint8)), ("P", C.c_void_p),
        ("b", C.c_void_p), ("index_now", C.c_int),
    ]


class OrcStats(C.Structure):
    _fields_ = [("sweeps", C.c_int), ("converged", C.c_int), ("resid_max", C.c_float),
                ("div_max", C.c_float), ("refine_rounds", C.c_int), ("div64_max", C.c_float)]


_lib = None
_ref = None


def restatement() -> C.CDLL:
    global _lib
    if _lib is None:
        path = build_oracle.build_restatement()
        _lib = C.CDLL(path)
        for name in ("orc_f32_step", "orc_f64_step"):
            getattr(_lib, name).restype = C.c_int
            getattr(_lib, name).argtypes = [C.POINTER(OrcState), C.POINTER(OrcParams), C.c_float,
                                            C.POINTER(OrcStats)]
        _lib.orc_f32_max_div.restype = C.c_float
        _lib.orc_f64_max_div.restype = C.c_float
    return _lib


def reference_available() -> bool:
    try:
        return reference() is not None
    except Exception:
        return False


def reference() -> Optional[C.CDLL]:
    global _ref
    if _ref is None:
        path = build_oracle.build_reference()
        if path is None or not os.path.exists(path):
            return None
        _ref = C.CDLL(path)
        _ref.ref_add_obstacle.restype = C.c_int
        _ref.ref_add_obstacle.argtypes = [C.c_float] * 7
        _ref.ref_add_source.restype = C.c_int
        _ref.ref_add_source.argtypes = [C.c_float] * 4
        _ref.ref_update_pos.argtypes = [C.c_int, C.c_float, C.c_float, C.c_float]
        _ref.ref_set_solver.argtypes = [C.c_int, C.c_double, C.c_float]
        _ref.ref_set_physics.argtypes = [C.c_float, C.c_float]
        _ref.ref_init.argtypes = [_F, C.c_uint, C.c_uint, C.c_uint]
        _ref.ref_simulate.argtypes = [_F, C.c_float]
        _ref.ref_fill_box.argtypes = [C.c_int] * 6 + [C.c_float]
        _ref.ref_max_threads.restype = C.c_int
    return _ref


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(_F)


def _objects(rows, width):
    if not rows:
        return np.zeros((1, width), np.float32), 0
    return np.ascontiguousarray(np.array(rows, np.float32).reshape(len(rows), width)), len(rows)


class OracleSim:
    """The restatement, holding the reference's two ping-pong buffers per field."""

    def __init__(self, scene, dtype=np.float32, scheme: Optional[int] = None):
        self.sc = scene
        self.dtype = np.dtype(dtype)
        self.scheme = scene.scheme if scheme is None else scheme
        cs, fs = scene.cell_shape, scene.face_shape
        self.rho = [scene.initial_density().astype(self.dtype).copy(), np.zeros(cs, self.dtype)]
        self.u = [scene.initial_velocity("u").astype(self.dtype).copy(), np.zeros(fs, self.dtype)]
        self.v = [scene.initial_velocity("v").astype(self.dtype).copy(), np.zeros(fs, self.dtype)]
        self.w = [scene.initial_velocity("w").astype(self.dtype).copy(), np.zeros(fs, self.dtype)]
        self.s = np.ascontiguousarray(scene.initial_mask().astype(np.uint8).copy())
        self.P = np.zeros(cs, self.dtype)
        self.b = np.zeros(cs, self.dtype)
        self.index_now = 1
        self.spheres, self.n_spheres = _objects(scene.spheres, 4)
        self.boxes, self.n_boxes = _objects(scene.boxes, 9)
        self.obstacles, self.n_obstacles = _objects(scene.obstacles, 7)
        self.last = OrcStats()
        self.hist = 0  # steps since the pressure history started (the library's omega_warm rule)
        self.nsteps = 0
        # smk_params.warm_extrapolate: the last pressure as saved by the previous step's rhs pass
        self.Ph = None
        self.ph_step = -2

    def _state(self) -> OrcState:
        st = OrcState()
        st.nx, st.ny, st.nz = self.sc.nx, self.sc.ny, self.sc.nz
        for i in range(2):
            st.rho[i] = self.rho[i].ctypes.data
            st.u[i] = self.u[i].ctypes.data
            st.v[i] = self.v[i].ctypes.data
            st.w[i] = self.w[i].ctypes.data
        st.s = self.s.ctypes.data_as(C.POINTER(C.c_uint8))
        st.P = self.P.ctypes.data
        st.b = self.b.ctypes.data
        st.index_now = self.index_now
        return st

    def _params(self) -> OrcParams:
        sc = self.sc
        p = OrcParams()
        p.gravity, p.buoyancy, p.clamp_const = sc.gravity, sc.buoyancy, sc.clamp_const
        p.clamp_mode, p.scheme, p.iterations = sc.clamp_mode, self.scheme, sc.iterations
        p.omega, p.tol, p.check_every, p.warm_start = sc.omega, sc.tol, sc.check_every, sc.warm_start
        # smk_params.omega_warm: warm-started pressure solves from step omega_warm_after on
        ow, after = getattr(sc, "omega_warm", 0.0), getattr(sc, "omega_warm_after", 2)
        if self.scheme == 1 and sc.warm_start and ow > 0.0 and self.hist >= after:
            p.omega = ow
        p.spheres, p.n_spheres = _fptr(self.spheres), self.n_spheres
        p.boxes, p.n_boxes = _fptr(self.boxes), self.n_boxes
        p.obstacles, p.n_obstacles = _fptr(self.obstacles), self.n_obstacles
        p.refine, p.refine_sweeps = getattr(sc, "refine", 0), getattr(sc, "refine_sweeps", 10)
        p.obstacle_velocity = getattr(sc, "obstacle_velocity", 0)
        p.solver = getattr(sc, "solver", 0)
        return p

    def _warm_extrapolate(self):
        """The library's extrapolated warm start (body_rhs with a pressure history,
        csrc/stage_bodies.cuh): the last pressure Pl is saved for the next step, and once two
        solves of the history exist and the previous step saved its Pl, the solve starts from
        Pl + a * (Pl - Ph) in the field's precision (a = the float factor; the restatement's rhs
        then zeroes the cells that are not projectable, as the library's does)."""
        sc = self.sc
        ea = float(np.float32(getattr(sc, "warm_extrapolate", 0.0)))
        if not (self.scheme == 1 and sc.warm_start and ea > 0.0):
            return
        pl = self.P.copy()
        if self.hist >= 2 and self.Ph is not None and self.ph_step == self.nsteps - 1:
            a = self.dtype.type(ea)
            self.P[...] = pl + a * (pl - self.Ph)
        self.Ph = pl
        self.ph_step = self.nsteps

    def step(self, dt: Optional[float] = None) -> OrcStats:
        lib = restatement()
        self._warm_extrapolate()
        st = self._state()
        p = self._params()
        out = OrcStats()
        fn = lib.orc_f32_step if self.dtype == np.float32 else lib.orc_f64_step
        fn(C.byref(st), C.byref(p), C.c_float(self.sc.dt if dt is None else dt), C.byref(out))
        self.index_now = st.index_now
        self.last = out
        self.hist += 1
        self.nsteps += 1
        return out

    def reset_history(self):
        """The pressure history starts over (as smk_write_state does): P = 0, omega again."""
        self.P[...] = 0
        self.hist = 0

    def run(self, steps: Optional[int] = None):
        for _ in range(self.sc.steps if steps is None else steps):
            self.step()
        return self

    def update_sphere(self, i: int, x: float, y: float, z: float):
        self.spheres[i, :3] = (x, y, z)

    @property
    def past(self) -> int:
        return self.index_now ^ 1

    def density(self) -> np.ndarray:
        """What simulate() returns: the density buffer written by the last step."""
        return self.rho[self.past]


def render(rho: np.ndarray, params) -> tuple:
    """The renderer restatement (render_oracle.cpp) on a density array [nz, ny, nx]; params: an
    smk_render_params-layout structure.  Returns (eye RGBA, composite RGB), rows bottom-up."""
    lib = restatement()
    r = np.ascontiguousarray(rho, np.float32)
    nz, ny, nx = r.shape
    eye = np.zeros((params.height, params.width, 4), np.float32)
    comp = np.zeros((params.height, params.width, 3), np.float32)
    fn = lib.orc_render
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    fn(r.ctypes.data, nx, ny, nz, C.addressof(params), eye.ctypes.data, comp.ctypes.data)
    return eye, comp


def proxy_planes(view_origin, view_dir, box_pos, dims, planes: int):
    """The proxy-plane restatement: (vertices [planes, 7, 3], counts [planes], triangles
    [planes, 6, 3])."""
    lib = restatement()
    f3 = lambda v: np.ascontiguousarray(v, np.float32)
    vo, vd, bp, dm = f3(view_origin), f3(view_dir), f3(box_pos), f3(dims)
    verts = np.zeros((planes, 7, 3), np.float32)
    counts = np.zeros(planes, np.int32)
    tris = np.zeros((planes, 6, 3), np.int32)
    lib.orc_proxy_planes.argtypes = [C.c_void_p] * 4 + [C.c_int] + [C.c_void_p] * 3
    lib.orc_proxy_planes(vo.ctypes.data, vd.ctypes.data, bp.ctypes.data, dm.ctypes.data, planes,
                         verts.ctypes.data, counts.ctypes.data, tris.ctypes.data)
    return verts, counts, tris


_refp = None


def reference_proxy_available() -> bool:
    global _refp
    if _refp is None:
        path = build_oracle.build_reference_proxy()
        if path is None or not os.path.exists(path):
            return False
        _refp = C.CDLL(path)
        _refp.refp_proxy.restype = C.c_int
        _refp.refp_proxy.argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                                          C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                                          C.c_void_p]
    return True


def reference_proxy_planes(view_origin, view_dir, box_pos, dims, planes: int):
    """The reference's own BoundingBox::generateProxyGeometry (project/boundingBox.cpp:133-181,
    built for the host by oracle/build_oracle.py step 4), converted to smk_proxy_planes' layout:
    (vertices [planes, 7, 3], counts [planes], triangles [planes, 6, 3] as indices into the
    [planes * 7] vertex array, -1 rows unused)."""
    if not reference_proxy_available():
        raise RuntimeError("reference proxy-geometry build unavailable (needs the reference checkout)")
    f3 = lambda v: np.ascontiguousarray(v, np.float32)
    vo, vd, bp, dm = f3(view_origin), f3(view_dir), f3(box_pos), f3(dims)
    maxv, maxi = 7 * planes, 18 * planes
    flat_v = np.zeros((maxv, 3), np.float32)
    flat_i = np.zeros(maxi, np.int16)
    nv, ni = C.c_int(), C.c_int()
    pts = np.zeros(planes, np.int32)
    toff = np.zeros(planes, np.int32)
    rc = _refp.refp_proxy(vo.ctypes.data, vd.ctypes.data, bp.ctypes.data, dm.ctypes.data, planes,
                          flat_v.ctypes.data, maxv, C.byref(nv), flat_i.ctypes.data, maxi, C.byref(ni),
                          pts.ctypes.data, toff.ctypes.data)
    if rc != 0:
        raise RuntimeError("refp_proxy: output too small")
    verts = np.zeros((planes, 7, 3), np.float32)
    tris = np.full((planes, 6, 3), -1, np.int32)
    voff = 0
    for i in range(planes):
        k = int(pts[i])
        verts[i, :k + 1] = flat_v[voff:voff + k + 1]
        t = flat_i[3 * toff[i]:3 * (toff[i] + k)].reshape(k, 3).astype(np.int32)
        tris[i, :k] = t - voff + 7 * i
        voff += k + 1
    return verts, pts.copy(), tris


def round_half(x: np.ndarray) -> np.ndarray:
    """The restatement's float -> binary16 -> float rounding (round to nearest even)."""
    lib = restatement()
    a = np.ascontiguousarray(x, np.float32)
    out = np.empty_like(a)
    lib.orc_round_half.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    lib.orc_round_half(a.ctypes.data, out.ctypes.data, a.size)
    return out


class RefHostSim:
    """The reference's own step (host build), driven through its public API."""

    def __init__(self, scene, threads: int = 0):
        lib = reference()
        if lib is None:
            raise RuntimeError("reference host build unavailable")
        self.lib = lib
        self.sc = scene
        if threads:
            lib.ref_set_threads(threads)
        rho = np.ascontiguousarray(scene.initial_density().astype(np.float32))
        lib.ref_init(_fptr(rho), scene.nx, scene.ny, scene.nz)
        lib.ref_set_physics(scene.gravity, scene.buoyancy)
        lib.ref_set_solver(scene.iterations, scene.omega, scene.clamp_const)
        for (x, y, z, r) in scene.spheres:
            lib.ref_add_source(x, y, z, r)
        for ob in scene.obstacles:
            lib.ref_add_obstacle(*ob)
        if scene.mask is not None or scene.u0 is not None:
            st = self.state()
            if scene.mask is not None:
                st["s"][...] = scene.mask
            for k in ("u", "v", "w"):
                a = getattr(scene, k + "0")
                if a is not None:
                    st[k][0][...] = a
            self.set_state(st)
        self.out = np.zeros(scene.cell_shape, np.float32)

    def state(self) -> dict:
        sc = self.sc
        cs, fs = sc.cell_shape, sc.face_shape
        st = {"rho": [np.zeros(cs, np.float32) for _ in range(2)],
              "u": [np.zeros(fs, np.float32) for _ in range(2)],
              "v": [np.zeros(fs, np.float32) for _ in range(2)],
              "w": [np.zeros(fs, np.float32) for _ in range(2)],
              "s": np.zeros(cs, np.uint8), "index_now": C.c_int(0)}
        self.lib.ref_get_state(*[_fptr(a) for k in ("rho", "u", "v", "w") for a in st[k]],
                               st["s"].ctypes.data_as(C.POINTER(C.c_uint8)),
                               C.byref(st["index_now"]))
        st["index_now"] = st["index_now"].value
        return st

    def set_state(self, st: dict):
        idx = C.c_int(st["index_now"])
        self.lib.ref_set_state(*[_fptr(a) for k in ("rho", "u", "v", "w") for a in st[k]],
                               st["s"].ctypes.data_as(C.POINTER(C.c_uint8)), C.byref(idx))

    def step(self, dt: Optional[float] = None) -> np.ndarray:
        for bx in self.sc.boxes:
            self.lib.ref_fill_box(int(bx[0]), int(bx[1]), int(bx[2]), int(bx[3]), int(bx[4]),
                                  int(bx[5]), C.c_float(bx[6]))
        self.lib.ref_simulate(_fptr(self.out), C.c_float(self.sc.dt if dt is None else dt))
        return self.out

    def run(self, steps: Optional[int] = None):
        for _ in range(self.sc.steps if steps is None else steps):
            self.step()
        return self

    def close(self):
        self.lib.ref_delete()
