"""Deterministic synthetic scenes for the smoke step.

The reference ships no datasets or benchmark inputs; every workload here is synthetic and is
generated from named seeds by a project-defined SplitMix64 counter stream, so the GPU library
and every oracle receive bit-identical inputs on any machine.

Geometry (emitter and obstacle centres, radii) is integer-valued, so the reference's
`powf(d, 2)` distance test (project/smokeSimulation.cu:265, :304) is exact and every
implementation rasterises the same cells.

Array layout is the reference's (project/smokeSimulation.cu:127-147): cells n_x*n_y*n_z and
faces (n_x+1)(n_y+1)(n_z+1), x fastest, as numpy arrays shaped (z, y, x).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Tuple

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


class SplitMix64:
    """Counter-based SplitMix64: value i of stream (seed, lane) is mix(base + (i+1)*GAMMA)."""

    def __init__(self, seed: int, lane: int = 0):
        with np.errstate(over="ignore"):
            self.base = _mix(np.array([(seed * 0x100000001B3 + lane) & 0xFFFFFFFFFFFFFFFF],
                                      dtype=np.uint64))[0]
        self.pos = 0

    def u64(self, n: int) -> np.ndarray:
        idx = np.arange(self.pos + 1, self.pos + n + 1, dtype=np.uint64)
        self.pos += n
        with np.errstate(over="ignore"):
            return _mix(self.base + idx * _GAMMA)

    def uniform(self, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        """float64 in [lo, hi) from the top 53 bits."""
        v = (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))
        return lo + (hi - lo) * v

    def uniform_f32(self, n: int, lo: float, hi: float) -> np.ndarray:
        return self.uniform(n, lo, hi).astype(np.float32)

    def integers(self, n: int, lo: int, hi: int) -> np.ndarray:
        """ints in [lo, hi)."""
        return (lo + np.floor(self.uniform(n) * (hi - lo))).astype(np.int64)


@dataclasses.dataclass
class Scene:
    """One simulation: grid, objects, initial state and solver settings."""

    name: str
    nx: int
    ny: int
    nz: int
    dt: float
    steps: int
    # objects in the reference's packing (see smoke_oracle.cpp)
    spheres: List[Tuple[float, float, float, float]] = dataclasses.field(default_factory=list)
    obstacles: List[Tuple[float, ...]] = dataclasses.field(default_factory=list)
    boxes: List[Tuple[float, ...]] = dataclasses.field(default_factory=list)
    mask: Optional[np.ndarray] = None          # uint8 (z,y,x), 1 = fluid; None = reference init
    u0: Optional[np.ndarray] = None            # initial face velocities for buffer [0]
    v0: Optional[np.ndarray] = None
    w0: Optional[np.ndarray] = None
    rho0: Optional[np.ndarray] = None          # initial density for buffer [0]
    gravity: float = -9.82
    buoyancy: float = 2.0
    clamp_const: float = 3.0
    clamp_mode: int = 0
    scheme: int = 0                            # 0 velocity SOR (reference), 1 pressure SOR
    iterations: int = 30
    omega: float = 1.9
    tol: float = 0.0
    check_every: int = 10
    warm_start: int = 0
    refine: int = 0                            # FP64-checked refinement rounds (pressure, tol > 0)
    refine_sweeps: int = 10
    obstacle_velocity: int = 0                 # 1: obstacles' velocity drives the fluid
    solver: int = 0                            # pressure scheme: 0 red-black SOR, 1 Jacobi (omega <= 1)
    omega_warm: float = 0.0                    # warm-started solves after omega_warm_after steps (0: off)
    omega_warm_after: int = 2
    warm_extrapolate: float = 0.0              # warm start from P + a (P - P_before) (0: off)

    @property
    def cells(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def cell_shape(self):
        return (self.nz, self.ny, self.nx)

    @property
    def face_shape(self):
        return (self.nz + 1, self.ny + 1, self.nx + 1)

    def initial_mask(self) -> np.ndarray:
        if self.mask is not None:
            return self.mask
        return reference_initial_mask(self.nx, self.ny, self.nz)

    def initial_density(self) -> np.ndarray:
        if self.rho0 is not None:
            return self.rho0
        return np.zeros(self.cell_shape, np.float32)

    def initial_velocity(self, which: str) -> np.ndarray:
        a = getattr(self, which + "0")
        return a if a is not None else np.zeros(self.face_shape, np.float32)


def reference_initial_mask(nx: int, ny: int, nz: int) -> np.ndarray:
    """initializeVolume's mask: fluid everywhere except the y = 0 floor plane
    (project/smokeSimulation.cu:200-207)."""
    s = np.ones((nz, ny, nx), np.uint8)
    s[:, 0, :] = 0
    return s


def sphere_mask(nx, ny, nz, centres_radii, base: np.ndarray) -> np.ndarray:
    """Mark solid every cell whose integer corner is strictly inside a sphere (same predicate as
    fillObstacle, project/smokeSimulation.cu:304-306), over the whole grid."""
    s = base.copy()
    z, y, x = np.meshgrid(np.arange(nz, dtype=np.float32), np.arange(ny, dtype=np.float32),
                          np.arange(nx, dtype=np.float32), indexing="ij")
    for (cx, cy, cz, r) in centres_radii:
        dx = x - np.float32(cx)
        dy = y - np.float32(cy)
        dz = z - np.float32(cz)
        d2 = dx * dx + dy * dy + dz * dz
        s[d2 < np.float32(r) * np.float32(r)] = 0
    return s


def bernoulli_mask(nx, ny, nz, p: float, seed: int) -> np.ndarray:
    """Reference initial mask plus cells made solid with probability p (seeded)."""
    s = reference_initial_mask(nx, ny, nz)
    rnd = SplitMix64(seed, lane=1).uniform(nx * ny * nz).reshape(nz, ny, nx)
    s[rnd < p] = 0
    return s


def noise_velocity(scene_shape_faces, amp: float, seed: int):
    rng = SplitMix64(seed, lane=2)
    n = int(np.prod(scene_shape_faces))
    return tuple(rng.uniform_f32(n, -amp, amp).reshape(scene_shape_faces) for _ in range(3))


# ---- the five workloads of the headline benchmark ------------------------------------------

def config_ref80(steps: int = 100, scheme: int = 0, emitter_velocity: bool = False) -> Scene:
    """80^3 reference step: sphere obstacle r=10 at (40,30,40), 10x4x10 box emitter at the bottom
    centre (density 1.0; upward velocity 2.0 only when emitter_velocity), dt=0.05, gravity and
    buoyancy on, reference clamp, 40 red-black iterations, velocity noise U[-0.1,0.1] seed 0."""
    n = 80
    sc = Scene("ref80", n, n, n, dt=0.05, steps=steps, iterations=40, scheme=scheme)
    sc.obstacles = [(40.0, 30.0, 40.0, 0.0, 0.0, 0.0, 10.0)]
    sc.boxes = [(35, 1, 35, 45, 5, 45, 1.0, 2.0, 1.0 if emitter_velocity else 0.0)]
    sc.u0, sc.v0, sc.w0 = noise_velocity(sc.face_shape, 0.1, seed=0)
    return sc


def _seeded_spheres(rng: SplitMix64, count: int, n: Tuple[int, int, int], r: int,
                    y_range=None) -> list:
    out = []
    nx, ny, nz = n
    for _ in range(count):
        x = int(rng.integers(1, r + 2, nx - r - 2)[0])
        if y_range is None:
            y = int(rng.integers(1, r + 2, ny - r - 2)[0])
        else:
            y = int(rng.integers(1, y_range[0], y_range[1])[0])
        z = int(rng.integers(1, r + 2, nz - r - 2)[0])
        out.append((float(x), float(y), float(z), float(r)))
    return out


def config_large(n: int = 256, steps: int = 50, max_sweeps: int = 200, tol: float = 1e-4) -> Scene:
    """Single large grid: Bernoulli(0.05) solids (seed 1) plus two r=24 spheres, four seeded
    sphere emitters (r=6, lower half), dt=0.02, pressure red-black SOR to max|div| <= tol capped
    at max_sweeps sweeps, residual checked every 6 sweeps (a group of 12 colour passes splits
    evenly into launches of 2, 4 or 6 passes)."""
    sc = Scene("large%d" % n, n, n, n, dt=0.02, steps=steps, scheme=1, iterations=max_sweeps,
               tol=tol, check_every=6)
    rng = SplitMix64(1, lane=3)
    r_obs = max(2, (24 * n) // 256)
    solids = _seeded_spheres(rng, 2, (n, n, n), r_obs)
    sc.mask = sphere_mask(n, n, n, solids, bernoulli_mask(n, n, n, 0.05, seed=1))
    r_em = max(2, (6 * n) // 256)
    sc.spheres = _seeded_spheres(rng, 4, (n, n, n), r_em, y_range=(r_em + 2, max(r_em + 3, n // 2)))
    return sc


def large_workload(n: int = 256, steps: int = 50, warm_start: int = 1) -> Scene:
    """The single-large-grid workload as the benchmark solves it: config_large with the pressure
    warm-started from the previous step, extrapolated along its last change by 0.5 once two
    solves exist (smk_params.warm_extrapolate), and, once the history is two steps long,
    over-relaxed with 1.75 instead of 1.9 (smk_params.omega_warm).  The residual rule stops at
    max|r| <= 0.995e-4: the divergence of the projected velocity, computed from the rounded face
    updates, can lie a few 1e-8 above the residual, and the workload's bound is max|div u| <=
    1e-4."""
    sc = config_large(n=n, steps=steps)
    sc.warm_start = warm_start
    if warm_start:
        sc.omega_warm, sc.omega_warm_after = 1.75, 2
        sc.warm_extrapolate = 0.5
        sc.tol = 0.995e-4
    return sc


def config_batched(count: int = 64, steps: int = 100, seed: int = 2, lo: int = 32, hi: int = 128,
                   scheme: int = 1, iterations: int = 40) -> List[Scene]:
    """Batched plain-precision grids: cube side log-uniform in [lo, hi] (seed 2), each with a
    seeded sphere solid and a box emitter; dt=0.05."""
    rng = SplitMix64(seed, lane=4)
    sides = np.round(np.exp(rng.uniform(count, math.log(lo), math.log(hi)))).astype(int)
    scenes = []
    for i, n in enumerate(sides):
        n = int(n)
        sc = Scene("batch%02d_%d" % (i, n), n, n, n, dt=0.05, steps=steps, scheme=scheme,
                   iterations=iterations)
        r = max(2, n // 8)
        solid = _seeded_spheres(rng, 1, (n, n, n), r)
        sc.mask = sphere_mask(n, n, n, solid, reference_initial_mask(n, n, n))
        b = max(2, n // 8)
        cx = int(rng.integers(1, b + 1, n - b - 1)[0])
        cz = int(rng.integers(1, b + 1, n - b - 1)[0])
        sc.boxes = [(cx - b // 2, 1, cz - b // 2, cx - b // 2 + b, 1 + max(2, b // 2), cz - b // 2 + b,
                     1.0, 0.0, 0.0)]
        scenes.append(sc)
    return scenes


def config_mixed(n: int = 512, steps: int = 20) -> Scene:
    """Large mixed-precision grid: Bernoulli(0.02) solids (seed 3), one 32x8x32 box emitter at
    the bottom centre, dt=0.02; pressure to max|div| <= 1e-4 checked every 6 sweeps (the
    single-grid workload's interval)."""
    sc = Scene("mixed%d" % n, n, n, n, dt=0.02, steps=steps, scheme=1, iterations=200, tol=1e-4,
               check_every=6)
    sc.mask = bernoulli_mask(n, n, n, 0.02, seed=3)
    bx, by, bz = max(2, 32 * n // 512), max(2, 8 * n // 512), max(2, 32 * n // 512)
    c = n // 2
    sc.boxes = [(c - bx // 2, 1, c - bz // 2, c - bx // 2 + bx, 1 + by, c - bz // 2 + bz, 1.0, 0.0, 0.0)]
    return sc


def small_scene(nx=20, ny=16, nz=18, steps=6, seed=11, scheme=0, iterations=30, obstacles=1,
                sources=1, boxes=1, noise=0.5, dt=0.05, **kw) -> Scene:
    """Small scene with every object kind, for stage and step parity tests (odd sizes allowed)."""
    rng = SplitMix64(seed, lane=5)
    sc = Scene("small_%dx%dx%d_s%d" % (nx, ny, nz, seed), nx, ny, nz, dt=dt, steps=steps,
               scheme=scheme, iterations=iterations, **kw)
    m = min(nx, ny, nz)
    for _ in range(obstacles):
        r = max(2, m // 5)
        x, y, z = (int(rng.integers(1, r, nx - r)[0]), int(rng.integers(1, r, ny - r)[0]),
                   int(rng.integers(1, r, nz - r)[0]))
        sc.obstacles.append((float(x), float(y), float(z), 0.0, 0.0, 0.0, float(r)))
    for _ in range(sources):
        r = max(2, m // 6)
        x, y, z = (int(rng.integers(1, 2, nx - 2)[0]), int(rng.integers(1, 2, ny - 2)[0]),
                   int(rng.integers(1, 2, nz - 2)[0]))
        sc.spheres.append((float(x), float(y), float(z), float(r)))
    for _ in range(boxes):
        x0 = int(rng.integers(1, 1, nx - 4)[0])
        z0 = int(rng.integers(1, 1, nz - 4)[0])
        sc.boxes.append((x0, 1, z0, x0 + 3, 3, z0 + 3, 1.0, 0.0, 0.0))
    if noise:
        sc.u0, sc.v0, sc.w0 = noise_velocity(sc.face_shape, noise, seed=seed)
    return sc
