"""CPU tests: the oracle restatement against the reference's own step.

The restatement (oracle/smoke_oracle.cpp) must reproduce the reference's host-built step
(project/smokeSimulation.cu compiled for the CPU, oracle/_ref) bit for bit on every field of
both ping-pong buffers, and must reproduce the committed golden vectors that were generated
from that build.  It also fixes the tolerances between the pressure-form projection, the
reference's velocity-form projection and the FP64 oracle.
"""
import numpy as np
import pytest

from oracle import oracle as O
from smoke_simulation_gb300 import scenes as S
from tests import helpers as H


def _run_oracle(sc, dtype=np.float32, scheme=None, steps=None):
    o = O.OracleSim(sc, dtype, scheme)
    o.run(steps)
    return o


@pytest.mark.parametrize("name,scene", [
    ("tiny", lambda: S.small_scene(12, 10, 11, steps=5, seed=3)),
    ("small_a", lambda: S.small_scene()),
    ("small_b", lambda: S.small_scene(17, 23, 19, seed=5, obstacles=2, sources=3)),
])
def test_restatement_matches_golden_small(name, scene):
    g = H.golden()["scenes"][name]
    o = _run_oracle(scene())
    assert H.state_hashes(H.oracle_state(o)) == g["final"]
    assert H.sha(o.density()) == g["density_out"]


def test_restatement_matches_tiny_fixture_arrays():
    fx = np.load(H.GOLDEN_DIR + "/tiny_state.npz")
    o = _run_oracle(S.small_scene(12, 10, 11, steps=5, seed=3))
    for k in ("rho", "u", "v", "w"):
        for j in range(2):
            assert H.bits_equal(getattr(o, k)[j], fx["%s%d" % (k, j)]), (k, j)
    assert np.array_equal(o.s, fx["s"])
    assert int(fx["index_now"]) == o.index_now
    assert H.bits_equal(o.density(), fx["density_out"])


def test_restatement_matches_golden_ref80():
    g = H.golden()["scenes"]["ref80"]
    sc = S.config_ref80(steps=100)
    o = O.OracleSim(sc)
    for k in range(100):
        o.step()
        if (k + 1) % 20 == 0:
            assert H.sha(o.density()) == g["density_every_20"][str(k + 1)], k + 1
    assert H.state_hashes(H.oracle_state(o)) == g["final"]


def test_restatement_matches_golden_app80():
    """The reference application's scene with a moving source and a physics change."""
    from tests.golden.make_golden import app80_scene
    g = H.golden()["scenes"]["app80"]
    sc = app80_scene()
    o = O.OracleSim(sc)
    o.step(0.01)
    for k in range(sc.steps):
        if k == 10:
            sc.gravity, sc.buoyancy = -5.0, 6.0
        o.update_sphere(0, *H.app80_path(k))
        o.step(0.05)
        assert H.sha(o.density()) == g["density_each_step"][str(k + 1)], k + 1
    assert H.state_hashes(H.oracle_state(o)) == g["final"]


needs_ref = pytest.mark.skipif(not O.reference_available(),
                               reason="reference host build unavailable on this machine")


@needs_ref
@pytest.mark.parametrize("dims,seed,kw", [
    ((9, 8, 7), 21, {}),
    ((16, 16, 16), 22, {"obstacles": 3, "sources": 3}),
    ((31, 12, 20), 23, {"noise": 4.0}),            # large velocities: clamp triggers
    ((5, 5, 5), 24, {"boxes": 0, "obstacles": 0}),
    ((3, 40, 4), 25, {}),                          # degenerate thin grid
])
def test_restatement_equals_reference_stepwise(dims, seed, kw):
    sc = S.small_scene(*dims, steps=4, seed=seed, **kw)
    a = O.OracleSim(sc)
    b = O.RefHostSim(sc)
    try:
        for k in range(sc.steps):
            a.step()
            b.step()
            msg = H.first_mismatch(H.oracle_state(a), b.state())
            assert msg == "", "step %d: %s" % (k, msg)
            assert H.bits_equal(a.density(), b.out)
    finally:
        b.close()


@needs_ref
def test_reference_thread_count_invariance():
    sc = S.small_scene(18, 17, 16, steps=3, seed=31)
    outs = []
    for threads in (1, 4):
        b = O.RefHostSim(sc, threads=threads)
        b.run()
        outs.append(b.state())
        b.close()
    assert H.first_mismatch(outs[0], outs[1]) == ""


def test_pressure_form_within_tolerance_of_reference_form():
    """Pressure-form SOR vs the reference's velocity-form SOR, 100 steps at 80^3 (FP32)."""
    sc = S.config_ref80(steps=40)
    a = _run_oracle(sc, scheme=0)
    b = _run_oracle(sc, scheme=1)
    assert H.max_abs(b.density(), a.density()) <= H.DENSITY_MAX_ABS
    assert H.rel_l2(b.density(), a.density()) <= H.DENSITY_REL_L2
    for k in ("u", "v", "w"):
        for j in range(2):
            assert H.max_abs(getattr(b, k)[j], getattr(a, k)[j]) <= H.VELOCITY_MAX_ABS, k
            assert H.rel_l2(getattr(b, k)[j], getattr(a, k)[j]) <= H.VELOCITY_REL_L2, k


@pytest.mark.parametrize("scheme", [0, 1])
def test_fp32_within_tolerance_of_fp64(scheme):
    sc = S.config_ref80(steps=40)
    a = _run_oracle(sc, np.float32, scheme)
    b = _run_oracle(sc, np.float64, scheme)
    assert H.max_abs(a.density(), b.density()) <= H.DENSITY_MAX_ABS
    assert H.rel_l2(a.density(), b.density()) <= H.DENSITY_REL_L2


def test_tolerance_rule():
    sc = S.config_large(n=48, steps=3)
    o = O.OracleSim(sc)
    for _ in range(3):
        st = o.step()
        assert st.sweeps % sc.check_every == 0 or st.sweeps == sc.iterations
        if st.converged:
            assert st.resid_max <= sc.tol
            assert st.div_max <= 2 * sc.tol
    # with the tolerance off, exactly the cap
    sc.tol = 0.0
    o = O.OracleSim(sc)
    st = o.step()
    assert st.sweeps == sc.iterations and st.converged == 0


def test_masks_are_identical_across_precisions():
    sc = S.small_scene(20, 16, 18, steps=3, seed=7, obstacles=2)
    a = _run_oracle(sc, np.float32)
    b = _run_oracle(sc, np.float64)
    assert np.array_equal(a.s, b.s)


def test_scene_generator_is_deterministic():
    a = S.config_large(n=64, steps=1)
    b = S.config_large(n=64, steps=1)
    assert np.array_equal(a.mask, b.mask) and a.spheres == b.spheres
    solid = 1.0 - a.mask.mean()
    assert 0.05 < solid < 0.15  # Bernoulli(0.05) + floor + two spheres
    sides = [s.nx for s in S.config_batched()]
    assert len(sides) == 64 and min(sides) >= 32 and max(sides) <= 128
    r = S.SplitMix64(7).uniform(1000)
    assert 0.45 < r.mean() < 0.55


def test_refinement_rounds_reduce_fp64_divergence():
    """FP64-checked refinement (oracle): after a solve capped well short of a tight tolerance,
    each correction round lowers the FP64-measured max|div u|; with a loose tolerance no round
    is applied."""
    from smoke_simulation_gb300 import scenes as S
    out = {}
    for refine, tol in ((0, 1e-5), (1, 1e-5), (3, 1e-5), (3, 10.0)):
        sc = S.small_scene(24, 20, 26, steps=2, seed=31, scheme=1, iterations=12, tol=tol,
                           check_every=4, warm_start=1)
        sc.refine, sc.refine_sweeps = refine, 8
        o = O.OracleSim(sc)
        for _ in range(sc.steps):
            st = o.step()
        out[(refine, tol)] = st
    assert out[(0, 1e-5)].refine_rounds == 0 and out[(0, 1e-5)].div64_max == -1.0
    assert out[(1, 1e-5)].refine_rounds == 1 and out[(3, 1e-5)].refine_rounds == 3
    assert out[(3, 1e-5)].div64_max < out[(1, 1e-5)].div64_max < out[(0, 1e-5)].div_max
    assert out[(3, 10.0)].refine_rounds == 0
    assert 0.0 <= out[(3, 10.0)].div64_max <= 10.0


def test_obstacle_velocity_drives_the_fluid():
    """With obstacle_velocity on, the fluid next to a moving obstacle moves with it; with it off
    (the reference), the obstacle's stored velocity has no effect."""
    from smoke_simulation_gb300 import scenes as S
    res = {}
    for on in (0, 1):
        for vx in (0.0, 2.0):
            sc = S.small_scene(24, 20, 24, steps=4, seed=43, scheme=1, iterations=40, obstacles=0, noise=0.0)
            sc.tol, sc.check_every, sc.obstacle_velocity = 1e-5, 5, on
            sc.obstacles = [(12.0, 10.0, 12.0, vx, 0.0, 0.0, 4.0)]
            o = O.OracleSim(sc)
            o.run()
            res[(on, vx)] = o.u[o.past].copy()
    assert np.array_equal(res[(0, 0.0)], res[(0, 2.0)])  # reference: velocity stored, unused
    near = np.s_[6:14, 6:14, 14:20]                       # (z, y, x) just past the obstacle
    assert np.abs(res[(1, 2.0)][near]).max() > 5 * np.abs(res[(1, 0.0)][near]).max() + 0.1


def test_jacobi_first_iteration_is_the_scaled_rhs():
    """The restatement's Jacobi solver (pressure scheme, solver 1), pinned by a direct numpy
    restatement: from a zero start one iteration sets P = (omega/acc) * b on every projectable
    cell (interior, fluid, >= 1 fluid neighbour; acc = its fluid neighbours) and 0 elsewhere."""
    sc = S.small_scene(20, 16, 18, steps=1, seed=5, scheme=1, iterations=1, solver=1, omega=0.8)
    o = O.OracleSim(sc)
    o.step()
    s = o.s.astype(bool)  # (z, y, x)
    nz, ny, nx = s.shape
    acc = np.zeros(s.shape, np.int32)
    inner = (slice(1, nz - 1), slice(1, ny - 1), slice(1, nx - 1))
    for ax in range(3):
        for sh in (-1, 1):
            acc[inner] += np.roll(s, sh, axis=ax)[inner]
    proj = np.zeros(s.shape, bool)
    proj[inner] = s[inner] & (acc[inner] > 0)
    w = np.zeros(s.shape, np.float32)
    w[proj] = np.float32(0.8) / acc[proj].astype(np.float32)
    expected = np.where(proj, w * o.b, np.float32(0))
    assert np.array_equal(o.P, expected)
    assert np.count_nonzero(o.P) > 0


def test_jacobi_reaches_the_sor_solution():
    """Solved to a tight tolerance, weighted Jacobi and red-black SOR give the same step (both
    satisfy the same discrete Poisson problem); Jacobi needs more iterations."""
    out = {}
    for solver, omega in ((0, 1.9), (1, 1.0)):
        sc = S.small_scene(20, 16, 18, steps=2, seed=7, scheme=1, iterations=20000, tol=1e-7,
                           check_every=10, solver=solver, omega=omega)
        o = O.OracleSim(sc, dtype=np.float64)
        sweeps = [o.step().sweeps for _ in range(sc.steps)]
        out[solver] = (o, sweeps)
    a, b = out[0][0], out[1][0]
    for k in ("u", "v", "w", "rho"):
        for j in range(2):
            x, y = getattr(a, k)[j], getattr(b, k)[j]
            assert H.rel_l2(x, y) < 1e-5, (k, j, H.rel_l2(x, y))
    assert min(out[1][1]) > max(out[0][1])


def _extrap_scene(a):
    sc = S.small_scene(24, 22, 26, steps=6, seed=19, scheme=1, iterations=120, tol=1e-4, check_every=3,
                       warm_start=1)
    sc.warm_extrapolate = a
    return sc


def test_warm_extrapolate_rule():
    """The extrapolated warm start as the library applies it (body_rhs with a pressure history):
    the first two steps of a history start from the last pressure (identical to a = 0), the third
    starts from P + a (P - P_before) computed in float32, and a history switched on between
    steps is saved by the next step and used one step later."""
    plain = O.OracleSim(_extrap_scene(0.0))
    ext = O.OracleSim(_extrap_scene(0.5))
    for k in range(2):
        plain.step()
        ext.step()
        assert np.array_equal(plain.P, ext.P) and H.first_mismatch(H.oracle_state(plain), H.oracle_state(ext)) == ""
    # the start of step 3, restated from the two saved solutions
    p1 = ext.P.copy()
    p0 = ext.Ph.copy()
    want = p1 + np.float32(0.5) * (p1 - p0)
    ext._warm_extrapolate()
    assert np.array_equal(ext.P, want) and not np.array_equal(want, p1)
    # switched on after two plain steps: step 3 saves, step 4 extrapolates
    late = O.OracleSim(_extrap_scene(0.0))
    ref = O.OracleSim(_extrap_scene(0.0))
    for k in range(4):
        if k == 2:
            late.sc.warm_extrapolate = 0.5
        late.step()
        ref.step()
        same = H.first_mismatch(H.oracle_state(late), H.oracle_state(ref)) == ""
        assert same == (k < 3), k
