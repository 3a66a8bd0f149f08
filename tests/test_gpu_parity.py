"""GPU parity tests through the C ABI.

REFERENCE scheme: bit-exact with the reference's own step (golden vectors generated from its
host build) and with the oracle restatement, on every field of both ping-pong buffers.
PRESSURE scheme: bit-exact with the oracle's pressure-form restatement (same operation order),
and within the stated tolerances (tests/helpers.py) of the reference form and of FP64.
"""
import ctypes as C

import numpy as np
import pytest

import smoke_simulation_gb300 as smk
from oracle import oracle as O
from smoke_simulation_gb300 import scenes as S
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _run_gpu(sc, steps=None, **over):
    sim = smk.from_scene(sc, **over)
    for _ in range(sc.steps if steps is None else steps):
        sim.step(sc.dt)
    return sim


@pytest.mark.parametrize("name,scene", [
    ("tiny", lambda: S.small_scene(12, 10, 11, steps=5, seed=3)),
    ("small_a", lambda: S.small_scene()),
    ("small_b", lambda: S.small_scene(17, 23, 19, seed=5, obstacles=2, sources=3)),
])
def test_reference_scheme_matches_golden_small(gpu, name, scene):
    g = H.golden()["scenes"][name]
    sim = _run_gpu(scene())
    st = sim.read_state()
    if H.state_hashes(st) != g["final"]:
        o = O.OracleSim(scene()).run()
        pytest.fail(H.first_mismatch(st, H.oracle_state(o)))
    assert H.sha(sim.read_density()) == g["density_out"]
    sim.close()


def test_reference_scheme_matches_golden_ref80(gpu):
    g = H.golden()["scenes"]["ref80"]
    sc = S.config_ref80(steps=100)
    sim = smk.from_scene(sc)
    out = np.zeros(sc.cell_shape, np.float32)
    for k in range(100):
        sim.simulate(out, sc.dt)
        if (k + 1) % 20 == 0:
            assert H.sha(out) == g["density_every_20"][str(k + 1)], k + 1
    assert H.state_hashes(sim.read_state()) == g["final"]
    sim.close()


@pytest.mark.parametrize("dims,seed,kw", [
    ((9, 8, 7), 21, {}),
    ((16, 16, 16), 22, {"obstacles": 3, "sources": 3}),
    ((31, 12, 20), 23, {"noise": 4.0}),
    ((5, 5, 5), 24, {"boxes": 0, "obstacles": 0}),
    ((3, 40, 4), 25, {}),
    ((67, 33, 45), 26, {"obstacles": 2, "sources": 2}),
])
def test_reference_scheme_equals_oracle_stepwise(gpu, dims, seed, kw):
    sc = S.small_scene(*dims, steps=4, seed=seed, **kw)
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc)
    for k in range(sc.steps):
        o.step()
        sim.step(sc.dt)
        msg = H.first_mismatch(sim.read_state(), H.oracle_state(o))
        assert msg == "", "step %d: %s" % (k, msg)
    sim.close()


def test_reference_api_symbols_match_golden_app80(gpu):
    """The reference's own C++ entry points (mangled names, exactly as main.cpp calls them)."""
    L = smk.lib()
    f = C.c_float
    init = L["_Z16initializeVolumePfjjj"]
    init.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint]
    add_src = L["_Z14addSmokeSourceffff"]
    add_src.argtypes = [f] * 4
    add_src.restype = C.c_int
    add_obs = L["_Z11addObstaclefffffff"]
    add_obs.argtypes = [f] * 7
    add_obs.restype = C.c_int
    upd = L["_Z15updateObjectPosifff"]
    upd.argtypes = [C.c_int, f, f, f]
    simulate = L["_Z8simulatePff"]
    simulate.argtypes = [C.c_void_p, f]
    grav = L["_Z10getGravityv"]
    grav.restype = C.POINTER(f)
    buoy = L["_Z11getBuoyancyv"]
    buoy.restype = C.POINTER(f)
    delete = L["_Z12deleteVolumev"]

    g = H.golden()["scenes"]["app80"]
    grid = np.zeros((80, 80, 80), np.float32)
    init(grid.ctypes.data, 80, 80, 80)
    sid = add_src(40.0, 40.0, 40.0, 5.0)
    add_obs(60.0, 10.0, 60.0, 0.0, 0.0, 0.0, 13.0)
    grav()[0], buoy()[0] = -9.82, 2.0
    simulate(grid.ctypes.data, 0.01)
    for k in range(20):
        if k == 10:
            grav()[0], buoy()[0] = -5.0, 6.0
        upd(sid, *H.app80_path(k))
        simulate(grid.ctypes.data, 0.05)
        assert H.sha(grid) == g["density_each_step"][str(k + 1)], k + 1
    delete()


@pytest.mark.parametrize("dims,seed", [((20, 16, 18), 11), ((33, 17, 29), 41), ((64, 64, 64), 42)])
@pytest.mark.parametrize("tol", [0.0, 1e-3])
@pytest.mark.parametrize("kernel", [(0, 1), (2, 7), (4, 32), (6, 5), (4, 3), (4, 32, 4), (4, 3, 4),
                                    (6, 5, 2 | smk.SWEEP_YCLUSTER), (6, 117, 2 | smk.SWEEP_YCLUSTER),
                                    (6, 5, 2 | smk.SWEEP_YCLUSTER | smk.SWEEP_YCLUSTER_N(2)),
                                    (6, 117, 2 | smk.SWEEP_YCLUSTER | smk.SWEEP_YCLUSTER_N(4))])
def test_pressure_scheme_equals_oracle(gpu, dims, seed, tol, kernel):
    """Every sweep kernel (one colour pass per launch, or temporally blocked with depth 2-6
    over several z-chunk sizes, with 2- and 4-row patches, and the y-cluster forms exchanging
    boundary rows through distributed shared memory: one cluster spanning y, clusters of 2 and
    of 4) reproduces the oracle bit for bit, including the tolerance rule's sweep counts and
    residuals."""
    sc = S.small_scene(*dims, steps=5, seed=seed, scheme=1, iterations=41, tol=tol,
                       check_every=5, obstacles=2)
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc, report_div=1)
    sim.set_sweep_kernel(*kernel)
    for k in range(sc.steps):
        ost = o.step()
        sim.step(sc.dt)
        st = sim.stats()
        assert st.sweeps == ost.sweeps, (k, st.sweeps, ost.sweeps)
        assert st.converged == ost.converged
        if tol > 0:
            assert st.resid_max == ost.resid_max
        assert st.div_max == ost.div_max
        msg = H.first_mismatch(sim.read_state(), H.oracle_state(o))
        assert msg == "", "step %d: %s" % (k, msg)
    sim.close()


@pytest.mark.parametrize("kernel", [(0, 1), (4, 11), (6, 25), (4, 11, 4), (6, 25, 2 | smk.SWEEP_YCLUSTER),
                                    (6, 25, 2 | smk.SWEEP_YCLUSTER | smk.SWEEP_YCLUSTER_N(2))])
def test_warm_start_equals_oracle(gpu, kernel):
    """Warm start (the pressure carried across steps, including through the blocked kernel's
    second buffer) follows the oracle bit for bit, and stays within the tolerance."""
    sc = S.small_scene(36, 30, 40, steps=6, seed=55, scheme=1, iterations=60, tol=1e-3,
                       check_every=6, obstacles=1, warm_start=1)
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc, report_div=1)
    sim.set_sweep_kernel(*kernel)
    for k in range(sc.steps):
        ost = o.step()
        sim.step(sc.dt)
        st = sim.stats()
        assert st.sweeps == ost.sweeps and st.div_max == ost.div_max
        assert H.first_mismatch(sim.read_state(), H.oracle_state(o)) == "", k
    sim.close()


def test_pressure_scheme_within_tolerance_of_reference_and_fp64(gpu):
    sc = S.config_ref80(steps=40)
    sim = _run_gpu(sc, projection=1)
    rho = sim.read_density()
    ref = O.OracleSim(sc, np.float32, 0).run()
    f64 = O.OracleSim(sc, np.float64, 0).run()
    assert H.max_abs(rho, ref.density()) <= H.DENSITY_MAX_ABS
    assert H.rel_l2(rho, ref.density()) <= H.DENSITY_REL_L2
    assert H.max_abs(rho, f64.density()) <= H.DENSITY_MAX_ABS
    assert H.rel_l2(rho, f64.density()) <= H.DENSITY_REL_L2
    sim.close()


def test_large_grid_properties(gpu):
    """256^3 workload, two steps: finite fields, mask kept bit-exact, tolerance rule honoured,
    and the post-projection divergence within the tolerance when converged."""
    sc = S.config_large(n=256, steps=2)
    sim = smk.from_scene(sc, report_div=1)
    for _ in range(2):
        sim.step(sc.dt)
        st = sim.stats()
        assert st.sweeps <= sc.iterations and (st.sweeps % sc.check_every == 0
                                                or st.sweeps == sc.iterations)
        if st.converged:
            assert st.resid_max <= sc.tol
        assert np.isfinite(st.div_max)
    s = sim.read_state()
    assert np.array_equal(s["s"], sc.mask)
    for k in ("rho", "u", "v", "w"):
        for j in range(2):
            assert np.isfinite(s[k][j]).all()
    rho = s["rho"][s["index_now"] ^ 1]
    assert 0.99 <= rho.max() <= 1.0 + 1e-6 and rho.min() >= -1e-6
    sim.close()


def test_state_roundtrip_and_resume(gpu):
    """read_state / write_state reproduce a run exactly (checkpoint / resume)."""
    sc = S.small_scene(24, 20, 22, steps=6, seed=9, scheme=1, iterations=20)
    a = _run_gpu(sc, steps=3)
    ck = a.read_state()
    b = smk.from_scene(sc)
    b.write_state(ck)
    for _ in range(3):
        a.step(sc.dt)
        b.step(sc.dt)
    assert H.first_mismatch(a.read_state(), b.read_state()) == ""
    a.close()
    b.close()


def test_density_to_device_buffer(gpu):
    import torch
    sc = S.small_scene(16, 12, 14, steps=2, seed=4)
    sim = _run_gpu(sc)
    dev = torch.empty(sc.cell_shape, dtype=torch.float32, device=gpu)
    stream = torch.cuda.current_stream().cuda_stream
    sim.read_density_device(dev.data_ptr(), stream)
    torch.cuda.synchronize()
    assert H.bits_equal(dev.cpu().numpy(), sim.read_density())
    sim.close()


def test_stage_timing_and_launch_count(gpu):
    sc = S.small_scene(32, 32, 32, steps=2, seed=5, scheme=1, iterations=10)
    sim = smk.from_scene(sc)
    sim.set_timing(True)
    n0 = sim.launch_count()
    sim.step(sc.dt)
    t = sim.stage_times()
    assert (t >= 0).all() and t[4] >= t[:4].sum() * 0.99
    assert sim.launch_count() > n0
    sim.close()


def test_graphs_and_autotune_do_not_change_results(gpu):
    """Graph replay (re-captured when dt or an object changes) and an autotuned sweep kernel
    give the same bits as direct launches with the default kernel."""
    sc = S.small_scene(48, 40, 56, steps=8, seed=17, scheme=1, iterations=30, tol=1e-3,
                       check_every=5, obstacles=1, sources=1)
    a = smk.from_scene(sc, report_div=1)
    b = smk.from_scene(sc, report_div=1)
    a.autotune()
    b.set_graphs(False)
    b.set_sweep_kernel(0, 1)
    for k in range(sc.steps):
        dt = sc.dt if k < 3 else 0.5 * sc.dt
        if k == 5:
            a.update_object_pos(len(sc.boxes), 20.0, 9.0, 21.0)
            b.update_object_pos(len(sc.boxes), 20.0, 9.0, 21.0)
        a.step(dt)
        b.step(dt)
        assert a.stats().sweeps == b.stats().sweeps
    assert H.first_mismatch(a.read_state(), b.read_state()) == ""
    a.close()
    b.close()


@pytest.mark.parametrize("depth,check,rows", [(6, 6, 2), (4, 6, 2), (2, 5, 2), (6, 1, 2), (4, 6, 4),
                                              (6, 6, 2 | smk.SWEEP_YCLUSTER),
                                              (6, 6, 2 | smk.SWEEP_YCLUSTER | smk.SWEEP_YCLUSTER_N(2))])
def test_device_group_loop_equals_unrolled_and_direct(gpu, depth, check, rows):
    """The graph's device-side WHILE loop over tolerance groups gives the bits, sweep counts,
    residuals and divergence of the unrolled graph and of direct launches, with stage timing on
    (events recorded inside the graph), and launches fewer kernels when the sweep cap is well
    above what the tolerance needs.  (4, 6): a group of three launches, so the loop body holds
    two groups."""
    # a cap well above the sweeps the tolerance needs, as in the benchmark workload
    sc = S.small_scene(40, 36, 44, steps=6, seed=29, scheme=1, iterations=150, tol=2e-4,
                       check_every=check, warm_start=1)
    sims = [smk.from_scene(sc, report_div=1) for _ in range(3)]
    for s in sims:
        s.set_sweep_kernel(depth, 17, rows)
    sims[1].set_graph_loops(False)
    sims[2].set_graphs(False)
    sims[0].set_timing(True)
    for k in range(sc.steps):
        stats = []
        for s in sims:
            s.step(sc.dt)
            st = s.stats()
            stats.append((st.sweeps, st.converged, st.resid_max, st.div_max))
        assert stats[0] == stats[1] == stats[2], (k, stats)
        t = sims[0].stage_times()
        assert t[5] > 0.0 and t[4] >= t[5]
    a, b, c = (s.read_state() for s in sims)
    assert H.first_mismatch(a, b) == "" and H.first_mismatch(a, c) == ""
    assert sims[0].launch_count() < sims[1].launch_count()
    for s in sims:
        s.close()


@pytest.mark.parametrize("graphs", [True, False])
def test_refinement_bit_exact_with_oracle(gpu, graphs):
    """FP64-checked refinement rounds: the GPU gives the oracle's bits, sweep counts, rounds
    applied and FP64 divergence, with the step replayed as a graph or launched directly."""
    sc = S.small_scene(24, 20, 26, steps=4, seed=31, scheme=1, iterations=12, tol=1e-5,
                       check_every=4, warm_start=1)
    sc.refine, sc.refine_sweeps = 3, 8
    sim = smk.from_scene(sc, report_div=1)
    sim.set_graphs(graphs)
    o = O.OracleSim(sc)
    for k in range(sc.steps):
        sim.step(sc.dt)
        so = o.step()
        sg = sim.stats()
        assert (sg.sweeps, sg.refine_rounds) == (so.sweeps, so.refine_rounds), k
        assert H.bits_equal(np.float32(sg.div64_max), np.float32(so.div64_max)), k
        assert H.bits_equal(np.float32(sg.div_max), np.float32(so.div_max)), k
    assert H.first_mismatch(sim.read_state(), H.oracle_state(o)) == ""
    sim.close()


def test_refinement_bf16_velocities_lowers_divergence(gpu):
    sc = S.small_scene(24, 20, 26, steps=3, seed=31, scheme=1, iterations=12, tol=1e-5,
                       check_every=4, warm_start=1)
    plain = smk.from_scene(sc, report_div=1, storage=smk.STORAGE_BF16_VEL)
    sc.refine, sc.refine_sweeps = 3, 8
    ref = smk.from_scene(sc, report_div=1, storage=smk.STORAGE_BF16_VEL)
    for _ in range(sc.steps):
        plain.step(sc.dt)
        ref.step(sc.dt)
    a, b = plain.stats(), ref.stats()
    assert b.refine_rounds == 3 and b.div64_max < 0.2 * a.div_max
    plain.close()
    ref.close()


@pytest.mark.parametrize("scheme", [0, 1])
def test_moving_obstacle_velocity_bit_exact(gpu, scheme):
    """An obstacle moved every step whose velocity drives the fluid (obstacle_velocity = 1):
    bit-exact with the oracle in both projection schemes."""
    sc = S.small_scene(28, 24, 30, steps=6, seed=41, scheme=scheme, iterations=30, obstacles=0)
    if scheme == 1:
        sc.tol, sc.check_every = 1e-4, 5
    sc.obstacle_velocity = 1
    sc.obstacles = [(10.0, 12.0, 15.0, 1.5, 0.25, -0.5, 4.0)]
    sim = smk.from_scene(sc)
    o = O.OracleSim(sc)
    oid = len(sc.boxes) + len(sc.spheres)
    for k in range(sc.steps):
        pos = (10.0 + 1.5 * sc.dt * (k + 1) * 10.0, 12.0, 15.0 - 0.5 * sc.dt * (k + 1) * 10.0)
        sim.update_object_pos(oid, *pos)
        o.obstacles[0, :3] = pos
        sim.step(sc.dt)
        o.step()
    assert H.first_mismatch(sim.read_state(), H.oracle_state(o)) == ""
    sim.close()


@pytest.mark.parametrize("tol,warm", [(0.0, 0), (1e-3, 0), (1e-3, 1)])
def test_jacobi_solver_equals_oracle(gpu, tol, warm):
    """The weighted Jacobi option of the pressure scheme (P and P2 ping-pong, one launch per
    iteration) reproduces the oracle bit for bit, tolerance rule and warm start included, with
    graph replay; a batch of Jacobi members runs as branches with the same results."""
    sc = S.small_scene(33, 17, 29, steps=5, seed=41, scheme=1, iterations=37, tol=tol, check_every=5,
                       obstacles=2, solver=smk.SOLVER_JACOBI, omega=0.9, warm_start=warm)
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc, report_div=1)
    twin = smk.from_scene(sc, report_div=1)
    batch = smk.Batch([twin])
    for k in range(sc.steps):
        ost = o.step()
        sim.step(sc.dt)
        batch.step(sc.dt)
        st = sim.stats()
        assert st.sweeps == ost.sweeps, (k, st.sweeps, ost.sweeps)
        assert st.converged == ost.converged
        if tol > 0:
            assert st.resid_max == ost.resid_max
        assert st.div_max == ost.div_max
        msg = H.first_mismatch(sim.read_state(), H.oracle_state(o))
        assert msg == "", "step %d: %s" % (k, msg)
    assert batch.info()[0] == smk.BATCH_BRANCHES
    assert H.first_mismatch(twin.read_state(), sim.read_state()) == ""
    batch.close()
    sim.close()
    twin.close()


def test_ycluster_sweep_rejects_tall_grids(gpu):
    """The y-cluster form with one cluster spanning y needs ny <= 256; clusters of 2 or 4 CTAs
    take any height, and other cluster sizes are rejected."""
    sc = S.small_scene(8, 300, 8, steps=1, seed=3, scheme=1, iterations=6)
    sim = smk.from_scene(sc)
    with pytest.raises(smk.SmokeError):
        sim.set_sweep_kernel(6, 17, 2 | smk.SWEEP_YCLUSTER)
    for n in (2, 4):
        sim.set_sweep_kernel(6, 17, 2 | smk.SWEEP_YCLUSTER | smk.SWEEP_YCLUSTER_N(n))
    for n in (1, 3, 8):
        with pytest.raises(smk.SmokeError):
            sim.set_sweep_kernel(6, 17, 2 | smk.SWEEP_YCLUSTER | smk.SWEEP_YCLUSTER_N(n))
    sim.close()


@pytest.mark.parametrize("n", [2, 4])
def test_ycluster_runs_equal_oracle_on_tall_grid(gpu, n):
    """Clusters of 2 and of 4 CTAs on a grid several clusters tall (140 rows: 3 clusters of 2,
    2 clusters of 4), so the halo at the ends of each cluster's rows and the exchange between the
    CTAs of a cluster both decide cells of the result: bit-exact with the oracle."""
    sc = S.small_scene(20, 140, 18, steps=4, seed=61, scheme=1, iterations=48, tol=1e-3,
                       check_every=6, obstacles=2, warm_start=1)
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc, report_div=1)
    sim.set_sweep_kernel(6, 7, 2 | smk.SWEEP_YCLUSTER | smk.SWEEP_YCLUSTER_N(n))
    for k in range(sc.steps):
        ost = o.step()
        sim.step(sc.dt)
        st = sim.stats()
        assert st.sweeps == ost.sweeps and st.resid_max == ost.resid_max and st.div_max == ost.div_max
        assert H.first_mismatch(sim.read_state(), H.oracle_state(o)) == "", k
    sim.close()


@pytest.mark.parametrize("kernel", [(6, 21), (6, 117), (4, 17), (2, 15), (4, 17, 4)])
def test_edge_windows_equal_oracle(gpu, kernel):
    """Windows that reach the grid's edge carry no halo on that side where that saves windows
    (depth 6: two along x at nx = 110, three along y at ny = 64), and a first z-chunk starts at
    plane 0 where that saves a pass of the unrolled loop (z-chunks 21, 17, 15): bit-exact with the
    oracle, sweep counts and residuals included."""
    sc = S.small_scene(110, 64, 40, steps=4, seed=91, scheme=1, iterations=36, tol=1e-3, check_every=6,
                       obstacles=2, warm_start=1)
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc, report_div=1)
    sim.set_sweep_kernel(*kernel)
    for k in range(sc.steps):
        ost = o.step()
        sim.step(sc.dt)
        st = sim.stats()
        assert st.sweeps == ost.sweeps and st.resid_max == ost.resid_max and st.div_max == ost.div_max, k
        assert H.first_mismatch(sim.read_state(), H.oracle_state(o)) == "", k
    sim.close()


@pytest.mark.parametrize("dims,seed,kw", [
    ((20, 16, 18), 11, {}),
    ((110, 70, 40), 12, {"obstacles": 2, "sources": 2}),   # two x windows, several y windows
    ((33, 17, 29), 13, {"noise": 4.0}),                     # clamp-triggering velocities
    ((3, 40, 4), 14, {}),
    ((64, 64, 64), 15, {"obstacles": 3}),
])
@pytest.mark.parametrize("kernel", [(0, 0), (2, 0), (4, 0), (4, 5), (2, 9), (4, 137)])
def test_velocity_sweep_kernels_equal_oracle(gpu, dims, seed, kw, kernel):
    """The reference scheme's projection with one colour pass per launch (depth 0) or
    temporally blocked (depth 2 or 4 passes per pass over HBM, several z-chunks, windows along x
    and y, partial launches from odd pass counts) gives the oracle's bits on every field of both
    ping-pong buffers after every step."""
    # 7 iterations: 14 passes (depth 4: launches of 4, 4, 4, 2); 6: 12 passes, an odd launch
    # count that the plan splits (4, 4, 3, 1) so the result ends in the state's buffer
    sc = S.small_scene(*dims, steps=3, seed=seed, iterations=7 if seed % 2 else 6, **kw)
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc)
    sim.set_velocity_sweep(*kernel)
    for k in range(sc.steps):
        o.step()
        sim.step(sc.dt)
        msg = H.first_mismatch(sim.read_state(), H.oracle_state(o))
        assert msg == "", "step %d: %s" % (k, msg)
    sim.close()


def test_velocity_sweep_golden_ref80_and_scheme_switch(gpu):
    """The 80^3 workload with the blocked velocity sweep reproduces the reference's golden
    density hashes; switching a simulation that used it to the warm-started PRESSURE scheme
    afterwards starts its pressure from zero (the sweep's scratch is not taken for a pressure
    history), as the oracle does."""
    g = H.golden()["scenes"]["ref80"]
    sc = S.config_ref80(steps=100)
    sim = smk.from_scene(sc)
    sim.set_velocity_sweep(4, 0)
    out = np.zeros(sc.cell_shape, np.float32)
    for k in range(40):
        sim.simulate(out, sc.dt)
        if (k + 1) % 20 == 0:
            assert H.sha(out) == g["density_every_20"][str(k + 1)], k + 1
    sc2 = S.small_scene(30, 24, 26, steps=4, seed=77, iterations=9)
    o = O.OracleSim(sc2)
    a = smk.from_scene(sc2)
    a.set_velocity_sweep(2, 0)
    for _ in range(2):
        a.step(sc2.dt)
        o.step()
    a.set_params(projection=smk.PROJECT_PRESSURE, warm_start=1, tol=1e-3, check_every=3, max_sweeps=30)
    o.scheme = 1
    sc2.tol, sc2.check_every, sc2.iterations, sc2.warm_start = 1e-3, 3, 30, 1
    for k in range(2):
        a.step(sc2.dt)
        o.step()
        assert H.first_mismatch(a.read_state(), H.oracle_state(o)) == "", k
    sim.close()
    a.close()


def test_velocity_sweep_autotune_keeps_results(gpu):
    """The REFERENCE-scheme autotuner (one-pass or blocked velocity sweep, z-chunks) does not
    change results: after tuning, the steps still give the oracle's bits."""
    sc = S.small_scene(70, 44, 52, steps=3, seed=19, iterations=11, obstacles=2)
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc)
    depth, zchunk, us = sim.autotune()
    assert depth in (0, 2, 4) and us > 0
    assert sim.velocity_sweep()[0] == depth
    for k in range(sc.steps):
        o.step()
        sim.step(sc.dt)
        assert H.first_mismatch(sim.read_state(), H.oracle_state(o)) == "", k
    sim.close()


def test_jacobi_with_refinement_bit_exact_with_oracle(gpu):
    """The FP32 weighted-Jacobi solve followed by FP64-checked refinement rounds (the
    mixed-precision configuration's solver): the oracle's bits, sweep counts, rounds and FP64
    divergence, with graph replay."""
    sc = S.small_scene(26, 22, 24, steps=4, seed=37, scheme=1, iterations=30, tol=1e-5, check_every=5,
                       warm_start=1, solver=smk.SOLVER_JACOBI, omega=0.9)
    sc.refine, sc.refine_sweeps = 2, 8
    sim = smk.from_scene(sc, report_div=1)
    o = O.OracleSim(sc)
    for k in range(sc.steps):
        sim.step(sc.dt)
        so = o.step()
        sg = sim.stats()
        assert (sg.sweeps, sg.refine_rounds) == (so.sweeps, so.refine_rounds), k
        assert H.bits_equal(np.float32(sg.div64_max), np.float32(so.div64_max)), k
    assert H.first_mismatch(sim.read_state(), H.oracle_state(o)) == ""
    sim.close()
