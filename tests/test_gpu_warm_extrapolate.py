"""The extrapolated warm start of the pressure solve (smk_params.warm_extrapolate).

Once two solves of a pressure history exist, a warm-started solve starts from the last pressure
extrapolated along its last change, P + a (P - P_before), in float arithmetic; the rhs pass keeps
the history in one more array.  The oracle applies the same rule step by step (oracle/oracle.py,
OracleSim).  These tests hold every field of both buffers, the sweep counts and the residuals to
it bit for bit: for the blocked kernels, the one-colour-pass kernel and the Jacobi solver, in
graph replay with and without the device-side group loop and as direct launches, across a state
write (which restarts the history), when the option is switched on between steps, with an
obstacle moving every step, for members of BRANCHES and GROUPED batches (the cooperative
colour passes and the blocked solve), and in the GROUPED serving form.
"""
import numpy as np
import pytest

import smoke_simulation_gb300 as smk
from oracle import oracle as O
from smoke_simulation_gb300 import scenes as S
from smoke_simulation_gb300 import serving as SV
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _scene(a=0.5, steps=8, **kw):
    sc = S.small_scene(40, 36, 44, steps=steps, seed=29, scheme=1, iterations=150, tol=2e-4, check_every=6,
                       obstacles=1, warm_start=1, **kw)
    sc.omega_warm, sc.omega_warm_after = 1.75, 2
    sc.warm_extrapolate = a
    return sc


def _check_step(sim, o, k):
    ost = o.step()
    st = sim.stats()
    assert st.sweeps == ost.sweeps and st.resid_max == ost.resid_max and st.div_max == ost.div_max, k
    msg = H.first_mismatch(sim.read_state(), H.oracle_state(o))
    assert msg == "", "step %d: %s" % (k, msg)
    return st


@pytest.mark.parametrize("mode", ["loop", "unrolled", "direct"])
@pytest.mark.parametrize("kernel", [(6, 17), (4, 11, 4), (2, 7), (0, 1)])
def test_extrapolated_warm_start_equals_oracle(gpu, mode, kernel):
    sc = _scene()
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc, report_div=1)
    sim.set_sweep_kernel(*kernel)
    if mode == "unrolled":
        sim.set_graph_loops(False)
    if mode == "direct":
        sim.set_graphs(False)
    for k in range(sc.steps):
        sim.step(sc.dt)
        st = _check_step(sim, o, k)
        assert st.converged == 1 and st.div_max <= 2e-4
    sim.close()
    # the extrapolation changes the iteration from the third step on
    plain = O.OracleSim(_scene(0.0)).run(sc.steps)
    assert H.first_mismatch(H.oracle_state(plain), H.oracle_state(o)) != ""


@pytest.mark.parametrize("tol", [0.0, 1e-3])
def test_extrapolated_warm_start_jacobi_equals_oracle(gpu, tol):
    sc = S.small_scene(33, 17, 29, steps=6, seed=41, scheme=1, iterations=37, tol=tol, check_every=5,
                       warm_start=1, solver=smk.SOLVER_JACOBI, omega=0.8)
    sc.warm_extrapolate = 0.5
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc, report_div=1)
    for k in range(sc.steps):
        sim.step(sc.dt)
        _check_step(sim, o, k)
    sim.close()


def test_extrapolated_warm_start_restarts_after_state_write(gpu):
    """Writing a state restarts the history: two plain warm starts (the first from zero), then
    extrapolated ones, as in a new simulation."""
    sc = _scene()
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc, report_div=1)
    for k in range(4):
        sim.step(sc.dt)
        _check_step(sim, o, k)
    sim.write_state(H.oracle_state(o))
    o.reset_history()
    for k in range(4):
        sim.step(sc.dt)
        _check_step(sim, o, k)
    sim.close()


def test_extrapolated_warm_start_switched_on_between_steps(gpu):
    """Switched on after three steps (smk_set_params): the next step saves the history and
    starts from the last pressure, the one after it extrapolates."""
    sc = _scene(0.0)
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc, report_div=1)
    for k in range(sc.steps):
        if k == 3:
            sc.warm_extrapolate = 0.5
            p = sim.params()
            p.warm_extrapolate = 0.5
            sim.set_params(p)
        sim.step(sc.dt)
        _check_step(sim, o, k)
    sim.close()


@pytest.mark.parametrize("graphs", [True, False])
def test_extrapolated_warm_start_moving_obstacle(gpu, graphs):
    """An obstacle moved every step changes which cells are projectable: the history keeps every
    cell's last pressure, and cells that become projectable start from its extrapolation."""
    sc = S.small_scene(28, 24, 30, steps=7, seed=41, scheme=1, iterations=60, tol=1e-4, check_every=5,
                       obstacles=0, warm_start=1)
    sc.warm_extrapolate = 0.5
    sc.obstacles = [(10.0, 12.0, 15.0, 0.0, 0.0, 0.0, 4.0)]
    sim = smk.from_scene(sc, report_div=1)
    sim.set_graphs(graphs)
    o = O.OracleSim(sc)
    oid = len(sc.boxes) + len(sc.spheres)
    for k in range(sc.steps):
        pos = (10.0 + 1.3 * (k + 1), 12.0, 15.0 - 0.7 * (k + 1))
        sim.update_object_pos(oid, *pos)
        o.obstacles[0, :3] = pos
        sim.step(sc.dt)
        _check_step(sim, o, k)
    sim.close()


@pytest.mark.parametrize("mode,blocked", [(smk.BATCH_BRANCHES, 0), (smk.BATCH_GROUPED, 0),
                                          (smk.BATCH_GROUPED, 37)])
def test_extrapolated_warm_start_in_batches(gpu, mode, blocked):
    """BRANCHES and GROUPED batches (the cooperative colour passes and the blocked solve) step
    each member as the oracle does alone: members with different factors, one without."""
    scs = [_scene(), S.small_scene(30, 34, 28, steps=6, seed=31, scheme=1, iterations=150, tol=2e-4,
                                   check_every=6, warm_start=1),
           S.small_scene(24, 20, 26, steps=6, seed=33, scheme=1, iterations=150, tol=2e-4, check_every=6,
                         warm_start=1)]
    scs[1].warm_extrapolate = 0.35
    sims = [smk.from_scene(sc) for sc in scs]
    oracles = [O.OracleSim(sc) for sc in scs]
    batch = smk.Batch(sims, mode=mode)
    if blocked:
        batch.set_blocked(blocked)
    for _ in range(5):
        batch.step([sc.dt for sc in scs])
        assert batch.info()[0] == mode
        for o in oracles:
            o.step()
    for i, (s, o) in enumerate(zip(sims, oracles)):
        assert H.first_mismatch(s.read_state(), H.oracle_state(o)) == "", i
    batch.close()
    for s in sims:
        s.close()


def test_grouped_serving_with_an_extrapolating_request(gpu):
    """In the GROUPED serving form a request with the extrapolated warm start is stepped in the
    grouped ticks with the others; every result equals the request alone."""
    arr = SV.poisson_stream(4, rate=1e6, seed=21, lo=12, hi=40, steps_lo=3, steps_hi=9)
    reqs = [(a.scene, a.steps) for a in arr]
    reqs[1][0].warm_extrapolate = 0.5
    srv = SV.Server(budget_bytes=10**10, max_active=4, mode=SV.SERVE_GROUPED)
    ids = [srv.submit(sc, steps) for sc, steps in reqs]
    for _ in range(10000):
        active, queued = srv.tick()
        if active == 0 and queued == 0:
            break
    for rid, (sc, steps) in zip(ids, reqs):
        assert srv.status(rid)[0] == SV.REQ_DONE
        sim = smk.from_scene(sc)
        for _ in range(steps):
            sim.step(sc.dt)
        assert H.bits_equal(srv.outputs[rid], sim.read_density()), rid
        sim.close()
    srv.close()


def test_warm_extrapolate_validated(gpu):
    sim = smk.Simulation(8, 8, 8)
    p = sim.params()
    for bad in (-0.1, 1.5, float("nan")):
        p.warm_extrapolate = bad
        with pytest.raises(smk.SmokeError):
            sim.set_params(p)
    sim.close()
