"""The over-relaxation schedule of warm-started pressure solves (smk_params.omega_warm).

From the (omega_warm_after + 1)-th step after the pressure history started, warm-started solves
use omega_warm instead of omega.  The oracle applies the same rule step by step (oracle/oracle.py,
OracleSim); these tests hold every field of both buffers, the sweep counts and the residuals to
it bit for bit across the switch, for the blocked and the one-colour-pass kernels, in graph replay
with and without the device-side group loop and as direct launches, after a state write (which
restarts the history), and for members of a BRANCHES batch.
"""
import pytest

import smoke_simulation_gb300 as smk
from oracle import oracle as O
from smoke_simulation_gb300 import scenes as S
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _scene(omega_warm=1.75):
    sc = S.small_scene(40, 36, 44, steps=6, seed=29, scheme=1, iterations=150, tol=2e-4, check_every=6,
                       obstacles=1, warm_start=1)
    sc.omega_warm, sc.omega_warm_after = omega_warm, 2
    return sc


@pytest.mark.parametrize("mode", ["loop", "unrolled", "direct"])
@pytest.mark.parametrize("kernel", [(6, 17), (4, 11, 4), (0, 1)])
def test_omega_warm_equals_oracle(gpu, mode, kernel):
    sc = _scene()
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc, report_div=1)
    sim.set_sweep_kernel(*kernel)
    if mode == "unrolled":
        sim.set_graph_loops(False)
    if mode == "direct":
        sim.set_graphs(False)
    sweeps = []
    for k in range(sc.steps):
        ost = o.step()
        sim.step(sc.dt)
        st = sim.stats()
        assert st.sweeps == ost.sweeps and st.resid_max == ost.resid_max and st.div_max == ost.div_max, k
        assert st.converged == 1 and st.div_max <= 2e-4
        sweeps.append(st.sweeps)
        msg = H.first_mismatch(sim.read_state(), H.oracle_state(o))
        assert msg == "", "step %d: %s" % (k, msg)
    sim.close()
    # the first omega_warm_after steps are those of omega throughout; later ones differ
    plain = O.OracleSim(_scene(0.0))
    plain_sweeps = [plain.step().sweeps for _ in range(sc.steps)]
    assert plain_sweeps[:2] == sweeps[:2]
    assert H.first_mismatch(H.oracle_state(plain), H.oracle_state(o)) != ""


def test_omega_warm_restarts_after_state_write(gpu):
    """Writing a state restarts the pressure history: the next omega_warm_after steps use omega
    again (P from zero), as in a new simulation."""
    sc = _scene()
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc, report_div=1)
    sim.set_sweep_kernel(6, 17)
    for _ in range(3):
        o.step()
        sim.step(sc.dt)
    sim.write_state(H.oracle_state(o))
    o.reset_history()
    for k in range(3):
        ost = o.step()
        sim.step(sc.dt)
        assert sim.stats().sweeps == ost.sweeps, k
        assert H.first_mismatch(sim.read_state(), H.oracle_state(o)) == "", k
    sim.close()


def test_omega_warm_branches_batch_equals_alone(gpu):
    """BRANCHES batch members follow the schedule like single grids (each member's own history)."""
    scs = [_scene(), S.small_scene(30, 34, 28, steps=6, seed=31, scheme=1, iterations=150, tol=2e-4,
                                   check_every=6, warm_start=1)]
    scs[1].omega_warm, scs[1].omega_warm_after = 1.8, 1
    batch_sims = [smk.from_scene(sc) for sc in scs]
    oracles = [O.OracleSim(sc) for sc in scs]
    batch = smk.Batch(batch_sims, mode=smk.BATCH_BRANCHES)
    for k in range(5):
        batch.step([sc.dt for sc in scs])
        for o in oracles:
            o.step()
    for s, o in zip(batch_sims, oracles):
        assert H.first_mismatch(s.read_state(), H.oracle_state(o)) == ""
    batch.close()
    for s in batch_sims:
        s.close()


@pytest.mark.parametrize("blocked", [0, 37])
def test_omega_warm_grouped_batch_equals_oracle(gpu, blocked):
    """GROUPED batches (the cooperative colour-pass projection, and the blocked solve) rebuild a
    member's record when its over-relaxation switches; members stay bit-exact with the oracle."""
    scs = S.config_batched(count=4, steps=6, seed=9, lo=16, hi=36, scheme=1, iterations=120)
    for i, sc in enumerate(scs):
        sc.tol, sc.check_every, sc.warm_start = 2e-4, 6, 1
        sc.omega_warm, sc.omega_warm_after = 1.75, 1 + (i % 2)
    sims = [smk.from_scene(sc) for sc in scs]
    oracles = [O.OracleSim(sc) for sc in scs]
    batch = smk.Batch(sims, mode=smk.BATCH_GROUPED)
    batch.set_blocked(blocked)
    for k in range(5):
        batch.step([sc.dt for sc in scs])
        assert batch.info()[0] == smk.BATCH_GROUPED
        for o in oracles:
            o.step()
    for i, (s, o) in enumerate(zip(sims, oracles)):
        assert H.first_mismatch(s.read_state(), H.oracle_state(o)) == "", i
    batch.close()
    for s in sims:
        s.close()
