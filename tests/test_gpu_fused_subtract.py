"""The gradient subtract fused into the last blocked sweep launch (PRESSURE scheme, FP32;
smk_set_fused_subtract, off by default).

A face moves inside the launch that applies the solve's last colour pass, by the thread that
owns the face's cell of that colour, with the operands of that cell's last update.  These tests
hold the result bit for bit to the oracle's separate subtract (oracle/smoke_oracle.cpp, the
restatement of smokeSimulation.cu:356-394 in pressure form) and check from the step statistics
that the fused path ran where it should and not where it cannot: every depth and patch height,
z-chunks cut inside the grid, edge windows, fixed sweep counts, the sweep cap with a last group
of one launch (not fusable) and of several, graphs with and without the device-side group loop,
and direct launches.  Under the tolerance rule the solve ends on the input of a check launch,
which only the end of that launch decides: the subtract then stays a pass of its own.
"""
import pytest

import smoke_simulation_gb300 as smk
from oracle import oracle as O
from smoke_simulation_gb300 import scenes as S
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _expect_fused(depth, iterations, check, tol, converged):
    """1 when the solve's last launch is known on the host and is a full launch of `depth`
    passes (a group's launches apply a shorter one first): with no tolerance, one group of every
    sweep; with one, only when the cap ended the solve, after a last group (of `check` sweeps,
    cut at the cap) of two launches or more, the first being its check launch."""
    if tol <= 0:
        return 1 if 2 * iterations >= depth else 0
    if converged:
        return 0
    passes = 2 * (iterations - ((iterations - 1) // check) * check)
    return 1 if passes > depth else 0


@pytest.mark.parametrize("dims,seed", [((20, 16, 18), 11), ((33, 17, 29), 41), ((70, 38, 45), 42)])
@pytest.mark.parametrize("tol,check", [(0.0, 5), (1e-3, 5), (1e-3, 2)])
@pytest.mark.parametrize("kernel", [(2, 7), (4, 32), (6, 5), (6, 117), (4, 3, 4), (4, 32, 4), (6, 21)])
def test_fused_subtract_equals_oracle(gpu, dims, seed, tol, check, kernel):
    sc = S.small_scene(*dims, steps=4, seed=seed, scheme=1, iterations=41, tol=tol,
                       check_every=check, obstacles=2, warm_start=1)
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc, report_div=1)
    sim.set_sweep_kernel(*kernel)
    sim.set_fused_subtract(True)
    for k in range(sc.steps):
        ost = o.step()
        sim.step(sc.dt)
        st = sim.stats()
        assert st.sweeps == ost.sweeps and st.div_max == ost.div_max, (k, st.sweeps, ost.sweeps)
        want = _expect_fused(kernel[0], sc.iterations, check, tol, st.converged)
        assert st.subtract_fused == want, (k, kernel, check, st.sweeps)
        msg = H.first_mismatch(sim.read_state(), H.oracle_state(o))
        assert msg == "", "step %d: %s" % (k, msg)
    sim.close()


@pytest.mark.parametrize("iterations,check,fused", [(40, 5, 1), (41, 5, 0)])
def test_fused_subtract_at_the_sweep_cap(gpu, iterations, check, fused):
    """A tolerance the cap stops first: the last group ends at the cap.  40 sweeps in groups of
    5 end with a group of two launches (fused, known on the host); 41 end with a group of one
    sweep, a single launch (the separate subtract runs)."""
    sc = S.small_scene(36, 30, 40, steps=3, seed=7, scheme=1, iterations=iterations, tol=1e-12,
                       check_every=check, obstacles=1)
    o = O.OracleSim(sc)
    sim = smk.from_scene(sc, report_div=1)
    sim.set_sweep_kernel(6, 17)
    sim.set_fused_subtract(True)
    for k in range(sc.steps):
        ost = o.step()
        sim.step(sc.dt)
        st = sim.stats()
        assert st.sweeps == ost.sweeps == iterations and not st.converged
        assert st.subtract_fused == fused
        assert H.first_mismatch(sim.read_state(), H.oracle_state(o)) == "", k
    sim.close()


@pytest.mark.parametrize("tol,iterations,fused", [(1e-12, 60, 1), (2e-4, 150, 0)])
@pytest.mark.parametrize("depth,check,rows", [(6, 6, 2), (4, 6, 2), (4, 6, 4), (2, 5, 2)])
def test_fused_subtract_graph_loop_unrolled_direct(gpu, depth, check, rows, tol, iterations, fused):
    """Inside the device-side group loop, in an unrolled graph and as direct launches: the same
    bits as the oracle, fused when the cap ends the solve (tol 1e-12, 60 sweeps in groups whose
    last holds two launches or more) and a separate pass when the tolerance rule does (2e-4,
    well within the 150-sweep cap)."""
    sc = S.small_scene(40, 36, 44, steps=4, seed=29, scheme=1, iterations=iterations, tol=tol,
                       check_every=check, warm_start=1)
    o = O.OracleSim(sc)
    sims = [smk.from_scene(sc, report_div=1) for _ in range(3)]
    for s in sims:
        s.set_sweep_kernel(depth, 17, rows)
        s.set_fused_subtract(True)
    sims[1].set_graph_loops(False)
    sims[2].set_graphs(False)
    for k in range(sc.steps):
        ost = o.step()
        for s in sims:
            s.step(sc.dt)
            st = s.stats()
            assert st.sweeps == ost.sweeps and st.converged == 1 - fused and st.subtract_fused == fused, k
    for s in sims:
        assert H.first_mismatch(s.read_state(), H.oracle_state(o)) == ""
        s.close()


def test_no_fusion_by_default_nor_for_bf16_jacobi_and_one_pass_kernels(gpu):
    """The switch is off by default; and forms whose subtract stays a pass of its own when it is
    on: BF16 velocity storage (the subtract also writes the FP32 copy of the projected faces),
    the Jacobi solver, and one colour pass per launch."""
    sc = S.small_scene(32, 28, 30, steps=2, seed=3, scheme=1, iterations=20, tol=1e-3, check_every=5)
    cases = [dict(storage=smk.STORAGE_BF16_VEL), dict(solver=smk.SOLVER_JACOBI, omega=0.8), dict(), None]
    for i, over in enumerate(cases):
        sim = smk.from_scene(sc, **(over or {}))
        if over is not None:
            sim.set_fused_subtract(True)
        if i == 2:
            sim.set_sweep_kernel(0, 1)
        for _ in range(sc.steps):
            sim.step(sc.dt)
            assert sim.stats().subtract_fused == 0, over
        sim.close()
