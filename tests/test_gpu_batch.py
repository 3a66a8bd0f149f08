"""GPU tests of batches: many uneven grids stepped as one CUDA graph give exactly the results
each grid gives alone (and the oracle's, for the pressure scheme)."""
import numpy as np
import pytest

import smoke_simulation_gb300 as smk
from oracle import oracle as O
from smoke_simulation_gb300 import scenes as S
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _scenes():
    scs = S.config_batched(count=6, steps=5, seed=9, lo=12, hi=40, scheme=1, iterations=24)
    for i, sc in enumerate(scs):
        sc.tol, sc.check_every = 1e-3, 4
        sc.u0, sc.v0, sc.w0 = S.noise_velocity(sc.face_shape, 0.3, seed=100 + i)
    scs[2].scheme = 0  # one member on the reference scheme
    scs[2].iterations = 10
    return scs


def test_batch_equals_alone_and_oracle(gpu):
    scs = _scenes()
    dts = [sc.dt * (1.0 + 0.1 * i) for i, sc in enumerate(scs)]
    batch_sims = [smk.from_scene(sc, report_div=1) for sc in scs]
    alone = [smk.from_scene(sc, report_div=1) for sc in scs]
    for s in batch_sims:
        s.autotune()
    for s in alone:
        s.set_graphs(False)
        s.set_sweep_kernel(0, 1)
    oracles = [O.OracleSim(sc) for sc in scs]
    batch = smk.Batch(batch_sims)
    for k in range(5):
        if k == 3:  # a mask change on one member: that batch step runs directly
            m = scs[1].initial_mask().copy()
            m[2:5, 2:5, 2:5] = 0
            batch_sims[1].set_mask(m)
            alone[1].set_mask(m)
            oracles[1].s[...] = m
        batch.step(dts)
        for s, dt in zip(alone, dts):
            s.step(dt)
        for o, dt in zip(oracles, dts):
            o.step(dt)
    for i in range(len(scs)):
        a = batch_sims[i].read_state()
        b = alone[i].read_state()
        assert H.first_mismatch(a, b) == "", i
        assert H.first_mismatch(a, H.oracle_state(oracles[i])) == "", i
        assert batch_sims[i].stats().sweeps == alone[i].stats().sweeps
    batch.close()
    for s in batch_sims + alone:
        s.close()


def test_batch_rejects_empty(gpu):
    import ctypes as C
    h = C.c_void_p()
    assert smk.lib().smk_batch_create(0, None, C.byref(h)) == 1


def _grouped_scenes(count=7, seed=11):
    scs = S.config_batched(count=count, steps=6, seed=seed, lo=8, hi=44, scheme=1, iterations=30)
    for i, sc in enumerate(scs):
        sc.u0, sc.v0, sc.w0 = S.noise_velocity(sc.face_shape, 0.3, seed=200 + i)
        # a mix of tolerance rules, group sizes and pressure starts across the members
        sc.tol = (1e-3, 0.0, 1e-4, 5e-4)[i % 4]
        sc.check_every = (4, 1, 6, 3)[i % 4]
        sc.warm_start = i % 2
    scs[1].iterations = 0  # a member without sweeps
    return scs


def _step_all(batch, alone, oracles, dts, steps, mask_step=None, scs=None, batch_sims=None):
    for k in range(steps):
        if k == mask_step:
            m = scs[1].initial_mask().copy()
            m[2:4, 2:4, 2:4] = 0
            batch_sims[1].set_mask(m)
            alone[1].set_mask(m)
            if oracles:
                oracles[1].s[...] = m
        batch.step(dts)
        for s, dt in zip(alone, dts):
            s.step(dt)
        for o, dt in zip(oracles or [], dts):
            o.step(dt)


def test_grouped_equals_alone_and_oracle(gpu):
    """One persistent launch per stage over 7 uneven grids (8..44 cells per side, per-member dt,
    tolerance, group size and pressure start) is bit-identical to each grid stepped alone and
    to the oracle, including a step with a mask change (run per member) in between."""
    scs = _grouped_scenes()
    dts = [sc.dt * (1.0 + 0.05 * i) for i, sc in enumerate(scs)]
    batch_sims = [smk.from_scene(sc, report_div=1) for sc in scs]
    alone = [smk.from_scene(sc, report_div=1) for sc in scs]
    for s in alone:
        s.set_graphs(False)
        s.autotune()
    oracles = [O.OracleSim(sc) for sc in scs]
    batch = smk.Batch(batch_sims, mode=smk.BATCH_GROUPED)
    _step_all(batch, alone, oracles, dts, 6, mask_step=3, scs=scs, batch_sims=batch_sims)
    mode, launches = batch.info()
    assert mode == smk.BATCH_GROUPED
    for i in range(len(scs)):
        a = batch_sims[i].read_state()
        assert H.first_mismatch(a, alone[i].read_state()) == "", i
        assert H.first_mismatch(a, H.oracle_state(oracles[i])) == "", i
        sa, sb = batch_sims[i].stats(), alone[i].stats()
        assert (sa.sweeps, sa.converged, sa.div_max, sa.resid_max) == (sb.sweeps, sb.converged, sb.div_max,
                                                                       sb.resid_max), i
    batch.close()
    for s in batch_sims + alone:
        s.close()


def test_grouped_launches_per_step_do_not_grow_with_members(gpu):
    scs = _grouped_scenes(count=12, seed=5)
    sims = [smk.from_scene(sc) for sc in scs]
    batch = smk.Batch(sims, mode=smk.BATCH_GROUPED)
    batch.step(0.05)  # first step: mask upload, per member
    _, l0 = batch.info()
    for _ in range(4):
        batch.step(0.05)
    mode, l1 = batch.info()
    assert mode == smk.BATCH_GROUPED
    assert (l1 - l0) == 4 * 5  # emitters, forcing, projection, two advections
    batch.close()
    for s in sims:
        s.close()


@pytest.mark.parametrize("storage", [smk.STORAGE_BF16, smk.STORAGE_BF16_VEL])
def test_grouped_bf16_members_equal_alone(gpu, storage):
    scs = _grouped_scenes(count=5, seed=13)
    batch_sims = [smk.from_scene(sc, report_div=1, storage=storage) for sc in scs]
    alone = [smk.from_scene(sc, report_div=1, storage=storage) for sc in scs]
    batch = smk.Batch(batch_sims, mode=smk.BATCH_GROUPED)
    _step_all(batch, alone, None, [0.05] * len(scs), 5)
    assert batch.info()[0] == smk.BATCH_GROUPED
    for i in range(len(scs)):
        assert H.first_mismatch(batch_sims[i].read_state(), alone[i].read_state()) == "", i
        assert batch_sims[i].stats().div_max == alone[i].stats().div_max
    batch.close()
    for s in batch_sims + alone:
        s.close()


def test_grouped_graphs_autotune_and_parity_changes_do_not_change_results(gpu):
    """Graph replay on/off, a tuned CTA count, and a member stepped on its own between batch
    steps (its ping-pong parity then differs from the others') leave the results unchanged."""
    scs = _grouped_scenes(count=6, seed=17)
    runs = []
    for variant in ("graphs", "direct", "tuned"):
        sims = [smk.from_scene(sc, report_div=1) for sc in scs]
        batch = smk.Batch(sims, mode=smk.BATCH_GROUPED)
        if variant == "direct":
            batch.set_graphs(False)
        for k in range(6):
            if k == 2 and variant == "tuned":
                c, us = batch.autotune()
                assert c >= 1 and us > 0
            if k == 3:
                sims[0].step(0.05)  # member 0 alone: parities now differ across the batch
            batch.step(0.05)
        assert batch.info()[0] == smk.BATCH_GROUPED
        runs.append([s.read_state() for s in sims])
        batch.close()
        for s in sims:
            s.close()
    for i in range(len(scs)):
        assert H.first_mismatch(runs[0][i], runs[1][i]) == "", i
        assert H.first_mismatch(runs[0][i], runs[2][i]) == "", i


def test_grouped_mode_rejects_reference_scheme(gpu):
    scs = _scenes()
    sims = [smk.from_scene(sc) for sc in scs]
    batch = smk.Batch(sims)
    with pytest.raises(smk.SmokeError):
        batch.set_mode(smk.BATCH_GROUPED)
    batch.step(0.05)
    batch.step(0.05)
    assert batch.info()[0] == smk.BATCH_BRANCHES
    batch.close()
    for s in sims:
        s.close()


@pytest.mark.parametrize("sched", [(1, 1, 1 << 20), (0, 4, 0), (2, 16, 300_000), (3, 7, 1 << 30)])
def test_grouped_schedules_do_not_change_results(gpu, sched):
    """CTAs per SM, z planes per tile and solve waves (1 MB, 300 kB: nearly one wave per grid)
    change only the speed."""
    scs = _grouped_scenes(count=6, seed=23)
    ref = [smk.from_scene(sc, report_div=1) for sc in scs]
    sims = [smk.from_scene(sc, report_div=1) for sc in scs]
    batch = smk.Batch(sims, mode=smk.BATCH_GROUPED)
    batch.set_schedule(*sched)
    assert batch.schedule() == sched
    for _ in range(4):
        batch.step(0.05)
        for s in ref:
            s.step(0.05)
    for i in range(len(scs)):
        assert H.first_mismatch(sims[i].read_state(), ref[i].read_state()) == "", i
        assert sims[i].stats().sweeps == ref[i].stats().sweeps
    batch.close()
    for s in sims + ref:
        s.close()


def _blocked_scenes(count=7, seed=31, lo=8, hi=70):
    scs = S.config_batched(count=count, steps=6, seed=seed, lo=lo, hi=hi, scheme=1, iterations=40)
    for i, sc in enumerate(scs):
        sc.u0, sc.v0, sc.w0 = S.noise_velocity(sc.face_shape, 0.3, seed=300 + i)
        sc.tol, sc.check_every = 2e-4, 6  # one group size and sweep cap for every member
        sc.warm_start = i % 2
    return scs


@pytest.mark.parametrize("zchunk,graphs,storage", [(17, True, smk.STORAGE_F32), (5, False, smk.STORAGE_F32),
                                                   (64, True, smk.STORAGE_BF16_VEL)])
def test_grouped_blocked_solve_equals_alone(gpu, zchunk, graphs, storage):
    """The grouped form with the blocked solve (depth-6 launches over every member's tiles, the
    tolerance groups as a device-side loop when captured, direct launches otherwise) is
    bit-identical to each grid stepped alone, sweep counts and residuals included, with warm
    and cold pressure starts, BF16 velocity storage and a step where the members' ping-pong
    parities differ."""
    scs = _blocked_scenes()
    batch_sims = [smk.from_scene(sc, report_div=1, storage=storage) for sc in scs]
    alone = [smk.from_scene(sc, report_div=1, storage=storage) for sc in scs]
    for s in alone:
        s.set_graphs(False)
        s.set_sweep_kernel(0, 1)
    batch = smk.Batch(batch_sims, mode=smk.BATCH_GROUPED)
    batch.set_blocked(zchunk)
    assert batch.blocked() == zchunk
    if not graphs:
        batch.set_graphs(False)
    for k in range(6):
        if k == 3:
            batch_sims[0].step(0.05)
            alone[0].step(0.05)
        batch.step(0.05)
        for s in alone:
            s.step(0.05)
    assert batch.info()[0] == smk.BATCH_GROUPED
    for i in range(len(scs)):
        assert H.first_mismatch(batch_sims[i].read_state(), alone[i].read_state()) == "", i
        sa, sb = batch_sims[i].stats(), alone[i].stats()
        assert (sa.sweeps, sa.converged, sa.div_max, sa.resid_max) == (sb.sweeps, sb.converged, sb.div_max,
                                                                       sb.resid_max), i
    batch.close()
    for s in batch_sims + alone:
        s.close()


def test_grouped_blocked_needs_shared_groups(gpu):
    """Members with different tolerance group sizes fall back to the colour-pass solve (same
    results); the autotuner may pick the blocked solve only when every member can use it."""
    scs = _grouped_scenes(count=5, seed=37)  # mixed group sizes and tolerances
    ref = [smk.from_scene(sc, report_div=1) for sc in scs]
    sims = [smk.from_scene(sc, report_div=1) for sc in scs]
    batch = smk.Batch(sims, mode=smk.BATCH_GROUPED)
    batch.set_blocked(17)
    for _ in range(3):
        batch.step(0.05)
        for s in ref:
            s.step(0.05)
    for i in range(len(scs)):
        assert H.first_mismatch(sims[i].read_state(), ref[i].read_state()) == "", i
    batch.close()
    scs2 = _blocked_scenes(count=5, seed=41, lo=20, hi=60)
    sims2 = [smk.from_scene(sc, report_div=1) for sc in scs2]
    ref2 = [smk.from_scene(sc, report_div=1) for sc in scs2]
    b2 = smk.Batch(sims2, mode=smk.BATCH_GROUPED)
    b2.step(0.05)
    for s in ref2:
        s.step(0.05)
    c, us = b2.autotune()
    assert us > 0 and (c == 0) == (b2.blocked() > 0)
    for _ in range(3):
        b2.step(0.05)
        for s in ref2:
            s.step(0.05)
    for i in range(len(scs2)):
        assert H.first_mismatch(sims2[i].read_state(), ref2[i].read_state()) == "", i
    b2.close()
    for s in sims + ref + sims2 + ref2:
        s.close()


@pytest.mark.parametrize("storage", [smk.STORAGE_F32, smk.STORAGE_BF16_VEL, smk.STORAGE_BF16])
def test_grouped_vector_stages_equal_per_cell(gpu, storage):
    """A grouped batch whose members use the 4-wide stage bodies gives the bits of the same batch
    with one cell per thread (grid sides 8..44: rows ending anywhere in a group of four)."""
    scs = _grouped_scenes(count=5, seed=19)
    a = [smk.from_scene(sc, report_div=1, storage=storage) for sc in scs]
    b = [smk.from_scene(sc, report_div=1, storage=storage) for sc in scs]
    for s in b:
        s.set_vector_stages(False)
    ba = smk.Batch(a, mode=smk.BATCH_GROUPED)
    bb = smk.Batch(b, mode=smk.BATCH_GROUPED)
    for _ in range(5):
        ba.step([0.05] * len(scs))
        bb.step([0.05] * len(scs))
    for i in range(len(scs)):
        assert H.first_mismatch(a[i].read_state(), b[i].read_state()) == "", i
        assert a[i].stats().div_max == b[i].stats().div_max, i
    ba.close()
    bb.close()
    for s in a + b:
        s.close()


@pytest.mark.parametrize("barrier", [1, 3])
def test_grid_barrier_wait_runs_out_and_recovers(gpu, barrier):
    """A grid-barrier wait of the cooperative grouped projection that runs out (CTA 0 made to
    skip one arrival, waits shortened to 20 ms): every CTA leaves the kernel, every member's next
    synchronisation reports SMK_ERR_TIMEOUT, and the context stays usable -- a new batch of fresh
    members then gives, bit for bit, what the same grids give stepped alone."""
    import ctypes as C
    scs = [sc for i, sc in enumerate(_scenes()) if i != 2]  # PRESSURE members only (GROUPED)
    sims = [smk.from_scene(sc, report_div=1) for sc in scs]
    batch = smk.Batch(sims, mode=smk.BATCH_GROUPED)
    batch.set_graphs(False)
    batch.set_schedule(0, 4, 0)  # the cooperative colour-pass solve: several grid barriers
    batch.step(scs[0].dt)
    for s in sims:
        s.sync()
    L = smk.lib()
    L.smk_inject_barrier_timeout.argtypes = [C.c_int, C.c_int]
    L.smk_barrier_timeout_report.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
    assert L.smk_inject_barrier_timeout(barrier, 20) == 0
    batch.step(scs[0].dt)
    left, ctas = C.c_int(), C.c_int()
    assert L.smk_barrier_timeout_report(C.byref(left), C.byref(ctas)) == 0
    assert ctas.value > 0 and left.value == ctas.value
    for s in sims:
        with pytest.raises(smk.SmokeError) as e:
            s.sync()
        assert e.value.code == smk.ERR_TIMEOUT
        s.sync()  # reported once; the context is usable
    batch.close()
    for s in sims:
        s.close()
    # fresh members on the same context: batched == alone, bit for bit
    fresh = [smk.from_scene(sc, report_div=1) for sc in scs]
    alone = [smk.from_scene(sc, report_div=1) for sc in scs]
    b2 = smk.Batch(fresh, mode=smk.BATCH_GROUPED)
    for _ in range(3):
        b2.step(scs[0].dt)
        for s, sc in zip(alone, scs):
            s.step(sc.dt)
    for a, b in zip(fresh, alone):
        assert H.first_mismatch(a.read_state(), b.read_state()) == ""
    b2.close()
    for s in fresh + alone:
        s.close()
