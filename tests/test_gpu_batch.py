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
