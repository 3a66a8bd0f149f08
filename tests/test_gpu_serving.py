"""GPU tests of the serving loop in both forms (per-request streams, one grouped step per tick):
continuous admission, overlap on the device, and each request's result identical alone and in
the mix."""
import numpy as np
import pytest

import smoke_simulation_gb300 as smk
from smoke_simulation_gb300 import scenes as S
from smoke_simulation_gb300 import serving as SV
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _requests():
    arr = SV.poisson_stream(7, rate=1e6, seed=21, lo=12, hi=40, steps_lo=3, steps_hi=9)
    return [(a.scene, a.steps) for a in arr]


def _alone(sc, steps):
    sim = smk.from_scene(sc)
    for _ in range(steps):
        sim.step(sc.dt)
    rho = sim.read_density()
    sim.close()
    return rho


@pytest.mark.parametrize("mode", [SV.SERVE_STREAMS, SV.SERVE_GROUPED])
def test_results_same_alone_and_in_the_mix(gpu, mode):
    reqs = _requests()
    srv = SV.Server(budget_bytes=10**10, max_active=3, mode=mode)  # 3 slots: later requests queue
    ids = [srv.submit(sc, steps) for sc, steps in reqs]
    seen_queue = False
    for _ in range(10000):
        active, queued = srv.tick()
        seen_queue = seen_queue or queued > 0
        assert active <= 3
        if active == 0 and queued == 0:
            break
    assert seen_queue
    for rid, (sc, steps) in zip(ids, reqs):
        state, done, err = srv.status(rid)
        assert state == SV.REQ_DONE and done == steps and err == 0
        assert H.bits_equal(srv.outputs[rid], _alone(sc, steps)), rid
    st = srv.stats()
    assert st.requests_completed == len(reqs)
    assert st.steps_completed == sum(s for _, s in reqs)
    assert 0 < st.p50_step_ms <= st.p99_step_ms <= st.max_step_ms
    srv.close()


@pytest.mark.parametrize("mode", [SV.SERVE_STREAMS, SV.SERVE_GROUPED])
def test_memory_budget_admission(gpu, mode):
    reqs = _requests()[:3]
    big = max(sc.nx for sc, _ in reqs)
    one = int(1.5 * ((big + 1 + 15) // 16 * 16) * (big + 1) ** 2 * 46) + (1 << 20)
    srv = SV.Server(budget_bytes=one, max_active=8, mode=mode)  # memory for about one request at a time
    ids = [srv.submit(sc, steps) for sc, steps in reqs]
    max_active = 0
    for _ in range(10000):
        active, queued = srv.tick()
        max_active = max(max_active, active)
        assert srv.stats().bytes_in_use <= one
        if active == 0 and queued == 0:
            break
    assert max_active <= 2
    for rid, (sc, steps) in zip(ids, reqs):
        assert srv.status(rid)[0] == SV.REQ_DONE
        assert H.bits_equal(srv.outputs[rid], _alone(sc, steps))
    srv.close()
