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


@pytest.mark.parametrize("mode,blocked", [(SV.SERVE_STREAMS, None), (SV.SERVE_GROUPED, None),
                                          (SV.SERVE_GROUPED, 0), (SV.SERVE_GROUPED, 17)])
def test_results_same_alone_and_in_the_mix(gpu, mode, blocked):
    """Each request's result is the same alone and in the mix, in both serving forms, the
    grouped one with its default (the blocked solve, 137-plane z-chunks), the colour passes (0)
    and 17-plane z-chunks."""
    reqs = _requests()
    srv = SV.Server(budget_bytes=10**10, max_active=3, mode=mode)  # 3 slots: later requests queue
    if blocked is not None:
        srv.set_blocked(blocked)
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


def _drain(srv):
    for _ in range(100000):
        active, queued = srv.tick()
        if active == 0 and queued == 0:
            return
    raise RuntimeError("server did not drain")


@pytest.mark.parametrize("mode", [SV.SERVE_STREAMS, SV.SERVE_GROUPED])
def test_injected_allocation_failure_fails_one_request(gpu, mode):
    """A device allocation that fails at admission (injected on the host) fails that request
    alone; the others run and give their results alone."""
    reqs = _requests()[:3]
    srv = SV.Server(budget_bytes=10**10, max_active=4, mode=mode)
    smk.lib().smk_inject_alloc_failures(1)
    ids = [srv.submit(sc, steps) for sc, steps in reqs]
    _drain(srv)
    smk.lib().smk_inject_alloc_failures(0)
    states = [srv.status(i) for i in ids]
    assert states[0][0] == SV.REQ_FAILED and states[0][2] == 3  # SMK_ERR_OOM
    for rid, (sc, steps), st in list(zip(ids, reqs, states))[1:]:
        assert st[0] == SV.REQ_DONE
        assert H.bits_equal(srv.outputs[rid], _alone(sc, steps))
    assert srv.stats().bytes_in_use == 0
    srv.close()


@pytest.mark.parametrize("mode", [SV.SERVE_STREAMS, SV.SERVE_GROUPED])
def test_cancel_active_and_queued_requests(gpu, mode):
    reqs = [(sc, steps + 20) for sc, steps in _requests()[:4]]
    srv = SV.Server(budget_bytes=10**10, max_active=2, mode=mode)
    ids = [srv.submit(sc, steps) for sc, steps in reqs]
    for _ in range(3):
        srv.tick()
    assert srv.status(ids[0])[0] == SV.REQ_ACTIVE and srv.status(ids[3])[0] == SV.REQ_QUEUED
    srv.cancel(ids[0])
    srv.cancel(ids[3])
    _drain(srv)
    st0, done0, _ = srv.status(ids[0])
    assert st0 == SV.REQ_CANCELLED and 0 < done0 < reqs[0][1]
    assert srv.status(ids[3])[:2] == (SV.REQ_CANCELLED, 0)
    for rid, (sc, steps) in zip(ids[1:3], reqs[1:3]):
        assert srv.status(rid)[0] == SV.REQ_DONE
        assert H.bits_equal(srv.outputs[rid], _alone(sc, steps))
    assert srv.stats().bytes_in_use == 0
    srv.close()


@pytest.mark.parametrize("mode", [SV.SERVE_STREAMS, SV.SERVE_GROUPED])
def test_device_resident_outputs(gpu, mode):
    """Final densities handed to device buffers (stream-ordered device copies, no host copy)
    are the results each request gives alone."""
    import torch
    reqs = _requests()[:4]
    srv = SV.Server(budget_bytes=10**10, max_active=2, mode=mode)
    outs = [torch.full(tuple(sc.cell_shape), -1.0, dtype=torch.float32, device="cuda") for sc, _ in reqs]
    ids = [srv.submit(sc, steps, out_device=o) for (sc, steps), o in zip(reqs, outs)]
    _drain(srv)
    torch.cuda.synchronize()
    for rid, (sc, steps), o in zip(ids, reqs, outs):
        assert srv.status(rid)[0] == SV.REQ_DONE
        assert H.bits_equal(o.cpu().numpy(), _alone(sc, steps))
    srv.close()
