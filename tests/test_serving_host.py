"""Host-side failure handling of the serving loop (no GPU needed): invalid limits and requests
come back as status codes, and a request larger than the whole memory budget fails on its own
without blocking the queue."""
import ctypes as C

import pytest

from smoke_simulation_gb300 import scenes as S
from smoke_simulation_gb300 import serving as SV


def test_invalid_server_limits(smoke_lib):
    L = SV._bind()
    h = C.c_void_p()
    assert L.smk_server_create(0, 4, C.byref(h)) == 1
    assert L.smk_server_create(10**9, 0, C.byref(h)) == 1


def test_invalid_and_oversized_requests_fail_alone(smoke_lib):
    srv = SV.Server(budget_bytes=10**6, max_active=4)
    with pytest.raises(Exception):
        srv.submit(S.Scene("bad", 2, 2, 2, dt=0.05, steps=1))  # grid below 3^3
    sc = S.Scene("too_big", 64, 64, 64, dt=0.05, steps=3, scheme=1)
    rid = srv.submit(sc, keep_output=False)
    state, done, err = srv.status(rid)
    assert state == SV.REQ_FAILED and err == 3 and done == 0  # SMK_ERR_OOM, never admitted
    st = srv.stats()
    assert st.queued == 0 and st.active == 0 and st.bytes_in_use == 0
    srv.close()


def test_poisson_stream_is_deterministic():
    a = SV.poisson_stream(20)
    b = SV.poisson_stream(20)
    assert [x.t for x in a] == [x.t for x in b]
    assert [x.scene.nx for x in a] == [x.scene.nx for x in b]
    assert all(48 <= x.scene.nx <= 192 and 50 <= x.steps <= 500 for x in a)
    gaps = [a[i + 1].t - a[i].t for i in range(len(a) - 1)]
    assert 0.001 < sum(gaps) / len(gaps) < 0.02  # ~1/200 s


def test_non_finite_inputs_are_rejected(smoke_lib):
    srv = SV.Server(budget_bytes=10**9, max_active=4)
    sc = S.Scene("nan_sphere", 16, 16, 16, dt=0.05, steps=2, scheme=1)
    sc.spheres = [(8.0, float("nan"), 8.0, 3.0)]
    with pytest.raises(Exception):
        srv.submit(sc)
    sc2 = S.Scene("nan_param", 16, 16, 16, dt=0.05, steps=2, scheme=1)
    with pytest.raises(Exception):
        srv.submit(sc2, gravity=float("inf"))
    sc3 = S.Scene("nan_dt", 16, 16, 16, dt=float("nan"), steps=2, scheme=1)
    with pytest.raises(Exception):
        srv.submit(sc3)
    assert srv.stats().queued == 0
    srv.close()


def test_cancel_a_queued_request(smoke_lib):
    srv = SV.Server(budget_bytes=10**9, max_active=1)
    a = srv.submit(S.Scene("a", 16, 16, 16, dt=0.05, steps=2, scheme=1), keep_output=False)
    b = srv.submit(S.Scene("b", 16, 16, 16, dt=0.05, steps=2, scheme=1), keep_output=False)
    srv.cancel(b)
    assert srv.status(b)[0] == SV.REQ_CANCELLED
    assert srv.status(a)[0] == SV.REQ_QUEUED and srv.stats().queued == 1
    srv.cancel(b)  # cancelling twice does nothing
    with pytest.raises(Exception):
        srv.cancel(12345)
    srv.close()


def test_injected_allocation_failure_hook(smoke_lib):
    import smoke_simulation_gb300 as smk
    L = smk.lib()
    L.smk_inject_alloc_failures.argtypes = [C.c_int]
    assert L.smk_inject_alloc_failures(1) == 0
    h = C.c_void_p()
    assert L.smk_create(8, 8, 8, None, C.byref(h)) == 3  # SMK_ERR_OOM, before any device work
    assert not h.value
    assert L.smk_inject_alloc_failures(-1) == 1
    assert L.smk_inject_alloc_failures(0) == 0
