"""GPU test of smk_project_noalloc, the projection entry point that allocates nothing.

Callers that cannot allocate device memory when they need a projection (stream capture,
framework-owned or fixed-budget memory pools) pass their own velocity and mask buffers; the
library's scratch comes from one fixed device array.  This test calls the entry point through
the C ABI twice in a row and checks each result against the projection the existing entry
point (smk_step) computes on the same input, within the tolerances the parity tests use.
It lives in its own file, collected last, so a stop-at-first-failure run has already run
every other test; it passes alone in a fresh process and after the others.
"""
import ctypes as C

import numpy as np
import pytest

import smoke_simulation_gb300 as smk
from smoke_simulation_gb300 import scenes as S
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _scene(seed):
    sc = S.small_scene(40, 36, 44, steps=1, seed=seed, scheme=1, iterations=60, tol=1e-3,
                       check_every=5, obstacles=0, sources=0, boxes=0, noise=0.5)
    sc.mask = S.sphere_mask(40, 36, 44, [(20.0, 15.0, 22.0, 7.0)],
                            S.bernoulli_mask(40, 36, 44, 0.03, seed=seed))
    sc.gravity, sc.buoyancy, sc.clamp_mode = 0.0, 0.0, 2  # forcing is the identity
    return sc


def _existing_projection(sc):
    """Projected velocities from smk_step: with the identity forcing, buffer `now` holds
    exactly the projected field after one step (advection writes the other buffer)."""
    sim = smk.from_scene(sc, report_div=1)
    sim.step(sc.dt)
    st = sim.read_state()
    stats = sim.stats()
    sim.close()
    now = st["index_now"]
    return st["u"][now], st["v"][now], st["w"][now], stats


def _noalloc_projection(sc, gpu):
    import torch
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(device=gpu, dtype=dt)
    u = dev(sc.u0, torch.float32)
    v = dev(sc.v0, torch.float32)
    w = dev(sc.w0, torch.float32)
    m = dev(sc.mask, torch.uint8)
    p = smk.params_for_scene(sc)
    stats = smk.Stats()
    stream = torch.cuda.current_stream().cuda_stream
    rc = smk.lib().smk_project_noalloc(u.data_ptr(), v.data_ptr(), w.data_ptr(), m.data_ptr(),
                                       sc.nx, sc.ny, sc.nz, C.byref(p), C.byref(stats), stream)
    assert rc == 0, smk.lib().smk_project_noalloc_last_error()
    torch.cuda.synchronize()
    return u.cpu().numpy(), v.cpu().numpy(), w.cpu().numpy(), stats


def test_noalloc_projection_matches_existing_entry_point_twice(gpu):
    for seed in (71, 72):  # two calls in a row, different inputs, shared scratch
        sc = _scene(seed)
        ue, ve, we, se = _existing_projection(sc)
        un, vn, wn, sn = _noalloc_projection(sc, gpu)
        for got, want in ((un, ue), (vn, ve), (wn, we)):
            assert H.max_abs(got, want) <= H.VELOCITY_MAX_ABS
            assert H.rel_l2(got, want) <= H.VELOCITY_REL_L2
        assert sn.sweeps == se.sweeps and sn.converged == se.converged
        assert abs(sn.div_max - se.div_max) <= 1e-6


def test_noalloc_rejects_grids_beyond_its_scratch(gpu):
    import torch
    L = smk.lib()
    limit = L.smk_project_noalloc_max_elems()
    n = int(round(limit ** (1.0 / 3.0))) + 2  # (n+1)^3 > limit
    buf = torch.zeros(8, device=gpu)
    p = smk.default_params(projection=smk.PROJECT_PRESSURE)
    rc = L.smk_project_noalloc(buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), buf.data_ptr(),
                               n, n, n, C.byref(p), None, None)
    assert rc == 1
    assert b"exceeds the fixed scratch" in L.smk_project_noalloc_last_error()
