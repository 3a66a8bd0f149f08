"""GPU test of smk_project_noalloc, the projection entry point that allocates nothing.

Some callers cannot allocate device memory when they need a projection: an application whose
device memory belongs to its own pool allocator or a fixed budget, or a plugin called from a
per-frame callback where cudaMalloc's device-wide synchronisation would stall other work.  They
pass their own velocity and mask buffers; the library's scratch comes from one fixed device
array that every call shares.  This test calls the entry point through the C ABI several times
in a row -- including a smaller grid right after a larger one, so the shared array still holds
the larger grid's data, and a call without statistics (the stream-ordered path) -- and checks
every result bit for bit against the projection the existing entry point (smk_step) computes
on the same input.  It lives in its own file, collected last, so a stop-at-first-failure run
has already run every other test; it passes alone in a fresh process and after the others.
"""
import ctypes as C

import numpy as np
import pytest

import smoke_simulation_gb300 as smk
from smoke_simulation_gb300 import scenes as S
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _scene(dims, seed):
    nx, ny, nz = dims
    sc = S.small_scene(nx, ny, nz, steps=1, seed=seed, scheme=1, iterations=60, tol=1e-3,
                       check_every=5, obstacles=0, sources=0, boxes=0, noise=0.5)
    sc.mask = S.sphere_mask(nx, ny, nz, [(nx // 2, ny // 2 - 3, nz // 2, 7.0)],
                            S.bernoulli_mask(nx, ny, nz, 0.03, seed=seed))
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


def _noalloc_projection(sc, gpu, with_stats=True):
    import torch
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(device=gpu, dtype=dt)
    u = dev(sc.u0, torch.float32)
    v = dev(sc.v0, torch.float32)
    w = dev(sc.w0, torch.float32)
    m = dev(sc.mask, torch.uint8)
    p = smk.params_for_scene(sc)
    stats = smk.Stats() if with_stats else None
    stream = torch.cuda.current_stream().cuda_stream
    rc = smk.lib().smk_project_noalloc(u.data_ptr(), v.data_ptr(), w.data_ptr(), m.data_ptr(),
                                       sc.nx, sc.ny, sc.nz, C.byref(p),
                                       C.byref(stats) if with_stats else None, stream)
    assert rc == 0, smk.lib().smk_project_noalloc_last_error()
    torch.cuda.synchronize()
    return u.cpu().numpy(), v.cpu().numpy(), w.cpu().numpy(), stats


@pytest.mark.parametrize("with_stats", [True, False])
def test_noalloc_projection_equals_existing_entry_point(gpu, with_stats):
    # calls in a row on the shared scratch: two grids of one size, then a smaller grid right
    # after a larger one (the array still holds the larger grid's pressure, rhs and flags)
    for dims, seed in (((40, 36, 44), 71), ((40, 36, 44), 72), ((23, 19, 27), 73)):
        sc = _scene(dims, seed)
        ue, ve, we, se = _existing_projection(sc)
        un, vn, wn, sn = _noalloc_projection(sc, gpu, with_stats)
        for name, got, want in (("u", un, ue), ("v", vn, ve), ("w", wn, we)):
            assert H.bits_equal(got, want), (dims, name, H.max_abs(got, want))
        if with_stats:
            assert (sn.sweeps, sn.converged) == (se.sweeps, se.converged), dims
            assert sn.resid_max == se.resid_max and sn.div_max == se.div_max, dims


def test_noalloc_rejects_grids_beyond_its_scratch_and_other_schemes(gpu):
    import torch
    L = smk.lib()
    limit = L.smk_project_noalloc_max_elems()
    n = int(round(limit ** (1.0 / 3.0))) + 2  # (n+1)^3 > limit
    buf = torch.zeros(8, device=gpu)
    ptr = buf.data_ptr()
    p = smk.default_params(projection=smk.PROJECT_PRESSURE)
    rc = L.smk_project_noalloc(ptr, ptr, ptr, ptr, n, n, n, C.byref(p), None, None)
    assert rc == 1
    assert b"exceeds the fixed scratch" in L.smk_project_noalloc_last_error()
    big = 2**31 - 1  # (nx + 1) must not wrap around
    assert L.smk_project_noalloc(ptr, ptr, ptr, ptr, big, 1, 1, C.byref(p), None, None) == 1
    assert L.smk_project_noalloc(ptr, ptr, ptr, ptr, 1, 1, 70000, C.byref(p), None, None) == 1
    for bad in (dict(projection=smk.PROJECT_REFERENCE), dict(solver=smk.SOLVER_JACOBI),
                dict(omega=float("nan")), dict(omega=2.5), dict(tol=float("inf")), dict(refine=1)):
        q = smk.default_params(**{"projection": smk.PROJECT_PRESSURE, **bad})
        assert L.smk_project_noalloc(ptr, ptr, ptr, ptr, 4, 4, 4, C.byref(q), None, None) == 1, bad
