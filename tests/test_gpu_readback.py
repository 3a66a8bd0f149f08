"""smk_simulate into page-locked memory: the density copied to the host slab by slab inside the
step, while the rest of the advection computes (smk_set_readback_slabs).

The advection then runs in z-slabs, and every slab's planes are copied as soon as they are
final.  These tests hold the returned density and the whole state bit for bit to a twin
simulation that steps and then copies, across slab counts (the automatic count, one slab, a
count that does not divide the velocity chunks, more slabs than chunks), grid depths that are and are not
multiples of the chunk size, both projection schemes, graph replay and direct launches, the
BF16 velocity storage (FP32 density: overlapped) and the all-BF16 storage (the copy after the
step), and a step that runs uncaptured (an object moved).  The 80^3 configuration through
simulate() into pinned memory gives the golden density hashes of the reference's simulate().
"""
import numpy as np
import pytest

import smoke_simulation_gb300 as smk
from smoke_simulation_gb300 import scenes as S
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _pinned(shape):
    torch = pytest.importorskip("torch")
    return torch.empty(tuple(shape), dtype=torch.float32, pin_memory=True).numpy()


@pytest.mark.parametrize("dims,seed", [((20, 16, 18), 11), ((33, 17, 29), 41), ((24, 20, 130), 5),
                                       ((40, 36, 49), 29), ((9, 8, 7), 3)])
@pytest.mark.parametrize("slabs", [-1, 1, 3, 8, 64])
@pytest.mark.parametrize("scheme", [0, 1])
def test_overlapped_readback_equals_copy_after_step(gpu, dims, seed, slabs, scheme):
    kw = dict(iterations=30) if scheme == 0 else dict(iterations=60, tol=1e-3, check_every=5, warm_start=1)
    sc = S.small_scene(*dims, steps=4, seed=seed, scheme=scheme, obstacles=1, **kw)
    a = smk.from_scene(sc)
    b = smk.from_scene(sc)
    a.set_readback_slabs(slabs)
    out = _pinned(sc.cell_shape)
    for k in range(sc.steps):
        out.fill(np.nan)
        a.simulate(out, sc.dt)
        b.step(sc.dt)
        want = b.read_density()
        assert H.bits_equal(out, want), (k, slabs)
        assert H.bits_equal(a.read_density(), want), k
    assert H.first_mismatch(a.read_state(), b.read_state()) == ""
    a.close()
    b.close()


@pytest.mark.parametrize("storage", [smk.STORAGE_F32, smk.STORAGE_BF16_VEL, smk.STORAGE_BF16])
@pytest.mark.parametrize("graphs", [True, False])
def test_overlapped_readback_storages_graphs_and_uncaptured_steps(gpu, storage, graphs):
    sc = S.small_scene(37, 22, 51, steps=6, seed=81, scheme=1, iterations=40, tol=1e-3, check_every=5,
                       obstacles=1, warm_start=1)
    sims = [smk.from_scene(sc, report_div=1, storage=storage) for _ in range(3)]
    sims[1].set_readback_slabs(0)  # the copy after the step
    for s in sims:
        s.set_graphs(graphs)
    outs = [_pinned(sc.cell_shape), _pinned(sc.cell_shape)]
    for k in range(sc.steps):
        if k == 3:
            for s in sims:
                s.update_object_pos(0, 12.0, 9.0, 8.0)
        sims[0].simulate(outs[0], sc.dt)
        sims[1].simulate(outs[1], sc.dt)
        sims[2].step(sc.dt)
        want = sims[2].read_density()
        assert H.bits_equal(outs[0], want) and H.bits_equal(outs[1], want), k
        st = [s.stats() for s in sims]
        assert st[0].sweeps == st[2].sweeps and st[0].div_max == st[2].div_max, k
    for s in sims[:2]:
        assert H.first_mismatch(s.read_state(), sims[2].read_state()) == ""
    for s in sims:
        s.close()


def test_simulate_alternating_with_step_and_buffers(gpu):
    """simulate() into two pinned buffers in turn, a pageable one, and plain steps between them:
    each call's output is the density of its own step."""
    sc = S.small_scene(30, 26, 40, steps=8, seed=17, scheme=1, iterations=50, tol=1e-3, check_every=5,
                       warm_start=1)
    a = smk.from_scene(sc)
    b = smk.from_scene(sc)
    bufs = [_pinned(sc.cell_shape), _pinned(sc.cell_shape), np.empty(sc.cell_shape, np.float32)]
    for k in range(sc.steps):
        b.step(sc.dt)
        want = b.read_density()
        if k % 4 == 3:
            a.step(sc.dt)
            assert H.bits_equal(a.read_density(), want), k
            continue
        out = bufs[k % 3]
        a.simulate(out, sc.dt)
        assert H.bits_equal(out, want), k
    a.close()
    b.close()


def test_ref80_golden_through_pinned_simulate(gpu):
    g = H.golden()["scenes"]["ref80"]
    sc = S.config_ref80(steps=100)
    sim = smk.from_scene(sc)
    out = _pinned(sc.cell_shape)
    for k in range(100):
        sim.simulate(out, sc.dt)
        if (k + 1) % 20 == 0:
            assert H.sha(out) == g["density_every_20"][str(k + 1)], k + 1
    assert H.state_hashes(sim.read_state()) == g["final"]
    sim.close()


def test_readback_slabs_validated_and_automatic_count(gpu):
    sim = smk.Simulation(8, 8, 8)
    for bad in (-2, 65):
        with pytest.raises(smk.SmokeError):
            sim.set_readback_slabs(bad)
    assert sim.readback_slabs() == 1  # automatic: one slab per 16 MiB of density, 1 to 8
    sim.set_readback_slabs(5)
    assert sim.readback_slabs() == 5
    sim.set_readback_slabs(0)
    assert sim.readback_slabs() == 0
    sim.close()
    for n, want in ((128, 1), (256, 4), (320, 7)):
        sim = smk.Simulation(n, n, n)
        assert sim.readback_slabs() == want, n
        sim.close()
