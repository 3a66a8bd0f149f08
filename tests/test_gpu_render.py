"""GPU tests of the headless half-angle slice renderer (smk_render): bit-exact with the CPU
restatement (oracle/render_oracle.cpp) for both blending orders, for an analytic density and for
a simulated one, in FP32 and BF16 density storage."""
import os

import numpy as np
import pytest

import smoke_simulation_gb300 as smk
from oracle import oracle as O
from smoke_simulation_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def _blob(n):
    z, y, x = np.mgrid[0:n, 0:n, 0:n]
    return np.exp(-((x - n / 2) ** 2 + (y - n / 3) ** 2 + (z - n / 2) ** 2) / (n * 0.8)).astype(np.float32)


@pytest.mark.parametrize("light", [(120.0, 80.0, 0.0), (0.0, 20.0, -120.0)])  # front-to-back, back-to-front
def test_render_bit_exact_with_restatement(gpu, light):
    n = 40
    sim = smk.Simulation(n, n, n)
    sim.set_density(_blob(n))
    rp = smk.default_render_params(width=120, height=72, light_res=64, planes=36)
    rp.light_pos[:] = light
    eye, comp = sim.render(rp)
    rho = sim.read_density()
    oe, oc = O.render(rho, rp)
    assert eye[..., 3].max() > 0.1
    assert np.array_equal(eye.view(np.uint32), oe.view(np.uint32))
    assert np.array_equal(comp.view(np.uint32), oc.view(np.uint32))
    sim.close()


@pytest.mark.parametrize("storage", [smk.STORAGE_F32, smk.STORAGE_BF16])
def test_render_simulated_density(gpu, storage):
    sc = S.config_ref80(steps=20, scheme=1)
    sc.tol, sc.check_every, sc.iterations = 1e-4, 6, 200
    sim = smk.from_scene(sc, storage=storage)
    for _ in range(sc.steps):
        sim.step(sc.dt)
    rp = smk.default_render_params(width=160, height=90, light_res=96, planes=50)
    eye, comp = sim.render(rp)
    oe, oc = O.render(sim.read_density(), rp)
    assert (eye[..., 3] > 0.01).sum() > 50
    assert np.array_equal(eye.view(np.uint32), oe.view(np.uint32))
    assert np.array_equal(comp.view(np.uint32), oc.view(np.uint32))
    sim.close()


@pytest.mark.parametrize("view_dir", [(-0.3, -0.2, 0.93), (0.0, 0.0, 1.0), (1.0, 1.0, 0.0), (-0.51, 0.67, -0.2)])
def test_proxy_planes_bit_exact_with_restatement(gpu, view_dir):
    """Proxy-plane polygons on the device equal the restatement; every polygon of the default
    box is a fan of at least 3 triangles around its centroid, inside the box."""
    dims = (80.0, 80.0, 80.0)
    v, c, t = smk.proxy_planes((0, 0, 0), view_dir, (0, 0, 0), dims, 50)
    ov, oc, ot = O.proxy_planes((0, 0, 0), view_dir, (0, 0, 0), dims, 50)
    assert np.array_equal(c, oc) and np.array_equal(t, ot)
    assert np.array_equal(v.view(np.uint32), ov.view(np.uint32))
    assert (c >= 3).all() and (c <= 6).all()
    assert np.abs(v).max() <= 40.0 + 1e-4


def test_proxy_planes_bit_exact_with_reference_golden(gpu):
    """Proxy-plane polygons on the device equal, bit for bit, the reference's own
    BoundingBox::generateProxyGeometry (project/boundingBox.cpp:133-181) recorded in
    tests/golden/proxy_planes.npz: the application's view, axis-aligned, diagonal and seeded
    directions, unequal box sides."""
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "proxy_planes.npz"))
    n = len([f for f in d.files if f.endswith("_args")])
    assert n >= 10
    for k in range(n):
        a = d["case%02d_args" % k]
        v, c, t = smk.proxy_planes(a[0:3], a[3:6], a[6:9], a[9:12], int(a[12]))
        assert np.array_equal(c, d["case%02d_counts" % k]) and np.array_equal(t, d["case%02d_triangles" % k]), k
        assert np.array_equal(v.view(np.uint32), d["case%02d_vertices" % k].view(np.uint32)), k
