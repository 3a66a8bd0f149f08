"""The renderer restatement (oracle/render_oracle.cpp), CPU only: its half-precision rounding is
IEEE binary16 round-to-nearest-even (checked against numpy's float16), an empty volume renders
the background, and the eye alpha of a volume grows with its density."""
import numpy as np
import pytest

from oracle import oracle as O


def _params(**kw):
    smk = pytest.importorskip("smoke_simulation_gb300")
    return smk.default_render_params(**kw)


def test_half_rounding_is_ieee_round_to_nearest_even():
    rng = np.random.default_rng(0)
    vals = np.concatenate([
        rng.standard_normal(200000).astype(np.float32) * np.float32(4.0),
        rng.uniform(0, 1e-4, 20000).astype(np.float32),                 # subnormal halves
        np.array([65504, 65519.99, 65520, 1e6, -1e6, 6.1035156e-05, 5.9604645e-08, 2.9802322e-08,
                  -0.0, 0.0, np.inf, -np.inf, 1 / 3, 2049, 2051], np.float32)])
    with np.errstate(over="ignore"):
        ref = vals.astype(np.float16).astype(np.float32)
    assert np.array_equal(O.round_half(vals).view(np.uint32), ref.view(np.uint32))


def test_empty_volume_renders_background(smoke_lib):
    rp = _params(width=48, height=32, light_res=16, planes=12)
    eye, comp = O.render(np.zeros((10, 12, 14), np.float32), rp)
    assert not eye.any()
    bg = np.array(rp.bg_color[:], np.float32)
    assert np.allclose(comp, bg[None, None, :], rtol=0, atol=0)


def test_alpha_grows_with_density(smoke_lib):
    rp = _params(width=64, height=40, light_res=24, planes=20)
    n = 24
    z, y, x = np.mgrid[0:n, 0:n, 0:n]
    blob = np.exp(-((x - 12) ** 2 + (y - 12) ** 2 + (z - 12) ** 2) / 20.0).astype(np.float32)
    a1 = O.render(0.3 * blob, rp)[0][..., 3]
    a2 = O.render(0.6 * blob, rp)[0][..., 3]
    assert a1.max() > 0.05
    assert (a2 >= a1 - 1e-3).all() and a2.sum() > a1.sum()


def _proxy_golden():
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "proxy_planes.npz"))
    out = []
    for k in range(len([f for f in d.files if f.endswith("_args")])):
        a = d["case%02d_args" % k]
        args = (a[0:3], a[3:6], a[6:9], a[9:12], int(a[12]))
        out.append((args, d["case%02d_vertices" % k], d["case%02d_counts" % k], d["case%02d_triangles" % k]))
    return out


def test_proxy_restatement_equals_reference_golden():
    """The proxy-plane restatement (the checker of smk_proxy_planes) gives, bit for bit, the
    reference's own BoundingBox::generateProxyGeometry output recorded in
    tests/golden/proxy_planes.npz (project/boundingBox.cpp:133-181 built for the host)."""
    for args, gv, gc, gt in _proxy_golden():
        v, c, t = O.proxy_planes(*args)
        assert np.array_equal(c, gc) and np.array_equal(t, gt), args
        assert np.array_equal(v.view(np.uint32), gv.view(np.uint32)), args


def test_proxy_restatement_equals_live_reference_build():
    """Where the reference checkout is present, the restatement equals the reference's own
    proxy-plane functions built for the host for many seeded view directions and plane counts."""
    if not O.reference_proxy_available():
        pytest.skip("the reference's proxy-plane build needs the reference checkout")
    rng = np.random.default_rng(5)
    for k in range(60):
        d = rng.standard_normal(3)
        dims = (80.0, 80.0, 80.0) if k % 3 else tuple(float(x) for x in rng.integers(8, 160, 3))
        args = (tuple(rng.uniform(-50, 50, 3)), tuple(d), (0.0, 0.0, 0.0), dims, int(rng.integers(2, 120)))
        rv, rc, rt = O.reference_proxy_planes(*args)
        v, c, t = O.proxy_planes(*args)
        assert np.array_equal(c, rc) and np.array_equal(t, rt), args
        assert np.array_equal(v.view(np.uint32), rv.view(np.uint32)), args
