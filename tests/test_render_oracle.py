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
