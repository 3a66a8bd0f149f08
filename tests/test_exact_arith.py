"""Host instances of the exact arithmetic the blocked REFERENCE-scheme sweep uses instead of the
FP64 pipe (csrc/exact_scale.cuh), on the CPU: float(double(q) * omega) and x / d for d = 1..6
must give the bits of the double product and of the IEEE float quotient (the reference's own
expressions, project/smokeSimulation.cu:38, :384) on seeded random bit patterns of every
exponent, on edge values, and for several omegas."""
import ctypes as C

import numpy as np
import pytest


def _lib(smoke_lib):
    fn = smoke_lib.smk_test_exact_arith
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.c_void_p]
    return fn


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    x = bits.view(np.float32)
    x = x[~np.isnan(x)]
    edge = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, 1e-45, -1e-45, 1.1754944e-38, 3.4028235e38,
                     -3.4028235e38, 2.0**-100, 2.0**100, 2.0**-126, 1.0 / 3.0, 6.0, 0.5 + 2**-24],
                    np.float32)
    return np.ascontiguousarray(np.concatenate([edge, x]).astype(np.float32))


@pytest.mark.parametrize("omega", [1.9, 1.0, 1.5, 0.7, 1.99, 1.3, 0.25])
def test_omega_scale_equals_double_product(smoke_lib, omega):
    fn = _lib(smoke_lib)
    x = _inputs(1 << 21, seed=int(omega * 1000))
    out = np.empty_like(x)
    assert fn(x.ctypes.data, None, x.size, omega, out.ctypes.data, None) == 0
    with np.errstate(over="ignore"):
        want = (x.astype(np.float64) * omega).astype(np.float32)
    assert np.array_equal(out.view(np.uint32), want.view(np.uint32))


def test_div_small_equals_ieee_quotient(smoke_lib):
    fn = _lib(smoke_lib)
    x = _inputs(1 << 21, seed=7)
    for d in range(1, 7):
        dd = np.full(x.size, d, np.int32)
        out = np.empty_like(x)
        assert fn(x.ctypes.data, dd.ctypes.data, x.size, 1.9, None, out.ctypes.data) == 0
        want = x / np.float32(d)
        assert np.array_equal(out.view(np.uint32), want.view(np.uint32)), d
