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


def _tiny_inputs(sub_stride, normal_stride, emax=31):
    """Every sub_stride-th subnormal and every normal_stride-th float with biased exponent
    1..emax, both signs: the operands of the tiny paths (results and quotients near and below
    2^-126)."""
    sub = np.arange(1, 1 << 23, sub_stride, dtype=np.uint32)
    nrm = np.arange(1 << 23, (emax + 1) << 23, normal_stride, dtype=np.uint32)
    bits = np.concatenate([sub, nrm])
    bits = np.concatenate([bits, bits | np.uint32(0x80000000)])
    return np.ascontiguousarray(bits.view(np.float32))


@pytest.mark.parametrize("omega,sub_stride", [(1.9, 1), (0.25, 7), (0.7, 7), (1.0, 7), (1.99, 7), (1.3, 7)])
def test_omega_scale_tiny_and_subnormal_operands(smoke_lib, omega, sub_stride):
    """Results below 2^-126 are rounded from the 53-bit product to the subnormal grid, as the
    conversion of the double product is (every subnormal q for omega = 1.9)."""
    fn = _lib(smoke_lib)
    x = _tiny_inputs(sub_stride, 13)
    out = np.empty_like(x)
    assert fn(x.ctypes.data, None, x.size, omega, out.ctypes.data, None) == 0
    want = (x.astype(np.float64) * omega).astype(np.float32)
    bad = np.flatnonzero(out.view(np.uint32) != want.view(np.uint32))
    assert bad.size == 0, (omega, x[bad[:4]], out[bad[:4]], want[bad[:4]])


@pytest.mark.parametrize("d", [1, 2, 3, 4, 5, 6])
def test_div_small_tiny_and_subnormal_operands(smoke_lib, d):
    """Every subnormal x and samples of every exponent below 2^-100 give the IEEE quotient's
    bits, normal quotients (x * 2^64 rescaled) and subnormal ones (integer rounding) alike."""
    fn = _lib(smoke_lib)
    x = _tiny_inputs(1, 11, emax=27)
    dd = np.full(x.size, d, np.int32)
    out = np.empty_like(x)
    assert fn(x.ctypes.data, dd.ctypes.data, x.size, 1.9, None, out.ctypes.data) == 0
    want = x / np.float32(d)
    bad = np.flatnonzero(out.view(np.uint32) != want.view(np.uint32))
    assert bad.size == 0, (d, x[bad[:4]], out[bad[:4]], want[bad[:4]])


@pytest.mark.parametrize("omega", [1.9, 0.25, 1.0, 1.99])
def test_cell_path_equals_quotient_then_double_product(smoke_lib, omega):
    """The sweep's per-cell p_t: the branch-free common path with the out-of-line path for rare
    operands gives float(double(x / d) * omega) (the reference's expression) on random bit
    patterns, edge values, zeros of both signs, and strided subnormals and small normals (the
    tests above cover every subnormal for the two functions on their own)."""
    fn = smoke_lib.smk_test_exact_cell
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_void_p]
    x = np.concatenate([_inputs(1 << 19, seed=11), _tiny_inputs(5 if omega == 1.9 else 37, 499)])
    x = np.ascontiguousarray(x)
    for d in range(1, 7):
        dd = np.full(x.size, d, np.int32)
        out = np.empty_like(x)
        assert fn(x.ctypes.data, dd.ctypes.data, x.size, omega, out.ctypes.data) == 0
        with np.errstate(over="ignore", invalid="ignore"):
            want = ((x / np.float32(d)).astype(np.float64) * omega).astype(np.float32)
        bad = np.flatnonzero(out.view(np.uint32) != want.view(np.uint32))
        assert bad.size == 0, (omega, d, x[bad[:4]], out[bad[:4]], want[bad[:4]])
