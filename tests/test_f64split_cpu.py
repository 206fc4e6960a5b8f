"""The integer-based FP64-minus-FP32 difference of the split-precision stage
(hopefoam_gb300/csrc/f64split.cuh), compiled for the host with g++ and
checked against FP64 arithmetic on seeded values over 60 binades, exact
zeros, equal operands and opposite signs.

Bound: |d - (q - b)| <= 1 ulp32(q - b) + 2^-45 |q| (the FP32 roundings of
qh - b and of the sum, plus the rounding of the 29 dropped significand bits)."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "hopefoam_gb300", "csrc")

SRC = r'''
#include "f64split.cuh"
extern "C" void minus_batch(const double* q, const float* b, float* out, int n) {
    for (int i = 0; i < n; i++) out[i] = f64s::minus_f32(q[i], b[i]);
}
extern "C" void trunc_batch(const double* q, float* out, int n) {
    for (int i = 0; i < n; i++) out[i] = f64s::trunc_f32(q[i]);
}
extern "C" void widen_batch(const float* x, double* out, int n) {
    for (int i = 0; i < n; i++) out[i] = f64s::widen(x[i]);
}
'''


@pytest.fixture(scope="module")
def f64split_lib():
    d = tempfile.mkdtemp(prefix="f64split_")
    src = os.path.join(d, "t.cpp")
    so = os.path.join(d, "t.so")
    with open(src, "w") as f:
        f.write(SRC)
    r = subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-I", CSRC, src, "-o", so], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail("g++ failed: " + r.stderr)
    return ctypes.CDLL(so)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def test_minus_f32_bound(f64split_lib):
    rng = np.random.default_rng(0)
    n = 400_000
    q = rng.standard_normal(n) * np.exp(rng.uniform(-30, 30, n))
    b = (q * (1 + rng.standard_normal(n) * np.exp(rng.uniform(-25, 0, n)))).astype(np.float32)
    q[:1000] = 0.0
    b[1000:2000] = 0.0
    q[2000:3000] = b[2000:3000]
    b[3000:4000] = -b[3000:4000]
    out = np.empty(n, np.float32)
    f64split_lib.minus_batch(_p(q), _p(b), _p(out), n)
    ref = q - b.astype(np.float64)
    ulp = np.spacing(np.abs(ref.astype(np.float32))).astype(np.float64)
    err = np.abs(out.astype(np.float64) - ref)
    assert np.all(err <= ulp + 2.0 ** -45 * np.abs(q) + 1e-37)
    # equal operands give exactly zero; q = 0 gives exactly -b
    assert np.all(out[2000:3000] == 0.0)
    assert np.all(out[:1000] == -b[:1000])


def test_minus_f32_special_values(f64split_lib):
    q = np.array([np.inf, -np.inf, np.nan, 1e300, 5e-320, -0.0, 2.0 ** -126, 2.0 ** -127])
    b = np.array([1.0, 1.0, 1.0, 1.0, 1.0, 2.0, 0.0, 0.0], np.float32)
    out = np.empty(q.size, np.float32)
    f64split_lib.minus_batch(_p(q), _p(b), _p(out), q.size)
    assert out[0] == np.inf and out[1] == -np.inf and np.isnan(out[2])
    assert out[3] == np.inf  # beyond FP32 range: the FP64 route rounds to infinity
    assert out[4] == -1.0 and out[5] == -2.0
    assert out[6] == np.float32(2.0 ** -126) and out[7] == 0.0  # below 2^-126 is taken as zero


def test_trunc_f32(f64split_lib):
    rng = np.random.default_rng(1)
    q = rng.standard_normal(100_000) * np.exp(rng.uniform(-40, 40, 100_000))
    out = np.empty(q.size, np.float32)
    f64split_lib.trunc_batch(_p(q), _p(out), q.size)
    o = out.astype(np.float64)
    assert np.all(np.abs(o) <= np.abs(q))  # toward zero
    assert np.all(np.abs(q - o) < np.spacing(np.abs(out)).astype(np.float64))  # less than one FP32 ulp


def test_widen_exact(f64split_lib):
    """FP32 -> FP64 from the bits: identical to the conversion for normal,
    zero, subnormal, infinite values (NaN stays NaN)."""
    rng = np.random.default_rng(11)
    x = np.concatenate([(rng.standard_normal(20000) * 10.0 ** rng.uniform(-30, 30, 20000)).astype(np.float32),
                        np.array([0.0, -0.0, 1e-45, -3e-40, 3.4e38, np.inf, -np.inf], np.float32)])
    out = np.empty(x.size, np.float64)
    f64split_lib.widen_batch(_p(x), _p(out), x.size)
    ref = x.astype(np.float64)
    assert np.array_equal(out.view(np.uint64), ref.view(np.uint64))
    nan = np.array([np.nan], np.float32)
    o = np.empty(1, np.float64)
    f64split_lib.widen_batch(_p(nan), _p(o), 1)
    assert np.isnan(o[0])
