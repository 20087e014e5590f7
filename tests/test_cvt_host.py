"""The integer-pipe FP64 <-> FP32 conversions of the FP64-bound kernels (nsp_cvt.cuh),
compiled for the host and checked against numpy's IEEE conversions: double -> float
rounds to nearest even (ties, carries into the exponent, overflow to Inf), float ->
double is exact, Inf and NaN survive, and magnitudes below 2^-126 (the float denormal
range, double denormals) flush to a zero of the same sign."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = r'''
#include <cstdint>
#include <cstring>
#include "nsp_cvt.cuh"
extern "C" void narrow(const double* x, float* y, int n) {
  for (int i = 0; i < n; i++) {
    uint64_t b; std::memcpy(&b, x + i, 8);
    const uint32_t f = nsp::f64_to_f32_bits(b);
    std::memcpy(y + i, &f, 4);
  }
}
extern "C" void widen(const float* x, double* y, int n) {
  for (int i = 0; i < n; i++) {
    uint32_t u; std::memcpy(&u, x + i, 4);
    const uint64_t d = nsp::f32_to_f64_bits(u);
    std::memcpy(y + i, &d, 8);
  }
}
'''


@pytest.fixture(scope="module")
def cvt(tmp_path_factory):
    d = tmp_path_factory.mktemp("cvt")
    src, lib = d / "cvt.cpp", d / "libcvt.so"
    src.write_text(SRC)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(ROOT, "nspipe-gpu_gb300", "csrc"),
                    "-I", os.path.join(cuda, "include"), str(src), "-o", str(lib)], check=True)
    L = ctypes.CDLL(str(lib))
    dp, fp = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float)
    L.narrow.argtypes = [dp, fp, ctypes.c_int]
    L.widen.argtypes = [fp, dp, ctypes.c_int]

    def narrow(x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty(x.size, np.float32)
        L.narrow(x.ctypes.data_as(dp), y.ctypes.data_as(fp), x.size)
        return y

    def widen(x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.empty(x.size, np.float64)
        L.widen(x.ctypes.data_as(fp), y.ctypes.data_as(dp), x.size)
        return y
    return narrow, widen


def same_bits(a, b):
    return np.array_equal(a.view(np.uint32 if a.dtype == np.float32 else np.uint64),
                          b.view(np.uint32 if b.dtype == np.float32 else np.uint64))


def test_narrow_rounds_to_nearest_even(cvt):
    narrow, _ = cvt
    rng = np.random.default_rng(7)
    x = rng.standard_normal(200000) * np.exp2(rng.integers(-120, 120, 200000))
    x = x[np.abs(x) >= 2.0 ** -126]  # the flush range is the next test's
    # exact ties: a float plus half an ulp (even and odd mantissas), and their neighbours
    f = rng.standard_normal(5000).astype(np.float32)
    half = np.spacing(np.abs(f)).astype(np.float64) / 2
    ties = np.concatenate([f.astype(np.float64) + half, f.astype(np.float64) - half,
                           np.nextafter(f.astype(np.float64) + half, np.inf)])
    big = np.array([3.4028234663852886e38, 3.4028235677973366e38, 3.402823669209385e38, 1e39, -1e300])
    for v in (x, ties, big):
        with np.errstate(over="ignore"):
            assert same_bits(narrow(v), v.astype(np.float32))


def test_narrow_specials_and_flush(cvt):
    narrow, _ = cvt
    v = np.array([0.0, -0.0, np.inf, -np.inf, 1e-39, -1e-39, 5e-324, -5e-324, 1e-300, 2.0 ** -126, -(2.0 ** -126)])
    y = narrow(v)
    assert same_bits(y[:4], v[:4].astype(np.float32))
    assert same_bits(y[4:9], np.array([0.0, -0.0, 0.0, -0.0, 0.0], np.float32))  # below 2^-126: signed zero
    assert y[9] == np.float32(2.0 ** -126) and y[10] == -np.float32(2.0 ** -126)  # the smallest normal stays
    n = narrow(np.array([np.nan, -np.nan]))
    assert np.isnan(n).all() and np.signbit(n[1]) and not np.signbit(n[0])


def test_widen_is_exact(cvt):
    _, widen = cvt
    rng = np.random.default_rng(8)
    bits = rng.integers(0, 2 ** 32, 200000, dtype=np.uint64).astype(np.uint32)
    f = bits.view(np.float32)
    normal = (np.abs(f) >= np.float32(2.0 ** -126)) & np.isfinite(f)
    assert same_bits(widen(f[normal]), f[normal].astype(np.float64))
    den = f[(np.abs(f) < np.float32(2.0 ** -126)) & (f != 0)]  # float denormals flush to signed zero
    w = widen(den)
    assert (w == 0).all() and np.array_equal(np.signbit(w), np.signbit(den))
    s = widen(np.array([np.inf, -np.inf, np.nan, 0.0, -0.0], np.float32))
    assert s[0] == np.inf and s[1] == -np.inf and np.isnan(s[2]) and s[3] == 0 and np.signbit(s[4])
