"""The FP64 step's exact helpers, compiled from their CUDA headers as host C++.

dtrig.cuh (table-driven sine and cosine) and fp64_exact.cuh (cdiv: division
by a constant through its host reciprocal; mul_pow2: scaling by a power of
two) use only CUDA's IEEE intrinsics (__fma_rn, __dmul_rn, __dadd_rn, bit
moves), which the shim below maps to the host's IEEE operations; the host
build uses -ffp-contract=off, as the intrinsics cannot be contracted.  So the
same source is checked here, without a GPU:

* dsin/dsincos within 3 ulps of glibc, special arguments handled;
* cdiv(a, b, 1/b) bitwise equal to a / b, signed zeros included;
* mul_pow2(x, 2^e) bitwise equal to x * 2^e, zeros, subnormals, Inf/NaN and
  results leaving the normal range included.

tests/test_dtrig.py checks the device build against the same bounds.
"""
import ctypes
import math
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "axions_gb300" / "csrc"
CUDA_INC = Path("/usr/local/cuda/include")

SHIM = r"""
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>
#define __device__
#define __forceinline__ inline
inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }
inline double __dmul_rn(double a, double b) { return a * b; }
inline double __dadd_rn(double a, double b) { return a + b; }
inline long long __double_as_longlong(double x) { long long u; std::memcpy(&u, &x, 8); return u; }
inline double __longlong_as_double(long long u) { double x; std::memcpy(&x, &u, 8); return x; }
inline int __double2hiint(double x) { return (int)(__double_as_longlong(x) >> 32); }
inline int __double2loint(double x) { return (int)(unsigned)(__double_as_longlong(x) & 0xffffffffLL); }
template <class T> inline T __ldg(const T* p) { return *p; }
"""

DRIVER = r"""
#include "dtrig.cuh"
#include "fp64_exact.cuh"
extern "C" {
void h_trig(const double* x, long n, double* out) {
    for (long i = 0; i < n; ++i) {
        double s, c;
        lat::dsincos(x[i], &s, &c);
        out[i] = lat::dsin(x[i]); out[n + i] = s; out[2 * n + i] = c;
    }
}
void h_cdiv(const double* a, const double* b, long n, double* out) {
    for (long i = 0; i < n; ++i) out[i] = lat::cdiv(a[i], b[i], 1.0 / b[i]);
}
void h_div(const double* a, const double* b, long n, double* out) {
    for (long i = 0; i < n; ++i) out[i] = a[i] / b[i];
}
void h_mul_pow2(const double* x, const double* p, long n, double* out, double* ref) {
    for (long i = 0; i < n; ++i) { out[i] = lat::mul_pow2(x[i], p[i]); ref[i] = x[i] * p[i]; }
}
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx or not (CUDA_INC / "cuda_runtime.h").exists():
        pytest.skip("needs g++ and the CUDA headers")
    d = tmp_path_factory.mktemp("fp64host")
    (d / "shim.h").write_text(SHIM)
    (d / "drv.cpp").write_text(DRIVER)
    so = d / "libfp64host.so"
    cmd = [gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", f"-I{CUDA_INC}", f"-I{CSRC}",
           "-include", str(d / "shim.h"), str(d / "drv.cpp"), "-o", str(so)]
    subprocess.run(cmd, check=True, capture_output=True)
    L = ctypes.CDLL(str(so))
    for f in (L.h_trig, L.h_cdiv, L.h_div, L.h_mul_pow2):
        f.restype = None
    return L


def dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def ulps(a, ref):
    return np.abs(a - ref) / np.spacing(np.maximum(np.abs(ref), 2.0 ** -1022))


def test_dtrig_host_build_within_3_ulps_of_glibc(lib):
    rng = np.random.default_rng(5)
    k = np.arange(-2000, 2000, dtype=np.float64)
    pts = np.concatenate([k * (math.pi / 256), (k + 0.5) * (math.pi / 256), k * math.pi, k * math.pi / 2])
    x = np.concatenate([rng.uniform(-60, 60, 200_000), rng.uniform(-6e4, 6e4, 20_000), rng.uniform(-0.05, 0.05, 20_000),
                        pts, np.nextafter(pts, np.inf), np.nextafter(pts, -np.inf)])
    out = np.empty(3 * x.size)
    lib.h_trig(dp(x), ctypes.c_long(x.size), dp(out))
    s1, s2, c2 = out.reshape(3, x.size)
    assert np.array_equal(s1, s2)
    ls = np.array([math.sin(v) for v in x])
    lc = np.array([math.cos(v) for v in x])
    for got, ref in ((s2, ls), (c2, lc)):
        u = ulps(got, ref)
        assert u.max() <= 3 and u.mean() < 0.5, (u.max(), u.mean())
    sp = np.array([0.0, -0.0, 5e-324, 1e-300, 2.0 ** 16, -1e10, np.inf, np.nan])
    o = np.empty(3 * sp.size)
    lib.h_trig(dp(sp), ctypes.c_long(sp.size), dp(o))
    s, _, c = o.reshape(3, sp.size)
    assert s[0] == 0.0 and not np.signbit(s[0]) and np.signbit(s[1]) and c[0] == 1.0 and s[2] == 5e-324
    assert s[4] == math.sin(2.0 ** 16) or ulps(np.array([s[4]]), np.array([math.sin(2.0 ** 16)]))[0] <= 2
    assert np.isnan(s[6]) and np.isnan(c[7])


def random_doubles(rng, n, emin, emax, zeros=0.0):
    bits = (rng.integers(1023 + emin, 1023 + emax, n, dtype=np.uint64) << np.uint64(52)) | \
        (rng.integers(0, 1 << 52, n, dtype=np.uint64)) | (rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63))
    x = bits.view(np.float64)
    if zeros:
        m = rng.random(n) < zeros
        x[m] = np.where(rng.random(m.sum()) < 0.5, 0.0, -0.0)
    return x


def test_cdiv_is_the_ieee_quotient(lib):
    rng = np.random.default_rng(11)
    n = 2_000_000
    a = random_doubles(rng, n, -450, 450, zeros=0.01)
    b = random_doubles(rng, n, -450, 450)
    b[: n // 4] = rng.choice([0.1, 0.05, 0.025, 1.0 / 3.0, 0.7, np.nextafter(1.0, 0.0)], n // 4)
    got, ref = np.empty(n), np.empty(n)
    lib.h_cdiv(dp(a), dp(b), ctypes.c_long(n), dp(got))
    lib.h_div(dp(a), dp(b), ctypes.c_long(n), dp(ref))
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))


def test_mul_pow2_is_the_ieee_product(lib):
    rng = np.random.default_rng(13)
    n = 1_000_000
    x = random_doubles(rng, n, -1022, 1023, zeros=0.01)
    special = np.array([5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, np.inf, -np.inf, np.nan])
    x[: special.size] = special
    x[special.size: 2000] = rng.uniform(-1, 1, 2000 - special.size) * 2.0 ** -1030   # subnormal
    p = 2.0 ** rng.integers(-3, 4, n).astype(np.float64)
    got, ref = np.empty(n), np.empty(n)
    lib.h_mul_pow2(dp(x), dp(p), ctypes.c_long(n), dp(got), dp(ref))
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(got[~nan].view(np.uint64), ref[~nan].view(np.uint64))
