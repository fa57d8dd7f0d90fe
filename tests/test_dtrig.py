"""The FP64 step's table-driven sine and cosine (dtrig.cuh) on the GPU, through
lat_dtrig_eval, against the host's libm (glibc: within about half an ulp of
the exact values) and against CUDA's own sin/cos.

Bounds: at most 4 ulps from libm at every argument and a mean below 0.5 ulp
(measured: 3 and 0.3; the exact error is at most 2.1 ulps).  CUDA's double
sin is documented to 2 ulps, so the two GPU sines are within 4 ulps of each
other.  The step's arguments are link phases and plaquette angles of order
1-100; the samples cover those, the reduction's table points and midpoints,
the zeros of sin and cos, tiny and huge arguments, and non-finite ones.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lattice_mod():
    from axions_gb300 import lattice
    lattice.load_library()
    return lattice


def ulps(a, ref):
    return np.abs(a - ref) / np.spacing(np.maximum(np.abs(ref), 2.0 ** -1022))


def samples():
    rng = np.random.default_rng(20261203)
    k = np.arange(-3000, 3000, dtype=np.float64)
    step = math.pi / 256
    pts = np.concatenate([k * step, (k + 0.5) * step, k * math.pi, k * math.pi / 2])
    return np.concatenate([rng.uniform(-60.0, 60.0, 400_000), rng.uniform(-6e4, 6e4, 50_000),
                           rng.uniform(-0.05, 0.05, 50_000), pts, np.nextafter(pts, np.inf),
                           np.nextafter(pts, -np.inf)])


def test_dtrig_within_ulps_of_libm_and_cuda(lattice_mod):
    x = samples()
    s1, s2, c2, cs, cc = lattice_mod.dtrig_eval(x)
    ls = np.array([math.sin(v) for v in x])
    lc = np.array([math.cos(v) for v in x])
    # the sine alone and the joint sincos give the same doubles
    assert np.array_equal(s1, s2)
    for got, ref, name in ((s2, ls, "sin"), (c2, lc, "cos")):
        u = ulps(got, ref)
        assert u.max() <= 4 and u.mean() < 0.5, (name, u.max(), u.mean(), x[np.argmax(u)])
    assert ulps(s2, cs).max() <= 4 and ulps(c2, cc).max() <= 4


def test_dtrig_special_arguments(lattice_mod):
    big = [2.0 ** 16, -2.0 ** 16, 1e10, 1e300]
    x = np.array([0.0, -0.0, 5e-324, -5e-324, 1e-300, 2.0 ** -27, -(2.0 ** -27), np.nextafter(2.0 ** -27, 0.0),
                  np.nextafter(2.0 ** 16, 0.0)] + big + [np.inf, -np.inf, np.nan])
    s1, s2, c2, cs, cc = lattice_mod.dtrig_eval(x)
    # sin x = x (with the sign of zero) and cos x = 1 below 2^-27
    for i in range(5):
        assert s1[i] == x[i] and np.signbit(s1[i]) == np.signbit(x[i]) and c2[i] == 1.0
    for i in range(5, 9):
        assert ulps(np.array([s2[i]]), np.array([math.sin(x[i])]))[0] <= 4
        assert ulps(np.array([c2[i]]), np.array([math.cos(x[i])]))[0] <= 4
    # |x| >= 2^16 is CUDA's sin/cos itself
    nb = len(big)
    assert np.array_equal(s1[9:9 + nb], cs[9:9 + nb]) and np.array_equal(c2[9:9 + nb], cc[9:9 + nb])
    assert np.all(np.isnan(s1[-3:])) and np.all(np.isnan(s2[-3:])) and np.all(np.isnan(c2[-3:]))


def test_dtrig_eval_rejects_bad_sizes(lattice_mod):
    import ctypes
    L = lattice_mod.load_library()
    x = np.zeros(1)
    out = np.zeros(5)
    dp = ctypes.POINTER(ctypes.c_double)
    assert L.lat_dtrig_eval(x.ctypes.data_as(dp), -1, out.ctypes.data_as(dp)) == -1
    assert L.lat_dtrig_eval(x.ctypes.data_as(dp), 0, out.ctypes.data_as(dp)) == 0
