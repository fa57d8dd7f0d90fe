"""CPU-only checks of the C ABI library: it loads, exports every entry point
declared in include/, fills the reference defaults, validates parameters, and
its host-side IC generator reproduces the reference's mt19937 draws."""
import ctypes
import math
import re

import numpy as np
import pytest

from conftest import ROOT, load_golden


def _declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = h.read_text()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(lat_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


@pytest.fixture(scope="module")
def L():
    from axions_gb300 import lattice
    return lattice.load_library()


def test_library_exports_every_declared_symbol(L):
    from axions_gb300 import lattice
    declared = _declared_symbols()
    assert declared, "no declarations found"
    assert set(lattice.EXPORTS) <= set(declared)
    for name in declared:
        assert hasattr(L, name), f"{name} declared in include/ but not exported"


def test_version_string(L):
    assert b"sm_103a" in L.lat_version()


def test_params_init_matches_reference_defaults(L):
    from axions_gb300 import lattice
    from axions_gb300.params import MODEL_AH, MODEL_MOORE, default_params
    for model in (MODEL_AH, MODEL_MOORE):
        p = lattice.params_init(model)
        q = default_params(model)
        assert p.as_dict() == q.as_dict()
    # moore_mpi_evolution.cpp:35  g = sqrt(0.5*lambda1*eta1^2/(q1^2+q2^2))
    p = lattice.params_init(MODEL_MOORE)
    assert p.g == math.sqrt(0.5 * 1.0 / 5.0)


def test_invalid_params_rejected_before_device(L):
    from axions_gb300 import lattice
    from axions_gb300.params import LAT_ERR_INVALID, make_params
    bad = [dict(nx=1), dict(dt=0.0), dict(precision=7), dict(bc=9), dict(abi_version=0),
           dict(nx=2000, ny=2000, nz=2000)]
    for kw in bad:
        p = make_params(0, n=8)
        for k, v in kw.items():
            setattr(p, k, v)
        h = ctypes.c_void_p()
        rc = L.lat_create(ctypes.byref(p), ctypes.byref(h))
        assert rc == LAT_ERR_INVALID, kw
        assert L.lat_last_error()


def test_host_ic_matches_reference_fixture():
    from axions_gb300 import lattice
    from axions_gb300.params import make_params
    z = load_golden("ref_mpi_ah_ic_s7")
    p = make_params(0, nx=int(z["nx"]), ny=int(z["ny"]), nz=int(z["nz"]))
    ic = lattice.random_phase_ic(p, int(z["seed"]))
    assert np.array_equal(ic, z["ic"][:, 1, :])
    assert np.array_equal(ic, z["ic"][:, 0, :])


def test_host_ic_matches_oracle(oracle_mod):
    from axions_gb300 import lattice
    from axions_gb300.params import MODEL_MOORE, make_params
    for model, indep in ((0, False), (MODEL_MOORE, False), (MODEL_MOORE, True)):
        p = make_params(model, nx=7, ny=6, nz=5, eta2=0.8)
        a = lattice.random_phase_ic(p, 1234, indep)
        b = oracle_mod.random_phase_ic(p, 1234, indep)
        assert np.array_equal(a, b[:, 0, :])
        if model == MODEL_MOORE and not indep:
            np.testing.assert_allclose(a[2] / 0.8, a[0], rtol=1e-15)


def test_no_device_is_reported_not_faked(L):
    """Without a GPU the library says so; it never falls back to the CPU."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from axions_gb300.params import LAT_ERR_NODEVICE, make_params
    p = make_params(0, n=8)
    h = ctypes.c_void_p()
    assert L.lat_create(ctypes.byref(p), ctypes.byref(h)) == LAT_ERR_NODEVICE


def test_new_entry_points_reject_bad_arguments_before_device(L):
    """lat_run and lat_dtrig_eval check their arguments before any CUDA call."""
    from axions_gb300.params import LAT_ERR_INVALID, LAT_OK
    dp = ctypes.POINTER(ctypes.c_double)
    buf = np.zeros(8)
    x = buf.ctypes.data_as(dp)
    cnt = ctypes.c_int64(0)
    assert L.lat_run(None, x, x, 0, 1, 0, None, 0, ctypes.byref(cnt), x, x) == LAT_ERR_INVALID
    assert L.lat_last_error()
    assert L.lat_dtrig_eval(x, -1, x) == LAT_ERR_INVALID
    assert L.lat_dtrig_eval(None, 1, x) == LAT_ERR_INVALID
    assert L.lat_dtrig_eval(x, 0, x) == LAT_OK   # nothing to do: no device needed


def test_large_fp64_lattices_are_accepted_with_64_bit_link_offsets(L):
    """The two-pass FP64 step addresses its 15 link-data slots through base
    pointers formed in 64-bit arithmetic, so a lattice whose 15*N passes 2^31
    (528x528x520 = 144,967,680 sites) is valid and its footprint counts the
    link data in full."""
    from axions_gb300.params import make_params
    L.lat_footprint_bytes.restype = ctypes.c_int64
    p = make_params(0, nx=528, ny=528, nz=520)
    N = 528 * 528 * 520
    assert 15 * N > 2 ** 31
    b = L.lat_footprint_bytes(ctypes.byref(p))
    fields_div_links = 5 * 2 * N * 8 + N * 8 + 15 * N * 8
    assert fields_div_links < b < fields_div_links + 64 * 2 ** 20


def test_side_products_cannot_wrap(L):
    """nx*ny*nz is formed only after each factor is bounded: sides whose
    product would overflow int64 are rejected, not wrapped into range."""
    from axions_gb300.params import LAT_ERR_INVALID, make_params
    L.lat_footprint_bytes.restype = ctypes.c_int64
    for nx, ny, nz in ((2, 2 ** 40, 2 ** 40), (4, 2 ** 62, 4), (65535, 2 ** 31 - 2, 2), (1000, 1000, 2148)):
        p = make_params(0, nx=nx, ny=ny, nz=nz)
        assert L.lat_footprint_bytes(ctypes.byref(p)) == LAT_ERR_INVALID, (nx, ny, nz)


def test_noalloc_validates_before_any_device_call(L):
    """The allocation-free step runs the library's parameter checks (and its
    own) before it touches CUDA, so bad blocks are rejected without a GPU."""
    from axions_gb300.params import BC_NEUMANN, F32, LAT_ERR_INVALID, MODEL_MOORE, make_params
    buf = np.zeros(8)
    x = ctypes.c_void_p(buf.ctypes.data)
    bad = [dict(precision=F32), dict(model=MODEL_MOORE), dict(bc=BC_NEUMANN), dict(tau0=0.0),
           dict(tau0=float("nan")), dict(ny=2 ** 40, nz=2 ** 40), dict(kernel_variant=1), dict(nx=65, ny=64, nz=64)]
    for kw in bad:
        p = make_params(0, n=8)
        for k, v in kw.items():
            setattr(p, k, v)
        assert L.lat_ah_step_f64_noalloc(ctypes.byref(p), x, 0, 1, None) == LAT_ERR_INVALID, kw
        assert L.lat_last_error()
