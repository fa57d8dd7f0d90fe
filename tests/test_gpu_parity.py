"""GPU parity through the C ABI against the reference (golden fixtures) and the
oracle (live, on the same seeded inputs).

Tolerances (FP64 path):
  * fields: normwise, max|d|/max|ref| <= 1e-12 and ||d||_2/||ref||_2 <= 1e-12
    over the whole state, and ||d||_2/||ref||_2 <= 1e-12 for every field
    (component) on its own.  (A single field's largest site difference over its
    own largest value reaches ~1.1e-12 after 300 chaotic steps: the FP64
    step's table-driven sin/cos differ from libm's in the last bits (at most
    3 ulps) for some arguments, and the dynamics amplify it.)
    Element-wise equality is therefore not possible; normwise agreement is the
    bar.
  * energy and summed Gauss deviation: relative 1e-12 (different summation
    order on top of the above).
  * string detection on identical fields: bit-exact (same double operations,
    -fmad=false, IEEE sqrt and division on both sides).
  * plaquette winding on identical fields: bit-exact.
"""
import numpy as np
import pytest

from conftest import load_golden, params_from_json

pytestmark = pytest.mark.gpu

TOL = 1e-12


def normwise(a, b):
    d = np.abs(a - b)
    return d.max() / np.abs(b).max(), np.linalg.norm(d) / np.linalg.norm(b)


def assert_fields_close(a, b, tol=TOL):
    mx, l2 = normwise(a, b)
    assert mx <= tol and l2 <= tol, f"max {mx:.3e} l2 {l2:.3e}"
    # field by field: the relative L2 error of every component on its own
    a2, b2 = a.reshape(a.shape[0], -1), b.reshape(b.shape[0], -1)
    for c in range(b2.shape[0]):
        ref = np.linalg.norm(b2[c])
        err = np.linalg.norm(a2[c] - b2[c])
        assert err <= tol * max(ref, 1e-300), f"component {c}: ||d|| {err:.3e}, ||ref|| {ref:.3e}"


@pytest.fixture(scope="module")
def lattice_mod():
    from axions_gb300 import lattice
    lattice.load_library()
    return lattice


def _replay_mpi(lattice_mod, z, p, precision=0):
    """The reference MPI loop body: detection (stringsExist latch) then a step
    with energy, through the C ABI."""
    p = p.copy()
    p.precision = precision
    lat = lattice_mod.Lattice(p)
    ic = lattice_mod.random_phase_ic(p, int(z["seed"]))
    lat.set_state(ic, ic, 0)
    nt, sf = int(z["nt"]), int(z["save_freq"])
    energies, frames, exist = [], [], True
    for n in range(nt):
        if n % sf == 0 and n >= p.damped_nt and exist:
            xyz = lat.detect(0)
            frames.append(xyz)
            exist = len(xyz) > 0
        energies.append(lat.step_diag().energy)
    st = lat.get_slots()
    lat.close()
    return st, np.array(energies), frames


@pytest.mark.parametrize("name", ["ref_mpi_ah_c1", "ref_mpi_ah_prs", "ref_mpi_ah_global", "ref_moore_mpi"])
def test_mpi_programs_against_reference(lattice_mod, name):
    z = load_golden(name)
    p = params_from_json(z["params"])
    st, energy, frames = _replay_mpi(lattice_mod, z, p)
    assert_fields_close(st, z["final"])
    ref_e = z["energy"]
    if np.all(np.isnan(ref_e)):       # g = 0: the reference's MPI energy is 0/0
        assert np.all(np.isnan(energy))
    else:
        np.testing.assert_allclose(energy, ref_e, rtol=TOL, atol=0)
    assert [len(f) for f in frames] == z["frame_counts"].tolist()
    np.testing.assert_allclose(np.concatenate(frames), z["frame_xyz"], rtol=0, atol=1e-9)


@pytest.mark.parametrize("name", ["ref_evol_ah_periodic", "ref_evol_ah_fixed", "ref_moore_evol"])
def test_openmp_programs_against_reference(lattice_mod, name):
    z = load_golden(name)
    p = params_from_json(z["params"])
    lat = lattice_mod.Lattice(p)
    lat.set_slots(z["ic"], 0)
    nt = int(z["nt"])
    out = lat.advance(nt, diag_every=1)
    E = np.array([o[1] for o in out])
    D = np.array([o[2] for o in out])
    now, _ = lat.get_state()
    assert_fields_close(now, z["final_newest"])
    np.testing.assert_allclose(E, z["energy"], rtol=TOL, atol=0)
    if p.model == 0:
        c = p.nx * p.ny * p.nz if p.bc == 0 else (p.nx - 2) * (p.ny - 2) * (p.nz - 2)
        np.testing.assert_allclose(D / c, z["deviation"], rtol=TOL, atol=0)
    else:
        c = (p.nx - 2) * (p.ny - 2) * (p.nz - 2)
        np.testing.assert_allclose(D / c / c, z["deviation"], rtol=TOL, atol=0)
    lat.close()


def test_config1_physics_64cubed_300_steps(lattice_mod, oracle_mod):
    """Config-1 physics (lambda=2, e=1, eta=1, dx=0.5, dt=0.1, Minkowski) on a
    64^3 seeded random-phase lattice, 300 steps, energy/Gauss every 10 steps."""
    from axions_gb300.params import ENERGY_EVOLUTION, make_params
    p = make_params(0, n=64, d=0.5, dt=0.1, lam=2.0, eta=1.0, g=1.0, damped_nt=0, dampFac=0.0, alpha=0.0,
                    energy_form=ENERGY_EVOLUTION)
    st = oracle_mod.random_phase_ic(p, 42)
    ref_diag = oracle_mod.evolve(p, st, 0, 300, diag_every=10)
    lat = lattice_mod.Lattice(p)
    lat.set_state(lattice_mod.random_phase_ic(p, 42), None, 0)
    out = lat.advance(300, diag_every=10)
    gpu = lat.get_slots()
    assert_fields_close(gpu, st)
    assert [o[0] for o in out] == [r[0] for r in ref_diag]
    np.testing.assert_allclose([o[1] for o in out], [r[1] for r in ref_diag], rtol=TOL)
    np.testing.assert_allclose([o[2] for o in out], [r[2] for r in ref_diag], rtol=1e-10)
    lat.close()


def test_prs_moore_48cubed(lattice_mod, oracle_mod):
    """Moore model, charges 1 and 2, PRS friction, independent phases, 100 steps."""
    from axions_gb300.params import MODEL_MOORE, make_params
    p = make_params(MODEL_MOORE, nx=48, ny=40, nz=36, d=0.5, dt=0.1, lam=2.0, lambda2=2.0, lambda12=0.3,
                    eta=1.0, eta2=1.0, q1=1.0, q2=2.0, g=1.0, damped_nt=20, dampFac=0.5, alpha=3.0)
    st = oracle_mod.random_phase_ic(p, 7, independent=True)
    ref = oracle_mod.evolve(p, st, 0, 100, diag_every=25)
    lat = lattice_mod.Lattice(p)
    lat.set_state(lattice_mod.random_phase_ic(p, 7, True), None, 0)
    out = lat.advance(100, diag_every=25)
    assert_fields_close(lat.get_slots(), st)
    np.testing.assert_allclose([o[1] for o in out], [r[1] for r in ref], rtol=TOL)
    for fld in (0, 1):   # fields agree to ~1e-13 here; a root of the bilinear
        # quadratic amplifies that near double roots, so crossings agree to 1e-6
        got, ref = lat.detect(fld), oracle_mod.detect(p, st, 100, fld)
        assert got.shape == ref.shape
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-6)
    lat.close()


@pytest.mark.parametrize("model", [0, 1])
def test_detection_bit_exact_on_identical_fields(lattice_mod, oracle_mod, model):
    from axions_gb300.params import make_params
    p = make_params(model, nx=40, ny=36, nz=32, d=0.5, dt=0.1, lam=2.0, g=1.0, damped_nt=0, alpha=0.0)
    st = oracle_mod.random_phase_ic(p, 3, independent=True)
    oracle_mod.evolve(p, st, 0, 20)
    lat = lattice_mod.Lattice(p)
    lat.set_slots(st, 20)
    for fld in range(1 + model):
        ref = oracle_mod.detect(p, st, 20, fld)
        got = lat.detect(fld)
        assert got.shape == ref.shape and len(ref) > 100
        assert np.array_equal(got, ref)
        w_ref, t_ref = oracle_mod.winding(p, st, 20, fld)
        w_got, t_got = lat.winding(fld)
        assert t_got == t_ref and np.array_equal(w_got, w_ref)
    lat.close()


def test_winding_conserved_through_every_cube(lattice_mod):
    """Strings neither begin nor end: the outward windings of the six faces of
    every cube sum to zero (exactly, as every edge enters two faces with
    opposite orientation)."""
    from axions_gb300.params import make_params
    p = make_params(0, nx=24, ny=20, nz=16)
    lat = lattice_mod.Lattice(p)
    ic = lattice_mod.random_phase_ic(p, 11)
    lat.set_state(ic, ic, 0)
    w, tot = lat.winding(0)
    assert tot > 0
    W = w.reshape(3, p.nx, p.ny, p.nz).astype(np.int32)
    div = (np.roll(W[0], -1, 0) - W[0]) + (np.roll(W[1], -1, 1) - W[1]) + (np.roll(W[2], -1, 2) - W[2])
    assert np.all(div == 0)
    assert tot == int(np.abs(W).sum())
    lat.close()


def test_diagnostics_read_only_and_consistent(lattice_mod, oracle_mod):
    from axions_gb300.params import ENERGY_EVOLUTION, make_params
    p = make_params(0, nx=20, ny=18, nz=16, d=0.5, dt=0.1, lam=2.0, g=1.0, damped_nt=0, alpha=3.0,
                    energy_form=ENERGY_EVOLUTION)
    st = oracle_mod.random_phase_ic(p, 5)
    oracle_mod.evolve(p, st, 0, 7)
    lat = lattice_mod.Lattice(p)
    lat.set_slots(st, 7)
    before = lat.get_slots()
    d1 = lat.diagnostics()
    assert np.array_equal(lat.get_slots(), before) and lat.time_step == 7
    d2 = lat.step_diag()
    ref = oracle_mod.diagnostics(p, st, 7)
    assert d1.time_step == d2.time_step == 7
    assert d1.energy == d2.energy and d1.gauss_abs_sum == d2.gauss_abs_sum
    np.testing.assert_allclose([d1.energy, d1.gauss_abs_sum], [ref.energy, ref.gauss_abs_sum], rtol=1e-12)
    lat.close()


def test_capacity_error_keeps_count(lattice_mod):
    import ctypes
    from axions_gb300.params import LAT_ERR_CAPACITY, make_params
    p = make_params(0, n=16)
    lat = lattice_mod.Lattice(p)
    ic = lattice_mod.random_phase_ic(p, 1)
    lat.set_state(ic, ic, 0)
    full = lat.detect(0)
    buf = np.zeros((5, 3))
    cnt = ctypes.c_int64(0)
    rc = lat.L.lat_detect_crossings(lat.h, 0, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 5,
                                    ctypes.byref(cnt))
    assert rc == LAT_ERR_CAPACITY and cnt.value == len(full)
    assert np.array_equal(buf, full[:5])
    lat.close()


def test_fp32_path_tracks_fp64(lattice_mod):
    """FP32 fields with FP64 reductions stay close to the FP64 path over a short run."""
    from axions_gb300.params import ENERGY_EVOLUTION, F32, make_params
    p = make_params(0, n=32, d=0.5, dt=0.1, lam=2.0, g=1.0, damped_nt=0, alpha=0.0, energy_form=ENERGY_EVOLUTION)
    ic = lattice_mod.random_phase_ic(p, 9)
    outs = []
    for prec in (0, F32):
        q = p.copy()
        q.precision = prec
        lat = lattice_mod.Lattice(q)
        lat.set_state(ic, ic, 0)
        outs.append((lat.advance(20, diag_every=5), lat.get_slots()))
        lat.close()
    (d64, s64), (d32, s32) = outs
    mx, l2 = normwise(s32, s64)
    assert l2 < 1e-4, l2
    np.testing.assert_allclose([d[1] for d in d32], [d[1] for d in d64], rtol=1e-5)
    np.testing.assert_allclose([d[2] for d in d32], [d[2] for d in d64], rtol=1e-3)


def test_twopass_strict_bitwise_equals_onepass(lattice_mod):
    """The two-pass FP64 step computes each link's sin/cos and plaquette sine
    once per site; in strict mode it must give the very same doubles as the
    one-pass kernel that evaluates them per use (as the reference does)."""
    from axions_gb300.params import ENERGY_EVOLUTION, make_params
    p = make_params(0, nx=30, ny=26, nz=22, d=0.5, dt=0.1, lam=2.0, g=1.0, damped_nt=5, dampFac=0.5, alpha=3.0,
                    energy_form=ENERGY_EVOLUTION)
    ic = lattice_mod.random_phase_ic(p, 17)
    res = []
    for variant in (0, 1):
        q = p.copy()
        q.kernel_variant = variant
        lat = lattice_mod.Lattice(q)
        lat.set_state(ic, ic, 0)
        d = lat.advance(30, diag_every=3)
        res.append((lat.get_slots(), d))
        lat.close()
    assert np.array_equal(res[0][0], res[1][0])
    assert res[0][1] == res[1][1]


@pytest.mark.parametrize("d", [0.5, 0.35])
def test_fp64_fast_meets_parity_bar(lattice_mod, oracle_mod, d):
    """LAT_F64_FAST (fused multiply-adds) against the oracle: 48^3, 300 steps,
    config-1 physics; also a spacing that is not a power of two."""
    from axions_gb300.params import ENERGY_EVOLUTION, F64_FAST, make_params
    p = make_params(0, n=48, d=d, dt=0.1, lam=2.0, eta=1.0, g=1.0, damped_nt=0, alpha=0.0,
                    energy_form=ENERGY_EVOLUTION)
    st = oracle_mod.random_phase_ic(p, 4)
    ref = oracle_mod.evolve(p, st, 0, 300, diag_every=50)
    q = p.copy()
    q.precision = F64_FAST
    lat = lattice_mod.Lattice(q)
    lat.set_state(lattice_mod.random_phase_ic(p, 4), None, 0)
    out = lat.advance(300, diag_every=50)
    assert_fields_close(lat.get_slots(), st)
    np.testing.assert_allclose([o[1] for o in out], [r[1] for r in ref], rtol=TOL)
    lat.close()


def test_strict_non_power_of_two_spacing(lattice_mod, oracle_mod):
    from axions_gb300.params import ENERGY_EVOLUTION, make_params
    p = make_params(0, nx=36, ny=32, nz=28, d=0.35, dt=0.05, lam=1.0, eta=1.0, g=0.8, damped_nt=10, dampFac=0.5,
                    alpha=3.0, energy_form=ENERGY_EVOLUTION)
    st = oracle_mod.random_phase_ic(p, 8)
    ref = oracle_mod.evolve(p, st, 0, 60, diag_every=20)
    lat = lattice_mod.Lattice(p)
    lat.set_state(lattice_mod.random_phase_ic(p, 8), None, 0)
    out = lat.advance(60, diag_every=20)
    assert_fields_close(lat.get_slots(), st)
    np.testing.assert_allclose([o[1] for o in out], [r[1] for r in ref], rtol=TOL)
    np.testing.assert_allclose([o[2] for o in out], [r[2] for r in ref], rtol=1e-10)
    lat.close()


@pytest.mark.parametrize("bc", [0, 1])
@pytest.mark.parametrize("sides", [(70, 29, 45), (70, 29, 44), (10, 3, 4)])
def test_fp32_tiled_kernel_odd_sizes(lattice_mod, bc, sides):
    """The tiled FP32 kernel (x-march, shared-memory staging) on sides that are
    not multiples of its tile (32 x 8) or of its x-chunk, periodic and fixed
    boundaries: it must track the FP64 path, and the one-pass FP32 kernel, to
    FP32 accuracy.  Periodic nz = 44 and nz = 4 take the 16-byte staging; the
    10 x 3 x 4 lattice is narrower than the tile on both y and z."""
    from axions_gb300.params import ENERGY_EVOLUTION, F32, make_params
    nx, ny, nz = sides
    p = make_params(0, nx=nx, ny=ny, nz=nz, d=0.5, dt=0.1, lam=2.0, g=1.0, damped_nt=3, dampFac=0.5, alpha=3.0,
                    energy_form=ENERGY_EVOLUTION, bc=bc)
    ic = lattice_mod.random_phase_ic(p, 23)
    res = {}
    for name, prec, var in (("f64", 0, 0), ("f32", F32, 0), ("f32_onepass", F32, 1)):
        q = p.copy()
        q.precision = prec
        q.kernel_variant = var
        lat = lattice_mod.Lattice(q)
        lat.set_state(ic, ic, 0)
        d = lat.advance(12, diag_every=4)
        res[name] = (lat.get_slots(), d)
        lat.close()
    s64 = res["f64"][0]
    for name in ("f32", "f32_onepass"):
        s, d = res[name]
        mx, l2 = normwise(s, s64)
        assert l2 < 2e-6 and mx < 2e-5, (name, mx, l2)
        np.testing.assert_allclose([x[1] for x in d], [x[1] for x in res["f64"][1]], rtol=1e-5)
        np.testing.assert_allclose([x[2] for x in d], [x[2] for x in res["f64"][1]], rtol=1e-4)


@pytest.mark.parametrize("bc,charges,current", [(0, (1.0, 2.0), 0), (1, (2.0, 1.0), 1), (0, (3.0, -1.0), 1)])
def test_fp32_tiled_moore(lattice_mod, bc, charges, current):
    """Moore model on the tiled FP32 kernel (two scalars, link factors
    e^{i q theta} as powers of e^{i theta}) against the FP64 path and the
    one-pass FP32 kernel, on sides that are not tile multiples."""
    from axions_gb300.params import ENERGY_EVOLUTION, F32, MODEL_MOORE, make_params
    q1, q2 = charges
    p = make_params(MODEL_MOORE, nx=40, ny=27, nz=37, d=0.5, dt=0.1, lam=2.0, lambda2=2.0, lambda12=0.3, eta=1.0,
                    eta2=1.0, q1=q1, q2=q2, g=0.8, damped_nt=3, dampFac=0.5, alpha=3.0, bc=bc,
                    energy_form=ENERGY_EVOLUTION, moore_current=current)
    ic = lattice_mod.random_phase_ic(p, 31, True)
    res = {}
    for name, prec, var in (("f64", 0, 0), ("f32", F32, 0), ("f32_onepass", F32, 1)):
        q = p.copy()
        q.precision = prec
        q.kernel_variant = var
        lat = lattice_mod.Lattice(q)
        lat.set_state(ic, ic, 0)
        d = lat.advance(12, diag_every=4)
        res[name] = (lat.get_slots(), d)
        lat.close()
    s64 = res["f64"][0]
    for name in ("f32", "f32_onepass"):
        s, d = res[name]
        mx, l2 = normwise(s, s64)
        assert l2 < 3e-6 and mx < 3e-5, (name, mx, l2)
        np.testing.assert_allclose([x[1] for x in d], [x[1] for x in res["f64"][1]], rtol=1e-5)
        np.testing.assert_allclose([x[2] for x in d], [x[2] for x in res["f64"][1]], rtol=1e-4)


@pytest.mark.parametrize("model", [0, 1])
@pytest.mark.parametrize("sides", [(70, 29, 44), (33, 17, 32), (40, 12, 100), (24, 20, 36), (10, 3, 4), (9, 5, 8)])
def test_fp32_tiled_vector_staging_is_bitwise_the_element_staging(lattice_mod, model, sides):
    """With periodic z and nz a multiple of 4 the tiled FP32 step stages its
    planes in 16-byte row chunks; kernel_variant 2 stages one element per
    copy.  Both fill the same shared-memory positions and the arithmetic is
    the same, so fields and diagnostics are bitwise equal.  The sides cover a
    partial last z tile, one tile wrapping at both ends, four tiles, a right
    edge cut to the lattice, and lattices narrower than the tile (nz = 4,
    ny = 3), whose halo indices wrap within one period."""
    from axions_gb300.params import ENERGY_EVOLUTION, F32, MODEL_MOORE, make_params
    nx, ny, nz = sides
    if model == 0:
        p = make_params(0, nx=nx, ny=ny, nz=nz, d=0.5, dt=0.1, lam=2.0, g=1.0, damped_nt=3, dampFac=0.5, alpha=3.0,
                        energy_form=ENERGY_EVOLUTION, precision=F32)
    else:
        p = make_params(MODEL_MOORE, nx=nx, ny=ny, nz=nz, d=0.5, dt=0.1, lam=2.0, lambda2=2.0, lambda12=0.5, eta=1.0,
                        eta2=1.0, q1=2.0, q2=1.0, g=1.0, damped_nt=3, dampFac=0.5, alpha=3.0,
                        energy_form=ENERGY_EVOLUTION, precision=F32)
    ic = lattice_mod.random_phase_ic(p, 31, independent=model == 1)
    out = []
    for variant in (0, 2):
        q = p.copy()
        q.kernel_variant = variant
        with lattice_mod.Lattice(q) as lat:
            lat.set_state(ic, ic, 0)
            d = lat.advance(11, diag_every=3)
            out.append((lat.get_slots(), d))
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1]
