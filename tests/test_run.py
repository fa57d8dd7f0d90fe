"""lat_run: a whole run from host state to host state in one call.

It must give, bit for bit, what lat_set_state + lat_advance + lat_get_state
give.  The cases cover both FP64 forms, FP32 and Moore, periodic, fixed and
Neumann walls, a first step that is an energy/Gauss step, one and two steps,
a single output array, two runs on one handle, and a stationary start passed
as one array for both levels (uploaded once and copied on the device) with
only the final level downloaded.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lattice_mod():
    from axions_gb300 import lattice
    lattice.load_library()
    return lattice


def start_state(lattice_mod, p, seed):
    """A state with distinct, non-trivial levels: the seeded IC advanced a few steps."""
    ic = lattice_mod.random_phase_ic(p, seed, independent=p.model == 1)
    with lattice_mod.Lattice(p) as lat:
        lat.set_state(ic, ic, 0)
        lat.advance(5)
        now, past = lat.get_state()
        return now, past, lat.time_step


def sequential(lattice_mod, p, now, past, t0, nsteps, diag_every):
    with lattice_mod.Lattice(p) as lat:
        lat.set_state(now, past, t0)
        d = lat.advance(nsteps, diag_every)
        a, b = lat.get_state()
        return d, a, b


def make(lattice_mod, precision=0, bc=0, model=0):
    from axions_gb300.params import ENERGY_EVOLUTION, MODEL_MOORE, make_params
    if model == 0:
        return make_params(0, nx=40, ny=36, nz=32, d=0.5, dt=0.1, lam=2.0, g=1.0, damped_nt=3, dampFac=0.5,
                           alpha=3.0, energy_form=ENERGY_EVOLUTION, precision=precision, bc=bc)
    return make_params(MODEL_MOORE, nx=24, ny=20, nz=16, d=0.5, dt=0.1, lam=2.0, lambda2=2.0, lambda12=0.3,
                       eta=1.0, eta2=1.0, q1=1.0, q2=2.0, g=1.0, energy_form=ENERGY_EVOLUTION, precision=precision)


@pytest.mark.parametrize("case", [
    dict(precision=0, bc=0, nsteps=7, diag_every=3),     # strict, overlap, first step a diagnostic step
    dict(precision=0, bc=0, nsteps=7, diag_every=4),     # strict, overlap, later diagnostic steps only
    dict(precision=0, bc=0, nsteps=1, diag_every=5),     # one step: first and last
    dict(precision=0, bc=0, nsteps=2, diag_every=0),
    dict(precision=2, bc=0, nsteps=6, diag_every=2),     # fast FP64, overlap
    dict(precision=0, bc=1, nsteps=5, diag_every=5),     # fixed walls, overlap
    dict(precision=0, bc=2, nsteps=4, diag_every=2),     # Neumann walls: the three calls in sequence
    dict(precision=1, bc=0, nsteps=5, diag_every=5),     # FP32: the three calls in sequence
    dict(precision=0, bc=0, nsteps=4, diag_every=2, model=1),  # Moore FP64: in sequence
])
def test_run_is_bitwise_the_three_calls(lattice_mod, case):
    p = make(lattice_mod, case["precision"], case["bc"], case.get("model", 0))
    now, past, t0 = start_state(lattice_mod, p, 7)
    ref_d, ref_now, ref_past = sequential(lattice_mod, p, now, past, t0, case["nsteps"], case["diag_every"])
    with lattice_mod.Lattice(p) as lat:
        d, got_now, got_past = lat.run(now, past, t0, case["nsteps"], case["diag_every"])
        assert lat.time_step == t0 + case["nsteps"]
    assert d == ref_d
    assert np.array_equal(got_now, ref_now) and np.array_equal(got_past, ref_past)


def test_run_twice_on_one_handle_and_one_output(lattice_mod):
    p = make(lattice_mod)
    now, past, t0 = start_state(lattice_mod, p, 11)
    _, ref_now, ref_past = sequential(lattice_mod, p, now, past, t0, 6, 3)
    _, ref_now2, _ = sequential(lattice_mod, p, ref_now, ref_past, t0 + 6, 3, 0)
    nc, N = ref_now.shape
    with lattice_mod.Lattice(p) as lat:
        lat.step(2)   # earlier work on the handle's stream
        _, a, b = lat.run(now, past, t0, 6, 3)
        assert np.array_equal(a, ref_now) and np.array_equal(b, ref_past)
        out = np.empty(nc * N)
        _, a2, _ = lat.run(a, b, t0 + 6, 3, 0, now_out=out)
        assert np.array_equal(a2, ref_now2)
        # the handle continues from the run's final state
        lat.step(1)
    with pytest.raises(ValueError):
        with lattice_mod.Lattice(p) as lat:
            lat.run(now, past, t0, 1, 0, now_out=np.empty(3))


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_stationary_start_as_one_array(lattice_mod, precision):
    """The same array for both levels (mpi_evolution.cpp:155-162) gives bit for
    bit what two equal arrays give, through lat_set_state and lat_run, and the
    run may skip the past level's download."""
    p = make(lattice_mod, precision)
    ic = lattice_mod.random_phase_ic(p, 13)
    twin = ic.copy()
    ref_d, ref_now, ref_past = sequential(lattice_mod, p, ic, twin, 0, 6, 3)
    with lattice_mod.Lattice(p) as lat:
        lat.set_state(ic, twin, 0)
        ra, rb = lat.get_state()
    with lattice_mod.Lattice(p) as lat:
        lat.set_state(ic, None, 0)
        a, b = lat.get_state()
        assert np.array_equal(a, ra) and np.array_equal(b, rb)
        d, got_now, got_past = lat.run(ic, None, 0, 6, 3, past_level=False)
        assert got_past is None
        assert d == ref_d and np.array_equal(got_now, ref_now)
        _, past_now = lat.get_state()
        assert np.array_equal(past_now, ref_past)
