"""String length by greedy chaining (ic_w_evolution.cpp:961-1087) on the GPU,
through the C ABI, against the reference's own per-step lengths (golden
fixtures made by running ic_w_evolution) and the oracle.

Bar: bit-exact.  On the same crossing list both GPU methods (the link-graph
component walk and the cooperative exhaustive walk) add the same doubles in
the reference's order.  With g = 0 the gauge links stay 0, so the FP64 step uses
no transcendental with a non-trivial argument and the GPU-evolved fields, and
hence the lengths, equal the reference's too.
"""
import numpy as np
import pytest

from conftest import load_golden, params_from_json

pytestmark = pytest.mark.gpu

ICW = ["ref_icw_len_periodic", "ref_icw_len_wide", "ref_icw_len_fixed", "ref_icw_len_nosplit"]


@pytest.fixture(scope="module")
def lattice_mod():
    from axions_gb300 import lattice
    lattice.load_library()
    return lattice


def _methods(p, lattice_mod):
    from axions_gb300.params import BC_PERIODIC
    if p.bc == BC_PERIODIC:
        return [lattice_mod.CHAIN_HASH, lattice_mod.CHAIN_EXHAUSTIVE]
    return [lattice_mod.CHAIN_EXHAUSTIVE]


@pytest.mark.parametrize("name", ICW)
def test_chaining_of_reference_crossings_bit_exact(lattice_mod, oracle_mod, name):
    """Crossing lists of the reference run (oracle fields, pinned bit-exact),
    chained on the GPU: every step's L0, L1 equal the reference's."""
    O = oracle_mod
    z = load_golden(name)
    p = params_from_json(z["params"])
    split = bool(z["split"])
    st = O.icfunc_random_ic(p, int(z["seed"]))
    for n in range(int(z["nt"])):
        xyz = O.detect(p, st, n, 0)
        for m in _methods(p, lattice_mod):
            L0, L1 = lattice_mod.string_length_points(p, xyz, split, m)
            assert (L0, L1) == (z["L0"][n], z["L1"][n]), (n, m, len(xyz))
        O.step(p, st, n)


@pytest.mark.parametrize("name", ["ref_icw_len_periodic", "ref_icw_len_fixed"])
def test_gpu_evolved_lengths_match_reference(lattice_mod, oracle_mod, name):
    """ic_w_evolution's loop on the GPU: IC, then per step detection and
    chaining on the device (lat_string_length) and an FP64 step."""
    z = load_golden(name)
    p = params_from_json(z["params"])
    split = bool(z["split"])
    st = oracle_mod.icfunc_random_ic(p, int(z["seed"]))
    lat = lattice_mod.Lattice(p)
    lat.set_slots(st, 0)
    for n in range(int(z["nt"])):
        L0, L1, cnt = lat.string_length(0, split)
        assert (L0, L1) == (z["L0"][n], z["L1"][n]), (n, cnt)
        lat.step()
    N = p.nx * p.ny * p.nz
    last = (int(z["nt"]) - 1) % 2
    got = lat.get_slots()[:2, last].reshape(2, N)
    assert np.array_equal(got, z["final_phi"])
    lat.close()


def _oracle_pair(oracle_mod, p, xyz, split=True):
    return oracle_mod.string_length(p, xyz, split)


def test_ties_duplicates_and_images(lattice_mod, oracle_mod):
    """Points on a grid (many exactly equal distances: the last index must
    win), duplicated points (distance 0), points on the box faces (minimum
    image), in a scrambled order."""
    from axions_gb300.params import make_params
    p = make_params(0, nx=12, ny=10, nz=8, d=0.5)
    rng = np.random.default_rng(1)
    # (i - x0)*dx with x0 = 5, 4, 3: the box is [-2.5, 3.5] x [-2, 3] x [-1.5, 2.5]
    g = np.stack(np.meshgrid((np.arange(12) - 5) * 0.5, (np.arange(10) - 4) * 0.5, (np.arange(8) - 3) * 0.5,
                             indexing="ij"), -1).reshape(-1, 3)
    keep = g[rng.random(len(g)) < 0.6]
    faces = keep.copy()
    faces[:40, 0] = 3.5   # the upper face, the periodic image of x = -2.5
    pts = np.concatenate([keep, keep[:50], faces[:40]])[rng.permutation(len(keep) + 90)]
    for split in (True, False):
        want = _oracle_pair(oracle_mod, p, pts, split)
        for m in (lattice_mod.CHAIN_HASH, lattice_mod.CHAIN_EXHAUSTIVE):
            assert lattice_mod.string_length_points(p, pts, split, m) == want


def test_wide_cutoff_and_few_cells(lattice_mod, oracle_mod):
    """dx = 1: the cutoff radius is 3 cells, so the hash has 1-3 cells per axis
    (offsets that wrap onto each other)."""
    from axions_gb300.params import make_params
    rng = np.random.default_rng(2)
    for n in (4, 7, 9):
        p = make_params(0, nx=n, ny=n + 1, nz=n + 2, d=1.0)
        lo = -np.array([(n - 1) // 2, n // 2, (n + 1) // 2], dtype=np.float64)
        L = np.array([n, n + 1, n + 2], dtype=np.float64)
        pts = lo + rng.random((300, 3)) * L
        want = _oracle_pair(oracle_mod, p, pts)
        for m in (lattice_mod.CHAIN_HASH, lattice_mod.CHAIN_EXHAUSTIVE):
            assert lattice_mod.string_length_points(p, pts, True, m) == want, (n, m)


def test_edge_cases(lattice_mod, oracle_mod):
    from axions_gb300.lattice import LatticeError
    from axions_gb300.params import make_params
    p = make_params(0, nx=16, ny=16, nz=16, d=0.5)
    c0 = 0.75
    for m in (lattice_mod.CHAIN_AUTO, lattice_mod.CHAIN_HASH, lattice_mod.CHAIN_EXHAUSTIVE):
        assert lattice_mod.string_length_points(p, np.zeros((0, 3)), True, m) == (0.0, 0.0)
        assert lattice_mod.string_length_points(p, np.array([[0.1, 0.2, 0.3]]), True, m) == (c0, 0.0)
        same = np.tile([[1.0, 2.0, -3.0]], (7, 1))
        assert lattice_mod.string_length_points(p, same, True, m) == _oracle_pair(oracle_mod, p, same)
    # outside the box: the hash refuses, the exhaustive walk follows the reference
    out = np.array([[0.0, 0.0, 0.0], [40.0, 0.0, 0.0], [40.2, 0.0, 0.0]])
    with pytest.raises(LatticeError):
        lattice_mod.string_length_points(p, out, True, lattice_mod.CHAIN_HASH)
    want = _oracle_pair(oracle_mod, p, out)
    assert lattice_mod.string_length_points(p, out, True, lattice_mod.CHAIN_AUTO) == want
    assert lattice_mod.string_length_points(p, out, True, lattice_mod.CHAIN_EXHAUSTIVE) == want


def test_hash_equals_exhaustive_at_size(lattice_mod):
    """Global strings on a 96^3 lattice after 200 FP32 steps (about 4*10^4
    crossings, beyond what the O(M^2) oracle does in a test): the link-graph
    walk and the cooperative exhaustive walk agree bit for bit, and the total
    lies within the range the plaquette winding estimate gives."""
    from axions_gb300.params import F32, make_params
    p = make_params(0, n=96, d=0.5, dt=0.1, lam=2.0, g=0.0, damped_nt=20, dampFac=0.5, alpha=0.0)
    p.precision = F32
    lat = lattice_mod.Lattice(p)
    lat.random_phase_ic_device(7)
    lat.advance(200)
    a = lat.string_length(0, True, lattice_mod.CHAIN_HASH)
    b = lat.string_length(0, True, lattice_mod.CHAIN_EXHAUSTIVE)
    assert a == b and 5000 < a[2] < 400000, a
    _, wabs = lat.winding(0, want_array=False)
    est = wabs * p.dx
    assert 0.2 * est < a[0] + a[1] < 3.0 * est
    lat.close()


def test_moore_second_field(lattice_mod, oracle_mod):
    from axions_gb300.params import MODEL_MOORE, make_params
    p = make_params(MODEL_MOORE, nx=14, ny=12, nz=10, d=0.5, dt=0.1, damped_nt=0, dampFac=0.0, alpha=0.0)
    st = oracle_mod.random_phase_ic(p, 3, independent=True)
    lat = lattice_mod.Lattice(p)
    lat.set_slots(st, 0)
    for field in (0, 1):
        want = _oracle_pair(oracle_mod, p, oracle_mod.detect(p, st, 0, field))
        got = lat.string_length(field, True)
        assert got[:2] == want
    lat.close()


def test_cooperative_walk_barrier_wait_is_bounded(lattice_mod, oracle_mod):
    """The exhaustive walk's grid barrier waits a bounded number of polls.
    With one barrier arrival that never comes and a bound of 1000 polls, the
    call returns LAT_ERR_TIMEOUT at once (no fault, no trap), and the device
    stays usable: the same call with the default bound then gives the
    reference's lengths."""
    import time

    from axions_gb300.params import LAT_ERR_TIMEOUT
    z = load_golden("ref_icw_len_fixed")
    p = params_from_json(z["params"])
    st = oracle_mod.icfunc_random_ic(p, int(z["seed"]))
    xyz = oracle_mod.detect(p, st, 0, 0)
    assert len(xyz) > 0
    L = lattice_mod.load_library()
    assert L.lat_set_chain_wait(1000, 1) == 0
    try:
        t0 = time.perf_counter()
        with pytest.raises(lattice_mod.LatticeError) as ei:
            lattice_mod.string_length_points(p, xyz, True, lattice_mod.CHAIN_EXHAUSTIVE)
        elapsed = time.perf_counter() - t0
    finally:
        assert L.lat_set_chain_wait(0, 0) == 0
    assert ei.value.code == LAT_ERR_TIMEOUT and "barrier" in str(ei.value)
    assert elapsed < 2.0, elapsed
    L0, L1 = lattice_mod.string_length_points(p, xyz, True, lattice_mod.CHAIN_EXHAUSTIVE)
    assert (L0, L1) == (z["L0"][0], z["L1"][0])
    assert L.lat_set_chain_wait(-1, 0) < 0 and L.lat_set_chain_wait(0, -1) < 0
