"""Pin the oracle (CPU restatement) against outputs of the reference itself.

The fixtures in tests/golden/ were produced by running the reference programs
(tests/golden/make_golden.py).  Fields, energies and crossing lists must agree
bit for bit; the only exception is mooreEvol's deviation column, which the
reference normalises per site before summing (mooreEvol.cpp:383), so it is
compared to 1e-13 relative.
"""
import numpy as np
import pytest

from conftest import load_golden, params_from_json

MPI_CASES = ["ref_mpi_ah_c1", "ref_mpi_ah_prs", "ref_mpi_ah_global", "ref_moore_mpi"]
OMP_CASES = ["ref_evol_ah_periodic", "ref_evol_ah_fixed", "ref_moore_evol"]
BC_CASES = ["ref_moore_evol_neumann", "ref_evol_bc_neumann", "ref_evol_bc_absorbing", "ref_evol_bc_absorbing_neumann",
            "ref_evol_bc_fixed_zper", "ref_evol_bc_per_zfixed"]


def evolution_deviation(p, D):
    """evolution.cpp:1404-1408: the x/y and z normalisations follow each axis's boundary."""
    from axions_gb300.params import BCZ_AS_XY, BCZ_PERIODIC, BC_PERIODIC
    pxy = p.bc == BC_PERIODIC
    pz = p.bc_z == BCZ_PERIODIC or (p.bc_z == BCZ_AS_XY and pxy)
    D = D / (p.nx * p.ny) if pxy else D / ((p.nx - 2) * (p.ny - 2))
    return D / p.nz if pz else D / (p.nz - 2)


def test_random_ic_matches_reference_mt19937(oracle_mod):
    from axions_gb300.params import make_params
    z = load_golden("ref_mpi_ah_ic_s7")
    p = make_params(0, nx=int(z["nx"]), ny=int(z["ny"]), nz=int(z["nz"]))
    st = oracle_mod.random_phase_ic(p, int(z["seed"]))
    assert np.array_equal(st, z["ic"])


def _run_mpi_program(O, z, p):
    """Replay the reference loop: detection (with the stringsExist latch) then step."""
    O.set_threads(1)
    st = O.random_phase_ic(p, int(z["seed"]))
    nt, sf = int(z["nt"]), int(z["save_freq"])
    energies, frames, exist = [], [], True
    for n in range(nt):
        if n % sf == 0 and n >= p.damped_nt and exist:
            xyz = O.detect(p, st, n, 0)
            frames.append(xyz)
            exist = len(xyz) > 0
        energies.append(O.step(p, st, n, diag=True).energy)
    return st, np.array(energies), frames


@pytest.mark.parametrize("name", MPI_CASES)
def test_mpi_programs_bit_exact(oracle_mod, name):
    z = load_golden(name)
    p = params_from_json(z["params"])
    st, energy, frames = _run_mpi_program(oracle_mod, z, p)
    assert np.array_equal(st, z["final"]), "fields (both time slots) differ from the reference"
    assert np.array_equal(energy, z["energy"], equal_nan=True)
    assert [len(f) for f in frames] == z["frame_counts"].tolist()
    assert np.array_equal(np.concatenate(frames), z["frame_xyz"])


@pytest.mark.parametrize("name", OMP_CASES + BC_CASES)
def test_openmp_programs_bit_exact(oracle_mod, name):
    O = oracle_mod
    O.set_threads(1)
    z = load_golden(name)
    p = params_from_json(z["params"])
    st = z["ic"].copy()
    nt = int(z["nt"])
    sf = int(z["save_freq"]) if "save_freq" in z.files else 0
    E, D, frames = [], [], []
    for n in range(nt):
        if sf and n % sf == 0:
            O.apply_boundaries(p, st, n)   # detection reads the level after its boundary step
            frames.append(O.detect(p, st, n, 0))
        d = O.step(p, st, n, diag=True)
        E.append(d.energy)
        D.append(d.gauss_abs_sum)
    E, D = np.array(E), np.array(D)
    assert np.array_equal(st[:, (nt + 1) % 2, :], z["final_newest"])
    assert np.array_equal(E, z["energy"])
    if p.model == 0:
        assert np.array_equal(evolution_deviation(p, D), z["deviation"])
    else:
        c = (p.nx - 2) * (p.ny - 2) * (p.nz - 2)               # mooreEvol.cpp:383,697
        np.testing.assert_allclose(D / c / c, z["deviation"], rtol=1e-13, atol=0)
    if sf:
        assert [len(f) for f in frames] == z["frame_counts"].tolist()
        assert np.array_equal(np.concatenate(frames), z["frame_xyz"])


def test_oracle_threads_do_not_change_fields(oracle_mod):
    """The in-place update is race-free: any thread count gives identical fields."""
    O = oracle_mod
    z = load_golden("ref_mpi_ah_prs")
    p = params_from_json(z["params"])
    outs = []
    for t in (1, 4):
        O.set_threads(t)
        st = O.random_phase_ic(p, int(z["seed"]))
        for n in range(int(z["nt"])):
            O.step(p, st, n)
        outs.append(st)
    O.set_threads(1)
    assert np.array_equal(outs[0], outs[1])
    assert np.array_equal(outs[0], z["final"])


ICW_CASES = ["ref_icw_len_periodic", "ref_icw_len_wide", "ref_icw_len_fixed", "ref_icw_len_nosplit"]


@pytest.mark.parametrize("name", ICW_CASES)
def test_string_length_chaining_bit_exact(oracle_mod, name):
    """ic_w_evolution: ic_func's minstd IC, then every step the greedy chaining
    length of the crossings (ic_w_evolution.cpp:961-1087) -- L0 and L1 of every
    step and the final field equal the reference's bit for bit."""
    O = oracle_mod
    z = load_golden(name)
    p = params_from_json(z["params"])
    split = bool(z["split"])
    st = O.icfunc_random_ic(p, int(z["seed"]))
    L0s, L1s = [], []
    for n in range(int(z["nt"])):
        L0, L1 = O.string_length(p, O.detect(p, st, n, 0), split)
        L0s.append(L0)
        L1s.append(L1)
        O.step(p, st, n)
    assert np.array_equal(np.array(L0s), z["L0"])
    assert np.array_equal(np.array(L1s), z["L1"])
    N = p.nx * p.ny * p.nz
    last = (int(z["nt"]) - 1) % 2
    v = st.reshape(5, 2, N)
    assert np.array_equal(v[:2, last], z["final_phi"])


def test_string_length_edge_cases(oracle_mod):
    """Empty list, one point (closes onto itself: the cutoff's square root),
    ties (the last of equally near points wins), and the minimum image."""
    from axions_gb300.params import make_params
    O = oracle_mod
    p = make_params(0, nx=16, ny=16, nz=16, d=0.5)
    c0 = 3 * 0.25
    assert O.string_length(p, np.zeros((0, 3))) == (0.0, 0.0)
    assert O.string_length(p, np.array([[0.1, 0.2, 0.3]])) == (c0, 0.0)
    assert O.string_length(p, np.array([[3.9, 0.0, 0.0]])) == (0.0, c0)
    # 0 -> (2 or 3, both at 0.5): 3 wins; 3 -> 1 (0.5) ... the walk order fixes the sum
    pts = np.array([[0.0, 0, 0], [0.0, 0.5, 0.5], [0.5, 0, 0], [-0.5, 0, 0]])
    L0, _ = O.string_length(p, pts)
    assert L0 > 0
    # periodic image: x = -3.9 and x = 3.9 are 0.2 apart on a box of 8
    L0, L1 = O.string_length(p, np.array([[-3.9, 0.0, 0.0], [3.9, 0.0, 0.0]]))
    assert L0 == 0 and abs(L1 - (0.2 + c0)) < 1e-15


BOOST_CASES = ["ref_boost_ic", "ref_boost_ic_vz"]


def boost_params(z):
    from axions_gb300.params import make_params
    return make_params(0, nx=int(z["nx"]), ny=int(z["ny"]), nz=int(z["nz"]), dx=float(z["dx"]), dy=float(z["dy"]),
                       dz=float(z["dz"]), dt=float(z["dt"]), g=float(z["g"]))


@pytest.mark.parametrize("name", BOOST_CASES)
def test_boost_ic_bit_exact(oracle_mod, name):
    """initialConditions.cpp "boost" (both levels of Data/ic.txt) from the
    straight-string table that singleSemiAnalytic.cpp produced."""
    z = load_golden(name)
    st, off = oracle_mod.boost_ic(boost_params(z), z["profile"][0], z["profile"][1], float(z["sor_h"]), z["v"])
    assert off == 0
    assert np.array_equal(st.reshape(5, 2, -1), z["ic"])


def test_boost_ic_forms_and_table_edge(oracle_mod):
    """The in-process form (ic_func.cpp) differs from the file form only in the
    rounding of the t = dt links; a table shorter than the lattice's reach
    gives |phi| = 1 and A = n/g off its end."""
    z = load_golden("ref_boost_ic")
    p = boost_params(z)
    a = oracle_mod.boost_ic(p, z["profile"][0], z["profile"][1], float(z["sor_h"]), z["v"], 0)[0].reshape(5, 2, -1)
    b = oracle_mod.boost_ic(p, z["profile"][0], z["profile"][1], float(z["sor_h"]), z["v"], 1)[0].reshape(5, 2, -1)
    assert np.array_equal(a[:, 0], b[:, 0]) and np.array_equal(a[:2], b[:2])
    assert np.allclose(a[2:, 1], b[2:, 1], rtol=0, atol=1e-15)
    short = z["profile"][:, :120]        # r < 1.2
    st, off = oracle_mod.boost_ic(p, short[0], short[1], float(z["sor_h"]), z["v"])
    assert off > 0
    v = st.reshape(5, 2, -1)
    far = np.hypot(v[0, 0], v[1, 0])
    assert np.sum(np.isclose(far, 1.0, rtol=0, atol=1e-15)) > 0
    with pytest.raises(RuntimeError):
        oracle_mod.boost_ic(p, short[0], short[1], 0.01, (0.0, 0.0, 0.0))


LOOP_CASES = ["ref_loop_collision_ic", "ref_loop_collision_ic_moving"]


@pytest.mark.parametrize("name", LOOP_CASES)
def test_loop_collision_ic_bit_exact(oracle_mod, name):
    """initialConditions.cpp "loop collision" (both levels of Data/ic.txt): the
    reference's placement on one lattice, and every string moving with dz != dy
    on another."""
    from axions_gb300.params import LOOP_COLLISION_KEYS
    z = load_golden(name)
    geo = {k: z[k] for k in LOOP_COLLISION_KEYS}
    st, off = oracle_mod.loop_collision_ic(boost_params(z), z["profile"][0], z["profile"][1], float(z["sor_h"]), geo)
    assert off == 0
    assert np.array_equal(st.reshape(5, 2, -1), z["ic"])


def test_loop_collision_default_geometry_is_the_references(oracle_mod):
    from axions_gb300.params import LOOP_COLLISION_KEYS, default_loop_collision
    z = load_golden("ref_loop_collision_ic")
    geo = default_loop_collision(int(z["nx"]), int(z["ny"]), int(z["nz"]), 0.5, 0.5, float(z["dz"]))
    for k in LOOP_COLLISION_KEYS:
        assert np.array_equal(np.array(geo[k], dtype=np.float64), z[k]), k


def test_icfunc_loop_collision_bit_exact(oracle_mod):
    """ic_w_evolution's own IC, ic_func.cpp's "loop collision" (:966-1720, the
    ic_type it ships with, :25), then three periodic steps: ic_w_evolution
    writes no IC, so the pin is what it writes -- the newest level after the
    steps and the L0/L1 string lengths of every step, bit for bit -- and its
    energies to 1e-12 (the reference sums them in its own OpenMP order)."""
    from axions_gb300.params import ENERGY_EVOLUTION, icfunc_loop_collision
    O = oracle_mod
    z = load_golden("ref_icfunc_loop_collision")
    p = params_from_json(z["params"])
    geo = icfunc_loop_collision(p.nx, p.ny, p.nz, p.dx, p.dy, p.dz)
    st, off = O.loop_collision_ic(p, z["profile"][0], z["profile"][1], float(z["sor_h"]), geo, form="ic_func")
    assert off == 0
    q = p.copy()
    q.energy_form = ENERGY_EVOLUTION
    diags = O.evolve(q, st.copy(), 0, int(z["nt"]), diag_every=1)
    L0s, L1s = [], []
    for n in range(int(z["nt"])):
        L0, L1 = O.string_length(p, O.detect(p, st, n, 0), True)
        L0s.append(L0)
        L1s.append(L1)
        O.step(p, st, n)
    assert np.array_equal(np.array(L0s), z["L0"])
    assert np.array_equal(np.array(L1s), z["L1"])
    last = (int(z["nt"]) - 1) % 2
    assert np.array_equal(st.reshape(5, 2, -1)[:, last], z["final"])
    assert np.allclose([d[1] for d in diags], z["energy"], rtol=1e-12, atol=0)


def test_icfunc_loop_collision_differs_from_initialconditions_form(oracle_mod):
    """The two loop-collision forms are different ICs on the same geometry (the
    ic_func form measures from lab-frame positions and keeps only the boost
    term of the one-forms), and the ic_func form rejects a string at rest."""
    from axions_gb300.params import icfunc_loop_collision
    z = load_golden("ref_icfunc_loop_collision")
    p = params_from_json(z["params"])
    geo = icfunc_loop_collision(p.nx, p.ny, p.nz, p.dx, p.dy, p.dz)
    a, _ = oracle_mod.loop_collision_ic(p, z["profile"][0], z["profile"][1], float(z["sor_h"]), geo, form="ic_func")
    b, _ = oracle_mod.loop_collision_ic(p, z["profile"][0], z["profile"][1], float(z["sor_h"]), geo)
    assert not np.array_equal(a, b)
    rest = dict(geo, v2s=[0.0, 0.0, 0.0])
    with pytest.raises(RuntimeError):
        oracle_mod.loop_collision_ic(p, z["profile"][0], z["profile"][1], float(z["sor_h"]), rest, form="ic_func")
    oracle_mod.loop_collision_ic(p, z["profile"][0], z["profile"][1], float(z["sor_h"]), rest)


SINE_CASES = ["ref_ng_sine_ic", "ref_ng_sine_ic_b", "ref_simple_sine_ic"]


def sine_params(z):
    from axions_gb300.params import make_params
    return make_params(0, nx=int(z["nx"]), ny=int(z["ny"]), nz=int(z["nz"]), dx=float(z["dx"]), dy=float(z["dy"]),
                       dz=float(z["dz"]), g=float(z["g"]))


@pytest.mark.parametrize("name", SINE_CASES)
def test_sine_string_ic_bit_exact(oracle_mod, name):
    """initialConditions.cpp "NG sine" (golden-section search for the closest
    point of a Nambu-Goto sine wave, fields reflected across z = 0) and
    "simple sine" (the string offset by eps*sin(Omega z)/Omega), with eps read
    from standard input: the one level of Data/ic.txt, in both slots."""
    z = load_golden(name)
    st, off = oracle_mod.sine_string_ic(sine_params(z), z["profile"][0], z["profile"][1], float(z["sor_h"]),
                                        float(z["eps"]), str(z["ic_type"]))
    assert off == 0
    v = st.reshape(5, 2, -1)
    assert np.array_equal(v[:, 0], z["ic"]) and np.array_equal(v[:, 1], z["ic"])


def test_ng_sine_column_is_the_closest_string_point(oracle_mod):
    """The golden-section result is a local minimum of the distance to the
    curve (xs(sigma), zs(sigma)), and normal_dist is the signed distance along
    the unit normal: |normal_dist| = |(x, z) - (xs, zs)|."""
    z = load_golden("ref_ng_sine_ic")
    eps, dz, nz = float(z["eps"]), float(z["dz"]), int(z["nz"])
    Om = oracle_mod.lib().orc_ng_omega(eps, dz, nz)
    for x, zz in ((0.7, 0.3), (-2.0, 1.5), (3.1, 4.0), (0.0, 0.0)):
        xs, zs, xsg, zsg, pm, nd = oracle_mod.ng_column(eps, Om, x, zz)
        assert abs(pm - 1.0) < 1e-12
        assert abs(abs(nd) - np.hypot(x - xs, zz - zs)) < 1e-6
