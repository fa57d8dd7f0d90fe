"""Neumann and absorbing boundaries and per-axis boundary kinds on the GPU,
against evolution.cpp itself (golden fixtures made by running it with
xyBC / zBC set) and the oracle.

Bars: FP64 fields field by field (each component) max|d|/max|ref| <= 1e-12;
energies and deviations 1e-12 relative; crossing frames with the same counts,
positions to 1e-6 (the fields differ in the last bits where the GPU's sin/cos
do).  FP32 tracks the FP64 oracle to 1e-4 over the short runs.
"""
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden, params_from_json

pytestmark = pytest.mark.gpu

TOL = 1e-12
CASES = ["ref_evol_bc_neumann", "ref_evol_bc_absorbing", "ref_evol_bc_absorbing_neumann",
         "ref_evol_bc_fixed_zper", "ref_evol_bc_per_zfixed"]


@pytest.fixture(scope="module")
def lattice_mod():
    from axions_gb300 import lattice
    lattice.load_library()
    return lattice


def assert_components_close(a, b, tol):
    for c in range(b.shape[0]):
        ref = np.max(np.abs(b[c]))
        err = np.max(np.abs(a[c] - b[c]))
        assert err <= tol * max(ref, 1e-300), f"component {c}: {err:.3e} vs max {ref:.3e}"


def deviation(p, D):
    from axions_gb300.params import BCZ_AS_XY, BCZ_PERIODIC, BC_PERIODIC
    pxy = p.bc == BC_PERIODIC
    pz = p.bc_z == BCZ_PERIODIC or (p.bc_z == BCZ_AS_XY and pxy)
    D = D / (p.nx * p.ny) if pxy else D / ((p.nx - 2) * (p.ny - 2))
    return D / p.nz if pz else D / (p.nz - 2)


@pytest.mark.parametrize("name", CASES)
def test_boundaries_against_reference(lattice_mod, name):
    """evolution.cpp's loop body: detection every saveFreq steps (after the
    boundary step of that level), then a step with energy and deviation."""
    z = load_golden(name)
    p = params_from_json(z["params"])
    lat = lattice_mod.Lattice(p)
    lat.set_slots(z["ic"], 0)
    nt, sf = int(z["nt"]), int(z["save_freq"])
    E, D, frames = [], [], []
    for n in range(nt):
        if n % sf == 0:
            frames.append(lat.detect(0))
        d = lat.step_diag()
        E.append(d.energy)
        D.append(d.gauss_abs_sum)
    now, _ = lat.get_state()
    assert_components_close(now, z["final_newest"], TOL)
    np.testing.assert_allclose(E, z["energy"], rtol=TOL, atol=0)
    np.testing.assert_allclose(deviation(p, np.array(D)), z["deviation"], rtol=TOL, atol=0)
    assert [len(f) for f in frames] == z["frame_counts"].tolist()
    np.testing.assert_allclose(np.concatenate(frames), z["frame_xyz"], rtol=0, atol=1e-6)
    lat.close()


@pytest.mark.parametrize("name", ["ref_evol_bc_neumann", "ref_evol_bc_absorbing"])
def test_fp32_boundaries_track_fp64(lattice_mod, oracle_mod, name):
    from axions_gb300.params import F32
    z = load_golden(name)
    p = params_from_json(z["params"])
    st = np.ascontiguousarray(z["ic"])
    for n in range(int(z["nt"])):
        oracle_mod.step(p, st, n)
    p32 = p.copy()
    p32.precision = F32
    lat = lattice_mod.Lattice(p32)
    lat.set_slots(z["ic"], 0)
    lat.step(int(z["nt"]))
    now, _ = lat.get_state()
    want = st.reshape(5, 2, -1)[:, (int(z["nt"]) + 1) % 2]
    assert np.max(np.abs(now - want)) <= 1e-4 * np.max(np.abs(want))
    lat.close()


def test_moore_neumann_walls_against_reference(lattice_mod):
    """mooreEvol.cpp with xyBC = neumann: phi1, phi2 transported along q1*theta,
    q2*theta (mooreEvol.cpp:114-160)."""
    z = load_golden("ref_moore_evol_neumann")
    p = params_from_json(z["params"])
    lat = lattice_mod.Lattice(p)
    lat.set_slots(z["ic"], 0)
    nt = int(z["nt"])
    out = lat.advance(nt, diag_every=1)
    now, _ = lat.get_state()
    assert_components_close(now, z["final_newest"], TOL)
    np.testing.assert_allclose([o[1] for o in out], z["energy"], rtol=TOL, atol=0)
    c = (p.nx - 2) * (p.ny - 2) * (p.nz - 2)              # mooreEvol.cpp:383,697
    np.testing.assert_allclose(np.array([o[2] for o in out]) / c / c, z["deviation"], rtol=TOL, atol=0)
    lat.close()


def test_neumann_layer_is_set_lazily(lattice_mod, oracle_mod):
    """get_state shows the level as stored; detection (like a step) first sets
    the level's Neumann layer, once."""
    z = load_golden("ref_evol_bc_neumann")
    p = params_from_json(z["params"])
    lat = lattice_mod.Lattice(p)
    lat.set_slots(z["ic"], 0)
    raw, _ = lat.get_state()
    assert np.array_equal(raw, z["ic"][:, 1])
    lat.detect(0)
    got, _ = lat.get_state()
    st = np.ascontiguousarray(z["ic"])
    oracle_mod.apply_boundaries(p, st, 0)
    assert_components_close(got, st[:, 1], TOL)
    assert not np.array_equal(got, raw)
    lat.detect(0)
    again, _ = lat.get_state()
    assert np.array_equal(again, got)
    lat.close()


def test_boundary_parameters_are_checked(lattice_mod):
    from axions_gb300.lattice import LatticeError
    from axions_gb300.params import (BC_ABSORBING, BC_NEUMANN, BCZ_NEUMANN, MODEL_MOORE, make_params)
    bad = [make_params(MODEL_MOORE, n=8, bc=BC_NEUMANN),                # Moore: no Neumann z
           make_params(0, n=8, bc=BC_ABSORBING),                         # absorbing z (bc_z same as bc)
           make_params(0, nx=6, ny=8, nz=8, bc=BC_ABSORBING, bc_z=BCZ_NEUMANN),  # z-Neumann needs nz <= nx
           make_params(0, n=8, bc=7)]
    for p in bad:
        with pytest.raises(LatticeError):
            lattice_mod.Lattice(p)


def test_evolution_program_with_absorbing_walls(tmp_path):
    """bin/evolution with xyBC=absorbing, zBC=periodic against the reference's
    valsPerLoop and finalField."""
    z = load_golden("ref_evol_bc_absorbing")
    p = params_from_json(z["params"])
    (tmp_path / "Data").mkdir()
    (tmp_path / "GifData").mkdir()
    ic = z["ic"]
    lines = [" ".join(repr(float(ic[c, t, s])) for c in range(5)) for t in (0, 1) for s in range(p.N)]
    (tmp_path / "Data" / "ic.txt").write_text("\n".join(lines) + "\n")
    nt = int(z["nt"])
    args = {"nx": p.nx, "ny": p.ny, "nz": p.nz, "nt": nt, "dx": p.dx, "dy": p.dy, "dz": p.dz, "dt": p.dt,
            "lambda": p.lam, "eta": p.eta, "g": p.g, "damped_nt": 0, "dampFac": 0, "alpha": p.alpha,
            "xyBC": "absorbing", "zBC": "periodic", "stationary_ic": "false", "stringDetect": "false",
            "finalOut": "true", "saveFreq": int(z["save_freq"])}
    cmd = [str(ROOT / "axions_gb300" / "bin" / "evolution"), f"out_dir={tmp_path}", "digits=17"]
    r = subprocess.run(cmd + [f"{k}={v}" for k, v in args.items()], input=b"t\n", capture_output=True, timeout=300)
    assert r.returncode == 0, r.stderr.decode()
    vals = np.array([float(t) for t in (tmp_path / "Data" / "valsPerLoop_t.txt").read_text().split()]).reshape(nt, -1)
    np.testing.assert_allclose(vals[:, 0], z["energy"], rtol=TOL, atol=0)
    np.testing.assert_allclose(vals[:, 1], z["deviation"], rtol=TOL, atol=0)
    final = np.array([float(t) for t in (tmp_path / "Data" / "finalField.txt").read_text().split()]).reshape(-1, 5).T
    assert_components_close(final, z["final_newest"], TOL)
