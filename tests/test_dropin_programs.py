"""The drop-in programs (axions_gb300/bin/*) against the reference's own output.

Each program takes the reference's parameter names and writes the reference's
files.  Run with the configurations of the golden fixtures (which were made by
running the reference programs), their text output must match the
reference's: energies and deviations to 1e-12 relative, crossing frames with
the same counts and positions to 1e-9, final fields normwise to 1e-12.  The
output precision is raised to 17 digits (`digits=17`) for the comparison; by
default the programs print 6 significant digits like the reference.
"""
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden, params_from_json

BIN = ROOT / "axions_gb300" / "bin"


def _run(prog, tmp_path, args, stdin=""):
    (tmp_path / "Data").mkdir(exist_ok=True)
    (tmp_path / "GifData").mkdir(exist_ok=True)
    cmd = [str(BIN / prog), f"out_dir={tmp_path}", "digits=17"] + [f"{k}={v}" for k, v in args.items()]
    return subprocess.run(cmd, input=stdin.encode(), capture_output=True, timeout=300)


def _cols(path):
    return np.array([float(t) for t in path.read_text().split()])


def _frames(tmp_path, prefix):
    out, f = [], 0
    while (tmp_path / "GifData" / f"{prefix}{f}.txt").exists():
        out.append(_cols(tmp_path / "GifData" / f"{prefix}{f}.txt").reshape(-1, 3))
        f += 1
    return out


def test_unknown_parameter_is_an_error(tmp_path):
    r = _run("mpi_evolution", tmp_path, {"no_such_constant": 1})
    assert r.returncode == 2 and b"unknown parameter" in r.stderr


def test_short_ic_file_is_rejected(tmp_path):
    (tmp_path / "Data").mkdir()
    (tmp_path / "Data" / "ic.txt").write_text("1 0 0 0 0\n")
    r = _run("evolution", tmp_path, {"nx": 4, "ny": 4, "nz": 4, "nt": 1}, stdin="t\n")
    assert r.returncode == 2 and b"expected" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ref_mpi_ah_prs", "ref_mpi_ah_c1", "ref_moore_mpi"])
def test_mpi_programs_reproduce_reference_output(tmp_path, name):
    z = load_golden(name)
    p = params_from_json(z["params"])
    moore = p.model == 1
    args = {"nx": p.nx, "ny": p.ny, "nz": p.nz, "nt": int(z["nt"]), "dx": p.dx, "dy": p.dy, "dz": p.dz, "dt": p.dt,
            "damped_nt": p.damped_nt, "dampFac": p.dampFac, "alpha": p.alpha, "saveFreq": int(z["save_freq"]),
            "outTag": "g", "seed": int(z["seed"]), "calcEnergy": "true"}
    if moore:
        args.update({"lambda1": p.lam, "lambda2": p.lambda2, "lambda12": p.lambda12, "q1": int(p.q1), "q2": int(p.q2)})
        prog, tag = "moore_mpi_evolution", f"g_nx{p.nx}_q1{int(p.q1)}_seed{int(z['seed'])}"
    else:
        args.update({"lambda": p.lam, "eta": p.eta, "g": p.g})
        prog, tag = "mpi_evolution", f"g_nx{p.nx}_seed{int(z['seed'])}"
    r = _run(prog, tmp_path, args)
    assert r.returncode == 0, r.stderr.decode()
    energy = _cols(tmp_path / "Data" / f"valsPerLoop_{tag}.txt")
    np.testing.assert_allclose(energy, z["energy"], rtol=1e-12, atol=0)
    frames = _frames(tmp_path, f"gifStringPosData_{tag}_")
    assert [len(f) for f in frames] == z["frame_counts"].tolist()
    np.testing.assert_allclose(np.concatenate(frames), z["frame_xyz"], rtol=0, atol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ref_evol_ah_periodic", "ref_evol_ah_fixed", "ref_moore_evol"])
def test_openmp_programs_reproduce_reference_output(tmp_path, name):
    z = load_golden(name)
    p = params_from_json(z["params"])
    moore = p.model == 1
    ic = z["ic"]                     # (comp, slot, N): slot 0 = past, slot 1 = now at step 0
    (tmp_path / "Data").mkdir()
    nc = ic.shape[0]
    if moore:
        lines = [" ".join(repr(float(ic[c, 1, s])) for c in range(nc)) for s in range(p.N)]
        (tmp_path / "Data" / "moore_ic.txt").write_text("\n".join(lines) + "\n")
        args = {"nx": p.nx, "ny": p.ny, "nz": p.nz, "nt": int(z["nt"]), "dx": p.dx, "dy": p.dy, "dz": p.dz,
                "dt": p.dt, "lambda1": p.lam, "lambda2": p.lambda2, "lambda12": p.lambda12, "q1": int(p.q1),
                "q2": int(p.q2), "makeGif": "false"}
        r = _run("mooreEvol", tmp_path, args)
        vals = "valsPerLoop.txt"
    else:
        lines = []
        for slot in (0, 1):
            lines += [" ".join(repr(float(ic[c, slot, s])) for c in range(nc)) for s in range(p.N)]
        (tmp_path / "Data" / "ic.txt").write_text("\n".join(lines) + "\n")
        bc = "periodic" if p.bc == 0 else "fixed"
        args = {"nx": p.nx, "ny": p.ny, "nz": p.nz, "nt": int(z["nt"]), "dx": p.dx, "dy": p.dy, "dz": p.dz,
                "dt": p.dt, "lambda": p.lam, "eta": p.eta, "g": p.g, "damped_nt": 0, "dampFac": 0.0,
                "alpha": p.alpha, "saveFreq": int(z["save_freq"]), "xyBC": bc, "zBC": bc, "stationary_ic": "false",
                "detectBuffer": "false", "finalOut": "true"}
        r = _run("evolution", tmp_path, args, stdin="g\n")
        vals = "valsPerLoop_g.txt"
    assert r.returncode == 0, r.stderr.decode()
    v = _cols(tmp_path / "Data" / vals).reshape(int(z["nt"]), -1)
    np.testing.assert_allclose(v[:, 0], z["energy"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(v[:, 1], z["deviation"], rtol=1e-12, atol=0)
    final = _cols(tmp_path / "Data" / "finalField.txt").reshape(p.N, nc).T
    ref = z["final_newest"]
    d = np.abs(final - ref)
    assert d.max() / np.abs(ref).max() <= 1e-12 and np.linalg.norm(d) / np.linalg.norm(ref) <= 1e-12
    if not moore:
        frames = _frames(tmp_path, "gifStringPosData_")
        assert [len(f) for f in frames] == z["frame_counts"].tolist()
        np.testing.assert_allclose(np.concatenate(frames), z["frame_xyz"], rtol=0, atol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ref_icw_len_periodic", "ref_icw_len_fixed", "ref_icw_len_nosplit"])
def test_icw_program_reproduces_reference_output(tmp_path, name):
    """bin/ic_w_evolution against ic_w_evolution itself: ic_func's random IC
    made in-process, then per step energy, deviation and the string length
    L0 [L1] (valsPerLoop_test.txt), and the last level (finalField.txt)."""
    z = load_golden(name)
    p = params_from_json(z["params"])
    split = bool(z["split"])
    nt = int(z["nt"])
    bc = "periodic" if p.bc == 0 else "fixed"
    args = {"nx": p.nx, "ny": p.ny, "nz": p.nz, "nt": nt, "dx": p.dx, "dy": p.dy, "dz": p.dz, "dt": p.dt,
            "xyBC": bc, "zBC": bc, "seed": int(z["seed"]), "splitLength": "true" if split else "false",
            "makeGif": "false", "ic_type": "random"}
    r = _run("ic_w_evolution", tmp_path, args)
    assert r.returncode == 0, r.stderr.decode()
    vals = _cols(tmp_path / "Data" / "valsPerLoop_test.txt").reshape(nt, 4 if split else 3)
    assert np.array_equal(vals[:, 2], z["L0"])
    if split:
        assert np.array_equal(vals[:, 3], z["L1"])
    assert np.max(np.abs(vals[:, 0] - z["energy"]) / np.abs(z["energy"])) <= 1e-12
    final = _cols(tmp_path / "Data" / "finalField.txt").reshape(-1, 5).T
    assert np.array_equal(final[:2], z["final_phi"])


@pytest.mark.gpu
def test_icw_program_loop_collision_reproduces_reference_output(tmp_path):
    """bin/ic_w_evolution with no ic_type builds what the reference's does,
    ic_func.cpp's "loop collision" (:25, :966-1720, read from
    Data/SOR_Fields.txt), then evolves: against the reference's run, energy per
    step to 1e-12, L0 and L1 per step to 1e-9, and the last level's fields to
    1e-12 of each component's largest value (g != 0: the step's sines are this
    library's, not libm's)."""
    z = load_golden("ref_icfunc_loop_collision")
    p = params_from_json(z["params"])
    nt = int(z["nt"])
    prof = z["profile"]
    (tmp_path / "Data").mkdir()
    (tmp_path / "Data" / "SOR_Fields.txt").write_text(
        "".join(f"{float(a)!r} {float(b)!r}\n" for a, b in zip(prof[0], prof[1])))
    args = {"nx": p.nx, "ny": p.ny, "nz": p.nz, "nt": nt, "dx": p.dx, "dy": p.dy, "dz": p.dz, "dt": p.dt, "g": p.g,
            "makeGif": "false", "SORnx": prof.shape[1], "SORa": float(z["sor_h"])}
    r = _run("ic_w_evolution", tmp_path, args)
    assert r.returncode == 0, r.stderr.decode()
    vals = _cols(tmp_path / "Data" / "valsPerLoop_test.txt").reshape(nt, 4)
    assert np.max(np.abs(vals[:, 0] - z["energy"]) / np.abs(z["energy"])) <= 1e-12
    for c, key in ((2, "L0"), (3, "L1")):
        assert np.max(np.abs(vals[:, c] - z[key])) <= 1e-9 * np.max(np.abs(z[key])), key
    final = _cols(tmp_path / "Data" / "finalField.txt").reshape(-1, 5).T
    for c in range(5):
        ref = np.max(np.abs(z["final"][c]))
        assert np.max(np.abs(final[c] - z["final"][c])) <= 1e-12 * ref, c


def test_icw_program_default_ic_needs_the_profile_table(tmp_path):
    """With no ic_type, bin/ic_w_evolution builds what the reference's ships
    with, ic_func.cpp's "loop collision" (:25), from Data/SOR_Fields.txt
    (ic_func.cpp:978); without the table it stops with that file's name."""
    r = _run("ic_w_evolution", tmp_path, {"nx": 5, "ny": 5, "nz": 5, "nt": 1})
    assert r.returncode != 0 and b"Data/SOR_Fields.txt" in r.stderr


def test_icw_program_rejects_unprovided_ic(tmp_path):
    r = _run("ic_w_evolution", tmp_path, {"nx": 4, "ny": 4, "nz": 4, "nt": 1, "ic_type": "NG sine"})
    assert r.returncode == 2 and b"ic_type" in r.stderr
