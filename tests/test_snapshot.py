"""Asynchronous snapshots (lat_snapshot_*) and the drop-in programs' gifData
frames, which are written from them while the run goes on.

A snapshot must hold the level that was current when it began, even when
steps are issued before it is waited for, bit for bit: |phi|^2 is re*re + im*im
in double on both sides (-fmad=false), a level is copied (FP64) or widened
exactly (FP32).
"""
import numpy as np
import pytest

from conftest import ROOT, load_golden, params_from_json

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lattice_mod():
    from axions_gb300 import lattice
    lattice.load_library()
    return lattice


def _lattice(lattice_mod, model, precision):
    from axions_gb300.params import make_params
    p = make_params(model, nx=20, ny=18, nz=16, d=0.5, dt=0.1, precision=precision, damped_nt=0, alpha=0.0)
    lat = lattice_mod.Lattice(p)
    lat.random_phase_ic_device(11, independent=(model == 1))
    lat.advance(3)
    return lat


@pytest.mark.parametrize("model,precision", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_snapshot_is_the_level_at_begin(lattice_mod, model, precision):
    lat = _lattice(lattice_mod, model, precision)
    now, _ = lat.get_state()
    mag = now[0] * now[0] + now[1] * now[1]
    if model == 1:
        mag = np.concatenate([mag, now[2] * now[2] + now[3] * now[3]])
    a = np.empty(lat.snapshot_doubles(lattice_mod.SNAP_MAGNITUDE))
    lat.snapshot_begin(lattice_mod.SNAP_MAGNITUDE, a)
    lat.step(4)                      # issued before the wait: must not leak into `a`
    lat.snapshot_wait()
    assert np.array_equal(a, mag)
    pinned = lattice_mod.PinnedArray(lat.snapshot_doubles(lattice_mod.SNAP_LEVEL))
    now2, _ = lat.get_state()
    lat.snapshot_begin(lattice_mod.SNAP_LEVEL, pinned.array)
    lat.step(2)
    lat.snapshot_wait()
    assert np.array_equal(pinned.array.reshape(now2.shape), now2)
    pinned.close()
    lat.close()


def test_back_to_back_snapshots(lattice_mod):
    lat = _lattice(lattice_mod, 0, 0)
    outs, want = [], []
    for _ in range(3):
        now, _ = lat.get_state()
        want.append(now[0] * now[0] + now[1] * now[1])
        o = np.empty(lat.snapshot_doubles(lattice_mod.SNAP_MAGNITUDE))
        lat.snapshot_begin(lattice_mod.SNAP_MAGNITUDE, o)   # waits for the previous copy itself
        outs.append(o)
        lat.step(1)
    lat.snapshot_wait()
    for o, w in zip(outs, want):
        assert np.array_equal(o, w)
    lat.close()


def test_gif_frames_of_the_evolution_program(tmp_path, oracle_mod):
    """bin/evolution with makeGif: frame f is |phi|^2 of level f*saveFreq + 1
    (evolution.cpp:1423-1441), written by the background writer; compared with
    the oracle's evolution of the same IC (FP64 bar, 1e-12)."""
    import subprocess
    z = load_golden("ref_evol_ah_periodic")
    p = params_from_json(z["params"])
    (tmp_path / "Data").mkdir()
    (tmp_path / "GifData").mkdir()
    ic = z["ic"]
    lines = [" ".join(repr(float(ic[c, 1, s])) for c in range(5)) for s in range(p.N)]
    (tmp_path / "Data" / "ic.txt").write_text("\n".join(lines) + "\n")
    nt, sf = int(z["nt"]), 4
    args = {"nx": p.nx, "ny": p.ny, "nz": p.nz, "nt": nt, "dx": p.dx, "dy": p.dy, "dz": p.dz, "dt": p.dt,
            "lambda": p.lam, "eta": p.eta, "g": p.g, "damped_nt": p.damped_nt, "dampFac": p.dampFac,
            "alpha": p.alpha, "makeGif": "true", "saveFreq": sf, "makeStringPosGif": "false"}
    cmd = [str(ROOT / "axions_gb300" / "bin" / "evolution"), f"out_dir={tmp_path}", "digits=17"]
    r = subprocess.run(cmd + [f"{k}={v}" for k, v in args.items()], input=b"t\n", capture_output=True, timeout=300)
    assert r.returncode == 0, r.stderr.decode()
    st = np.ascontiguousarray(np.stack([ic[:, 1], ic[:, 1]], axis=1))
    frames = 0
    for n in range(nt):
        oracle_mod.step(p, st, n)
        if n % sf == 0:
            lv = st.reshape(5, 2, -1)[:, (n + 2) % 2]
            want = lv[0] * lv[0] + lv[1] * lv[1]
            got = np.array([float(t) for t in (tmp_path / "GifData" / f"gifData_{frames}.txt").read_text().split()])
            assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want))
            frames += 1
    assert not (tmp_path / "GifData" / f"gifData_{frames}.txt").exists()
