"""Generate golden fixtures by running the reference programs themselves.

The reference ships no tests, fixtures or golden outputs.  This script builds
its programs with oracle/ref/build_ref.py (parameters substituted into a
scratch copy; 17-digit output; a single-rank MPI stub that dumps the fields),
runs them on small seeded lattices, and stores inputs and outputs as .npz files
next to this script.  tests/test_oracle_golden.py then pins the oracle's CPU
restatement against these files, and the GPU parity tests use them directly.

Run it in a container that has the reference sources:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.ref import build_ref  # noqa: E402
from axions_gb300.params import (BC_FIXED, BC_PERIODIC, ENERGY_EVOLUTION, ENERGY_MPI,  # noqa: E402
                                 MODEL_AH, MODEL_MOORE, MOORE_CURRENT_CHARGE, MOORE_CURRENT_PLAIN,
                                 make_params)

OUT = Path(__file__).resolve().parent


def _fmt(v: float) -> str:
    return repr(float(v))


def _params_json(p) -> str:
    return json.dumps(p.as_dict())


def read_dump(work: Path, ncomp: int, N: int) -> np.ndarray:
    raw = np.fromfile(work / "Data" / "axr_fields.bin", dtype=np.float64)
    assert raw.size == ncomp * 2 * N, (raw.size, ncomp, N)
    return raw.reshape(ncomp, 2, N)


def read_frames(work: Path, prefix: str):
    frames = []
    f = 0
    while True:
        path = work / "GifData" / f"{prefix}{f}.txt"
        if not path.exists():
            break
        vals = build_ref.read_columns(path)
        frames.append(vals.reshape(-1, 3))
        f += 1
    return frames


def pack_frames(frames):
    counts = np.array([len(a) for a in frames], dtype=np.int64)
    xyz = np.concatenate(frames, axis=0) if frames else np.zeros((0, 3))
    return counts, xyz


# --------------------------------------------------------------------------
# mpi_evolution.cpp: random-phase IC from mt19937, in-place update, PRS + damping
# --------------------------------------------------------------------------
def gen_mpi_ah(name, nx, ny, nz, nt, lam, g, damped_nt, dampFac, alpha, seed, saveFreq, dt=0.1, d=0.5):
    consts = {"nx": nx, "ny": ny, "nz": nz, "nt": nt, "dx": d, "dy": d, "dz": d, "dt": dt,
              "lambda": lam, "eta": 1.0, "g": g, "damped_nt": damped_nt, "dampFac": dampFac,
              "alpha": alpha, "scaling": 1.0, "makeStringPosGif": True, "saveFreq": saveFreq,
              "countRate": 10, "outTag": "g", "ic_type": "random", "seed": seed,
              "stringDetect": True, "detectBuffer": True, "calcEnergy": True}
    build_ref.build("mpi_evolution", name, consts)
    work = build_ref.run(name)
    p = make_params(MODEL_AH, nx=nx, ny=ny, nz=nz, d=d, dt=dt, lam=lam, eta=1.0, g=g,
                    damped_nt=damped_nt, dampFac=dampFac, alpha=alpha, scaling=1.0, tau0=1.0,
                    energy_form=ENERGY_MPI, bc=BC_PERIODIC)
    N = nx * ny * nz
    final = read_dump(work, 5, N)
    energy = build_ref.read_columns(work / "Data" / f"valsPerLoop_g_nx{nx}_seed{seed}.txt")
    frames = read_frames(work, f"gifStringPosData_g_nx{nx}_seed{seed}_")
    counts, xyz = pack_frames(frames)
    np.savez_compressed(OUT / f"{name}.npz", program="mpi_evolution", params=_params_json(p), seed=seed,
                        nt=nt, save_freq=saveFreq, final=final, energy=energy,
                        frame_counts=counts, frame_xyz=xyz)
    print(name, "energy lines", energy.size, "frames", counts.tolist())


def gen_mpi_ah_ic(name, nx, ny, nz, seed):
    consts = {"nx": nx, "ny": ny, "nz": nz, "nt": 0, "ic_type": "random", "seed": seed, "eta": 1.0}
    build_ref.build("mpi_evolution", name, consts)
    work = build_ref.run(name)
    N = nx * ny * nz
    ic = read_dump(work, 5, N)
    np.savez_compressed(OUT / f"{name}.npz", program="mpi_evolution", seed=seed, nx=nx, ny=ny, nz=nz, ic=ic)
    print(name, "ic ok")


# --------------------------------------------------------------------------
# moore_mpi_evolution.cpp: equal-phase random IC, current without q
# --------------------------------------------------------------------------
def gen_moore_mpi(name, nx, ny, nz, nt, lam1, lam2, lam12, q1, q2, damped_nt, dampFac, alpha, seed,
                  saveFreq, dt=0.1, d=0.5):
    consts = {"nx": nx, "ny": ny, "nz": nz, "nt": nt, "dx": d, "dy": d, "dz": d, "dt": dt,
              "lambda1": lam1, "lambda2": lam2, "lambda12": lam12, "eta1": 1.0, "eta2": 1.0,
              "q1": q1, "q2": q2, "damped_nt": damped_nt, "dampFac": dampFac, "alpha": alpha,
              "scaling": 1.0, "makeStringPosGif": True, "saveFreq": saveFreq, "countRate": 10,
              "outTag": "g", "ic_type": "random", "seed": seed, "stringDetect": True,
              "detectBuffer": True, "calcEnergy": True}
    build_ref.build("moore_mpi_evolution", name, consts)
    work = build_ref.run(name)
    g = float(np.sqrt(0.5 * lam1 * 1.0 ** 2 / (q1 * q1 + q2 * q2)))
    p = make_params(MODEL_MOORE, nx=nx, ny=ny, nz=nz, d=d, dt=dt, lam=lam1, lambda2=lam2, lambda12=lam12,
                    eta=1.0, eta2=1.0, q1=float(q1), q2=float(q2), g=g, damped_nt=damped_nt,
                    dampFac=dampFac, alpha=alpha, scaling=1.0, tau0=1.0, energy_form=ENERGY_MPI,
                    bc=BC_PERIODIC, moore_current=MOORE_CURRENT_PLAIN)
    N = nx * ny * nz
    final = read_dump(work, 7, N)
    energy = build_ref.read_columns(work / "Data" / f"valsPerLoop_g_nx{nx}_q1{q1}_seed{seed}.txt")
    frames = read_frames(work, f"gifStringPosData_g_nx{nx}_q1{q1}_seed{seed}_")
    counts, xyz = pack_frames(frames)
    np.savez_compressed(OUT / f"{name}.npz", program="moore_mpi_evolution", params=_params_json(p), seed=seed,
                        nt=nt, save_freq=saveFreq, final=final, energy=energy,
                        frame_counts=counts, frame_xyz=xyz)
    print(name, "energy lines", energy.size, "frames", counts.tolist())


# --------------------------------------------------------------------------
# evolution.cpp: two-level IC from a file, energy + Gauss every step
# --------------------------------------------------------------------------
def _two_level_ic(rng, N, ncomp_phi, amp_theta):
    """Random |phi| and phase, small random link phases; past level perturbed."""
    now = []
    for _ in range(ncomp_phi // 2):
        r = 0.3 + 0.9 * rng.random(N)
        ph = 2 * np.pi * rng.random(N)
        now += [r * np.cos(ph), r * np.sin(ph)]
    for _ in range(3):
        now.append(amp_theta * (2 * rng.random(N) - 1))
    now = np.array(now)
    past = now + 0.02 * (2 * rng.random(now.shape) - 1)
    return now, past


XY_KIND = {"periodic": BC_PERIODIC, "neumann": 2, "absorbing": 3}
Z_KIND = {"periodic": 1, "neumann": 3}


def gen_evolution(name, nx, ny, nz, nt, lam, g, alpha, bc, seed, saveFreq=4, dt=0.1, d=0.5, xyBC=None, zBC=None):
    """evolution.cpp; xyBC / zBC (the reference's strings) default to bc for all axes."""
    rng = np.random.default_rng(seed)
    N = nx * ny * nz
    now, past = _two_level_ic(rng, N, 2, 0.4)
    bcs = "periodic" if bc == BC_PERIODIC else "fixed"
    xyBC = xyBC or bcs
    zBC = zBC or bcs
    bc = XY_KIND.get(xyBC, BC_FIXED)
    bc_z = Z_KIND.get(zBC, 2)
    consts = {"nx": nx, "ny": ny, "nz": nz, "nt": nt, "dx": d, "dy": d, "dz": d, "dt": dt,
              "lambda": lam, "eta": 1.0, "g": g, "damped_nt": 0, "dampFac": 0.0, "alpha": alpha,
              "scaling": 1.0, "makeGif": False, "makeStringPosGif": True, "saveFreq": saveFreq,
              "xyBC": xyBC, "zBC": zBC, "stringPos": False, "stationary_ic": False,
              "stringDetect": True, "detectBuffer": False, "splitLength": False, "finalOut": True}
    build_ref.build("evolution", name, consts)
    # "data" IC: level block 0 = slot 0 (past at step 0), block 1 = slot 1 (now)
    lines = []
    for lev in (past, now):
        for s in range(N):
            lines.append(" ".join(_fmt(lev[c, s]) for c in range(5)))
    work = build_ref.run(name, stdin="g\n", ic_lines=lines)
    vals = build_ref.read_columns(work / "Data" / "valsPerLoop_g.txt").reshape(nt, -1)
    final_newest = build_ref.read_columns(work / "Data" / "finalField.txt").reshape(N, 5).T.copy()
    frames = read_frames(work, "gifStringPosData_")
    counts, xyz = pack_frames(frames)
    p = make_params(MODEL_AH, nx=nx, ny=ny, nz=nz, d=d, dt=dt, lam=lam, eta=1.0, g=g, damped_nt=0,
                    dampFac=0.0, alpha=alpha, scaling=1.0, tau0=1.0, energy_form=ENERGY_EVOLUTION, bc=bc, bc_z=bc_z)
    ic = np.stack([past, now], axis=1)  # (comp, slot, N)
    np.savez_compressed(OUT / f"{name}.npz", program="evolution", params=_params_json(p), nt=nt,
                        save_freq=saveFreq, ic=ic, final_newest=final_newest, energy=vals[:, 0],
                        deviation=vals[:, 1], frame_counts=counts, frame_xyz=xyz)
    print(name, "vals", vals.shape, "frames", counts.tolist())


# --------------------------------------------------------------------------
# mooreEvol.cpp: fixed boundaries, stationary IC from file, q-weighted current
# --------------------------------------------------------------------------
def gen_moore_evol(name, nx, ny, nz, nt, lam1, lam2, lam12, q1, q2, seed, dt=0.1, d=0.5, xyBC="fixed"):
    rng = np.random.default_rng(seed)
    N = nx * ny * nz
    now, _ = _two_level_ic(rng, N, 4, 0.4)
    consts = {"nx": nx, "ny": ny, "nz": nz, "nt": nt, "dx": d, "dy": d, "dz": d, "dt": dt,
              "eta1": 1.0, "eta2": 1.0, "lambda1": lam1, "lambda2": lam2, "lambda12": lam12,
              "q1": q1, "q2": q2, "makeGif": False, "saveFreq": 10, "xyBC": xyBC}
    build_ref.build("mooreEvol", name, consts)
    lines = [" ".join(_fmt(now[c, s]) for c in range(7)) for s in range(N)]
    work = build_ref.run(name, ic_lines=lines, ic_name="moore_ic.txt")
    vals = build_ref.read_columns(work / "Data" / "valsPerLoop.txt").reshape(nt, 2)
    final_newest = build_ref.read_columns(work / "Data" / "finalField.txt").reshape(N, 7).T.copy()
    g = float(np.sqrt(0.5 * lam1 * 1.0 ** 2 / (q1 * q1 + q2 * q2)))
    p = make_params(MODEL_MOORE, nx=nx, ny=ny, nz=nz, d=d, dt=dt, lam=lam1, lambda2=lam2, lambda12=lam12,
                    eta=1.0, eta2=1.0, q1=float(q1), q2=float(q2), g=g, damped_nt=0, dampFac=0.0,
                    alpha=0.0, scaling=1.0, tau0=1.0, energy_form=ENERGY_EVOLUTION,
                    bc=2 if xyBC == "neumann" else BC_FIXED, bc_z=2, moore_current=MOORE_CURRENT_CHARGE)
    ic = np.stack([now, now], axis=1)
    np.savez_compressed(OUT / f"{name}.npz", program="mooreEvol", params=_params_json(p), nt=nt, ic=ic,
                        final_newest=final_newest, energy=vals[:, 0], deviation=vals[:, 1])
    print(name, "vals", vals.shape)


def gen_icw_length(name, nx, ny, nz, nt, bc, seed, d=0.35, split=True):
    """ic_w_evolution: IC from ic_func's "random" branch (minstd_rand, seed),
    evolution without friction, string length by greedy chaining every step
    (ic_w_evolution.cpp:961-1087); valsPerLoop = energy dev L0 [L1]."""
    s = "periodic" if bc == BC_PERIODIC else "fixed"
    consts = {"nx": nx, "ny": ny, "nz": nz, "nt": nt, "dx": d, "dy": d, "dz": d, "dt": 0.05,
              "makeGif": False, "xyBC": s, "zBC": s, "splitLength": bool(split)}
    build_ref.build("ic_w_evolution", name, consts, {"ic_func.cpp": {"ic_type": "random", "seed": float(seed)}})
    work = build_ref.run(name)
    ncol = 4 if split else 3
    vals = build_ref.read_columns(work / "Data" / "valsPerLoop_test.txt").reshape(nt, ncol)
    N = nx * ny * nz
    final = build_ref.read_columns(work / "Data" / "finalField.txt").reshape(N, 5).T.copy()
    p = make_params(MODEL_AH, nx=nx, ny=ny, nz=nz, d=d, dt=0.05, lam=1.0, eta=1.0, g=0.0, damped_nt=0,
                    dampFac=0.0, alpha=0.0, scaling=1.0, tau0=1.0, bc=bc)
    L1 = vals[:, 3] if split else np.zeros(nt)
    np.savez_compressed(OUT / f"{name}.npz", program="ic_w_evolution", params=_params_json(p), seed=seed, nt=nt,
                        split=bool(split), L0=vals[:, 2], L1=L1, energy=vals[:, 0], final_phi=final[:2])
    print(name, "vals", vals.shape)


def gen_initial_conditions(name, nx, ny, nz, seed, mean, stdev, g):
    """initialConditions.cpp, ic_type "random": Data/ic.txt (17 digits)."""
    consts = {"nx": nx, "ny": ny, "nz": nz, "ic_type": "random", "seed": float(seed), "mean": float(mean),
              "stdev": float(stdev), "g": float(g)}
    build_ref.build("initialConditions", name, consts)
    work = build_ref.run(name)
    ic = build_ref.read_columns(work / "Data" / "ic.txt").reshape(nx * ny * nz, 5).T.copy()
    np.savez_compressed(OUT / f"{name}.npz", program="initialConditions", nx=nx, ny=ny, nz=nz, seed=seed, mean=mean,
                        stdev=stdev, g=g, dx=0.5, ic=ic)
    print(name, ic.shape)


def gen_sor(name, nx, h, g, tol=1e-3):
    """singleSemiAnalytic.cpp on one thread (its OpenMP sweep updates in place,
    so only the single-thread order is reproducible): Data/SOR_Fields.txt."""
    build_ref.build("singleSemiAnalytic", name, {"nx": nx, "h": float(h), "g": float(g), "tol": float(tol)})
    work = build_ref.run(name, threads=1)
    tab = build_ref.read_columns(work / "Data" / "SOR_Fields.txt").reshape(nx, 2).T.copy()
    np.savez_compressed(OUT / f"{name}.npz", program="singleSemiAnalytic", nx=nx, h=h, g=g, tol=tol, w=1.5, n=1.0,
                        lam=1.0, eta=1.0, profile=tab)
    print(name, tab.shape)
    return tab


def gen_boost_ic(name, nx, ny, nz, g, dt, v, profile, sor_h, dz=0.5):
    """initialConditions.cpp, ic_type "boost" (a z-directed string boosted with
    velocity v): Data/ic.txt, two levels (17 digits), from the given profile
    table placed where the program reads it (dir_path/SOR_Fields.txt)."""
    m = profile.shape[1]
    consts = {"nx": nx, "ny": ny, "nz": nz, "ic_type": "boost", "g": float(g), "dt": float(dt),
              "v1x": float(v[0]), "v1y": float(v[1]), "v1z": float(v[2]), "SORnx": m, "SORa": float(sor_h),
              "dz": float(dz)}
    build_ref.build("initialConditions", name, consts)
    work = build_ref.SCRATCH / name
    lines = [f"{float(profile[0, r])!r} {float(profile[1, r])!r}" for r in range(m)]
    (work / "SOR_Fields.txt").write_text("\n".join(lines) + "\n")
    work = build_ref.run(name)
    ic = build_ref.read_columns(work / "Data" / "ic.txt").reshape(2, nx * ny * nz, 5).transpose(2, 0, 1).copy()
    np.savez_compressed(OUT / f"{name}.npz", program="initialConditions", ic_type="boost", nx=nx, ny=ny, nz=nz,
                        dx=0.5, dy=0.5, dz=dz, g=g, dt=dt, v=np.array(v, dtype=np.float64), sor_h=sor_h,
                        profile=profile, ic=ic)
    print(name, ic.shape)


def gen_loop_collision_ic(name, nx, ny, nz, g, dt, profile, sor_h, dz=0.5, geometry=None):
    """initialConditions.cpp, ic_type "loop collision": Data/ic.txt, two levels
    (17 digits), from the profile table at dir_path/Data/SOR_Fields.txt.
    `geometry` overrides the string positions and velocities (pos1s, pos1a,
    pos2s, pos2a, v1s, v1a, v2s, v2a); by default they follow the lattice
    (initialConditions.cpp:72-84)."""
    m = profile.shape[1]
    consts = {"nx": nx, "ny": ny, "nz": nz, "ic_type": "loop collision", "g": float(g), "dt": float(dt),
              "SORnx": m, "SORa": float(sor_h), "dz": float(dz)}
    geo = dict(pos1s=[0.15 * (ny - 1) * 0.5, -0.25 * (nz - 1) * dz], pos1a=[-0.15 * (ny - 1) * 0.5, 0.25 * (nz - 1) * dz],
               pos2s=[0.25 * (nx - 1) * 0.5, 0.0], pos2a=[-0.25 * (nx - 1) * 0.5, 0.0],
               v1s=[0.0, -0.75, 0.0], v1a=[0.0, 0.75, 0.0], v2s=[0.0, 0.0, 0.0], v2a=[0.0, 0.0, 0.0])
    if geometry:
        geo.update(geometry)
        consts.update(geometry)
    build_ref.build("initialConditions", name, consts)
    work = build_ref.SCRATCH / name
    lines = [f"{float(profile[0, r])!r} {float(profile[1, r])!r}" for r in range(m)]
    (work / "Data" / "SOR_Fields.txt").write_text("\n".join(lines) + "\n")
    work = build_ref.run(name)
    ic = build_ref.read_columns(work / "Data" / "ic.txt").reshape(2, nx * ny * nz, 5).transpose(2, 0, 1).copy()
    np.savez_compressed(OUT / f"{name}.npz", program="initialConditions", ic_type="loop collision", nx=nx, ny=ny,
                        nz=nz, dx=0.5, dy=0.5, dz=dz, g=g, dt=dt, sor_h=sor_h, profile=profile, ic=ic,
                        **{k: np.array(v, dtype=np.float64) for k, v in geo.items()})
    print(name, ic.shape)


def gen_icfunc_loop_collision(name, nx, ny, nz, nt, g, d=0.35, dt=0.05, sor_h=0.01, profile=None):
    """ic_w_evolution with ic_func's shipped ic_type, "loop collision"
    (ic_func.cpp:25, 966-1720), built in process from the profile table at
    dir_path/Data/SOR_Fields.txt (ic_func's own dir_path), then nt steps of
    periodic evolution.  ic_w_evolution writes no IC, so the fixture holds what
    it does write: valsPerLoop (energy, Gauss deviation, L0, L1 per step) and
    finalField (both fields of the newest level after nt steps)."""
    if profile is None:
        profile = np.load(OUT / "ref_sor_gauge.npz")["profile"]
    m = profile.shape[1]
    consts = {"nx": nx, "ny": ny, "nz": nz, "nt": nt, "dx": d, "dy": d, "dz": d, "dt": float(dt), "g": float(g),
              "makeGif": False}
    build_ref.build("ic_w_evolution", name, consts,
                    {"ic_func.cpp": {"ic_type": "loop collision", "SORnx": m, "SORa": float(sor_h)}})
    work = build_ref.SCRATCH / name
    lines = [f"{float(profile[0, r])!r} {float(profile[1, r])!r}" for r in range(m)]
    (work / "Data" / "SOR_Fields.txt").write_text("\n".join(lines) + "\n")
    work = build_ref.run(name)
    vals = build_ref.read_columns(work / "Data" / "valsPerLoop_test.txt").reshape(nt, 4)
    N = nx * ny * nz
    final = build_ref.read_columns(work / "Data" / "finalField.txt").reshape(N, 5).T.copy()
    p = make_params(MODEL_AH, nx=nx, ny=ny, nz=nz, d=d, dt=dt, lam=1.0, eta=1.0, g=g, damped_nt=0,
                    dampFac=0.0, alpha=0.0, scaling=1.0, tau0=1.0, bc=BC_PERIODIC)
    np.savez_compressed(OUT / f"{name}.npz", program="ic_w_evolution", ic_type="loop collision",
                        params=_params_json(p), nt=nt, sor_h=sor_h, profile=profile, energy=vals[:, 0],
                        deviation=vals[:, 1], L0=vals[:, 2], L1=vals[:, 3], final=final)
    print(name, "vals", vals.shape)


def gen_sine_ic(name, kind, nx, ny, nz, g, eps, profile, sor_h, dz=0.5):
    """initialConditions.cpp, ic_type "NG sine" or "simple sine" (a straight
    string perturbed by a sine wave of amplitude eps, which the program reads
    from standard input): Data/ic.txt, one level (17 digits), from the
    profile table at dir_path/Data/SOR_Fields.txt."""
    m = profile.shape[1]
    consts = {"nx": nx, "ny": ny, "nz": nz, "ic_type": kind, "g": float(g), "SORnx": m, "SORa": float(sor_h),
              "dz": float(dz)}
    build_ref.build("initialConditions", name, consts)
    work = build_ref.SCRATCH / name
    lines = [f"{float(profile[0, r])!r} {float(profile[1, r])!r}" for r in range(m)]
    (work / "Data" / "SOR_Fields.txt").write_text("\n".join(lines) + "\n")
    work = build_ref.run(name, stdin=f"{eps!r}\n")
    ic = build_ref.read_columns(work / "Data" / "ic.txt").reshape(nx * ny * nz, 5).T.copy()
    np.savez_compressed(OUT / f"{name}.npz", program="initialConditions", ic_type=kind, nx=nx, ny=ny, nz=nz,
                        dx=0.5, dy=0.5, dz=dz, g=g, eps=eps, sor_h=sor_h, profile=profile, ic=ic)
    print(name, ic.shape)


def main():
    args = sys.argv[1:]
    if args[:1] == ["--reference"] and len(args) >= 2:
        build_ref.set_reference(args[1])
        args = args[2:]
    if not build_ref.reference_available():
        raise SystemExit("usage: make_golden.py --reference <reference checkout> [gen_...(...) ...] "
                         "(or set AXIONS_REFERENCE); fixtures can only be made where the reference is")
    only = args
    if only:
        for call in only:
            eval(call)
        return
    gen_mpi_ah_ic("ref_mpi_ah_ic_s7", 6, 5, 4, seed=7)
    # config-1 physics (lambda=2, e=1, dx=0.5, dt=0.1, Minkowski, no damping)
    gen_mpi_ah("ref_mpi_ah_c1", 14, 12, 10, 30, lam=2.0, g=1.0, damped_nt=0, dampFac=0.0, alpha=0.0,
               seed=42, saveFreq=10)
    # PRS friction + damping phase + detection buffer
    gen_mpi_ah("ref_mpi_ah_prs", 12, 10, 8, 20, lam=2.0, g=1.0, damped_nt=6, dampFac=0.5, alpha=3.0,
               seed=5, saveFreq=5)
    # global strings (g = 0), the reference default
    gen_mpi_ah("ref_mpi_ah_global", 10, 10, 10, 12, lam=1.0, g=0.0, damped_nt=4, dampFac=0.5, alpha=3.0,
               seed=3, saveFreq=4)
    gen_evolution("ref_evol_ah_periodic", 12, 10, 8, 12, lam=2.0, g=1.0, alpha=3.0, bc=BC_PERIODIC, seed=11)
    gen_evolution("ref_evol_ah_fixed", 11, 10, 9, 10, lam=2.0, g=0.7, alpha=0.0, bc=BC_FIXED, seed=12)
    gen_moore_mpi("ref_moore_mpi", 12, 10, 8, 20, 2.0, 2.0, 0.5, 2, 1, damped_nt=6, dampFac=0.5, alpha=3.0,
                  seed=9, saveFreq=5)
    gen_moore_evol("ref_moore_evol", 10, 9, 8, 12, 2.0, 2.0, 0.5, 2, 1, seed=13)
    # string length (the reference default spacing 0.35; a wide cutoff; fixed walls; no split)
    gen_icw_length("ref_icw_len_periodic", 17, 15, 13, 40, BC_PERIODIC, seed=3)
    gen_icw_length("ref_icw_len_wide", 13, 12, 11, 16, BC_PERIODIC, seed=4, d=1.0)
    gen_icw_length("ref_icw_len_fixed", 15, 15, 15, 25, BC_FIXED, seed=5)
    gen_icw_length("ref_icw_len_nosplit", 11, 13, 9, 12, BC_PERIODIC, seed=6, d=0.5, split=False)
    gen_initial_conditions("ref_initial_conditions", 7, 6, 5, seed=42, mean=0.0, stdev=0.5, g=0.5)
    # boundary kinds of evolution.cpp:166-265,446-691,1375-1408 (nz <= nx for a Neumann z, see orc_apply_boundaries)
    gen_moore_evol("ref_moore_evol_neumann", 10, 9, 8, 10, 2.0, 2.0, 0.5, 2, 1, seed=26, xyBC="neumann")
    gen_evolution("ref_evol_bc_neumann", 10, 9, 8, 10, lam=2.0, g=0.7, alpha=3.0, bc=BC_FIXED, seed=21, saveFreq=3,
                  xyBC="neumann", zBC="neumann")
    gen_evolution("ref_evol_bc_absorbing", 11, 10, 8, 12, lam=2.0, g=0.7, alpha=0.0, bc=BC_FIXED, seed=22, saveFreq=4,
                  xyBC="absorbing", zBC="periodic")
    gen_evolution("ref_evol_bc_absorbing_neumann", 10, 10, 7, 10, lam=1.0, g=1.0, alpha=3.0, bc=BC_FIXED, seed=23,
                  saveFreq=5, xyBC="absorbing", zBC="neumann")
    gen_evolution("ref_evol_bc_fixed_zper", 9, 9, 8, 8, lam=2.0, g=0.7, alpha=0.0, bc=BC_FIXED, seed=24, saveFreq=4,
                  xyBC="fixed", zBC="periodic")
    gen_evolution("ref_evol_bc_per_zfixed", 9, 8, 9, 8, lam=2.0, g=0.7, alpha=3.0, bc=BC_FIXED, seed=25, saveFreq=4,
                  xyBC="periodic", zBC="fixed")
    # straight-string profiles (global and gauged) and the boosted-string IC built on the gauged one
    gen_sor("ref_sor_global", 3001, 0.01, 0.0)
    prof = gen_sor("ref_sor_gauge", 2001, 0.01, 1.0)
    gen_boost_ic("ref_boost_ic", 13, 12, 11, 1.0, 0.05, (0.24, 0.6 * (1 - 0.4 ** 2) ** 0.5, 0.0), prof, 0.01)
    # a velocity with a z part and dz != dy (initialConditions.cpp:745 takes zb with dy at t = 0)
    gen_boost_ic("ref_boost_ic_vz", 12, 11, 13, 0.8, 0.1, (0.3, -0.2, 0.45), prof, 0.01, dz=0.4)
    # loop collision: the reference geometry, and every string moving (pair 2 too) with dz != dy
    gen_loop_collision_ic("ref_loop_collision_ic", 14, 12, 16, 1.0, 0.05, prof, 0.01)
    gen_loop_collision_ic("ref_loop_collision_ic_moving", 13, 15, 12, 0.7, 0.1, prof, 0.01, dz=0.4,
                          geometry=dict(pos1s=[1.1, -0.9], pos1a=[-0.8, 1.3], pos2s=[1.4, 0.2], pos2a=[-1.2, -0.3],
                                        v1s=[0.1, -0.5, 0.3], v1a=[0.0, 0.6, -0.2], v2s=[0.3, 0.2, 0.0],
                                        v2a=[-0.25, -0.3, 0.1]))
    # ic_w_evolution's own IC, ic_func's older loop collision (no rest-frame positions, boost-only one-forms)
    gen_icfunc_loop_collision("ref_icfunc_loop_collision", 21, 19, 23, 3, g=0.8, profile=prof)


if __name__ == "__main__":
    main()
