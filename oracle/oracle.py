"""Python access to the oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; it is the checker, never the thing measured or shipped.

State arrays use the reference layout (see oracle/lattice_oracle.h):
shape (ncomp, 2, N) float64, slot = time-level parity.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

from axions_gb300.params import LatParams

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liblattice_oracle.so"


class LatDiag(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("gauss_abs_sum", ctypes.c_double),
                ("sites", ctypes.c_int64), ("time_step", ctypes.c_int64)]


_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        P = ctypes.POINTER
        dp = P(ctypes.c_double)
        L.orc_step.argtypes = [P(LatParams), dp, ctypes.c_int64, P(LatDiag)]
        L.orc_diagnostics.argtypes = [P(LatParams), dp, ctypes.c_int64, P(LatDiag)]
        L.orc_detect.argtypes = [P(LatParams), dp, ctypes.c_int64, ctypes.c_int, dp, ctypes.c_int64,
                                 P(ctypes.c_int64)]
        L.orc_winding.argtypes = [P(LatParams), dp, ctypes.c_int64, ctypes.c_int, P(ctypes.c_int8),
                                  P(ctypes.c_int64)]
        L.orc_random_phase_ic.argtypes = [P(LatParams), ctypes.c_uint32, ctypes.c_int, dp]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_get_threads.restype = ctypes.c_int
        L.orc_mt_seed.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
        L.orc_uniform_0_2pi.argtypes = [ctypes.c_void_p]
        L.orc_uniform_0_2pi.restype = ctypes.c_double
        L.orc_apply_boundaries.argtypes = [P(LatParams), dp, ctypes.c_int64]
        L.orc_icfunc_random_ic.argtypes = [P(LatParams), ctypes.c_uint32, dp]
        L.orc_boost_ic.argtypes = [P(LatParams), ctypes.c_void_p, ctypes.c_void_p, dp]
        L.orc_boost_ic.restype = ctypes.c_int64
        for name in ("orc_loop_collision_ic", "orc_icfunc_loop_collision_ic"):
            getattr(L, name).argtypes = [P(LatParams), ctypes.c_void_p, ctypes.c_void_p, dp]
            getattr(L, name).restype = ctypes.c_int64
        L.orc_string_length.argtypes = [P(LatParams), dp, ctypes.c_int64, ctypes.c_int, dp, dp]
        for name in ("orc_ng_sine_ic", "orc_simple_sine_ic"):
            getattr(L, name).argtypes = [P(LatParams), ctypes.c_void_p, ctypes.c_double, dp]
            getattr(L, name).restype = ctypes.c_int64
        L.orc_ng_omega.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int64]
        L.orc_ng_omega.restype = ctypes.c_double
        L.orc_set_trig_perturbation.argtypes = [ctypes.c_double]
        L.orc_ng_column.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


def empty_state(p: LatParams) -> np.ndarray:
    return np.zeros((p.ncomp, 2, p.N), dtype=np.float64)


def random_phase_ic(p: LatParams, seed: int, independent: bool = False) -> np.ndarray:
    st = empty_state(p)
    lib().orc_random_phase_ic(ctypes.byref(p), ctypes.c_uint32(seed), int(independent), _dp(st))
    return st


def uniform_phases(seed: int, count: int) -> np.ndarray:
    """The first `count` draws of uniform_real_distribution(0, 2pi) over mt19937(seed)."""
    g = ctypes.create_string_buffer(624 * 4 + 8)
    L = lib()
    L.orc_mt_seed(g, ctypes.c_uint32(seed))
    return np.array([L.orc_uniform_0_2pi(g) for _ in range(count)])


def step(p: LatParams, st: np.ndarray, n: int, diag: bool = False):
    d = LatDiag()
    rc = lib().orc_step(ctypes.byref(p), _dp(st), int(n), ctypes.byref(d) if diag else None)
    if rc != 0:
        raise RuntimeError(f"orc_step rc={rc}")
    return d if diag else None


def diagnostics(p: LatParams, st: np.ndarray, n: int) -> LatDiag:
    d = LatDiag()
    rc = lib().orc_diagnostics(ctypes.byref(p), _dp(st), int(n), ctypes.byref(d))
    if rc != 0:
        raise RuntimeError(f"orc_diagnostics rc={rc}")
    return d


def evolve(p: LatParams, st: np.ndarray, n0: int, nsteps: int, diag_every: int = 0):
    """Run nsteps from TimeStep n0; return list of (n, energy, gauss_abs_sum)."""
    out = []
    for n in range(n0, n0 + nsteps):
        want = diag_every > 0 and n % diag_every == 0
        d = step(p, st, n, diag=want)
        if want:
            out.append((n, d.energy, d.gauss_abs_sum))
    return out


def detect(p: LatParams, st: np.ndarray, n: int, field: int = 0) -> np.ndarray:
    L = lib()
    cnt = ctypes.c_int64(0)
    rc = L.orc_detect(ctypes.byref(p), _dp(st), int(n), int(field), None, 0, ctypes.byref(cnt))
    if rc != 0:
        raise RuntimeError(f"orc_detect rc={rc}")
    xyz = np.zeros((max(cnt.value, 1), 3), dtype=np.float64)
    rc = L.orc_detect(ctypes.byref(p), _dp(st), int(n), int(field), _dp(xyz), cnt.value, ctypes.byref(cnt))
    if rc != 0:
        raise RuntimeError(f"orc_detect rc={rc}")
    return xyz[: cnt.value]


def winding(p: LatParams, st: np.ndarray, n: int, field: int = 0):
    out = np.zeros((3, p.N), dtype=np.int8)
    tot = ctypes.c_int64(0)
    rc = lib().orc_winding(ctypes.byref(p), _dp(st), int(n), int(field),
                           out.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)), ctypes.byref(tot))
    if rc != 0:
        raise RuntimeError(f"orc_winding rc={rc}")
    return out, int(tot.value)


def apply_boundaries(p: LatParams, st: np.ndarray, n: int) -> None:
    """Neumann boundaries of level n in place (evolution.cpp:194-265)."""
    rc = lib().orc_apply_boundaries(ctypes.byref(p), _dp(st), int(n))
    if rc != 0:
        raise RuntimeError(f"orc_apply_boundaries rc={rc}")


def icfunc_random_ic(p: LatParams, seed: int) -> np.ndarray:
    """ic_func.cpp:647-683 "random" IC (minstd_rand, uniform in [-1, 1])."""
    st = empty_state(p)
    rc = lib().orc_icfunc_random_ic(ctypes.byref(p), int(seed), _dp(st))
    if rc != 0:
        raise RuntimeError(f"orc_icfunc_random_ic rc={rc}")
    return st


def boost_ic(p: LatParams, phi: np.ndarray, A: np.ndarray, h: float, v, form: int = 0, winding: float = 1.0):
    """Boosted straight-string IC (initialConditions.cpp:710-992, form 0;
    ic_func.cpp:685-964, form 1) from the profile table (phi, A) with spacing h.
    Returns (state, number of evaluations off the table)."""
    from axions_gb300.params import boost_ic as _b, string_profile
    prof, keep = string_profile(phi, A, h, winding)
    b = _b(v, form)
    st = empty_state(p)
    off = lib().orc_boost_ic(ctypes.byref(p), ctypes.byref(prof), ctypes.byref(b), _dp(st))
    del keep
    if off < 0:
        raise RuntimeError("orc_boost_ic: bad arguments")
    return st, int(off)


def loop_collision_ic(p: LatParams, phi: np.ndarray, A: np.ndarray, h: float, geometry: dict, winding: float = 1.0,
                      form: str = "initialConditions"):
    """Loop-collision IC: initialConditions.cpp:994-1716, or with form="ic_func"
    ic_func.cpp:966-1720 (the form ic_w_evolution builds in process).
    `geometry` holds pos1s, pos1a, pos2s, pos2a, v1s, v1a, v2s, v2a.  Returns
    (state, number of evaluations off the table)."""
    from axions_gb300.params import loop_collision_ic as _c, string_profile
    if form not in ("initialConditions", "ic_func"):
        raise ValueError("form must be initialConditions or ic_func")
    prof, keep = string_profile(phi, A, h, winding)
    c = _c(**geometry)
    st = empty_state(p)
    fn = lib().orc_loop_collision_ic if form == "initialConditions" else lib().orc_icfunc_loop_collision_ic
    off = fn(ctypes.byref(p), ctypes.byref(prof), ctypes.byref(c), _dp(st))
    del keep
    if off < 0:
        raise RuntimeError("loop collision IC: bad arguments")
    return st, int(off)


def set_trig_perturbation(frac: float) -> None:
    """Test only: one-ulp moves of a fraction `frac` of the step's sin/cos
    results (0 restores the reference's values)."""
    lib().orc_set_trig_perturbation(float(frac))


def sine_string_ic(p: LatParams, phi: np.ndarray, A: np.ndarray, h: float, eps: float, kind: str,
                   winding: float = 1.0):
    """Perturbed straight string of initialConditions.cpp: kind "NG sine"
    (:113-486) or "simple sine" (:488-668), amplitude eps (the value the
    reference reads from standard input), one level in both slots.  Returns
    (state, number of evaluations off the table)."""
    from axions_gb300.params import string_profile
    fn = {"NG sine": "orc_ng_sine_ic", "simple sine": "orc_simple_sine_ic"}[kind]
    prof, keep = string_profile(phi, A, h, winding)
    st = empty_state(p)
    off = getattr(lib(), fn)(ctypes.byref(p), ctypes.byref(prof), float(eps), _dp(st))
    del keep
    if off < 0:
        raise RuntimeError(f"{fn}: bad arguments")
    return st, int(off)


def ng_column(eps: float, Omega: float, x: float, z: float) -> np.ndarray:
    """(xs, zs, xs_sigma, zs_sigma, paraVecMag, normal_dist) of the NG-sine
    string point closest to (x, z)."""
    out = np.zeros(6)
    lib().orc_ng_column(float(eps), float(Omega), float(x), float(z), _dp(out))
    return out


def string_length(p: LatParams, xyz: np.ndarray, split: bool = True):
    """(L0, L1) by greedy chaining of the crossings `xyz` (ic_w_evolution.cpp:961-1087)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    L0 = ctypes.c_double(0)
    L1 = ctypes.c_double(0)
    rc = lib().orc_string_length(ctypes.byref(p), _dp(xyz) if len(xyz) else None, len(xyz), int(bool(split)),
                                 ctypes.byref(L0), ctypes.byref(L1))
    if rc != 0:
        raise RuntimeError(f"orc_string_length rc={rc}")
    return L0.value, L1.value


def now_slot(n: int) -> int:
    return (n + 1) % 2


def past_slot(n: int) -> int:
    return n % 2
