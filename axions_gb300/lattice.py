"""Python mirror of the C ABI in include/lattice_gpu.h (ctypes).

This is how tests, the benchmark and Python users drive the CUDA library.  It
loads axions_gb300/liblattice_gpu.so from this package directory and raises if
it is missing or cannot reach a GPU: there is no CPU fallback.

Array conventions (same as the C ABI): a level is float64 of shape
(ncomp, nx*ny*nz); components AH = (phi_re, phi_im, theta_x, theta_y,
theta_z), Moore = (phi1_re, phi1_im, phi2_re, phi2_im, theta_x, theta_y,
theta_z); sites in linear order (i*ny + j)*nz + k.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from .params import (LAT_ERR_CAPACITY, LAT_OK, LatParams, MODEL_AH, make_params)  # noqa: F401

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "liblattice_gpu.so"

# every entry point declared in include/lattice_gpu.h
EXPORTS = [
    "lat_version", "lat_last_error", "lat_params_init", "lat_random_phase_ic", "lat_create", "lat_destroy",
    "lat_set_stream", "lat_get_params", "lat_num_components", "lat_time_step", "lat_device_bytes",
    "lat_kernel_launches",
    "lat_set_state", "lat_get_state", "lat_step", "lat_step_diag", "lat_advance", "lat_run", "lat_diagnostics",
    "lat_detect_crossings", "lat_winding", "lat_string_length", "lat_string_length_points", "lat_set_chain_wait",
    "lat_snapshot_doubles", "lat_snapshot_begin", "lat_snapshot_wait", "lat_host_alloc", "lat_host_free",
    "lat_ah_step_f64_noalloc",
    "lat_batch_create", "lat_batch_destroy", "lat_batch_add", "lat_batch_remove", "lat_batch_size",
    "lat_batch_kernel_launches", "lat_batch_set_chunk", "lat_batch_advance", "lat_batch_take_diags",
    "lat_random_phase_ic_device", "lat_boost_ic_device", "lat_loop_collision_ic_device",
    "lat_icfunc_loop_collision_ic_device",
    "lat_ng_sine_ic_device", "lat_simple_sine_ic_device", "lat_philox4x32_10", "lat_dtrig_eval", "lat_autotune", "lat_get_tuning", "lat_set_tuning",
    "lat_tune_cache_save", "lat_tune_cache_load", "lat_footprint_bytes",
    "lat_server_create", "lat_server_submit", "lat_server_poll", "lat_server_wait", "lat_server_diags",
    "lat_server_get_stats", "lat_server_destroy",
]


class LatTuning(ctypes.Structure):
    _fields_ = [("chunk", ctypes.c_int32), ("candidates", ctypes.c_int32), ("ms_per_step", ctypes.c_double)]


class LatDiag(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("gauss_abs_sum", ctypes.c_double),
                ("sites", ctypes.c_int64), ("time_step", ctypes.c_int64)]


class LatticeError(RuntimeError):
    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed with status {code}: {msg}")
        self.code = code


_lib = None


def load_library(path: Path | None = None):
    """Load the CUDA library (build it first with axions_gb300.build)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} not found: build it with `python -m axions_gb300.build` "
                           "(no CPU fallback exists)")
    L = ctypes.CDLL(str(p))
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    dp = P(ctypes.c_double)
    L.lat_version.restype = ctypes.c_char_p
    L.lat_last_error.restype = ctypes.c_char_p
    L.lat_params_init.argtypes = [P(LatParams), ctypes.c_int32]
    L.lat_random_phase_ic.argtypes = [P(LatParams), ctypes.c_uint32, ctypes.c_int32, dp]
    L.lat_create.argtypes = [P(LatParams), P(vp)]
    L.lat_destroy.argtypes = [vp]
    L.lat_set_stream.argtypes = [vp, vp]
    L.lat_get_params.argtypes = [vp, P(LatParams)]
    L.lat_num_components.argtypes = [vp]
    L.lat_time_step.argtypes = [vp]
    L.lat_time_step.restype = ctypes.c_int64
    L.lat_device_bytes.argtypes = [vp]
    L.lat_device_bytes.restype = ctypes.c_int64
    L.lat_kernel_launches.argtypes = [vp]
    L.lat_kernel_launches.restype = ctypes.c_int64
    L.lat_set_state.argtypes = [vp, dp, dp, ctypes.c_int64]
    L.lat_get_state.argtypes = [vp, dp, dp]
    L.lat_step.argtypes = [vp, ctypes.c_int32]
    L.lat_step_diag.argtypes = [vp, P(LatDiag)]
    L.lat_advance.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, P(LatDiag), ctypes.c_int64, P(ctypes.c_int64)]
    L.lat_run.argtypes = [vp, dp, dp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, P(LatDiag), ctypes.c_int64,
                          P(ctypes.c_int64), dp, dp]
    L.lat_diagnostics.argtypes = [vp, P(LatDiag)]
    L.lat_detect_crossings.argtypes = [vp, ctypes.c_int32, dp, ctypes.c_int64, P(ctypes.c_int64)]
    L.lat_winding.argtypes = [vp, ctypes.c_int32, P(ctypes.c_int8), P(ctypes.c_int64)]
    L.lat_string_length.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, dp, dp, P(ctypes.c_int64)]
    L.lat_snapshot_doubles.argtypes = [vp, ctypes.c_int32]
    L.lat_snapshot_doubles.restype = ctypes.c_int64
    L.lat_snapshot_begin.argtypes = [vp, ctypes.c_int32, dp]
    L.lat_snapshot_wait.argtypes = [vp]
    L.lat_host_alloc.argtypes = [ctypes.c_int64]
    L.lat_host_alloc.restype = vp
    L.lat_host_free.argtypes = [vp]
    L.lat_string_length_points.argtypes = [P(LatParams), dp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, dp, dp]
    L.lat_set_chain_wait.argtypes = [ctypes.c_int64, ctypes.c_int32]
    L.lat_ah_step_f64_noalloc.argtypes = [P(LatParams), vp, ctypes.c_int64, ctypes.c_int32, vp]
    L.lat_batch_create.argtypes = [ctypes.c_int32, P(vp)]
    L.lat_batch_destroy.argtypes = [vp]
    L.lat_batch_add.argtypes = [vp, vp, ctypes.c_int32, ctypes.c_int64]
    L.lat_batch_remove.argtypes = [vp, vp]
    L.lat_batch_size.argtypes = [vp]
    L.lat_batch_kernel_launches.argtypes = [vp]
    L.lat_batch_kernel_launches.restype = ctypes.c_int64
    L.lat_batch_advance.argtypes = [vp, ctypes.c_int32]
    L.lat_batch_set_chunk.argtypes = [vp, ctypes.c_int32]
    L.lat_batch_take_diags.argtypes = [vp, vp, P(LatDiag), ctypes.c_int64, P(ctypes.c_int64)]
    u32p = P(ctypes.c_uint32)
    L.lat_random_phase_ic_device.argtypes = [vp, ctypes.c_uint64, ctypes.c_int32]
    L.lat_boost_ic_device.argtypes = [vp, vp, vp, P(ctypes.c_int64)]
    L.lat_loop_collision_ic_device.argtypes = [vp, vp, vp, P(ctypes.c_int64)]
    L.lat_icfunc_loop_collision_ic_device.argtypes = [vp, vp, vp, P(ctypes.c_int64)]
    L.lat_ng_sine_ic_device.argtypes = [vp, vp, ctypes.c_double, P(ctypes.c_int64)]
    L.lat_simple_sine_ic_device.argtypes = [vp, vp, ctypes.c_double, P(ctypes.c_int64)]
    L.lat_philox4x32_10.argtypes = [u32p, u32p, u32p]
    L.lat_dtrig_eval.argtypes = [dp, ctypes.c_int64, dp]
    L.lat_autotune.argtypes = [vp, ctypes.c_int32, P(LatTuning)]
    L.lat_get_tuning.argtypes = [vp, P(LatTuning)]
    L.lat_set_tuning.argtypes = [vp, P(LatTuning)]
    L.lat_tune_cache_save.argtypes = [ctypes.c_char_p]
    L.lat_tune_cache_load.argtypes = [ctypes.c_char_p]
    L.lat_footprint_bytes.argtypes = [P(LatParams)]
    L.lat_footprint_bytes.restype = ctypes.c_int64
    L.lat_server_create.argtypes = [vp, P(vp)]
    L.lat_server_submit.argtypes = [vp, vp, P(ctypes.c_int64)]
    L.lat_server_poll.argtypes = [vp, ctypes.c_int64, vp]
    L.lat_server_wait.argtypes = [vp, ctypes.c_int64, ctypes.c_double, vp]
    L.lat_server_diags.argtypes = [vp, ctypes.c_int64, P(LatDiag), ctypes.c_int64, P(ctypes.c_int64)]
    L.lat_server_get_stats.argtypes = [vp, vp]
    L.lat_server_destroy.argtypes = [vp]
    if path is None:
        _lib = L
    return L


def _dp(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check(fn: str, rc: int):
    if rc != LAT_OK:
        raise LatticeError(fn, rc, (load_library().lat_last_error() or b"").decode())


def params_init(model: int = MODEL_AH) -> LatParams:
    p = LatParams()
    _check("lat_params_init", load_library().lat_params_init(ctypes.byref(p), int(model)))
    return p


def random_phase_ic(p: LatParams, seed: int, independent: bool = False) -> np.ndarray:
    """Seeded uniform-phase IC of mpi_evolution.cpp:287-312 (one level, (ncomp, N))."""
    out = np.zeros((p.ncomp, p.N), dtype=np.float64)
    _check("lat_random_phase_ic",
           load_library().lat_random_phase_ic(ctypes.byref(p), ctypes.c_uint32(seed), int(bool(independent)), _dp(out)))
    return out


def philox4x32_10(counter, key):
    """Philox-4x32-10 (the generator of Lattice.random_phase_ic_device) on the host."""
    c = (ctypes.c_uint32 * 4)(*counter)
    k = (ctypes.c_uint32 * 2)(*key)
    out = (ctypes.c_uint32 * 4)()
    _check("lat_philox4x32_10", load_library().lat_philox4x32_10(c, k, out))
    return list(out)


def dtrig_eval(x):
    """The FP64 step's sine and cosine at the doubles x, on the current GPU.
    Returns (sin, sincos_sin, sincos_cos, cuda_sin, cuda_cos) as arrays."""
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    out = np.empty(5 * x.size, dtype=np.float64)
    _check("lat_dtrig_eval", load_library().lat_dtrig_eval(_dp(x), x.size, _dp(out)))
    return tuple(out.reshape(5, x.size))


def tune_cache_save(path) -> None:
    _check("lat_tune_cache_save", load_library().lat_tune_cache_save(str(path).encode()))


def tune_cache_load(path) -> int:
    rc = load_library().lat_tune_cache_load(str(path).encode())
    if rc < 0:
        _check("lat_tune_cache_load", rc)
    return rc


class Lattice:
    """One lattice resident on the current CUDA device."""

    def __init__(self, params: LatParams):
        self.L = load_library()
        self.params = params.copy()
        h = ctypes.c_void_p()
        _check("lat_create", self.L.lat_create(ctypes.byref(self.params), ctypes.byref(h)))
        self.h = h
        self.ncomp = self.params.ncomp
        self.N = self.params.N

    # lifetime ------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.lat_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # properties ------------------------------------------------------------
    @property
    def time_step(self) -> int:
        return int(self.L.lat_time_step(self.h))

    @property
    def kernel_launches(self) -> int:
        return int(self.L.lat_kernel_launches(self.h))

    @property
    def device_bytes(self) -> int:
        return int(self.L.lat_device_bytes(self.h))

    def random_phase_ic_device(self, seed: int, independent: bool = False):
        """Random-phase IC drawn on the GPU (Philox-4x32-10); state at TimeStep 0."""
        _check("lat_random_phase_ic_device",
               self.L.lat_random_phase_ic_device(self.h, ctypes.c_uint64(seed), int(bool(independent))))

    def boost_ic_device(self, phi, A, h: float, v, form: int = 0, winding: float = 1.0) -> int:
        """Boosted straight-string IC (initialConditions.cpp:710-992, form 0;
        ic_func.cpp:685-964, form 1) from the profile table (phi, A) with
        spacing h, built on the GPU; state at TimeStep 0.  Returns the number
        of site evaluations that fell beyond the table."""
        from .params import boost_ic, string_profile
        prof, keep = string_profile(phi, A, h, winding)
        b = boost_ic(v, form)
        off = ctypes.c_int64(0)
        _check("lat_boost_ic_device", self.L.lat_boost_ic_device(self.h, ctypes.byref(prof), ctypes.byref(b),
                                                                 ctypes.byref(off)))
        del keep
        return int(off.value)

    def loop_collision_ic_device(self, phi, A, h: float, geometry: dict | None = None, winding: float = 1.0,
                                 form: str = "initialConditions") -> int:
        """Loop-collision IC from the profile table (phi, A) with spacing h,
        built on the GPU; state at TimeStep 0.  form "initialConditions":
        initialConditions.cpp:994-1716, `geometry` (pos1s, pos1a, pos2s, pos2a,
        v1s, v1a, v2s, v2a) defaulting to its placement for this lattice; form
        "ic_func": the older ic_func.cpp:966-1720 that ic_w_evolution builds,
        defaulting to ic_func.cpp:61-72.  Returns the number of site
        evaluations beyond the table."""
        from .params import default_loop_collision, icfunc_loop_collision, loop_collision_ic, string_profile
        if form not in ("initialConditions", "ic_func"):
            raise ValueError("form must be initialConditions or ic_func")
        p = self.params
        geo = (default_loop_collision if form == "initialConditions" else icfunc_loop_collision)(
            p.nx, p.ny, p.nz, p.dx, p.dy, p.dz)
        geo.update(geometry or {})
        prof, keep = string_profile(phi, A, h, winding)
        c = loop_collision_ic(**geo)
        off = ctypes.c_int64(0)
        name = "lat_loop_collision_ic_device" if form == "initialConditions" else "lat_icfunc_loop_collision_ic_device"
        _check(name, getattr(self.L, name)(self.h, ctypes.byref(prof), ctypes.byref(c), ctypes.byref(off)))
        del keep
        return int(off.value)

    def sine_string_ic_device(self, phi, A, h: float, eps: float, kind: str = "NG sine",
                              winding: float = 1.0) -> int:
        """A straight string perturbed by a sine wave (initialConditions.cpp
        "NG sine" :113-486 or "simple sine" :488-668, amplitude eps) from the
        profile table (phi, A) with spacing h, built on the GPU into both slots;
        state at TimeStep 0.  Returns the number of evaluations beyond the table."""
        from .params import string_profile
        fn = {"NG sine": "lat_ng_sine_ic_device", "simple sine": "lat_simple_sine_ic_device"}[kind]
        prof, keep = string_profile(phi, A, h, winding)
        off = ctypes.c_int64(0)
        _check(fn, getattr(self.L, fn)(self.h, ctypes.byref(prof), float(eps), ctypes.byref(off)))
        del keep
        return int(off.value)

    def autotune(self, trial_steps: int = 3) -> LatTuning:
        t = LatTuning()
        _check("lat_autotune", self.L.lat_autotune(self.h, int(trial_steps), ctypes.byref(t)))
        return t

    @property
    def tuning(self) -> LatTuning:
        t = LatTuning()
        _check("lat_get_tuning", self.L.lat_get_tuning(self.h, ctypes.byref(t)))
        return t

    def set_chunk(self, chunk: int):
        t = LatTuning()
        t.chunk = int(chunk)
        _check("lat_set_tuning", self.L.lat_set_tuning(self.h, ctypes.byref(t)))

    def set_stream(self, stream_handle: int | None):
        _check("lat_set_stream", self.L.lat_set_stream(self.h, ctypes.c_void_p(stream_handle or 0)))

    # state -----------------------------------------------------------------
    def set_state(self, now: np.ndarray, past: np.ndarray | None = None, time_step: int = 0):
        now = np.ascontiguousarray(now, dtype=np.float64).reshape(self.ncomp, self.N)
        past = now if past is None else np.ascontiguousarray(past, dtype=np.float64).reshape(self.ncomp, self.N)
        _check("lat_set_state", self.L.lat_set_state(self.h, _dp(now), _dp(past), int(time_step)))

    def set_slots(self, st: np.ndarray, time_step: int):
        """Upload a reference-layout state (ncomp, 2, N) whose slot parity matches time_step."""
        now = np.ascontiguousarray(st[:, (time_step + 1) % 2, :])
        past = np.ascontiguousarray(st[:, time_step % 2, :])
        self.set_state(now, past, time_step)

    def get_state(self, now: np.ndarray | None = None, past: np.ndarray | None = None):
        """Download (now, past) as float64 arrays of shape (ncomp, N).  Arrays
        passed in (C-contiguous float64 of that shape, e.g. views of pinned
        buffers reused across calls) receive the levels; others are allocated."""
        out = []
        for a in (now, past):
            if a is None:
                a = np.empty((self.ncomp, self.N), dtype=np.float64)
            elif a.dtype != np.float64 or not a.flags.c_contiguous or a.size != self.ncomp * self.N:
                raise ValueError("get_state: output arrays must be C-contiguous float64 of ncomp*N elements")
            out.append(a)
        _check("lat_get_state", self.L.lat_get_state(self.h, _dp(out[0]), _dp(out[1])))
        return out[0].reshape(self.ncomp, self.N), out[1].reshape(self.ncomp, self.N)

    def get_slots(self) -> np.ndarray:
        n = self.time_step
        now, past = self.get_state()
        st = np.empty((self.ncomp, 2, self.N), dtype=np.float64)
        st[:, (n + 1) % 2, :] = now
        st[:, n % 2, :] = past
        return st

    # evolution ---------------------------------------------------------------
    def step(self, nsteps: int = 1):
        _check("lat_step", self.L.lat_step(self.h, int(nsteps)))

    def step_diag(self) -> LatDiag:
        d = LatDiag()
        _check("lat_step_diag", self.L.lat_step_diag(self.h, ctypes.byref(d)))
        return d

    def advance(self, nsteps: int, diag_every: int = 0):
        """Run nsteps; return a list of (time_step, energy, gauss_abs_sum)."""
        cap = 0
        if diag_every > 0:
            n0 = self.time_step
            cap = sum(1 for n in range(n0, n0 + nsteps) if n % diag_every == 0)
        buf = (LatDiag * max(cap, 1))()
        cnt = ctypes.c_int64(0)
        _check("lat_advance", self.L.lat_advance(self.h, int(nsteps), int(diag_every), buf, int(cap), ctypes.byref(cnt)))
        return [(buf[q].time_step, buf[q].energy, buf[q].gauss_abs_sum) for q in range(cnt.value)]

    def run(self, now: np.ndarray, past: np.ndarray | None, time_step: int, nsteps: int, diag_every: int = 0,
            now_out: np.ndarray | None = None, past_out: np.ndarray | None = None, past_level: bool = True):
        """set_state + advance + get_state in one call (lat_run).  past None:
        a stationary start, both levels `now` (uploaded once).  Returns
        (diagnostics, now_out, past_out); output arrays passed in (C-contiguous
        float64 of ncomp*N elements, e.g. pinned buffers) are filled, others
        allocated; with past_level False the past level is not downloaded and
        past_out is None."""
        now = np.ascontiguousarray(now, dtype=np.float64).reshape(self.ncomp, self.N)
        past = now if past is None else np.ascontiguousarray(past, dtype=np.float64).reshape(self.ncomp, self.N)
        outs = []
        for a, want in ((now_out, True), (past_out, past_level)):
            if not want:
                outs.append(None)
                continue
            if a is None:
                a = np.empty((self.ncomp, self.N), dtype=np.float64)
            elif a.dtype != np.float64 or not a.flags.c_contiguous or a.size != self.ncomp * self.N:
                raise ValueError("run: output arrays must be C-contiguous float64 of ncomp*N elements")
            outs.append(a)
        cap = 0
        if diag_every > 0:
            cap = sum(1 for n in range(time_step, time_step + nsteps) if n % diag_every == 0)
        buf = (LatDiag * max(cap, 1))()
        cnt = ctypes.c_int64(0)
        _check("lat_run", self.L.lat_run(self.h, _dp(now), _dp(past), int(time_step), int(nsteps), int(diag_every),
                                         buf, int(cap), ctypes.byref(cnt), _dp(outs[0]),
                                         _dp(outs[1]) if outs[1] is not None else None))
        diags = [(buf[q].time_step, buf[q].energy, buf[q].gauss_abs_sum) for q in range(cnt.value)]
        return (diags, outs[0].reshape(self.ncomp, self.N),
                outs[1].reshape(self.ncomp, self.N) if outs[1] is not None else None)

    def diagnostics(self) -> LatDiag:
        d = LatDiag()
        _check("lat_diagnostics", self.L.lat_diagnostics(self.h, ctypes.byref(d)))
        return d

    # detection -----------------------------------------------------------------
    def detect(self, field: int = 0) -> np.ndarray:
        cnt = ctypes.c_int64(0)
        _check("lat_detect_crossings", self.L.lat_detect_crossings(self.h, int(field), None, 0, ctypes.byref(cnt)))
        n = cnt.value
        xyz = np.zeros((max(n, 1), 3), dtype=np.float64)
        if n:
            _check("lat_detect_crossings",
                   self.L.lat_detect_crossings(self.h, int(field), _dp(xyz), n, ctypes.byref(cnt)))
        return xyz[:n]

    # asynchronous snapshots ------------------------------------------------------
    def snapshot_begin(self, kind: int, out: np.ndarray):
        """Start copying |phi|^2 (SNAP_MAGNITUDE) or the level (SNAP_LEVEL) of the
        current level into `out` (float64, snapshot_doubles(kind) values; keep it
        alive until snapshot_wait)."""
        n = int(self.L.lat_snapshot_doubles(self.h, int(kind)))
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size >= n
        self._snap_out = out
        _check("lat_snapshot_begin", self.L.lat_snapshot_begin(self.h, int(kind), _dp(out)))

    def snapshot_wait(self):
        _check("lat_snapshot_wait", self.L.lat_snapshot_wait(self.h))
        self._snap_out = None

    def snapshot_doubles(self, kind: int) -> int:
        return int(self.L.lat_snapshot_doubles(self.h, int(kind)))

    def count_crossings(self, field: int = 0) -> int:
        """Number of bilinear crossings on the current level (nothing copied)."""
        cnt = ctypes.c_int64(0)
        _check("lat_detect_crossings", self.L.lat_detect_crossings(self.h, int(field), None, 0, ctypes.byref(cnt)))
        return int(cnt.value)

    def winding(self, field: int = 0, want_array: bool = True):
        tot = ctypes.c_int64(0)
        out = np.zeros((3, self.N), dtype=np.int8) if want_array else None
        ptr = out.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)) if want_array else None
        _check("lat_winding", self.L.lat_winding(self.h, int(field), ptr, ctypes.byref(tot)))
        return out, int(tot.value)

    def string_length(self, field: int = 0, split: bool = True, method: int = 0):
        """(L0, L1, crossings): greedy chaining of the current level's crossings
        (lat_string_length; ic_w_evolution.cpp:961-1087)."""
        L0, L1, cnt = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_int64(0)
        _check("lat_string_length", self.L.lat_string_length(self.h, int(field), int(bool(split)), int(method),
                                                             ctypes.byref(L0), ctypes.byref(L1), ctypes.byref(cnt)))
        return L0.value, L1.value, int(cnt.value)


class Batch:
    """Many FP32 lattices advanced together (lat_batch_* of the C ABI).

    Every lattice of the batch steps in the same kernel launches; a call
    advancing K steps is one CUDA graph.  Results per lattice are bitwise the
    same as stepping it alone.
    """

    def __init__(self, max_jobs: int = 64):
        self.L = load_library()
        b = ctypes.c_void_p()
        _check("lat_batch_create", self.L.lat_batch_create(int(max_jobs), ctypes.byref(b)))
        self.b = b
        self.members = []

    def add(self, lat: "Lattice", diag_every: int = 0, stop_step: int | None = None) -> int:
        stop = (1 << 62) if stop_step is None else int(stop_step)
        rc = self.L.lat_batch_add(self.b, lat.h, int(diag_every), stop)
        if rc < 0:
            _check("lat_batch_add", rc)
        self.members.append(lat)
        return rc

    def remove(self, lat: "Lattice"):
        _check("lat_batch_remove", self.L.lat_batch_remove(self.b, lat.h))
        self.members.remove(lat)

    def advance(self, nsteps: int) -> int:
        rc = self.L.lat_batch_advance(self.b, int(nsteps))
        if rc < 0:
            _check("lat_batch_advance", rc)
        return rc

    def take_diags(self, lat: "Lattice"):
        cnt = ctypes.c_int64(0)
        _check("lat_batch_take_diags", self.L.lat_batch_take_diags(self.b, lat.h, None, 0, ctypes.byref(cnt)))
        n = cnt.value
        buf = (LatDiag * max(n, 1))()
        _check("lat_batch_take_diags", self.L.lat_batch_take_diags(self.b, lat.h, buf, n, ctypes.byref(cnt)))
        return [(buf[q].time_step, buf[q].energy, buf[q].gauss_abs_sum) for q in range(n)]

    @property
    def size(self) -> int:
        return int(self.L.lat_batch_size(self.b))

    @property
    def kernel_launches(self) -> int:
        return int(self.L.lat_batch_kernel_launches(self.b))

    def set_chunk(self, chunk: int):
        """x-planes per work item of every lattice (0: the per-shape default)."""
        _check("lat_batch_set_chunk", self.L.lat_batch_set_chunk(self.b, int(chunk)))

    def close(self):
        if getattr(self, "b", None) is not None and self.b.value:
            self.L.lat_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_int64), ("tick_steps", ctypes.c_int32), ("max_running", ctypes.c_int32)]


class JobSpec(ctypes.Structure):
    _fields_ = [("params", LatParams), ("seed", ctypes.c_uint64), ("nsteps", ctypes.c_int32),
                ("diag_every", ctypes.c_int32), ("independent", ctypes.c_int32), ("winding_at_end", ctypes.c_int32)]


class JobResult(ctypes.Structure):
    _fields_ = [("job_id", ctypes.c_int64), ("status", ctypes.c_int32), ("ndiag", ctypes.c_int32),
                ("submit_s", ctypes.c_double), ("start_s", ctypes.c_double), ("end_s", ctypes.c_double),
                ("final_energy", ctypes.c_double), ("final_gauss", ctypes.c_double),
                ("winding_abs", ctypes.c_int64), ("site_updates", ctypes.c_int64)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in ("submitted", "queued", "running", "done", "failed", "site_updates",
                                              "ticks", "running_bytes", "pooled_bytes", "peak_bytes")] + \
               [("busy_s", ctypes.c_double), ("wall_s", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


CHAIN_AUTO, CHAIN_HASH, CHAIN_EXHAUSTIVE = 0, 1, 2
SNAP_MAGNITUDE, SNAP_LEVEL = 0, 1


class PinnedArray:
    """float64 array in page-locked host memory (lat_host_alloc), for snapshots
    that overlap the steps."""

    def __init__(self, n: int):
        self.L = load_library()
        self.ptr = self.L.lat_host_alloc(8 * max(int(n), 1))
        if not self.ptr:
            raise LatticeError("lat_host_alloc", -2, (self.L.lat_last_error() or b"").decode())
        buf = (ctypes.c_double * max(int(n), 1)).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=np.float64, count=int(n))

    def close(self):
        if self.ptr:
            self.array = None
            self.L.lat_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        self.close()


def string_length_points(p: LatParams, xyz: np.ndarray, split: bool = True, method: int = CHAIN_AUTO):
    """(L0, L1) of a host crossing list chained on the current device (lat_string_length_points)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    L0, L1 = ctypes.c_double(0), ctypes.c_double(0)
    ptr = _dp(xyz) if len(xyz) else None
    _check("lat_string_length_points",
           load_library().lat_string_length_points(ctypes.byref(p), ptr, len(xyz), int(bool(split)), int(method),
                                                   ctypes.byref(L0), ctypes.byref(L1)))
    return L0.value, L1.value


def footprint_bytes(p: LatParams) -> int:
    """Device bytes a lattice with these parameters holds (lat_footprint_bytes)."""
    return int(load_library().lat_footprint_bytes(ctypes.byref(p)))


class Server:
    """Job queue with continuous batching on the current device (lat_server_*)."""

    def __init__(self, hbm_budget_bytes: int, tick_steps: int = 25, max_running: int = 128):
        self.L = load_library()
        cfg = ServerConfig(int(hbm_budget_bytes), int(tick_steps), int(max_running))
        s = ctypes.c_void_p()
        _check("lat_server_create", self.L.lat_server_create(ctypes.byref(cfg), ctypes.byref(s)))
        self.s = s

    def submit(self, params: LatParams, seed: int, nsteps: int, diag_every: int = 0, independent: bool = False,
               winding_at_end: bool = True) -> int:
        spec = JobSpec(params, int(seed), int(nsteps), int(diag_every), int(bool(independent)), int(bool(winding_at_end)))
        jid = ctypes.c_int64()
        _check("lat_server_submit", self.L.lat_server_submit(self.s, ctypes.byref(spec), ctypes.byref(jid)))
        return jid.value

    def poll(self, job_id: int) -> JobResult:
        r = JobResult()
        _check("lat_server_poll", self.L.lat_server_poll(self.s, int(job_id), ctypes.byref(r)))
        return r

    def wait(self, job_id: int, timeout_s: float = 600.0) -> JobResult:
        r = JobResult()
        _check("lat_server_wait", self.L.lat_server_wait(self.s, int(job_id), float(timeout_s), ctypes.byref(r)))
        return r

    def diags(self, job_id: int):
        cnt = ctypes.c_int64()
        _check("lat_server_diags", self.L.lat_server_diags(self.s, int(job_id), None, 0, ctypes.byref(cnt)))
        buf = (LatDiag * max(cnt.value, 1))()
        _check("lat_server_diags", self.L.lat_server_diags(self.s, int(job_id), buf, cnt.value, ctypes.byref(cnt)))
        return [(buf[q].time_step, buf[q].energy, buf[q].gauss_abs_sum) for q in range(cnt.value)]

    def stats(self) -> ServerStats:
        st = ServerStats()
        _check("lat_server_get_stats", self.L.lat_server_get_stats(self.s, ctypes.byref(st)))
        return st

    def close(self):
        if getattr(self, "s", None) is not None and self.s.value:
            self.L.lat_server_destroy(self.s)
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
