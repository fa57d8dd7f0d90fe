"""Parameter block of the lattice library, mirrored for Python (ctypes).

Field names and defaults are the reference's compile-time constants
(mpi_evolution.cpp:15-60 for Abelian-Higgs, moore_mpi_evolution.cpp:15-65 for
the Moore model); the layout is `lat_params` of include/lattice_gpu.h.
"""
from __future__ import annotations

import ctypes
import math

LAT_ABI_VERSION = 1

LAT_OK = 0
LAT_ERR_INVALID = -1
LAT_ERR_NOMEM = -2
LAT_ERR_CUDA = -3
LAT_ERR_TIMEOUT = -4
LAT_ERR_CAPACITY = -5
LAT_ERR_STATE = -6
LAT_ERR_NODEVICE = -7

MODEL_AH = 0
MODEL_MOORE = 1
F64 = 0
F32 = 1
F64_FAST = 2
BC_PERIODIC = 0
BC_FIXED = 1
BC_NEUMANN = 2
BC_ABSORBING = 3
BCZ_AS_XY, BCZ_PERIODIC, BCZ_FIXED, BCZ_NEUMANN = 0, 1, 2, 3
ENERGY_EVOLUTION = 0
ENERGY_MPI = 1
MOORE_CURRENT_PLAIN = 0
MOORE_CURRENT_CHARGE = 1


class LatParams(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_int32),
        ("model", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("bc", ctypes.c_int32),
        ("nx", ctypes.c_int64),
        ("ny", ctypes.c_int64),
        ("nz", ctypes.c_int64),
        ("dx", ctypes.c_double),
        ("dy", ctypes.c_double),
        ("dz", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("lam", ctypes.c_double),      # C name: lambda
        ("eta", ctypes.c_double),
        ("lambda2", ctypes.c_double),
        ("eta2", ctypes.c_double),
        ("lambda12", ctypes.c_double),
        ("g", ctypes.c_double),
        ("q1", ctypes.c_double),
        ("q2", ctypes.c_double),
        ("damped_nt", ctypes.c_int32),
        ("moore_current", ctypes.c_int32),
        ("dampFac", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("scaling", ctypes.c_double),
        ("tau0", ctypes.c_double),
        ("energy_form", ctypes.c_int32),
        ("kernel_variant", ctypes.c_int32),
        ("bc_z", ctypes.c_int32),
        ("reserved_i", ctypes.c_int32),
        ("reserved", ctypes.c_double * 3),
    ]

    @property
    def N(self) -> int:
        return int(self.nx) * int(self.ny) * int(self.nz)

    @property
    def ncomp(self) -> int:
        return 7 if self.model == MODEL_MOORE else 5

    def copy(self) -> "LatParams":
        c = LatParams()
        ctypes.pointer(c)[0] = self
        return c

    def as_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            if name.startswith("reserved"):
                continue
            d[name] = getattr(self, name)
        return d


def default_params(model: int = MODEL_AH) -> LatParams:
    """Reference defaults (mpi_evolution.cpp:15-60 / moore_mpi_evolution.cpp:15-65).

    The same values are filled by lat_params_init() in the C library.
    """
    p = LatParams()
    p.abi_version = LAT_ABI_VERSION
    p.model = model
    p.precision = F64
    p.bc = BC_PERIODIC
    p.nx = p.ny = p.nz = 1001
    p.dx = p.dy = p.dz = 0.25
    p.dt = 0.05
    p.damped_nt = 200
    p.dampFac = 0.5
    p.alpha = 3.0
    p.scaling = 1.0
    p.tau0 = 1.0
    p.energy_form = ENERGY_MPI
    if model == MODEL_AH:
        p.lam = 1.0
        p.eta = 1.0
        p.g = 0.0 * math.sqrt(0.5 * 1.0)
        p.lambda2 = 0.0
        p.eta2 = 0.0
        p.lambda12 = 0.0
        p.q1 = 1.0
        p.q2 = 0.0
        p.moore_current = MOORE_CURRENT_PLAIN
    else:
        p.lam = 1.0
        p.lambda2 = 1.0
        p.lambda12 = 0.0
        p.eta = 1.0
        p.eta2 = 1.0
        p.q1 = 2.0
        p.q2 = 1.0
        p.g = math.sqrt(0.5 * 1.0 * 1.0 ** 2 / (2 * 2 + 1 * 1))
        p.moore_current = MOORE_CURRENT_PLAIN
    return p


def make_params(model: int = MODEL_AH, **kw) -> LatParams:
    """Defaults overridden by keyword (reference names; `lambda` may be given as `lam`)."""
    p = default_params(model)
    for k, v in kw.items():
        if k == "lambda":
            k = "lam"
        if k in ("lambda1",):
            k = "lam"
        if k in ("eta1",):
            k = "eta"
        if k == "n":
            p.nx = p.ny = p.nz = int(v)
            continue
        if k == "d":
            p.dx = p.dy = p.dz = float(v)
            continue
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


# ---- string initial conditions (lat_string_profile, lat_boost_ic) ----------
IC_FORM_FILE = 0        # initialConditions.cpp rounding
IC_FORM_INPROCESS = 1   # ic_func.cpp rounding


class LatStringProfile(ctypes.Structure):
    _fields_ = [("phi", ctypes.POINTER(ctypes.c_double)), ("A", ctypes.POINTER(ctypes.c_double)),
                ("m", ctypes.c_int64), ("h", ctypes.c_double), ("winding", ctypes.c_double)]


class LatBoostIC(ctypes.Structure):
    _fields_ = [("v", ctypes.c_double * 3), ("form", ctypes.c_int32), ("reserved", ctypes.c_int32)]


def string_profile(phi, A, h: float, winding: float = 1.0):
    """A LatStringProfile over float64 copies of phi and A; returns (struct,
    arrays) — keep the arrays alive while the struct is in use."""
    import numpy as np
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    A = np.ascontiguousarray(A, dtype=np.float64)
    if phi.shape != A.shape or phi.ndim != 1:
        raise ValueError("phi and A must be 1-d arrays of the same length")
    dp = ctypes.POINTER(ctypes.c_double)
    s = LatStringProfile(phi.ctypes.data_as(dp), A.ctypes.data_as(dp), len(phi), float(h), float(winding))
    return s, (phi, A)


def boost_ic(v, form: int = IC_FORM_FILE) -> LatBoostIC:
    b = LatBoostIC()
    for q in range(3):
        b.v[q] = float(v[q])
    b.form = int(form)
    return b


class LatLoopCollisionIC(ctypes.Structure):
    _fields_ = [("pos1s", ctypes.c_double * 2), ("pos1a", ctypes.c_double * 2), ("pos2s", ctypes.c_double * 2),
                ("pos2a", ctypes.c_double * 2), ("v1s", ctypes.c_double * 3), ("v1a", ctypes.c_double * 3),
                ("v2s", ctypes.c_double * 3), ("v2a", ctypes.c_double * 3)]


LOOP_COLLISION_KEYS = ("pos1s", "pos1a", "pos2s", "pos2a", "v1s", "v1a", "v2s", "v2a")


def loop_collision_ic(**geo) -> LatLoopCollisionIC:
    """LatLoopCollisionIC from keyword arrays (all eight keys required)."""
    c = LatLoopCollisionIC()
    for k in LOOP_COLLISION_KEYS:
        dst = getattr(c, k)
        src = geo[k]
        if len(src) != len(dst):
            raise ValueError(f"{k} needs {len(dst)} values")
        for q in range(len(dst)):
            dst[q] = float(src[q])
    return c


def icfunc_loop_collision(nx: int, ny: int, nz: int, dx: float, dy: float, dz: float) -> dict:
    """ic_func.cpp:61-72: pair 1 (x-directed) at y = +-2, z = -+0.25 L_z and pair
    2 (z-directed) at x = +-0.25 L_x, y = -+1, every string moving at 0.6 with
    the directions of the reference's constants."""
    a, b = 0.6 * 0.4, 0.6 * math.sqrt(1 - 0.4 ** 2)
    return dict(pos1s=[2.0, -0.25 * (nz - 1) * dz], pos1a=[-2.0, 0.25 * (nz - 1) * dz],
                pos2s=[0.25 * (nx - 1) * dx, -1.0], pos2a=[-0.25 * (nx - 1) * dx, 1.0],
                v1s=[0.0, -b, -a], v1a=[0.0, b, a], v2s=[a, b, 0.0], v2a=[-a, -b, 0.0])


def default_loop_collision(nx: int, ny: int, nz: int, dx: float, dy: float, dz: float) -> dict:
    """initialConditions.cpp:72-84: pair 1 at y = +-0.15 L_y, z = -+0.25 L_z moving
    along y at -+0.75; pair 2 at x = +-0.25 L_x at rest."""
    return dict(pos1s=[0.15 * (ny - 1) * dy, -0.25 * (nz - 1) * dz], pos1a=[-0.15 * (ny - 1) * dy, 0.25 * (nz - 1) * dz],
                pos2s=[0.25 * (nx - 1) * dx, 0.0], pos2a=[-0.25 * (nx - 1) * dx, 0.0],
                v1s=[0.0, -0.75, 0.0], v1a=[0.0, 0.75, 0.0], v2s=[0.0, 0.0, 0.0], v2a=[0.0, 0.0, 0.0])
