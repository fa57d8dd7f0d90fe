"""The allocation-free stepping entry point, lat_ah_step_f64_noalloc.

It serves callers that cannot let a library allocate device memory (a host
application that owns every byte of device memory through its own pool or
budget, or a stepping loop that cannot pay for cudaMalloc's device-wide
synchronisation).  The test owns the fields (allocated here with torch, as
such a caller would from its own pool), calls the entry point through the C
ABI twice in a row, and checks each result against the handle-based
lat_step on the same inputs.  The two run the same launchers on the same
inputs, so the fields must be equal bit for bit.  Cases cover both update
forms (power-of-two spacing, which multiplies by exact reciprocals, and a
general spacing, which divides), periodic and fixed walls, and both FP64
precisions the entry point takes.

This file is named to be collected last, and it passes both on its own in a
fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _params(n_sides, d, bc, precision):
    from axions_gb300.params import ENERGY_EVOLUTION, make_params
    nx, ny, nz = n_sides
    return make_params(0, nx=nx, ny=ny, nz=nz, d=d, dt=0.1 * d / 0.5, lam=2.0, eta=1.0, g=1.0, damped_nt=6,
                       dampFac=0.5, alpha=3.0, energy_form=ENERGY_EVOLUTION, bc=bc, precision=precision)


@pytest.mark.parametrize("d,bc", [(0.5, 0), (0.3, 1)], ids=["pow2-periodic", "general-fixed"])
@pytest.mark.parametrize("precision", [0, 2], ids=["f64", "f64_fast"])
def test_noalloc_steps_match_handle_steps_on_two_calls(d, bc, precision):
    torch = pytest.importorskip("torch")
    from axions_gb300 import lattice

    L = lattice.load_library()
    p = _params((40, 36, 32), d, bc, precision)
    ic = lattice.random_phase_ic(p, 21)

    # caller-owned device fields in the reference slot layout [5][2][N]
    st0 = np.stack([ic, ic], axis=1)                     # both slots = IC at TimeStep 0
    dev = torch.from_numpy(st0.copy()).to("cuda")
    stream = torch.cuda.current_stream()

    with lattice.Lattice(p) as lat:
        lat.set_state(ic, ic, 0)
        n = 0
        for nsteps in (9, 7):                            # two calls in a row
            rc = L.lat_ah_step_f64_noalloc(ctypes.byref(p), ctypes.c_void_p(dev.data_ptr()), n, nsteps,
                                           ctypes.c_void_p(stream.cuda_stream))
            assert rc == 0, L.lat_last_error()
            torch.cuda.synchronize()
            lat.step(nsteps)
            n += nsteps
            got = dev.cpu().numpy()
            ref = lat.get_slots()
            assert lat.time_step == n
            assert np.array_equal(got, ref), "allocation-free step differs from lat_step"


def test_noalloc_rejects_lattices_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from axions_gb300 import lattice
    from axions_gb300.params import LAT_ERR_INVALID

    L = lattice.load_library()
    p = _params((65, 64, 64), 0.5, 0, 0)                  # one plane more than 64^3
    assert p.N > 262144
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = L.lat_ah_step_f64_noalloc(ctypes.byref(p), ctypes.c_void_p(dummy.data_ptr()), 0, 1, None)
    assert rc == LAT_ERR_INVALID
    assert b"LAT_NOALLOC_MAX_SITES" in L.lat_last_error()
