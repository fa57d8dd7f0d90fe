"""Device-side random-phase IC (Philox-4x32-10) and the tiled-step tuner."""
import numpy as np
import pytest


# Known-answer vectors of Philox-4x32-10 from the Random123 distribution
# (counter, key -> output); they also match Triton's tl.randint4x.
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expect", PHILOX_KAT)
def test_philox_known_answers(ctr, key, expect):
    from axions_gb300 import lattice
    assert tuple(lattice.philox4x32_10(ctr, key)) == expect


def _u01(a, b):
    return ((a >> 5) * 67108864.0 + (b >> 6)) / 9007199254740992.0


@pytest.mark.gpu
@pytest.mark.parametrize("precision,model", [(0, 0), (1, 0), (1, 1)])
def test_device_ic_matches_host_philox(precision, model):
    from axions_gb300 import lattice
    from axions_gb300.params import make_params
    p = make_params(model, nx=20, ny=18, nz=16, precision=precision, eta=1.3, eta2=0.7)
    seed = (7 << 32) | 99
    with lattice.Lattice(p) as lat:
        lat.random_phase_ic_device(seed, independent=True)
        now, past = lat.get_state()
        assert lat.time_step == 0
    assert np.array_equal(now, past)
    tol = 1e-15 if precision == 0 else 2e-7
    for s in (0, 1, 5, 4000, p.N - 1):
        out = lattice.philox4x32_10((s, 0, 0, 0), (seed & 0xFFFFFFFF, seed >> 32))
        ph = 2 * np.pi * _u01(out[0], out[1])
        np.testing.assert_allclose(now[0:2, s], [1.3 * np.cos(ph), 1.3 * np.sin(ph)], atol=tol * 2)
        if model == 1:
            ph2 = 2 * np.pi * _u01(out[2], out[3])
            np.testing.assert_allclose(now[2:4, s], [0.7 * np.cos(ph2), 0.7 * np.sin(ph2)], atol=tol * 2)
    theta = now[-3:]
    assert not theta.any()
    ph = np.arctan2(now[1], now[0])
    assert abs(np.mean(np.cos(ph))) < 0.05 and abs(np.mean(np.sin(ph))) < 0.05


@pytest.mark.gpu
def test_autotune_changes_nothing_but_speed(tmp_path):
    """The tuner picks a chunk from timings on a scratch lattice; results of
    the tuned handle equal those of any other chunk (the chunk only decides
    which CTA computes which plane), and the choice round-trips through the
    cache file."""
    from axions_gb300 import lattice
    from axions_gb300.params import F32, make_params
    p = make_params(0, nx=64, ny=48, nz=40, d=0.5, dt=0.1, lam=2.0, g=1.0, precision=F32)
    ref = None
    for chunk in (4, 16, 128):
        with lattice.Lattice(p) as lat:
            lat.random_phase_ic_device(3)
            lat.set_chunk(chunk)
            lat.advance(6)
            st = lat.get_slots()
        if ref is None:
            ref = st
        assert np.array_equal(st, ref)
    with lattice.Lattice(p) as lat:
        lat.random_phase_ic_device(3)
        before = lat.get_slots()
        t = lat.autotune(2)
        assert t.candidates >= 3 and t.chunk in (4, 8, 16, 32, 64, 128) and t.ms_per_step > 0
        assert np.array_equal(lat.get_slots(), before)
        assert lat.tuning.chunk == t.chunk
    path = tmp_path / "tune.json"
    lattice.tune_cache_save(path)
    assert lattice.tune_cache_load(path) >= 1
    with lattice.Lattice(p) as lat2:   # new handles of the shape start tuned
        assert lat2.tuning.chunk == t.chunk
