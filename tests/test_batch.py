"""Batched stepping (lat_batch_*): many lattices in the same launches.

A lattice's result must not depend on its company: fields and recorded
diagnostics are compared bit for bit against the same lattice advanced alone
through its own handle (lat_advance), for a mix of models, sizes, couplings
and stop steps, over several calls with a lattice leaving and one joining.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lat(lattice, model, sides, seed, lam, g, q=(1.0, 2.0), bc=0):
    from axions_gb300.params import ENERGY_EVOLUTION, F32, MODEL_MOORE, make_params
    nx, ny, nz = sides
    if model == 0:
        p = make_params(0, nx=nx, ny=ny, nz=nz, d=0.5, dt=0.1, lam=lam, eta=1.0, g=g, damped_nt=4, dampFac=0.5,
                        alpha=3.0, energy_form=ENERGY_EVOLUTION, precision=F32, bc=bc)
    else:
        p = make_params(MODEL_MOORE, nx=nx, ny=ny, nz=nz, d=0.5, dt=0.1, lam=lam, lambda2=lam, lambda12=0.0, eta=1.0,
                        eta2=1.0, q1=q[0], q2=q[1], g=g, damped_nt=4, dampFac=0.5, alpha=3.0,
                        energy_form=ENERGY_EVOLUTION, precision=F32, bc=bc)
    lat = lattice.Lattice(p)
    ic = lattice.random_phase_ic(p, seed, independent=model == 1)
    lat.set_state(ic, ic, 0)
    return lat


SPECS = [  # model, sides, seed, lambda, g, stop, diag_every
    (0, (48, 48, 48), 1, 1.0, 0.7, 23, 5),
    (0, (40, 36, 44), 2, 3.0, 1.5, 17, 4),
    (1, (32, 40, 36), 3, 2.0, 1.0, 23, 6),
    (0, (24, 20, 33), 4, 0.6, 1.9, 9, 3),
]


def _run_batch(lattice, specs, ticks):
    lats = [_lat(lattice, m, s, sd, lam, g) for (m, s, sd, lam, g, _, _) in specs]
    with lattice.Batch(8) as b:
        for lat, spec in zip(lats, specs):
            b.add(lat, diag_every=spec[6], stop_step=spec[5])
        active = [b.advance(t) for t in ticks]
        out = [(lat.time_step, lat.get_slots(), b.take_diags(lat)) for lat in lats]
    for lat in lats:
        lat.close()
    return active, out


def test_batch_alone_and_in_the_mix_bitwise():
    """Each lattice in a mixed batch (two models, four sizes and couplings,
    different stop steps) gives bitwise the same fields and diagnostics as in a
    batch of its own."""
    from axions_gb300 import lattice
    active, mix = _run_batch(lattice, SPECS, [7, 7, 7, 7])
    assert active[0] == 4 and active[-1] == 0
    for spec, (n, st, d) in zip(SPECS, mix):
        _, [(n1, st1, d1)] = _run_batch(lattice, [spec], [7, 7, 7, 7])
        assert n == n1 == spec[5]
        assert np.array_equal(st, st1)
        assert d == d1


def test_batch_matches_the_single_lattice_path():
    """The batch runs the same tile code as lat_advance on a handle, in a
    different kernel; the two agree to FP32 rounding."""
    from axions_gb300 import lattice
    _, mix = _run_batch(lattice, SPECS, [7, 7, 7, 7])
    for spec, (n, st, d) in zip(SPECS, mix):
        (model, sides, seed, lam, g, stop, de) = spec
        lat = _lat(lattice, model, sides, seed, lam, g)
        dref = lat.advance(stop, diag_every=de)
        ref = lat.get_slots()
        lat.close()
        diff = np.abs(st - ref)
        assert diff.max() / np.abs(ref).max() < 1e-5 and np.linalg.norm(diff) / np.linalg.norm(ref) < 1e-6
        assert [x[0] for x in d] == [x[0] for x in dref]
        np.testing.assert_allclose([x[1] for x in d], [x[1] for x in dref], rtol=1e-6)
        np.testing.assert_allclose([x[2] for x in d], [x[2] for x in dref], rtol=1e-6)


def test_batch_join_and_leave_between_calls():
    from axions_gb300 import lattice
    a_ref = _lat(lattice, 0, (36, 32, 40), 11, 2.0, 1.0)
    a_ref.advance(20, diag_every=5)
    b_ref = _lat(lattice, 1, (32, 32, 32), 12, 2.0, 1.0, q=(2.0, 1.0))
    b_ref.advance(12, diag_every=4)
    a = _lat(lattice, 0, (36, 32, 40), 11, 2.0, 1.0)
    bm = _lat(lattice, 1, (32, 32, 32), 12, 2.0, 1.0, q=(2.0, 1.0))
    with lattice.Batch(4) as b:
        b.add(a, diag_every=5, stop_step=20)
        b.advance(8)                       # a alone
        b.add(bm, diag_every=4, stop_step=12)
        b.advance(8)                       # a and bm
        a.step(0)
        b.remove(a)                        # a leaves with 4 steps to go
        a.advance(4, diag_every=5)         # ... which it takes on its own handle
        b.advance(8)                       # bm finishes
        assert a.time_step == 20 and bm.time_step == 12
        for got, ref in ((a.get_slots(), a_ref.get_slots()), (bm.get_slots(), b_ref.get_slots())):
            diff = np.abs(got - ref)
            assert np.linalg.norm(diff) / np.linalg.norm(ref) < 1e-6
    for x in (a, bm, a_ref, b_ref):
        x.close()


def test_batch_rejects_fp64_handles():
    from axions_gb300 import lattice
    from axions_gb300.params import make_params
    lat = lattice.Lattice(make_params(0, n=16))
    with lattice.Batch(2) as b:
        with pytest.raises(lattice.LatticeError):
            b.add(lat)
    lat.close()


def test_batch_chunk_changes_only_the_diagnostic_sums():
    """The x-chunk of the work items decides the tiling only: the fields are
    bitwise the same for any chunk, the diagnostics agree to the rounding of
    their partial sums."""
    from axions_gb300 import lattice
    specs = SPECS[:2] + SPECS[3:]
    ref = None
    for chunk in (0, 4, 16, 128):
        lats = [_lat(lattice, m, s, sd, lam, g) for (m, s, sd, lam, g, _, _) in specs]
        with lattice.Batch(4) as b:
            b.set_chunk(chunk)
            for lat, spec in zip(lats, specs):
                b.add(lat, diag_every=spec[6], stop_step=spec[5])
            while b.advance(7) > 0:
                pass
            out = [(lat.get_slots(), b.take_diags(lat)) for lat in lats]
        for lat in lats:
            lat.close()
        if ref is None:
            ref = out
            continue
        for (st, d), (st0, d0) in zip(out, ref):
            assert np.array_equal(st, st0)
            assert [x[0] for x in d] == [x[0] for x in d0]
            np.testing.assert_allclose([x[1] for x in d], [x[1] for x in d0], rtol=1e-12)
            np.testing.assert_allclose([x[2] for x in d], [x[2] for x in d0], rtol=1e-12)
    with lattice.Batch(1) as b:
        with pytest.raises(lattice.LatticeError):
            b.set_chunk(-1)
