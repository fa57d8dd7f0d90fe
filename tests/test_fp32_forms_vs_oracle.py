"""The FP32 forms against the FP64 oracle: one job run alone (lat_advance),
inside a batch (lat_batch_*), and through the serving loop (lat_server_*).

The job is one unit of the reference's loop body (mpi_evolution.cpp:381-501,
with the energy and Gauss diagnostics of evolution.cpp:322-427; Moore:
moore_mpi_evolution.cpp:432-550): Abelian-Higgs 48^3 or Moore 40^3 (charges
1 and 2), dx = 0.5, dt = 0.1, PRS friction, 200 steps, energy/Gauss every 20
steps.  Its initial state is the FP32 device IC of the job's seed (Philox
phases, stored in float), so the oracle starts from exactly the same values,
read back as doubles.  Stated FP32 tolerances against the oracle:

  * fields, whole state: ||d||_2 / ||ref||_2 <= 1e-4 (and per field <= 1e-3);
  * energy at every diagnostic step: relative 1e-5;
  * summed Gauss deviation |G| at every diagnostic step: relative 1e-4;
  * served job (no fields come back): its diagnostics as above, and the
    winding total of the final level within 1 % of the oracle's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NSTEPS, DIAG = 200, 20
TOL_FIELD_L2, TOL_FIELD_COMP_L2, TOL_E, TOL_G, TOL_WIND = 1e-4, 1e-3, 1e-5, 1e-4, 0.01


def _job(model):
    from axions_gb300.params import ENERGY_EVOLUTION, F32, MODEL_MOORE, make_params
    if model == 0:
        p = make_params(0, n=48, d=0.5, dt=0.1, lam=1.5, eta=1.0, g=0.9, damped_nt=0, alpha=3.0, scaling=1.0,
                        tau0=1.0, energy_form=ENERGY_EVOLUTION, precision=F32)
    else:
        p = make_params(MODEL_MOORE, n=40, d=0.5, dt=0.1, lam=2.0, lambda2=2.0, lambda12=0.0, eta=1.0, eta2=1.0,
                        q1=1.0, q2=2.0, g=1.0, damped_nt=0, alpha=3.0, scaling=1.0, tau0=1.0,
                        energy_form=ENERGY_EVOLUTION, precision=F32)
    return p, 300 + model


@pytest.fixture(scope="module", params=[0, 1], ids=["ah", "moore"])
def oracle_run(request, oracle_mod):
    from axions_gb300 import lattice
    model = request.param
    p, seed = _job(model)
    with lattice.Lattice(p) as lat:
        lat.random_phase_ic_device(seed, independent=model == 1)
        st = lat.get_slots()                 # the FP32 IC as doubles
    q = p.copy()
    q.precision = 0
    diags = oracle_mod.evolve(q, st, 0, NSTEPS, diag_every=DIAG)
    wind = oracle_mod.winding(q, st, NSTEPS, 0)[1]
    return model, p, seed, st, diags, wind


def _check_diags(got, ref):
    assert [g[0] for g in got] == [r[0] for r in ref] == list(range(0, NSTEPS, DIAG))
    e = max(abs(g[1] - r[1]) / abs(r[1]) for g, r in zip(got, ref))
    gs = max(abs(g[2] - r[2]) / abs(r[2]) for g, r in zip(got, ref) if r[2] != 0)
    assert e <= TOL_E, e
    assert gs <= TOL_G, gs
    return e, gs


def _check_fields(got, ref):
    l2 = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert l2 <= TOL_FIELD_L2, l2
    a, b = got.reshape(got.shape[0], -1), ref.reshape(ref.shape[0], -1)
    for c in range(b.shape[0]):
        r = np.linalg.norm(a[c] - b[c]) / np.linalg.norm(b[c])
        assert r <= TOL_FIELD_COMP_L2, (c, r)
    return l2


def test_fp32_job_alone_against_oracle(oracle_run):
    from axions_gb300 import lattice
    model, p, seed, st, ref, _ = oracle_run
    with lattice.Lattice(p) as lat:
        lat.random_phase_ic_device(seed, independent=model == 1)
        got = lat.advance(NSTEPS, DIAG)
        slots = lat.get_slots()
    e, g = _check_diags(got, ref)
    l2 = _check_fields(slots, st)
    print(f"fp32 alone model={model}: field l2 {l2:.2e} energy {e:.2e} gauss {g:.2e}")


def test_fp32_job_in_a_batch_against_oracle(oracle_run):
    from axions_gb300 import lattice
    from axions_gb300.params import ENERGY_EVOLUTION, F32, make_params
    model, p, seed, st, ref, _ = oracle_run
    lat = lattice.Lattice(p)
    lat.random_phase_ic_device(seed, independent=model == 1)
    other = lattice.Lattice(make_params(0, nx=36, ny=28, nz=40, d=0.5, dt=0.1, lam=3.0, g=1.3, alpha=0.0,
                                        damped_nt=0, energy_form=ENERGY_EVOLUTION, precision=F32))
    other.random_phase_ic_device(5)
    with lattice.Batch(4) as b:
        b.add(lat, diag_every=DIAG, stop_step=NSTEPS)
        b.add(other, diag_every=10, stop_step=130)
        while b.advance(25) > 0:
            pass
        got = b.take_diags(lat)
    slots = lat.get_slots()
    lat.close()
    other.close()
    e, g = _check_diags(got, ref)
    l2 = _check_fields(slots, st)
    print(f"fp32 batch model={model}: field l2 {l2:.2e} energy {e:.2e} gauss {g:.2e}")


def test_fp32_job_served_against_oracle(oracle_run):
    from axions_gb300 import lattice
    model, p, seed, st, ref, wind = oracle_run
    with lattice.Server(8 << 30, tick_steps=25) as srv:
        other = srv.submit(_job(1 - model)[0], seed=9, nsteps=150, diag_every=30, independent=True)
        jid = srv.submit(p, seed=seed, nsteps=NSTEPS, diag_every=DIAG, independent=model == 1)
        r = srv.wait(jid)
        got = srv.diags(jid)
        assert srv.wait(other).status == 2
    assert r.status == 2
    e, g = _check_diags(got, ref)
    assert abs(r.winding_abs - wind) <= TOL_WIND * wind, (r.winding_abs, wind)
    print(f"fp32 served model={model}: energy {e:.2e} gauss {g:.2e} winding {r.winding_abs} vs {wind}")
