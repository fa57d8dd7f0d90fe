"""Serving loop (lat_server_*): admission by HBM footprint, continuous
batching, and results that do not depend on the other jobs."""
import time

import numpy as np
import pytest


def _job_params(model, n, lam, g, q=(1.0, 2.0)):
    from axions_gb300.params import ENERGY_EVOLUTION, F32, MODEL_MOORE, make_params
    if model == 0:
        return make_params(0, n=n, d=0.5, dt=0.1, lam=lam, eta=1.0, g=g, damped_nt=0, alpha=0.0,
                           energy_form=ENERGY_EVOLUTION, precision=F32)
    return make_params(MODEL_MOORE, n=n, d=0.5, dt=0.1, lam=lam, lambda2=lam, eta=1.0, eta2=1.0, q1=q[0], q2=q[1], g=g,
                       damped_nt=0, alpha=0.0, energy_form=ENERGY_EVOLUTION, precision=F32)


def test_footprint_rejects_bad_params():
    from axions_gb300 import lattice
    from axions_gb300.params import LAT_ERR_INVALID, make_params
    p = make_params(0, n=8)
    p.dt = -1.0
    assert lattice.footprint_bytes(p) == LAT_ERR_INVALID
    good = make_params(0, n=8, precision=1)
    assert lattice.footprint_bytes(good) >= 8 ** 3 * 4 * 11


@pytest.mark.gpu
@pytest.mark.parametrize("model,n,prec", [(0, 40, 1), (1, 36, 1), (0, 32, 0)])
def test_footprint_is_what_a_lattice_holds(model, n, prec):
    from axions_gb300 import lattice
    p = _job_params(model, n, 2.0, 1.0)
    p.precision = prec
    with lattice.Lattice(p) as lat:
        assert lat.device_bytes == lattice.footprint_bytes(p)


X = (0, 48, 1.5, 0.9)   # the job under test: AH 48^3


@pytest.mark.gpu
def test_served_job_same_alone_and_in_the_mix():
    from axions_gb300 import lattice
    px = _job_params(*X)
    with lattice.Server(8 << 30, tick_steps=10) as srv:
        jid = srv.submit(px, seed=77, nsteps=60, diag_every=10)
        alone = srv.wait(jid)
        d_alone = srv.diags(jid)
    assert alone.status == 2 and len(d_alone) == 6
    rng = np.random.default_rng(5)
    with lattice.Server(8 << 30, tick_steps=10) as srv:
        others = []
        for k in range(4):   # jobs already running when X arrives
            m = int(rng.integers(0, 2))
            others.append(srv.submit(_job_params(m, int(rng.choice([32, 40, 56])), 2.0, 1.0), seed=k, nsteps=80,
                                     diag_every=20, independent=True))
        time.sleep(0.05)
        jid = srv.submit(px, seed=77, nsteps=60, diag_every=10)
        for k in range(4):   # and jobs that arrive after it
            others.append(srv.submit(_job_params(0, 44, 3.0, 1.2), seed=100 + k, nsteps=30, diag_every=10))
        mix = srv.wait(jid)
        d_mix = srv.diags(jid)
        for o in others:
            assert srv.wait(o).status == 2
    for f in ("final_energy", "final_gauss", "winding_abs", "site_updates", "ndiag"):
        assert getattr(mix, f) == getattr(alone, f), f
    assert d_mix == d_alone


@pytest.mark.gpu
def test_admission_respects_the_hbm_budget():
    from axions_gb300 import lattice
    p = _job_params(0, 64, 2.0, 1.0)
    fp = lattice.footprint_bytes(p)
    budget = 2 * fp + fp // 2           # room for two 64^3 jobs at a time
    with lattice.Server(budget, tick_steps=5) as srv:
        ids = [srv.submit(_job_params(0, 64, 2.0 + 0.1 * k, 1.0), seed=k, nsteps=20) for k in range(6)]
        results = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert all(r.status == 2 for r in results)
    assert st.peak_bytes <= budget and st.done == 6
    starts = sorted(r.start_s for r in results)
    ends = sorted(r.end_s for r in results)
    assert starts[2] >= ends[0] - 1e-9   # the third job waited for the first to finish


@pytest.mark.gpu
def test_job_larger_than_the_budget_fails_cleanly():
    from axions_gb300 import lattice
    from axions_gb300.params import LAT_ERR_CAPACITY
    with lattice.Server(1 << 20, tick_steps=5) as srv:
        jid = srv.submit(_job_params(0, 64, 2.0, 1.0), seed=1, nsteps=5)
        r = srv.wait(jid, 60)
    assert r.status == LAT_ERR_CAPACITY
