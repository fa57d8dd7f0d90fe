"""Straight-string profile by successive over-relaxation (no GPU):
bin/singleSemiAnalytic against singleSemiAnalytic.cpp itself, run on one
thread (golden fixtures made by running it; its OpenMP sweep updates in place,
so only the single-thread order is reproducible).  The bar is bit-exact: the
drop-in performs the same double operations and libm calls in the same order.
"""
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden

BIN = ROOT / "axions_gb300" / "bin" / "singleSemiAnalytic"


def _run(tmp_path, **args):
    cmd = [str(BIN), f"out_dir={tmp_path}"] + [f"{k}={v}" for k, v in args.items()]
    return subprocess.run(cmd, capture_output=True, timeout=300)


def _profile(tmp_path):
    t = np.array([float(x) for x in (tmp_path / "Data" / "SOR_Fields.txt").read_text().split()])
    return t.reshape(-1, 2).T


@pytest.mark.parametrize("name", ["ref_sor_global", "ref_sor_gauge"])
def test_sor_profile_equals_reference(tmp_path, name):
    z = load_golden(name)
    r = _run(tmp_path, nx=int(z["nx"]), h=float(z["h"]), g=float(z["g"]), tol=float(z["tol"]), digits=17)
    assert r.returncode == 0, r.stderr.decode()
    assert b"Number of iterations:" in r.stdout
    got = _profile(tmp_path)
    assert np.array_equal(got, z["profile"])
    # the physics it encodes: f(0) = 0 rising to eta (as 1 - O(1/r^2) for a
    # global string), A(0) = 0 rising to n/g for a gauged string
    assert got[0, 0] == 0 and abs(got[0, -1] - 1) < 2e-3
    if float(z["g"]) != 0:
        assert got[1, 0] == 0 and abs(got[1, -1] - 1) < 1e-2


def test_sor_restart_from_its_own_table_converges_at_once(tmp_path):
    """ic_type = 1 reads Data/SOR_Fields.txt as the starting point: a converged
    table at full precision is already within tolerance, so one sweep runs."""
    z = load_golden("ref_sor_global")
    args = dict(nx=int(z["nx"]), h=float(z["h"]), g=float(z["g"]), tol=float(z["tol"]), digits=17)
    assert _run(tmp_path, **args).returncode == 0
    r = _run(tmp_path, ic_type=1, **args)
    assert r.returncode == 0, r.stderr.decode()
    assert b"Number of iterations: 1\n" in r.stdout


def test_sor_rejects_a_too_short_grid(tmp_path):
    assert _run(tmp_path, nx=2).returncode != 0
