"""Initial-condition pipeline on the host (no GPU): bin/initialConditions
against initialConditions.cpp itself (golden fixture made by running it), and
the field-table reader/writer the drop-in programs use (text and binary)."""
import subprocess

import numpy as np

from conftest import ROOT, load_golden

BIN = ROOT / "axions_gb300" / "bin"


def _run(tmp_path, args):
    (tmp_path / "Data").mkdir(exist_ok=True)
    cmd = [str(BIN / "initialConditions"), f"out_dir={tmp_path}"] + [f"{k}={v}" for k, v in args.items()]
    return subprocess.run(cmd, capture_output=True, timeout=300)


def _table(path, cols):
    return np.array([float(t) for t in path.read_text().split()]).reshape(-1, cols)


def test_random_ic_equals_reference(tmp_path):
    """normal_distribution over default_random_engine, as initialConditions.cpp:670-708."""
    z = load_golden("ref_initial_conditions")
    args = {"nx": int(z["nx"]), "ny": int(z["ny"]), "nz": int(z["nz"]), "seed": int(z["seed"]),
            "mean": float(z["mean"]), "stdev": float(z["stdev"]), "g": float(z["g"]), "digits": 17}
    r = _run(tmp_path, args)
    assert r.returncode == 0, r.stderr.decode()
    got = _table(tmp_path / "Data" / "ic.txt", 5).T
    assert np.array_equal(got, z["ic"])


def test_default_text_format_is_ostream_precision_6(tmp_path):
    z = load_golden("ref_initial_conditions")
    args = {"nx": int(z["nx"]), "ny": int(z["ny"]), "nz": int(z["nz"]), "seed": int(z["seed"]),
            "mean": float(z["mean"]), "stdev": float(z["stdev"]), "g": float(z["g"])}
    assert _run(tmp_path, args).returncode == 0
    want = "".join(" ".join("%.6g" % v for v in row) + "\n" for row in z["ic"].T)
    assert (tmp_path / "Data" / "ic.txt").read_text() == want


def test_convert_round_trip_and_messy_text(tmp_path):
    rng = np.random.default_rng(5)
    n = 4 * 5 * 6
    vals = rng.standard_normal((n, 5)) * 10.0 ** rng.integers(-12, 12, (n, 5))
    vals[0, 0] = -0.0
    lines = []
    for i, row in enumerate(vals):
        toks = [repr(float(v)) for v in row]
        if i % 3 == 0:
            toks = ["+" + t if not t.startswith("-") else t for t in toks]
        sep = "\t " if i % 5 == 0 else " "
        lines.append(("  " if i % 7 == 0 else "") + sep.join(toks) + ("\r\n" if i % 2 else "\n"))
        if i % 11 == 0:
            lines.append("   \n")
    (tmp_path / "Data").mkdir()
    (tmp_path / "Data" / "a.txt").write_text("".join(lines))
    dims = {"nx": 4, "ny": 5, "nz": 6, "ic_type": "convert"}
    assert _run(tmp_path, dict(dims, ic_in="a.txt", ic_file="a.bin")).returncode == 0
    raw = (tmp_path / "Data" / "a.bin").read_bytes()
    assert raw[:8] == b"AXIONSB1"
    assert np.array_equal(np.frombuffer(raw[24:], dtype="<f8").reshape(n, 5), vals)
    r = _run(tmp_path, dict(dims, ic_in="a.bin", ic_file="b.txt", digits=17))
    assert r.returncode == 0, r.stderr.decode()
    back = _table(tmp_path / "Data" / "b.txt", 5)
    assert np.array_equal(back, vals) and np.signbit(back[0, 0])


def test_large_table_parses_across_threads(tmp_path):
    """300k rows: the file is cut into many per-thread runs of whole lines."""
    rng = np.random.default_rng(6)
    nx, ny, nz = 100, 60, 50
    vals = rng.uniform(-1, 1, (nx * ny * nz, 5))
    (tmp_path / "Data").mkdir()
    with open(tmp_path / "Data" / "big.txt", "w") as f:
        np.savetxt(f, vals, fmt="%.17g")
    r = _run(tmp_path, {"nx": nx, "ny": ny, "nz": nz, "ic_type": "convert", "ic_in": "big.txt", "ic_file": "big.bin"})
    assert r.returncode == 0, r.stderr.decode()
    got = np.frombuffer((tmp_path / "Data" / "big.bin").read_bytes()[24:], dtype="<f8").reshape(-1, 5)
    assert np.array_equal(got, vals)


def test_bad_tables_are_rejected(tmp_path):
    (tmp_path / "Data").mkdir()
    dims = {"nx": 2, "ny": 2, "nz": 1, "ic_type": "convert", "ic_file": "o.bin"}
    good = "1 2 3 4 5\n" * 4
    cases = {
        "short.txt": ("1 2 3 4 5\n" * 3, b"expected 4 lines"),
        "cols.txt": (good.replace("1 2 3 4 5\n", "1 2 3 4\n", 1), b"expected 5 values"),
        "extra.txt": (good.replace("1 2 3 4 5\n", "1 2 3 4 5 6\n", 1), b"more than 5"),
        "token.txt": (good.replace("3", "x", 1), b"bad or non-finite"),
        "nan.txt": (good.replace("3", "nan", 1), b"bad or non-finite"),
    }
    for name, (text, msg) in cases.items():
        (tmp_path / "Data" / name).write_text(text)
        r = _run(tmp_path, dict(dims, ic_in=name))
        assert r.returncode == 2 and msg in r.stderr, (name, r.stderr)
    (tmp_path / "Data" / "ok.txt").write_text(good)
    assert _run(tmp_path, dict(dims, ic_in="ok.txt")).returncode == 0
    r = _run(tmp_path, dict(dims, nx=3, ic_in="o.bin", ic_file="p.txt"))
    assert r.returncode == 2 and b"expected" in r.stderr
