"""The constants of the FP64 step's table-driven sine and cosine
(axions_gb300/csrc/dtrig_table.inc), checked on the host.

* every table entry is within two ulps of libm's sin/cos of j*pi/256 taken
  at well-conditioned arguments (the entries are correctly rounded; the
  reference's argument is rounded to a double), with exact zeros and ones at
  the multiples of pi/2;
* the Cody-Waite split of pi/256: the first two parts carry at most 30
  significant bits (k*P1 and k*P2 exact for |k| < 2^23) and the three sum to
  pi/256 within 1e-30;
* the polynomial coefficients are close to the Taylor ones (they are fitted
  on |r| <= pi/512);
* with mpmath present, the file is exactly what gen_dtrig_table.py writes.
"""
import math
import re
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

CSRC = Path(__file__).resolve().parents[1] / "axions_gb300" / "csrc"
INC = CSRC / "dtrig_table.inc"


def parse():
    text = INC.read_text()
    consts = {m.group(1): float.fromhex(m.group(2))
              for m in re.finditer(r"constexpr double (kDtrig\w+) = (-?0x[0-9a-fp.+-]+);", text)}
    n = int(re.search(r"constexpr int kDtrigEntries = (\d+);", text).group(1))
    pairs = re.findall(r"\{(-?0x[0-9a-fp.+-]+), (-?0x[0-9a-fp.+-]+)\},", text)
    table = np.array([[float.fromhex(a), float.fromhex(b)] for a, b in pairs])
    return consts, n, table


def sig_bits(x: float) -> int:
    m, _ = math.frexp(abs(x))
    f = Fraction(m)
    return f.denominator.bit_length() - 1


def reference_table(n=512):
    """sin and cos of j*pi/256 from libm at well-conditioned arguments only:
    the first octant directly, the rest of the quadrant by cos/sin of the
    complement, the other quadrants by exact symmetry."""
    q0 = []
    for m in range(n // 4):
        if m <= n // 8:
            x = m * math.pi / (n // 2)
            q0.append((math.sin(x), math.cos(x)))
        else:
            x = (n // 4 - m) * math.pi / (n // 2)
            q0.append((math.cos(x), math.sin(x)))
    out = []
    for j in range(n):
        s, c = q0[j % (n // 4)]
        out.append([(s, c), (c, -s), (-s, -c), (-c, s)][j // (n // 4)])
    return np.array(out)


def test_table_entries_within_two_ulps_of_libm():
    """The table holds the correctly rounded values; the libm reference (at an
    argument rounded to a double) is within about 1.5 ulps of them."""
    consts, n, table = parse()
    assert n == 512 and table.shape == (512, 2)
    ref = reference_table(n)
    zero = ref == 0.0
    assert np.array_equal(table == 0.0, zero)
    err = np.abs(table - ref)[~zero] / np.spacing(np.abs(ref[~zero]))
    assert err.max() <= 2.0, err.max()
    assert table[0, 1] == 1.0 and table[128, 0] == 1.0 and table[256, 1] == -1.0 and table[384, 0] == -1.0


def test_cody_waite_split_and_coefficients():
    c, _, _ = parse()
    a, b, cc = c["kDtrigStepA"], c["kDtrigStepB"], c["kDtrigStepC"]
    assert sig_bits(a) <= 30 and sig_bits(b) <= 30
    # pi/256 to 36 digits
    pi256 = Fraction(314159265358979323846264338327950288, 10 ** 35) / 256
    assert abs(Fraction(a) + Fraction(b) + Fraction(cc) - pi256) < Fraction(1, 10 ** 30)
    assert c["kDtrigInvStep"] == 256 / math.pi
    assert abs(c["kDtrigS3"] + 1 / 6) < 1e-12 and abs(c["kDtrigS5"] - 1 / 120) < 1e-8
    assert abs(c["kDtrigC2"] + 0.5) < 1e-12 and abs(c["kDtrigC4"] - 1 / 24) < 1e-7


def test_table_file_is_the_generators_output(tmp_path):
    pytest.importorskip("mpmath")
    import importlib.util
    import shutil
    gen = tmp_path / "gen_dtrig_table.py"
    shutil.copy(CSRC / "gen_dtrig_table.py", gen)
    spec = importlib.util.spec_from_file_location("gen_dtrig_table", gen)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.main()
    assert (tmp_path / "dtrig_table.inc").read_text() == INC.read_text()
