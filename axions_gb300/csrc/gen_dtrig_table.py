"""Writes dtrig_table.inc, the constants of the FP64 sine/cosine in dtrig.cuh.

* the table (sin(j*pi/256), cos(j*pi/256)), j = 0..511, each rounded to the
  nearest double from a 60-digit evaluation (exact zeros and ones at the
  multiples of pi/2);
* pi/256 split in three parts for the Cody-Waite reduction: the first two
  carry 30 significant bits each (so k*P1 and k*P2 are exact for |k| < 2^23,
  i.e. |x| < 2^23 pi/256 > 2^16), the third is the nearest double to the rest;
* 256/pi rounded to the nearest double;
* the polynomials for |r| <= R = pi/512 (with a margin for the rounding of k):
      sin r = r + r^3 (s3 + s5 r^2),   cos r - 1 = r^2 (c2 + c4 r^2),
  where s3 + s5 u and c2 + c4 u interpolate (sin r - r)/r^3 and
  (cos r - 1)/r^2 as functions of u = r^2 at the two Chebyshev nodes of
  [0, R^2] (near-minimax linear fits).  Their largest errors over the
  interval are printed, relative to r for the sine and absolute for cos r - 1.

Run: python gen_dtrig_table.py (needs mpmath).
"""
from pathlib import Path

import mpmath as mp

mp.mp.dps = 60
NT = 512                     # table entries over one period
STEP = 2 * mp.pi / NT        # pi/256


def hexd(v) -> str:
    return float(v).hex()


def split(x, bits):
    e = int(mp.floor(mp.log(abs(x), 2)))
    scale = mp.mpf(2) ** (bits - 1 - e)
    return mp.nint(x * scale) / scale


def fit(f, umax):
    """Linear interpolation of f(u) at the Chebyshev nodes of [0, umax]."""
    n0 = umax / 2 * (1 - mp.cos(mp.pi / 4))
    n1 = umax / 2 * (1 + mp.cos(mp.pi / 4))
    b = (f(n1) - f(n0)) / (n1 - n0)
    a = f(n0) - b * n0
    return a, b


def main() -> None:
    R = STEP / 2 * (1 + mp.mpf(2) ** -20)
    fs = lambda u: (mp.sin(mp.sqrt(u)) - mp.sqrt(u)) / mp.sqrt(u) ** 3
    fc = lambda u: (mp.cos(mp.sqrt(u)) - 1) / u
    s3, s5 = fit(fs, R * R)
    c2, c4 = fit(fc, R * R)
    s3, s5, c2, c4 = (mp.mpf(float(v)) for v in (s3, s5, c2, c4))
    es = max(abs((r + r ** 3 * (s3 + s5 * r * r)) - mp.sin(r)) / r for r in mp.linspace(R / 1000, R, 400))
    ec = max(abs(r * r * (c2 + c4 * r * r) - (mp.cos(r) - 1)) for r in mp.linspace(0, R, 400))
    print(f"sin r relative error <= {mp.nstr(es, 3)}, cos r - 1 absolute error <= {mp.nstr(ec, 3)}")
    p1 = split(STEP, 30)
    p2 = split(STEP - p1, 30)
    p3 = STEP - p1 - p2
    assert float(p1) == p1 and float(p2) == p2
    lines = ["// Generated by gen_dtrig_table.py: constants of the FP64 sine/cosine (dtrig.cuh).",
             f"constexpr double kDtrigInvStep = {hexd(1 / STEP)};  // 256/pi",
             f"constexpr double kDtrigStepA = {hexd(p1)};  // pi/256, first 30 bits",
             f"constexpr double kDtrigStepB = {hexd(p2)};  // next 30 bits",
             f"constexpr double kDtrigStepC = {hexd(p3)};  // the rest",
             f"constexpr double kDtrigS3 = {hexd(s3)};",
             f"constexpr double kDtrigS5 = {hexd(s5)};",
             f"constexpr double kDtrigC2 = {hexd(c2)};",
             f"constexpr double kDtrigC4 = {hexd(c4)};",
             f"constexpr int kDtrigEntries = {NT};",
             f"// {{sin(j*pi/256), cos(j*pi/256)}}, j = 0..{NT - 1}",
             f"static __device__ const double2 kDtrigTable[{NT}] = {{"]
    for j in range(NT):
        a = j * STEP
        s, c = mp.sin(a), mp.cos(a)
        # exact zeros at the multiples of pi/2 (mpmath leaves ~1e-60 there)
        if j % (NT // 2) == 0:
            s = mp.mpf(0)
        if j % (NT // 2) == NT // 4:
            c = mp.mpf(0)
        lines.append(f"    {{{hexd(s)}, {hexd(c)}}},")
    lines.append("};")
    out = Path(__file__).resolve().parent / "dtrig_table.inc"
    out.write_text("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
