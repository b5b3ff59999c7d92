"""The kernels' exp for psi = 1 - exp(-rho): the integer fixed-point
evaluation (lbmath::lb_exp) against the FP64 table routine it replaced
(lbmath::lb_exp_fp64, still used outside 2^-83 <= |x| <= 707) and, where
they differ, against the exact value rounded as the reference's 80-bit
evaluation rounds it (to 64 significant bits, then to 53)."""
import decimal
import math
from fractions import Fraction

import numpy as np

from oracle import oracle as orc


def _double_rounded(x: float) -> float:
    decimal.getcontext().prec = 90
    fr = Fraction(decimal.Decimal(x).exp())
    out = fr
    for bits in (64, 53):
        e = math.floor(math.log2(out))
        while Fraction(2) ** e > out:
            e -= 1
        while Fraction(2) ** (e + 1) <= out:
            e += 1
        v = out * Fraction(2) ** (bits - 1 - e)
        fl = v.numerator // v.denominator
        rem = v - fl
        if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and fl % 2 == 1):
            fl += 1
        out = Fraction(fl) / Fraction(2) ** (bits - 1 - e)
    return float(out)


def test_integer_exp_matches_fp64_exp_or_the_exact_double_rounding():
    rng = np.random.default_rng(21)
    x = np.concatenate([-3.0 * rng.random(3_000_000), rng.uniform(-707.0, 707.0, 300_000),
                        np.ldexp(rng.random(200_000) - 0.5, -rng.integers(0, 80, 200_000))])
    a = orc.exp(x, mode=1)
    b = orc.exp(x, mode=2)
    diff = np.flatnonzero(a.view(np.uint64) != b.view(np.uint64))
    assert len(diff) < 50, len(diff)  # ~1.4e-7 of the arguments
    for i in diff:
        assert a[i] == _double_rounded(float(x[i])), float(x[i]).hex()


def test_integer_exp_range_edges():
    # the integer range's ends and the FP64 routine beyond them agree with
    # the exact double rounding
    xs = [707.0, -707.0, np.nextafter(707.0, 0.0), 2.0 ** -83, -(2.0 ** -83), 2.0 ** -84,
          np.nextafter(707.0, 1e9), 1e-300, -1e-20, 3.5, -0.7, 0.0]
    got = orc.exp(np.array(xs), mode=1)
    for x, g in zip(xs, got):
        assert g == _double_rounded(float(x)), float(x).hex()
