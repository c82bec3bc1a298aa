"""The plain method's macro step divides the momentum sums by rho through one shared
correctly rounded reciprocal y = RN(1/rho) and Markstein's correction (csrc/lbm_exact.cu,
div_rcp): q = RN(x y), r = RN(x - rho q) (one fma), result RN(q + r y) (one fma).  Here the
claim that this is the correctly rounded quotient RN(x / rho) is checked exhaustively in
binary floating point with 5- to 9-bit significands (every pair of significands; the
binade does not matter for a normal quotient), in exact rational arithmetic, with every
operation rounded to nearest-even as the GPU rounds it.  The device code is compared with
CUDA's IEEE division by test_gpu_parity.py::test_integer_pipe_arithmetic_matches_fp64."""
from fractions import Fraction

import pytest


def rn(x, p):
    """x rounded to the nearest p-bit binary floating-point number, ties to even."""
    if x == 0:
        return Fraction(0)
    sign = -1 if x < 0 else 1
    x = abs(x)
    e = 0
    while x >= 2:
        x /= 2
        e += 1
    while x < 1:
        x *= 2
        e -= 1
    m = x * (1 << (p - 1))
    fl = m.numerator // m.denominator
    rem = m - fl
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and fl % 2 == 1):
        fl += 1
    return sign * Fraction(fl, 1 << (p - 1)) * Fraction(2) ** e


@pytest.mark.parametrize("p", [5, 6, 7, 8, 9])
def test_shared_reciprocal_division_is_correctly_rounded(p):
    n = 1 << (p - 1)
    bad = []
    for bs in range(n, 2 * n):
        b = Fraction(bs, n)
        y = rn(1 / b, p)
        for as_ in range(n, 2 * n):
            a = Fraction(as_, n)
            q = rn(a * y, p)
            r = rn(a - b * q, p)
            if rn(q + r * y, p) != rn(a / b, p):
                bad.append((a, b))
    assert not bad, bad[:5]
