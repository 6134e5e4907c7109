"""The payoff fixed-point split of the path kernels, against exact rationals.

A request's payoffs are summed in units of 2^E, E the binary exponent of its
spot (2^(E-1) <= S0 < 2^E): every path's payoff enters the sums as
q = round(y * 2^47) and q2 = round(y^2 * 2^43), y = pay * 2^-E, ties to even,
cut into 25-bit limbs (the oracle's hexo_oracle.cpp folds the same
integers).  The FP32 form squares the float payoff exactly; the FP64 form
rounds y^2 to double first, as the reference's double arithmetic does.
Python's Fraction and round() (ties to even) give the exact expected
integers, at spot levels from 2^-60 to just under 2^60.
"""
import math
from fractions import Fraction

import numpy as np
import pytest

from hestonexotics_gb300 import engine as E

pytestmark = pytest.mark.gpu

M25 = (1 << 25) - 1
BAD = 0xFFFFFFFF
SPOTS = [100.0, 1e-3, 1.0, 3.0e7, 2.0 ** -60, 2.0 ** 60 * (1 - 2.0 ** -53)]


def expected(pay: float, f32: bool, S0: float):
    E_ = math.frexp(S0)[1]
    v = float(np.float32(pay)) if f32 else float(pay)
    if not (v >= 0.0) or math.isinf(v):       # NaN, negative, infinite (-0 is valid)
        return [BAD] * 6
    y = Fraction(v) / Fraction(2) ** E_
    if y >= 2 ** 16:
        return [BAD] * 6
    q = round(y * 2 ** 47)
    if f32:
        sq = y * y
    else:                                      # y * y as an IEEE double product (y itself exact)
        yd = math.ldexp(v, -E_)
        sq = Fraction(yd * yd) if yd != 0.0 else Fraction(0)
    q2 = round(sq * 2 ** 43)
    return [q & M25, (q >> 25) & M25, q >> 50, q2 & M25, (q2 >> 25) & M25, q2 >> 50]


def payoff_values(S0: float, seed: int = 11):
    rng = np.random.default_rng(seed)
    E_ = math.frexp(S0)[1]
    top = 2.0 ** (16 + E_)                     # the first rejected payoff
    vals = [0.0, -0.0, 1e-45, 1e-40, 2.0 ** -126, top, top * (1 - 2.0 ** -24), top * (1 - 2.0 ** -53), top * 2,
            float("nan"), float("inf"), -float("inf"), -1.0, -1e-30]
    for e in range(-30, 17):                   # every exponent of y that the sums can see, both mantissa ends
        for m in (1.0, 1.5, 2.0 - 2.0 ** -23):
            vals.append(math.ldexp(m, e + E_))
    # ties of y 2^47: odd multiples of 2^-48 (in units of 2^E)
    vals += list(np.ldexp(2.0 * rng.integers(0, 1 << 22, 2000) + 1.0, E_ - 48))
    # log-uniform over the whole range, and typical payoffs of a book on this spot
    vals += list(np.ldexp(2.0 ** rng.uniform(-40.0, 16.0, 8000), E_))
    vals += list(rng.uniform(0.0, 1.5 * S0, 8000))
    return np.array([v for v in vals if math.isnan(v) or abs(v) < 1e300], dtype=np.float64)


@pytest.fixture(scope="module")
def eng():
    return E.Engine(0)


@pytest.mark.parametrize("S0", SPOTS)
@pytest.mark.parametrize("precision", [E.FP32, E.FP64])
def test_payoff_limbs_exact(eng, precision, S0):
    if precision == E.FP32 and not (2.0 ** -126 < S0 < 2.0 ** 127):
        pytest.skip("spot outside the float range")
    pay = payoff_values(S0)
    if precision == E.FP64:                    # doubles that are not floats as well
        rng = np.random.default_rng(12)
        E_ = math.frexp(S0)[1]
        pay = np.concatenate([pay, rng.uniform(0.0, 2.0 * S0, 8000), np.ldexp(2.0 ** rng.uniform(-60.0, 16.0, 8000), E_)])
    got = eng.payoff_limbs(pay, precision, S0)
    f32 = precision == E.FP32
    bad = [(float(p), list(g), exp) for p, g in zip(pay, got) if list(g) != (exp := expected(float(p), f32, S0))]
    assert not bad, bad[:5]
