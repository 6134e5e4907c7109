"""The payoff fixed-point split of the path kernels, against exact rationals.

Every path's payoff enters the price sums as q = round(pay * 2^40) and
q2 = round(pay^2 * 2^24), ties to even, cut into 25-bit limbs (the oracle's
hexo_oracle.cpp folds the same integers).  The FP32 form squares the float
payoff exactly; the FP64 form rounds pay^2 to double first, as the reference's
double arithmetic does.  Python's Fraction and round() (ties to even) give the
exact expected integers.
"""
from fractions import Fraction

import numpy as np
import pytest

from hestonexotics_gb300 import engine as E

pytestmark = pytest.mark.gpu

M25 = (1 << 25) - 1
BAD = 0xFFFFFFFF


def expected(pay: float, f32: bool):
    v = float(np.float32(pay)) if f32 else float(pay)
    if not (v >= 0.0 and v < 8388608.0):      # NaN, inf, negative, >= 2^23 (-0 is valid)
        return [BAD] * 6
    x = Fraction(v)
    q = round(x * 2 ** 40)
    sq = x * x if f32 else Fraction(v * v)    # v * v: IEEE double product
    q2 = round(sq * 2 ** 24)
    return [q & M25, (q >> 25) & M25, q >> 50, q2 & M25, (q2 >> 25) & M25, q2 >> 50]


def payoff_values(seed: int = 11):
    rng = np.random.default_rng(seed)
    vals = [0.0, -0.0, 1e-45, 1e-40, 2.0 ** -126, 2.0 ** -17, 2.0 ** -16, 1024.0, 2048.0, 8192.0,
            float(np.nextafter(np.float32(8388608.0), np.float32(0.0))), 8388608.0, 1e7,
            float("nan"), float("inf"), -float("inf"), -1.0, -1e-30]
    for e in range(-149, 23):                  # every float exponent, both mantissa ends
        for m in (1.0, 1.5, 2.0 - 2.0 ** -23):
            vals.append(m * 2.0 ** e)
    for t in (2.0 ** -17, 1024.0, 2048.0, 8192.0):
        f = np.float32(t)
        vals += [float(np.nextafter(f, np.float32(0.0))), float(np.nextafter(f, np.float32(1e30)))]
    # ties of pay 2^40: odd multiples of 2^-41
    vals += list((2.0 * rng.integers(0, 1 << 22, 2000) + 1.0) * 2.0 ** -41)
    # log-uniform over the whole range, and typical payoffs of a 100-spot book
    vals += list(2.0 ** rng.uniform(-40.0, 23.0, 20000))
    vals += list(rng.uniform(0.0, 150.0, 20000))
    return np.array(vals, dtype=np.float64)


@pytest.fixture(scope="module")
def eng():
    return E.Engine(0)


@pytest.mark.parametrize("precision", [E.FP32, E.FP64])
def test_payoff_limbs_exact(eng, precision):
    pay = payoff_values()
    if precision == E.FP64:                    # doubles that are not floats as well
        rng = np.random.default_rng(12)
        pay = np.concatenate([pay, rng.uniform(0.0, 200.0, 20000), 2.0 ** rng.uniform(-60.0, 23.0, 20000)])
    got = eng.payoff_limbs(pay, precision)
    f32 = precision == E.FP32
    bad = [(float(p), list(g), exp) for p, g in zip(pay, got) if list(g) != (exp := expected(float(p), f32))]
    assert not bad, bad[:5]
