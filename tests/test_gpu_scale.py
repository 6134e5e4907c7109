"""Prices and standard errors at every spot level.

The engine sums payoffs in units of 2^E, E the binary exponent of the spot,
so its standard error keeps its relative precision from S0 = 1e-3 to 1e8.
The check does not go through the fixed-point sums at all: the kernel's own
per-path final values (hexo_debug_path_finals, the same paths and streams)
give the payoffs, and a plain float64 mean and standard deviation of those
in numpy is the expected price and standard error.

Tolerances: the standard error to 1e-6 relative and the price to 1e-10
relative of the numpy figures (the FP64 form, and the FP32 form against its
own float payoffs); the FP64 price to 1e-10 relative of the oracle.  The reference computes no standard error
(HSimulation.tpp:40 keeps only the mean payoff); its price is the mean.
"""
import numpy as np
import pytest

from hestonexotics_gb300 import engine as E
from hestonexotics_gb300._lib import HexoError

pytestmark = pytest.mark.gpu

SPOTS = [1e-3, 1e-2, 1.0, 100.0, 1e6, 1e8]
N = 4096


def book(S0):
    K = S0 * np.array([0.8, 1.0, 1.3, 0.8, 1.0, 1.3])
    kinds = np.array([E.ASIAN] * 3 + [E.EUROPEAN] * 3, dtype=np.uint32)
    return E.Options(K, 1.0, kinds)


@pytest.mark.parametrize("S0", SPOTS)
@pytest.mark.parametrize("precision", [E.FP64, E.FP32])
def test_price_and_stderr_match_per_path_payoffs(engine, oracle, S0, precision):
    params = E.Params(0.04, 0.04, -0.7, 1.5, 0.5, r=0.02)
    opts = book(S0)
    cfg = E.Config(n_paths=N, steps=63, seed=3, stream=5, precision=precision)
    price, se = engine.price(params, S0, opts, cfg)
    asian, euro = engine.path_finals(params, S0, opts, cfg, 0, N)
    disc = np.exp(-params.r * 1.0)
    for i in range(len(opts)):
        f = (asian if opts.payoff[i] == E.ASIAN else euro)[:, 0]
        if precision == E.FP32:   # the kernel's float payoff: max(0, float(f) - float(K))
            pay = np.maximum(np.float32(0), f.astype(np.float32) - np.float32(opts.strike[i])).astype(np.float64)
        else:
            pay = np.maximum(0.0, f - opts.strike[i])
        want_p = disc * pay.mean()
        want_se = disc * pay.std(ddof=1) / np.sqrt(N)
        assert want_se > 0.0
        np.testing.assert_allclose(se[i], want_se, rtol=1e-6, err_msg=f"S0={S0} option {i}")
        np.testing.assert_allclose(price[i], want_p, rtol=1e-10, err_msg=f"S0={S0} option {i}")
    if precision == E.FP64:
        o = opts
        op, ose, _ = oracle.price_paths(params.as_array(), S0, o.strike, o.T, o.payoff.astype(np.uint8),
                                        n_default=N, steps=63, seed=3, stream=5)
        np.testing.assert_allclose(price, op, rtol=1e-10, atol=0)
        np.testing.assert_allclose(se, ose, rtol=1e-8)


def test_prices_scale_with_the_spot(engine):
    # the QE scheme is homogeneous in (S0, K): at spots that differ by a power
    # of two the paths differ by that exact factor up to the rounding of
    # log S0, so prices agree to ~1e-13 and standard errors likewise
    params = E.Params(0.04, 0.04, -0.7, 1.5, 0.5, r=0.02)
    cfg = E.Config(n_paths=N, steps=63, seed=3)
    base_p, base_se = engine.price(params, 100.0, book(100.0), cfg)
    for k in (-40, -7, 20, 52):
        S0 = 100.0 * 2.0 ** k
        p, se = engine.price(params, S0, book(S0), cfg)
        np.testing.assert_allclose(p / 2.0 ** k, base_p, rtol=1e-11)
        np.testing.assert_allclose(se / 2.0 ** k, base_se, rtol=1e-9)


def test_payoff_beyond_the_fixed_point_range(engine):
    # a payoff of 2^17 S0 or more is outside [0, 2^16 2^E): HEXO_ERR_NUMERIC
    params = E.Params(0.04, 0.04, -0.7, 1.5, 0.5)
    for S0 in (1e-3, 100.0, 1e8):
        opts = E.Options(np.array([-(2.0 ** 17) * S0]), 1.0, E.EUROPEAN)
        with pytest.raises(HexoError) as ei:
            engine.price(params, S0, opts, E.Config(n_paths=64, steps=10))
        assert ei.value.status == 6


def test_spot_outside_the_supported_range(engine):
    params = E.Params(0.04, 0.04, -0.7, 1.5, 0.5)
    for S0 in (2.0 ** -61, 2.0 ** 60, 0.0, -1.0):
        with pytest.raises(HexoError) as ei:
            engine.price(params, S0, E.Options(np.array([1.0]), 1.0, 0), E.Config(n_paths=64, steps=10))
        assert ei.value.status == 1
