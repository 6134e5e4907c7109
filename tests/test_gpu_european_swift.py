"""European Monte Carlo prices against the SWIFT restatement.

The SWIFT restatement (oracle/swift.cpp) is pinned to the reference's golden
prices and gradients.  The engine's European calls (QE paths, daily grid)
must lie within 3 standard errors of it, in both forms; this checks the
scheme, drift, discounting and the terminal interpolation together.
"""
import numpy as np
import pytest

from hestonexotics_gb300 import engine as E

pytestmark = pytest.mark.gpu

SETS = [
    # v0, theta, rho, kappa, sigma, r
    (0.04, 0.04, -0.7, 1.5, 0.5, 0.02),
    (0.09, 0.09, 0.04, 1.0, 1.0, 0.02),   # the reference unit tests' parameter set
    (0.02, 0.06, -0.3, 3.0, 0.3, 0.0),
]


@pytest.mark.parametrize("precision", [E.FP64, E.FP32])
@pytest.mark.parametrize("k", range(len(SETS)))
def test_european_within_3se_of_swift(engine, oracle, precision, k):
    v0, th, rho, kap, sig, r = SETS[k]
    S0 = 100.0
    T = np.repeat([0.25, 1.0], 3)
    K = np.tile([90.0, 100.0, 110.0], 2)
    opts = E.Options(K, T, E.EUROPEAN)
    cfg = E.Config(n_paths=1 << 20, step_mode=E.STEP_GRID, steps_per_year=252.0, seed=7, precision=precision)
    params = E.Params(v0, th, rho, kap, sig, r)
    p, se = engine.price(params, S0, opts, cfg)
    want = np.concatenate([oracle.swift_price([v0, th, rho, kap, sig], t, r, S0, K[T == t],
                                              oracle.swift_params([v0, th, rho, kap, sig], t, r, S0, 90.0, 110.0,
                                                                  trunc_precision=1e-10))
                           for t in (0.25, 1.0)])
    z = (p - want) / se
    assert np.all(np.abs(z) < 3.0), z
