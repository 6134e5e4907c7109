"""SWIFT European pricer of the library (hexo_swift_*).

CPU: the dynamic wavelet parameters (host-only) equal the oracle's
restatement of SwiftParameters (src/SWIFT.cpp:21-35) exactly.
GPU: prices and gradients against the reference's known answers
(src/UnitTest.cpp pricing_test / gradient_test, sum of absolute differences
below 1e-9 as there), and against the oracle's restatement on other
parameter sets to 1e-10 absolute (S = 100: relative to the strike scale).
"""
import numpy as np
import pytest

from conftest import golden, unhex
from hestonexotics_gb300 import engine as E


def _golden():
    g = golden("swift_golden.json")
    p = E.Params(*g["params5"], r=g["r"])
    chains = [(T, np.array(K)) for T, K in zip(g["expiries"], g["strikes"])]
    return g, p, chains


def test_dynamic_params_equal_oracle(oracle):
    g, p, chains = _golden()
    for prec in (1e-7, 1e-10):
        for T, K in chains:
            got = E.swift_params_dynamic(p, T, g["S"], K.min(), K.max(), prec)
            want = oracle.swift_params(g["params5"], T, g["r"], g["S"], K.min(), K.max(), trunc_precision=prec)
            assert [got["m"], got["exp2_m"], got["k1"], got["k2"], got["J"]] == [int(want[0]), int(want[1]),
                                                                               int(want[5]), int(want[6]), int(want[7])]
            np.testing.assert_allclose([got["sqrt_exp2_m"], got["lower"], got["upper"]], want[[2, 3, 4]], rtol=1e-13)


@pytest.mark.gpu
def test_gpu_golden_prices_and_gradients(engine):
    g, p, chains = _golden()
    out = engine.swift(p, g["S"], chains, grad=True, swift_params=g["swift_params"])
    price = np.concatenate([o[0] for o in out])
    grad = np.concatenate([o[1] for o in out])
    assert np.sum(np.abs(price - unhex(g["prices"]))) < g["price_tolerance_sum_abs"]
    want = unhex(g["grad"]).reshape(40, 5)
    imap = g["grad_index_map"]
    diff = sum(abs(want[i, imap[j]] - grad[i, j]) for i in range(40) for j in range(5))
    assert diff < g["grad_tolerance_sum_abs"]


@pytest.mark.gpu
def test_gpu_matches_oracle_dynamic(engine, oracle):
    rng = np.random.default_rng(4)
    reqs, wants = [], []
    for _ in range(6):
        p5 = [rng.uniform(0.01, 0.09), rng.uniform(0.01, 0.09), rng.uniform(-0.9, -0.1), rng.uniform(0.5, 5.0),
              rng.uniform(0.1, 1.0)]
        r = rng.uniform(0.0, 0.05)
        chains = [(T, np.geomspace(60.0, 160.0, 25)) for T in (1 / 12, 0.5, 2.0)]
        reqs.append((E.Params(*p5, r=r), 100.0, chains))
        wants.append([oracle.swift_price(p5, T, r, 100.0, K, oracle.swift_params(p5, T, r, 100.0, K.min(), K.max()),
                                         grad=True) for T, K in chains])
    outs = engine.swift_batch(reqs, grad=True)
    for out, want in zip(outs, wants):
        for (gp, gg), (wp, wg) in zip(out, want):
            np.testing.assert_allclose(gp, wp, rtol=0, atol=1e-10)
            np.testing.assert_allclose(gg, wg, rtol=0, atol=1e-8)


@pytest.mark.gpu
def test_calibration_callbacks_match_oracle(engine, oracle):
    g, p, chains = _golden()
    cal = engine.calibration(g["S"], g["r"], chains)
    x = cal.prices(g["params5"])
    jac = cal.jacobian(g["params5"])
    want_x, want_j = [], []
    for T, K in chains:
        sp = oracle.swift_params(g["params5"], T, g["r"], g["S"], K.min(), K.max())
        wp, wg = oracle.swift_price(g["params5"], T, g["r"], g["S"], K, sp, grad=True)
        want_x.append(wp)
        want_j.append(wg)
    np.testing.assert_allclose(x, np.concatenate(want_x), rtol=0, atol=1e-12)
    np.testing.assert_allclose(jac, np.concatenate(want_j), rtol=0, atol=1e-10)
    cal.close()


def _levenberg_marquardt(f, jac, p0, x_obs, iters=100):
    """A plain Levenberg-Marquardt loop (levmar's damping: mu starts at
    1e-3 max diag(J'J), halved... on success, doubled on failure)."""
    p = np.array(p0, dtype=float)
    r = x_obs - f(p)
    J = jac(p)
    A = J.T @ J
    mu = 1e-3 * A.diagonal().max()
    for _ in range(iters):
        gvec = J.T @ r
        if np.abs(gvec).max() < 1e-10:
            break
        dp = np.linalg.solve(A + mu * np.eye(5), gvec)
        if np.linalg.norm(dp) < 1e-10 * (np.linalg.norm(p) + 1e-10):
            break
        pn = p + dp
        ok = pn[0] > 0 and pn[1] > 0 and abs(pn[2]) < 1 and pn[3] > 0 and pn[4] > 0
        rn = x_obs - f(pn) if ok else None
        if ok and np.all(np.isfinite(rn)) and rn @ rn < r @ r:
            p, r = pn, rn
            J = jac(p)
            A = J.T @ J
            mu *= 1.0 / 3.0
        else:
            mu *= 2.0
    return p


@pytest.mark.gpu
def test_calibration_recovers_parameters(engine):
    # the reference's levmar_test (src/UnitTest.cpp:480-509): prices at p,
    # start from p + 0.2 in every component, recover p within 1e-2 (sum)
    g, p, chains = _golden()
    cal = engine.calibration(g["S"], g["r"], chains)
    p_true = np.array(g["params5"])
    x_obs = cal.prices(p_true)
    got = _levenberg_marquardt(cal.prices, cal.jacobian, p_true + 0.2, x_obs)
    assert np.abs(got - p_true).sum() < 1e-2, got
    cal.close()


@pytest.mark.gpu
def test_gpu_fft_golden_prices_and_gradients(engine):
    # the same known answers with both transforms evaluated by the FFT
    g, p, chains = _golden()
    out = engine.swift(p, g["S"], chains, grad=True, swift_params=g["swift_params"], method=2)
    price = np.concatenate([o[0] for o in out])
    grad = np.concatenate([o[1] for o in out])
    assert np.sum(np.abs(price - unhex(g["prices"]))) < g["price_tolerance_sum_abs"]
    want = unhex(g["grad"]).reshape(40, 5)
    imap = g["grad_index_map"]
    assert sum(abs(want[i, imap[j]] - grad[i, j]) for i in range(40) for j in range(5)) < g["grad_tolerance_sum_abs"]


@pytest.mark.gpu
@pytest.mark.parametrize("J", [1024, 8192, 65536])
def test_gpu_fft_equals_direct_sums(engine, J):
    # the dynamic wavelet parameters of random sets with J frequencies: the
    # FFT (O(J log J)) and the direct sums (O(J (k2 - k1))) give the same
    # prices and gradients to rounding
    rng = np.random.default_rng(J)
    for _ in range(3):
        p = E.Params(rng.uniform(0.01, 0.09), rng.uniform(0.01, 0.09), rng.uniform(-0.9, -0.1),
                     rng.uniform(0.5, 5.0), rng.uniform(0.1, 1.0), r=rng.uniform(0.0, 0.05))
        chains = [(T, np.geomspace(60.0, 160.0, 20)) for T in (0.25, 1.0, 3.0)]
        sps = []
        for T, K in chains:
            sp = E.swift_params_dynamic(p, T, 100.0, K.min(), K.max(), 1e-10)
            assert sp["k2"] - sp["k1"] + 1 <= 4 * J
            sp["J"] = J
            sps.append(sp)
        direct = engine.swift(p, 100.0, chains, grad=True, swift_params=sps, method=1)
        fft = engine.swift(p, 100.0, chains, grad=True, swift_params=sps, method=2)
        for (pd, gd), (pf, gf) in zip(direct, fft):
            np.testing.assert_allclose(pf, pd, rtol=1e-9, atol=1e-10 * 100.0)
            np.testing.assert_allclose(gf, gd, rtol=1e-8, atol=1e-9 * 100.0)
