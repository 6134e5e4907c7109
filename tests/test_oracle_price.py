"""The oracle port, pinned against the reference's own pricing code (CPU only).

tests/golden/ref_price.json holds the untouched HSimulation::price<> run on
one OpenMP thread (the reference's stream partition: one RNG(2^20, 1) shared
by all paths, the trailing step included); tests/golden/ref_paths.json holds
per-path payoffs through the reference's HQEAnderson/contract classes with
one RNG(16, 42 + k) per path.  The reference build uses -ffast-math and FMA
contraction, so agreement is to a few 1e-15 relative, not bit for bit.
"""
import numpy as np
import pytest

from conftest import golden, unhex

REL = 1e-12


def test_reference_partition_reproduces_untouched_price(oracle):
    for case in golden("ref_price.json"):
        T = np.repeat(case["T"], [len(s) for s in case["strikes"]])
        K = np.array([k for s in case["strikes"] for k in s])
        params7 = case["params5"] + [0.0, 0.0]
        got, n = oracle.price_reference_partition(params7, case["S"], K, T, case["kind"], case["steps"],
                                                  case["n_sims"], n_threads=1)
        want = unhex(case["prices"])
        assert n == case["n_sims"]
        np.testing.assert_allclose(got, want, rtol=REL, atol=0)


def test_per_path_port_matches_reference_classes(oracle):
    for case in golden("ref_paths.json"):
        T = np.repeat(case["T"], [len(s) for s in case["strikes"]])
        K = np.array([k for s in case["strikes"] for k in s])
        params7 = case["params5"] + [0.0, 0.0]
        n = case["n_paths"]
        asian, euro = oracle.path_finals(params7, case["S"], K, T, case["kind"], n_default=n, steps=case["steps"],
                                         seed=case["seed"], path_lo=0, path_hi=n)
        finals = asian if case["kind"] == 0 else euro
        mat = np.searchsorted(np.unique(T), T)
        pay = np.maximum(0.0, finals[:, mat] - K[None, :])
        want = unhex(case["payoffs"]).reshape(n, len(K))
        np.testing.assert_allclose(pay, want, rtol=REL, atol=1e-12 * case["S"])


def test_per_path_prices_are_means_of_reference_payoffs(oracle):
    for case in golden("ref_paths.json"):
        T = np.repeat(case["T"], [len(s) for s in case["strikes"]])
        K = np.array([k for s in case["strikes"] for k in s])
        n = case["n_paths"]
        price, se, _ = oracle.price_paths(case["params5"] + [0.0, 0.0], case["S"], K, T, case["kind"],
                                          n_default=n, steps=case["steps"], seed=case["seed"])
        pay = unhex(case["payoffs"]).reshape(n, len(K))
        np.testing.assert_allclose(price, pay.mean(axis=0), rtol=1e-11, atol=1e-12)
        np.testing.assert_allclose(se, pay.std(axis=0, ddof=1) / np.sqrt(n), rtol=1e-6, atol=1e-12)


def test_zero_drift_is_bit_neutral(oracle):
    # r = q = 0 reproduces the reference's undiscounted, drift-free prices exactly
    K = np.array([90.0, 100.0, 110.0])
    p = [0.04, 0.04, -0.7, 1.5, 0.5, 0.0, 0.0]
    a, _, la = oracle.price_paths(p, 100.0, K, 1.0, 0, n_default=512, steps=50)
    b, _, lb = oracle.price_paths(p, 100.0, K, 1.0, 0, n_default=512, steps=50, threads=1)
    assert np.array_equal(la, lb) and np.array_equal(a, b)


def test_limb_sums_merge_exactly_across_shards(oracle):
    K = np.array([95.0, 100.0, 105.0])
    T = np.array([0.5, 0.5, 1.0])
    p = [0.05, 0.04, -0.5, 2.0, 0.6, 0.03, 0.01]
    kw = dict(n_default=3000, steps=40)
    _, _, full = oracle.price_paths(p, 100.0, K, T, [0, 1, 0], **kw)
    _, _, a = oracle.price_paths(p, 100.0, K, T, [0, 1, 0], path_lo=0, path_hi=1234, **kw)
    _, _, b = oracle.price_paths(p, 100.0, K, T, [0, 1, 0], path_lo=1234, path_hi=3000, **kw)
    assert np.array_equal(full, a + b)


def test_ragged_path_counts(oracle):
    # option o is priced on paths k < n_paths[o]; paths beyond every option's count are not simulated
    K = np.array([100.0, 100.0, 100.0])
    T = np.array([0.25, 0.5, 1.0])
    p = [0.04, 0.04, -0.7, 1.5, 0.5, 0.0, 0.0]
    npaths = np.array([500, 2000, 1000], dtype=np.uint64)
    price, _, limbs = oracle.price_paths(p, 100.0, K, T, 0, npaths, steps=30)
    for o in range(3):
        alone, _, l1 = oracle.price_paths(p, 100.0, K[o:o + 1], T[o:o + 1], 0, npaths[o:o + 1], steps=30)
        # the same paths, the same stream per path: identical sums whenever the
        # schedule up to T_o is identical (one maturity per option here only
        # for the first option; the others share earlier steps)
        if o == 0:
            assert np.array_equal(l1[0], limbs[0])
    assert np.all(price > 0)


def test_branch_counts_walk_the_reference_step_count(oracle):
    # T = 1 at 252 steps: the time sum in double stays below 1 after 252
    # steps, so each path takes 253 (HSimulation.tpp:35-36); the quadratic
    # share drops when the Feller condition is violated (more mass near 0)
    base = [0.04, 0.04, -0.7, 1.5, 0.5, 0.0, 0.0]
    feller = [0.04, 0.04, -0.9, 0.5, 1.0, 0.0, 0.0]
    q, n = oracle.branch_counts(base, 100.0, [100.0], [1.0], [0], n_default=512, steps=252, seed=42)
    qf, nf = oracle.branch_counts(feller, 100.0, [100.0], [1.0], [0], n_default=512, steps=252, seed=42)
    assert n == nf == 512 * 253
    assert 0.5 < q / n < 1.0 and 0.0 < qf / nf < q / n
    # a path range splits the counts exactly
    q1, n1 = oracle.branch_counts(base, 100.0, [100.0], [1.0], [0], n_default=512, steps=252, seed=42, path_hi=200)
    q2, n2 = oracle.branch_counts(base, 100.0, [100.0], [1.0], [0], n_default=512, steps=252, seed=42, path_lo=200)
    assert (q1 + q2, n1 + n2) == (q, n)


def test_geometric_control_variate_agrees_with_plain_estimator(oracle):
    # the control variate's estimate is the plain one plus a zero-mean
    # correction: within a few plain standard errors, with a much smaller
    # standard error on the Asian options; Europeans untouched
    from hestonexotics_gb300 import workloads as W
    rq, cfg = W.single_chain(n_paths=1 << 14)
    o = rq.options
    args = (rq.params.as_array(), rq.S0, o.strike, o.T, o.payoff.astype(np.uint8), o.n_paths)
    kw = dict(n_default=cfg.n_paths, step_mode=cfg.step_mode, steps=cfg.steps, steps_per_year=cfg.steps_per_year,
              seed=rq.seed)
    p, se, _ = oracle.price_paths(*args, **kw)
    pc, sec = oracle.price_paths_cv(*args, **kw)
    asian = o.payoff == 0
    np.testing.assert_array_equal(pc[~asian], p[~asian])
    np.testing.assert_array_equal(sec[~asian], se[~asian])
    liquid = asian & (p > 0.05)          # enough paths in the money for the regression
    z = np.abs(pc - p)[liquid] / se[liquid]
    assert z.max() < 4.0, z.max()
    assert np.median(se[liquid] / sec[liquid]) > 5.0
    eg = oracle.geo_calls(*args[:5], step_mode=cfg.step_mode, steps=cfg.steps, steps_per_year=cfg.steps_per_year)
    assert np.all(eg[~asian] == 0.0) and np.all(eg[asian] >= -1e-9) and np.all(eg[asian] < rq.S0)
