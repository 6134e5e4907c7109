"""GPU pricing against the oracle and the reference golden vectors.

Tolerances (written where used):
  * FP64 form vs the oracle / reference payoffs: 1e-10 relative on prices
    (absolute 1e-12 * S0 for prices that are essentially zero), the bar the
    plain form is held to; per-path final values to 1e-12 relative.
  * FP32 form vs the FP64 oracle on the same streams: 1e-4 relative for
    prices above 1e-3 * S0, and inside one standard error everywhere.
  * Launch shapes, batching, graphs and shards: bit-identical.
"""
import numpy as np
import pytest

from conftest import golden, unhex
from hestonexotics_gb300 import engine as E
from hestonexotics_gb300 import workloads as W
from hestonexotics_gb300._lib import HexoError

pytestmark = pytest.mark.gpu

FP64_REL = 1e-10


def oracle_price(oracle, req, cfg, **kw):
    o = req.options
    return oracle.price_paths(req.params.as_array(), req.S0, o.strike, o.T, o.payoff.astype(np.uint8), o.n_paths,
                              n_default=cfg.n_paths, step_mode=cfg.step_mode, steps=cfg.steps,
                              steps_per_year=cfg.steps_per_year, seed=req.seed, stream=req.stream, **kw)


def assert_fp64_close(got, want, S0):
    np.testing.assert_allclose(got, want, rtol=FP64_REL, atol=1e-12 * S0)


def test_plain_asian_fp64(engine, oracle):
    req, cfg = W.plain_asian()
    p, se = engine.price(req.params, req.S0, req.options, cfg)
    op, ose, _ = oracle_price(oracle, req, cfg)
    assert_fp64_close(p, op, req.S0)
    np.testing.assert_allclose(se, ose, rtol=1e-8)
    assert 2.0 < p[0] < 8.0 and 0 < se[0] < 0.1


def test_golden_reference_payoffs(engine):
    # per-path payoffs from the reference's own classes, one RNG(16, 42 + k) per path
    for case in golden("ref_paths.json"):
        T = np.repeat(case["T"], [len(s) for s in case["strikes"]])
        K = np.array([k for s in case["strikes"] for k in s])
        n = case["n_paths"]
        opts = E.Options(K, T, case["kind"])
        cfg = E.Config(n_paths=n, steps=case["steps"], seed=case["seed"])
        params = E.Params(*case["params5"])
        p, se = engine.price(params, case["S"], opts, cfg)
        pay = unhex(case["payoffs"]).reshape(n, len(K))
        np.testing.assert_allclose(p, pay.mean(axis=0), rtol=FP64_REL, atol=1e-12 * case["S"])
        asian, euro = engine.path_finals(params, case["S"], opts, cfg, 0, n)
        finals = asian if case["kind"] == 0 else euro
        mat = np.searchsorted(np.unique(T), T)
        np.testing.assert_allclose(np.maximum(0.0, finals[:, mat] - K), pay, rtol=1e-12, atol=1e-12 * case["S"])


def test_path_finals_fp64(engine, oracle):
    req, cfg = W.single_chain(n_paths=700)
    cfg.steps = 40
    cfg.step_mode = E.STEP_REFERENCE
    o = req.options
    ga, ge = engine.path_finals(req.params, req.S0, o, cfg, 0, 700)
    oa, oe = oracle.path_finals(req.params.as_array(), req.S0, o.strike, o.T, o.payoff.astype(np.uint8),
                                n_default=700, steps=40, seed=req.seed, path_lo=0, path_hi=700)
    np.testing.assert_allclose(ga, oa, rtol=1e-12)
    np.testing.assert_allclose(ge, oe, rtol=1e-12)


@pytest.mark.parametrize("mode", [E.STEP_REFERENCE, E.STEP_GRID])
def test_chain_fp64(engine, oracle, mode):
    req, cfg = W.single_chain(n_paths=1 << 13)
    cfg.step_mode = mode
    cfg.steps = 50
    p, se = engine.price(req.params, req.S0, req.options, cfg)
    op, ose, _ = oracle_price(oracle, req, cfg)
    assert_fp64_close(p, op, req.S0)
    np.testing.assert_allclose(se, ose, rtol=1e-7, atol=1e-12)


def test_feller_violating_fp64(engine, oracle):
    req, cfg = W.feller_violating(n_paths=1 << 12)
    p, se = engine.price(req.params, req.S0, req.options, cfg)
    op, _, _ = oracle_price(oracle, req, cfg)
    assert_fp64_close(p, op, req.S0)


def fp32_check(p32, se32, p64, S0):
    big = p64 > 1e-3 * S0
    rel = np.abs(p32 - p64) / np.where(big, p64, 1.0)
    assert rel[big].max() <= 1e-4, rel[big].max()
    assert np.all(np.abs(p32 - p64) <= np.maximum(se32, 1e-9 * S0))


@pytest.mark.parametrize("maker", [W.single_chain, W.feller_violating])
def test_fp32_vs_fp64_oracle(engine, oracle, maker):
    req, cfg = maker(n_paths=1 << 14)
    p64, _, _ = oracle_price(oracle, req, cfg)
    cfg.precision = E.FP32
    p32, se32 = engine.price(req.params, req.S0, req.options, cfg)
    fp32_check(p32, se32, p64, req.S0)


def test_fp32_vs_fp64_every_set_of_the_uneven_batch(engine):
    # all 64 parameter sets (high vol-of-vol ones included), 1/32 of the paths:
    # the FP32 form against the FP64 form on the same streams
    reqs, cfg32 = W.uneven_batch(seed=2, precision=E.FP32, path_scale=1 / 32)
    cfg64 = E.Config(**{**cfg32.__dict__, "precision": E.FP64})
    o32 = engine.price_batch(reqs, cfg32)
    o64 = engine.price_batch(reqs, cfg64)
    for rq, (p32, se32), (p64, _) in zip(reqs, o32, o64):
        fp32_check(p32, se32, p64, rq.S0)


def test_launch_shapes_bit_identical(engine):
    req, cfg = W.single_chain(n_paths=5000)
    cfg.steps_per_year = 52.0
    ref = None
    for prec in (E.FP64, E.FP32):
        cfg.precision = prec
        ref = None
        for block, ppt, unroll in [(256, 1, 1), (128, 1, 2), (512, 1, 4), (128, 2, 1), (256, 2, 2), (128, 4, 1)]:
            cfg.block, cfg.paths_per_thread, cfg.unroll = block, ppt, unroll
            p, se = engine.price(req.params, req.S0, req.options, cfg)
            if ref is None:
                ref = (p, se)
            assert np.array_equal(p, ref[0]) and np.array_equal(se, ref[1]), (prec, block, ppt, unroll)


def test_batch_equals_alone(engine):
    reqs, cfg = W.uneven_batch(n_sets=5, path_scale=1 / 256, precision=E.FP32)
    mixed = engine.price_batch(reqs, cfg)
    for rq, (p, se) in zip(reqs, mixed):
        alone = engine.price_batch([rq], cfg)[0]
        assert np.array_equal(p, alone[0]) and np.array_equal(se, alone[1])


def test_prepared_graph_relaunch(engine):
    reqs, cfg = W.uneven_batch(n_sets=3, path_scale=1 / 512, precision=E.FP32)
    b = engine.prepare_batch(reqs, cfg)
    b.launch()
    first = [(p.copy(), s.copy()) for p, s in b.collect()]
    b.launch()
    b.launch()
    second = b.collect()
    for (p1, s1), (p2, s2) in zip(first, second):
        assert np.array_equal(p1, p2) and np.array_equal(s1, s2)
    direct = engine.price_batch(reqs, cfg)
    for (p1, _), (p2, _) in zip(first, direct):
        assert np.array_equal(p1, p2)
    info = b.info()
    assert info["nominal_path_steps"] > 0 and info["n_sets"] == 3
    b.close()


def test_uneven_batch_fp64_vs_oracle(engine, oracle):
    # every one of the benchmark batch's 64 sets (their own parameters, chains,
    # schedules and stream numbers) at 1/1024 of their paths, against the oracle
    reqs, cfg = W.uneven_batch(seed=2, path_scale=1 / 1024, precision=E.FP64)
    out = engine.price_batch(reqs, cfg)
    for rq, (p, se) in zip(reqs, out):
        op, ose, _ = oracle_price(oracle, rq, cfg)
        assert_fp64_close(p, op, rq.S0)
        np.testing.assert_allclose(se, ose, rtol=1e-7, atol=1e-12 * rq.S0)


@pytest.mark.parametrize("maker", [W.single_chain, W.feller_violating])
def test_precision_sweep_fp32_vs_fp64(engine, maker):
    # the chain (8 maturities x 50 strikes x Asian/European) and the
    # Feller-violating set at 2^16, 2^20 and 2^24 paths: the FP32 form within
    # 1e-4 relative of the FP64 form on the same streams (prices above
    # 1e-3 S0) and inside one FP32 standard error everywhere
    for n in (1 << 16, 1 << 20, 1 << 24):
        req, cfg64 = maker(n_paths=n, precision=E.FP64)
        p64, _ = engine.price(req.params, req.S0, req.options, cfg64)
        p32, se32 = engine.price(req.params, req.S0, req.options, E.Config(**{**cfg64.__dict__, "precision": E.FP32}))
        fp32_check(p32, se32, p64, req.S0)


def test_shards_merge_bit_identical(engine):
    req, cfg = W.single_chain(n_paths=6000)
    cfg.steps_per_year = 100.0
    full = engine.partial(req.params, req.S0, req.options, cfg, 0, 6000)
    a = engine.partial(req.params, req.S0, req.options, cfg, 0, 2500)
    b = engine.partial(req.params, req.S0, req.options, cfg, 2500, 6000)
    assert np.array_equal(full, a + b)
    p_merge, se_merge = E.finalize_limbs(req.params, req.S0, req.options, cfg, a + b)
    p, se = engine.price(req.params, req.S0, req.options, cfg)
    assert np.array_equal(p, p_merge) and np.array_equal(se, se_merge)


@pytest.mark.parametrize("n_shards", [2, 3])
def test_batch_shards_merge_bit_identical(engine, n_shards):
    # a whole batch split into n_shards launches (range r of every request's
    # paths in launch r), merged by adding limbs: the prices of one launch
    from hestonexotics_gb300 import shard as S
    reqs, cfg = W.uneven_batch(n_sets=5, path_scale=1 / 512, precision=E.FP32)
    want = engine.price_batch(reqs, cfg)
    parts = [engine.batch_partial(reqs, cfg, r, n_shards) for r in range(n_shards)]
    got = S.finalize_batch(reqs, cfg, sum(parts))
    for (pw, sw), (pg, sg) in zip(want, got):
        assert np.array_equal(pw, pg) and np.array_equal(sw, sg)
    # the prepared (graph) form of a shard gives the same limbs, launch after launch
    b = engine.prepare_batch_partial(reqs, cfg, 1, n_shards)
    for _ in range(2):
        b.launch()
        assert np.array_equal(b.collect_limbs(), parts[1])
    b.close()


def test_limbs_match_oracle_exactly_where_payoffs_do(engine, oracle):
    # FP64 payoffs agree with the oracle to ~1e-16; their fixed-point sums then agree to a few units
    req, cfg = W.plain_asian(n_paths=3000)
    g = engine.partial(req.params, req.S0, req.options, cfg, 0, 3000)
    _, _, o = oracle_price(oracle, req, cfg)
    v = lambda l: int(l[0]) + (int(l[1]) << 25) + (int(l[2]) << 50)
    assert abs(v(g[0]) - v(o[0])) <= 3000


def test_ragged_paths_and_many_options(engine, oracle):
    rng = np.random.default_rng(5)
    n = 150
    T = np.repeat([0.1, 0.35, 0.35001, 1.2], [40, 70, 20, 20])
    K = rng.uniform(70, 140, n)
    kind = rng.integers(0, 2, n)
    npaths = rng.choice([1, 31, 33, 257, 1000, 4099], n).astype(np.uint64)
    opts = E.Options(K, T, kind, npaths)
    params = E.Params(0.05, 0.03, -0.5, 2.5, 0.7, r=0.01, q=0.02)
    cfg = E.Config(n_paths=1000, step_mode=E.STEP_GRID, seed=99)
    p, se = engine.price(params, 100.0, opts, cfg)
    req = E.Request(params, 100.0, opts, seed=99)
    op, ose, _ = oracle_price(oracle, req, cfg)
    assert_fp64_close(p, op, 100.0)
    one = npaths == 1
    assert np.all(se[one] == 0.0)


def test_single_path_and_tiny_maturity(engine, oracle):
    params = E.Params(0.04, 0.04, -0.7, 1.5, 0.5)
    opts = E.Options(np.array([0.0, 100.0, 1e6]), np.array([1e-4, 1e-4, 1e-4]), np.array([0, 1, 1]))
    cfg = E.Config(n_paths=1, steps=1)
    p, se = engine.price(params, 100.0, opts, cfg)
    req = E.Request(params, 100.0, opts, seed=cfg.seed)
    op, _, _ = oracle_price(oracle, req, cfg)
    assert_fp64_close(p, op, 100.0)
    assert p[2] == 0.0


def test_invalid_request_errors(engine):
    params = E.Params(0.04, 0.04, -0.7, 1.5, 0.5)
    with pytest.raises(HexoError) as ei:
        engine.price(params, 100.0, E.Options(np.array([100.0]), 0.0, 0), E.Config())
    assert ei.value.status == 1
    with pytest.raises(HexoError):
        engine.price(params, 100.0, E.Options(np.array([100.0]), 1.0, 0), E.Config(block=100))


EDGE_SETS = [
    # v0, theta, rho, kappa, sigma, r: the ends of the admissible ranges
    (0.04, 0.04, -1.0, 1.5, 0.5, 0.02),     # rho = -1: the spot noise has no own part (K3 = 0)
    (0.04, 0.04, 1.0, 1.5, 0.5, 0.02),      # rho = +1
    (0.0, 0.04, -0.7, 1.5, 0.5, 0.02),      # v0 = 0
    (0.04, 0.04, -0.7, 1.5, 0.01, 0.02),    # sigma -> 0: always the quadratic branch
    (0.04, 0.04, -0.7, 1.5, 2.0, 0.02),     # sigma = 2: mostly the exponential branch
    (0.04, 0.04, -0.7, 20.0, 0.5, 0.0),     # fast mean reversion
    (0.04, 0.04, -0.7, 0.01, 0.5, 0.05),    # slow mean reversion
    (0.09, 1e-4, -0.5, 2.0, 0.3, 0.0),      # theta -> 0
]


@pytest.mark.parametrize("k", range(len(EDGE_SETS)))
def test_parameter_edges_fp64_vs_oracle_and_fp32(engine, oracle, k):
    v0, th, rho, kap, sig, r = EDGE_SETS[k]
    params = E.Params(v0, th, rho, kap, sig, r)
    S0 = 100.0
    T = np.repeat([1 / 52, 0.5, 2.0], 4)
    K = np.tile([50.0, 95.0, 105.0, 400.0], 3)   # deep in and far out of the money included
    kinds = np.tile([E.ASIAN, E.EUROPEAN], 6).astype(np.uint32)
    req = E.Request(params, S0, E.Options(K, T, kinds), seed=11)
    cfg = E.Config(n_paths=1 << 12, step_mode=E.STEP_GRID, steps_per_year=252.0, seed=11, precision=E.FP64)
    p64, _ = engine.price(params, S0, req.options, E.Config(**{**cfg.__dict__, "seed": 11}))
    op, _, _ = oracle_price(oracle, req, cfg)
    assert_fp64_close(p64, op, S0)
    p32, se32 = engine.price(params, S0, req.options, E.Config(**{**cfg.__dict__, "precision": E.FP32}))
    fp32_check(p32, se32, p64, S0)


def test_extreme_spot_levels(engine, oracle):
    for S0 in (2.0 ** -60, 1e-3, 1e4, 1e8, 2.0 ** 59):
        params = E.Params(0.04, 0.04, -0.7, 1.5, 0.5, 0.02)
        K = S0 * np.array([0.8, 1.0, 1.2])
        req = E.Request(params, S0, E.Options(K, 1.0, E.ASIAN), seed=3)
        cfg = E.Config(n_paths=1 << 12, steps=63, seed=3, precision=E.FP64)
        p64, _ = engine.price(params, S0, req.options, E.Config(**{**cfg.__dict__}))
        op, _, _ = oracle_price(oracle, req, cfg)
        assert_fp64_close(p64, op, S0)


def test_trim_frees_the_kept_memory_and_calls_still_agree(engine):
    req, cfg = W.single_chain(n_paths=2000)
    first = engine.price(req.params, req.S0, req.options, cfg)
    engine.trim()
    engine.trim()   # nothing kept: a no-op
    again = engine.price(req.params, req.S0, req.options, cfg)
    assert np.array_equal(first[0], again[0]) and np.array_equal(first[1], again[1])


def test_small_batches_spread_over_every_sm(engine):
    # 65,536 paths fill 256 CTAs of 256 threads; narrower CTAs spread them over
    # all 2 x SM slots (same results: the launch shape does not change them)
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    req, cfg = W.plain_asian(n_paths=65536)
    for prec in (E.FP64, E.FP32):
        cfg.precision = prec
        b = engine.prepare_batch([req], cfg)
        b.launch()
        (p, se), = b.collect()
        info = b.info()
        b.close()
        per = -(-65536 // (2 * sms))
        assert info["block"] == max(128, -(-per // 32) * 32) < 256
        want = engine.price(req.params, req.S0, req.options, E.Config(**{**cfg.__dict__, "block": 256}))
        assert np.array_equal(p, want[0]) and np.array_equal(se, want[1])


def test_continue_a_request_with_more_paths(engine):
    # a request priced on 4,000 paths is continued to 10,000 without
    # recomputing the first 4,000: the limbs of paths [4000, 10000) add to the
    # kept limbs, and the sum finalises to the prices of 10,000 paths at once
    req, cfg = W.single_chain(n_paths=4000)
    first = engine.partial(req.params, req.S0, req.options, cfg, 0, 4000)
    more = E.Config(**{**cfg.__dict__, "n_paths": 10000})
    rest = engine.partial(req.params, req.S0, req.options, more, 4000, 10000)
    p, se = E.finalize_limbs(req.params, req.S0, req.options, more, first + rest)
    want = engine.price(req.params, req.S0, req.options, more)
    assert np.array_equal(p, want[0]) and np.array_equal(se, want[1])
