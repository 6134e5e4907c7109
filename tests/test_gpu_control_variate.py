"""The geometric-average control variate (hexo_mc_cfg.control_variate = 1).

Tolerances (written where used):
  * FP64 form vs the oracle's restatement on the same streams: 1e-8
    relative on prices, with 1e-9 * S0 absolute for the cancellation in
    Lewis's integral on deep out-of-the-money strikes; standard errors 1e-6.
  * Control variate vs the reference's estimator on the same paths: within
    4 plain standard errors, with a much smaller standard error.
  * FP32 form vs FP64 form: 1e-4 relative or one control-variate standard
    error, whichever is larger.
  * Europeans, batching and request order: bit-identical.
"""
import numpy as np
import pytest

from hestonexotics_gb300 import engine as E
from hestonexotics_gb300 import workloads as W
from hestonexotics_gb300._lib import HexoError

pytestmark = pytest.mark.gpu


def oracle_cv(oracle, req, cfg):
    o = req.options
    return oracle.price_paths_cv(req.params.as_array(), req.S0, o.strike, o.T, o.payoff.astype(np.uint8), o.n_paths,
                                 n_default=cfg.n_paths, step_mode=cfg.step_mode, steps=cfg.steps,
                                 steps_per_year=cfg.steps_per_year, seed=req.seed, stream=req.stream)


@pytest.mark.parametrize("maker", [W.single_chain, W.feller_violating, W.plain_asian])
def test_fp64_control_variate_equals_oracle(engine, oracle, maker):
    req, cfg = maker(n_paths=1 << 13)
    cfg.precision = E.FP64
    cfg.control_variate = 1
    p, se = engine.price(req.params, req.S0, req.options, cfg)
    op, ose = oracle_cv(oracle, req, cfg)
    np.testing.assert_allclose(p, op, rtol=1e-8, atol=1e-9 * req.S0)
    np.testing.assert_allclose(se, ose, rtol=1e-6, atol=1e-12 * req.S0)


def test_fp64_control_variate_many_maturities_equals_oracle(engine, oracle):
    """A set with more control-variate maturities than the warp-per-pair recursion takes (32) runs the
    one-thread-per-(maturity, node) recursion; short maturities keep the oracle's recursion quick."""
    req, cfg = W.single_chain(n_paths=1 << 12)
    T = np.arange(1, 41) * 5 / 252.0                       # 40 maturities, 5 to 200 trading days
    req.options = E.Options(strike=np.full(40, req.S0), T=T, payoff=E.ASIAN)
    cfg.precision = E.FP64
    cfg.control_variate = 1
    p, se = engine.price(req.params, req.S0, req.options, cfg)
    op, ose = oracle_cv(oracle, req, cfg)
    np.testing.assert_allclose(p, op, rtol=1e-8, atol=1e-9 * req.S0)
    np.testing.assert_allclose(se, ose, rtol=1e-6, atol=1e-12 * req.S0)


def test_control_variate_against_the_plain_estimator(engine):
    req, cfg = W.single_chain(n_paths=1 << 16, precision=E.FP32)
    p, se = engine.price(req.params, req.S0, req.options, cfg)
    cfg.control_variate = 1
    pc, sec = engine.price(req.params, req.S0, req.options, cfg)
    asian = req.options.payoff == E.ASIAN
    np.testing.assert_array_equal(pc[~asian], p[~asian])       # Europeans: the reference's estimator
    liquid = asian & (p > 0.05)
    assert np.max(np.abs(pc - p)[liquid] / se[liquid]) < 4.0
    assert np.median(se[liquid] / sec[liquid]) > 5.0           # measured about 13x on this chain


def test_fp32_control_variate_vs_fp64(engine):
    req, cfg = W.single_chain(n_paths=1 << 14, precision=E.FP64)
    cfg.control_variate = 1
    p64, se64 = engine.price(req.params, req.S0, req.options, cfg)
    cfg.precision = E.FP32
    p32, _ = engine.price(req.params, req.S0, req.options, cfg)
    big = p64 > 1e-3 * req.S0
    assert np.all(np.abs(p32 - p64)[big] <= np.maximum(1e-4 * p64[big], se64[big]))


def test_control_variate_batch_equals_alone(engine):
    reqs, cfg = W.uneven_batch(n_sets=4, path_scale=1 / 256, precision=E.FP32)
    cfg.control_variate = 1
    together = engine.price_batch(reqs, cfg)
    for rq, (p, se) in zip(reqs, together):
        pa, sa = engine.price_batch([rq], cfg)[0]
        np.testing.assert_array_equal(p, pa)
        np.testing.assert_array_equal(se, sa)
    rev = engine.price_batch(reqs[::-1], cfg)
    for (p, _), (pr, _) in zip(together, rev[::-1]):
        np.testing.assert_array_equal(p, pr)


def test_control_variate_unsupported_paths(engine):
    req, cfg = W.single_chain(n_paths=1024)
    cfg.control_variate = 1
    with pytest.raises(HexoError):
        engine.partial(req.params, req.S0, req.options, cfg, 0, 512)
    cfg.control_variate = 2
    with pytest.raises(HexoError):
        engine.price(req.params, req.S0, req.options, cfg)


def test_control_variate_through_the_server(engine):
    reqs, cfg = W.uneven_batch(n_sets=6, seed=11, path_scale=1 / 256, precision=E.FP32)
    cfg.control_variate = 1
    alone = [engine.price_batch([rq], cfg)[0] for rq in reqs]
    with engine.server(cfg, max_batch_requests=3, max_inflight=2) as srv:
        mixed = [srv.wait(t) for t in [srv.submit(rq) for rq in reqs]]
    for (pa, sa), (pm, sm) in zip(alone, mixed):
        np.testing.assert_array_equal(pa, pm)
        np.testing.assert_array_equal(sa, sm)


def test_control_variate_launch_shapes_bit_identical(engine):
    req, cfg = W.single_chain(n_paths=5000, precision=E.FP32)
    cfg.control_variate = 1
    out = []
    for block in (128, 256, 512):
        cfg.block = block
        out.append(engine.price(req.params, req.S0, req.options, cfg))
    for p, se in out[1:]:
        np.testing.assert_array_equal(p, out[0][0])
        np.testing.assert_array_equal(se, out[0][1])
    cfg.block, cfg.paths_per_thread = 256, 2     # the control variate runs one path per thread
    with pytest.raises(HexoError):
        engine.price(req.params, req.S0, req.options, cfg)
