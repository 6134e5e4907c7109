"""The QE branch mix the kernels report, against the oracle's walk.

Each launch reports the QE steps of its active paths that took the quadratic
branch (HSimulation.tpp:63-68; the rest took the exponential one,
tpp:70-73).  With every option of a request on the same path count, each
path is walked to the same last maturity by the kernel and by the oracle,
so the counts must be equal exactly, in both forms: the FP64 form takes the
reference's decisions, and the FP32 form must take the same ones (its
double-single variance and exact tie-breaks exist for that).  On the
uneven batch the two forms run the same tiles, so their counts must agree.
"""
import numpy as np
import pytest

from hestonexotics_gb300 import engine as E
from hestonexotics_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def kernel_counts(engine, reqs, cfg):
    b = engine.prepare_batch(reqs, cfg)
    b.launch()
    b.collect()
    inf = b.info()
    b.close()
    return inf["quad_steps"], inf["executed_path_steps"]


def oracle_counts(oracle, req, cfg):
    o = req.options
    return oracle.branch_counts(req.params.as_array(), req.S0, o.strike, o.T, o.payoff.astype(np.uint8), o.n_paths,
                                n_default=cfg.n_paths, step_mode=cfg.step_mode, steps=cfg.steps,
                                steps_per_year=cfg.steps_per_year, seed=req.seed, stream=req.stream)


CASES = {
    "plain_asian": lambda: W.plain_asian(n_paths=8192),
    "chain": lambda: W.single_chain(n_paths=4096),
    "feller_violating": lambda: W.feller_violating(n_paths=4096),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_branch_counts_equal_oracle_in_both_forms(engine, oracle, case):
    req, cfg = CASES[case]()
    want_q, want_n = oracle_counts(oracle, req, cfg)
    assert 0 < want_q <= want_n
    for prec in (E.FP64, E.FP32):
        cfg.precision = prec
        q, n = kernel_counts(engine, [req], cfg)
        assert n == want_n, (prec, n, want_n)
        assert q == want_q, (prec, q, want_q)


def test_branch_counts_fp32_equal_fp64_on_the_uneven_batch(engine):
    reqs, cfg32 = W.uneven_batch(seed=2, precision=E.FP32, path_scale=1 / 64)
    cfg64 = E.Config(**{**cfg32.__dict__, "precision": E.FP64})
    q32, n32 = kernel_counts(engine, reqs, cfg32)
    q64, n64 = kernel_counts(engine, reqs, cfg64)
    assert n32 == n64 and 0 < q64 < n64
    assert q32 == q64, (q32, q64)
