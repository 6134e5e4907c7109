"""Seeded synthetic workloads with the shapes of the pricing configurations.

The reference prices live option chains downloaded from Tradier
(src/WebAPI.cpp:94-116); there is no network here, so these generators
stand in for them with the stated parameter ranges, maturities, strikes and
path counts.

  plain_asian()      one arithmetic-Asian call, S0=100, K=100, T=1, r=0.02,
                     v0=0.04, kappa=1.5, theta=0.04, sigma=0.5, rho=-0.7,
                     252 reference steps, 65,536 paths, seed 42
  single_chain()     one parameter set (seed 1); maturities 1/12..3 y on the
                     252/y grid; 50 log-spaced strikes in [0.6, 1.6] S0 per
                     maturity; Asian and European calls; 2^20 paths
  feller_violating() kappa=0.5, theta=0.04, sigma=1, rho=-0.9, v0=0.04
  uneven_batch()     64 parameter sets (seed 2), chains of 10-400 options,
                     maturities U[0.02, 5] y snapped to the daily grid, paths
                     per distinct maturity log-uniform in [2^14, 2^22],
                     Asian:European 3:1
  request_stream()   Poisson arrivals (seed 3) of single-set requests with
                     1-400 options and target-SE path counts

Every request of a batch or of a request stream gets its own stream number
(seed word 1 of its paths' generators), so no two requests share a path's
random stream even where their seed ranges [seed, seed + paths) overlap.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .engine import ASIAN, EUROPEAN, FP32, FP64, STEP_GRID, STEP_REFERENCE, Config, Options, Params, Request

S0_DEFAULT = 100.0
CHAIN_MATURITIES = (1 / 12, 1 / 4, 1 / 2, 3 / 4, 1.0, 1.5, 2.0, 3.0)


def plain_asian(r: float = 0.02, n_paths: int = 65536):
    params = Params(v0=0.04, theta=0.04, rho=-0.7, kappa=1.5, sigma=0.5, r=r, q=0.0)
    opts = Options(strike=np.array([100.0]), T=1.0, payoff=ASIAN)
    cfg = Config(n_paths=n_paths, step_mode=STEP_REFERENCE, steps=252, seed=42, precision=FP64)
    return Request(params, 100.0, opts, seed=42), cfg


def draw_params(rng: np.random.Generator) -> Params:
    v0 = rng.uniform(0.01, 0.09)
    theta = rng.uniform(0.01, 0.09)
    kappa = rng.uniform(0.5, 5.0)
    sigma = rng.uniform(0.1, 1.0)
    rho = rng.uniform(-0.9, -0.1)
    r = rng.uniform(0.0, 0.05)
    return Params(v0=v0, theta=theta, rho=rho, kappa=kappa, sigma=sigma, r=r, q=0.0)


def chain_options(S0: float = S0_DEFAULT, n_strikes: int = 50, kinds=(ASIAN, EUROPEAN),
                  maturities=CHAIN_MATURITIES) -> Options:
    strikes = np.geomspace(0.6 * S0, 1.6 * S0, n_strikes)
    K, T, P = [], [], []
    for t in maturities:
        for kind in kinds:
            K.append(strikes)
            T.append(np.full(n_strikes, t))
            P.append(np.full(n_strikes, kind))
    return Options(strike=np.concatenate(K), T=np.concatenate(T), payoff=np.concatenate(P))


def single_chain(n_paths: int = 1 << 20, precision: int = FP64, seed: int = 1, kinds=(ASIAN, EUROPEAN)):
    rng = np.random.default_rng(seed)
    params = draw_params(rng)
    req = Request(params, S0_DEFAULT, chain_options(kinds=kinds), seed=seed)
    cfg = Config(n_paths=n_paths, step_mode=STEP_GRID, steps_per_year=252.0, seed=seed, precision=precision)
    return req, cfg


def feller_violating(n_paths: int = 1 << 20, precision: int = FP64):
    params = Params(v0=0.04, theta=0.04, rho=-0.9, kappa=0.5, sigma=1.0, r=0.02, q=0.0)
    req = Request(params, S0_DEFAULT, chain_options(), seed=7)
    cfg = Config(n_paths=n_paths, step_mode=STEP_GRID, steps_per_year=252.0, seed=7, precision=precision)
    return req, cfg


def _snap_daily(T: np.ndarray) -> np.ndarray:
    return np.maximum(5, np.rint(T * 252.0)) / 252.0


def uneven_batch(n_sets: int = 64, seed: int = 2, precision: int = FP32, path_scale: float = 1.0):
    """64 parameter sets with uneven chains.  path_scale < 1 shrinks every path
    count (for quick tests); 1.0 is the full workload."""
    rng = np.random.default_rng(seed)
    reqs = []
    for s in range(n_sets):
        params = draw_params(rng)
        n_opts = int(rng.integers(10, 401))
        T = _snap_daily(rng.uniform(0.02, 5.0, n_opts))
        K = S0_DEFAULT * np.exp(rng.uniform(math.log(0.6), math.log(1.6), n_opts))
        kind = np.where(rng.random(n_opts) < 0.75, ASIAN, EUROPEAN).astype(np.uint32)
        uT = np.unique(T)
        paths_u = np.rint(2.0 ** rng.uniform(14.0, 22.0, len(uT)))
        paths_u = np.maximum(1, np.rint(paths_u * path_scale)).astype(np.uint64)
        n_paths = paths_u[np.searchsorted(uT, T)]
        reqs.append(Request(params, S0_DEFAULT, Options(strike=K, T=T, payoff=kind, n_paths=n_paths),
                            seed=int(rng.integers(0, 2 ** 32)), stream=s))
    cfg = Config(n_paths=1 << 14, step_mode=STEP_GRID, steps_per_year=252.0, seed=seed, precision=precision)
    return reqs, cfg


@dataclass
class Arrival:
    t: float          # seconds after the stream starts
    request: Request


def target_paths(S0: float, target_se_frac: float = 1e-3, payoff_sd_frac: float = 0.2,
                 lo: int = 1 << 14, hi: int = 1 << 22) -> int:
    """Paths for a target standard error of target_se_frac * S0, given a payoff
    standard deviation of about payoff_sd_frac * S0 (an at-the-money call
    with ~20% volatility), clamped to [lo, hi]."""
    n = (payoff_sd_frac / target_se_frac) ** 2
    return int(min(hi, max(lo, round(n))))


def request_stream(rate_per_s: float, duration_s: float, seed: int = 3, max_opts: int = 400):
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    while True:
        t += rng.exponential(1.0 / rate_per_s)
        if t > duration_s:
            break
        params = draw_params(rng)
        n = int(rng.integers(1, max_opts + 1))
        T = _snap_daily(rng.uniform(0.02, 5.0, n))
        K = S0_DEFAULT * np.exp(rng.uniform(math.log(0.6), math.log(1.6), n))
        kind = np.where(rng.random(n) < 0.75, ASIAN, EUROPEAN).astype(np.uint32)
        npaths = target_paths(S0_DEFAULT)
        out.append(Arrival(t, Request(params, S0_DEFAULT, Options(strike=K, T=T, payoff=kind, n_paths=npaths),
                                      seed=int(rng.integers(0, 2 ** 32)), stream=len(out))))
    cfg = Config(n_paths=1 << 14, step_mode=STEP_GRID, steps_per_year=252.0, seed=seed, precision=FP32)
    return out, cfg


def stream_overlaps(requests, n_default: int = 1 << 14):
    """Pairs (i, j, paths) of requests whose paths share SHISHUA streams: the
    same stream number and overlapping seed ranges [seed, seed + n) modulo
    2^32, n the request's largest path count.  Empty for the workloads here."""
    spans = []
    for i, rq in enumerate(requests):
        n = rq.options.n_paths.astype(np.uint64)
        n = int(np.where(n == 0, np.uint64(n_default), n).max())
        spans.append((int(rq.stream) & 0xFFFFFFFF, int(rq.seed) & 0xFFFFFFFF, n, i))
    out = []
    by_stream = {}
    for st, seed, n, i in spans:
        by_stream.setdefault(st, []).append((seed, n, i))
    for group in by_stream.values():
        for a in range(len(group)):
            for b in range(a + 1, len(group)):
                (sa, na, ia), (sb, nb, ib) = group[a], group[b]
                d = (sb - sa) % (1 << 32)            # b's first seed as an offset into a's range
                shared = max(0, min(na, d + nb) - d) + max(0, min(nb, (1 << 32) - d + na) - ((1 << 32) - d))
                if shared:
                    out.append((ia, ib, shared))
    return out
