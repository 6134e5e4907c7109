"""The bounds-checked build (libhexo_mc_checks.so, HEXO_CHECKS).

Compiled from the same sources with every descriptor, conversion-queue,
payoff-window, sum-slot and ring index of the path kernels checked; a failed
check would set an error bit, record the check's code and the offending index,
skip the access and return HEXO_ERR_CHECK.  Here the small cases of the other
tests (every entry point that launches the path kernels: one-shot, batches,
prepared graphs, shards, serving with requests split across launches, the
no-allocation call, the control variate, several launch shapes) run through
it in a child process.  None may fail a check, and every price and standard
error must equal the ordinary library's bit for bit (the checks change no
arithmetic).
"""
import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent


def run_cases(out_path: str) -> None:
    """Prices the cases with the library the bindings loaded; saves every array."""
    from hestonexotics_gb300 import _lib as L
    from hestonexotics_gb300 import engine as E
    from hestonexotics_gb300 import workloads as W
    res = {}
    eng = E.Engine(0)
    try:
        rq, cfg = W.plain_asian(n_paths=4096)
        for prec in (E.FP64, E.FP32):
            cfg.precision = prec
            res[f"asian_{prec}"] = np.stack(eng.price(rq.params, rq.S0, rq.options, cfg))
        rq, cfg = W.single_chain(n_paths=3000)
        for prec in (E.FP64, E.FP32):
            cfg.precision = prec
            res[f"chain_{prec}"] = np.stack(eng.price(rq.params, rq.S0, rq.options, cfg))
            for block, ppt, unroll in ((128, 2, 2), (512, 1, 4), (128, 4, 1)):
                c = E.Config(**{**cfg.__dict__, "block": block, "paths_per_thread": ppt, "unroll": unroll})
                res[f"chain_{prec}_{block}_{ppt}_{unroll}"] = np.stack(eng.price(rq.params, rq.S0, rq.options, c))
            c = E.Config(**{**cfg.__dict__, "control_variate": 1})
            res[f"chain_cv_{prec}"] = np.stack(eng.price(rq.params, rq.S0, rq.options, c))
        rng = np.random.default_rng(5)
        n = 150
        T = np.repeat([0.1, 0.35, 0.35001, 1.2], [40, 70, 20, 20])
        opts = E.Options(rng.uniform(70, 140, n), T, rng.integers(0, 2, n),
                         rng.choice([1, 31, 33, 257, 1000, 4099], n).astype(np.uint64))
        params = E.Params(0.05, 0.03, -0.5, 2.5, 0.7, r=0.01, q=0.02)
        res["ragged"] = np.stack(eng.price(params, 100.0, opts, E.Config(n_paths=1000, step_mode=E.STEP_GRID, seed=99)))
        reqs, cfg = W.uneven_batch(n_sets=5, path_scale=1 / 512, precision=E.FP32)
        for i, (p, s) in enumerate(eng.price_batch(reqs, cfg)):
            res[f"batch_{i}"] = np.stack([p, s])
        b = eng.prepare_batch(reqs, cfg)
        b.launch()
        for i, (p, s) in enumerate(b.collect()):
            res[f"graph_{i}"] = np.stack([p, s])
        b.close()
        res["shard"] = eng.batch_partial(reqs, cfg, 1, 3).astype(np.int64)
        with eng.server(cfg, max_batch_requests=3, max_inflight=2, launch_path_steps=1 << 21) as srv:
            for i, (p, s) in enumerate([srv.wait(srv.submit(r)) for r in reqs]):
                res[f"served_{i}"] = np.stack([p, s])
        rq, cfg = W.single_chain(n_paths=2000)
        keep = np.arange(0, len(rq.options), 7)[:100]
        o = E.Options(rq.options.strike[keep], rq.options.T[keep], rq.options.payoff[keep])
        price, se = np.zeros(len(o)), np.zeros(len(o))
        pp, cc = rq.params.c(), cfg.c()
        st = L.load().hexo_price_noalloc(C.byref(pp), float(rq.S0), o.c_array(), len(o), C.byref(cc),
                                         price.ctypes.data_as(C.POINTER(C.c_double)),
                                         se.ctypes.data_as(C.POINTER(C.c_double)), None)
        if st != 0:
            raise L.HexoError(st, "hexo_price_noalloc")
        res["noalloc"] = np.stack([price, se])
    finally:
        eng.close()
    np.savez(out_path, **res)


def test_checked_build_matches_and_trips_no_check(tmp_path):
    from hestonexotics_gb300 import build
    build.build()   # both libraries
    env = {**os.environ, "HEXO_LIB": "checks"}
    code = (f"import sys; sys.path[:0] = [{str(HERE.parent)!r}, {str(HERE)!r}]\n"
            "from hestonexotics_gb300 import _lib as L\n"
            "assert L.LIB_PATH.name == 'libhexo_mc_checks.so', L.LIB_PATH\n"
            f"import test_gpu_checks as T; T.run_cases({str(tmp_path / 'checked.npz')!r})\n")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    run_cases(str(tmp_path / "plain.npz"))
    a, b = np.load(tmp_path / "checked.npz"), np.load(tmp_path / "plain.npz")
    assert sorted(a.files) == sorted(b.files)
    for k in a.files:
        assert np.array_equal(a[k], b[k], equal_nan=True), k
