"""The oracle's random numbers, pinned (CPU only).

* SHISHUA's 16 initialisation constants are recomputed from their definition
  (hex digits of (sqrt(5)-1)/2) and checked in both the oracle's and the
  device code's source; the last four also appear in the reference's
  shishua_inline_patch.diff context.
* The oracle's restated RNG two-buffer wrapper reproduces, bit for bit, the
  draws of the reference's own RNG class (tests/golden/rng_draws.json, made
  from src/RNG.cpp by tests/golden/make_golden.py).
* The float32 AS241 restatement agrees with an accurate inverse normal to
  float precision, and handles P = 0 and P = 1 as as241.f90:99-102 does.
* The deterministic float logarithm used by AS241's tail stays within one
  float ulp of the correctly rounded logarithm.
"""
import re
from math import isqrt

import numpy as np
import pytest

from conftest import ROOT, golden, unhex


def phi_words():
    B = 1024
    x = (isqrt(5 << (2 * B)) - (1 << B)) // 2
    return [(x >> (B - 64 * (i + 1))) & ((1 << 64) - 1) for i in range(16)]


@pytest.mark.parametrize("path", ["oracle/shishua.h", "hestonexotics_gb300/csrc/hexo_device.cuh"])
def test_shishua_constants_from_definition(path):
    text = (ROOT / path).read_text()
    found = [int(h, 16) for h in re.findall(r"0x([0-9A-F]{16})ull", text)]
    assert found[:16] == phi_words()


def test_patch_context_constants():
    # the reference's patch file shows the last row of the constant table
    patch = ROOT.parent / "reference" / "shishua_inline_patch.diff"
    if not patch.exists():
        pytest.skip("reference checkout not present")
    shown = [int(h, 16) for h in re.findall(r"0x([0-9A-F]{16})", patch.read_text())][:4]
    assert shown == phi_words()[12:]


def test_rng_draws_match_reference_class(oracle):
    for case in golden("rng_draws.json"):
        got = oracle.rng_draws(case["seed"], case["size"], np.array(case["kinds"], dtype=np.uint8))
        want = unhex(case["draws"])
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), (case["seed"], case["size"])


def test_uniform_definition(oracle):
    # u = (double)w / (double)UINT64_MAX over the first block (RNG.cpp:31)
    words = oracle.shishua_words([5, 0, 0, 0], 16)
    draws = oracle.rng_draws(5, 16, np.ones(16, dtype=np.uint8))
    assert np.array_equal(draws, words.astype(np.float64) / 18446744073709551616.0)


def test_live_reference_rng(oracle):
    ref = oracle.ref_lib()
    if ref is None:
        pytest.skip("reference-compiled harness not built")
    import ctypes as C
    rng = np.random.default_rng(99)
    for seed in (11, 123456789):
        kinds = (rng.random(5000) < 0.05).astype(np.uint8)
        out = np.zeros(len(kinds))
        ref.ref_rng_draws(C.c_uint32(seed), C.c_uint32(16), C.c_void_p(kinds.ctypes.data), C.c_uint64(len(kinds)),
                          C.c_void_p(out.ctypes.data))
        assert np.array_equal(oracle.rng_draws(seed, 16, kinds).view(np.uint64), out.view(np.uint64))


def test_ppnd16_accuracy(oracle):
    special = pytest.importorskip("scipy.special")
    ps = np.concatenate([np.linspace(1e-6, 1 - 1e-6, 2001), np.geomspace(1e-18, 0.07, 300)])
    for p in ps:
        v, ifault = oracle.ppnd16(p)
        assert ifault == 0
        exact = special.ndtri(p)
        # float32 evaluation: a few float ulps relative (absolute near 0)
        assert abs(v - exact) <= 4e-7 * max(1.0, abs(exact)), (p, v, exact)


def test_ppnd16_faults(oracle):
    assert oracle.ppnd16(0.0) == (0.0, 1)
    assert oracle.ppnd16(1.0) == (0.0, 1)
    assert oracle.ppnd16(0.5) == (0.0, 0)
    v, f = oracle.ppnd16(0.975)
    assert f == 0 and abs(v - 1.959963985) < 1e-6


def _logf_err_ulps(oracle, xs):
    got = np.array([oracle.logf(float(x)) for x in xs], dtype=np.float32)
    exact = np.log(xs.astype(np.float64))
    ulp = np.spacing(np.abs(exact).astype(np.float32)).astype(np.float64)
    return np.abs(got.astype(np.float64) - exact) / ulp, got, exact


def test_logf_tail_domain_within_one_ulp(oracle):
    # AS241 takes the log only of R = min(P, 1-P) < 0.075 (as241.f90:94-104)
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.uniform(0, 0.075, 20000), np.geomspace(1e-19, 0.075, 20000)]).astype(np.float32)
    xs = xs[xs > 0]
    err, got, exact = _logf_err_ulps(oracle, xs)
    assert err.max() <= 1.0
    # nearly always the correctly rounded result
    assert np.mean(got != exact.astype(np.float32)) < 0.02


def test_logf_elsewhere_within_two_ulps(oracle):
    rng = np.random.default_rng(4)
    xs = np.concatenate([rng.uniform(0.075, 4, 5000), np.geomspace(1e-37, 1e30, 5000)]).astype(np.float32)
    err, _, _ = _logf_err_ulps(oracle, xs)
    assert err.max() <= 2.0


def test_draw_moments_like_the_reference_rng_test(oracle):
    # the reference's rng_test (UnitTest.cpp:528-564) checks the mean and
    # variance of RNG(2^20, 1) uniforms and normals; here 2^21 of each from
    # the same generator, within 5 standard errors of the exact moments
    n = 1 << 21
    kinds = np.concatenate([np.ones(n, dtype=np.uint8), np.zeros(n, dtype=np.uint8)])
    d = oracle.rng_draws(1, 1 << 20, kinds)
    u, z = d[:n], d[n:]
    assert abs(u.mean() - 0.5) < 5 * np.sqrt(1 / 12 / n)
    assert abs(u.var() - 1 / 12) < 5 * np.sqrt(1 / 180 / n)
    assert abs(z.mean()) < 5 / np.sqrt(n)
    assert abs(z.var() - 1.0) < 5 * np.sqrt(2.0 / n)
    assert u.min() >= 0.0 and u.max() <= 1.0
