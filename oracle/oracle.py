"""ORACLE / TEST INFRASTRUCTURE ONLY.

ctypes wrapper over the CPU oracle (oracle/_build/liboracle.so, the port of
the reference's pricing path) and, where it was built, over
oracle/_ref/libhexo_ref.so (the reference's own sources).  Imported only by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, to check
results against; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_EXACT = HERE / "_build" / "liboracle.so"
LIB_FAST = HERE / "_build" / "liboracle_fast.so"
LIB_REF = HERE / "_ref" / "libhexo_ref.so"

_D = C.POINTER(C.c_double)
_cache = {}


def build():
    subprocess.run(["make", "-C", str(HERE), "-j4"], check=True, capture_output=True)


def _load(path: Path):
    if path in _cache:
        return _cache[path]
    if not path.exists():
        build()
    lib = C.CDLL(str(path))
    lib.oracle_price_paths.restype = C.c_int
    lib.oracle_path_finals.restype = C.c_int
    lib.oracle_price_reference_partition.restype = C.c_int64
    lib.oracle_ppnd16.restype = C.c_double
    lib.oracle_ppnd16.argtypes = [C.c_double, C.POINTER(C.c_int)]
    lib.oracle_logf_c.restype = C.c_float
    lib.oracle_logf_c.argtypes = [C.c_float]
    _cache[path] = lib
    return lib


def lib(fast: bool = False):
    return _load(LIB_FAST if fast else LIB_EXACT)


def ref_lib():
    """The reference-compiled harness, or None where it cannot exist."""
    if not LIB_REF.exists():
        return None
    if LIB_REF in _cache:
        return _cache[LIB_REF]
    r = C.CDLL(str(LIB_REF))
    _cache[LIB_REF] = r
    return r


def _p(a):
    return C.c_void_p(a.ctypes.data)


def shishua_words(seed4, n_words: int) -> np.ndarray:
    s = np.ascontiguousarray(seed4, dtype=np.uint64)
    out = np.zeros(n_words, dtype=np.uint64)
    lib().oracle_shishua_words(_p(s), C.c_uint64(n_words), _p(out))
    return out


def rng_draws(seed: int, block_words: int, kinds, stream: int = 0) -> np.ndarray:
    k = np.ascontiguousarray(kinds, dtype=np.uint8)
    out = np.zeros(len(k))
    lib().oracle_rng_draws(C.c_uint32(seed & 0xFFFFFFFF), C.c_uint32(stream & 0xFFFFFFFF), C.c_uint32(block_words),
                           _p(k), C.c_uint64(len(k)), _p(out))
    return out


def ppnd16(p: float):
    ifault = C.c_int(0)
    v = lib().oracle_ppnd16(float(p), C.byref(ifault))
    return v, ifault.value


def logf(x: float) -> float:
    return lib().oracle_logf_c(float(x))


def normals(words) -> np.ndarray:
    w = np.ascontiguousarray(words, dtype=np.uint64)
    out = np.zeros(len(w))
    lib().oracle_normals(_p(w), C.c_uint64(len(w)), _p(out))
    return out


def _opts(strike, T, kind, n_paths, n_default):
    strike = np.ascontiguousarray(strike, dtype=np.float64)
    T = np.ascontiguousarray(np.broadcast_to(T, strike.shape), dtype=np.float64)
    kind = np.ascontiguousarray(np.broadcast_to(kind, strike.shape), dtype=np.uint8)
    if n_paths is None:
        n_paths = n_default
    n_paths = np.ascontiguousarray(np.broadcast_to(n_paths, strike.shape), dtype=np.uint64).copy()
    n_paths[n_paths == 0] = n_default
    return strike, T, kind, n_paths


def price_paths(params7, S0, strike, T, kind, n_paths=None, *, n_default=65536, step_mode=0, steps=252,
                steps_per_year=252.0, seed=42, stream=0, block_words=16, path_lo=0, path_hi=None, threads=None,
                fast=False):
    """Per-path stream partition (the GPU's).  Returns (price, stderr, limbs[n,6] uint64)."""
    strike, T, kind, n_paths = _opts(strike, T, kind, n_paths, n_default)
    p = np.ascontiguousarray(params7, dtype=np.float64)
    n = len(strike)
    price = np.zeros(n)
    se = np.zeros(n)
    sums = np.zeros(6 * n, dtype=np.uint64)
    hi = int(n_paths.max()) if path_hi is None else int(path_hi)
    th = threads or os.cpu_count() or 1
    rc = lib(fast).oracle_price_paths(_p(p), C.c_double(S0), C.c_uint32(n), _p(strike), _p(T), _p(kind),
                                      _p(n_paths), C.c_uint32(step_mode), C.c_uint32(steps),
                                      C.c_double(steps_per_year), C.c_uint32(seed & 0xFFFFFFFF),
                                      C.c_uint32(stream & 0xFFFFFFFF), C.c_uint32(block_words),
                                      C.c_uint64(path_lo), C.c_uint64(hi), C.c_int(th), _p(price), _p(se),
                                      _p(sums))
    if rc != 0:
        raise ValueError(f"oracle_price_paths failed: {rc}")
    return price, se, sums.reshape(n, 6)


def branch_counts(params7, S0, strike, T, kind, n_paths=None, *, n_default=65536, step_mode=0, steps=252,
                  steps_per_year=252.0, seed=42, stream=0, block_words=16, path_lo=0, path_hi=None, threads=None):
    """(quadratic-branch QE steps, all QE steps) of the per-path partition."""
    strike, T, kind, n_paths = _opts(strike, T, kind, n_paths, n_default)
    p = np.ascontiguousarray(params7, dtype=np.float64)
    counts = np.zeros(2, dtype=np.uint64)
    hi = int(n_paths.max()) if path_hi is None else int(path_hi)
    th = threads or os.cpu_count() or 1
    rc = lib().oracle_branch_counts(_p(p), C.c_double(S0), C.c_uint32(len(strike)), _p(strike), _p(T), _p(kind),
                                    _p(n_paths), C.c_uint32(step_mode), C.c_uint32(steps), C.c_double(steps_per_year),
                                    C.c_uint32(seed & 0xFFFFFFFF), C.c_uint32(stream & 0xFFFFFFFF),
                                    C.c_uint32(block_words), C.c_uint64(path_lo), C.c_uint64(hi), C.c_int(th),
                                    _p(counts))
    if rc != 0:
        raise ValueError(f"oracle_branch_counts failed: {rc}")
    return int(counts[0]), int(counts[1])


def geo_calls(params7, S0, strike, T, kind, *, step_mode=0, steps=252, steps_per_year=252.0):
    """E[(G - K)^+] of the geometric control variate per Asian option (0 for the others), undiscounted."""
    strike, T, kind, _ = _opts(strike, T, kind, None, 1)
    p = np.ascontiguousarray(params7, dtype=np.float64)
    out = np.zeros(len(strike))
    rc = lib().oracle_geo_calls(_p(p), C.c_double(S0), C.c_uint32(len(strike)), _p(strike), _p(T), _p(kind),
                                C.c_uint32(step_mode), C.c_uint32(steps), C.c_double(steps_per_year), _p(out))
    if rc != 0:
        raise ValueError(f"oracle_geo_calls failed: {rc}")
    return out


def price_paths_cv(params7, S0, strike, T, kind, n_paths=None, *, n_default=65536, step_mode=0, steps=252,
                   steps_per_year=252.0, seed=42, stream=0, block_words=16, path_lo=0, path_hi=None, threads=None):
    """price_paths with the geometric control variate on the Asian options: (price, stderr)."""
    strike, T, kind, n_paths = _opts(strike, T, kind, n_paths, n_default)
    p = np.ascontiguousarray(params7, dtype=np.float64)
    n = len(strike)
    price, se = np.zeros(n), np.zeros(n)
    hi = int(n_paths.max()) if path_hi is None else int(path_hi)
    th = threads or os.cpu_count() or 1
    rc = lib().oracle_price_paths_cv(_p(p), C.c_double(S0), C.c_uint32(n), _p(strike), _p(T), _p(kind),
                                     _p(n_paths), C.c_uint32(step_mode), C.c_uint32(steps),
                                     C.c_double(steps_per_year), C.c_uint32(seed & 0xFFFFFFFF),
                                     C.c_uint32(stream & 0xFFFFFFFF), C.c_uint32(block_words), C.c_uint64(path_lo),
                                     C.c_uint64(hi), C.c_int(th), _p(price), _p(se))
    if rc != 0:
        raise ValueError(f"oracle_price_paths_cv failed: {rc}")
    return price, se


def path_finals(params7, S0, strike, T, kind, n_paths=None, *, n_default=65536, step_mode=0, steps=252,
                steps_per_year=252.0, seed=42, stream=0, block_words=16, path_lo=0, path_hi=64):
    strike, T, kind, n_paths = _opts(strike, T, kind, n_paths, n_default)
    p = np.ascontiguousarray(params7, dtype=np.float64)
    m = len(np.unique(T))
    n = path_hi - path_lo
    a = np.zeros(n * m)
    e = np.zeros(n * m)
    nm = C.c_uint32()
    rc = lib().oracle_path_finals(_p(p), C.c_double(S0), C.c_uint32(len(strike)), _p(strike), _p(T), _p(kind),
                                  _p(n_paths), C.c_uint32(step_mode), C.c_uint32(steps), C.c_double(steps_per_year),
                                  C.c_uint32(seed & 0xFFFFFFFF), C.c_uint32(stream & 0xFFFFFFFF),
                                  C.c_uint32(block_words), C.c_uint64(path_lo), C.c_uint64(path_hi), _p(a), _p(e),
                                  C.byref(nm))
    if rc != 0:
        raise ValueError(f"oracle_path_finals failed: {rc}")
    return a.reshape(n, m), e.reshape(n, m)


def price_reference_partition(params7, S0, strike, T, kind, steps, n_sims, *, n_threads=1, buf_words=1 << 20,
                              omp_threads=1, fast=False):
    """The reference's own thread partition (undiscounted, as price() returns)."""
    strike = np.ascontiguousarray(strike, dtype=np.float64)
    T = np.ascontiguousarray(np.broadcast_to(T, strike.shape), dtype=np.float64)
    kind = np.ascontiguousarray(np.broadcast_to(kind, strike.shape), dtype=np.uint8)
    p = np.ascontiguousarray(params7, dtype=np.float64)
    out = np.zeros(len(strike))
    n = lib(fast).oracle_price_reference_partition(_p(p), C.c_double(S0), C.c_uint32(len(strike)), _p(strike), _p(T),
                                                   _p(kind), C.c_uint32(steps), C.c_uint32(n_sims),
                                                   C.c_int(n_threads), C.c_uint32(buf_words), C.c_int(omp_threads),
                                                   _p(out))
    if n < 0:
        raise ValueError("oracle_price_reference_partition failed")
    return out, int(n)


# ------------------------------------------------------------------ SWIFT

SWIFT_TRUNCATION_RELEASE = 1e-7   # FASTMATH build (Makefile.am:67, SWIFT.cpp:12-16)


def swift_params(params5, tau, r, S, K_min, K_max, trunc_precision=SWIFT_TRUNCATION_RELEASE) -> np.ndarray:
    """Dynamic wavelet parameters {m, 2^m, sqrt 2^m, lower, upper, k1, k2, J} (SWIFT.cpp:21-35)."""
    p = np.ascontiguousarray(params5, dtype=np.float64)
    out = np.zeros(8)
    rc = lib().oracle_swift_params(_p(p), C.c_double(tau), C.c_double(r), C.c_double(S), C.c_double(K_min),
                                   C.c_double(K_max), C.c_double(trunc_precision), _p(out))
    if rc != 0:
        raise RuntimeError("swift parameters did not converge")
    return out


def swift_price(params5, tau, r, S, strikes, sp8=None, grad=False):
    """European call prices of one expiry by the SWIFT restatement; with
    grad=True also the [n, 5] gradient in (v0, vm, rho, kappa, sigma) order."""
    strikes = np.ascontiguousarray(strikes, dtype=np.float64)
    p = np.ascontiguousarray(params5, dtype=np.float64)
    if sp8 is None:
        sp8 = swift_params(p, tau, r, S, strikes.min(), strikes.max())
    sp8 = np.ascontiguousarray(sp8, dtype=np.float64)
    n = len(strikes)
    price = np.zeros(n)
    g = np.zeros(5 * n) if grad else None
    rc = lib().oracle_swift_price(_p(p), C.c_double(tau), C.c_double(r), C.c_double(S), _p(strikes), C.c_uint32(n),
                                  _p(sp8), _p(price), _p(g) if grad else None)
    if rc != 0:
        raise RuntimeError("swift pricing failed")
    return (price, g.reshape(n, 5)) if grad else price


def heston_chf_grad(params5, tau, u: complex) -> np.ndarray:
    p = np.ascontiguousarray(params5, dtype=np.float64)
    out = np.zeros(12)
    lib().oracle_heston_chf_grad(_p(p), C.c_double(tau), C.c_double(u.real), C.c_double(u.imag), _p(out))
    return out[0::2] + 1j * out[1::2]


# ------------------------------------------------------------ work counts

def nominal_path_steps(T, n_paths, *, step_mode=1, steps=252, steps_per_year=252.0) -> int:
    """Nominal path-steps of one request, counted as the reference walks its
    time grid (HSimulation.tpp:29-46): a path runs to the last maturity whose
    options it prices, and reaching maturity T_j takes steps_j grid steps
    (the `steps` argument per maturity, or max(5, round(steps_per_year T_j)) on
    the daily grid).  Paths that a later maturity needs count that
    maturity's steps.  Pure Python: the CPU baseline counts its own work."""
    T = np.asarray(T, dtype=np.float64)
    n = np.asarray(n_paths, dtype=np.uint64)
    uT = np.unique(T)
    if step_mode == 1:
        st = np.maximum(5.0, np.rint(steps_per_year * uT)).astype(np.int64)
    else:
        st = np.full(len(uT), int(steps), dtype=np.int64)
    mat_paths = np.array([int(n[T == t].max()) for t in uT], dtype=np.int64)
    thr = np.zeros(len(uT) + 1, dtype=np.int64)
    for j in range(len(uT) - 1, -1, -1):           # paths that reach maturity j
        thr[j] = max(thr[j + 1], mat_paths[j])
    return int(sum((int(thr[j]) - int(thr[j + 1])) * int(st[j]) for j in range(len(uT))))
