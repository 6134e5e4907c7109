"""Python face of the engine: a thin, typed wrapper over the C ABI.

Every computation runs in libhexo_mc.so on the GPU; this module only
marshals arrays.  ``Engine`` owns one ``hexo_ctx`` (one device, one stream).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _lib as L

ASIAN = 0
EUROPEAN = 1
STEP_REFERENCE = 0
STEP_GRID = 1
FP64 = 0
FP32 = 1


@dataclass
class Params:
    """HParams (reference src/inc/HDistribution.h:9-24: v_0, v_m, rho, kappa,
    sigma) plus the rates r and q, which the reference does not have."""
    v0: float
    theta: float
    rho: float
    kappa: float
    sigma: float
    r: float = 0.0
    q: float = 0.0

    def c(self) -> L.hexo_params:
        return L.hexo_params(self.v0, self.theta, self.rho, self.kappa, self.sigma, self.r, self.q)

    def as_array(self) -> np.ndarray:
        return np.array([self.v0, self.theta, self.rho, self.kappa, self.sigma, self.r, self.q], dtype=np.float64)


@dataclass
class Config:
    n_paths: int = 65536
    step_mode: int = STEP_REFERENCE
    steps: int = 252
    steps_per_year: float = 252.0
    seed: int = 42
    rng_block_words: int = 16
    precision: int = FP64
    block: int = 0
    paths_per_thread: int = 0
    unroll: int = 0
    control_variate: int = 0   # 1: Asian options with the geometric-average control variate
    stream: int = 0            # seed word 1 of the paths' streams (hexo_price, partial, no-allocation)

    def c(self) -> L.hexo_mc_cfg:
        return L.hexo_mc_cfg(self.n_paths, self.step_mode, self.steps, self.steps_per_year, self.seed & 0xFFFFFFFF,
                             self.rng_block_words, self.precision, self.block, self.paths_per_thread, self.unroll,
                             self.control_variate, self.stream & 0xFFFFFFFF)


@dataclass
class Options:
    """Structure of arrays of options: strike, maturity, payoff kind, paths (0 = config default)."""
    strike: np.ndarray
    T: np.ndarray
    payoff: np.ndarray
    n_paths: np.ndarray = field(default=None)

    def __post_init__(self):
        self.strike = np.ascontiguousarray(self.strike, dtype=np.float64)
        self.T = np.ascontiguousarray(np.broadcast_to(self.T, self.strike.shape), dtype=np.float64)
        self.payoff = np.ascontiguousarray(np.broadcast_to(self.payoff, self.strike.shape), dtype=np.uint32)
        if self.n_paths is None:
            self.n_paths = np.zeros(self.strike.shape, dtype=np.uint64)
        self.n_paths = np.ascontiguousarray(np.broadcast_to(self.n_paths, self.strike.shape), dtype=np.uint64)

    def __len__(self):
        return int(self.strike.shape[0])

    _DTYPE = np.dtype([("strike", "<f8"), ("T", "<f8"), ("payoff", "<u4"), ("reserved", "<u4"),
                       ("n_paths", "<u8")])

    def c_array(self):
        n = len(self)
        rec = np.zeros(max(n, 1), dtype=self._DTYPE)
        rec["strike"][:n] = self.strike
        rec["T"][:n] = self.T
        rec["payoff"][:n] = self.payoff
        rec["n_paths"][:n] = self.n_paths
        return (L.hexo_option * max(n, 1)).from_buffer(rec)   # the ctypes array keeps rec alive


@dataclass
class Request:
    """One pricing request.  Path k draws from the SHISHUA stream seeded
    {seed + k, stream, 0, 0}: give the requests of one batch or one server
    different stream numbers so that no two share a path's stream."""
    params: Params
    S0: float
    options: Options
    seed: int = 42
    stream: int = 0


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _u64p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


class Batch:
    """A batch planned and uploaded once (hexo_batch_prepare), launchable many times."""

    def __init__(self, engine: "Engine", handle: C.c_void_p, keep: list, outputs: list):
        self.engine = engine
        self.handle = handle
        self._keep = keep
        self.outputs = outputs  # [(price, stderr)] per request

    def launch(self):
        self.engine._check(L.load().hexo_batch_launch(self.handle))

    def collect(self):
        self.engine._check(L.load().hexo_batch_collect(self.handle))
        return self.outputs

    def collect_limbs(self) -> np.ndarray:
        """Waits for the last launch; its exact limb sums, [options of all requests, 6] uint64."""
        n = sum(len(p) for p, _ in self.outputs)
        limbs = np.zeros(n * L.HEXO_LIMBS, dtype=np.uint64)
        self.engine._check(L.load().hexo_batch_collect_limbs(self.handle, _u64p(limbs)))
        return limbs.reshape(n, L.HEXO_LIMBS)

    def info(self) -> dict:
        inf = L.hexo_batch_info()
        self.engine._check(L.load().hexo_batch_info_get(self.handle, C.byref(inf)))
        return {k: getattr(inf, k) for k, _ in L.hexo_batch_info._fields_}

    def close(self):
        if self.handle:
            L.load().hexo_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching server on an engine's context (hexo_server_*).

    ``submit`` queues a request and returns a ticket at once; ``wait`` blocks
    until that request is priced and returns its (price, stderr) arrays."""

    def __init__(self, engine: "Engine", cfg: Config, mem_cap_bytes: int = 0, max_batch_requests: int = 0,
                 max_inflight: int = 0, launch_path_steps: int = 0):
        self.engine = engine
        self._lib = engine._lib
        opts = L.hexo_server_opts(cfg.c(), mem_cap_bytes, max_batch_requests, max_inflight, launch_path_steps)
        self.handle = C.c_void_p()
        engine._check(self._lib.hexo_server_create(engine._ctx, C.byref(opts), C.byref(self.handle)))
        self._pending = {}   # ticket -> (keep-alive objects, outputs)

    def prepare(self, rq: Request):
        """Marshals a request ahead of time; pass the result to submit_prepared."""
        return self.engine._requests([rq])

    def submit(self, rq: Request) -> int:
        return self.submit_prepared(self.prepare(rq))

    def submit_prepared(self, prepared) -> int:
        arr, keep, outputs = prepared
        t = C.c_uint64()
        st = self._lib.hexo_server_submit(self.handle, arr, C.byref(t))
        if st != L.HEXO_OK:
            raise L.HexoError(st, "hexo_server_submit failed")
        self._pending[t.value] = (keep, outputs[0])
        return t.value

    def poll(self, ticket: int) -> bool:
        done = C.c_int()
        st = self._lib.hexo_server_poll(self.handle, ticket, C.byref(done))
        if done.value:
            self._finish(ticket, st)
        elif st != L.HEXO_OK:
            raise L.HexoError(st, "hexo_server_poll failed")
        return bool(done.value)

    def wait(self, ticket: int, timeout_ms: int = 600_000):
        st = self._lib.hexo_server_wait(self.handle, ticket, timeout_ms)
        return self._finish(ticket, st)

    def _finish(self, ticket: int, st: int):
        if st == L.HEXO_ERR_TIMEOUT:
            raise L.HexoError(st, "request still running")
        keep, out = self._pending.pop(ticket, (None, None))
        if st != L.HEXO_OK:
            raise L.HexoError(st, "request failed")
        return out

    def stats(self) -> dict:
        s = L.hexo_server_stats()
        self.engine._check(self._lib.hexo_server_stats_get(self.handle, C.byref(s)))
        return {k: getattr(s, k) for k, _ in L.hexo_server_stats._fields_}

    def close(self):
        if self.handle:
            self._lib.hexo_server_destroy(self.handle)
            self.handle = None
            self._pending.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Calibration:
    """The reference's calibration objective on the GPU (hexo_calib_*):
    ``prices(p)`` and ``jacobian(p)`` for p = (v0, vm, rho, kappa, sigma), as
    its Levenberg-Marquardt callbacks compute them."""

    def __init__(self, engine: "Engine", S: float, r: float, chains, trunc_precision: float = 0.0):
        self.engine = engine
        self._lib = engine._lib
        taus = np.ascontiguousarray([t for t, _ in chains], dtype=np.float64)
        counts = np.ascontiguousarray([len(k) for _, k in chains], dtype=np.uint32)
        strikes = np.ascontiguousarray(np.concatenate([np.asarray(k, dtype=np.float64) for _, k in chains]))
        self.n = int(counts.sum())
        self.handle = C.c_void_p()
        engine._check(self._lib.hexo_calib_create(engine._ctx, float(S), float(r), _dp(taus),
                                                  counts.ctypes.data_as(C.POINTER(C.c_uint32)), _dp(strikes),
                                                  len(counts), float(trunc_precision), C.byref(self.handle)))

    def prices(self, p) -> np.ndarray:
        p = np.ascontiguousarray(p, dtype=np.float64)
        x = np.zeros(self.n)
        self.engine._check(self._lib.hexo_calib_prices(self.handle, _dp(p), _dp(x)))
        return x

    def jacobian(self, p) -> np.ndarray:
        p = np.ascontiguousarray(p, dtype=np.float64)
        j = np.zeros((self.n, 5))
        self.engine._check(self._lib.hexo_calib_jacobian(self.handle, _dp(p), _dp(j)))
        return j

    def close(self):
        if self.handle:
            self._lib.hexo_calib_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Engine:
    def __init__(self, device: int = 0, mem_cap_bytes: int = 0, autotune_cache: str | None = None):
        lib = L.load()
        self._lib = lib
        self._ctx = C.c_void_p()
        opts = L.hexo_ctx_opts(device, mem_cap_bytes, autotune_cache.encode() if autotune_cache else None, 0)
        st = lib.hexo_ctx_create(C.byref(self._ctx), C.byref(opts))
        if st != L.HEXO_OK:
            raise L.HexoError(st, "hexo_ctx_create failed")

    # ------------------------------------------------------------ plumbing
    def _check(self, st: int):
        if st != L.HEXO_OK:
            buf = C.create_string_buffer(512)
            self._lib.hexo_ctx_last_error(self._ctx, buf, 512)
            raise L.HexoError(st, buf.value.decode(errors="replace"))

    def close(self):
        if self._ctx:
            self._lib.hexo_ctx_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def trim(self):
        """Frees the device and pinned memory the context keeps between one-shot calls."""
        self._check(self._lib.hexo_ctx_trim(self._ctx))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return self._lib.hexo_ctx_stream(self._ctx) or 0

    # ------------------------------------------------------------- pricing
    def price(self, params: Params, S0: float, options: Options, cfg: Config):
        n = len(options)
        price = np.zeros(n)
        se = np.zeros(n)
        opts = options.c_array()
        c = cfg.c()
        p = params.c()
        self._check(self._lib.hexo_price(self._ctx, C.byref(p), float(S0), opts, n, C.byref(c), _dp(price), _dp(se)))
        return price, se

    def _requests(self, requests: Sequence[Request]):
        arr = (L.hexo_request * len(requests))()
        keep, outputs = [], []
        for i, rq in enumerate(requests):
            n = len(rq.options)
            opts = rq.options.c_array()
            price = np.zeros(n)
            se = np.zeros(n)
            keep += [opts, price, se]
            outputs.append((price, se))
            arr[i].params = rq.params.c()
            arr[i].S0 = float(rq.S0)
            arr[i].opts = C.cast(opts, C.POINTER(L.hexo_option))
            arr[i].n_opts = n
            arr[i].seed = int(rq.seed) & 0xFFFFFFFF
            arr[i].stream = int(rq.stream) & 0xFFFFFFFF
            arr[i].price_out = _dp(price)
            arr[i].stderr_out = _dp(se)
        keep.append(arr)
        return arr, keep, outputs

    def price_batch(self, requests: Sequence[Request], cfg: Config):
        arr, keep, outputs = self._requests(requests)
        c = cfg.c()
        self._check(self._lib.hexo_price_batch(self._ctx, arr, len(requests), C.byref(c)))
        return outputs

    def prepare_batch(self, requests: Sequence[Request], cfg: Config) -> Batch:
        arr, keep, outputs = self._requests(requests)
        c = cfg.c()
        keep.append(c)
        h = C.c_void_p()
        self._check(self._lib.hexo_batch_prepare(self._ctx, arr, len(requests), C.byref(c), C.byref(h)))
        return Batch(self, h, keep, outputs)

    def batch_partial(self, requests: Sequence[Request], cfg: Config, shard: int, n_shards: int) -> np.ndarray:
        """Shard `shard` of n_shards of a batch (range `shard` of every request's
        paths) in one launch: limb sums [options of all requests, 6] uint64."""
        arr, keep, outputs = self._requests(requests)
        n = sum(len(rq.options) for rq in requests)
        limbs = np.zeros(n * L.HEXO_LIMBS, dtype=np.uint64)
        c = cfg.c()
        self._check(self._lib.hexo_price_batch_partial(self._ctx, arr, len(requests), C.byref(c), int(shard),
                                                       int(n_shards), _u64p(limbs)))
        return limbs.reshape(n, L.HEXO_LIMBS)

    def prepare_batch_partial(self, requests: Sequence[Request], cfg: Config, shard: int, n_shards: int) -> Batch:
        """The same shard as a captured graph; launch, then collect_limbs()."""
        arr, keep, outputs = self._requests(requests)
        c = cfg.c()
        keep.append(c)
        h = C.c_void_p()
        self._check(self._lib.hexo_batch_prepare_partial(self._ctx, arr, len(requests), C.byref(c), int(shard),
                                                         int(n_shards), C.byref(h)))
        return Batch(self, h, keep, outputs)

    def server(self, cfg: Config, **kw) -> Server:
        return Server(self, cfg, **kw)

    def calibration(self, S: float, r: float, chains, trunc_precision: float = 0.0) -> Calibration:
        return Calibration(self, S, r, chains, trunc_precision)

    def swift(self, params: Params, S: float, chains, grad: bool = False, swift_params=None,
              trunc_precision: float = 0.0, method: int = 0):
        """SWIFT European call prices (and gradients in v0, theta, rho, kappa,
        sigma) for chains [(tau, strikes), ...]; swift_params: per chain a
        dict / 8-sequence of the reference's SwiftParameters, or None for the
        reference's dynamic choice; method: 0 automatic, 1 direct sums, 2 FFT.
        Returns [price] or [(price, grad[n, 5])]."""
        return self.swift_batch([(params, S, chains)], grad, None if swift_params is None else [swift_params],
                                trunc_precision, method)[0]

    def swift_batch(self, requests, grad: bool = False, swift_params=None, trunc_precision: float = 0.0,
                    method: int = 0):
        """requests: [(Params, S, [(tau, strikes), ...]), ...], priced in one call."""
        reqs = (L.hexo_swift_request * len(requests))()
        keep, outs = [], []
        for q, (params, S, chains) in enumerate(requests):
            arr = (L.hexo_swift_chain * max(1, len(chains)))()
            res = []
            for c, (tau, K) in enumerate(chains):
                K = np.ascontiguousarray(K, dtype=np.float64)
                price = np.zeros(len(K))
                g = np.zeros((len(K), 5)) if grad else None
                arr[c].tau = float(tau)
                arr[c].strikes = _dp(K)
                arr[c].n = len(K)
                sp = swift_params[q][c] if swift_params is not None and swift_params[q] is not None else None
                if sp is not None:
                    v = list(sp.values()) if isinstance(sp, dict) else list(sp)
                    spc = L.hexo_swift_params(int(v[0]), int(v[1]), float(v[2]), float(v[3]), float(v[4]),
                                              int(v[5]), int(v[6]), int(v[7]), 0)
                    keep.append(spc)
                    arr[c].params = C.pointer(spc)
                arr[c].trunc_precision = trunc_precision
                arr[c].method = int(method)
                arr[c].price_out = _dp(price)
                arr[c].grad_out = _dp(g) if grad else None
                keep += [K, price, g]
                res.append((price, g) if grad else price)
            keep.append(arr)
            reqs[q].params = params.c()
            reqs[q].S = float(S)
            reqs[q].chains = C.cast(arr, C.POINTER(L.hexo_swift_chain))
            reqs[q].n_chains = len(chains)
            outs.append(res)
        self._check(self._lib.hexo_swift_price(self._ctx, reqs, len(requests)))
        return outs

    def partial(self, params: Params, S0: float, options: Options, cfg: Config, path_lo: int, path_hi: int):
        n = len(options)
        limbs = np.zeros(n * L.HEXO_LIMBS, dtype=np.uint64)
        opts = options.c_array()
        c = cfg.c()
        p = params.c()
        self._check(self._lib.hexo_price_partial(self._ctx, C.byref(p), float(S0), opts, n, C.byref(c),
                                                 int(path_lo), int(path_hi), _u64p(limbs)))
        return limbs.reshape(n, L.HEXO_LIMBS)

    def autotune(self, requests: Sequence[Request], cfg: Config):
        arr, keep, outputs = self._requests(requests)
        c = cfg.c()
        res = L.hexo_tune_result()
        entries = (L.hexo_tune_entry * 45)()
        self._check(self._lib.hexo_autotune(self._ctx, arr, len(requests), C.byref(c), C.byref(res), entries, 45))
        table = [(entries[i].block, entries[i].paths_per_thread, entries[i].unroll, entries[i].ms)
                 for i in range(res.n_tried)]
        return {"block": res.block, "paths_per_thread": res.paths_per_thread, "unroll": res.unroll,
                "best_ms": res.best_ms, "table": table}

    # --------------------------------------------------------------- debug
    def rng_words(self, seed: int, n_streams: int, n_words: int, stream: int = 0) -> np.ndarray:
        out = np.zeros(n_streams * n_words, dtype=np.uint64)
        self._check(self._lib.hexo_debug_rng_words(self._ctx, seed & 0xFFFFFFFF, stream & 0xFFFFFFFF, n_streams,
                                                   n_words, _u64p(out)))
        return out.reshape(n_streams, n_words)

    def rng_draws(self, seed: int, n_streams: int, kinds: np.ndarray, stream: int = 0) -> np.ndarray:
        kinds = np.ascontiguousarray(kinds, dtype=np.uint8)
        out = np.zeros(n_streams * len(kinds))
        self._check(self._lib.hexo_debug_rng_draws(self._ctx, seed & 0xFFFFFFFF, stream & 0xFFFFFFFF, n_streams,
                                                   kinds.ctypes.data_as(C.POINTER(C.c_uint8)), len(kinds), _dp(out)))
        return out.reshape(n_streams, len(kinds))

    def normals(self, words: np.ndarray) -> np.ndarray:
        words = np.ascontiguousarray(words, dtype=np.uint64)
        out = np.zeros(len(words))
        self._check(self._lib.hexo_debug_normals(self._ctx, _u64p(words), len(words), _dp(out)))
        return out

    def as241_check(self, branch: int, bits_lo: int, bits_hi: int) -> tuple[int, int]:
        """Float bit patterns in [bits_lo, bits_hi) through AS241's central branch (0) or tail (1) with the
        kernels' division and root and with the IEEE intrinsics, or (2) raw words with high words in
        [bits_lo, bits_hi) through the 32-bit input stage and the exact one: (number of disagreements,
        smallest disagreeing b or 2^64 - 1)."""
        out = np.zeros(2, dtype=np.uint64)
        self._check(self._lib.hexo_debug_as241_check(self._ctx, branch, bits_lo, bits_hi, _u64p(out)))
        return int(out[0]), int(out[1])

    def payoff_limbs(self, pay: np.ndarray, precision: int, S0: float = 100.0) -> np.ndarray:
        """The kernels' 25-bit limbs of round(y 2^47) and round(y^2 2^43), y = pay 2^-E with
        2^(E-1) <= S0 < 2^E, [n, 6]."""
        pay = np.ascontiguousarray(pay, dtype=np.float64)
        out = np.zeros(len(pay) * 6, dtype=np.uint32)
        self._check(self._lib.hexo_debug_payoff_limbs(self._ctx, _dp(pay), len(pay), precision, float(S0),
                                                      out.ctypes.data_as(C.POINTER(C.c_uint32))))
        return out.reshape(len(pay), 6)

    def pipe_peaks(self) -> dict:
        out = np.zeros(5)
        self._check(self._lib.hexo_debug_pipe_peaks(self._ctx, _dp(out)))
        return {"fp32_fma": out[0], "fp64_fma": out[1], "mufu": out[2], "int32": out[3], "int32_alu": out[4]}

    def path_finals(self, params: Params, S0: float, options: Options, cfg: Config, path_lo: int, path_hi: int):
        n = path_hi - path_lo
        m_max = len(np.unique(options.T))
        a = np.zeros(n * m_max)
        e = np.zeros(n * m_max)
        nm = C.c_uint32()
        opts = options.c_array()
        c = cfg.c()
        p = params.c()
        self._check(self._lib.hexo_debug_path_finals(self._ctx, C.byref(p), float(S0), opts, len(options),
                                                     C.byref(c), path_lo, path_hi, _dp(a), _dp(e), C.byref(nm)))
        m = nm.value
        return a[: n * m].reshape(n, m), e[: n * m].reshape(n, m)


def swift_params_dynamic(params: Params, tau: float, S: float, K_min: float, K_max: float,
                         trunc_precision: float = 1e-7) -> dict:
    """Host-only: the reference's dynamic SWIFT parameters for one expiry (SWIFT.cpp:21-35)."""
    out = L.hexo_swift_params()
    p = params.c()
    st = L.load().hexo_swift_params_dynamic(C.byref(p), tau, S, K_min, K_max, trunc_precision, C.byref(out))
    if st != L.HEXO_OK:
        raise L.HexoError(st, "hexo_swift_params_dynamic")
    return {k: getattr(out, k) for k in ("m", "exp2_m", "sqrt_exp2_m", "lower", "upper", "k1", "k2", "J")}


def finalize_limbs(params: Params, S0: float, options: Options, cfg: Config, limbs: np.ndarray):
    """Host-only finalisation of (merged) limb sums of a request with spot S0;
    bit-identical to the device finaliser."""
    lib = L.load()
    n = len(options)
    limbs = np.ascontiguousarray(limbs, dtype=np.uint64).reshape(-1)
    price = np.zeros(n)
    se = np.zeros(n)
    p = params.c()
    c = cfg.c()
    st = lib.hexo_finalize_limbs(C.byref(p), float(S0), options.c_array(), n, C.byref(c), _u64p(limbs), _dp(price),
                                 _dp(se))
    if st != L.HEXO_OK:
        raise L.HexoError(st, "hexo_finalize_limbs")
    return price, se
