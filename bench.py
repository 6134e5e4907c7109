#!/usr/bin/env python3
"""Benchmark of the Heston Monte Carlo engine (one JSON line on rank 0).

Workload (one step): the uneven batch, 64 parameter sets (seed 2), chains of
10-400 options with maturities U[0.02, 5] y on the daily grid, paths per
distinct maturity log-uniform in [2^14, 2^22], Asian:European 3:1, priced in
the batched FP32 form by one persistent kernel launched through a captured
CUDA graph.  Synthetic data (the reference prices live Tradier chains).

  value      nominal path-steps/s of the graph launches, inputs resident on
             the device, CUDA events on the engine's stream, L2 flushed
             between timed launches
  e2e        the same metric through hexo_price_batch with host buffers
             (planning, upload, run and result download inside the timing)
  fp64_plain the plain FP64 form, one request per launch, on every set at
             full paths: device-timed and end to end, the FP32 form's
             speed-up over it and its error against it (the last key)
  roofline   the path kernel's algorithmic operations per second on the pipe
             that binds (FP32 FMA, MUFU or integer ALU, each against this
             GPU's lane rate measured in the run), with the branch mix p_Q
             the kernel counted
  serving    Poisson request streams (50-2000 req/s, at least 1,000
             requests each) through the continuous-batching server (FP32),
             p50/p99 submit-to-completion latency, against the first requests
             of each stream priced one per plain FP64 launch
  cpu_baseline / --impl reference
             the oracle port of the reference's CPU path (OpenMP over all
             host cores) on the same bounded sample in both arms: all 64 sets
             at 1/256 of their paths, its work counted by the oracle

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]
  python bench.py --precision-sweep | --swift | --configs | --autotune [--path-scale S]   (reports, not the benchmark)
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

METRIC = "Heston path-steps/s, 1 GB300: batched FP32 vs plain FP64 at ≤1e-4 rel; p99 ms"
UNIT = "path-steps/s"
WORKLOAD = "uneven_batch_64sets_fp32_graph"

# Algorithmic operations per path-step of the scheme, by the pipe that
# executes them in the FP32 form, counted in the reference's operation order
# (HSimulation.tpp:52-86, as241.f90, RNG.cpp) with p = the measured share of
# quadratic-branch steps, n_N = 1 + p normals and 1 - p uniforms per step,
# and c = 0.85 the share of AS241 draws on its central branch:
#   FP32 FMA pipe: QE 3 (m) + 2 (s^2) + 1 (m^2) + 7 p (quadratic branch)
#     + 5 (1 - p) (exponential branch) + 9 (log-spot) + 1 (time) + 3 (Asian)
#     = 24 + 2 p; AS241 5 + 31 = 36 per normal;
#   MUFU (XU): divides 5 - 2 p (QE) + n_N (AS241); square roots 1 + 2 p
#     + n_N (1 - c); exp 1, log 1 - p + n_N (1 - c); 2 word conversions;
#   INT ALU: SHISHUA, 122 shift/logic/add operations per 16-word block,
#     2 words per step.
AS241_CENTRAL = 0.85
SHISHUA_ALU_PER_WORD = 122.0 / 16.0


def alg_ops_per_path_step(p: float) -> dict:
    n_n = 1.0 + p
    tail = n_n * (1.0 - AS241_CENTRAL)
    return {"fp32_fma": 24.0 + 2.0 * p + 36.0 * n_n,
            "mufu": (5.0 - 2.0 * p + n_n) + (1.0 + 2.0 * p + tail) + 1.0 + (1.0 - p + tail) + 2.0,
            "int32_alu": 2.0 * SHISHUA_ALU_PER_WORD}

# DRAM bytes (read + write) of one launch of the FP32 path kernel on this
# workload, from a one-pass Nsight Compute capture of the full batch (30.83 MB
# read, 0 written, 5.41 s): the 16 private copies of the payoff sums
# (11.1 MB) and the descriptors the launch reads (19.7 MB, most of them the
# 1.0M tiles), against 19.9 MB of algorithmic bytes (descriptors and results).
PATHS_KERNEL_DRAM_BYTES = 30.83e6
PATHS_KERNEL_DRAM_NOTE = ("DRAM bytes per launch of the full batch, one-pass ncu capture: the 16 private copies "
                          "of the sums and the descriptors; algorithmic bytes 19.9 MB")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.path = Path(tempfile.mkstemp(prefix="clocks", suffix=".csv")[1])
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def plan_stats(reqs, cfg):
    import ctypes as C
    from hestonexotics_gb300 import _lib as L
    from hestonexotics_gb300.engine import Engine
    arr, keep, _ = Engine._requests(None, reqs)
    c = cfg.c()
    st = L.hexo_plan_stats()
    rc = L.load().hexo_plan_stats_get(arr, len(reqs), C.byref(c), C.byref(st))
    if rc != 0:
        raise RuntimeError(f"hexo_plan_stats_get failed: {rc}")
    return st


# ------------------------------------------------------------ CPU baseline

CPU_PATH_SCALE = 1 / 256


def workload_config():
    """The workload both arms name: the same dict in the engine line and in
    the reference line."""
    from hestonexotics_gb300 import workloads as W
    from oracle import oracle as O
    reqs, _ = W.uneven_batch(seed=2)
    return {"workload": WORKLOAD, "sets": len(reqs), "seed": 2,
            "options": int(sum(len(r.options) for r in reqs)),
            "nominal_path_steps": int(sum(O.nominal_path_steps(r.options.T, r.options.n_paths) for r in reqs)),
            "paths": "2^14-2^22 per distinct maturity, log-uniform", "step_mode": "grid 252/y",
            "payoffs": "Asian:European 3:1"}


def cpu_sample(rank: int):
    """A bounded sample of the workload for the CPU: all 64 sets, every path
    count scaled by 1/256 (same parameter sets, maturities, strikes, step
    schedules and branch mix; 1.16e9 nominal path-steps, a few seconds on a
    few dozen cores).  Its work is counted by the oracle's own walk of the
    time grid, so the CPU legs load no engine code."""
    from hestonexotics_gb300 import workloads as W
    from oracle import oracle as O
    reqs, cfg = W.uneven_batch(seed=2 + rank, path_scale=CPU_PATH_SCALE)
    nominal = sum(O.nominal_path_steps(r.options.T, r.options.n_paths, step_mode=cfg.step_mode, steps=cfg.steps,
                                       steps_per_year=cfg.steps_per_year) for r in reqs)
    return reqs, cfg, nominal


def cpu_sample_step(O, reqs, cfg, threads):
    t0 = time.perf_counter()
    for rq in reqs:
        _oracle_price_fast(O, rq, cfg, threads)
    return time.perf_counter() - t0


def run_cpu_baseline(rank: int, steps: int = 3):
    from oracle import oracle as O
    O.build()
    reqs, cfg, nominal = cpu_sample(rank)
    threads = os.cpu_count() or 1
    cpu_sample_step(O, reqs[:4], cfg, threads)      # warm-up: page in, spin up the thread pool
    times = [cpu_sample_step(O, reqs, cfg, threads) for _ in range(max(1, steps))]
    t = statistics.median(times)
    return {"value": nominal / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"all 64 sets with every path count x{CPU_PATH_SCALE:g} ({nominal:.3e} nominal path-steps, "
                      f"counted by the oracle), oracle port of the reference loop (-O3 -ffast-math, OpenMP "
                      f"{threads} threads), median of {len(times)}", "seconds": t, "nominal_path_steps": nominal}


def _oracle_price_fast(O, rq, cfg, threads):
    o = rq.options
    return O.price_paths(rq.params.as_array(), rq.S0, o.strike, o.T, o.payoff.astype(np.uint8), o.n_paths,
                         n_default=cfg.n_paths, step_mode=cfg.step_mode, steps=cfg.steps,
                         steps_per_year=cfg.steps_per_year, seed=rq.seed, stream=rq.stream, threads=threads,
                         fast=True)


# -------------------------------------------------------------- serving

def _pct(xs, q):
    return float(np.percentile(np.asarray(xs), q)) if xs else None


def run_serving(eng, rates, min_requests, min_seconds, fp64_requests):
    """Open-loop Poisson request streams (workloads.request_stream, seed 3)
    against the continuous-batching server (FP32 form), each rate run for at
    least min_seconds and min_requests arrivals, and the first fp64_requests
    arrivals of the same stream priced one request per plain FP64 launch,
    first come first served.  Latency is submit (arrival) to completion."""
    from hestonexotics_gb300 import FP64
    from hestonexotics_gb300 import workloads as W
    out = []
    for rate in rates:
        duration = max(min_seconds, min_requests / rate)
        arrivals, cfg = W.request_stream(rate, duration, seed=3)
        row = {"rate": rate, "requests": len(arrivals), "seconds": round(duration, 2)}
        srv = eng.server(cfg, max_batch_requests=64, max_inflight=3)
        prepared = [srv.prepare(a.request) for a in arrivals]
        tickets = []
        t0 = time.perf_counter()
        for a, pr in zip(arrivals, prepared):
            d = t0 + a.t - time.perf_counter()
            if d > 0:
                time.sleep(d)
            tickets.append(srv.submit_prepared(pr))
        ok = 0
        for t in tickets:
            try:
                srv.wait(t)
                ok += 1
            except Exception:
                pass
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        row["fp32"] = {"p50_ms": round(st["p50_ms"], 2), "p99_ms": round(st["p99_ms"], 2),
                       "mean_ms": round(st["mean_ms"], 2), "completed": ok, "launches": st["batches"],
                       "queued_max": st["queued_max"], "mem_peak_mb": round(st["mem_peak"] / 2 ** 20, 1),
                       "path_steps_per_s": st["nominal_path_steps"] / wall}
        if fp64_requests:
            cfg64 = type(cfg)(**{**cfg.__dict__, "precision": FP64})
            lat = []
            sub = arrivals[:fp64_requests]
            t0 = time.perf_counter()
            for a in sub:
                d = t0 + a.t - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                eng.price_batch([a.request], cfg64)
                lat.append((time.perf_counter() - (t0 + a.t)) * 1e3)
            row["fp64_one_per_launch"] = {"p50_ms": round(_pct(lat, 50), 2), "p99_ms": round(_pct(lat, 99), 2),
                                          "completed": len(lat)}
        out.append(row)
    return out


# ------------------------------------------------------- plain FP64 form

def run_fp64_plain(eng, reqs, cfg64, fp32_outputs, flush, stream):
    """The plain FP64 form on every set of the batch, one request per launch:
    device time of each request's graph launch with CUDA events on the
    engine's stream (L2 flushed before each), and end to end per request
    through the public calls with host buffers (hexo_batch_prepare: planning
    and upload; hexo_batch_launch; hexo_batch_collect: the download).  The
    FP32 prices of the timed batch are checked against these FP64 prices on
    the same streams."""
    import torch
    dev_ms, e2e_s, nominal = 0.0, 0.0, 0
    rel, n_big, in_se, n_opts = 0.0, 0, 0, 0
    for rq, (p32, se32) in zip(reqs, fp32_outputs):
        t0 = time.perf_counter()
        b = eng.prepare_batch([rq], cfg64)
        with torch.cuda.stream(stream):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        t1 = time.perf_counter()
        b.launch()
        with torch.cuda.stream(stream):
            e1.record(stream)
        (p64, _), = b.collect()
        t2 = time.perf_counter()
        nominal += b.info()["nominal_path_steps"]
        b.close()
        e2e_s += (t1 - t0) + (t2 - t1)
        dev_ms += e0.elapsed_time(e1)
        big = p64 > 1e-3 * rq.S0
        if big.any():
            rel = max(rel, float(np.max(np.abs(p32[big] - p64[big]) / p64[big])))
        n_big += int(big.sum())
        in_se += int(np.sum(np.abs(p32 - p64) <= np.maximum(se32, 1e-9 * rq.S0)))
        n_opts += len(p64)
    return {"value": nominal / (dev_ms * 1e-3), "e2e": nominal / e2e_s, "sets": len(reqs),
            "nominal_path_steps": nominal, "device_s": dev_ms * 1e-3, "e2e_s": e2e_s,
            "fp32_vs_fp64_max_rel_err": rel, "prices_checked": n_big, "fp32_within_1se_frac": in_se / max(1, n_opts)}


# ------------------------------------------------------ precision sweep

def run_precision_sweep(eng, counts):
    """The single-chain batch (8 maturities x 50 strikes x Asian/European,
    seed 1) and the Feller-violating set, FP32 form against the FP64 form on
    the same streams (the FP64 form matches the oracle to 1e-10), at each
    path count: worst relative error over prices above 1e-3 S0, worst
    |error| / standard error, and the median standard error / price."""
    from hestonexotics_gb300 import FP32, FP64
    from hestonexotics_gb300 import workloads as W
    out = []
    for name, make in (("single_chain_seed1", W.single_chain), ("feller_violating", W.feller_violating)):
        for n in counts:
            rq, cfg64 = make(n_paths=n, precision=FP64)
            _, cfg32 = make(n_paths=n, precision=FP32)
            t0 = time.perf_counter()
            p64, se64 = eng.price(rq.params, rq.S0, rq.options, cfg64)
            t64 = time.perf_counter() - t0
            t0 = time.perf_counter()
            p32, se32 = eng.price(rq.params, rq.S0, rq.options, cfg32)
            t32 = time.perf_counter() - t0
            big = p64 > 1e-3 * rq.S0
            rel = np.abs(p32 - p64)[big] / p64[big]
            z = np.abs(p32 - p64) / np.maximum(se64, 1e-300)
            out.append({"set": name, "paths": n, "options": len(p64), "max_rel_err": float(rel.max()),
                        "median_rel_err": float(np.median(rel)), "max_err_over_se": float(z.max()),
                        "within_1se_frac": float(np.mean(z <= 1.0)),
                        "median_se_over_price": float(np.median(se64[big] / p64[big])),
                        "fp64_s": t64, "fp32_s": t32})
    return out


# ------------------------------------------------------- single requests

def run_configs_report(eng):
    """The two single-request configurations: the plain Asian (S0 = K = 100,
    T = 1, 252 reference steps, 65,536 paths, seed 42) and the single chain
    (seed 1, 8 maturities x 50 strikes x Asian/European, 2^20 paths, daily
    grid).  Per form: end-to-end path-steps/s of one hexo_price call (host
    buffers in and out, median of 5 after a warm-up) and the path kernel's
    own time; beside them the oracle port on all host cores with the same
    per-path streams (median of 5), and, for the plain Asian, the port of
    the reference's own thread partition (price()'s n / threads paths per
    thread from one RNG(2^20, 1 << tid) each, HSimulation.tpp:23-29)."""
    from oracle import oracle as O
    from hestonexotics_gb300 import FP32, FP64
    from hestonexotics_gb300 import workloads as W
    O.build()
    threads = os.cpu_count() or 1
    out = []
    for name, make in (("plain_asian_65536", lambda prec: W.plain_asian(n_paths=65536)),
                       ("single_chain_seed1_2^20", lambda prec: W.single_chain(n_paths=1 << 20, precision=prec))):
        row = {"config": name}
        for tag, prec in (("fp64", FP64), ("fp32", FP32)):
            rq, cfg = make(prec)
            cfg.precision = prec
            nominal = plan_stats([rq], cfg).nominal_path_steps
            eng.price(rq.params, rq.S0, rq.options, cfg)
            ts = []
            for _ in range(5):
                t0 = time.perf_counter()
                eng.price(rq.params, rq.S0, rq.options, cfg)
                ts.append(time.perf_counter() - t0)
            b = eng.prepare_batch([rq], cfg)
            kms = []
            for _ in range(4):
                b.launch()
                b.collect()
                kms.append(b.info()["last_kernel_ms"])
            b.close()
            row[tag] = {"e2e_path_steps_per_s": nominal / statistics.median(ts),
                        "e2e_ms": 1e3 * statistics.median(ts), "kernel_ms": min(kms[1:]),
                        "kernel_path_steps_per_s": nominal / (min(kms[1:]) * 1e-3)}
            # the geometric control variate on the Asian options: same paths, smaller error
            p_plain, se_plain = eng.price(rq.params, rq.S0, rq.options, cfg)
            cfg.control_variate = 1
            eng.price(rq.params, rq.S0, rq.options, cfg)
            ts = []
            for _ in range(3):
                t0 = time.perf_counter()
                p_cv, se_cv = eng.price(rq.params, rq.S0, rq.options, cfg)
                ts.append(time.perf_counter() - t0)
            cfg.control_variate = 0
            asian = (rq.options.payoff == 0) & (p_plain > 0.05)
            ratio = float(np.median(se_plain[asian] / se_cv[asian])) if asian.any() else None
            row[tag]["control_variate"] = {
                "e2e_ms": 1e3 * statistics.median(ts), "asian_options": int(asian.sum()),
                "median_se_ratio_plain_over_cv": ratio,
                "paths_for_equal_error": (1.0 / ratio ** 2) if ratio else None}
        rq, cfg = make(FP64)
        row["nominal_path_steps"] = nominal
        ts = []
        for _ in range(5):
            t0 = time.perf_counter()
            _oracle_price_fast(O, rq, cfg, threads)
            ts.append(time.perf_counter() - t0)
        row["cpu_port"] = {"path_steps_per_s": nominal / statistics.median(ts), "cores": threads,
                           "seconds": statistics.median(ts)}
        if name.startswith("plain_asian"):
            o = rq.options
            ts = []
            for _ in range(5):
                t0 = time.perf_counter()
                O.price_reference_partition(rq.params.as_array(), rq.S0, o.strike, o.T, o.payoff.astype(np.uint8),
                                            cfg.steps, cfg.n_paths, n_threads=threads, omp_threads=threads,
                                            fast=True)
                ts.append(time.perf_counter() - t0)
            row["cpu_reference_partition"] = {"path_steps_per_s": nominal / statistics.median(ts), "cores": threads,
                                              "seconds": statistics.median(ts)}
        out.append(row)
    return out


# ------------------------------------------------------------------ SWIFT

def run_swift_report(eng, n_sets=1024):
    """SWIFT European prices with gradients: the reference's calibration
    objective (8 chains x 5 strikes, the unit tests' chains, dynamic
    wavelet parameters) per evaluation on the GPU and in the oracle's CPU
    restatement (one thread, direct sums instead of FFTW), and a batch of
    parameter sets x 8 chains x 50 strikes."""
    import json as _json
    from hestonexotics_gb300 import engine as E
    from hestonexotics_gb300 import workloads as W
    from oracle import oracle as O
    g = _json.loads((ROOT / "tests" / "golden" / "swift_golden.json").read_text())
    chains = [(T, np.array(K)) for T, K in zip(g["expiries"], g["strikes"])]
    cal = eng.calibration(g["S"], g["r"], chains)
    p = np.array(g["params5"])
    for _ in range(3):
        cal.jacobian(p + 1e-9 * _)
    ts = []
    for k in range(50):
        q = p * (1.0 + 1e-6 * (k + 1))      # a new p each time: no cached evaluation
        t0 = time.perf_counter()
        cal.prices(q)
        cal.jacobian(q)
        ts.append(time.perf_counter() - t0)
    gpu_ms = 1e3 * statistics.median(ts)
    O.build()
    t0 = time.perf_counter()
    for T, K in chains:
        sp = O.swift_params(g["params5"], T, g["r"], g["S"], K.min(), K.max())
        O.swift_price(g["params5"], T, g["r"], g["S"], K, sp, grad=True)
    cpu_ms = 1e3 * (time.perf_counter() - t0)
    rng = np.random.default_rng(5)
    reqs = []
    for _ in range(n_sets):
        prm = W.draw_params(rng)
        reqs.append((prm, 100.0, [(T, np.geomspace(60.0, 160.0, 50)) for T in W.CHAIN_MATURITIES]))
    eng.swift_batch(reqs[:8], grad=True)
    t0 = time.perf_counter()
    eng.swift_batch(reqs, grad=True)
    tb = time.perf_counter() - t0
    n_opts = n_sets * len(W.CHAIN_MATURITIES) * 50
    # the two transforms by direct sums and by FFT at large J: one chain whose
    # range k2 - k1 fills the 4J the frequencies allow (m raised until it does)
    prm = W.draw_params(np.random.default_rng(6))
    K = np.geomspace(60.0, 160.0, 50)
    transforms = []
    for J in (1024, 8192, 65536):
        sp = E.swift_params_dynamic(prm, 1.0, 100.0, K.min(), K.max(), 1e-7)
        while 2 * (sp["k2"] - sp["k1"] + 1) <= 4 * J:   # finer wavelet scale: a wider k range
            sp["m"] += 1
            sp["exp2_m"] *= 2
            sp["sqrt_exp2_m"] = float(np.sqrt(sp["exp2_m"]))
            sp["k1"] = int(np.ceil(sp["exp2_m"] * sp["lower"]))
            sp["k2"] = int(np.floor(sp["exp2_m"] * sp["upper"]))
        if sp["k2"] - sp["k1"] + 1 > 4 * J:
            sp["m"] -= 1
            sp["exp2_m"] //= 2
            sp["sqrt_exp2_m"] = float(np.sqrt(sp["exp2_m"]))
            sp["k1"] = int(np.ceil(sp["exp2_m"] * sp["lower"]))
            sp["k2"] = int(np.floor(sp["exp2_m"] * sp["upper"]))
        sp["J"] = J
        row = {"J": J, "k_range": sp["k2"] - sp["k1"] + 1}
        for name, method in (("direct_ms", 1), ("fft_ms", 2)):
            eng.swift(prm, 100.0, [(1.0, K)], grad=True, swift_params=[sp], method=method)
            ts = []
            for _ in range(5):
                t0 = time.perf_counter()
                eng.swift(prm, 100.0, [(1.0, K)], grad=True, swift_params=[sp], method=method)
                ts.append(time.perf_counter() - t0)
            row[name] = 1e3 * statistics.median(ts)
        transforms.append(row)
    return {"calibration_eval": {"chains": 8, "observations": 40, "gpu_ms_prices_and_jacobian": gpu_ms,
                                 "oracle_cpu_ms_1_thread": cpu_ms,
                                 "oracle_note": "direct-sum restatement; the reference uses FFTW and Eigen"},
            "batch": {"sets": n_sets, "chains_per_set": len(W.CHAIN_MATURITIES), "strikes_per_chain": 50,
                      "seconds": tb, "options_per_s_with_gradients": n_opts / tb},
            "transforms_one_chain_50_strikes": transforms}


# -------------------------------------------------------------- engine arm

def run_engine(args, rank, world, local):
    import torch
    from hestonexotics_gb300 import FP32, FP64, Engine
    from hestonexotics_gb300 import workloads as W

    torch.cuda.set_device(local)
    if args.precision_sweep or args.autotune or args.swift or args.configs or args.fp64_only:
        eng = Engine(local)
        out = {"metric": METRIC, "unit": UNIT}
        if args.fp64_only:
            reqs, cfg = W.uneven_batch(seed=2, precision=FP64, path_scale=args.path_scale)
            stream = torch.cuda.ExternalStream(eng.stream)
            flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
            nan = [(np.full(len(r.options), np.nan), np.full(len(r.options), np.nan)) for r in reqs]
            r64 = run_fp64_plain(eng, reqs, cfg, nan, flush, stream)
            out["fp64_plain"] = {k: v for k, v in r64.items() if not k.startswith("fp32")}
            out["workload"] = f"{WORKLOAD}_paths_x{args.path_scale:g}"
        if args.precision_sweep:
            out["precision_sweep"] = run_precision_sweep(eng, [1 << k for k in (16, 18, 20, 22, 24)])
        if args.swift:
            out["swift"] = run_swift_report(eng)
        if args.configs:
            out["configs"] = run_configs_report(eng)
        if args.autotune:
            reqs, cfg = W.uneven_batch(seed=2, precision=FP32, path_scale=args.path_scale)
            out["autotune"] = {"workload": f"{WORKLOAD}_paths_x{args.path_scale:g}", **eng.autotune(reqs, cfg)}
            reqs, cfg = W.uneven_batch(seed=2, precision=FP64, path_scale=args.path_scale / 4)
            out["autotune_fp64"] = {"workload": f"uneven_batch_64sets_fp64_paths_x{args.path_scale / 4:g}",
                                    **eng.autotune(reqs, cfg)}
        eng.close()
        return out if rank == 0 else None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    eng = Engine(local)
    reqs, cfg = W.uneven_batch(seed=2, precision=FP32, path_scale=args.path_scale)
    # one GPU: the whole batch; N GPUs: range `rank` of every request's paths on each,
    # merged by one SUM all-reduce of the exact limb sums per step
    batch = eng.prepare_batch(reqs, cfg) if world == 1 else eng.prepare_batch_partial(reqs, cfg, rank, world)
    info = batch.info()
    nominal_batch = plan_stats(reqs, cfg).nominal_path_steps   # the whole batch, all ranks together
    stream = torch.cuda.ExternalStream(eng.stream)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    for _ in range(args.warmup):
        batch.launch()
        batch.collect()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    step_ms, kernel_ms = [], []
    merged = None
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()                      # L2 flush between timed launches (not timed)
            ev[k][0].record(stream)
        batch.launch()
        with torch.cuda.stream(stream):
            ev[k][1].record(stream)
        if world == 1:
            batch.collect()
            step_ms.append(ev[k][0].elapsed_time(ev[k][1]))
        else:                                  # the exchange: one SUM all-reduce of every request's limbs
            import torch.distributed as dist
            limbs = batch.collect_limbs()
            t0 = time.perf_counter()
            tl = torch.from_numpy(limbs.astype(np.int64)).to(f"cuda:{local}")
            dist.all_reduce(tl, op=dist.ReduceOp.SUM)
            merged = tl.cpu().numpy().astype(np.uint64)
            step_ms.append(ev[k][0].elapsed_time(ev[k][1]) + 1e3 * (time.perf_counter() - t0))
        last = batch.info()
        kernel_ms.append(last["last_kernel_ms"])
    p_quad = last["quad_steps"] / max(1, last["executed_path_steps"])   # branch mix the kernel counted
    barrier()
    clk = clocks.stop()
    total_ms = sum(step_ms)
    nominal = info["nominal_path_steps"]       # this rank's share
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([total_ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = nominal_batch * args.steps / (total_ms * 1e-3)
    if world == 1:
        fp32_outputs = [(p.copy(), s.copy()) for p, s in batch.outputs]
    else:
        from hestonexotics_gb300 import shard as S
        fp32_outputs = S.finalize_batch(reqs, cfg, merged)
    batch.close()

    # e2e: host buffers through the public call; N GPUs: the sharded batch
    # (planning, upload, one launch per rank, the limbs' all-reduce, the host finaliser)
    e2e_s = []
    for _ in range(max(1, min(args.steps, 2))):
        barrier()
        t0 = time.perf_counter()
        if world == 1:
            eng.price_batch(reqs, cfg)
        else:
            from hestonexotics_gb300 import shard as S
            S.price_batch_sharded(reqs, cfg, engine=eng)
        e2e_s.append(time.perf_counter() - t0)
    e2e_t = statistics.median(e2e_s)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_t], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_t = float(t.item())
    e2e_value = nominal_batch / e2e_t

    result = None
    if rank == 0:
        # the plain FP64 form on every set (or the first --fp64-sets), one request per launch
        cfg64 = type(cfg)(**{**cfg.__dict__, "precision": FP64})
        n64 = min(args.fp64_sets, len(reqs))
        fp64 = run_fp64_plain(eng, reqs[:n64], cfg64, fp32_outputs[:n64], flush, stream) if n64 else None

        peaks = eng.pipe_peaks()
        kms = statistics.mean(kernel_ms)
        # per pipe: the path-steps/s its measured peak allows; the smallest binds
        ops = alg_ops_per_path_step(p_quad)
        rate = nominal / (kms * 1e-3)
        pipes = {k: {"ops_per_path_step": round(ops[k], 2), "peak_lane_ops_per_s": peaks[k],
                     "bound_path_steps_per_s": peaks[k] / ops[k], "frac": rate / (peaks[k] / ops[k])}
                 for k in ops}
        bind = min(pipes, key=lambda k: pipes[k]["bound_path_steps_per_s"])
        achieved = ops[bind] * rate / 1e9
        peak = peaks[bind] / 1e9
        serving = None
        if args.serve_rates:
            rates = [float(x) for x in args.serve_rates.split(",") if x]
            serving = run_serving(eng, rates, args.serve_min_requests, args.serve_seconds, args.serve_fp64_requests)
        sweep = None
        if args.sweep_paths:   # the chain and the Feller-violating set, FP32 against FP64
            rows = run_precision_sweep(eng, [1 << int(x) for x in args.sweep_paths.split(",") if x])
            sweep = [{k: r[k] for k in ("set", "paths", "max_rel_err", "max_err_over_se", "within_1se_frac")}
                     for r in rows]
        cpu = run_cpu_baseline(rank, steps=args.cpu_baseline_steps) if args.cpu_baseline_steps > 0 else None
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f32 paths, f32 AS241, exact integer sums, f64 finalise",
            "data": "synthetic (seeded uneven 64-set batch; the reference prices live option chains)",
            "config": workload_config() if args.path_scale == 1.0 else
            {**workload_config(), "workload": f"{WORKLOAD}_paths_x{args.path_scale:g}",
             "nominal_path_steps": int(nominal_batch)},
            "launch": {"form": "FP32, one persistent launch of the whole batch through a captured CUDA graph",
                       "paths": info["n_paths"], "executed_path_steps": info["executed_path_steps"],
                       "tiles": info["n_tiles"], "block": info["block"], "paths_per_thread": info["paths_per_thread"],
                       "unroll": info["unroll"], "grid": info["grid"], "l2": "flushed between timed launches",
                       "parallelism": "one GPU" if world == 1 else
                       f"paths of every request split over {world} GPUs, one SUM all-reduce of the limbs per step"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": info["h2d_bytes"],
                    "d2h_bytes_per_step": info["d2h_bytes"],
                    "what": "hexo_price_batch with host buffers: planning, upload, run, download"},
            "roofline": {"bound": f"compute: {bind} pipe (no tensor-core or HBM bound on this path)",
                         "achieved": achieved, "peak": peak, "unit": f"Gop/s ({bind} lane ops)",
                         "frac": achieved / peak, "traffic": PATHS_KERNEL_DRAM_BYTES,
                         "traffic_note": PATHS_KERNEL_DRAM_NOTE,
                         "peak_source": "lane rates measured in this run by hexo_debug_pipe_peaks (of measured)",
                         "p_quadratic": p_quad, "as241_central_share": AS241_CENTRAL,
                         "pipes": pipes, "kernel_ms": kms},
            "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                           "what": "graph launch of the whole batch"},
            "serving": serving,
            "precision_sweep": sweep,
            "cpu_baseline": {k: v for k, v in cpu.items() if k != "nominal_path_steps"} if cpu else None,
            "clocks": clk,
            "gpu_launches": args.steps * 2,
            "fp64_plain": {"value": fp64["value"], "e2e": fp64["e2e"], "unit": UNIT, "sets": fp64["sets"],
                           "fp32_speedup": value / fp64["value"], "fp32_speedup_e2e": e2e_value / fp64["e2e"],
                           "fp32_vs_fp64_max_rel_err": fp64["fp32_vs_fp64_max_rel_err"],
                           "prices_checked": fp64["prices_checked"],
                           "fp32_within_1se_frac": fp64["fp32_within_1se_frac"],
                           "what": "one request per launch, full paths; value device-timed, e2e "
                                   "through hexo_batch_prepare/launch/collect"} if fp64 else None,
        }
    eng.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return result


def run_reference(args, rank, world):
    """The reference's CPU path (the oracle port; the reference itself is a
    C++ command-line program that cannot be installed as a package) on all
    host cores, each step the bounded sample of the workload that
    cpu_sample names; no engine code is loaded."""
    if rank != 0:
        return None
    from oracle import oracle as O
    O.build()
    reqs, cfg, nominal = cpu_sample(rank)
    threads = os.cpu_count() or 1
    for _ in range(max(0, args.warmup)):
        cpu_sample_step(O, reqs, cfg, threads)
    steps = [cpu_sample_step(O, reqs, cfg, threads) for _ in range(max(1, args.steps))]
    value = nominal * len(steps) / sum(steps)
    sample = (f"all 64 sets with every path count x{CPU_PATH_SCALE:g} ({nominal:.3e} nominal path-steps per step, "
              f"counted by the oracle), oracle port of the reference loop (-O3 -ffast-math, OpenMP {threads} threads)")
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(steps), "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f64 (reference CPU path)",
            "data": "synthetic (seeded uneven 64-set batch, bounded sample per step)",
            "config": workload_config(), "impl": "reference",
            "cpu_baseline": {"kind": "port", "cores": threads, "sample": sample, "value": value},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--serve-rates", default="50,200,500,1000,2000",
                    help="request rates of the serving leg ('' = skip)")
    ap.add_argument("--serve-min-requests", type=int, default=1000,
                    help="each rate runs until at least this many requests have arrived")
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="and for at least this long")
    ap.add_argument("--serve-fp64-requests", type=int, default=300,
                    help="the first requests of each stream also priced one per plain FP64 launch (0 = skip)")
    ap.add_argument("--precision-sweep", action="store_true",
                    help="instead of the benchmark: FP32 vs FP64 errors on the single chain at 2^16..2^24 paths")
    ap.add_argument("--swift", action="store_true",
                    help="instead of the benchmark: SWIFT pricer and calibration-callback timings")
    ap.add_argument("--configs", action="store_true",
                    help="instead of the benchmark: the plain Asian and the single chain as single requests, "
                         "GPU both forms against the CPU port")
    ap.add_argument("--autotune", action="store_true",
                    help="instead of the benchmark: the launch-shape sweep on the uneven batch (use --path-scale)")
    ap.add_argument("--fp64-only", action="store_true",
                    help="instead of the benchmark: the plain FP64 leg alone (every set, one request per launch)")
    ap.add_argument("--cpu-baseline-steps", type=int, default=3,
                    help="timed steps of the CPU baseline leg (median; 0 = skip)")
    ap.add_argument("--fp64-sets", type=int, default=64,
                    help="sets of the plain FP64 leg (the first ones; 64 = all, 0 = skip)")
    ap.add_argument("--sweep-paths", default="16,20,24",
                    help="log2 path counts of the precision sweep in the benchmark line ('' = skip)")
    ap.add_argument("--path-scale", type=float, default=1.0,
                    help="scales every path count of the batch (1.0 = the benchmark workload; smaller for profiling)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        out = run_engine(args, rank, world, local)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
