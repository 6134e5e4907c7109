"""Generates tests/golden/*.json from the reference's own sources.

Runs only where the reference checkout exists: it builds
oracle/_ref/libhexo_ref.so (the reference's src/RNG.cpp and the
HSimulation/contract templates, compiled unmodified, plus the project's
SHISHUA and AS241 restatement; see oracle/Makefile) and records

  rng_draws.json      draws of the reference RNG class, RNG(size, seed),
                      for fixed draw-kind sequences
  ref_price.json      the untouched HSimulation::price<HQEAnderson<...>> on one
                      OpenMP thread (the reference's own stream partition)
  ref_paths.json      per-path payoffs through the reference's HQEAnderson and
                      contract classes with one RNG(16, seed + k) per path
  swift_golden.json   the SWIFT known answers of the reference's unit tests,
                      read as text from src/UnitTest.cpp: inputs (:155-181),
                      the 40 prices of pricing_test (:221-261) and the 200
                      gradient entries of gradient_test (:278-478) with its
                      component map (:479)

Floats are stored as float.hex() strings so the fixtures are bit-exact.
Usage:  OMP_NUM_THREADS=1 python tests/golden/make_golden.py [swift]
"""
from __future__ import annotations

import ctypes as C
import json
import os
import re
import subprocess
import sys
from pathlib import Path

import numpy as np

os.environ["OMP_NUM_THREADS"] = "1"
HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
from hestonexotics_gb300.build import reference_src  # noqa: E402

REF = reference_src()   # HEXO_REFERENCE_SRC, or the checkout beside the repository


def P(a):
    return C.c_void_p(a.ctypes.data)


def hexlist(a):
    return [float(x).hex() for x in np.asarray(a, dtype=np.float64).ravel()]


C0 = dict(params5=[0.04, 0.04, -0.7, 1.5, 0.5], S=100.0)
CASES = [
    # name, chain maturities, strikes per chain, steps, n_sims
    ("c0_asian_atm", [1.0], [[100.0]], 252, 4096),
    ("three_chains", [0.25, 0.5, 1.0], [[95.0, 105.0], [100.0], [90.0, 100.0, 110.0]], 63, 2000),
    ("short_dated", [1 / 12, 0.1], [[98.0, 100.0, 102.0], [100.0]], 21, 3000),
]


def _numbers(text):
    return [float(x) for x in re.findall(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?", text)]


def _block(src, start_pat, end_pat="};"):
    i = re.search(start_pat, src).end()
    j = src.index(end_pat, i)
    return src[i:j]


def swift_golden():
    """The SWIFT known answers of src/UnitTest.cpp, parsed from its text."""
    src = (REF / "UnitTest.cpp").read_text()
    expiries = _numbers(_block(src, r"std::vector<double>\s+expiries\s*=\s*\{"))
    strikes_txt = _block(src, r"std::vector<std::vector<double>>\s+strikes\s*=\s*\{", "};")
    strikes = [_numbers(row) for row in re.findall(r"\{([^{}]*)\}", strikes_txt)]
    params_txt = _block(src, r"std::vector<swift_parameters>\s+params\s*=\s*\{", "};")
    swift = [_numbers(row) for row in re.findall(r"\{([^{}]*)\}", params_txt)]
    p_txt = _block(src, r"double\s+p\[5\]\s*=\s*\{", "};")
    p5 = [float(x) for x in re.findall(r"([-+]?\d*\.\d+|\d+\.)", re.sub(r"//[^\n]*", "", p_txt))]
    prices = _numbers(_block(src, r"std::vector<ffloat>\s+prices\s*=\s*\{"))
    grad = _numbers(_block(src, r"std::vector<ffloat>\s+grad\s*=\s*\{"))
    index_map = [int(x) for x in _numbers(_block(src, r"std::vector<ffloat>\s+index_map\s*=\s*\{"))]
    risk_free = float(re.search(r"HDistribution new_distr\(heston_params,expiries_arg\[i\],([0-9.]+)\)", src).group(1))
    tol_p = float(re.search(r"#define PRICING_TOLERANCE\s+(\S+)", src).group(1))
    tol_g = float(re.search(r"#define GRADIENT_TOLERANCE\s+(\S+)", src).group(1))
    assert len(expiries) == 8 and len(strikes) == 8 and len(swift) == 8 and len(p5) == 5
    assert len(prices) == 40 and len(grad) == 200 and sorted(index_map) == [0, 1, 2, 3, 4]
    out = {"source": "src/UnitTest.cpp pricing_test / gradient_test", "S": 1.0, "r": risk_free,
           "params5": p5, "expiries": expiries, "strikes": strikes, "swift_params": swift,
           "prices": [float(x).hex() for x in prices], "grad": [float(x).hex() for x in grad],
           "grad_index_map": index_map, "price_tolerance_sum_abs": tol_p, "grad_tolerance_sum_abs": tol_g}
    (HERE / "swift_golden.json").write_text(json.dumps(out, indent=1))


def main():
    if REF is None:
        print("reference checkout not found (set HEXO_REFERENCE_SRC to its src/); nothing to do", file=sys.stderr)
        return 1
    swift_golden()
    if sys.argv[1:] == ["swift"]:
        return 0
    subprocess.run(["make", "-C", str(ROOT / "oracle"), "ref", f"REF_SRC={REF}"], check=True)
    lib = C.CDLL(str(ROOT / "oracle" / "_ref" / "libhexo_ref.so"))

    # 1. RNG draws
    rng = np.random.default_rng(12345)
    draws = []
    for seed, size in [(1, 16), (42, 16), (7, 32), (0x80000005, 16), (3, 1 << 12)]:
        kinds = (rng.random(600) < 0.2).astype(np.uint8)
        out = np.zeros(len(kinds))
        lib.ref_rng_draws(C.c_uint32(seed), C.c_uint32(size), P(kinds), C.c_uint64(len(kinds)), P(out))
        draws.append({"seed": seed, "size": size, "kinds": kinds.tolist(), "draws": hexlist(out)})
    (HERE / "rng_draws.json").write_text(json.dumps(draws))

    # 2. untouched price<>, one thread
    prices = []
    p5 = np.array(C0["params5"])
    for name, T, strikes, steps, n in CASES:
        Ta = np.array(T)
        opc = np.array([len(s) for s in strikes], dtype=np.uint32)
        K = np.array([k for s in strikes for k in s])
        for kind in (0, 1):
            out = np.zeros(len(K))
            lib.ref_price(kind, P(p5), C.c_double(C0["S"]), C.c_uint32(len(Ta)), P(Ta), P(opc), P(K),
                          C.c_uint32(n), C.c_uint32(steps), P(out))
            prices.append({"name": name, "kind": kind, "T": T, "strikes": strikes, "steps": steps, "n_sims": n,
                           "params5": C0["params5"], "S": C0["S"], "prices": hexlist(out)})
    (HERE / "ref_price.json").write_text(json.dumps(prices))

    # 3. per-path payoffs with one stream per path
    paths = []
    for name, T, strikes, steps, _ in CASES:
        Ta = np.array(T)
        opc = np.array([len(s) for s in strikes], dtype=np.uint32)
        K = np.array([k for s in strikes for k in s])
        n = 256
        for kind in (0, 1):
            out = np.zeros(n * len(K))
            lib.ref_paths(kind, P(p5), C.c_double(C0["S"]), C.c_uint32(len(Ta)), P(Ta), P(opc), P(K),
                          C.c_uint32(steps), C.c_uint32(42), C.c_uint32(16), C.c_uint64(0), C.c_uint64(n), P(out))
            paths.append({"name": name, "kind": kind, "T": T, "strikes": strikes, "steps": steps, "seed": 42,
                          "block_words": 16, "n_paths": n, "params5": C0["params5"], "S": C0["S"],
                          "payoffs": hexlist(out)})
    (HERE / "ref_paths.json").write_text(json.dumps(paths))
    print("wrote", [p.name for p in HERE.glob("*.json")])
    return 0


if __name__ == "__main__":
    sys.exit(main())
