"""The C-ABI boundary without a GPU: the library loads, exports every
function include/hexo_mc.h declares, its struct layouts match the Python
bindings, and the host-only parts (planning, finalisation, validation) work.
"""
import ctypes as C
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

from hestonexotics_gb300 import _lib as L
from hestonexotics_gb300 import engine as E
from hestonexotics_gb300 import workloads as W

HEADER = ROOT / "include" / "hexo_mc.h"


@pytest.fixture(scope="module")
def lib():
    from hestonexotics_gb300 import build
    build.build()
    return L.load()


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]*?\b(hexo_\w+)\s*\(", text, re.M)))


def test_every_declared_function_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", str(L.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(hexo_\w+)\b", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    assert set(names) == set(L.PROTOTYPES), set(names) ^ set(L.PROTOTYPES)


def test_struct_layouts_match_header(tmp_path):
    structs = ["hexo_params", "hexo_option", "hexo_mc_cfg", "hexo_ctx_opts", "hexo_request", "hexo_batch_info",
               "hexo_plan_stats", "hexo_tune_result", "hexo_tune_entry", "hexo_server_opts", "hexo_server_stats",
               "hexo_swift_params", "hexo_swift_chain", "hexo_swift_request"]
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include "hexo_mc.h"\nint main(void){\n' +
                   "".join(f'printf("%zu\\n", sizeof({s}));\n' for s in structs) + "return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    for s, n in zip(structs, sizes):
        assert C.sizeof(getattr(L, s)) == n, s


def test_header_compiles_as_c_and_cpp(tmp_path):
    for comp, ext in (("gcc", "c"), ("g++", "cpp")):
        f = tmp_path / f"h.{ext}"
        f.write_text('#include "hexo_mc.h"\nint main(void){ hexo_mc_cfg c; hexo_mc_cfg_default(&c); return 0; }\n')
        subprocess.run([comp, "-fsyntax-only", "-I", str(ROOT / "include"), str(f)], check=True)


def _stats(lib, reqs, cfg):
    arr, keep, _ = E.Engine._requests(None, reqs)
    c = cfg.c()
    st = L.hexo_plan_stats()
    rc = lib.hexo_plan_stats_get(arr, len(reqs), C.byref(c), C.byref(st))
    return rc, st


def test_plan_counts_plain_asian(lib):
    req, cfg = W.plain_asian()
    rc, st = _stats(lib, [req], cfg)
    assert rc == 0
    assert st.nominal_path_steps == 65536 * 252
    # t += 1/252 in double stays below 1 after 252 steps: the reference takes 253 (HSimulation.tpp:84)
    assert st.executed_path_steps == 65536 * 253
    assert st.n_segments == 1 and st.n_maturities == 1


def _schedule(lib, params, S0, opts, cfg):
    n = len(np.unique(opts.T))
    steps = np.zeros(n, dtype=np.uint64)
    tmtp = np.zeros(n)
    mats = np.zeros(n)
    nm = C.c_uint32()
    p = params.c()
    c = cfg.c()
    rc = lib.hexo_plan_schedule(C.byref(p), S0, opts.c_array(), len(opts), C.byref(c), n,
                                steps.ctypes.data_as(C.POINTER(C.c_uint64)), tmtp.ctypes.data_as(C.POINTER(C.c_double)),
                                mats.ctypes.data_as(C.POINTER(C.c_double)), C.byref(nm))
    assert rc == 0 and nm.value == n
    return steps, tmtp, mats


def reference_time_walk(T, steps):
    """The reference's time stepping (HSimulation.tpp:29-46), walked in double."""
    t, j, dt, k = 0.0, 0, T[0] / steps[0], 0
    out_steps, out_tmtp = [], []
    while j < len(T):
        tp = t
        t += dt
        k += 1
        while j < len(T) and t >= T[j]:
            out_steps.append(k)
            out_tmtp.append(T[j] - tp)
            j += 1
            if j < len(T):
                dt = T[j] / steps[j]
    return out_steps, out_tmtp


@pytest.mark.parametrize("mode", [E.STEP_REFERENCE, E.STEP_GRID])
def test_schedule_matches_reference_time_walk(lib, mode):
    req, cfg = W.single_chain(n_paths=1024)
    cfg.step_mode = mode
    cfg.steps = 100
    steps, tmtp, mats = _schedule(lib, req.params, req.S0, req.options, cfg)
    uT = np.unique(req.options.T)
    n = [100] * len(uT) if mode == E.STEP_REFERENCE else [max(5, int(round(252 * t))) for t in uT]
    ws, wt = reference_time_walk(list(uT), n)
    assert list(steps) == ws
    assert np.array_equal(tmtp, np.array(wt))
    assert np.array_equal(mats, uT)


def test_grid_extra_steps_quirk(lib):
    # 252 steps of 1/252 do not reach 1.0 in double: one extra step; T = 1/12 at 21 steps needs exactly 21
    p = E.Params(0.04, 0.04, -0.7, 1.5, 0.5)
    cfg = E.Config(step_mode=E.STEP_REFERENCE, steps=252)
    s, _, _ = _schedule(lib, p, 100.0, E.Options(np.array([100.0]), 1.0, 0), cfg)
    assert list(s) == [253]
    cfg.steps = 21
    s, _, _ = _schedule(lib, p, 100.0, E.Options(np.array([100.0]), 1 / 12, 0), cfg)
    assert list(s) == [21]


def test_uneven_batch_plans(lib):
    reqs, cfg = W.uneven_batch(n_sets=4, path_scale=1 / 64)
    rc, st = _stats(lib, reqs, cfg)
    assert rc == 0
    assert st.n_options == sum(len(r.options) for r in reqs)
    assert st.executed_path_steps >= st.nominal_path_steps > 0


def test_control_variate_plans(lib):
    # the control variate adds internal slots but neither options nor steps
    reqs, cfg = W.uneven_batch(n_sets=4, path_scale=1 / 64)
    rc0, st0 = _stats(lib, reqs, cfg)
    cfg.control_variate = 1
    rc1, st1 = _stats(lib, reqs, cfg)
    assert rc0 == rc1 == 0
    assert st1.n_options == st0.n_options == sum(len(r.options) for r in reqs)
    assert (st1.nominal_path_steps, st1.executed_path_steps) == (st0.nominal_path_steps, st0.executed_path_steps)
    cfg.control_variate = 2
    rc2, _ = _stats(lib, reqs, cfg)
    assert rc2 == 1  # HEXO_ERR_INVALID


@pytest.mark.parametrize("bad", [
    dict(v0=float("nan")), dict(theta=0.0), dict(kappa=-1.0), dict(sigma=0.0), dict(rho=1.5)])
def test_invalid_parameters_rejected(lib, bad):
    req, cfg = W.plain_asian()
    kw = dict(v0=0.04, theta=0.04, rho=-0.7, kappa=1.5, sigma=0.5)
    kw.update(bad)
    req.params = E.Params(**kw)
    rc, _ = _stats(lib, [req], cfg)
    assert rc == 1  # HEXO_ERR_INVALID


def test_invalid_options_rejected(lib):
    req, cfg = W.plain_asian()
    for opts in (E.Options(np.array([100.0]), -1.0, 0), E.Options(np.array([100.0]), 1.0, 7),
                 E.Options(np.array([np.inf]), 1.0, 0)):
        req.options = opts
        rc, _ = _stats(lib, [req], cfg)
        assert rc == 1
    req, cfg = W.plain_asian()
    cfg.rng_block_words = 32
    rc, _ = _stats(lib, [req], cfg)
    assert rc == 4  # HEXO_ERR_UNSUPPORTED


def test_host_finaliser_from_oracle_limbs(lib, oracle):
    # the engine's host finaliser turns exact limb sums into the oracle's price
    K = np.array([90.0, 100.0, 120.0])
    p = E.Params(0.04, 0.05, -0.6, 1.2, 0.4, r=0.03)
    price, se, limbs = oracle.price_paths(p.as_array(), 100.0, K, 1.0, [0, 1, 0], n_default=4000, steps=60)
    opts = E.Options(K, 1.0, np.array([0, 1, 0]))
    cfg = E.Config(n_paths=4000, steps=60)
    fp, fse = E.finalize_limbs(p, 100.0, opts, cfg, limbs)
    np.testing.assert_allclose(fp, price, rtol=1e-14)
    np.testing.assert_allclose(fse, se, rtol=1e-9)


def test_abi_version_matches_header_and_bindings(lib):
    m = re.search(r"#define\s+HEXO_ABI_VERSION\s+(\d+)u", HEADER.read_text())
    assert m and int(m.group(1)) == L.ABI_VERSION == lib.hexo_abi_version()


def test_checked_build_exports_the_same_functions(lib):
    from hestonexotics_gb300 import build
    assert build.LIB_CHECKS.exists()
    out = subprocess.run(["nm", "-D", "--defined-only", str(build.LIB_CHECKS)], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r"\b(hexo_\w+)\b", out))
    assert set(declared_functions()) <= exported


def test_requests_of_a_workload_never_share_a_path_stream():
    # path k of a request draws from the stream seeded {seed + k, stream, 0, 0}:
    # requests with their own stream numbers share none, whatever their seeds
    import dataclasses
    reqs, _ = W.uneven_batch(seed=2)
    assert W.stream_overlaps(reqs) == []
    arrivals, _ = W.request_stream(500.0, 2.0, seed=3)
    assert W.stream_overlaps([a.request for a in arrivals]) == []
    # with the seed word alone, two sets of the benchmark batch shared 2.7M path streams
    same = [dataclasses.replace(r, stream=0) for r in reqs]
    assert W.stream_overlaps(same) == [(18, 37, 2723757)] or W.stream_overlaps(same) == [(37, 18, 2723757)]


def test_batch_shard_ranges_cover_every_path_once():
    from hestonexotics_gb300 import shard as S
    for n in (1, 7, 1000, 4194304, 4194305):
        for world in (1, 2, 3, 8):
            spans = [S.shard_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
