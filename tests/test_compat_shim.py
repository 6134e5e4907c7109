"""The C++ drop-in shim (include/hexo/reference_compat.h).

CPU: a program written against the reference's interface
(tests/compat/shim_main.cpp) compiles and links with the shim's stand-alone
types, and against the reference's own headers (src/inc) where a checkout
exists.  GPU: the program's HSimulation::price<hexo::GpuQE<...>> calls return
the engine's own FP64 prices bit for bit, and an out-of-order chain list
throws std::runtime_error as the reference's debug check would.
"""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT
from hestonexotics_gb300 import engine as E

SRC = ROOT / "tests" / "compat" / "shim_main.cpp"
LIBDIR = ROOT / "hestonexotics_gb300"
def _ref_inc() -> Path:
    from hestonexotics_gb300.build import reference_src
    src = reference_src()   # HEXO_REFERENCE_SRC, or the checkout beside the repository
    return src / "inc" if src is not None else Path("/nonexistent")


REF_INC = _ref_inc()


def _build(out: Path, extra):
    from hestonexotics_gb300 import build
    build.build()
    cmd = ["g++", "-std=c++17", "-O1", *extra, "-I", str(ROOT / "include"), str(SRC), "-L", str(LIBDIR),
           "-lhexo_mc", f"-Wl,-rpath,{LIBDIR}", "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_shim_builds_standalone(tmp_path):
    assert _build(tmp_path / "shim", ["-Wall", "-Werror", "-DHEXO_COMPAT_STANDALONE_TYPES"]).exists()


def test_shim_builds_against_reference_headers(tmp_path):
    if not (REF_INC / "HSimulation.h").exists():
        pytest.skip("no reference checkout here")
    # RNG.h includes shishua.h, which the reference downloads at build time; the oracle's stands in
    extra = ["-fopenmp", "-DFP_SIZE=8", "-DNDEBUG", "-I", str(REF_INC), "-I", str(ROOT / "oracle")]
    assert _build(tmp_path / "shim_ref", extra).exists()


@pytest.mark.gpu
def test_shim_prices_equal_engine(tmp_path, engine):
    exe = _build(tmp_path / "shim", ["-DHEXO_COMPAT_STANDALONE_TYPES"])
    n = 20000
    out = subprocess.run([str(exe), str(n)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = out.stdout.split("\n")
    asian = np.array([float.fromhex(l.split()[1]) for l in lines if l.startswith("asian")])
    euro = np.array([float.fromhex(l.split()[1]) for l in lines if l.startswith("euro")])
    assert "unordered refused" in out.stdout
    T = np.array([0.25, 0.25, 0.5, 0.5, 1.0, 1.0])
    K = np.array([95.0, 105.0, 100.0, 110.0, 90.0, 100.0])
    params = E.Params(0.04, 0.04, -0.7, 1.5, 0.5)
    cfg = E.Config(n_paths=n, step_mode=E.STEP_REFERENCE, steps=63, seed=1, precision=E.FP64)
    for kind, got in ((E.ASIAN, asian), (E.EUROPEAN, euro)):
        want, _ = engine.price(params, 100.0, E.Options(K, T, kind), cfg)
        assert np.array_equal(got, want)
