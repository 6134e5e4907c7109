"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer (CPU).

The reference's debug build compiles with -fsanitize=undefined and
-fsanitize=address (Makefile.am:62-65).  The host parts of this project are
built the same way and run on small problems: the engine's planner and host
finaliser (csrc/hexo_plan.cpp, no CUDA involved) through
tests/sanitize/plan_main.cpp, and the CPU oracle through
tests/sanitize/oracle_main.cpp.  Any sanitizer report fails the run.  The
device code's counterpart is the bounds-checked build, HEXO_CHECKS
(tests/test_gpu_checks.py).
"""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SAN = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer", "-g", "-O1"]
ENV = {**os.environ, "ASAN_OPTIONS": "detect_leaks=0:abort_on_error=0", "UBSAN_OPTIONS": "print_stacktrace=1",
       "OMP_NUM_THREADS": "2"}


def _run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    assert r.returncode == 0, f"{' '.join(map(str, cmd))}\n{r.stdout[-3000:]}\n{r.stderr[-6000:]}"
    return r


@pytest.fixture(scope="module")
def compilers():
    if shutil.which("g++") is None or shutil.which("gcc") is None:
        pytest.skip("no host compiler")


def test_planner_and_finaliser_under_sanitizers(compilers, tmp_path):
    exe = tmp_path / "plan_san"
    csrc = ROOT / "hestonexotics_gb300" / "csrc"
    _run(["g++", "-std=c++17", *SAN, "-I", str(ROOT / "include"), "-I", str(csrc),
          str(ROOT / "tests" / "sanitize" / "plan_main.cpp"), str(csrc / "hexo_plan.cpp"), "-o", str(exe)])
    r = _run([str(exe)], env=ENV, timeout=600)
    assert "0 failed checks" in r.stdout
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr


def test_oracle_under_sanitizers(compilers, tmp_path):
    exe = tmp_path / "oracle_san"
    o = ROOT / "oracle"
    as241 = tmp_path / "as241.o"
    _run(["gcc", "-O1", "-g", "-ffp-contract=off", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
          "-c", str(o / "as241.c"), "-o", str(as241)])
    _run(["g++", "-std=c++17", "-fopenmp", "-ffp-contract=off", *SAN, "-I", str(o),
          str(ROOT / "tests" / "sanitize" / "oracle_main.cpp"), str(o / "hexo_oracle.cpp"), str(o / "swift.cpp"),
          str(as241), "-o", str(exe)])
    r = _run([str(exe)], env=ENV, timeout=600)
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr
