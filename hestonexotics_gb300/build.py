"""Builds the engine's shared libraries in-tree.

  libhexo_mc.so         the engine
  libhexo_mc_checks.so  the same sources compiled with HEXO_CHECKS: every
                        descriptor, queue, window and slot index of the path
                        kernels is bounds-checked, and a failed check is
                        reported as HEXO_ERR_CHECK instead of touching
                        memory (the tests run the small cases through it)

CUDA sources are compiled for sm_103a only (GB300), host sources with g++
(shared by both libraries); translation units compile in parallel.  Used by
``__graft_entry__.build()`` and by ``python -m hestonexotics_gb300.build``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = PKG / "libhexo_mc.so"
OUT_CHECKS = PKG / "_build_checks"
LIB_CHECKS = PKG / "libhexo_mc_checks.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INCLUDES = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "--expt-relaxed-constexpr"] + INCLUDES
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall", "-Wextra",
             "-I", str(CUDA_HOME / "include")] + INCLUDES
LINK_LIBS = ["-L", str(CUDA_HOME / "lib64"), "-lcudart_static", "-lrt", "-lpthread", "-ldl"]


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    return cu, cpp


def _stale(obj: Path, deps) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}):\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def build(verbose: bool = False, jobs: int | None = None, extra_nvcc=None, checks: bool = True) -> Path:
    """Compiles every CUDA/C++ source and links libhexo_mc.so (and, with
    checks, libhexo_mc_checks.so); returns the engine library's path."""
    variants = [(OUT, LIB, [])] + ([(OUT_CHECKS, LIB_CHECKS, ["-DHEXO_CHECKS"])] if checks else [])
    cu, cpp = _sources()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").rglob("*.h"))
    jobs_list, links = [], []
    host_objs = []
    OUT.mkdir(exist_ok=True)
    for src in cpp:   # host code has no checked variant: one object for both libraries
        obj = OUT / (src.stem + ".cpp.o")
        host_objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs_list.append(["g++"] + CXX_FLAGS + ["-c", str(src), "-o", str(obj)])
    for out, lib, defs in variants:
        out.mkdir(exist_ok=True)
        objs = []
        for src in cu:
            obj = out / (src.stem + ".o")
            objs.append(obj)
            if _stale(obj, [src] + headers):
                jobs_list.append([NVCC] + NVCC_FLAGS + defs + (extra_nvcc or []) + ["-c", str(src), "-o", str(obj)])
        links.append((lib, objs + host_objs))
    if jobs_list:
        n = jobs or min(len(jobs_list), os.cpu_count() or 4)
        with ThreadPoolExecutor(max_workers=n) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs_list))
    for lib, objs in links:
        if not lib.exists() or _stale(lib, objs):
            tmp = lib.with_suffix(".so.tmp")
            _run(["g++", "-shared", "-o", str(tmp)] + [str(o) for o in objs] + LINK_LIBS, verbose)
            os.replace(tmp, lib)
    return LIB


def reference_src() -> Path | None:
    """The reference checkout's src/ directory: HEXO_REFERENCE_SRC, else a
    checkout named `reference` beside this repository; None when neither
    exists (as on machines without the reference)."""
    env = os.environ.get("HEXO_REFERENCE_SRC")
    for cand in ([Path(env)] if env else []) + [ROOT.parent / "reference" / "src"]:
        if (cand / "RNG.cpp").exists():
            return cand
    return None


def build_oracle(verbose: bool = False) -> None:
    """Builds the CPU oracle (test infrastructure) and, where the reference
    checkout exists, the library compiled from the reference's own sources."""
    oracle = ROOT / "oracle"
    _run(["make", "-C", str(oracle), "-j4"], verbose)
    ref = reference_src()
    if ref is not None:
        _run(["make", "-C", str(oracle), "ref", f"REF_SRC={ref}"], verbose)


def clean() -> None:
    for d in (OUT, OUT_CHECKS):
        shutil.rmtree(d, ignore_errors=True)
    for lib in (LIB, LIB_CHECKS):
        if lib.exists():
            lib.unlink()


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    print(build(verbose="-v" in sys.argv))
