"""Builds the engine's shared library, libhexo_mc.so, in-tree.

CUDA sources are compiled for sm_103a only (GB300), host sources with g++;
translation units compile in parallel.  Used by ``__graft_entry__.build()``
and by ``python -m hestonexotics_gb300.build``.
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

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INCLUDES = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "--expt-relaxed-constexpr"] + INCLUDES
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall", "-Wextra",
             "-I", str(CUDA_HOME / "include")] + INCLUDES


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


def build(verbose: bool = False, jobs: int | None = None, extra_nvcc=None) -> Path:
    """Compiles every CUDA/C++ source and links libhexo_mc.so; returns its path."""
    OUT.mkdir(exist_ok=True)
    cu, cpp = _sources()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").rglob("*.h"))
    jobs_list = []
    objs = []
    for src in cu:
        obj = OUT / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs_list.append([NVCC] + NVCC_FLAGS + (extra_nvcc or []) + ["-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = OUT / (src.stem + ".cpp.o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs_list.append(["g++"] + CXX_FLAGS + ["-c", str(src), "-o", str(obj)])
    if jobs_list:
        n = jobs or min(len(jobs_list), os.cpu_count() or 4)
        with ThreadPoolExecutor(max_workers=n) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs_list))
    if jobs_list or not LIB.exists() or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run(["g++", "-shared", "-o", str(tmp)] + [str(o) for o in objs] +
             ["-L", str(CUDA_HOME / "lib64"), "-lcudart_static", "-lrt", "-lpthread", "-ldl"], verbose)
        os.replace(tmp, LIB)
    return LIB


def build_oracle(verbose: bool = False) -> None:
    """Builds the CPU oracle (test infrastructure) and, where the reference
    checkout exists, the library compiled from the reference's own sources."""
    oracle = ROOT / "oracle"
    _run(["make", "-C", str(oracle), "-j4"], verbose)
    if Path("/root/reference/src/RNG.cpp").exists():
        _run(["make", "-C", str(oracle), "ref"], verbose)


def clean() -> None:
    shutil.rmtree(OUT, ignore_errors=True)
    if LIB.exists():
        LIB.unlink()


if __name__ == "__main__":
    if "--clean" in sys.argv:
        clean()
    print(build(verbose="-v" in sys.argv))
