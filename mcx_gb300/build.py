"""Build recipe of libmcx_gb300.so (the engine) and the oracle's shared library.

The engine is compiled for sm_103a only, in-tree, with nvcc and g++; translation units are
compiled in parallel and linked with the static CUDA runtime.  Nothing here needs a GPU.
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
BUILD = PKG / "_build"
LIB = PKG / "libmcx_gb300.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "libmcx_oracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "--use_fast_math"] + ARCH
CXX_FLAGS = ["-O2", "-fPIC", "-pthread", "-std=c++17", "-Wall", "-Wno-unused-function"]

CU_SOURCES = ["transport.cu", "engine.cu", "noalloc.cu", "denoise.cu"]
CPP_SOURCES = ["preprocess.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 engine needs the CUDA toolkit to build")


def _cuda_include() -> str:
    return str(Path(_nvcc()).resolve().parent.parent / "include")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))


def build_engine(force: bool = False, verbose: bool = False) -> Path:
    """Compile the CUDA engine into mcx_gb300/libmcx_gb300.so (sm_103a)."""
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I" + str(ROOT / "include"), "-I" + str(CSRC)]
    jobs = []
    objs = []
    hdrs = _headers()
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + hdrs):
            jobs.append([nvcc, *NVCC_FLAGS, *inc, "-c", str(CSRC / src), "-o", str(obj)])
    for src in CPP_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + hdrs):
            jobs.append(["g++", *CXX_FLAGS, *inc, "-I" + _cuda_include(), "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for _ in ex.map(_run, jobs):
            pass
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-Xcompiler", "-fPIC", "-lpthread"])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(force: bool = False, verbose: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure) into oracle/_build/libmcx_oracle.so."""
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    src = ORACLE_DIR / "mcx_oracle.cpp"
    if force or _stale(ORACLE_LIB, [src, ORACLE_DIR / "mcx_oracle.h"]):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        _run(["g++", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c++17", "-o", str(tmp), str(src)])
        os.replace(tmp, ORACLE_LIB)
    if verbose:
        print(f"built {ORACLE_LIB}")
    return ORACLE_LIB


def build_all(force: bool = False, verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_engine, force, verbose)
        b = ex.submit(build_oracle, force, verbose)
        a.result()
        b.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose=True)
