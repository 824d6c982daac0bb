"""Build recipe for the native parts of afquantumsim_gb300.

Everything is compiled in-tree (outputs under ``_build/`` folders, which are
git-ignored):

* ``afquantumsim_gb300/_build/libaqsg.so`` - the C-ABI engine (CUDA, sm_103a)
* ``afquantumsim_gb300/_build/libaqs.so``  - the ``aqs::`` C++ layer over it
* ``oracle/_build/libaqs_oracle.so``       - the CPU oracle (test infrastructure)

Only nvcc / g++ / gcc are used, translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
CPP = PKG / "cpp"
BUILD = PKG / "_build"
ORACLE = ROOT / "oracle"
ORACLE_BUILD = ORACLE / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"] + ARCH
CU_SOURCES = ["api.cu", "gate_kernels.cu", "measure_kernels.cu", "tile_kernels.cu", "fusion.cu", "batch.cu", "server.cu", "tune.cu", "circuit_text.cu", "noise.cu"]
CPP_SOURCES = ["quantum.cpp", "quantum_gates.cpp", "quantum_algo.cpp"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _cuda_lib() -> str:
    home = Path(_nvcc()).resolve().parent.parent
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        if (home / sub / "libcudart.so").exists():
            return str(home / sub)
    return str(home / "lib64")


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed ({res.returncode}): {' '.join(cmd)}\n"
                           f"{res.stdout}\n{res.stderr}")
    if verbose and res.stderr.strip():
        print(res.stderr, flush=True)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_engine(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile libaqsg.so (CUDA C-ABI engine) for sm_103a."""
    BUILD.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "aqsg.h"]
    objs, steps = [], []
    for src in CU_SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            steps.append([_nvcc(), *NVCC_FLAGS, "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=jobs or len(steps) or 1) as ex:
        list(ex.map(lambda c: _run(c, verbose), steps))
    lib = BUILD / "libaqsg.so"
    if _stale(lib, objs):
        _run([_nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(lib),
              *map(str, objs)], verbose)
    return lib


def build_cpp(verbose: bool = False) -> Path:
    """Compile the aqs:: C++ layer (libaqs.so) over libaqsg.so."""
    srcs = [CPP / s for s in CPP_SOURCES if (CPP / s).exists()]
    lib = BUILD / "libaqs.so"
    if not srcs:
        return lib
    deps = srcs + list((CPP / "aqs").glob("*.h")) + [BUILD / "libaqsg.so"]
    if _stale(lib, deps):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall",
              f"-I{CPP}", f"-I{ROOT / 'include'}", *map(str, srcs),
              f"-L{BUILD}", "-laqsg", "-Wl,-rpath,$ORIGIN", "-o", str(lib)], verbose)
    return lib


def build_oracle(verbose: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure) with OpenMP."""
    ORACLE_BUILD.mkdir(parents=True, exist_ok=True)
    src = ORACLE / "aqs_oracle.c"
    lib = ORACLE_BUILD / "libaqs_oracle.so"
    if _stale(lib, [src, ORACLE / "aqs_oracle.h", ROOT / "include" / "aqsg.h"]):
        _run(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              "-std=c11", "-Wall", str(src), "-lm", "-o", str(lib)], verbose)
    return lib


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f_eng = ex.submit(build_engine, verbose)
        f_orc = ex.submit(build_oracle, verbose)
        f_eng.result()
        f_orc.result()
    build_cpp(verbose)


if __name__ == "__main__":
    import sys
    build_all(verbose="-v" in sys.argv)
    print("built", BUILD, ORACLE_BUILD)
