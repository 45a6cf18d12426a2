"""Build recipe for libtbk (sm_103a) and the CPU oracle.

Compiles every translation unit of ``csrc/`` in parallel with nvcc for
``-gencode arch=compute_103a,code=sm_103a`` and links ``_build/libtbk.so``
(static CUDA runtime, so the library loads without a CUDA install on the
loader path).  The oracle (test infrastructure) is built by ``make -C oracle``.

Usage: ``python -m tight_binding_gb300.build`` (or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libtbk.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", str(ROOT / "include")]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
             "-I", str(ROOT / "include"), "-I", "/usr/local/cuda/include"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(verbose: bool = False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    jobs = []
    objs = []
    for src in _sources():
        obj = OUT / (src.stem + (".cu.o" if src.suffix == ".cu" else ".cpp.o"))
        objs.append(obj)
        if not _stale(obj, [src] + headers):
            continue
        if src.suffix == ".cu":
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        else:
            cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, "-c", str(src), "-o", str(obj)]
        jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, fut in zip(jobs, [ex.submit(_run, c) for c in jobs]):
                fut.result()
                if verbose:
                    print(" ".join(cmd), file=sys.stderr)
    if _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-cudart", "static",
              "-Xcompiler", "-fPIC"])
    return LIB


CPP_TEST = ROOT / "tests" / "cpp" / "test_tbk_cpp.cpp"
CPP_TEST_BIN = OUT / "test_tbk_cpp"


def build_cpp_test() -> Path:
    """The C++ program that drives the path through include/tbk.hpp (run by a GPU test)."""
    deps = [CPP_TEST, ROOT / "include" / "tbk.hpp", ROOT / "include" / "tbk.h", LIB]
    if _stale(CPP_TEST_BIN, deps):
        _run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-I", str(ROOT / "include"),
              str(CPP_TEST), "-L", str(OUT), "-ltbk", "-Wl,-rpath,$ORIGIN", "-o", str(CPP_TEST_BIN)])
    return CPP_TEST_BIN


SHIM_TEST = ROOT / "tests" / "cpp" / "test_numerics_cuda_shim.cpp"
SHIM_TEST_BIN = OUT / "test_numerics_cuda_shim"


def build_shim_test() -> Path:
    """The drop-in shim (include/tbk_numerics_cuda.hpp) compiled against the
    Eigen stand-in, as the reference's numerics_cuda.cu would include it."""
    deps = [SHIM_TEST, ROOT / "include" / "tbk_numerics_cuda.hpp", ROOT / "include" / "tbk.h", LIB]
    if _stale(SHIM_TEST_BIN, deps):
        _run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-I", str(ROOT / "include"),
              "-I", str(ROOT / "tests" / "cpp" / "eigen_standin"), str(SHIM_TEST), "-L", str(OUT), "-ltbk",
              "-Wl,-rpath,$ORIGIN", "-o", str(SHIM_TEST_BIN)])
    return SHIM_TEST_BIN


def build_oracle() -> Path:
    _run(["make", "-s", "-C", str(ROOT / "oracle")])
    return ROOT / "oracle" / "_build" / "libkpm_oracle.so"


BASELINE_SRC = ROOT / "baseline" / "cusparse_kpm.cu"
BASELINE_LIB = ROOT / "baseline" / "_build" / "libref_cusparse.so"


def build_baseline() -> Path:
    """The reference's cuSPARSE + cuBLAS moments algorithm restated as a timing
    baseline (baseline/cusparse_kpm.cu); not linked into libtbk."""
    if _stale(BASELINE_LIB, [BASELINE_SRC]):
        BASELINE_LIB.parent.mkdir(parents=True, exist_ok=True)
        _run([_nvcc(), *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", str(BASELINE_SRC),
              "-o", str(BASELINE_LIB), "-lcusparse", "-lcublas", "-Xlinker", "-rpath=/usr/local/cuda/lib64"])
    return BASELINE_LIB


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        side = ex.submit(build_baseline)
        build_library(verbose)
        side.result()
    build_cpp_test()
    build_shim_test()
    build_oracle()


if __name__ == "__main__":
    build_all(verbose=True)
    print(LIB)
