"""The C++ mirror of the reference API (include/tbk.hpp): it compiles against
the C ABI on the host, and the C++ program built from tests/cpp runs its
checks on the GPU."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_header_compiles_standalone():
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-I", str(ROOT / "include"),
                        "-x", "c++", "-"], input='#include "tbk.hpp"\nint main() { return 0; }\n',
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_cpp_program(gpu):
    from tight_binding_gb300 import build
    exe = build.build_cpp_test()
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout, r.stdout


def test_numerics_cuda_shim_compiles():
    """include/tbk_numerics_cuda.hpp with the reference's declarations and the Eigen stand-in."""
    from tight_binding_gb300 import build
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-I", str(ROOT / "include"),
                        "-I", str(ROOT / "tests" / "cpp" / "eigen_standin"), str(build.SHIM_TEST)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_numerics_cuda_shim_program(gpu):
    """The shim's two overloads run the moments through libtbk (exact ring traces)."""
    from tight_binding_gb300 import build
    exe = build.build_shim_test()
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout, r.stdout
