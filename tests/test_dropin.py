"""The drop-in C/C++ headers: the C ABI header is valid C, the C++ headers
compile with a host compiler, and a driver written like the reference's own
test programs (tests/cpp/dropin_test.cu) builds with nvcc against the library
and -- on a GPU -- passes against its CPU stable multisplit, for library
functors (precompiled kernels) and user functors (kernels instantiated in the
caller's translation unit)."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
BUILD = ROOT / "tests" / "_build"
CUDA_INC = "/usr/local/cuda/include"


def _nvcc():
    from gpumultisplit_gb300 import build as gbuild

    return gbuild.nvcc_path()


def test_c_header_is_valid_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "gpumultisplit.h"\nint main(void) { gms_bucket_desc d = {0}; (void)d; return 0; }\n')
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-I", str(ROOT / "include"), str(src)],
                   check=True)


def test_cpp_headers_compile_with_host_compiler(tmp_path):
    if not os.path.isdir(CUDA_INC):
        pytest.skip("CUDA headers not found")
    src = tmp_path / "t.cpp"
    src.write_text('#include "api/multisplit.cuh"\n#include "api/multisplit_sort.cuh"\n'
                   '#include "api/multisplit_histogram.cuh"\n'
                   '#include "kernels/compaction/multisplit2_compaction.cuh"\n'
                   "int main() { multisplit_context c(8); (void)c; return 0; }\n")
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", str(ROOT / "include"),
                    "-I", str(ROOT / "include" / "gpumultisplit"), "-I", CUDA_INC, str(src)], check=True)


def build_driver() -> Path:
    from gpumultisplit_gb300 import build as gbuild

    lib = gbuild.build()
    BUILD.mkdir(parents=True, exist_ok=True)
    exe = BUILD / "dropin_test"
    src = ROOT / "tests" / "cpp" / "dropin_test.cu"
    deps = [src, lib] + list((ROOT / "include" / "gpumultisplit").rglob("*.cuh"))
    if exe.exists() and all(exe.stat().st_mtime > p.stat().st_mtime for p in deps):
        return exe
    subprocess.run([_nvcc(), *gbuild.ARCH_FLAGS, "-O2", "-std=c++17", "-I", str(ROOT / "include"),
                    "-I", str(ROOT / "include" / "gpumultisplit"), "-I", str(ROOT / "gpumultisplit_gb300" / "csrc"),
                    str(src), "-L", str(lib.parent), "-lgpumultisplit", "-Xlinker", "-rpath", "-Xlinker",
                    str(lib.parent), "-o", str(exe)], check=True)
    return exe


def test_driver_builds():
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc not available")
    assert build_driver().exists()


@pytest.mark.gpu
def test_driver_passes_on_gpu():
    exe = build_driver()
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout
