"""Host helpers of the C ABI that need no GPU (hsspack_gb300/csrc/host_util.h),
compiled with the host compiler and run: MDSTEDC's split test against the
reference's expression, and the host fill / scatter of packed eigenvectors."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    for base in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if base and os.path.exists(os.path.join(base, "include", "vector_types.h")):
            return os.path.join(base, "include")
    nvcc = shutil.which("nvcc")
    if nvcc:
        inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
        if os.path.exists(os.path.join(inc, "vector_types.h")):
            return inc
    return None


def test_host_util(tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if not cxx or not inc:
        pytest.skip("needs g++ and CUDA's vector_types.h")
    exe = str(tmp_path / "host_util_test")
    subprocess.run([cxx, "-std=c++17", "-O2", "-pthread", "-I", os.path.join(ROOT, "hsspack_gb300", "csrc"),
                    "-I", inc, os.path.join(ROOT, "tests", "host_util_test.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
