"""The C++ face (include/arborx_gb300/ArborX_GB300.hpp): compiles against the
C ABI on any host (no GPU), and on a GPU the C++ restatement of the reference
tests (tests/cpp/tst_facade.cpp) passes."""

import os
import shutil
import subprocess

import pytest

from tests.conftest import ROOT

CUDA = "/usr/local/cuda"


def _compile(out):
    from arborx_gb300 import build as b

    lib = b.build()
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    libdir = os.path.dirname(lib)
    cmd = [
        cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Wextra",
        os.path.join(ROOT, "tests", "cpp", "tst_facade.cpp"),
        "-I" + os.path.join(ROOT, "include"), "-I" + CUDA + "/include",
        "-L" + libdir, "-larborx_gb300", "-L" + CUDA + "/lib64", "-lcudart",
        "-Wl,-rpath," + libdir, "-Wl,-rpath," + CUDA + "/lib64", "-o", out,
    ]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def test_facade_compiles(tmp_path):
    _compile(str(tmp_path / "tst_facade"))


@pytest.mark.gpu
def test_facade_reference_cases(tmp_path, ax):
    exe = _compile(str(tmp_path / "tst_facade"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failures" in r.stdout


def _compile_cuda(out):
    from arborx_gb300 import build as b

    lib = b.build()
    libdir = os.path.dirname(lib)
    nvcc = b._nvcc()
    cmd = [
        nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
        os.path.join(ROOT, "tests", "cpp", "tst_callbacks.cu"),
        "-I" + os.path.join(ROOT, "include"), "-L" + libdir, "-larborx_gb300",
        "-Xlinker", "-rpath," + libdir, "-o", out,
    ]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def test_callbacks_compile(tmp_path):
    _compile_cuda(str(tmp_path / "tst_callbacks"))


@pytest.mark.gpu
def test_callbacks_and_per_thread_queries(tmp_path, ax):
    exe = _compile_cuda(str(tmp_path / "tst_callbacks"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failures" in r.stdout
