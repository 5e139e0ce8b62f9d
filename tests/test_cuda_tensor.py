"""Jet::CudaTensor (the reference's device tensor type, column-major over its
labels) through the C++ host API: tests/cpp/cuda_tensor_test.cpp compiled
against include/ and libjetgpu.so. On the CPU the program is only compiled
(every template of the header instantiated); on the GPU it runs and checks
construction, conversions to and from Jet::Tensor (labels reversed), rename,
reshape, column-major slicing and transposes, contractions (exact small
cases, random tensors against Jet::Tensor, planned contraction into a
preallocated output in either label order, complex128), additions, and a
TaskBasedContractor network over CudaTensor."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(out_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    pkg = os.path.join(REPO, "jet_gb300")
    cmd = [cxx, "-std=c++17", "-O1", "-I" + os.path.join(REPO, "include"),
           "-I" + os.path.join(pkg, "include"), "-I" + os.path.join(cuda_home, "include"),
           os.path.join(REPO, "tests", "cpp", "cuda_tensor_test.cpp"), "-L" + pkg, "-ljetgpu",
           "-Wl,-rpath," + pkg, "-o", out_path]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]


def test_cuda_tensor_header_compiles(tmp_path):
    _compile(str(tmp_path / "cuda_tensor_test"))


@pytest.mark.gpu
def test_cuda_tensor_behaviour(tmp_path, cuda):
    exe = str(tmp_path / "cuda_tensor_test")
    _compile(exe)
    res = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0 and "ALL OK" in res.stdout, res.stdout[-4000:] + res.stderr[-2000:]
