"""The C++ host API through programs compiled against include/ and
libjetgpu.so (tests/cpp/).

tbc_dot_test.cpp (host only, runs on the CPU): TaskBasedContractor's DOT dump
of a two-network task graph with a shared step, reduction and deletions.

cuda_tensor_test.cpp: Jet::CudaTensor (the reference's device tensor type,
column-major over its labels). On the CPU the program is only compiled
(every template of the header instantiated); on the GPU it runs and checks
construction, conversions to and from Jet::Tensor (labels reversed), rename,
reshape, column-major slicing and transposes, contractions (exact small
cases, random tensors against Jet::Tensor, planned contraction into a
preallocated output in either label order, complex128), additions, and a
TaskBasedContractor network over CudaTensor.

tile_plan_test.cu (host only, runs on the CPU): the tiled permute's plan for
non-power-of-2 dims replayed pass by pass against the plain permutation,
with every slot and offset checked against its buffer.

replay_plan_test.cpp (host only, runs on the CPU): the TaskBasedContractor
replay's grouping of tiny steps and its arena plan on random contraction
DAGs: runs hold only independent tiny steps, and no two buffers live at the
same time overlap.

skinny_plan_test.cu (host only, runs on the CPU): the skinny contraction's
launch parameters (row digits, tabulated offsets, batch offsets, C strides)
replayed against the permuted operands' offsets for random shapes, axis
orders and batch modes.

tensor_labels_test.cpp (host only, runs on the CPU): Jet::Tensor's label ->
dimension map, built when first read, against the reference's eager rules
through construction, renames, SetShape, copies, moves and equality.
pool_limit_test.cpp (GPU): device memory exhaustion injected through a capped
library pool raises Jet::Exception from Tensor::ContractTensors,
TaskBasedContractor and SlicedContractor, and each recovers once the cap is
lifted."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(out_path, source="cuda_tensor_test.cpp"):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    pkg = os.path.join(REPO, "jet_gb300")
    cmd = [cxx, "-std=c++17", "-O1", "-I" + os.path.join(REPO, "include"),
           "-I" + os.path.join(pkg, "include"), "-I" + os.path.join(cuda_home, "include"),
           os.path.join(REPO, "tests", "cpp", source), "-L" + pkg, "-ljetgpu",
           "-Wl,-rpath," + pkg, "-o", out_path]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]


def test_tile_permute_plan(tmp_path):
    nvcc = shutil.which("nvcc") or os.path.join(
        os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    pkg = os.path.join(REPO, "jet_gb300")
    exe = str(tmp_path / "tile_plan_test")
    cmd = [nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I" + os.path.join(REPO, "include"), "-I" + os.path.join(pkg, "csrc"),
           os.path.join(REPO, "tests", "cpp", "tile_plan_test.cu"), "-L" + pkg, "-ljetgpu",
           "-Xlinker", "-rpath", "-Xlinker", pkg, "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]
    res = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    assert res.stdout.startswith("ok ")


def test_skinny_plan(tmp_path):
    nvcc = shutil.which("nvcc") or os.path.join(
        os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    pkg = os.path.join(REPO, "jet_gb300")
    exe = str(tmp_path / "skinny_plan_test")
    cmd = [nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I" + os.path.join(REPO, "include"), "-I" + os.path.join(pkg, "csrc"),
           os.path.join(REPO, "tests", "cpp", "skinny_plan_test.cu"), "-L" + pkg, "-ljetgpu",
           "-Xlinker", "-rpath", "-Xlinker", pkg, "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]
    res = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    assert res.stdout.startswith("ok ")


def test_replay_plan(tmp_path):
    exe = str(tmp_path / "replay_plan_test")
    _compile(exe, "replay_plan_test.cpp")
    res = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    assert res.stdout.startswith("ok ")


def test_tensor_label_map(tmp_path):
    exe = str(tmp_path / "tensor_labels_test")
    _compile(exe, "tensor_labels_test.cpp")
    res = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    assert res.stdout.startswith("ok")


def test_cuda_tensor_header_compiles(tmp_path):
    _compile(str(tmp_path / "cuda_tensor_test"))


@pytest.mark.gpu
def test_cuda_tensor_behaviour(tmp_path, cuda):
    exe = str(tmp_path / "cuda_tensor_test")
    _compile(exe)
    res = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0 and "ALL OK" in res.stdout, res.stdout[-4000:] + res.stderr[-2000:]


def test_pool_limit_program_compiles(tmp_path):
    _compile(str(tmp_path / "pool_limit_test"), "pool_limit_test.cpp")


@pytest.mark.gpu
def test_pool_limit_raises_jet_exception_and_recovers(tmp_path, cuda):
    """Device memory exhaustion injected on the host (a capped pool): the
    contraction raises Jet::Exception, the cap lifted it succeeds with the
    uncapped result, and the failed attempts hold no device memory."""
    exe = str(tmp_path / "pool_limit_test")
    _compile(exe, "pool_limit_test.cpp")
    res = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0 and "ALL OK" in res.stdout, res.stdout[-4000:] + res.stderr[-2000:]


def test_task_graph_dot_dump(tmp_path):
    exe = str(tmp_path / "tbc_dot_test")
    _compile(exe, "tbc_dot_test.cpp")
    res = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    out = res.stdout.splitlines()
    assert out[:2] == ["shared 0", "shared 1"]
    assert out[2] == "digraph Taskflow {" and out[-1] == "}"
    nodes = {l.split(" ")[0]: l.split('"')[1] for l in out if "[label=" in l}
    edges = {tuple(l.rstrip(";").split(" -> ")) for l in out if " -> " in l}
    by_label = {v: k for k, v in nodes.items()}
    shared = by_label["3:ik"]
    r0, r1 = by_label["4:i:results[0]"], by_label["4:i:results[1]"]
    s0, s1 = by_label["store 4:i:results[0]"], by_label["store 4:i:results[1]"]
    red = by_label["reduce"]
    # The shared first step feeds both networks' second steps.
    assert {(shared, r0), (shared, r1), (r0, s0), (r1, s1), (s0, red), (s1, red)} <= edges
    # A tensor is deleted after every task that consumes it.
    assert {(r0, by_label["3:ik:delete"]), (r1, by_label["3:ik:delete"])} <= edges
    assert len(nodes) == 10
