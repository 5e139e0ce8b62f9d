"""Builds jet_gb300/_jet_bindings*.so: the pybind11 module over the C++17 host
API, linked against libjetgpu.so. pybind11's headers are taken from the
PyTorch installation (torch ships them), located without importing torch."""
from __future__ import annotations

import glob
import importlib.util
import os
import subprocess
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
SRC = os.path.join(PKG, "host", "bindings.cpp")


def _pybind_include() -> str:
    spec = importlib.util.find_spec("torch")
    if spec is not None and spec.origin:
        inc = os.path.join(os.path.dirname(spec.origin), "include")
        if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    spec = importlib.util.find_spec("pybind11")
    if spec is not None and spec.origin:
        inc = os.path.join(os.path.dirname(spec.origin), "include")
        if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    raise RuntimeError("pybind11 headers not found (looked in torch and pybind11)")


def output_path() -> str:
    return os.path.join(PKG, "_jet_bindings" + sysconfig.get_config_var("EXT_SUFFIX"))


def build_bindings(verbose: bool = False) -> str:
    out = output_path()
    deps = [SRC, os.path.join(PKG, "libjetgpu.so"), os.path.join(REPO, "include", "jetgpu.h")]
    deps += glob.glob(os.path.join(PKG, "include", "**", "*.hpp"), recursive=True)
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
           "-I" + sysconfig.get_paths()["include"], "-I" + _pybind_include(),
           "-I" + os.path.join(PKG, "include"), "-I" + os.path.join(REPO, "include"),
           "-I" + os.path.join(cuda_home, "include"),
           SRC, "-o", out + ".tmp", "-L" + PKG, "-ljetgpu", "-Wl,-rpath,$ORIGIN"]
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if verbose or res.returncode != 0:
        print(res.stdout)
    if res.returncode != 0:
        raise RuntimeError("building the host-API bindings failed:\n" + " ".join(cmd))
    os.replace(out + ".tmp", out)
    return out
