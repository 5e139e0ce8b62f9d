"""Builds the in-tree native libraries of jet_gb300.

  libjetgpu.so   -- the C-ABI CUDA library (include/jetgpu.h), sm_103a only,
                    compiled with nvcc from jet_gb300/csrc/*.cu.
  _jet_bindings  -- the Python extension over the C++17 host API
                    (jet_gb300/include/jet/*.hpp), linked against libjetgpu.so.

Translation units compile in parallel; objects are rebuilt only when a source
or header is newer. Outputs stay inside the package directory.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys
import sysconfig
from typing import List

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libjetgpu.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = os.path.join(cuda_home, "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _headers() -> List[str]:
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + [os.path.join(REPO_DIR, "include", "jetgpu.h")])


def _newer(target: str, deps: List[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: List[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout)


def nvcc_flags(extra: List[str] = ()) -> List[str]:
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            "--expt-relaxed-constexpr", "-I" + os.path.join(REPO_DIR, "include"), *extra]


def build_library(verbose: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdrs = _headers()
    nvcc = _nvcc()
    objs, jobs = [], []
    for src in sources:
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if ptxas_v or _newer(obj, [src] + hdrs):
            extra = ["-Xptxas", "-v"] if ptxas_v else []
            jobs.append([nvcc, *nvcc_flags(extra), "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, fut in [(c, ex.submit(subprocess.run, c, stdout=subprocess.PIPE,
                                           stderr=subprocess.STDOUT, text=True)) for c in jobs]:
                res = fut.result()
                if verbose or ptxas_v:
                    sys.stdout.write(res.stdout)
                if res.returncode != 0:
                    raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + res.stdout)
    if _newer(LIB_PATH, objs):
        tmp = LIB_PATH + ".tmp"
        _run([nvcc, ARCH, "-shared", "-o", tmp, *objs])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def _load_sibling(name: str):
    """Imports a module of this directory by path: building must not import
    the jet_gb300 package, whose __init__ needs the libraries being built."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("jet_gb300_" + name,
                                                  os.path.join(PKG_DIR, name + ".py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def build_all(verbose: bool = False) -> None:
    build_library(verbose=verbose)
    _load_sibling("_bindings_build").build_bindings(verbose=verbose)


if __name__ == "__main__":
    build_library(verbose=True, ptxas_v="--ptxas-v" in sys.argv)
    print(LIB_PATH)
