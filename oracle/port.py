"""The CPU port of the reference contraction path: oracle/jet_oracle.c's
permuter (a restatement of DefaultPermuter, OpenMP-parallel) plus the
row-major CBLAS cgemm/zgemm the reference calls (TensorHelpers.hpp:47-61),
reached through numpy's matmul on the same OpenBLAS.

TEST INFRASTRUCTURE ONLY: the timed CPU baseline of bench.py and a checker
for tests. Built by `build()` (gcc, OpenMP) into oracle/liboracle.so.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "jet_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")
_lib = None


def build() -> str:
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp"
        subprocess.run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", tmp, SRC],
                       check=True)
        os.replace(tmp, LIB)
    return LIB


def _load():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        _lib.oracle_permute.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_uint64),
                                        ctypes.POINTER(ctypes.c_int32), ctypes.c_int, ctypes.c_int]
    return _lib


def max_threads() -> int:
    return int(_load().oracle_max_threads())


def permute(x: np.ndarray, shape: Sequence[int], perm: Sequence[int], nthreads: int = 0,
            out: np.ndarray = None) -> np.ndarray:
    lib = _load()
    x = np.ascontiguousarray(x)
    if out is None:
        out = np.empty_like(x)
    sh = (ctypes.c_uint64 * max(1, len(shape)))(*shape)
    pm = (ctypes.c_int32 * max(1, len(perm)))(*perm)
    rc = lib.oracle_permute(x.ctypes.data, out.ctypes.data, len(shape), sh, pm, x.itemsize,
                            nthreads)
    if rc != 0:
        raise ValueError("oracle_permute: bad arguments")
    return out


def contract(a: np.ndarray, a_shape, a_perm, b: np.ndarray, b_shape, b_perm, m: int, n: int,
             k: int, nthreads: int = 0) -> np.ndarray:
    """Tensor::ContractTensors data path: transpose both operands, then one
    row-major complex GEMM (alpha = 1, beta = 0)."""
    at = permute(a, a_shape, a_perm, nthreads)
    bt = permute(b, b_shape, b_perm, nthreads)
    return np.matmul(at.reshape(m, k), bt.reshape(k, n)).reshape(-1)
