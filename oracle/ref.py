"""ctypes access to oracle/_ref/libjetref.so: the reference Jet headers
compiled unmodified in this container (recipe: oracle/ref_build/Makefile).

TEST INFRASTRUCTURE ONLY: used to pin the oracle restatement and to generate
the golden fixtures under tests/golden/. The library is x86-only and is not
present on machines where the reference tree is absent; callers must treat
`available()` == False as "skip".
"""
from __future__ import annotations

import ctypes
import os
from typing import List, Optional, Sequence, Tuple

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_ref", "libjetref.so")
_lib = None


def available() -> bool:
    return _load() is not None


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        return None
    try:
        _lib = ctypes.CDLL(_LIB_PATH)
    except OSError:
        return None
    _lib.jetref_last_error.restype = ctypes.c_char_p
    return _lib


class RefError(RuntimeError):
    pass


def _sz(vals: Sequence[int]):
    arr = (ctypes.c_size_t * max(1, len(vals)))(*[int(v) for v in vals])
    return arr


def _labels(labels: Sequence[str]) -> bytes:
    return ",".join(labels).encode()


def _dt(dtype) -> Tuple[int, np.dtype]:
    dt = np.dtype(dtype)
    if dt == np.complex64:
        return 0, dt
    if dt == np.complex128:
        return 1, dt
    raise TypeError(dtype)


def _check(rc: int):
    if rc != 0:
        raise RefError(_load().jetref_last_error().decode())


def _out_buffers(cap: int, dt):
    rank = ctypes.c_size_t(0)
    shape = (ctypes.c_size_t * 64)()
    labels = ctypes.create_string_buffer(1 << 16)
    data = np.zeros(max(1, cap), dtype=dt)
    return rank, shape, labels, data


def _unpack(rank, shape, labels, data):
    r = rank.value
    sh = [int(shape[i]) for i in range(r)]
    lb_str = labels.value.decode()
    lb = lb_str.split(",") if lb_str else []
    n = 1
    for d in sh:
        n *= d
    return lb, sh, data[:n].copy()


def tensor_transpose(data: np.ndarray, shape, old_labels, new_labels) -> np.ndarray:
    lib = _load()
    code, dt = _dt(data.dtype)
    inp = np.ascontiguousarray(data, dtype=dt)
    out = np.zeros_like(inp)
    _check(lib.jetref_tensor_transpose(code, ctypes.c_size_t(len(shape)), _sz(shape),
                                       _labels(old_labels), _labels(new_labels),
                                       inp.ctypes.data_as(ctypes.c_void_p),
                                       out.ctypes.data_as(ctypes.c_void_p)))
    return out


def permuter_transpose(backend: int, data: np.ndarray, shape, old_labels, new_labels) -> np.ndarray:
    """backend 0 = DefaultPermuter<1024>, 1 = QFlexPermuter<1024,32>,
    2 = QFlexPermuter<64,32>; complex64 data."""
    lib = _load()
    inp = np.ascontiguousarray(data, dtype=np.complex64)
    n = 1
    for d in shape:
        n *= int(d)
    out = np.zeros(max(n, inp.size, 1), dtype=np.complex64)
    _check(lib.jetref_permuter_transpose(backend, ctypes.c_size_t(len(shape)), _sz(shape),
                                         _labels(old_labels), _labels(new_labels),
                                         inp.ctypes.data_as(ctypes.c_void_p),
                                         ctypes.c_size_t(inp.size),
                                         out.ctypes.data_as(ctypes.c_void_p)))
    return out[:n]


def contract(a_labels, a_shape, a_data, b_labels, b_shape, b_data):
    lib = _load()
    code, dt = _dt(a_data.dtype)
    a = np.ascontiguousarray(a_data, dtype=dt)
    b = np.ascontiguousarray(b_data, dtype=dt)
    cap = a.size * b.size + 1
    rank, shape, labels, data = _out_buffers(cap, dt)
    _check(lib.jetref_contract(code, ctypes.c_size_t(len(a_shape)), _sz(a_shape), _labels(a_labels),
                               a.ctypes.data_as(ctypes.c_void_p),
                               ctypes.c_size_t(len(b_shape)), _sz(b_shape), _labels(b_labels),
                               b.ctypes.data_as(ctypes.c_void_p),
                               ctypes.byref(rank), shape, labels, ctypes.c_size_t(len(labels)),
                               data.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(data.size)))
    return _unpack(rank, shape, labels, data)


def slice_index(labels_, shape_, data_, index: str, value: int):
    lib = _load()
    code, dt = _dt(data_.dtype)
    a = np.ascontiguousarray(data_, dtype=dt)
    rank, shape, labels, data = _out_buffers(a.size, dt)
    _check(lib.jetref_slice_index(code, ctypes.c_size_t(len(shape_)), _sz(shape_), _labels(labels_),
                                  a.ctypes.data_as(ctypes.c_void_p), index.encode(),
                                  ctypes.c_size_t(value), ctypes.byref(rank), shape, labels,
                                  ctypes.c_size_t(len(labels)), data.ctypes.data_as(ctypes.c_void_p),
                                  ctypes.c_size_t(data.size)))
    return _unpack(rank, shape, labels, data)


def add_tensors(a_labels, a_shape, a_data, b_labels, b_shape, b_data):
    lib = _load()
    code, dt = _dt(a_data.dtype)
    a = np.ascontiguousarray(a_data, dtype=dt)
    b = np.ascontiguousarray(b_data, dtype=dt)
    rank, shape, labels, data = _out_buffers(max(a.size, b.size), dt)
    _check(lib.jetref_add_tensors(code, ctypes.c_size_t(len(a_shape)), _sz(a_shape), _labels(a_labels),
                                  a.ctypes.data_as(ctypes.c_void_p),
                                  ctypes.c_size_t(len(b_shape)), _sz(b_shape), _labels(b_labels),
                                  b.ctypes.data_as(ctypes.c_void_p),
                                  ctypes.byref(rank), shape, labels, ctypes.c_size_t(len(labels)),
                                  data.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(data.size)))
    return _unpack(rank, shape, labels, data)


def network_contract(tensors: List[Tuple[List[str], List[int], np.ndarray]],
                     path: Sequence[Tuple[int, int]], sliced: Sequence[str] = (),
                     slice_value: int = 0, out_cap: Optional[int] = None):
    """Returns (labels, shape, data, total_flops, total_memory)."""
    lib = _load()
    code, dt = _dt(tensors[0][2].dtype)
    ranks = [len(t[1]) for t in tensors]
    shapes_flat = [d for t in tensors for d in t[1]]
    keep = [np.ascontiguousarray(t[2], dtype=dt) for t in tensors]
    labels_arr = (ctypes.c_char_p * len(tensors))(*[_labels(t[0]) for t in tensors])
    datas = (ctypes.c_void_p * len(tensors))(*[k.ctypes.data for k in keep])
    flat_path = [int(x) for p in path for x in p]
    cap = out_cap or (1 << 22)
    rank, shape, labels, data = _out_buffers(cap, dt)
    flops = ctypes.c_double(0)
    mem = ctypes.c_double(0)
    _check(lib.jetref_network_contract(code, ctypes.c_size_t(len(tensors)), _sz(ranks), _sz(shapes_flat),
                                       labels_arr, datas, ctypes.c_size_t(len(path)), _sz(flat_path),
                                       _labels(sliced), ctypes.c_ulonglong(slice_value),
                                       ctypes.byref(flops), ctypes.byref(mem), ctypes.byref(rank),
                                       shape, labels, ctypes.c_size_t(len(labels)),
                                       data.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(data.size)))
    lb, sh, d = _unpack(rank, shape, labels, data)
    return lb, sh, d, flops.value, mem.value
