"""ctypes binding of the C-ABI library libjetgpu.so (include/jetgpu.h).

This is the Python-side FFI a maintainer of the reference would add next to
its pybind bindings: plain pointers, sizes and a stream, int status codes.
Device memory and streams come from PyTorch (torch.cuda tensors); PyTorch is
plumbing here, every computation runs in libjetgpu.so.

Importing this module fails loudly (ImportError) when the library has not
been built; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import re
from typing import List, Optional, Sequence

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libjetgpu.so")
HEADER_PATH = os.path.join(os.path.dirname(_PKG), "include", "jetgpu.h")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        "libjetgpu.so is not built; run `python -c \"import __graft_entry__ as g; g.build()\"` "
        "or `python -m jet_gb300.build`")

lib = ctypes.CDLL(LIB_PATH)

OK = 0
ERR_INVALID = 1
ERR_CUDA = 2
ERR_UNSUPPORTED = 3
ERR_WORKSPACE = 4
ERR_TIMEOUT = 5
ERR_MEMORY = 6

C64 = 0
C128 = 1

PREC_FP32 = 0
PREC_TF32X3 = 1
PREC_AUTO = 2
PREC_BF16X3 = 3
PREC_FP16X3 = 4
PREC_TUNED = 5

ALGO_4M = 0
ALGO_3M = 1

# Word formats of the split stages (jetgpu_split_planes / jetgpu_gemm_split).
FMT_TF32 = 0
FMT_BF16 = 1
FMT_FP16 = 2
SPLIT_NEG_IM = 1  # extra planes 4, 5: -im hi, lo (B of the N = 256 main loop)
SPLIT_SUM = 2  # extra planes 4, 5: hi, lo of re + im (3M operands)

_u64p = ctypes.POINTER(ctypes.c_uint64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_vp = ctypes.c_void_p

lib.jetgpu_last_error.restype = ctypes.c_char_p
lib.jetgpu_contract_workspace_size.restype = ctypes.c_size_t
lib.jetgpu_contract_workspace_size.argtypes = [ctypes.c_int, _u64p, _i32p, ctypes.c_int, _u64p,
                                               _i32p, ctypes.c_uint64, ctypes.c_uint64,
                                               ctypes.c_uint64, ctypes.c_int, ctypes.c_int]
lib.jetgpu_contract_workspace_size_algo.restype = ctypes.c_size_t
lib.jetgpu_contract_workspace_size_algo.argtypes = [
    ctypes.c_int, _u64p, _i32p, ctypes.c_int, _u64p, _i32p, ctypes.c_uint64, ctypes.c_uint64,
    ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int]
lib.jetgpu_split_planes.argtypes = [_vp, ctypes.c_int, _u64p, _i32p, ctypes.c_uint64,
                                    ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                    ctypes.c_int, ctypes.c_int, _vp, _vp, _vp]
lib.jetgpu_gemm_split.argtypes = [_vp, _vp, _vp, ctypes.c_uint64, ctypes.c_uint64,
                                  ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, _vp, ctypes.c_float, _vp]
lib.jetgpu_permute.argtypes = [_vp, _vp, ctypes.c_int, _u64p, _i32p, ctypes.c_int, _vp]
lib.jetgpu_permute_batched.argtypes = [_vp, _vp, ctypes.c_uint64, ctypes.c_int, _u64p, _i32p,
                                       ctypes.c_int, _vp]
lib.jetgpu_multiply.argtypes = [_vp, _vp, _vp, ctypes.c_uint64, ctypes.c_uint64,
                                ctypes.c_uint64, ctypes.c_int, _vp]
lib.jetgpu_contract.argtypes = [_vp, ctypes.c_int, _u64p, _i32p, _vp, ctypes.c_int, _u64p, _i32p,
                                _vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int, _vp, ctypes.c_size_t, _vp]
lib.jetgpu_split_tf32.argtypes = [_vp, ctypes.c_int, _u64p, _i32p, ctypes.c_uint64,
                                  ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                                  ctypes.c_int, _vp, _vp]
lib.jetgpu_set_tc_variant.argtypes = [ctypes.c_int]
lib.jetgpu_set_tc_persistent.argtypes = [ctypes.c_int]
lib.jetgpu_set_tc_group_m.argtypes = [ctypes.c_int]
lib.jetgpu_set_tc_chunk_depth.argtypes = [ctypes.c_int]
lib.jetgpu_set_auto_form.argtypes = [ctypes.c_int]
lib.jetgpu_gemm_tf32x3.argtypes = [_vp, _vp, _vp, ctypes.c_uint64, ctypes.c_uint64,
                                   ctypes.c_uint64, ctypes.c_uint64, ctypes.c_float, _vp]
lib.jetgpu_split_bf16.argtypes = [_vp, ctypes.c_int, _u64p, _i32p, ctypes.c_uint64,
                                  ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                                  _vp, _vp]
lib.jetgpu_gemm_bf16x3.argtypes = [_vp, _vp, _vp, ctypes.c_uint64, ctypes.c_uint64,
                                   ctypes.c_uint64, ctypes.c_uint64, ctypes.c_float, _vp]
lib.jetgpu_split_fp16.argtypes = [_vp, ctypes.c_int, _u64p, _i32p, ctypes.c_uint64,
                                  ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, _vp, _vp, _vp]
lib.jetgpu_gemm_fp16x3.argtypes = [_vp, _vp, _vp, ctypes.c_uint64, ctypes.c_uint64,
                                   ctypes.c_uint64, ctypes.c_uint64, _vp, ctypes.c_float, _vp]
lib.jetgpu_contract_batched_workspace_size.restype = ctypes.c_size_t
lib.jetgpu_contract_batched_workspace_size.argtypes = [
    ctypes.c_uint64, ctypes.c_int, _u64p, _i32p, ctypes.c_int, ctypes.c_int, _u64p, _i32p,
    ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int]
lib.jetgpu_contract_batched.argtypes = [
    ctypes.c_uint64, _vp, ctypes.c_int, _u64p, _i32p, ctypes.c_int, _vp, ctypes.c_int, _u64p,
    _i32p, ctypes.c_int, _vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
    ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_size_t, _vp]
lib.jetgpu_contract_batched_hinted.argtypes = [
    ctypes.c_uint64, _vp, ctypes.c_int, _u64p, _i32p, ctypes.c_int, _vp, ctypes.c_int, _u64p,
    _i32p, ctypes.c_int, _vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
    ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp, ctypes.c_size_t, _vp]
class GroupTask(ctypes.Structure):
    """jetgpu_group_task (include/jetgpu.h)."""
    _fields_ = [("A", _vp), ("B", _vp), ("C", _vp), ("batch", ctypes.c_uint64),
                ("m", ctypes.c_uint64), ("n", ctypes.c_uint64), ("k", ctypes.c_uint64),
                ("a_bat", _vp), ("a_row", _vp), ("a_col", _vp),
                ("b_bat", _vp), ("b_row", _vp), ("b_col", _vp)]


lib.jetgpu_group_tiles.restype = ctypes.c_uint64
lib.jetgpu_group_tiles.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
lib.jetgpu_contract_group.argtypes = [_vp, ctypes.c_int, ctypes.c_uint64, ctypes.c_int, _vp]
lib.jetgpu_add.argtypes = [_vp, _vp, _vp, ctypes.c_uint64, ctypes.c_int, _vp]
lib.jetgpu_conj.argtypes = [_vp, _vp, ctypes.c_uint64, ctypes.c_int, _vp]
lib.jetgpu_slice_sum_f64.argtypes = [_vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, _vp,
                                     ctypes.c_int, _vp]
lib.jetgpu_slice_gather.argtypes = [_vp, ctypes.c_int, _u64p, ctypes.c_int, _i32p, _u64p,
                                    ctypes.c_uint64, ctypes.c_uint64, _vp, ctypes.c_int, _vp]
lib.jetgpu_max_exponent.argtypes = [_vp, ctypes.c_uint64, ctypes.c_int, _vp, _vp]
lib.jetgpu_slice_scatter_add.argtypes = [_vp, ctypes.c_int, _u64p, ctypes.c_int, _i32p, _u64p,
                                         ctypes.c_uint64, _vp, ctypes.c_int, _vp]
lib.jetgpu_take_device_status.argtypes = [ctypes.POINTER(ctypes.c_int)]
lib.jetgpu_probe_bounded_wait.argtypes = [ctypes.c_uint, _vp]
lib.jetgpu_device_info.argtypes = [ctypes.POINTER(ctypes.c_int)] * 3
lib.jetgpu_set_autotune_min_work.argtypes = [ctypes.c_uint64]
lib.jetgpu_autotune_count.restype = ctypes.c_size_t
lib.jetgpu_autotune_count.argtypes = []
lib.jetgpu_autotune_entry.argtypes = [ctypes.c_size_t, _u64p, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_float)]
lib.jetgpu_malloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(_vp)]
lib.jetgpu_free.argtypes = [_vp]
lib.jetgpu_set_pool_limit.argtypes = [ctypes.c_size_t]
lib.jetgpu_pool_bytes_in_use.restype = ctypes.c_size_t
lib.jetgpu_pool_bytes_in_use.argtypes = []
lib.jetgpu_range_push.argtypes = [ctypes.c_char_p]
lib.jetgpu_range_push.restype = None
lib.jetgpu_range_pop.argtypes = []
lib.jetgpu_range_pop.restype = None


class JetGpuError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"jetgpu error {code}: {msg}")
        self.code = code


def check(rc: int) -> None:
    if rc != OK:
        raise JetGpuError(rc, lib.jetgpu_last_error().decode())


def declared_symbols() -> List[str]:
    """Entry points declared in include/jetgpu.h."""
    text = open(HEADER_PATH).read()
    return sorted(set(re.findall(r"\b(jetgpu_\w+)\s*\(", text)))


def u64(vals: Sequence[int]):
    return (ctypes.c_uint64 * max(1, len(vals)))(*[int(v) for v in vals])


def i32(vals: Sequence[int]):
    return (ctypes.c_int32 * max(1, len(vals)))(*[int(v) for v in vals])


def dtype_code(dtype) -> int:
    import torch

    if dtype in (torch.complex64, np.complex64) or str(dtype) in ("complex64", "torch.complex64"):
        return C64
    if dtype in (torch.complex128, np.complex128) or str(dtype) in ("complex128", "torch.complex128"):
        return C128
    raise TypeError(f"unsupported dtype {dtype}")


def _stream(stream) -> Optional[int]:
    import torch

    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _ptr(t) -> Optional[int]:
    return None if t is None else t.data_ptr()


def permute(x, shape: Sequence[int], perm: Sequence[int], out=None, batch: int = 1, stream=None):
    """out[new] = x[old], new axis j = old axis perm[j] (batch tensors back to back)."""
    import torch

    if out is None:
        out = torch.empty_like(x)
    if batch == 1:
        rc = lib.jetgpu_permute(_ptr(x), _ptr(out), len(shape), u64(shape), i32(perm),
                                dtype_code(x.dtype), _stream(stream))
    else:
        rc = lib.jetgpu_permute_batched(_ptr(x), _ptr(out), batch, len(shape), u64(shape),
                                        i32(perm), dtype_code(x.dtype), _stream(stream))
    check(rc)
    return out


def multiply(a, b, m: int, n: int, k: int, out=None, stream=None):
    import torch

    if out is None:
        out = torch.empty(m * n, dtype=a.dtype, device=a.device)
    check(lib.jetgpu_multiply(_ptr(a), _ptr(b), _ptr(out), m, n, k, dtype_code(a.dtype),
                              _stream(stream)))
    return out


def contract_workspace_size(a_shape, a_perm, b_shape, b_perm, m, n, k, dtype_c, precision,
                            algo=ALGO_4M) -> int:
    return int(lib.jetgpu_contract_workspace_size_algo(len(a_shape), u64(a_shape), i32(a_perm),
                                                       len(b_shape), u64(b_shape), i32(b_perm),
                                                       m, n, k, dtype_c, precision, algo))


def contract(a, a_shape, a_perm, b, b_shape, b_perm, m, n, k, precision=PREC_FP32,
             out=None, workspace=None, scale_a=0, scale_b=0, stream=None, algo=ALGO_4M):
    """C[m x n] = permute(A)[m x k] permute(B)[k x n] through jetgpu_contract
    (algo ALGO_3M: three real products, split forms only)."""
    import torch

    dc = dtype_code(a.dtype)
    if out is None:
        out = torch.empty(max(m * n, 1), dtype=a.dtype, device=a.device)
    need = contract_workspace_size(a_shape, a_perm, b_shape, b_perm, m, n, k, dc, precision,
                                   algo)
    if workspace is None and need:
        workspace = torch.empty(need, dtype=torch.uint8, device=a.device)
    ws_bytes = 0 if workspace is None else workspace.numel() * workspace.element_size()
    check(lib.jetgpu_contract(_ptr(a), len(a_shape), u64(a_shape), i32(a_perm), _ptr(b),
                              len(b_shape), u64(b_shape), i32(b_perm), _ptr(out), m, n, k, dc,
                              precision, algo, scale_a, scale_b, _ptr(workspace), ws_bytes,
                              _stream(stream)))
    return out


def contract_batched(batch, a, a_shape, a_perm, a_batched, b, b_shape, b_perm, b_batched,
                     m, n, k, precision=PREC_FP32, out=None, workspace=None, stream=None):
    """C[b] = contract(A[b], B[b]) (shared operands have a_batched/b_batched False)."""
    import torch

    dc = dtype_code(a.dtype)
    if out is None:
        out = torch.empty(max(batch * m * n, 1), dtype=a.dtype, device=a.device)
    need = int(lib.jetgpu_contract_batched_workspace_size(
        batch, len(a_shape), u64(a_shape), i32(a_perm), int(a_batched), len(b_shape),
        u64(b_shape), i32(b_perm), int(b_batched), m, n, k, dc, precision))
    if workspace is None and need:
        workspace = torch.empty(need, dtype=torch.uint8, device=a.device)
    ws_bytes = 0 if workspace is None else workspace.numel() * workspace.element_size()
    check(lib.jetgpu_contract_batched(batch, _ptr(a), len(a_shape), u64(a_shape), i32(a_perm),
                                      int(a_batched), _ptr(b), len(b_shape), u64(b_shape),
                                      i32(b_perm), int(b_batched), _ptr(out), m, n, k, dc,
                                      precision, ALGO_4M, 0, 0, _ptr(workspace), ws_bytes,
                                      _stream(stream)))
    return out


def contract_batched_hinted(batch, a, a_shape, a_perm, a_batched, b, b_shape, b_perm, b_batched,
                            m, n, k, precision=PREC_FP32, a_emax=None, b_emax=None, c_emax=None,
                            out=None, workspace=None, stream=None):
    """contract_batched passing max-exponent hints (device int32 tensors of one
    element, or None): a_emax / b_emax known exponents of the operands,
    c_emax receives C's when the product runs on the tensor cores."""
    import torch

    dc = dtype_code(a.dtype)
    if out is None:
        out = torch.empty(max(batch * m * n, 1), dtype=a.dtype, device=a.device)
    need = int(lib.jetgpu_contract_batched_workspace_size(
        batch, len(a_shape), u64(a_shape), i32(a_perm), int(a_batched), len(b_shape),
        u64(b_shape), i32(b_perm), int(b_batched), m, n, k, dc, precision))
    if workspace is None and need:
        workspace = torch.empty(need, dtype=torch.uint8, device=a.device)
    ws_bytes = 0 if workspace is None else workspace.numel() * workspace.element_size()
    check(lib.jetgpu_contract_batched_hinted(
        batch, _ptr(a), len(a_shape), u64(a_shape), i32(a_perm), int(a_batched), _ptr(b),
        len(b_shape), u64(b_shape), i32(b_perm), int(b_batched), _ptr(out), m, n, k, dc,
        precision, ALGO_4M, _ptr(a_emax), _ptr(b_emax), _ptr(c_emax), _ptr(workspace), ws_bytes,
        _stream(stream)))
    return out


def view_offsets(shape, axes):
    """Element offsets in a row-major tensor of `shape` of every index
    combination of `axes` (first axis slowest): a grouped task's table."""
    import numpy as np

    strides = [1] * len(shape)
    for j in range(len(shape) - 2, -1, -1):
        strides[j] = strides[j + 1] * shape[j + 1]
    out = np.zeros(1, dtype=np.int64)
    for ax in axes:
        out = (out[:, None] + np.arange(shape[ax], dtype=np.int64)[None, :] * strides[ax]).ravel()
    return out


def contract_group(tasks, stream=None):
    """Grouped launch (jetgpu_contract_group). `tasks`: list of dicts with
    A, B, C (device tensors of one dtype), batch, m, n, k and the six offset
    tables a_bat, a_row, a_col, b_bat, b_row, b_col (int64 device tensors).
    Returns the device buffer holding the task array (keep it alive until the
    launch has run)."""
    import torch

    if not tasks:
        return None
    arr = (GroupTask * len(tasks))()
    total = 0
    for q, t in zip(arr, tasks):
        q.A, q.B, q.C = _ptr(t["A"]), _ptr(t["B"]), _ptr(t["C"])
        q.batch, q.m, q.n, q.k = t["batch"], t["m"], t["n"], t["k"]
        for f in ("a_bat", "a_row", "a_col", "b_bat", "b_row", "b_col"):
            setattr(q, f, _ptr(t[f]))
        total += int(lib.jetgpu_group_tiles(t["batch"], t["m"], t["n"]))
    dev = tasks[0]["A"].device
    raw = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(dev)
    check(lib.jetgpu_contract_group(_ptr(raw), len(tasks), total,
                                    dtype_code(tasks[0]["A"].dtype), _stream(stream)))
    return raw


def contract_group_at(tasks_ptr: int, n_tasks: int, total_tiles: int, dtype_c: int,
                      stream=None) -> None:
    """jetgpu_contract_group on a task array already on the device (its
    address, task count, summed jetgpu_group_tiles and dtype code)."""
    check(lib.jetgpu_contract_group(tasks_ptr, n_tasks, total_tiles, dtype_c, _stream(stream)))


def split_tf32(x, shape, perm, rows, cols, pitch, planes, scale_exp=0, n_planes=4,
               stream=None):
    """Permute + TF32 hi/lo split into 4 (or 6) planes of rows x pitch floats."""
    check(lib.jetgpu_split_tf32(_ptr(x), len(shape), u64(shape), i32(perm), rows, cols, pitch,
                                rows * pitch, scale_exp, n_planes, _ptr(planes),
                                _stream(stream)))
    return planes


def set_tc_variant(variant: int) -> None:
    """0: default main loops; 1: TF32 with N = 256 MMAs (six B planes);
    2: BF16 with 32-byte rows in 6 stages."""
    check(lib.jetgpu_set_tc_variant(int(variant)))


def set_tc_persistent(on: bool) -> None:
    """Tensor-core products as one persistent CTA per SM (default) or one CTA
    per tile."""
    check(lib.jetgpu_set_tc_persistent(int(bool(on))))


def set_tc_group_m(group_m: int) -> None:
    """Tile rows per group of the tensor-core products' tile order (default 8)."""
    check(lib.jetgpu_set_tc_group_m(int(group_m)))


def set_auto_form(precision: int) -> None:
    """Split form of PREC_AUTO's tensor-core steps: PREC_FP16X3 (default),
    PREC_TF32X3 or PREC_BF16X3."""
    check(lib.jetgpu_set_auto_form(int(precision)))


def set_tc_chunk_depth(k_depth: int) -> None:
    """K depth accumulated in tensor memory per fold (0 = defaults)."""
    check(lib.jetgpu_set_tc_chunk_depth(int(k_depth)))


def tc_b_planes() -> int:
    return int(lib.jetgpu_tc_b_planes())


def gemm_tf32x3(a_planes, b_planes, m, n, k, kpitch, out, out_scale=1.0, stream=None):
    check(lib.jetgpu_gemm_tf32x3(_ptr(a_planes), _ptr(b_planes), _ptr(out), m, n, k, kpitch,
                                 out_scale, _stream(stream)))
    return out


def split_bf16(x, shape, perm, rows, cols, pitch, planes, scale_exp=0, stream=None):
    """Permute + BF16 hi/lo split into 4 planes of rows x pitch 16-bit words."""
    check(lib.jetgpu_split_bf16(_ptr(x), len(shape), u64(shape), i32(perm), rows, cols, pitch,
                                rows * pitch, scale_exp, _ptr(planes), _stream(stream)))
    return planes


def gemm_bf16x3(a_planes, b_planes, m, n, k, kpitch, out, out_scale=1.0, stream=None):
    check(lib.jetgpu_gemm_bf16x3(_ptr(a_planes), _ptr(b_planes), _ptr(out), m, n, k, kpitch,
                                 out_scale, _stream(stream)))
    return out


def split_fp16(x, shape, perm, rows, cols, pitch, planes, e_max, stream=None):
    """Permute + FP16 hi/lo split of x scaled by 2^(14 - *e_max) (e_max: a
    device int32 tensor holding the max exponent of x)."""
    check(lib.jetgpu_split_fp16(_ptr(x), len(shape), u64(shape), i32(perm), rows, cols, pitch,
                                rows * pitch, _ptr(e_max), _ptr(planes), _stream(stream)))
    return planes


def gemm_fp16x3(a_planes, b_planes, m, n, k, kpitch, out, e_max2, out_scale=1.0, stream=None):
    """FP16x3 product of split planes; e_max2: device int32[2], the max
    exponents of A and B."""
    check(lib.jetgpu_gemm_fp16x3(_ptr(a_planes), _ptr(b_planes), _ptr(out), m, n, k, kpitch,
                                 _ptr(e_max2), out_scale, _stream(stream)))
    return out


def split_planes(x, shape, perm, rows, cols, pitch, planes, fmt, extra=0, e_max=None,
                 stream=None):
    """Permute + hi/lo split in any word format (FMT_TF32 / FMT_BF16 / FMT_FP16)
    into 4 planes, or 6 with extra=SPLIT_SUM (hi, lo of re + im: 3M operands;
    FP16 then scales by 2^(13 - *e_max))."""
    check(lib.jetgpu_split_planes(_ptr(x), len(shape), u64(shape), i32(perm), rows, cols, pitch,
                                  rows * pitch, int(fmt), int(extra), _ptr(e_max), _ptr(planes),
                                  _stream(stream)))
    return planes


def gemm_split(a_planes, b_planes, m, n, k, kpitch, out, fmt, algo=ALGO_4M, e_max2=None,
               out_scale=1.0, stream=None, variant=0):
    """Split-precision product of planes written by split_planes (ALGO_3M
    reads six planes per operand; variant 1, the N = 256 main loop, six B
    planes written with extra=SPLIT_NEG_IM)."""
    check(lib.jetgpu_gemm_split(_ptr(a_planes), _ptr(b_planes), _ptr(out), m, n, k, kpitch,
                                int(fmt), int(algo), int(variant), _ptr(e_max2), out_scale,
                                _stream(stream)))
    return out


def add(a, b, out=None, stream=None):
    import torch

    if out is None:
        out = torch.empty_like(a)
    check(lib.jetgpu_add(_ptr(a), _ptr(b), _ptr(out), a.numel(), dtype_code(a.dtype),
                         _stream(stream)))
    return out


def conj(a, out=None, stream=None):
    import torch

    if out is None:
        out = torch.empty_like(a)
    check(lib.jetgpu_conj(_ptr(a), _ptr(out), a.numel(), dtype_code(a.dtype), _stream(stream)))
    return out


def slice_sum_f64(results, n_slices: int, size: int, out=None, accumulate=False, stream=None):
    import torch

    if out is None:
        out = torch.zeros(size, dtype=torch.complex128, device=results.device)
    check(lib.jetgpu_slice_sum_f64(_ptr(results), n_slices, size, dtype_code(results.dtype),
                                   _ptr(out), int(bool(accumulate)), _stream(stream)))
    return out


def slice_gather(x, shape, axes, value_strides, first_value, n_values, out=None, stream=None):
    import torch

    fixed = set(axes)
    out_size = 1
    for i, d in enumerate(shape):
        if i not in fixed:
            out_size *= int(d)
    if out is None:
        out = torch.empty(max(out_size * n_values, 1), dtype=x.dtype, device=x.device)
    check(lib.jetgpu_slice_gather(_ptr(x), len(shape), u64(shape), len(axes), i32(axes),
                                  u64(value_strides), first_value, n_values, _ptr(out),
                                  dtype_code(x.dtype), _stream(stream)))
    return out


def slice_scatter_add(sliced, shape, axes, value_strides, value, full, stream=None):
    """full[positions of slice `value`] += sliced (adjoint of slice_gather for
    one slice value); returns `full`."""
    check(lib.jetgpu_slice_scatter_add(_ptr(sliced), len(shape), u64(shape), len(axes),
                                       i32(axes), u64(value_strides), int(value), _ptr(full),
                                       dtype_code(full.dtype), _stream(stream)))
    return full


def max_exponent(x, stream=None, out=None):
    """Max binary exponent of |re|, |im| over x: an int, or written (without
    synchronising) into the device int32 tensor `out` when one is given."""
    import torch

    e = out if out is not None else torch.empty(1, dtype=torch.int32, device=x.device)
    check(lib.jetgpu_max_exponent(_ptr(x), x.numel(), dtype_code(x.dtype), _ptr(e),
                                  _stream(stream)))
    return e if out is not None else int(e.item())


AUTOTUNE_CANDIDATES = ("fp32", "tf32x3", "tf32x3_wide", "fp16x3", "fp16x3_rowmajor",
                       "fp16x3_wide")


def set_autotune_min_work(mnk: int) -> None:
    """PREC_TUNED tunes contractions whose m n k times the batch is at least
    `mnk` (default 2^20); smaller ones take AUTO's rule."""
    check(lib.jetgpu_set_autotune_min_work(int(mnk)))


def autotune_clear() -> None:
    check(lib.jetgpu_autotune_clear())


def autotune_table():
    """The autotuner's entries: batch, m, n, k, the chosen form and the
    measured ms per contraction of each candidate (None: not timed)."""
    out = []
    for i in range(int(lib.jetgpu_autotune_count())):
        bmnk = (ctypes.c_uint64 * 4)()
        prec, var, grp = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        times = (ctypes.c_float * len(AUTOTUNE_CANDIDATES))()
        check(lib.jetgpu_autotune_entry(i, bmnk, ctypes.byref(prec), ctypes.byref(var),
                                        ctypes.byref(grp), times))
        if prec.value == PREC_FP32:
            choice = "fp32"
        elif prec.value == PREC_FP16X3:
            choice = ("fp16x3_rowmajor" if grp.value == 1 else
                      "fp16x3_wide" if var.value == 1 else "fp16x3")
        else:
            choice = "tf32x3_wide" if var.value == 1 else "tf32x3"
        out.append({"batch": bmnk[0], "m": bmnk[1], "n": bmnk[2], "k": bmnk[3],
                    "choice": choice,
                    "ms": {c: (float(t) if t >= 0 else None)
                           for c, t in zip(AUTOTUNE_CANDIDATES, times)}})
    return out


def set_pool_limit(nbytes: int) -> None:
    """Caps the device bytes the library allocator may hold at once (0: no
    cap). Allocations past the cap fail with ERR_MEMORY before any CUDA call."""
    check(lib.jetgpu_set_pool_limit(int(nbytes)))


def pool_bytes_in_use() -> int:
    return int(lib.jetgpu_pool_bytes_in_use())


def malloc(nbytes: int) -> int:
    """Raw device allocation from the library allocator (an address)."""
    p = _vp()
    check(lib.jetgpu_malloc(int(nbytes), ctypes.byref(p)))
    return p.value or 0


def free(ptr: int) -> None:
    check(lib.jetgpu_free(_vp(ptr)))


class nvtx_range:
    """NVTX range over a `with` block (visible to nsys / ncu)."""

    def __init__(self, name: str):
        self.name = name.encode()

    def __enter__(self):
        lib.jetgpu_range_push(self.name)
        return self

    def __exit__(self, *exc):
        lib.jetgpu_range_pop()
        return False


def take_device_status() -> int:
    v = ctypes.c_int(0)
    check(lib.jetgpu_take_device_status(ctypes.byref(v)))
    return v.value


def device_info():
    sm, ma, mi = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
    check(lib.jetgpu_device_info(ctypes.byref(sm), ctypes.byref(ma), ctypes.byref(mi)))
    return sm.value, ma.value, mi.value
