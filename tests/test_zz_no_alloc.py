"""jetgpu_contract_noalloc, the contraction entry point that allocates nothing.

It serves callers that cannot allocate device memory at the time they
contract: work recorded inside a CUDA stream capture (cudaMalloc is illegal
there), hosts that keep the GPU under their own fixed memory budget, and loops
where an allocation would synchronise the device. Its scratch is one 32 MiB
array inside the library, shared by every call.

The test calls it through the C ABI twice in a row on different inputs and
compares each result with jetgpu_contract (caller-provided workspace) and
with the complex128 oracle contraction of the same labelled tensors, under
the tolerances of the other contraction tests: 1e-5 relative for complex64,
1e-12 for complex128. It also checks that a contraction needing more scratch
than the array holds is refused with a clear error. This file is collected
last so that a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _lib():
    from jet_gb300 import capi

    lib = capi.lib
    lib.jetgpu_contract_noalloc.argtypes = [
        ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64),
        ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p, ctypes.c_int,
        ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p,
        ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    lib.jetgpu_contract_noalloc_max_scratch.restype = ctypes.c_size_t
    return capi, lib


def _noalloc(capi, lib, a, a_shape, a_perm, b, b_shape, b_perm, m, n, k, precision):
    import torch

    out = torch.full((max(m * n, 1),), float("nan"), dtype=a.dtype, device=a.device)
    rc = lib.jetgpu_contract_noalloc(
        a.data_ptr(), len(a_shape), capi.u64(a_shape), capi.i32(a_perm), b.data_ptr(),
        len(b_shape), capi.u64(b_shape), capi.i32(b_perm), out.data_ptr(), m, n, k,
        capi.dtype_code(a.dtype), precision, capi.ALGO_4M, 0, 0,
        torch.cuda.current_stream().cuda_stream)
    capi.check(rc)
    return out


def _operands(seed, dtype, nl, nc, nr, dev):
    import torch

    from oracle import jet_oracle as jo

    left = ["l%d" % i for i in range(nl)]
    common = ["c%d" % i for i in range(nc)]
    right = ["r%d" % i for i in range(nr)]
    a_lab = [(left + common)[i] for i in cases.permutation(seed, nl + nc)]
    b_lab = [(common + right)[i] for i in cases.permutation(seed + 1, nc + nr)]
    a = cases.tensor_data(seed, [2] * (nl + nc), dtype)
    b = cases.tensor_data(seed + 2, [2] * (nc + nr), dtype)
    lft = [x for x in a_lab if x not in b_lab]
    com = [x for x in a_lab if x in b_lab]
    rgt = [x for x in b_lab if x not in a_lab]
    want = jo.contract_tensors(jo.OTensor.make(a_lab, [2] * (nl + nc), a, np.complex128),
                               jo.OTensor.make(b_lab, [2] * (nc + nr), b, np.complex128))
    return dict(oracle=np.asarray(want.data).reshape(-1),
                a=torch.from_numpy(a).to(dev), a_shape=[2] * (nl + nc),
                a_perm=[a_lab.index(x) for x in lft + com],
                b=torch.from_numpy(b).to(dev), b_shape=[2] * (nc + nr),
                b_perm=[b_lab.index(x) for x in com + rgt],
                m=2 ** nl, n=2 ** nr, k=2 ** nc)


def _rel(x, y):
    return float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))


@pytest.mark.parametrize("dtype,precision", [("complex64", 1), ("complex64", 0),
                                             ("complex128", 0)])
def test_noalloc_matches_contract_twice(cuda, dtype, precision):
    import torch

    capi, lib = _lib()
    tol = 1e-5 if dtype == "complex64" else 1e-12
    for call, seed in enumerate((71, 83)):  # two calls in a row, different inputs
        o = _operands(seed, dtype, 9, 9, 8, cuda)
        got = _noalloc(capi, lib, o["a"], o["a_shape"], o["a_perm"], o["b"], o["b_shape"],
                       o["b_perm"], o["m"], o["n"], o["k"], precision)
        want = capi.contract(o["a"], o["a_shape"], o["a_perm"], o["b"], o["b_shape"],
                             o["b_perm"], o["m"], o["n"], o["k"], precision=precision)
        torch.cuda.synchronize()
        g = got.cpu().numpy()
        w = want.cpu().numpy()
        assert np.all(np.isfinite(g)), call
        assert _rel(g, w) <= tol, (call, _rel(g, w))
        assert _rel(g, o["oracle"]) <= tol, (call, _rel(g, o["oracle"]))
    assert capi.take_device_status() == 0


def test_noalloc_rejects_oversized_contraction(cuda):
    import torch

    capi, lib = _lib()
    limit = lib.jetgpu_contract_noalloc_max_scratch()
    assert limit == 32 << 20
    # TF32x3 scratch is 16 * (M + N) * K bytes: M = N = K = 2^11 needs 128 MiB.
    m = n = k = 2 ** 11
    a = torch.zeros(m * k, dtype=torch.complex64, device=cuda)
    b = torch.zeros(k * n, dtype=torch.complex64, device=cuda)
    c = torch.zeros(m * n, dtype=torch.complex64, device=cuda)
    rc = lib.jetgpu_contract_noalloc(
        a.data_ptr(), 2, capi.u64([m, k]), capi.i32([0, 1]), b.data_ptr(), 2,
        capi.u64([k, n]), capi.i32([0, 1]), c.data_ptr(), m, n, k, capi.C64, capi.PREC_TF32X3,
        capi.ALGO_4M, 0, 0, torch.cuda.current_stream().cuda_stream)
    assert rc == capi.ERR_WORKSPACE
    assert b"allocation-free entry point" in lib.jetgpu_last_error()
