"""Skinny contractions (skinny.cu): one side of the product at most 16 wide
and k <= 64, read from the operands' own layouts without transposes.

Checked against the complex128 oracle (Tensor::ContractTensors restated) on
gate-on-state shapes as the reference's networks have them -- qubit and
qutrit gates on any positions of a large tensor, gate first or second --
against the transposing path bit for bit (explicit jetgpu_permute +
jetgpu_multiply, which runs the same FMA sequence for m, n > 1), and through
the batched entry point against single contractions.

Tolerances (relative Frobenius error against complex128): complex64 1e-5
(FP32 FMA over k <= 64), complex128 1e-12."""
import numpy as np
import pytest

import cases
from oracle import jet_oracle as jo


def _plan(a_labels, a_shape, b_labels, b_shape):
    """Tensor::ContractTensors label algebra (Tensor.hpp:714-741)."""
    left = jo.vector_subtraction(a_labels, b_labels)
    right = jo.vector_subtraction(b_labels, a_labels)
    common = jo.vector_intersection(a_labels, b_labels)
    ad = dict(zip(a_labels, a_shape))
    bd = dict(zip(b_labels, b_shape))
    m = int(np.prod([ad[x] for x in left])) if left else 1
    n = int(np.prod([bd[x] for x in right])) if right else 1
    k = int(np.prod([ad[x] for x in common])) if common else 1
    return ([a_labels.index(x) for x in left + common], [b_labels.index(x) for x in common + right],
            m, n, k, left + right)


def _gate_case(seed, rank, dim, q_in, q_out, dtype):
    """A state-like tensor of `rank` axes of `dim` and a gate reading q_in of
    them (at seeded positions) and writing q_out new ones."""
    lab = ["s%d" % i for i in range(rank)]
    pos = cases.permutation(seed, rank)[:q_in]
    g_in = [lab[p] for p in pos]
    g_out = ["o%d" % i for i in range(q_out)]
    g_lab = g_out + g_in
    order = cases.permutation(seed + 5, len(g_lab))
    g_lab = [g_lab[i] for i in order]
    s_shape, g_shape = [dim] * rank, [dim] * len(g_lab)
    return (lab, s_shape, cases.tensor_data(seed, s_shape, dtype),
            g_lab, g_shape, cases.tensor_data(seed + 1, g_shape, dtype))


def _rel(got, want):
    return np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300)


def _dev(x, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(x).reshape(-1)).to(dev)


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
@pytest.mark.parametrize("dim,rank,q_in,q_out", [(2, 20, 1, 1), (2, 20, 2, 2), (2, 19, 3, 3),
                                                 (2, 18, 4, 4), (2, 18, 6, 1), (2, 18, 1, 0),
                                                 (2, 18, 3, 0), (3, 12, 1, 1), (3, 12, 2, 2),
                                                 (3, 11, 3, 1), (2, 16, 2, 3)])
@pytest.mark.parametrize("gate_first", [False, True])
def test_gate_on_state_matches_oracle(cuda, dtype, dim, rank, q_in, q_out, gate_first):
    from jet_gb300 import capi

    seed = 100 * dim + 10 * rank + 3 * q_in + q_out
    s_lab, s_shape, s, g_lab, g_shape, g = _gate_case(seed, rank, dim, q_in, q_out, dtype)
    if gate_first:
        a_lab, a_shape, a, b_lab, b_shape, b = g_lab, g_shape, g, s_lab, s_shape, s
    else:
        a_lab, a_shape, a, b_lab, b_shape, b = s_lab, s_shape, s, g_lab, g_shape, g
    a_perm, b_perm, m, n, k, lab = _plan(a_lab, a_shape, b_lab, b_shape)
    assert min(m, n) <= 16 and k <= 64
    assert capi.contract_workspace_size(a_shape, a_perm, b_shape, b_perm, m, n, k,
                                        capi.dtype_code(dtype), capi.PREC_FP32) == 0
    want = jo.contract_tensors(jo.OTensor.make(a_lab, a_shape, a, np.complex128),
                               jo.OTensor.make(b_lab, b_shape, b, np.complex128))
    assert want.indices == lab
    tol = 1e-5 if dtype == np.complex64 else 1e-12
    for prec in (capi.PREC_FP32, capi.PREC_AUTO):
        if dtype == np.complex128 and prec != capi.PREC_FP32:
            continue
        got = capi.contract(_dev(a, cuda), a_shape, a_perm, _dev(b, cuda), b_shape, b_perm, m, n,
                            k, precision=prec).cpu().numpy()[: m * n]
        assert _rel(got, want.data.reshape(-1)) <= tol, (prec, _rel(got, want.data.reshape(-1)))
    assert capi.take_device_status() == 0


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
@pytest.mark.parametrize("dim,rank,q_in,q_out", [(2, 8, 2, 2), (2, 10, 1, 1), (3, 5, 2, 2),
                                                 (2, 9, 6, 1), (2, 4, 1, 0), (3, 6, 1, 1),
                                                 (2, 12, 3, 3)])
@pytest.mark.parametrize("gate_first", [False, True])
def test_tiny_outputs_match_oracle_and_transposing_bits(cuda, dtype, dim, rank, q_in, q_out,
                                                        gate_first):
    """Outputs of at most 4096 elements (skinny_tiny_kernel: one thread per
    output, no shared memory): the oracle, and where m, n > 1 the same bits
    as permute + multiply."""
    import torch

    from jet_gb300 import capi

    seed = 1000 + 100 * dim + 10 * rank + 3 * q_in + q_out
    s_lab, s_shape, st, g_lab, g_shape, g = _gate_case(seed, rank, dim, q_in, q_out, dtype)
    if gate_first:
        a_lab, a_shape, a, b_lab, b_shape, b = g_lab, g_shape, g, s_lab, s_shape, st
    else:
        a_lab, a_shape, a, b_lab, b_shape, b = s_lab, s_shape, st, g_lab, g_shape, g
    a_perm, b_perm, m, n, k, lab = _plan(a_lab, a_shape, b_lab, b_shape)
    assert m * n <= 4096
    want = jo.contract_tensors(jo.OTensor.make(a_lab, a_shape, a, np.complex128),
                               jo.OTensor.make(b_lab, b_shape, b, np.complex128))
    da, db = _dev(a, cuda), _dev(b, cuda)
    got = capi.contract(da, a_shape, a_perm, db, b_shape, b_perm, m, n, k)
    tol = 1e-5 if dtype == np.complex64 else 1e-12
    assert _rel(got.cpu().numpy()[: m * n], want.data.reshape(-1)) <= tol
    if m > 1 and n > 1:
        ref = capi.multiply(capi.permute(da, a_shape, a_perm), capi.permute(db, b_shape, b_perm),
                            m, n, k)
        torch.cuda.synchronize()
        assert torch.equal(got[: m * n], ref[: m * n])


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
@pytest.mark.parametrize("q_in,q_out,gate_first", [(2, 2, False), (3, 3, True), (1, 1, False),
                                                   (4, 2, True), (6, 4, False)])
def test_same_bits_as_the_transposing_path(cuda, dtype, q_in, q_out, gate_first):
    """m, n > 1: the skinny kernel's FMA sequence is gemm_kernel's, so its
    result equals permute + multiply bit for bit."""
    import torch

    from jet_gb300 import capi

    s_lab, s_shape, s, g_lab, g_shape, g = _gate_case(7 + q_in, 17, 2, q_in, q_out, dtype)
    if gate_first:
        a_lab, a_shape, a, b_lab, b_shape, b = g_lab, g_shape, g, s_lab, s_shape, s
    else:
        a_lab, a_shape, a, b_lab, b_shape, b = s_lab, s_shape, s, g_lab, g_shape, g
    a_perm, b_perm, m, n, k, _ = _plan(a_lab, a_shape, b_lab, b_shape)
    assert m > 1 and n > 1
    da, db = _dev(a, cuda), _dev(b, cuda)
    got = capi.contract(da, a_shape, a_perm, db, b_shape, b_perm, m, n, k)
    at = capi.permute(da, a_shape, a_perm)
    bt = capi.permute(db, b_shape, b_perm)
    ref = capi.multiply(at, bt, m, n, k)
    torch.cuda.synchronize()
    assert torch.equal(got[: m * n], ref[: m * n])


def test_any_axis_order_and_unaligned_output(cuda):
    """Free axes in a shuffled order (rows over many index axes), unit axes,
    a scale, and an output 8 bytes off 16-byte alignment (no vector stores)."""
    import torch

    from jet_gb300 import capi

    rng = np.random.default_rng(3)
    shape = [2, 3, 1, 2, 5, 2, 3, 2, 7, 2, 1, 4]
    a = cases.tensor_data(31, shape, np.complex64)
    common_axes = [1, 9, 6]                       # k = 3 * 2 * 3 = 18
    free = [i for i in range(len(shape)) if i not in common_axes]
    free = [free[i] for i in rng.permutation(len(free))]
    a_perm = free + common_axes
    m = int(np.prod([shape[i] for i in free]))
    k = 18
    n = 4
    b = cases.tensor_data(32, [3, 4, 2, 3], np.complex64)  # axes (c1, j, c9, c6)
    b_shape, b_perm = [3, 4, 2, 3], [0, 2, 3, 1]
    a_t = np.transpose(a.astype(np.complex128).reshape(shape), a_perm).reshape(m, k)
    b_t = np.transpose(b.astype(np.complex128).reshape(b_shape), b_perm).reshape(k, n)
    want = (a_t @ b_t) * 2.0 ** 3
    for offset in (0, 1):
        buf = torch.empty(m * n + 1, dtype=torch.complex64, device=cuda)
        out = buf[offset:offset + m * n]
        capi.contract(_dev(a, cuda), shape, a_perm, _dev(b, cuda), b_shape, b_perm, m, n, k,
                      out=out, scale_a=5, scale_b=-2)
        got = out.cpu().numpy().reshape(m, n)
        assert _rel(got, want) <= 1e-5, offset


@pytest.mark.parametrize("s,k", [(5, 5), (6, 64), (7, 3), (10, 12), (12, 1), (15, 33)])
@pytest.mark.parametrize("gate_first", [False, True])
def test_widths_between_the_built_ones(cuda, s, k, gate_first):
    """Small extents the kernel rounds up (5-7 to 8, 10-15 to 16), with
    contracted extents that are not multiples of the load chunk, over a row
    count that ends in a partial warp."""
    from jet_gb300 import capi

    big_shape = [13, k, 31, 8]
    big = cases.tensor_data(600 + s, big_shape, np.complex64)
    small = cases.tensor_data(700 + k, [s, k], np.complex64)
    rows = 13 * 31 * 8
    big_t = np.transpose(big.astype(np.complex128).reshape(big_shape), [0, 2, 3, 1]).reshape(rows, k)
    small_m = small.astype(np.complex128).reshape(s, k)
    if gate_first:
        got = capi.contract(_dev(small, cuda), [s, k], [0, 1], _dev(big, cuda), big_shape,
                            [1, 0, 2, 3], s, rows, k)
        want = small_m @ big_t.T
        m, n = s, rows
    else:
        got = capi.contract(_dev(big, cuda), big_shape, [0, 2, 3, 1], _dev(small, cuda), [s, k],
                            [1, 0], rows, s, k)
        want = big_t @ small_m.T
        m, n = rows, s
    assert _rel(got.cpu().numpy()[: m * n].reshape(m, n), want) <= 1e-5


def test_more_axes_than_the_index_tables_fall_back(cuda):
    """Free axes that merge into more than the kernel's 12 index axes take
    the transposing path; the result is the same."""
    from jet_gb300 import capi

    r = 16
    shape = [2] * r
    a = cases.tensor_data(41, shape, np.complex64)
    common_axes = [15]
    free = [i for i in range(r - 1)][::-1]        # reversed: no two axes merge
    a_perm = free + common_axes
    m, k, n = 2 ** 15, 2, 2
    b = cases.tensor_data(42, [2, 2], np.complex64)
    want = (np.transpose(a.astype(np.complex128).reshape(shape), a_perm).reshape(m, k)
            @ b.astype(np.complex128).reshape(k, n))
    assert capi.contract_workspace_size(shape, a_perm, [2, 2], [0, 1], m, n, k,
                                        capi.dtype_code(np.complex64), capi.PREC_FP32) > 0
    got = capi.contract(_dev(a, cuda), shape, a_perm, _dev(b, cuda), [2, 2], [0, 1], m, n, k)
    assert _rel(got.cpu().numpy()[: m * n].reshape(m, n), want) <= 1e-5


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
@pytest.mark.parametrize("modes", [(0, 1), (1, 1), (1, 2), (2, 1), (2, 2), (0, 2), (1, 0),
                                   (2, 0)])
@pytest.mark.parametrize("gate_first", [False, True])
def test_batched_matches_single(cuda, dtype, modes, gate_first):
    """Batch modes 1 (tensors back to back) and 2 (batch axes inside the
    operand, leading its permutation) on either side; each batch item equals
    the single contraction of its slice."""
    import torch

    from jet_gb300 import capi

    batch = 3
    rank = 14
    s_lab, s_shape, _, g_lab, g_shape, _ = _gate_case(77, rank, 2, 2, 2, dtype)

    def operand(lab, shape, mode, seed):
        if mode == 0:
            return lab, shape, cases.tensor_data(seed, shape, dtype), None
        data = cases.tensor_data(seed, [batch] + shape, dtype).reshape([batch] + shape)
        if mode == 1:
            return lab, shape, data, None
        # Mode 2: the batch axis sits inside the tensor (position 1).
        moved = np.moveaxis(data, 0, 1)
        return lab, shape, np.ascontiguousarray(moved), data

    if gate_first:
        specs = [(g_lab, g_shape), (s_lab, s_shape)]
    else:
        specs = [(s_lab, s_shape), (g_lab, g_shape)]
    ops = [operand(specs[i][0], specs[i][1], modes[i], 500 + i) for i in range(2)]
    a_lab, a_shape = ops[0][0], ops[0][1]
    b_lab, b_shape = ops[1][0], ops[1][1]
    a_perm, b_perm, m, n, k, _ = _plan(a_lab, a_shape, b_lab, b_shape)

    def full(shape, perm, mode):
        if mode != 2:
            return shape, perm
        sh = [shape[0], batch] + shape[1:]
        pm = [1] + [p if p == 0 else p + 1 for p in perm]
        return sh, pm

    fa_shape, fa_perm = full(a_shape, a_perm, modes[0])
    fb_shape, fb_perm = full(b_shape, b_perm, modes[1])
    out = capi.contract_batched(batch, _dev(ops[0][2], cuda), fa_shape, fa_perm, modes[0],
                                _dev(ops[1][2], cuda), fb_shape, fb_perm, modes[1], m, n, k)
    torch.cuda.synchronize()
    got = out.cpu().numpy()[: batch * m * n]
    tol = 1e-5 if dtype == np.complex64 else 1e-12
    for bi in range(batch):
        def item(op, mode):
            if mode == 0:
                return op[2]
            src = op[3] if mode == 2 else op[2].reshape([batch] + op[1])
            return src[bi]
        want = (np.transpose(item(ops[0], modes[0]).astype(np.complex128).reshape(a_shape),
                             a_perm).reshape(m, k)
                @ np.transpose(item(ops[1], modes[1]).astype(np.complex128).reshape(b_shape),
                               b_perm).reshape(k, n))
        assert _rel(got[bi * m * n:(bi + 1) * m * n].reshape(m, n), want) <= tol, bi
    assert capi.take_device_status() == 0


pytestmark = pytest.mark.gpu


def test_more_than_2_to_32_rows(cuda):
    """Row indices past 32 bits (the 64-bit row decode): a 2^32 + 96 row
    tensor times a 1 x 1 matrix (k = 1, s = 1), 34 GB each way; sampled rows
    against complex128 products."""
    import torch

    from jet_gb300 import capi

    free, total = torch.cuda.mem_get_info()
    m = (1 << 32) + 96
    if free < 3 * m * 8:
        pytest.skip("needs about 103 GB of free device memory")
    a = torch.empty(m, dtype=torch.complex64, device=cuda)
    chunk = 1 << 28
    for lo in range(0, m, chunk):
        idx = torch.arange(lo, min(lo + chunk, m), device=cuda, dtype=torch.int64)
        a[lo:lo + idx.numel()].real.copy_(((idx % 1009) - 504).float() * 2.0 ** -10)
        a[lo:lo + idx.numel()].imag.copy_(((idx % 997) - 498).float() * 2.0 ** -11)
    del idx
    b = torch.tensor([0.75 - 0.5j], dtype=torch.complex64, device=cuda)
    assert capi.contract_workspace_size([m, 1], [0, 1], [1, 1], [0, 1], m, 1, 1,
                                        capi.C64, capi.PREC_FP32) == 0
    out = capi.contract(a, [m, 1], [0, 1], b, [1, 1], [0, 1], m, 1, 1)
    torch.cuda.synchronize()
    rows = torch.tensor([0, 1, 4095, (1 << 31) + 7, (1 << 32) - 1, 1 << 32, m - 1],
                        device=cuda)
    got = out[rows].cpu().numpy()
    want = a[rows].cpu().numpy().astype(np.complex128) * complex(0.75, -0.5)
    assert np.allclose(got, want, rtol=1e-6, atol=0), (got, want)
    assert capi.take_device_status() == 0
