"""GPU contraction parity through the C-ABI (jetgpu_contract / jetgpu_multiply).

Tolerances (relative Frobenius error against complex128):
  plain complex64 (FP32 FMA) ........ 1e-5
  complex128 (FP64 FMA) ............. 1e-12
  TF32x3 split precision (complex64)  1e-5
Small integer-valued cases of the reference tests are exact."""
import numpy as np
import pytest

import cases
from oracle import jet_oracle as jo

pytestmark = pytest.mark.gpu


def _dev(x, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(x)).to(dev)


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
    a_perm = [a_labels.index(x) for x in left + common]
    b_perm = [b_labels.index(x) for x in common + right]
    return a_perm, b_perm, m, n, k, left + right


@pytest.fixture(params=[0, 1], ids=["n128", "n256"])
def tc_variant(request, cuda):
    """Runs a test under both main-loop shapes of the tensor-core product."""
    from jet_gb300 import capi

    capi.set_tc_variant(request.param)
    yield request.param
    capi.set_tc_variant(0)


def _rel(got, want):
    return np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300)


def _run(cuda, c, precision):
    from jet_gb300 import capi

    a = cases.tensor_data(c["seed"], c["a_shape"], c["dtype"])
    b = cases.tensor_data(c["seed"] + 1, c["b_shape"], c["dtype"])
    a_perm, b_perm, m, n, k, lab = _plan(c["a_labels"], c["a_shape"], c["b_labels"], c["b_shape"])
    out = capi.contract(_dev(a, cuda), c["a_shape"], a_perm, _dev(b, cuda), c["b_shape"], b_perm,
                        m, n, k, precision=precision)
    return out.cpu().numpy()[: m * n], lab


def test_reference_contractions_plain(cuda, golden):
    from jet_gb300 import capi

    for c in golden["ref"]["contract"]:
        got, lab = _run(cuda, c, capi.PREC_FP32)
        assert lab == c["out_labels"]
        want = np.array([complex(x, y) for x, y in c["out"]])
        tol = 1e-5 if c["dtype"] == "complex64" else 1e-12
        assert _rel(got, want) <= tol, c


def test_reference_contractions_tf32x3(cuda, golden, tc_variant):
    from jet_gb300 import capi

    for c in golden["ref"]["contract"]:
        if c["dtype"] != "complex64":
            continue
        got, _ = _run(cuda, c, capi.PREC_TF32X3)
        want = np.array([complex(x, y) for x, y in c["out"]])
        assert _rel(got, want) <= 1e-5, c


def test_reference_literal_values(cuda):
    """Test_Tensor.cpp:537-541 / 515-535: exact results."""
    from jet_gb300 import capi

    for prec in (capi.PREC_FP32, capi.PREC_TF32X3):
        a = np.full(24, 0.5 + 0.25j, np.complex64)
        out = capi.contract(_dev(a, cuda), [2, 3, 4], [0, 1, 2], _dev(a, cuda), [3, 4, 2],
                            [0, 1, 2], 2, 2, 12, precision=prec).cpu().numpy()
        assert np.all(out == np.complex64(2.25 + 3j))
        ones = np.ones(4, np.complex64)
        s = capi.contract(_dev(ones, cuda), [2, 2], [0, 1], _dev(ones, cuda), [2, 2], [0, 1],
                          1, 1, 4, precision=prec).cpu().numpy()
        assert s[0] == 4


@pytest.mark.parametrize("m,n,k", [(128, 128, 16), (256, 128, 64), (200, 136, 100),
                                   (1024, 512, 256), (130, 300, 33), (4096, 256, 1024),
                                   (64, 512, 2048), (129, 131, 77), (300, 257, 64)])
def test_tf32x3_random_gemm(cuda, m, n, k, tc_variant):
    """Random N(0, 1/2) complex entries scaled by 2^-10 (the config-1
    distribution) against the complex128 product."""
    import torch

    from jet_gb300 import capi

    rng = np.random.default_rng(m * 7 + n * 13 + k)
    a = ((rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))) * np.sqrt(0.5) * 2**-10)
    b = ((rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))) * np.sqrt(0.5) * 2**-10)
    a64, b64 = a.astype(np.complex64), b.astype(np.complex64)
    want = a64.astype(np.complex128) @ b64.astype(np.complex128)
    for prec, tol in ((capi.PREC_TF32X3, 1e-5), (capi.PREC_FP32, 1e-5)):
        out = capi.contract(_dev(a64.reshape(-1), cuda), [m, k], [0, 1],
                            _dev(b64.reshape(-1), cuda), [k, n], [0, 1], m, n, k,
                            precision=prec)
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(m, n)
        assert _rel(got, want) <= tol, (prec, _rel(got, want))
    assert capi.take_device_status() == 0


def test_tf32x3_transposed_operands_config1_shape_reduced(cuda, tc_variant):
    """Config-1 structure at reduced size: A rank 21, B rank 19, 10 shared
    labels, both seeded-randomly permuted."""
    from jet_gb300 import capi

    nl, nc, nr = 11, 10, 9
    left = ["l%d" % i for i in range(nl)]
    common = ["c%d" % i for i in range(nc)]
    right = ["r%d" % i for i in range(nr)]
    a_lab = [(left + common)[i] for i in cases.permutation(901, nl + nc)]
    b_lab = [(common + right)[i] for i in cases.permutation(902, nc + nr)]
    a_shape, b_shape = [2] * (nl + nc), [2] * (nc + nr)
    rng = np.random.default_rng(5)
    a = ((rng.standard_normal(2 ** (nl + nc)) + 1j * rng.standard_normal(2 ** (nl + nc)))
         * np.sqrt(0.5) * 2**-10).astype(np.complex64)
    b = ((rng.standard_normal(2 ** (nc + nr)) + 1j * rng.standard_normal(2 ** (nc + nr)))
         * np.sqrt(0.5) * 2**-10).astype(np.complex64)
    a_perm, b_perm, m, n, k, lab = _plan(a_lab, a_shape, b_lab, b_shape)
    want = jo.contract_tensors(jo.OTensor.make(a_lab, a_shape, a, np.complex128),
                               jo.OTensor.make(b_lab, b_shape, b, np.complex128))
    assert want.indices == lab
    for prec in (capi.PREC_TF32X3, capi.PREC_FP32):
        out = capi.contract(_dev(a, cuda), a_shape, a_perm, _dev(b, cuda), b_shape, b_perm,
                            m, n, k, precision=prec).cpu().numpy()
        assert _rel(out, want.data) <= 1e-5, prec


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (1, 1, 100000), (7, 1, 5), (3000, 1, 4096),
                                   (1, 5000, 64), (1, 3, 300000), (2, 2, 0), (5, 7, 1),
                                   (333, 77, 1), (2, 1, 200000), (3, 1, 70001), (9, 1, 1000),
                                   (1, 2, 400000), (1, 5, 123457), (1, 300, 5000),
                                   (64, 64, 8192), (200, 100, 3000), (27, 243, 729)])
@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_multiply_vector_and_edge_shapes(cuda, m, n, k, dtype):
    """GEMV, GEMV^T, DOTU and k = 0 cases of MultiplyTensorData, including few
    rows or columns over a long k (several warps or threads per row / column)
    and small matrices over a long k (k split across CTAs)."""
    from jet_gb300 import capi

    a = cases.tensor_data(m * 3 + k, [m * k], dtype)
    b = cases.tensor_data(n * 5 + k, [k * n], dtype)
    want = (a.astype(np.complex128).reshape(m, k) @ b.astype(np.complex128).reshape(k, n))
    for prec in (capi.PREC_FP32, capi.PREC_AUTO):
        out = capi.contract(_dev(a, cuda), [m, k], [0, 1], _dev(b, cuda), [k, n], [0, 1],
                            m, n, k, precision=prec).cpu().numpy()[: m * n].reshape(m, n)
        tol = 1e-5 if dtype == np.complex64 else 1e-12
        if k == 0:
            assert np.all(out == 0)
        else:
            assert _rel(out, want) <= tol
    direct = capi.multiply(_dev(a, cuda), _dev(b, cuda), m, n, k).cpu().numpy()[: m * n]
    if k:
        assert _rel(direct.reshape(m, n), want) <= (1e-5 if dtype == np.complex64 else 1e-12)


@pytest.mark.parametrize("m,n,k", [(16, 32, 4096), (2, 2, 2048), (16, 32, 1 << 18),
                                   (32, 16, 100003), (5, 7, 65536), (32, 16, 2049),
                                   (12, 30, 50000), (3, 17, 9000)])
@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_small_output_long_k(cuda, m, n, k, dtype):
    """Products with a small output and a long k (gemm_small_kernel: M <= 16
    and N <= 32 or M <= 32 and N <= 16, k >= 2048), k split into ranges
    reduced in a fixed order: against complex128, and the same bits on a
    second run; a permuted operand and a batch sharing A."""
    import torch

    from jet_gb300 import capi

    a = cases.tensor_data(m * 11 + k, [m * k], dtype)
    b = cases.tensor_data(n * 13 + k, [k * n], dtype)
    want = a.astype(np.complex128).reshape(m, k) @ b.astype(np.complex128).reshape(k, n)
    tol = 1e-5 if dtype == np.complex64 else 1e-12
    da, db = _dev(a, cuda), _dev(b, cuda)
    outs = []
    for prec in (capi.PREC_FP32, capi.PREC_AUTO, capi.PREC_FP32):
        out = capi.contract(da, [m, k], [0, 1], db, [k, n], [0, 1], m, n, k, precision=prec)
        torch.cuda.synchronize()
        outs.append(out[: m * n].clone())
        assert _rel(out.cpu().numpy()[: m * n].reshape(m, n), want) <= tol, prec
    assert torch.equal(outs[0], outs[2])
    # A stored transposed (k x m, permutation [1, 0]); A shared by a batch of 3 Bs.
    at = np.ascontiguousarray(a.reshape(m, k).T)
    got = capi.contract(_dev(at, cuda), [k, m], [1, 0], db, [k, n], [0, 1], m, n, k)
    assert _rel(got.cpu().numpy()[: m * n].reshape(m, n), want) <= tol
    b3 = np.concatenate([b, 2 * b, -b])
    got3 = capi.contract_batched(3, da, [m, k], [0, 1], 0, _dev(b3, cuda), [k, n], [0, 1], 1,
                                 m, n, k).cpu().numpy()[: 3 * m * n].reshape(3, m, n)
    for i, f in enumerate((1, 2, -1)):
        assert _rel(got3[i], f * want) <= tol, i
    assert capi.take_device_status() == 0


def test_power_of_two_scales(cuda, tc_variant):
    from jet_gb300 import capi

    m = n = 256
    k = 128
    a = cases.tensor_data(3, [m * k], np.complex64)
    b = cases.tensor_data(4, [k * n], np.complex64)
    want = (a.astype(np.complex128).reshape(m, k) @ b.astype(np.complex128).reshape(k, n)) * 2.0**(20 - 7)
    for prec in (capi.PREC_FP32, capi.PREC_TF32X3):
        out = capi.contract(_dev(a, cuda), [m, k], [0, 1], _dev(b, cuda), [k, n], [0, 1], m, n, k,
                            precision=prec, scale_a=20, scale_b=-7).cpu().numpy().reshape(m, n)
        assert _rel(out, want) <= 1e-5


def test_tmem_chunk_depth_controls_accumulation_error(cuda):
    """The K depth accumulated in tensor memory per fold: shorter is more
    accurate (3xTF32, k = 4096, config-1 data); the default is 16."""
    from jet_gb300 import capi

    m, n, k = 512, 256, 4096
    rng = np.random.default_rng(17)
    a = ((rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))) * np.sqrt(0.5)
         * 2**-10).astype(np.complex64)
    b = ((rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))) * np.sqrt(0.5)
         * 2**-10).astype(np.complex64)
    want = a.astype(np.complex128) @ b.astype(np.complex128)
    errs = {}
    try:
        for depth in (0, 16, 128):
            capi.set_tc_chunk_depth(depth)
            out = capi.contract(_dev(a.reshape(-1), cuda), [m, k], [0, 1],
                                _dev(b.reshape(-1), cuda), [k, n], [0, 1], m, n, k,
                                precision=capi.PREC_TF32X3).cpu().numpy().reshape(m, n)
            errs[depth] = _rel(out, want)
    finally:
        capi.set_tc_chunk_depth(0)
    assert errs[0] == errs[16]
    assert errs[16] < errs[128]
    assert errs[16] <= 1e-6, errs


@pytest.mark.parametrize("precision", [1, 3, 4])
def test_persistent_and_per_tile_launches_agree_bitwise(cuda, precision):
    """The persistent tensor-core launch (one CTA per SM walking the tiles)
    computes every tile exactly as the one-CTA-per-tile launch: same bits, for
    partial edge tiles, a single product of fewer tiles than SMs (static
    order) and a batch of more tiles than SMs (tiles drawn from the counter)."""
    import torch

    from jet_gb300 import capi

    m, n, k, batch = 1100, 1900, 600, 3  # 135 tiles per product, 405 in the batch
    g = torch.Generator(device=cuda)
    g.manual_seed(precision)
    a = torch.randn(batch * m * k, dtype=torch.complex64, device=cuda, generator=g)
    b = torch.randn(batch * k * n, dtype=torch.complex64, device=cuda, generator=g)
    outs = []
    try:
        for persistent in (1, 0):
            capi.set_tc_persistent(persistent)
            c = capi.contract_batched(batch, a, [m, k], [0, 1], 1, b, [k, n], [0, 1], 1, m, n, k,
                                      precision=precision)
            c1 = capi.contract(a[: m * k], [m, k], [0, 1], b[: k * n], [k, n], [0, 1], m, n, k,
                               precision=precision)
            outs.append((c.clone(), c1.clone()))
    finally:
        capi.set_tc_persistent(1)
    assert torch.equal(outs[0][0].view(torch.int64), outs[1][0].view(torch.int64))
    assert torch.equal(outs[0][1].view(torch.int64), outs[1][1].view(torch.int64))
    want = (a[: m * k].view(m, k).cpu().numpy().astype(np.complex128)
            @ b[: k * n].view(k, n).cpu().numpy().astype(np.complex128))
    got = outs[0][0][: m * n].view(m, n).cpu().numpy()
    assert np.linalg.norm(got - want) <= 1e-5 * np.linalg.norm(want)
