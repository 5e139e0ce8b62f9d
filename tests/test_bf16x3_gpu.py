"""BF16x3 split-precision contraction (JETGPU_PREC_BF16X3) through the C-ABI.

The split stage is checked bit-exactly against a numpy model of its rounding
(round to nearest even: hi = RN_bf16(x), lo = RN_bf16(x - hi)). The product
is checked two ways:
  * against complex128 at 1e-5 relative Frobenius error (the bound the
    split forms are held to), and
  * against the exact-arithmetic value of the three-product sum of the same
    BF16 pieces: the difference is the FP32 accumulation alone, within 2e-6
    of the result's norm.
The three-product sum drops lo*lo and the residual x - hi - lo (both about
2^-17 relative), so its truncation is about 4e-6 on the config-1 data."""
import numpy as np
import pytest

import cases
from oracle import jet_oracle as jo

pytestmark = pytest.mark.gpu


def _dev(x, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(x)).to(dev)


def _rn_bf16_bits(x):
    """BF16 words of float32 x, round to nearest even."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def _bf16_value(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32)


def _split_model(x):
    x = np.asarray(x, np.float32)
    hi = _rn_bf16_bits(x)
    lo = _rn_bf16_bits(x - _bf16_value(hi))
    return hi, lo


def _product_model(a, b):
    """sum over (hi*hi + hi*lo + lo*hi) of the four real products, exact."""
    def pieces(x):
        h, l = _split_model(x)
        return _bf16_value(h).astype(np.float64), _bf16_value(l).astype(np.float64)

    arh, arl = pieces(a.real)
    aih, ail = pieces(a.imag)
    brh, brl = pieces(b.real)
    bih, bil = pieces(b.imag)

    def p(x0, x1, y0, y1):
        return x0 @ y0 + x0 @ y1 + x1 @ y0

    return (p(arh, arl, brh, brl) - p(aih, ail, bih, bil)) + 1j * (
        p(arh, arl, bih, bil) + p(aih, ail, brh, brl))


@pytest.fixture(params=[0, 1, 2], ids=["rows64", "n256", "rows32x6"])
def bf16_variant(request, cuda):
    """Runs a test under the BF16 main loops: 3 stages of 64-byte rows, N = 256
    MMAs over six B planes (contractions only; the stage entry points read
    four B planes and keep the default loop), and 6 stages of 32-byte rows."""
    from jet_gb300 import capi

    capi.set_tc_variant(request.param)
    yield request.param
    capi.set_tc_variant(0)


def _rel(got, want):
    return np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300)


def _config1_data(rng, rows, cols):
    return ((rng.standard_normal((rows, cols)) + 1j * rng.standard_normal((rows, cols)))
            * np.sqrt(0.5) * 2**-10).astype(np.complex64)


@pytest.mark.parametrize("shape,perm", [([2] * 12, None), ([3, 5, 7, 4], [2, 0, 3, 1]),
                                        ([16, 8], [1, 0]), ([3] * 12, None),
                                        ([6, 9, 5, 7, 20, 8], [3, 5, 1, 4, 0, 2])])
def test_split_bf16_bit_exact(cuda, shape, perm):
    """Planes equal the rounding model word for word, on random values,
    exact rounding ties (low 16 bits 0x8000), zeros and FP32 subnormals; both
    the bit-permutation kernel (power-of-2 shapes) and the tiled kernel
    (other dims)."""
    import torch

    from jet_gb300 import capi

    rank = len(shape)
    if perm is None:
        perm = cases.permutation(77, rank)
    size = int(np.prod(shape))
    rng = np.random.default_rng(size)
    x = (rng.standard_normal(size) + 1j * rng.standard_normal(size)).astype(np.complex64)
    re = x.real.copy()
    # Finite ties: sign, an exponent in [2^-16, 2^16) and 7 random mantissa bits.
    high = rng.integers(0x3780, 0x4780, 64, dtype=np.uint32) | (
        rng.integers(0, 2, 64, dtype=np.uint32) << 15)
    ties = (high << 16) | np.uint32(0x8000)
    re[:64] = ties.view(np.float32)
    re[64:70] = 0.0
    re[70:76] = np.array([1e-39, -3e-40, 1.2e-38, -1e-45, 5e-42, 2e-40], np.float32)
    x = (re + 1j * x.imag).astype(np.complex64)
    out_shape = [shape[p] for p in perm]
    cols = out_shape[-1]
    rows = size // cols
    pitch = (cols + 7) // 8 * 8
    planes = torch.zeros(4 * rows * pitch, dtype=torch.int16, device=cuda)
    capi.split_bf16(_dev(x, cuda), shape, perm, rows, cols, pitch, planes)
    got = planes.cpu().numpy().view(np.uint16).reshape(4, rows, pitch)[:, :, :cols]
    xt = np.transpose(x.reshape(shape), perm).reshape(rows, cols)
    rh, rl = _split_model(xt.real)
    ih, il = _split_model(xt.imag)
    for p, want in enumerate((rh, rl, ih, il)):
        assert np.array_equal(got[p], want), p


@pytest.mark.parametrize("m,n,k", [(128, 128, 32), (256, 128, 64), (200, 136, 100),
                                   (1024, 512, 256), (130, 300, 33), (4096, 256, 1024),
                                   (64, 512, 2048), (384, 256, 4096), (129, 131, 77),
                                   (300, 257, 64)])
def test_bf16x3_random_gemm(cuda, m, n, k, bf16_variant):
    """Config-1 value distribution against complex128 (1e-5) and against the
    exact three-product model (2e-6, the accumulation alone)."""
    from jet_gb300 import capi

    rng = np.random.default_rng(m * 7 + n * 13 + k)
    a = _config1_data(rng, m, k)
    b = _config1_data(rng, k, n)
    want = a.astype(np.complex128) @ b.astype(np.complex128)
    model = _product_model(a, b)
    out = capi.contract(_dev(a.reshape(-1), cuda), [m, k], [0, 1], _dev(b.reshape(-1), cuda),
                        [k, n], [0, 1], m, n, k, precision=capi.PREC_BF16X3)
    got = out.cpu().numpy().reshape(m, n)
    assert _rel(got, want) <= 1e-5, _rel(got, want)
    assert np.linalg.norm(got - model) <= 2e-6 * np.linalg.norm(want)
    assert capi.take_device_status() == 0


def test_bf16x3_stages_equal_contract(cuda, bf16_variant):
    """jetgpu_split_bf16 + jetgpu_gemm_bf16x3 give jetgpu_contract's result
    bit for bit (the contraction is those two stages)."""
    import torch

    from jet_gb300 import capi

    m, n, k = 512, 256, 200
    rng = np.random.default_rng(3)
    a = _config1_data(rng, m, k)
    b = _config1_data(rng, k, n)
    da, db = _dev(a.reshape(-1), cuda), _dev(b.reshape(-1), cuda)
    ref = capi.contract(da, [m, k], [0, 1], db, [k, n], [0, 1], m, n, k,
                        precision=capi.PREC_BF16X3).cpu().numpy()
    kp = (k + 7) // 8 * 8
    pa = torch.empty(4 * m * kp, dtype=torch.int16, device=cuda)
    pb = torch.empty(4 * n * kp, dtype=torch.int16, device=cuda)
    capi.split_bf16(da, [m, k], [0, 1], m, k, kp, pa)
    capi.split_bf16(db, [k, n], [1, 0], n, k, kp, pb)
    c = torch.empty(m * n, dtype=torch.complex64, device=cuda)
    capi.gemm_bf16x3(pa, pb, m, n, k, kp, c)
    if bf16_variant == 1:
        # N = 256 MMAs in the contraction, N = 128 in the stages: the same
        # three-product sums in another instruction shape.
        assert _rel(c.cpu().numpy(), ref) <= 1e-6
    else:
        assert np.array_equal(c.cpu().numpy(), ref)


def test_bf16x3_reference_contractions(cuda, golden):
    """The reference's own ContractTensors results (complex64 cases)."""
    from jet_gb300 import capi

    for c in golden["ref"]["contract"]:
        if c["dtype"] != "complex64":
            continue
        a = cases.tensor_data(c["seed"], c["a_shape"], c["dtype"])
        b = cases.tensor_data(c["seed"] + 1, c["b_shape"], c["dtype"])
        left = jo.vector_subtraction(c["a_labels"], c["b_labels"])
        right = jo.vector_subtraction(c["b_labels"], c["a_labels"])
        common = jo.vector_intersection(c["a_labels"], c["b_labels"])
        ad = dict(zip(c["a_labels"], c["a_shape"]))
        bd = dict(zip(c["b_labels"], c["b_shape"]))
        m = int(np.prod([ad[x] for x in left])) if left else 1
        n = int(np.prod([bd[x] for x in right])) if right else 1
        k = int(np.prod([ad[x] for x in common])) if common else 1
        a_perm = [c["a_labels"].index(x) for x in left + common]
        b_perm = [c["b_labels"].index(x) for x in common + right]
        got = capi.contract(_dev(a, cuda), c["a_shape"], a_perm, _dev(b, cuda), c["b_shape"],
                            b_perm, m, n, k, precision=capi.PREC_BF16X3).cpu().numpy()[: m * n]
        want = np.array([complex(x, y) for x, y in c["out"]])
        assert _rel(got, want) <= 1e-5, c


def test_bf16x3_exact_values(cuda):
    """Test_Tensor.cpp:537-541 / 515-535 values are BF16-exact: exact results."""
    from jet_gb300 import capi

    a = np.full(24, 0.5 + 0.25j, np.complex64)
    out = capi.contract(_dev(a, cuda), [2, 3, 4], [0, 1, 2], _dev(a, cuda), [3, 4, 2],
                        [0, 1, 2], 2, 2, 12, precision=capi.PREC_BF16X3).cpu().numpy()
    assert np.all(out == np.complex64(2.25 + 3j))


def test_bf16x3_transposed_operands_config1_shape_reduced(cuda, bf16_variant):
    """Config-1 structure at reduced size: A rank 21, B rank 19, 10 shared
    labels, both seeded-randomly permuted, against the oracle."""
    from jet_gb300 import capi

    nl, nc, nr = 11, 10, 9
    left = ["l%d" % i for i in range(nl)]
    common = ["c%d" % i for i in range(nc)]
    right = ["r%d" % i for i in range(nr)]
    a_lab = [(left + common)[i] for i in cases.permutation(901, nl + nc)]
    b_lab = [(common + right)[i] for i in cases.permutation(902, nc + nr)]
    a_shape, b_shape = [2] * (nl + nc), [2] * (nc + nr)
    rng = np.random.default_rng(5)
    a = _config1_data(rng, 1, 2 ** (nl + nc)).reshape(-1)
    b = _config1_data(rng, 1, 2 ** (nc + nr)).reshape(-1)
    lft = [x for x in a_lab if x not in b_lab]
    com = [x for x in a_lab if x in b_lab]
    rgt = [x for x in b_lab if x not in a_lab]
    a_perm = [a_lab.index(x) for x in lft + com]
    b_perm = [b_lab.index(x) for x in com + rgt]
    want = jo.contract_tensors(jo.OTensor.make(a_lab, a_shape, a, np.complex128),
                               jo.OTensor.make(b_lab, b_shape, b, np.complex128))
    assert want.indices == lft + rgt
    out = capi.contract(_dev(a, cuda), a_shape, a_perm, _dev(b, cuda), b_shape, b_perm,
                        2 ** nl, 2 ** nr, 2 ** nc, precision=capi.PREC_BF16X3).cpu().numpy()
    assert _rel(out, want.data) <= 1e-5


def test_bf16x3_power_of_two_scales(cuda):
    from jet_gb300 import capi

    m = n = 256
    k = 128
    a = cases.tensor_data(3, [m * k], np.complex64)
    b = cases.tensor_data(4, [k * n], np.complex64)
    want = (a.astype(np.complex128).reshape(m, k) @ b.astype(np.complex128).reshape(k, n)) \
        * 2.0**(20 - 7)
    out = capi.contract(_dev(a, cuda), [m, k], [0, 1], _dev(b, cuda), [k, n], [0, 1], m, n, k,
                        precision=capi.PREC_BF16X3, scale_a=20,
                        scale_b=-7).cpu().numpy().reshape(m, n)
    assert _rel(out, want) <= 1e-5


def test_bf16x3_through_tensor_api(cuda):
    """Jet::Tensor ContractTensors under Gpu::SetPrecision(BF16x3)."""
    import jet_gb300 as jet

    rng = np.random.default_rng(11)
    a = _config1_data(rng, 1, 2 ** 14).reshape(-1)
    b = _config1_data(rng, 1, 2 ** 14).reshape(-1)
    a_lab = ["i%d" % j for j in range(7)] + ["c%d" % j for j in range(7)]
    b_lab = ["c%d" % j for j in range(7)][::-1] + ["o%d" % j for j in range(7)]
    ta = jet.Tensor(indices=a_lab, shape=[2] * 14, data=list(a), dtype="complex64")
    tb = jet.Tensor(indices=b_lab, shape=[2] * 14, data=list(b), dtype="complex64")
    want = jo.contract_tensors(jo.OTensor.make(a_lab, [2] * 14, a, np.complex128),
                               jo.OTensor.make(b_lab, [2] * 14, b, np.complex128))
    prev = jet.get_precision()
    jet.set_precision(jet.PREC_BF16X3)
    try:
        got = jet.contract_tensors(ta, tb)
    finally:
        jet.set_precision(prev)
    assert list(got.indices) == want.indices
    assert _rel(np.array(got.data), want.data) <= 1e-5
