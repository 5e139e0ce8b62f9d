"""FP16x3 split-precision contraction (JETGPU_PREC_FP16X3) through the C-ABI.

Each operand is scaled by 2^s, s = 14 - e_max (clamped to [-120, 120]),
e_max the binary exponent of its largest |re| or |im|, then split into FP16
hi = RN_fp16(2^s x) and lo = RN_fp16(2^s x - hi); the product's epilogue
multiplies by 2^-(s_A + s_B).

Checks: the split bit-exactly against a numpy model (numpy's float16
conversion is IEEE round-to-nearest-even with subnormals); the product
against complex128 at 1e-5 and against the exact value of its three-product
sum at 2e-6 (the FP32 accumulation alone); operands far outside FP16's range
(2^-60 and 2^+40), a zero operand, the power-of-two user scales, the two
stage entry points against jetgpu_contract, the reference's golden
contractions."""
import numpy as np
import pytest

import cases
from oracle import jet_oracle as jo

pytestmark = pytest.mark.gpu


def _dev(x, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(x)).to(dev)


def _rel(got, want):
    return np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300)


def _emax(x):
    """Binary exponent of the largest |re|, |im| (-1000 when all zero)."""
    m = max(float(np.max(np.abs(x.real))), float(np.max(np.abs(x.imag))))
    return -1000 if m == 0 else int(np.floor(np.log2(np.float32(m))))


def _scale_exp(e):
    return int(min(120, max(-120, 14 - e)))


def _split_model(x, s):
    """FP16 words of hi, lo of x * 2^s (x float32)."""
    xs = (np.asarray(x, np.float32) * np.float32(2.0**s)).astype(np.float32)
    hi = xs.astype(np.float16)
    lo = (xs - hi.astype(np.float32)).astype(np.float16)
    return hi, lo


def _product_model(a, b):
    sa, sb = _scale_exp(_emax(a)), _scale_exp(_emax(b))

    def pieces(x, s):
        h, l = _split_model(x, s)
        return h.astype(np.float64), l.astype(np.float64)

    arh, arl = pieces(a.real, sa)
    aih, ail = pieces(a.imag, sa)
    brh, brl = pieces(b.real, sb)
    bih, bil = pieces(b.imag, sb)

    def p(x0, x1, y0, y1):
        return x0 @ y0 + x0 @ y1 + x1 @ y0

    c = (p(arh, arl, brh, brl) - p(aih, ail, bih, bil)) + 1j * (
        p(arh, arl, bih, bil) + p(aih, ail, brh, brl))
    return c * 2.0 ** -(sa + sb)


def _data(rng, rows, cols, scale=2**-10):
    return ((rng.standard_normal((rows, cols)) + 1j * rng.standard_normal((rows, cols)))
            * np.sqrt(0.5) * scale).astype(np.complex64)


@pytest.mark.parametrize("shape,perm,scale", [([2] * 12, None, 1.0), ([3, 5, 7, 4], [2, 0, 3, 1], 2.0**-70),
                                              ([16, 8], [1, 0], 2.0**50), ([3] * 12, None, 1.0)])
def test_split_fp16_bit_exact(cuda, shape, perm, scale):
    """Planes equal the model word for word, with exact rounding ties, zeros,
    and values 2^-20 and 2^-30 below the maximum (FP16 subnormal lo words);
    bit-permutation and tiled kernels; three operand magnitudes."""
    import torch

    from jet_gb300 import capi

    rank = len(shape)
    if perm is None:
        perm = cases.permutation(91, rank)
    size = int(np.prod(shape))
    rng = np.random.default_rng(size + 1)
    x = (rng.standard_normal(size) + 1j * rng.standard_normal(size)).astype(np.complex64)
    re = x.real.copy()
    # Ties of the FP32 -> FP16 rounding after scaling by 2^14 / max: 11 random
    # significant bits plus exactly half a unit of the 11th.
    ties = (rng.integers(1024, 2048, 32) + 0.5) * 2.0 ** rng.integers(-12, 0, 32)
    re[:32] = (ties * np.sign(rng.standard_normal(32))).astype(np.float32)
    re[32:38] = 0.0
    re[38:44] = re[38:44] * np.float32(2.0**-20)
    re[44:50] = re[44:50] * np.float32(2.0**-30)
    x = ((re + 1j * x.imag) * np.float32(scale)).astype(np.complex64)
    e = torch.empty(1, dtype=torch.int32, device=cuda)
    capi.max_exponent(_dev(x, cuda), out=e)
    assert int(e.item()) == _emax(x)
    out_shape = [shape[p] for p in perm]
    cols = out_shape[-1]
    rows = size // cols
    pitch = (cols + 7) // 8 * 8
    planes = torch.zeros(4 * rows * pitch, dtype=torch.int16, device=cuda)
    capi.split_fp16(_dev(x, cuda), shape, perm, rows, cols, pitch, planes, e)
    got = planes.cpu().numpy().view(np.uint16).reshape(4, rows, pitch)[:, :, :cols]
    xt = np.transpose(x.reshape(shape), perm).reshape(rows, cols)
    s = _scale_exp(_emax(x))
    rh, rl = _split_model(xt.real, s)
    ih, il = _split_model(xt.imag, s)
    for p, want in enumerate((rh, rl, ih, il)):
        assert np.array_equal(got[p], want.view(np.uint16)), p


@pytest.mark.parametrize("m,n,k", [(128, 128, 32), (256, 128, 64), (200, 136, 100),
                                   (1024, 512, 256), (130, 300, 33), (4096, 256, 1024),
                                   (64, 512, 2048), (384, 256, 4096), (129, 131, 77),
                                   (300, 257, 64)])
def test_fp16x3_random_gemm(cuda, m, n, k):
    """Config-1 distribution against complex128 (1e-5) and against the exact
    three-product model (2e-6)."""
    from jet_gb300 import capi

    rng = np.random.default_rng(m * 11 + n * 5 + k)
    a = _data(rng, m, k)
    b = _data(rng, k, n)
    want = a.astype(np.complex128) @ b.astype(np.complex128)
    model = _product_model(a, b)
    got = capi.contract(_dev(a.reshape(-1), cuda), [m, k], [0, 1], _dev(b.reshape(-1), cuda),
                        [k, n], [0, 1], m, n, k,
                        precision=capi.PREC_FP16X3).cpu().numpy().reshape(m, n)
    assert _rel(got, want) <= 1e-5, _rel(got, want)
    assert np.linalg.norm(got - model) <= 2e-6 * np.linalg.norm(want)
    assert capi.take_device_status() == 0


@pytest.mark.parametrize("m,n,k", [(128, 128, 32), (200, 136, 100), (1024, 512, 256),
                                   (130, 300, 33), (384, 256, 4096)])
def test_fp16x3_n256_main_loop(cuda, m, n, k):
    """The N = 256 main loop (jetgpu_set_tc_variant(1): stacked [Br; Bi] and
    [-Bi; Br] B operands on six FP16 planes) against complex128 and the exact
    three-product model."""
    from jet_gb300 import capi

    rng = np.random.default_rng(m * 3 + n * 7 + k)
    a = _data(rng, m, k)
    b = _data(rng, k, n)
    want = a.astype(np.complex128) @ b.astype(np.complex128)
    model = _product_model(a, b)
    capi.set_tc_variant(1)
    try:
        got = capi.contract(_dev(a.reshape(-1), cuda), [m, k], [0, 1],
                            _dev(b.reshape(-1), cuda), [k, n], [0, 1], m, n, k,
                            precision=capi.PREC_FP16X3).cpu().numpy().reshape(m, n)
    finally:
        capi.set_tc_variant(0)
    assert _rel(got, want) <= 1e-5, _rel(got, want)
    assert np.linalg.norm(got - model) <= 2e-6 * np.linalg.norm(want)
    assert capi.take_device_status() == 0


@pytest.mark.parametrize("sa,sb", [(2.0**-60, 2.0**40), (2.0**30, 2.0**-50), (2.0**-100, 1.0)])
def test_fp16x3_operands_outside_fp16_range(cuda, sa, sb):
    from jet_gb300 import capi

    m, n, k = 256, 256, 512
    rng = np.random.default_rng(4)
    a = _data(rng, m, k, sa)
    b = _data(rng, k, n, sb)
    want = a.astype(np.complex128) @ b.astype(np.complex128)
    got = capi.contract(_dev(a.reshape(-1), cuda), [m, k], [0, 1], _dev(b.reshape(-1), cuda),
                        [k, n], [0, 1], m, n, k,
                        precision=capi.PREC_FP16X3).cpu().numpy().reshape(m, n)
    assert _rel(got, want) <= 1e-5, _rel(got, want)


def test_fp16x3_zero_operand_and_user_scales(cuda):
    from jet_gb300 import capi

    m, n, k = 256, 128, 256
    rng = np.random.default_rng(8)
    a = _data(rng, m, k)
    z = np.zeros((k, n), np.complex64)
    got = capi.contract(_dev(a.reshape(-1), cuda), [m, k], [0, 1], _dev(z.reshape(-1), cuda),
                        [k, n], [0, 1], m, n, k, precision=capi.PREC_FP16X3).cpu().numpy()
    assert np.all(got == 0)
    b = _data(rng, k, n)
    want = (a.astype(np.complex128) @ b.astype(np.complex128)) * 2.0**(20 - 7)
    got = capi.contract(_dev(a.reshape(-1), cuda), [m, k], [0, 1], _dev(b.reshape(-1), cuda),
                        [k, n], [0, 1], m, n, k, precision=capi.PREC_FP16X3, scale_a=20,
                        scale_b=-7).cpu().numpy().reshape(m, n)
    assert _rel(got, want) <= 1e-5


def test_fp16x3_stages_equal_contract(cuda):
    """max exponent + jetgpu_split_fp16 (A, B) + jetgpu_gemm_fp16x3 give
    jetgpu_contract's result bit for bit."""
    import torch

    from jet_gb300 import capi

    m, n, k = 512, 256, 200
    rng = np.random.default_rng(3)
    a = _data(rng, m, k, 2.0**-30)
    b = _data(rng, k, n, 2.0**12)
    da, db = _dev(a.reshape(-1), cuda), _dev(b.reshape(-1), cuda)
    ref = capi.contract(da, [m, k], [0, 1], db, [k, n], [0, 1], m, n, k,
                        precision=capi.PREC_FP16X3).cpu().numpy()
    e = torch.empty(2, dtype=torch.int32, device=cuda)
    capi.max_exponent(da, out=e[0:1])
    capi.max_exponent(db, out=e[1:2])
    kp = (k + 7) // 8 * 8
    pa = torch.empty(4 * m * kp, dtype=torch.int16, device=cuda)
    pb = torch.empty(4 * n * kp, dtype=torch.int16, device=cuda)
    capi.split_fp16(da, [m, k], [0, 1], m, k, kp, pa, e[0:1])
    capi.split_fp16(db, [k, n], [1, 0], n, k, kp, pb, e[1:2])
    c = torch.empty(m * n, dtype=torch.complex64, device=cuda)
    capi.gemm_fp16x3(pa, pb, m, n, k, kp, c, e)
    assert np.array_equal(c.cpu().numpy(), ref)


def test_fp16x3_reference_contractions(cuda, golden):
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
                            b_perm, m, n, k, precision=capi.PREC_FP16X3).cpu().numpy()[: m * n]
        want = np.array([complex(x, y) for x, y in c["out"]])
        assert _rel(got, want) <= 1e-5, c


def test_fp16x3_exact_values(cuda):
    from jet_gb300 import capi

    a = np.full(24, 0.5 + 0.25j, np.complex64)
    out = capi.contract(_dev(a, cuda), [2, 3, 4], [0, 1, 2], _dev(a, cuda), [3, 4, 2],
                        [0, 1, 2], 2, 2, 12, precision=capi.PREC_FP16X3).cpu().numpy()
    assert np.all(out == np.complex64(2.25 + 3j))


def test_auto_form_knob(cuda):
    """PREC_AUTO's tensor-core steps take the form set by set_auto_form; the
    FP16 form applies from 2^30 multiply-adds (m n k), smaller steps take
    TF32x3."""
    from jet_gb300 import capi

    rng = np.random.default_rng(12)

    def run(prec, m, n, k, da, db):
        return capi.contract(da, [m, k], [0, 1], db, [k, n], [0, 1], m, n, k,
                             precision=prec).cpu().numpy()

    big = (2048, 1024, 512)      # 2^30
    small = (1024, 512, 512)     # 2^28
    ops = {}
    for shape in (big, small):
        m, n, k = shape
        ops[shape] = (_dev(_data(rng, m, k).reshape(-1), cuda),
                      _dev(_data(rng, k, n).reshape(-1), cuda))
    try:
        for form in (capi.PREC_TF32X3, capi.PREC_FP16X3, capi.PREC_BF16X3):
            capi.set_auto_form(form)
            assert np.array_equal(run(capi.PREC_AUTO, *big, *ops[big]),
                                  run(form, *big, *ops[big]))
        capi.set_auto_form(capi.PREC_FP16X3)
        assert np.array_equal(run(capi.PREC_AUTO, *small, *ops[small]),
                              run(capi.PREC_TF32X3, *small, *ops[small]))
    finally:
        capi.set_auto_form(capi.PREC_FP16X3)


@pytest.mark.parametrize("producer", [1, 3, 4, 5])
def test_exponent_hints_pass_between_steps(cuda, producer):
    """A tensor-core product records its output's max exponent (the value the
    scan would find); FP16x3 with that hint gives the same bits as with the
    scan; plain products record nothing (the consumer then scans)."""
    import torch

    from jet_gb300 import capi

    g = torch.Generator(device=cuda)
    g.manual_seed(producer)
    m, k, n, n2 = 384, 256, 320, 200
    a = torch.randn(m * k, dtype=torch.complex64, device=cuda, generator=g) * 2.0**-30
    b = torch.randn(k * n, dtype=torch.complex64, device=cuda, generator=g)
    x = torch.randn(n * n2, dtype=torch.complex64, device=cuda, generator=g) * 2.0**20
    e = torch.empty(1, dtype=torch.int32, device=cuda)
    c = capi.contract_batched_hinted(1, a, [m, k], [0, 1], 0, b, [k, n], [0, 1], 0, m, n, k,
                                     precision=producer, c_emax=e)
    recorded = int(e.item())
    if producer == capi.PREC_TUNED:  # the tuner may pick the plain form
        assert recorded == capi.max_exponent(c[: m * n]) or recorded < -1000
    else:
        assert recorded == capi.max_exponent(c[: m * n])
    d_scan = capi.contract(c, [m, n], [0, 1], x, [n, n2], [0, 1], m, n2, n,
                           precision=capi.PREC_FP16X3)
    d_hint = capi.contract_batched_hinted(1, c, [m, n], [0, 1], 0, x, [n, n2], [0, 1], 0, m, n2,
                                          n, precision=capi.PREC_FP16X3, a_emax=e)
    assert torch.equal(d_scan.view(torch.int64), d_hint.view(torch.int64))
    capi.contract_batched_hinted(1, a, [m, k], [0, 1], 0, b, [k, n], [0, 1], 0, m, n, k,
                                 precision=capi.PREC_FP32, c_emax=e)
    assert int(e.item()) < -1000
    assert capi.take_device_status() == 0
