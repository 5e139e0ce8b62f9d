"""The 3M ("Gauss") complex product of the split forms (JETGPU_ALGO_3M).

  P1 = Ar Br,  P2 = Ai Bi,  P3 = (Ar + Ai)(Br + Bi),
  Cr = P1 - P2,  Ci = P3 - P1 - P2,

each real product as three tensor-core products of hi/lo pieces. The
reference has one complex product, cblas_cgemm (TensorHelpers.hpp:47-61);
this is a faster way to compute the same C, and its results are held to the
same bound as the 4M forms: 1e-5 relative (Frobenius) against the complex128
oracle contraction of the same labelled tensors.

Checked here:
  * the split stage's sum planes: hi + lo of re + im reconstructs the sum to
    the word format's precision (TF32 2^-21, BF16 2^-16, FP16 2^-21 of the
    largest value, after the operand's power-of-two scale);
  * contractions of edge and ragged shapes (m, n not multiples of the
    128-row tile, k not a multiple of the 32-element stage, k below one
    stage) in TF32X3, BF16X3 and FP16X3 against the oracle;
  * that 3M is refused with the plain and automatic forms and in batches.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _rel(got, want):
    return float(np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300))


def _operands(seed, nl, nc, nr, dims=None):
    from oracle import jet_oracle as jo

    left = ["l%d" % i for i in range(nl)]
    common = ["c%d" % i for i in range(nc)]
    right = ["r%d" % i for i in range(nr)]
    dims = dims or {}
    d = lambda x: dims.get(x, 2)  # noqa: E731
    a_lab = [(left + common)[i] for i in cases.permutation(seed, nl + nc)]
    b_lab = [(common + right)[i] for i in cases.permutation(seed + 1, nc + nr)]
    a_shape = [d(x) for x in a_lab]
    b_shape = [d(x) for x in b_lab]
    a = cases.tensor_data(seed, a_shape, np.complex64)
    b = cases.tensor_data(seed + 2, b_shape, np.complex64)
    want = jo.contract_tensors(jo.OTensor.make(a_lab, a_shape, a, np.complex128),
                               jo.OTensor.make(b_lab, b_shape, b, np.complex128))
    lft = [x for x in a_lab if x not in b_lab]
    com = [x for x in a_lab if x in b_lab]
    rgt = [x for x in b_lab if x not in a_lab]
    m = int(np.prod([d(x) for x in lft])) if lft else 1
    n = int(np.prod([d(x) for x in rgt])) if rgt else 1
    k = int(np.prod([d(x) for x in com])) if com else 1
    return dict(a=a, b=b, a_shape=a_shape, b_shape=b_shape,
                a_perm=[a_lab.index(x) for x in lft + com],
                b_perm=[b_lab.index(x) for x in com + rgt], m=m, n=n, k=k,
                want=np.asarray(want.data).reshape(-1))


@pytest.mark.parametrize("fmt", [0, 1, 2], ids=["tf32", "bf16", "fp16"])
def test_sum_planes_reconstruct_the_sums(cuda, fmt):
    import torch

    from jet_gb300 import capi

    rows, cols = 96, 80
    rng = np.random.default_rng(4 + fmt)
    x = ((rng.standard_normal(rows * cols) + 1j * rng.standard_normal(rows * cols))
         * 2.0**-7).astype(np.complex64)
    xd = torch.from_numpy(x).to(cuda)
    pitch = cols + (-cols) % 8
    word = torch.float32 if fmt == 0 else torch.int16
    planes = torch.zeros(6 * rows * pitch, dtype=word, device=cuda)
    e = torch.zeros(1, dtype=torch.int32, device=cuda)
    if fmt == 2:
        capi.max_exponent(xd, out=e)
    capi.split_planes(xd, [rows, cols], [0, 1], rows, cols, pitch, planes, fmt,
                      extra=capi.SPLIT_SUM, e_max=e if fmt == 2 else None)
    torch.cuda.synchronize()
    if fmt == 0:
        pl = planes.view(6, rows, pitch)[:, :, :cols].double().cpu().numpy()
        scale, tol = 1.0, 2.0**-21
    else:
        hf = planes.view(torch.bfloat16 if fmt == 1 else torch.float16)
        pl = hf.view(6, rows, pitch)[:, :, :cols].double().cpu().numpy()
        scale = 1.0 if fmt == 1 else 2.0 ** (13 - int(e.item()))
        tol = 2.0**-16 if fmt == 1 else 2.0**-21
    xm = x.reshape(rows, cols).astype(np.complex128) * scale
    re, im = xm.real, xm.imag
    # FP16 lo words of small elements go subnormal: 2^-24 absolute spacing.
    floor = 2.0**-24 if fmt == 2 else 0.0
    for (h, lo), want, mag in (((0, 1), re, np.abs(re)), ((2, 3), im, np.abs(im)),
                               ((4, 5), re + im, np.abs(re) + np.abs(im))):
        err = np.abs(pl[h] + pl[lo] - want)
        assert np.all(err <= tol * mag + floor), (fmt, h, float((err - tol * mag).max()))
    if fmt == 2:
        # The largest |re|, |im| sits in [2^13, 2^14), so |re + im| < 2^15.
        big = max(np.abs(re).max(), np.abs(im).max())
        assert 2.0**13 <= big < 2.0**14 and np.abs(pl[4] + pl[5]).max() < 2.0**15


SHAPES = [
    # (nl, nc, nr, dims of some labels): m, n, k
    (8, 9, 8, None),          # 256 x 256 x 512
    (7, 6, 9, None),          # 128 x 512 x 64
    (7, 3, 7, None),          # k = 8: below one stage
    (5, 5, 6, {"l0": 3, "c0": 5, "r0": 3}),   # m = 48, k = 80, n = 96: ragged
    (9, 5, 7, {"c1": 3, "l2": 5, "r3": 3}),   # m = 1280, k = 48, n = 192
]


@pytest.mark.parametrize("shape", SHAPES, ids=[str(s[:3]) for s in SHAPES])
@pytest.mark.parametrize("precision", [1, 3, 4], ids=["tf32x3", "bf16x3", "fp16x3"])
def test_3m_contraction_matches_oracle(cuda, shape, precision):
    import torch

    from jet_gb300 import capi

    nl, nc, nr, dims = shape
    o = _operands(31 + nl + 7 * nc, nl, nc, nr, dims)
    a = torch.from_numpy(o["a"]).to(cuda)
    b = torch.from_numpy(o["b"]).to(cuda)
    got3 = capi.contract(a, o["a_shape"], o["a_perm"], b, o["b_shape"], o["b_perm"], o["m"],
                         o["n"], o["k"], precision=precision, algo=capi.ALGO_3M)
    got4 = capi.contract(a, o["a_shape"], o["a_perm"], b, o["b_shape"], o["b_perm"], o["m"],
                         o["n"], o["k"], precision=precision)
    torch.cuda.synchronize()
    g3 = got3.cpu().numpy()
    g4 = got4.cpu().numpy()
    assert capi.take_device_status() == 0
    assert np.all(np.isfinite(g3))
    assert _rel(g3, o["want"]) <= 1e-5, _rel(g3, o["want"])
    assert _rel(g4, o["want"]) <= 1e-5


def test_3m_workspace_holds_six_planes(cuda):
    from jet_gb300 import capi

    o = _operands(5, 8, 9, 8)
    args = (o["a_shape"], o["a_perm"], o["b_shape"], o["b_perm"], o["m"], o["n"], o["k"],
            capi.C64, capi.PREC_BF16X3)
    w4 = capi.contract_workspace_size(*args)
    w3 = capi.contract_workspace_size(*args, algo=capi.ALGO_3M)
    # B is sized for six planes in both (the N = 256 main loop reads six);
    # 3M adds the two sum planes of A.
    assert w3 - w4 == 2 * (2 * o["m"] * o["k"])


@pytest.mark.parametrize("precision", [0, 2, 5])
def test_3m_refused_outside_split_forms(cuda, precision):
    import torch

    from jet_gb300 import capi

    o = _operands(6, 7, 7, 7)
    a = torch.from_numpy(o["a"]).to(cuda)
    b = torch.from_numpy(o["b"]).to(cuda)
    with pytest.raises(capi.JetGpuError, match="3M product"):
        capi.contract(a, o["a_shape"], o["a_perm"], b, o["b_shape"], o["b_perm"], o["m"],
                      o["n"], o["k"], precision=precision, algo=capi.ALGO_3M)
