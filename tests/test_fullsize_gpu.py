"""Parity at the full config-1 size (A: 2^27, B: 2^25 complex64 elements;
M = 2^14, N = 2^12, K = 2^13), through properties that do not need the
oracle to run the whole problem:
  * the permute is bit-exact: a round trip through the inverse permutation
    returns the input bytes, and 4096 sampled outputs match index arithmetic;
  * the BF16 split reconstructs every element: |x - (hi + lo)| <= 2^-16 |x|;
  * the contraction (BF16x3, TF32x3, FP16x3; 4M and 3M) against complex128 products of
    the oracle's CPU transposes of A and B: every 16th row of C (1024 rows,
    a quarter of a billion entries) exactly, and all of C through a
    Freivalds-style sketch U^T C V (U: M x 8, V: N x 8 complex Gaussian),
    whose relative Frobenius difference from (U^T A')(B' V) estimates C's
    normwise error; both within 1e-5;
  * the contraction is linear in B within 2e-5."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_LEFT, N_COMMON, N_RIGHT = 14, 13, 12


def _workload():
    """Seeded label permutations of both operands, as the config-1 benchmark."""
    import cases

    left = ["l%d" % i for i in range(N_LEFT)]
    common = ["c%d" % i for i in range(N_COMMON)]
    right = ["r%d" % i for i in range(N_RIGHT)]
    a_lab = [(left + common)[i] for i in cases.permutation(1234, N_LEFT + N_COMMON)]
    b_lab = [(common + right)[i] for i in cases.permutation(1235, N_COMMON + N_RIGHT)]
    lft = [x for x in a_lab if x not in b_lab]
    rgt = [x for x in b_lab if x not in a_lab]
    com = [x for x in a_lab if x in b_lab]
    return dict(a_shape=[2] * len(a_lab), b_shape=[2] * len(b_lab),
                a_perm=[a_lab.index(x) for x in lft + com],
                b_perm=[b_lab.index(x) for x in com + rgt],
                m=2 ** N_LEFT, n=2 ** N_RIGHT, k=2 ** N_COMMON)


@pytest.fixture(scope="module")
def data(cuda):
    import torch

    w = _workload()
    g = torch.Generator(device=cuda)
    g.manual_seed(77)
    a = torch.randn(w["m"] * w["k"], dtype=torch.complex64, device=cuda, generator=g) * 2.0**-10
    b = torch.randn(w["k"] * w["n"], dtype=torch.complex64, device=cuda, generator=g) * 2.0**-10
    return w, a, b


def _inverse(perm):
    inv = [0] * len(perm)
    for j, p in enumerate(perm):
        inv[p] = j
    return inv


def test_permute_round_trip_and_samples(data):
    import torch

    from jet_gb300 import capi

    w, a, _ = data
    shape, perm = w["a_shape"], w["a_perm"]
    p = capi.permute(a, shape, perm)
    back = capi.permute(p, [shape[i] for i in perm], _inverse(perm))
    assert torch.equal(back.view(torch.int64), a.view(torch.int64))
    # out[o] = in[i]: bit j of o (from the least significant end) is bit
    # perm[rank-1-j'] of i in the input's own axis order.
    rank = len(shape)
    rng = np.random.default_rng(3)
    o = rng.integers(0, 2 ** rank, 4096, dtype=np.int64)
    i = np.zeros_like(o)
    for jo in range(rank):  # output axis jo holds input axis perm[jo]
        bit = (o >> (rank - 1 - jo)) & 1
        i |= bit << (rank - 1 - perm[jo])
    got = p.cpu().numpy()[o]
    want = a.cpu().numpy()[i]
    assert np.array_equal(got.view(np.int64), want.view(np.int64))


def test_bf16_split_reconstructs_every_element(data):
    import torch

    from jet_gb300 import capi

    w, a, _ = data
    m, k = w["m"], w["k"]
    planes = torch.empty(4 * m * k, dtype=torch.int16, device=a.device)
    capi.split_bf16(a, w["a_shape"], w["a_perm"], m, k, k, planes)
    pl = planes.view(torch.bfloat16).float().view(4, m * k)
    x = capi.permute(a, w["a_shape"], w["a_perm"])
    re, im = x.real, x.imag
    err_re = (re - (pl[0] + pl[1])).abs()
    err_im = (im - (pl[2] + pl[3])).abs()
    assert bool((err_re <= re.abs() * 2.0**-16).all())
    assert bool((err_im <= im.abs() * 2.0**-16).all())


@pytest.fixture(scope="module")
def oracle_operands(data):
    """A' (M x K) and B' (K x N): the operands in ContractTensors' order,
    transposed on the CPU by the oracle (numpy), complex64, plus the
    complex128 sketch factors U^T A' (8 x K) and B' V (K x 8)."""
    from oracle import jet_oracle as jo

    w, a, b = data
    m, n, k = w["m"], w["n"], w["k"]
    r_a, r_b = len(w["a_shape"]), len(w["b_shape"])
    a_lab = ["x%d" % i for i in range(r_a)]
    b_lab = ["y%d" % i for i in range(r_b)]
    at = jo.transpose(jo.OTensor(a_lab, list(w["a_shape"]), a.cpu().numpy()),
                      [a_lab[i] for i in w["a_perm"]]).data.reshape(m, k)
    bt = jo.transpose(jo.OTensor(b_lab, list(w["b_shape"]), b.cpu().numpy()),
                      [b_lab[i] for i in w["b_perm"]]).data.reshape(k, n)
    rng = np.random.default_rng(9)
    u = (rng.standard_normal((m, 8)) + 1j * rng.standard_normal((m, 8))) / np.sqrt(2)
    v = (rng.standard_normal((n, 8)) + 1j * rng.standard_normal((n, 8))) / np.sqrt(2)
    uta = u.T @ at.astype(np.complex128)        # 8 x K
    btv = bt.astype(np.complex128) @ v          # K x 8
    return dict(at=at, bt=bt, u=u, v=v, sketch=uta @ btv)


@pytest.mark.parametrize("precision", ["bf16x3", "tf32x3", "fp16x3", "bf16x3_3m", "fp16x3_3m",
                                       "tf32x3_3m"])
def test_contraction_matches_fp64_every_16th_row_and_sketch(data, oracle_operands, precision):
    from jet_gb300 import capi

    w, a, b = data
    m, n, k = w["m"], w["n"], w["k"]
    form, _, algo = precision.partition("_")
    prec = {"bf16x3": capi.PREC_BF16X3, "tf32x3": capi.PREC_TF32X3,
            "fp16x3": capi.PREC_FP16X3}[form]
    c = capi.contract(a, w["a_shape"], w["a_perm"], b, w["b_shape"], w["b_perm"], m, n, k,
                      precision=prec, algo=capi.ALGO_3M if algo == "3m" else capi.ALGO_4M)
    got = c.view(m, n).cpu().numpy()
    assert capi.take_device_status() == 0
    o = oracle_operands
    rows = np.arange(0, m, 16)
    want = o["at"][rows].astype(np.complex128) @ o["bt"].astype(np.complex128)
    rel_rows = np.linalg.norm(got[rows] - want) / np.linalg.norm(want)
    assert rel_rows <= 1e-5, rel_rows
    sk = o["u"].T @ (got.astype(np.complex128) @ o["v"])
    rel_sketch = np.linalg.norm(sk - o["sketch"]) / np.linalg.norm(o["sketch"])
    assert rel_sketch <= 1e-5, rel_sketch


def test_contraction_linear_in_b(data):
    import torch

    from jet_gb300 import capi

    w, a, b = data
    m, n, k = w["m"], w["n"], w["k"]
    g = torch.Generator(device=a.device)
    g.manual_seed(78)
    b2 = torch.randn(b.shape, dtype=b.dtype, device=b.device, generator=g) * 2.0**-10

    def con(x):
        return capi.contract(a, w["a_shape"], w["a_perm"], x, w["b_shape"], w["b_perm"], m, n, k,
                             precision=capi.PREC_BF16X3)

    lhs = con(b + b2)
    rhs = con(b) + con(b2)
    assert float(torch.linalg.vector_norm(lhs - rhs)) <= 2e-5 * float(torch.linalg.vector_norm(lhs))
