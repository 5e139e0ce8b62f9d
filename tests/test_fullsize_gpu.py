"""Parity at the full config-1 size (A: 2^27, B: 2^25 complex64 elements;
M = 2^14, N = 2^12, K = 2^13), through properties that do not need the
oracle to run the whole problem:
  * the permute is bit-exact: a round trip through the inverse permutation
    returns the input bytes, and 4096 sampled outputs match index arithmetic;
  * the BF16 split reconstructs every element: |x - (hi + lo)| <= 2^-16 |x|;
  * the contraction (BF16x3, TF32x3) matches complex128 on 16 sampled rows of
    C within 1e-5, and is linear in B within 2e-5."""
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


@pytest.mark.parametrize("precision", ["bf16x3", "tf32x3"])
def test_contraction_rows_match_fp64(data, precision):
    from jet_gb300 import capi

    w, a, b = data
    m, n, k = w["m"], w["n"], w["k"]
    prec = capi.PREC_BF16X3 if precision == "bf16x3" else capi.PREC_TF32X3
    c = capi.contract(a, w["a_shape"], w["a_perm"], b, w["b_shape"], w["b_perm"], m, n, k,
                      precision=prec)
    rows = np.random.default_rng(5).choice(m, 16, replace=False)
    at = capi.permute(a, w["a_shape"], w["a_perm"]).view(m, k)[rows].cpu().numpy()
    bt = capi.permute(b, w["b_shape"], w["b_perm"]).view(k, n).cpu().numpy()
    want = at.astype(np.complex128) @ bt.astype(np.complex128)
    got = c.view(m, n)[rows].cpu().numpy()
    assert np.linalg.norm(got - want) <= 1e-5 * np.linalg.norm(want)
    assert capi.take_device_status() == 0


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
