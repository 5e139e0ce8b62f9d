"""Batched contraction (jetgpu_contract_batched): every batch element equals
the single contraction of its slice (jetgpu_contract), for batched/shared
operand combinations, both arithmetic forms, complex64 and complex128."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _case(seed, nl, nc, nr, dtype, batch, a_b, b_b, dev):
    import torch

    left = ["l%d" % i for i in range(nl)]
    common = ["c%d" % i for i in range(nc)]
    right = ["r%d" % i for i in range(nr)]
    a_lab = [(left + common)[i] for i in cases.permutation(seed, nl + nc)]
    b_lab = [(common + right)[i] for i in cases.permutation(seed + 1, nc + nr)]
    na, nb = 2 ** (nl + nc), 2 ** (nc + nr)
    a = cases.tensor_data(seed, [na * (batch if a_b else 1)], dtype)
    b = cases.tensor_data(seed + 3, [nb * (batch if b_b else 1)], dtype)
    lft = [x for x in a_lab if x not in b_lab]
    com = [x for x in a_lab if x in b_lab]
    rgt = [x for x in b_lab if x not in a_lab]
    return dict(a=torch.from_numpy(a).to(dev), b=torch.from_numpy(b).to(dev),
                a_shape=[2] * (nl + nc), b_shape=[2] * (nc + nr),
                a_perm=[a_lab.index(x) for x in lft + com],
                b_perm=[b_lab.index(x) for x in com + rgt],
                m=2 ** nl, n=2 ** nr, k=2 ** nc, na=na, nb=nb)


# (dtype, precision, tensor-core main-loop variant): variant 0 for every form;
# variant 1 shapes only the TF32x3 main loop and variant 2 only the BF16x3 one.
_FORMS = [("complex64", 0, 0), ("complex64", 1, 0), ("complex64", 3, 0), ("complex64", 4, 0),
          ("complex128", 0, 0), ("complex64", 1, 1), ("complex64", 3, 2)]


@pytest.mark.parametrize("a_b,b_b", [(1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("dtype,precision,variant", _FORMS)
@pytest.mark.parametrize("shape", [(7, 6, 8), (1, 9, 3), (4, 10, 1), (0, 5, 0), (8, 8, 8),
                                   (6, 14, 0), (0, 16, 3), (0, 18, 0)])
def test_batched_matches_single(cuda, a_b, b_b, dtype, precision, variant, shape):
    from jet_gb300 import capi

    capi.set_tc_variant(variant)

    batch = 5
    nl, nc, nr = shape
    c = _case(1000 + nl * 31 + nc * 7 + nr, nl, nc, nr, dtype, batch, a_b, b_b, cuda)
    m, n, k = c["m"], c["n"], c["k"]
    out = capi.contract_batched(batch, c["a"], c["a_shape"], c["a_perm"], a_b, c["b"],
                                c["b_shape"], c["b_perm"], b_b, m, n, k,
                                precision=precision).cpu().numpy()[: batch * m * n]
    tol = 1e-5 if dtype == "complex64" else 1e-12
    for bi in range(batch):
        ai = c["a"][bi * c["na"]:(bi + 1) * c["na"]] if a_b else c["a"]
        bj = c["b"][bi * c["nb"]:(bi + 1) * c["nb"]] if b_b else c["b"]
        want = capi.contract(ai, c["a_shape"], c["a_perm"], bj, c["b_shape"], c["b_perm"], m, n,
                             k, precision=0).cpu().numpy()[: m * n]
        got = out[bi * m * n:(bi + 1) * m * n]
        err = np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300)
        assert err <= tol, (bi, err)
    assert capi.take_device_status() == 0
    capi.set_tc_variant(0)


@pytest.mark.parametrize("precision", [0, 1, 3, 4])
@pytest.mark.parametrize("modes", [(2, 2), (2, 0), (0, 2), (2, 1), (1, 2)])
def test_batch_axes_inside_the_permutation(cuda, precision, modes):
    """a_batched / b_batched = 2: the operand is one tensor whose batch axes
    (two of them here, anywhere in its layout) lead its permutation. Same bits
    as reordering the batch to the front first and passing mode 1."""
    import torch

    from jet_gb300 import capi

    rng = np.random.default_rng(17 + 3 * modes[0] + modes[1] + 10 * precision)
    batch, m, k, n = 4, 2 ** 7, 2 ** 6, 2 ** 6

    def operand(mode, lead, tail, seed):
        # Own axes: log2(lead) + log2(tail) axes of 2, in a random layout
        # order; mode 2 adds two batch axes of 2 at random places.
        own = int(np.log2(lead)) + int(np.log2(tail))
        labels = ["o%d" % i for i in range(own)]
        layout = [labels[i] for i in rng.permutation(own)]
        if mode == 2:
            for b in ("s0", "s1"):
                layout.insert(int(rng.integers(0, len(layout) + 1)), b)
        count = batch if mode == 1 else 1
        g = torch.Generator(device=cuda)
        g.manual_seed(seed)
        x = torch.randn(count * 2 ** len(layout), dtype=torch.complex64, device=cuda, generator=g)
        shape = [2] * len(layout)
        own_perm = [layout.index(l) for l in labels]
        if mode == 2:
            perm = [layout.index("s0"), layout.index("s1")] + own_perm
            # The reference: batch axes moved to the front, then mode 1.
            front = capi.permute(x, shape, [layout.index("s0"), layout.index("s1")] +
                                 [i for i, l in enumerate(layout) if l not in ("s0", "s1")])
            rest = [l for l in layout if l not in ("s0", "s1")]
            ref = (front, [2] * len(rest), [rest.index(l) for l in labels], 1)
            return (x, shape, perm, 2), ref
        return (x, shape, own_perm, mode), (x, shape, own_perm, mode)

    (a, a_ref) = operand(modes[0], m, k, 5)
    (b, b_ref) = operand(modes[1], k, n, 6)
    got = capi.contract_batched(batch, a[0], a[1], a[2], a[3], b[0], b[1], b[2], b[3], m, n, k,
                                precision=precision)
    want = capi.contract_batched(batch, a_ref[0], a_ref[1], a_ref[2], a_ref[3], b_ref[0],
                                 b_ref[1], b_ref[2], b_ref[3], m, n, k, precision=precision)
    assert torch.equal(got.view(torch.int64), want.view(torch.int64))
    assert capi.take_device_status() == 0
