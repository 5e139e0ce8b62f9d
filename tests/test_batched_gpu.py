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


@pytest.mark.parametrize("a_b,b_b", [(1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("dtype,precision", [("complex64", 0), ("complex64", 1),
                                             ("complex64", 3), ("complex64", 4),
                                             ("complex128", 0)])
@pytest.mark.parametrize("shape", [(7, 6, 8), (1, 9, 3), (4, 10, 1), (0, 5, 0), (8, 8, 8),
                                   (6, 14, 0), (0, 16, 3), (0, 18, 0)])
@pytest.mark.parametrize("variant", [0, 1, 2])
def test_batched_matches_single(cuda, a_b, b_b, dtype, precision, shape, variant):
    from jet_gb300 import capi

    if (variant == 1 and precision != 1) or (variant == 2 and precision != 3):
        pytest.skip("variant 1 shapes the TF32x3 main loop, variant 2 the BF16x3 one")
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
