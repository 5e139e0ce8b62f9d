"""GPU permute parity through the C-ABI (jetgpu_permute): bit-exact against
the reference Permuter golden vectors, the compiled reference's transposes
(SHA-256 fixtures), and the oracle on larger seeded tensors; round trips at
full size."""
import hashlib

import numpy as np
import pytest

import cases
from oracle import jet_oracle as jo

pytestmark = pytest.mark.gpu


def _to_dev(x, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(x)).to(dev)


def _perm_of(old, new):
    pos = {l: i for i, l in enumerate(old)}
    return [pos[l] for l in new]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_permuter_golden_vectors(cuda, golden):
    from jet_gb300 import capi

    for c in golden["permuter"]["cases"]:
        x = np.array([complex(a, b) for a, b in c["input"]], np.complex64)
        got = capi.permute(_to_dev(x, cuda), c["shape"], _perm_of(c["old"], c["new"]))
        want = np.array([complex(a, b) for a, b in c["expected"]], np.complex64)
        assert np.array_equal(got.cpu().numpy(), want), c["source"]


def test_transposes_match_reference_bit_exact(cuda, golden):
    from jet_gb300 import capi

    for c in golden["ref"]["transpose"]:
        x = cases.tensor_data(c["seed"], c["shape"], c["dtype"])
        got = capi.permute(_to_dev(x, cuda), c["shape"], _perm_of(c["old"], c["new"]))
        assert _sha(got.cpu().numpy()) == c["sha256"], c


@pytest.mark.parametrize("rank", [12, 13, 16, 20, 22])
@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_random_pow2_vs_oracle(cuda, rank, dtype):
    from jet_gb300 import capi

    for rep in range(3):
        seed = 40000 + 100 * rank + rep
        shape = [2] * rank
        lab = cases.labels(rank)
        perm = cases.permutation(seed, rank)
        x = cases.tensor_data(seed, shape, dtype)
        got = capi.permute(_to_dev(x, cuda), shape, perm).cpu().numpy()
        want = jo.transpose(jo.OTensor.make(lab, shape, x, dtype), [lab[i] for i in perm]).data
        assert np.array_equal(got, want)


@pytest.mark.parametrize("shape", [[4, 2, 8, 2, 16, 2, 8], [64, 2, 128, 4], [2, 2, 1, 2, 2, 1, 256, 8],
                                   [3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3], [5, 1, 7, 2, 3, 6], [1, 1, 1]])
def test_mixed_shapes_vs_oracle(cuda, shape):
    from jet_gb300 import capi

    r = len(shape)
    lab = cases.labels(r)
    for rep in range(2):
        seed = 50000 + 7 * r + rep
        perm = cases.permutation(seed, r)
        x = cases.tensor_data(seed, shape, np.complex64)
        got = capi.permute(_to_dev(x, cuda), shape, perm).cpu().numpy()
        want = jo.transpose(jo.OTensor.make(lab, shape, x, np.complex64),
                            [lab[i] for i in perm]).data
        assert np.array_equal(got, want)


@pytest.mark.parametrize("shape,batch,dtype", [([3] * 12, 1, np.complex64), ([3] * 12, 1, np.complex128),
                                               ([9, 5, 7, 3, 11, 4, 7], 1, np.complex64),
                                               ([6] * 7, 1, np.complex128), ([3] * 11, 3, np.complex64),
                                               ([5, 2, 9, 2, 3, 7, 2, 5, 2], 4, np.complex128),
                                               ([1000, 3, 7, 2], 1, np.complex64),
                                               ([3] * 8, 3, np.complex64)])
def test_non_pow2_tiled_vs_oracle(cuda, shape, batch, dtype):
    """Non-power-of-2 dims of at least 2^18 elements per launch take the tiled
    kernel (several tiles per pass of a CTA, batches enumerated with the
    tiles); smaller ones, and shapes whose innermost axes are too long for a
    tile of at most 1024 elements, take the gather kernel. Bit-exact against
    the oracle's transpose for each batch item."""
    from jet_gb300 import capi

    r = len(shape)
    lab = cases.labels(r)
    size = int(np.prod(shape))
    for rep in range(2):
        seed = 61000 + 13 * r + rep
        perm = cases.permutation(seed, r)
        x = cases.tensor_data(seed, [batch * size], dtype)
        got = capi.permute(_to_dev(x, cuda), shape, perm, batch=batch).cpu().numpy()
        for b in range(batch):
            want = jo.transpose(jo.OTensor.make(lab, shape, x[b * size:(b + 1) * size], dtype),
                                [lab[i] for i in perm]).data
            assert np.array_equal(got[b * size:(b + 1) * size], want), b


@pytest.mark.parametrize("shape,perm,batch,dtype", [
    ([3] * 12, [8, 9, 10, 11, 4, 5, 6, 7, 0, 1, 2, 3], 1, np.complex64),
    ([3] * 12, [8, 9, 10, 11, 4, 5, 6, 7, 0, 1, 2, 3], 2, np.complex128),
    ([3] * 12, [6, 7, 8, 9, 10, 11, 0, 1, 2, 3, 4, 5], 1, np.complex64),
    ([9] * 6, [3, 4, 5, 0, 1, 2], 1, np.complex64)])
def test_merged_axes_tiled_on_original_axes_vs_oracle(cuda, shape, perm, batch, dtype):
    """Blocks of axes that stay in order merge into axes of 81 to 729 on both
    sides, too long for a tile of at most 1024 elements; the tile plan is then
    built on the original axes. Bit-exact against the oracle per batch item."""
    from jet_gb300 import capi

    r = len(shape)
    lab = cases.labels(r)
    size = int(np.prod(shape))
    seed = 62000 + 17 * r + batch
    x = cases.tensor_data(seed, [batch * size], dtype)
    got = capi.permute(_to_dev(x, cuda), shape, perm, batch=batch).cpu().numpy()
    for b in range(batch):
        want = jo.transpose(jo.OTensor.make(lab, shape, x[b * size:(b + 1) * size], dtype),
                            [lab[i] for i in perm]).data
        assert np.array_equal(got[b * size:(b + 1) * size], want), b


def test_batched_permute(cuda):
    from jet_gb300 import capi

    shape = [2] * 13
    perm = cases.permutation(77, 13)
    batch = 5
    x = cases.tensor_data(77, [batch] + shape, np.complex64)
    got = capi.permute(_to_dev(x, cuda), shape, perm, batch=batch).cpu().numpy()
    want = np.ascontiguousarray(
        np.transpose(x.reshape([batch] + shape), [0] + [p + 1 for p in perm])).reshape(-1)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("rank,dtype", [(27, "complex64"), (26, "complex128")])
def test_full_size_round_trip(cuda, rank, dtype):
    """Config-1 sized tensors: permute then the inverse permutation restores
    the input bit for bit, and a permute moves every element exactly once
    (checksum of sums per output bit-plane)."""
    import torch

    from jet_gb300 import capi

    tdt = getattr(torch, dtype)
    shape = [2] * rank
    perm = cases.permutation(rank * 31, rank)
    inv = [0] * rank
    for j, p in enumerate(perm):
        inv[p] = j
    g = torch.Generator(device=cuda)
    g.manual_seed(rank)
    x = torch.randn(2 ** rank, dtype=tdt, device=cuda, generator=g)
    y = capi.permute(x, shape, perm)
    z = capi.permute(y, [2] * rank, inv)
    assert torch.equal(z, x)
    # The element at old multi-index 0...01 (last axis = 1) moves to the
    # output position of that axis.
    j = perm.index(rank - 1)
    assert torch.equal(y[1 << (rank - 1 - j)], x[1])
    assert capi.take_device_status() == 0


def test_empty_and_unit_shapes(cuda):
    import torch

    from jet_gb300 import capi

    x = torch.arange(6, dtype=torch.float32, device=cuda).to(torch.complex64)
    y = capi.permute(x, [1, 6, 1], [2, 0, 1])
    assert torch.equal(x, y)
    s = torch.tensor([3 + 4j], dtype=torch.complex64, device=cuda)
    assert torch.equal(capi.permute(s, [], []), s)
