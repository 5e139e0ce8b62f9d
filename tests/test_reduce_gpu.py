"""GPU parity of the element-wise and reduction entry points: AddTensors,
Conj, the FP64 cross-slice sum and the device SliceIndex gather."""
import hashlib

import numpy as np
import pytest

import cases
from oracle import jet_oracle as jo

pytestmark = pytest.mark.gpu


def _dev(x, dev):
    import torch

    return torch.from_numpy(np.ascontiguousarray(x)).to(dev)


def test_add_tensors_reference_cases(cuda, golden):
    """Tensor::AddTensors = transpose B into A's order, then add."""
    from jet_gb300 import capi

    for c in golden["ref"]["add"]:
        a = cases.tensor_data(c["seed"], c["a_shape"], c["dtype"])
        b = cases.tensor_data(c["seed"] + 1, c["b_shape"], c["dtype"])
        perm = [c["b_labels"].index(x) for x in c["a_labels"]]
        bt = capi.permute(_dev(b, cuda), c["b_shape"], perm)
        out = capi.add(_dev(a, cuda), bt).cpu().numpy()
        assert hashlib.sha256(out.tobytes()).hexdigest() == c["sha256"]


def test_conj(cuda):
    from jet_gb300 import capi

    for dt in (np.complex64, np.complex128):
        x = cases.tensor_data(1, [1000], dt)
        assert np.array_equal(capi.conj(_dev(x, cuda)).cpu().numpy(), np.conj(x))


@pytest.mark.parametrize("n_slices,size", [(1, 1), (4096, 1), (37, 3), (5, 1 << 16), (1000, 300)])
@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_slice_sum_f64(cuda, n_slices, size, dtype):
    from jet_gb300 import capi

    r = cases.tensor_data(n_slices + size, [n_slices * size], dtype)
    want = r.astype(np.complex128).reshape(n_slices, size).sum(axis=0)
    got = capi.slice_sum_f64(_dev(r, cuda), n_slices, size).cpu().numpy()
    assert np.allclose(got, want, rtol=1e-13, atol=1e-13)
    got2 = capi.slice_sum_f64(_dev(r, cuda), n_slices, size,
                              out=_dev(got.copy(), cuda), accumulate=True).cpu().numpy()
    assert np.allclose(got2, 2 * want, rtol=1e-13, atol=1e-13)


def test_slice_gather_reference_cases(cuda, golden):
    """Single-axis slices equal Tensor::SliceIndex (Tensor.hpp:493-526)."""
    from jet_gb300 import capi

    for c in golden["ref"]["slice"]:
        x = cases.tensor_data(c["seed"], c["shape"], c["dtype"])
        ax = c["labels"].index(c["index"])
        out = capi.slice_gather(_dev(x, cuda), c["shape"], [ax], [1], c["value"], 1)
        got = out.cpu().numpy()
        assert hashlib.sha256(got.tobytes()).hexdigest() == c["sha256"]


def test_slice_gather_network_values(cuda):
    """A run of network-wide slice values: value v unravels row-major over the
    sliced dims (3, 2, 4); this tensor carries the first and last of them."""
    from jet_gb300 import capi

    shape = [4, 5, 3, 2]
    lab = ["p", "q", "r", "s"]  # sliced indices of the network: r (3), t (2), p (4)
    x = cases.tensor_data(9, shape, np.complex64)
    axes = [2, 0]
    strides = [2 * 4, 1]  # r is outermost, p innermost
    first, count = 5, 17
    got = capi.slice_gather(_dev(x, cuda), shape, axes, strides, first, count).cpu().numpy()
    t = jo.OTensor.make(lab, shape, x, np.complex64)
    outs = []
    for v in range(first, first + count):
        rv, pv = (v // 8) % 3, v % 4
        s = jo.slice_index(jo.slice_index(t, "r", rv), "p", pv)
        outs.append(s.data)
    assert np.array_equal(got, np.concatenate(outs))


def test_max_exponent(cuda):
    from jet_gb300 import capi

    x = np.zeros(5000, np.complex64)
    assert capi.max_exponent(_dev(x, cuda)) == -1000
    x[1234] = 3.0 - 0.5j
    assert capi.max_exponent(_dev(x, cuda)) == 1
    x[17] = 1j * 2.0**-30
    assert capi.max_exponent(_dev(x.astype(np.complex128), cuda)) == 1
