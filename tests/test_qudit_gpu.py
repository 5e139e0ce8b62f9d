"""Qutrit circuits (local dimension 3; the non-power-of-2 path: mixed-radix
permutes, odd-sized products): amplitudes on the GPU against the complex128
oracle, plain and AUTO forms, and a sliced run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle(net, path):
    from oracle import jet_oracle as jo

    tn = jo.OTensorNetwork()
    for lab, sh, d in net.tensors:
        tn.add_tensor(jo.OTensor.make(lab, sh, d, np.complex128))
    return tn.contract(path).data[0]


@pytest.mark.parametrize("precision", [0, 2])
def test_qutrit_5x5_amplitude(cuda, precision):
    import jet_gb300 as jet
    from jet_gb300 import circuits

    net = circuits.qudit_circuit_network(5, 5, 8, d=3, seed=4)
    path = circuits.find_path(net, restarts=4, seed=4)
    want = _oracle(net, path)
    old = jet.get_precision()
    jet.set_precision(precision)
    try:
        tn = jet.TensorNetwork(dtype="complex64")
        for lab, sh, d in net.tensors:
            tn.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype="complex64"))
        got = tn.contract(path).data[0]
    finally:
        jet.set_precision(old)
    assert abs(got - want) <= 1e-5 * abs(want)


def test_qutrit_sliced(cuda):
    import jet_gb300 as jet
    from jet_gb300 import circuits

    net = circuits.qudit_circuit_network(4, 4, 6, d=3, seed=7)
    path = circuits.find_path(net, restarts=4, seed=7)
    sliced = circuits.choose_slices(net, path, 2)
    want = _oracle(net, path)
    tn = jet.TensorNetwork(dtype="complex128")
    for lab, sh, d in net.tensors:
        tn.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype="complex128"))
    sc = jet.SlicedContractorC128(tn, path, sliced, 0)
    sc.set_batch_size(3)
    assert sc.num_slices == 9
    got = sc.contract()[0]
    assert abs(got - want) <= 1e-10 * abs(want)
