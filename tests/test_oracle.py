"""Pins the CPU oracle (oracle/jet_oracle.py) before it is trusted.

  * against the golden vectors of the reference's own tests (committed under
    tests/golden/, parsed from test/Test_Permuter.cpp and produced by the
    compiled reference headers);
  * against literal expectations of Test_Tensor.cpp, Test_TensorNetwork.cpp,
    Test_PathInfo.cpp and python/tests/test_task_based_contractor.py;
  * against the compiled reference itself when oracle/_ref is present.
"""
import hashlib

import numpy as np
import pytest

import cases
from oracle import jet_oracle as jo
from oracle import ref


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _c(lst, dtype):
    return np.array([complex(a, b) for a, b in lst], dtype=dtype)


def test_permuter_golden_vectors(golden):
    for c in golden["permuter"]["cases"]:
        t = jo.OTensor.make(c["old"], c["shape"], _c(c["input"], np.complex64), np.complex64)
        got = jo.transpose(t, c["new"]).data
        assert np.array_equal(got, _c(c["expected"], np.complex64)), c["source"]


def test_transpose_vs_reference(golden):
    for c in golden["ref"]["transpose"]:
        x = cases.tensor_data(c["seed"], c["shape"], c["dtype"])
        got = jo.transpose(jo.OTensor.make(c["old"], c["shape"], x, c["dtype"]), c["new"]).data
        assert _sha(got) == c["sha256"], c


def test_contract_vs_reference(golden):
    for c in golden["ref"]["contract"]:
        a = cases.tensor_data(c["seed"], c["a_shape"], c["dtype"])
        b = cases.tensor_data(c["seed"] + 1, c["b_shape"], c["dtype"])
        out = jo.contract_tensors(jo.OTensor.make(c["a_labels"], c["a_shape"], a, np.complex128),
                                  jo.OTensor.make(c["b_labels"], c["b_shape"], b, np.complex128))
        assert out.indices == c["out_labels"]
        assert out.shape == c["out_shape"]
        want = _c(c["out"], np.complex128)
        tol = 1e-5 if c["dtype"] == "complex64" else 1e-12
        assert np.linalg.norm(out.data - want) <= tol * max(np.linalg.norm(want), 1e-30)


def test_slice_and_add_vs_reference(golden):
    for c in golden["ref"]["slice"]:
        x = cases.tensor_data(c["seed"], c["shape"], c["dtype"])
        out = jo.slice_index(jo.OTensor.make(c["labels"], c["shape"], x, c["dtype"]),
                             c["index"], c["value"])
        assert out.indices == c["out_labels"] and out.shape == c["out_shape"]
        assert _sha(out.data) == c["sha256"]
    for c in golden["ref"]["add"]:
        a = cases.tensor_data(c["seed"], c["a_shape"], c["dtype"])
        b = cases.tensor_data(c["seed"] + 1, c["b_shape"], c["dtype"])
        out = jo.add_tensors(jo.OTensor.make(c["a_labels"], c["a_shape"], a, c["dtype"]),
                             jo.OTensor.make(c["b_labels"], c["b_shape"], b, c["dtype"]))
        assert out.indices == c["out_labels"]
        assert _sha(out.data) == c["sha256"]


def test_network_vs_reference(golden):
    for c in golden["ref"]["network"]:
        tensors, path = cases.network(dict(c))
        tn = jo.OTensorNetwork()
        for lab, sh, d in tensors:
            tn.add_tensor(jo.OTensor.make(lab, sh, d, np.complex128))
        if c["sliced"]:
            tn.slice_indices(c["sliced"], c["slice_value"])
        info = jo.OPathInfo(tn, path)
        assert info.total_flops() == c["flops"]
        assert info.total_memory() == c["memory"]
        out = tn.contract(path)
        want = _c(c["out"], np.complex128)
        assert np.allclose(out.data, want, rtol=1e-5, atol=1e-7)


def test_literal_expectations():
    # Test_Tensor.cpp:537-541: (0.5+0.25i) tensors of shape 2x3x4 / 3x4x2.
    a = jo.OTensor.make(["a", "b", "c"], [2, 3, 4], np.full(24, 0.5 + 0.25j))
    b = jo.OTensor.make(["b", "c", "d"], [3, 4, 2], np.full(24, 0.5 + 0.25j))
    c = jo.contract_tensors(a, b)
    assert c.indices == ["a", "d"] and np.all(c.data == 2.25 + 3j)
    # Test_Tensor.cpp:579-598 SliceIndex.
    t = jo.OTensor.make(["x", "y"], [2, 3], [1, 2, 3, 4, 5, 6])
    assert list(jo.slice_index(t, "y", 2).data) == [3, 6]
    # Test_Tensor.cpp:652-667 AddTensors with swapped labels.
    l = jo.OTensor.make(["i", "j"], [2, 2], [1, 2, 3, 4])
    r = jo.OTensor.make(["j", "i"], [2, 2], [1j, 2j, 3j, 4j])
    assert list(jo.add_tensors(l, r).data) == [1 + 1j, 2 + 3j, 3 + 2j, 4 + 4j]
    # Test_TensorNetwork.cpp:293-316: slice [1, :, 2] of A0B1C2 (values i + 2i j).
    tn = jo.OTensorNetwork()
    shape = [2, 3, 4]
    vals = np.arange(24) * (1 + 2j)
    tn.add_tensor(jo.OTensor.make(["A0", "B1", "C2"], shape, vals))
    tn.add_tensor(jo.OTensor.make(["D3"], [2], [0, 1 + 2j]))
    tn.slice_indices(["A0", "C2"], 1 * 4 + 2)
    node = tn.nodes[0]
    assert node.name == "A0(1)B1C2(2)"
    assert node.tensor.indices == ["B1"]
    assert list(node.tensor.data) == [14 + 28j, 18 + 36j, 22 + 44j]
    with pytest.raises(ValueError, match="Sliced index does not exist."):
        tn.slice_indices(["E0"], 0)


def test_task_names_and_totals():
    # python/tests/test_task_based_contractor.py:18-50 (the conftest network:
    # A(i,j) = [[1,0],[0,1]]... contracted with path [[0,1],[2,3]]).
    tn = jo.OTensorNetwork()
    tn.add_tensor(jo.OTensor.make(["i", "j"], [2, 2], [1, 0, 0, 1]))
    tn.add_tensor(jo.OTensor.make(["j", "k"], [2, 2], [1, 0, 0, 1]))
    tn.add_tensor(jo.OTensor.make(["k"], [2], [1, -1j]))
    info = jo.OPathInfo(tn, [(0, 1), (2, 3)])
    names = [jo.task_name(s) for s in info.steps]
    assert names == ["0:ij", "1:jk", "2:k", "3:ik", "4:i"]
    assert info.total_flops() == 2 * 2 * 4 + 2 * 4
    assert info.step_memory(3) + info.step_memory(4) == 6


@pytest.mark.skipif(not ref.available(), reason="compiled reference not present")
def test_oracle_matches_compiled_reference_random():
    rng = np.random.default_rng(7)
    for r in range(2, 12):
        shape = [int(x) for x in rng.integers(1, 4, size=r)]
        lab = ["y%d" % i for i in range(r)]
        x = cases.tensor_data(100 + r, shape, np.complex64)
        new = [lab[i] for i in rng.permutation(r)]
        want = ref.tensor_transpose(x, shape, lab, new)
        got = jo.transpose(jo.OTensor.make(lab, shape, x, np.complex64), new).data
        assert np.array_equal(got, want)
