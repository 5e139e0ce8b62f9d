"""The Jet Python API (C++17 host API via pybind) on the GPU: the cases of the
reference's python/tests (test_tensor.py, test_tensor_network.py,
test_pathinfo.py, test_task_based_contractor.py) and C++ tests
(Test_Tensor.cpp, Test_TensorNetwork.cpp, Test_TaskBasedContractor.cpp)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DTYPES = ["complex64", "complex128"]


@pytest.fixture(scope="module")
def jet(cuda):
    import jet_gb300

    return jet_gb300


@pytest.fixture
def tensor_network(jet):
    def make(dtype):
        A = jet.Tensor(shape=[2, 2], indices=["i", "j"], data=[1, 1j, -1j, 1], dtype=dtype)
        B = jet.Tensor(shape=[2, 2], indices=["j", "k"], data=[1, 0, 0, 1], dtype=dtype)
        C = jet.Tensor(shape=[2], indices=["k"], data=[1, 0], dtype=dtype)
        tn = jet.TensorNetwork(dtype=dtype)
        tn.add_tensor(A, ["A", "Hermitian"])
        tn.add_tensor(B, ["B", "Identity", "Real"])
        tn.add_tensor(C, ["C", "Vector", "Real"])
        return tn

    return make


@pytest.mark.parametrize("dtype", DTYPES)
def test_tensor_basics(jet, dtype):
    t = jet.Tensor(shape=[1, 2, 3], indices=["i", "j", "k"], data=range(6), dtype=dtype)
    assert t.data == [0, 1, 2, 3, 4, 5]
    assert t.index_to_dimension_map == {"i": 1, "j": 2, "k": 3}
    assert jet.Tensor(other=t, dtype=dtype) == t
    t.data = [9, 8, 7, 6, 5, 4]
    assert t.data == [9, 8, 7, 6, 5, 4]
    assert jet.Tensor(shape=[1, 2, 3], dtype=dtype).indices == ["?a", "?b", "?c"]
    r = jet.Tensor(shape=[1, 2], indices=["i", "j"], data=[1j, 2 + 3j], dtype=dtype)
    assert repr(r) == "Size = 2\nIndices = {i  j}\nData = {(0,1)  (2,3)}"


@pytest.mark.parametrize("dtype", DTYPES)
def test_contract_tensors_reference_cases(jet, dtype):
    # Test_Tensor.cpp:515-563 and python/tests/test_tensor.py:181-187.
    a = jet.Tensor(indices=["a", "b", "c"], shape=[2, 3, 4], data=[0.5 + 0.25j] * 24, dtype=dtype)
    b = jet.Tensor(indices=["b", "c", "d"], shape=[3, 4, 2], data=[0.5 + 0.25j] * 24, dtype=dtype)
    c = jet.contract_tensors(a, b)
    assert c.indices == ["a", "d"] and c.shape == [2, 2]
    assert c.data == [2.25 + 3j] * 4
    t1 = jet.Tensor(indices=["a", "b"], shape=[2, 2], data=[0, 1, 1, 0], dtype=dtype)
    t2 = jet.Tensor(indices=["b"], shape=[2], data=[1, 0], dtype=dtype)
    assert jet.contract_tensors(t1, t2) == jet.Tensor(indices=["a"], shape=[2], data=[0, 1],
                                                      dtype=dtype)
    t1 = jet.Tensor(indices=["a"], shape=[2], data=[0, 1], dtype=dtype)
    t2 = jet.Tensor(indices=["a", "b"], shape=[2, 2], data=[0, 1, 2, 3], dtype=dtype)
    assert t1.contract_with_tensor(t2).data == [2, 3]
    s1 = jet.Tensor(indices=["a", "b"], shape=[2, 2], data=[1] * 4, dtype=dtype)
    s = jet.contract_tensors(s1, s1)
    assert s.indices == [] and s.data == [4] and s.is_scalar()


@pytest.mark.parametrize("dtype", DTYPES)
def test_transpose_slice_add_reshape_conj(jet, dtype):
    t = jet.Tensor(indices=["x", "y"], shape=[2, 3], data=[1, 2, 3, 4, 5, 6], dtype=dtype)
    tt = jet.transpose(t, ["y", "x"])
    assert tt.indices == ["y", "x"] and tt.shape == [3, 2] and tt.data == [1, 4, 2, 5, 3, 6]
    assert jet.transpose(t, [1, 0]) == tt
    assert jet.slice_index(t, "x", 1).data == [4, 5, 6]
    assert jet.slice_index(t, "y", 2).data == [3, 6]
    assert jet.slice_index(t, "y", 2).indices == ["x"]
    lhs = jet.Tensor(indices=["i", "j"], shape=[2, 2], data=[1, 2, 3, 4], dtype=dtype)
    rhs = jet.Tensor(indices=["j", "i"], shape=[2, 2], data=[1j, 2j, 3j, 4j], dtype=dtype)
    assert jet.add_tensors(lhs, rhs).data == [1 + 1j, 2 + 3j, 3 + 2j, 4 + 4j]
    r = jet.reshape(t, [3, 2])
    assert r.indices == ["?a", "?b"] and r.data == t.data
    with pytest.raises(RuntimeError, match="Size is inconsistent between tensors."):
        jet.reshape(t, [3, 3])
    assert jet.conj(jet.Tensor(indices=["x"], shape=[1], data=[0.5 + 0.25j], dtype=dtype)).data == [0.5 - 0.25j]
    with pytest.raises(RuntimeError, match="Number of indices cannot be zero."):
        jet.transpose(jet.Tensor(dtype=dtype), ["y", "x"])
    with pytest.raises(RuntimeError, match="Size of ordering must match number of tensor indices."):
        jet.transpose(jet.Tensor(dtype=dtype), [1, 0])
    with pytest.raises(RuntimeError, match="Tensor addition with disjoint indices is not supported."):
        jet.add_tensors(lhs, jet.Tensor(indices=["i", "k"], shape=[2, 2], dtype=dtype))


@pytest.mark.parametrize("dtype", DTYPES)
def test_tensor_network_contract_and_slice(jet, dtype):
    tn = jet.TensorNetwork(dtype=dtype)
    a1 = jet.Tensor(indices=["A"], shape=[3], data=[0, 1, 2], dtype=dtype)
    tn.add_tensor(a1)
    tn.add_tensor(a1)
    assert tn.contract().data == [5]
    assert tn.path == [(0, 1)]
    tn = jet.TensorNetwork(dtype=dtype)
    a = jet.Tensor(indices=["A0", "B1", "C2"], shape=[2, 3, 4],
                   data=[i + 2j * i for i in range(24)], dtype=dtype)
    b = jet.Tensor(indices=["D3"], shape=[2], data=[0, 1], dtype=dtype)
    tn.add_tensor(a)
    tn.add_tensor(b)
    tn.slice_indices(["A0", "C2"], 1 * 4 + 2)
    node = tn.nodes[0]
    assert node.name == "A0(1)B1C2(2)"
    assert node.indices == ["A0(1)", "B1", "C2(2)"]
    assert node.tensor.indices == ["B1"]
    assert node.tensor.data == [14 + 28j, 18 + 36j, 22 + 44j]
    with pytest.raises(RuntimeError, match="Sliced index does not exist."):
        tn.slice_indices(["E0", "B0"], 0)


@pytest.mark.parametrize("dtype", DTYPES)
def test_task_based_contractor(jet, dtype, tensor_network):
    # python/tests/test_task_based_contractor.py:18-50.
    tn = tensor_network(dtype)
    path = jet.PathInfo(tn=tn, path=[[0, 1], [2, 3]])
    tbc = jet.TaskBasedContractor(dtype=dtype)
    assert tbc.add_contraction_tasks(tn, path) == 0
    assert tbc.add_deletion_tasks() == 4
    assert tbc.add_reduction_task() == 1
    tbc.contract()
    want = jet.Tensor(shape=[2], indices=["i"], data=[1, -1j], dtype=dtype)
    assert tbc.name_to_tensor_map == {"0:ij": None, "1:jk": None, "2:k": None, "3:ik": None,
                                      "4:i:results[0]": want}
    assert tbc.name_to_parents_map == {"0:ij": {"3:ik"}, "1:jk": {"3:ik"},
                                       "2:k": {"4:i:results[0]"}, "3:ik": {"4:i:results[0]"}}
    assert tbc.results == [want]
    assert tbc.reduction_result == want
    assert tbc.flops == 2 * 2 * 4 + 2 * 4
    assert tbc.memory == 6


def test_pathinfo(jet):
    p = jet.PathInfo()
    assert p.num_leaves == 0 and p.steps == [] and p.path == [] and p.total_flops() == 0
    tn = jet.TensorNetwork()
    ia = tn.add_tensor(jet.Tensor(), ["A"])
    ib = tn.add_tensor(jet.Tensor(), ["B"])
    tn.add_tensor(jet.Tensor(), ["C"])
    info = jet.PathInfo(tn, [(ia, ib)])
    assert info.num_leaves == 3 and info.path == [(ia, ib)] and len(info.steps) == 4


def test_sliced_networks_share_tasks_and_reduce(jet):
    """Several slices of one circuit network in one contractor: shared
    slice-independent tasks, and the FP64 reduction equals the unsliced
    amplitude (oracle in complex128)."""
    from jet_gb300 import circuits
    from oracle import jet_oracle as jo

    net = circuits.random_circuit_network(3, 3, 4, seed=13)
    path = circuits.greedy_path(net, seed=13)
    sliced = circuits.choose_slices(net, path, 2)
    tbc = jet.TaskBasedContractor(dtype="complex64")
    shared = 0
    for v in range(4):
        tn = jet.TensorNetwork(dtype="complex64")
        for lab, sh, d in net.tensors:
            tn.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype="complex64"))
        tn.slice_indices(sliced, v)
        shared += tbc.add_contraction_tasks(tn, jet.PathInfo(tn, path))
    tbc.add_deletion_tasks()
    tbc.add_reduction_task()
    tbc.contract()
    assert shared > 0
    otn = jo.OTensorNetwork()
    for lab, sh, d in net.tensors:
        otn.add_tensor(jo.OTensor.make(lab, sh, d, np.complex128))
    want = otn.contract(path).data[0]
    got = tbc.reduction_result.data[0]
    assert abs(got - want) <= 1e-5 * abs(want)


@pytest.mark.parametrize("precision", [0, 2])
def test_config0_amplitude(jet, precision):
    """4x4 grid, 8 cycles: TensorNetwork::Contract(path) on the GPU against the
    complex128 oracle and the reference's own CPU result (golden). Whole
    networks use plain FP32 or AUTO (a split form on the large steps only):
    forcing a split form onto ~200 steps of 2x2 gates compounds the tensor
    core's biased accumulation past 1e-5."""
    import json
    import os

    from jet_gb300 import circuits
    from oracle import jet_oracle as jo

    net = circuits.random_circuit_network(4, 4, 8, seed=14)
    path = circuits.greedy_path(net, seed=14)
    old = jet.get_precision()
    jet.set_precision(precision)
    try:
        tn = jet.TensorNetwork(dtype="complex64")
        for lab, sh, d in net.tensors:
            tn.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype="complex64"))
        got = tn.contract(path).data[0]
    finally:
        jet.set_precision(old)
    otn = jo.OTensorNetwork()
    for lab, sh, d in net.tensors:
        otn.add_tensor(jo.OTensor.make(lab, sh, d, np.complex128))
    want = otn.contract(path).data[0]
    assert abs(got - want) <= 1e-5 * abs(want)
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "ref_cases.json")) as f:
        ref_case = [c for c in json.load(f)["network"] if c["rows"] == 4][0]
    ref_amp = complex(*ref_case["out"][0])
    assert abs(got - ref_amp) <= 1e-5 * abs(ref_amp)


@pytest.mark.parametrize("precision", [0, 2])
def test_repeated_contract_replays_a_graph(jet, precision):
    """Repeated TaskBasedContractor.contract() calls of the same tasks: the
    first runs eagerly, the second captures the contractions into one CUDA
    graph and every later call replays it. Every call's results (two networks
    sharing tasks, their FP64 reduction) equal those of a contractor that
    runs eagerly, bit for bit, with the replay's independent tiny steps in
    grouped launches (the default) and without."""
    from jet_gb300 import circuits

    net = circuits.random_circuit_network(3, 4, 6, seed=31)
    path = circuits.greedy_path(net, seed=31)
    sliced = circuits.choose_slices(net, path, 1)
    old = jet.get_precision()
    jet.set_precision(precision)
    try:
        def build(replay, grouping=True):
            tbc = jet.TaskBasedContractor(dtype="complex64")
            tbc.set_graph_replay(replay)
            tbc.set_grouping(grouping)
            for v in range(2):
                tn = jet.TensorNetwork(dtype="complex64")
                for lab, sh, d in net.tensors:
                    tn.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d),
                                             dtype="complex64"))
                tn.slice_indices(sliced, v)
                tbc.add_contraction_tasks(tn, jet.PathInfo(tn, path))
            tbc.add_deletion_tasks()
            tbc.add_reduction_task()
            return tbc

        eager = build(False)
        eager.contract()
        want = [complex(r.data[0]) for r in eager.results] + [eager.reduction_result.data[0]]
        for grouping in (True, False):
            tbc = build(True, grouping)
            for call in range(4):
                tbc.contract()
                got = [complex(r.data[0]) for r in tbc.results] + [tbc.reduction_result.data[0]]
                assert got == want, (grouping, call)
                assert tbc.has_replay_graph == (call >= 1)
    finally:
        jet.set_precision(old)
