"""Tensor-network JSON files: the serialized strings of the reference's
python/tests/test_tensor_network_io.py, round trips, error messages and the
reference's m10 benchmark file layout (a synthetic file of that schema).
Host-side only: loading builds tensors without device work."""
import json
import re

import pytest

NET = """
{ "tensors": [
    [["A", "Hermitian"], ["i", "j"], [2, 2], [[1.0, 0.0], [0.0, 1.0], [-0.0, -1.0], [1.0, 0.0]]],
    [["B", "Identity", "Real"], ["j", "k"], [2, 2], [[1.0, 0.0], [0.0, 0.0], [0.0, 0.0], [1.0, 0.0]]],
    [["C", "Vector", "Real"], ["k"], [2], [[1.0, 0.0], [0.0, 0.0]]]
]}"""
NET_PATH = NET.replace('{ "tensors"', '{ "path": [[0, 2], [2, 1]], "tensors"')


@pytest.fixture(scope="module")
def jet():
    import jet_gb300

    return jet_gb300


def _tn(jet, dtype):
    A = jet.Tensor(shape=[2, 2], indices=["i", "j"], data=[1, 1j, -1j, 1], dtype=dtype)
    B = jet.Tensor(shape=[2, 2], indices=["j", "k"], data=[1, 0, 0, 1], dtype=dtype)
    C = jet.Tensor(shape=[2], indices=["k"], data=[1, 0], dtype=dtype)
    tn = jet.TensorNetwork(dtype=dtype)
    tn.add_tensor(A, ["A", "Hermitian"])
    tn.add_tensor(B, ["B", "Identity", "Real"])
    tn.add_tensor(C, ["C", "Vector", "Real"])
    return tn


@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
def test_serialize_matches_reference_strings(jet, dtype):
    ser = jet.TensorNetworkSerializer(dtype=dtype)
    tn = _tn(jet, dtype)
    assert ser(tn) == re.sub(r"\s+", "", NET)
    path = jet.PathInfo(tn, [(0, 2), (2, 1)])
    assert ser(tn, path) == re.sub(r"\s+", "", NET_PATH)


@pytest.mark.parametrize("dtype", ["complex64", "complex128"])
def test_deserialize(jet, dtype):
    tnf = jet.TensorNetworkSerializer(dtype=dtype)(NET_PATH)
    nodes = tnf.tensors.nodes
    assert [n.tags for n in nodes] == [["A", "Hermitian"], ["B", "Identity", "Real"],
                                       ["C", "Vector", "Real"]]
    assert nodes[0].tensor.indices == ["i", "j"] and nodes[0].tensor.data == [1, 1j, -1j, 1]
    assert tnf.path.path == [(0, 2), (2, 1)]
    rev = jet.TensorNetworkSerializer(dtype=dtype)(NET, True)
    assert rev.tensors.nodes[0].tensor.indices == ["j", "i"]


def test_errors(jet):
    ser = jet.TensorNetworkSerializer()
    with pytest.raises(jet.TensorFileException, match="root element must be an object."):
        ser("[1, 2]")
    with pytest.raises(jet.TensorFileException, match="root object must contain 'tensors' key"):
        ser('{"path": []}')
    with pytest.raises(jet.TensorFileException, match="Invalid element at index 1 of tensor 0"):
        ser('{"tensors": [[[], ["i"], [2], [[1, 0], ["x", 0]]]]}')


def test_benchmark_file_schema(jet):
    """A file in the layout of the reference's m10.json (rank-3 tensors, tags
    list first, a path over node ids) loads with its path."""
    tensors = [[["ROUND_0", "GATE_%d" % i], ["a%d" % i, "a%d" % (i + 1), "x%d" % i], [2, 2, 2],
                [[1.0, 0.0]] * 8] for i in range(4)]
    js = json.dumps({"path": [[0, 1], [2, 3], [4, 5]], "tensors": tensors})
    tnf = jet.TensorNetworkSerializer(dtype="complex64")(js)
    assert tnf.tensors.num_tensors == 4
    assert len(tnf.path.steps) == 7


@pytest.mark.parametrize("name,tensors,steps", [("m10", 322, 321), ("m12", 410, 409)])
def test_reference_benchmark_networks_load(jet, name, tensors, steps):
    """The reference's m10 / m12 networks (golden npz form) rebuilt as JSON
    text of the reference's schema load through the serializer with their
    stored paths; where the reference tree is present, the npz holds exactly
    the tensors of the reference's own file."""
    import os

    import numpy as np

    import make_network_fixtures as mk

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    ts, path = mk.load_network_npz(os.path.join(here, name + "_network.npz"))
    assert len(ts) == tensors and len(path) == steps
    tnf = jet.TensorNetworkSerializer(dtype="complex64")(mk.network_json_text(ts, path))
    assert tnf.tensors.num_tensors == tensors
    assert tnf.path.path == path
    node = tnf.tensors.nodes[7]
    assert node.tensor.indices == ts[7][1] and node.tags == ts[7][0]
    assert np.allclose(np.array(node.tensor.data, dtype=np.complex64), ts[7][3])
    src = os.path.join(mk.reference_root(), "examples", "paper_benchmarks", "data_files",
                       name + ".json")
    if os.path.exists(src):
        with open(src) as f:
            js = json.load(f)
        assert [tuple(p) for p in js["path"]] == path
        for (tg, lb, sh, d), t in zip(ts, js["tensors"]):
            assert tg == t[0] and lb == t[1] and sh == t[2]
            assert np.array_equal(d, np.array([complex(*x) for x in t[3]], dtype=np.complex64))
