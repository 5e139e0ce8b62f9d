"""Jet::SlicedContractor on the GPU: every slice of a sliced network along one
path, in batched launches replayed from one CUDA graph, summed in FP64.

Parity: the slice sum equals the unsliced network's value from the complex128
oracle (TensorNetwork::Contract restated), within 1e-5 relative (complex64)
or 1e-12 (complex128); bitstring alternatives give each bitstring's own
amplitude; the reference's own sliced result (golden) matches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def jet(cuda):
    import jet_gb300

    return jet_gb300


def _oracle(net, path):
    from oracle import jet_oracle as jo

    tn = jo.OTensorNetwork()
    for lab, sh, d in net.tensors:
        tn.add_tensor(jo.OTensor.make(lab, sh, d, np.complex128))
    return tn.contract(path)


def _tn(jet, net, dtype):
    tn = jet.TensorNetwork(dtype=dtype)
    for lab, sh, d in net.tensors:
        tn.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype=dtype))
    return tn


def _oracle_slice(net, path, sliced, value):
    from oracle import jet_oracle as jo

    tn = jo.OTensorNetwork()
    for lab, sh, d in net.tensors:
        tn.add_tensor(jo.OTensor.make(lab, sh, d, np.complex128))
    tn.slice_indices(sliced, value)
    return tn.contract(path).data[0]


@pytest.mark.parametrize("dtype,precision", [("complex64", 0), ("complex64", 2),
                                             ("complex128", 0)])
@pytest.mark.parametrize("batch", [1, 4, 16])
def test_sliced_amplitude_matches_unsliced(jet, dtype, precision, batch):
    """Each slice equals the oracle's SliceIndices + Contract value (1e-5
    relative in complex64); the slice sum equals the unsliced amplitude within
    1e-5 of the summed magnitudes sum_v |slice_v| (the slices cancel, so the
    sum is smaller than its terms); partial ranges add up."""
    from jet_gb300 import circuits

    net = circuits.random_circuit_network(4, 4, 8, seed=21, dtype=np.dtype(dtype))
    path = circuits.find_path(net, restarts=2, seed=21)
    sliced = circuits.choose_slices(net, path, 4)
    want = _oracle(net, path).data[0]
    per_slice = [_oracle_slice(net, path, sliced, v) for v in range(16)]
    scale = sum(abs(x) for x in per_slice)
    cls = jet.SlicedContractorC64 if dtype == "complex64" else jet.SlicedContractorC128
    sc = cls(_tn(jet, net, dtype), path, sliced, precision)
    sc.set_batch_size(batch)
    assert sc.num_slices == 16 and sc.batch_size == batch
    tol = 1e-5 if dtype == "complex64" else 1e-12
    got = sc.contract()
    assert sc.result_indices == [] and len(got) == 1
    assert abs(got[0] - want) <= tol * scale
    if batch == 1:
        for v in range(16):
            one = sc.contract(v, 1)[0]
            assert abs(one - per_slice[v]) <= tol * max(abs(per_slice[v]), 1e-3 * scale), v
    half = 8 if batch <= 8 else 16
    if half < 16:
        a = sc.contract(0, half)[0]
        b = sc.contract(half, 16 - half)[0]
        assert abs(a - sum(per_slice[:half])) <= tol * scale
        assert abs(a + b - want) <= tol * scale
    # Contracting again reuses the captured graph and gives the same value.
    assert abs(sc.contract()[0] - got[0]) <= tol * scale


def test_reference_sliced_network_golden(jet, golden):
    """The 3x3 network sliced over 2 bonds at one slice value: the compiled
    reference's TensorNetwork::SliceIndices + Contract result."""
    from jet_gb300 import circuits

    case = [c for c in golden["ref"]["network"] if c["rows"] == 3 and c["cols"] == 3][0]
    net = circuits.random_circuit_network(3, 3, 4, seed=case["seed"])
    path = circuits.greedy_path(net, seed=case["seed"])
    sliced = case["sliced"]
    sc = jet.SlicedContractorC64(_tn(jet, net, "complex64"), path, sliced, 0)
    sc.set_batch_size(1)
    got = sc.contract(case["slice_value"], 1)[0]
    want = complex(*case["out"][0])
    assert abs(got - want) <= 1e-5 * abs(want)


@pytest.mark.parametrize("precision", [0, 2])
def test_bitstring_alternatives_share_prefix(jet, precision):
    """Output caps of 8 seeded bitstrings as alternatives of the cap leaves:
    one run yields every bitstring's amplitude (sliced over 3 bonds)."""
    from jet_gb300 import circuits

    rows, cols, cyc = 3, 4, 6
    n = rows * cols
    rng = np.random.default_rng(5)
    bits = rng.integers(0, 2, size=(8, n))
    net0 = circuits.random_circuit_network(rows, cols, cyc, seed=9)
    path = circuits.find_path(net0, restarts=2, seed=9)
    sliced = circuits.choose_slices(net0, path, 3)
    tn = _tn(jet, net0, "complex64")
    sc = jet.SlicedContractorC64(tn, path, sliced, precision)
    sc.set_batch_size(4)
    cap_ids = list(range(len(net0.tensors) - n, len(net0.tensors)))
    for q, node in enumerate(cap_ids):
        vals = []
        for b in bits:
            vals += [1, 0] if b[q] == 0 else [0, 1]
        sc.set_leaf_alternatives(node, vals, len(bits))
    got = sc.contract()
    assert sc.result_indices == ["$b"] and len(got) == len(bits)
    for i, b in enumerate(bits):
        net_b = circuits.random_circuit_network(rows, cols, cyc, seed=9, bitstring=b)
        want = _oracle(net_b, path).data[0]
        assert abs(got[i] - want) <= 1e-5 * abs(want), i


def test_open_result_indices(jet):
    """A network with open output wires (no output caps on 3 qubits): the
    sliced sum is a tensor over the open labels."""
    from jet_gb300 import circuits
    from oracle import jet_oracle as jo

    net = circuits.random_circuit_network(3, 3, 4, seed=2)
    open_caps = net.tensors[-3:]
    net.tensors = net.tensors[:-3]
    net.open_labels = [t[0][0] for t in open_caps]
    path = circuits.find_path(net, restarts=2, seed=2)
    sliced = circuits.choose_slices(net, path, 2)
    want = _oracle(net, path)
    sc = jet.SlicedContractorC64(_tn(jet, net, "complex64"), path, sliced, 0)
    sc.set_batch_size(2)
    got = np.array(sc.contract())
    labels = sc.result_indices
    assert sorted(labels) == sorted(want.indices)
    wt = jo.transpose(want, labels).data
    assert np.linalg.norm(got - wt) <= 1e-5 * np.linalg.norm(wt)


def _steps_mnk(net, path):
    """(m, n, k) of every pairwise step of `path` (ContractTensors label algebra)."""
    nodes = [(list(lab), list(sh)) for lab, sh, _ in net.tensors]
    out = []
    for a, b in path:
        (la, sa), (lb, sb) = nodes[a], nodes[b]
        ad, bd = dict(zip(la, sa)), dict(zip(lb, sb))
        left = [x for x in la if x not in lb]
        right = [x for x in lb if x not in la]
        common = [x for x in la if x in lb]
        m = int(np.prod([ad[x] for x in left])) if left else 1
        n = int(np.prod([bd[x] for x in right])) if right else 1
        k = int(np.prod([ad[x] for x in common])) if common else 1
        out.append((m, n, k))
        nodes.append((left + right, [ad[x] for x in left] + [bd[x] for x in right]))
    return out


@pytest.mark.parametrize("precision", [0, 2])
def test_network_amplitude_within_1e5_of_fp64(jet, precision):
    """A 30-qubit, 10-cycle circuit amplitude (2^34 flops, tensor-core steps
    under AUTO) sliced over 2 bonds: the complex64 result is within 1e-5 of
    the complex128 FP64 result of the same path. The tensor core's own
    accumulation rounds toward zero, and its bias compounds along a network;
    this bounds it at the amplitude."""
    from jet_gb300 import circuits

    net = circuits.random_circuit_network(5, 6, 10, seed=3)
    best = None
    for s in range(4):
        p = circuits.greedy_path(net, seed=s, score="gain")
        f, _ = circuits.path_cost(net, p)
        if best is None or f < best[0]:
            best = (f, p)
    path = best[1]
    tc_steps = [s for s in _steps_mnk(net, path) if s[0] >= 128 and s[1] >= 64 and s[2] >= 32]
    assert len(tc_steps) >= 2
    sliced = circuits.choose_slices(net, path, 2)
    ref = jet.SlicedContractorC128(_tn(jet, net, "complex128"), path, sliced, 0)
    ref.set_batch_size(2)
    want = ref.contract()[0]
    del ref
    sc = jet.SlicedContractorC64(_tn(jet, net, "complex64"), path, sliced, precision)
    sc.set_batch_size(2)
    got = sc.contract()[0]
    assert abs(got - want) <= 1e-5 * abs(want), abs(got - want) / abs(want)


def test_profile_chunk_times_every_launch(jet):
    """profile_chunk: one entry per slice gather, path step, result reorder
    and the slice sum of a chunk, each with a device time; the chunk's sum is
    left in the accumulator and later contractions are unaffected."""
    from jet_gb300 import circuits

    net = circuits.random_circuit_network(4, 4, 8, seed=21, dtype=np.dtype("complex64"))
    path = circuits.find_path(net, restarts=2, seed=21)
    sliced = circuits.choose_slices(net, path, 4)
    sc = jet.SlicedContractorC64(_tn(jet, net, "complex64"), path, sliced, 2)
    sc.set_batch_size(4)
    want = sc.contract()[0]
    prof = sc.profile_chunk(4)
    kinds = [e["kind"] for e in prof]
    assert kinds.count("slice sum") == 1 and kinds[-1] == "slice sum"
    assert kinds.count("gather") >= 1 and kinds.count("contract") + kinds.count("group") >= 1
    assert set(kinds) <= {"gather", "contract", "group", "result reorder", "slice sum"}
    assert all(e["ms"] >= 0 for e in prof)
    steps = [e["step"] for e in prof if e["kind"] in ("contract", "group")]
    assert steps == sorted(steps) and len(set(steps)) == len(steps)
    assert all(0 <= s < len(path) for s in steps)
    with pytest.raises(Exception, match="multiple of the batch size"):
        sc.profile_chunk(2)
    assert sc.contract()[0] == want


@pytest.mark.parametrize("precision", [2, 4])
def test_exponent_hints_do_not_change_the_amplitude(jet, precision):
    """Passing recorded exponents between the steps (default) skips scans but
    gives the same bits as scanning every FP16x3 operand."""
    from jet_gb300 import circuits

    net = circuits.random_circuit_network(5, 6, 10, seed=3)
    best = None
    for s in range(4):
        p = circuits.greedy_path(net, seed=s, score="gain")
        f, _ = circuits.path_cost(net, p)
        if best is None or f < best[0]:
            best = (f, p)
    path = best[1]
    sliced = circuits.choose_slices(net, path, 2)
    sc = jet.SlicedContractorC64(_tn(jet, net, "complex64"), path, sliced, precision)
    sc.set_batch_size(2)
    with_hints = sc.contract()
    sc.set_exponent_hints(False)
    scanned = sc.contract()
    assert with_hints == scanned
