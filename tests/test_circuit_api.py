"""The circuit front-end (jet_gb300.circuit / gate / state), which mirrors
the reference's python/jet/circuit.py, gate.py and state.py API.

CPU: wire labels, operations, validation messages, the gate registry's
names, gate matrices (unitarity, known values, adjoint and scale), the
tensor network's structure. GPU (marked): amplitudes and an expectation value
of circuits built through the API, contracted on the GPU, against a numpy
state-vector simulation in complex128."""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def jet():
    import jet_gb300

    return jet_gb300


REFERENCE_NAMES = [
    "Hadamard", "hadamard", "H", "h", "PauliX", "paulix", "X", "x", "NOT", "not", "PauliY",
    "pauliy", "Y", "y", "PauliZ", "pauliz", "Z", "z", "S", "s", "T", "t", "SX", "sx",
    "PhaseShift", "phaseshift", "CPhaseShift", "cphaseshift", "CX", "cx", "CNOT", "cnot", "CY",
    "cy", "CZ", "cz", "SWAP", "swap", "ISWAP", "iswap", "CSWAP", "cswap", "Toffoli", "toffoli",
    "RX", "rx", "RY", "ry", "RZ", "rz", "Rot", "rot", "CRX", "crx", "CRY", "cry", "CRZ", "crz",
    "CRot", "crot", "U1", "u1", "U2", "u2", "U3", "u3"]


def test_wire_index(jet):
    assert jet.Wire(id_=1, depth=2).index == "1-2"


def test_constructor_and_validation(jet):
    c = jet.Circuit(num_wires=4, dim=2)
    assert list(c.wires) == [jet.Wire(i, 0, False) for i in range(4)]
    assert list(c.operations) == [jet.Operation(jet.Qubit(), [i]) for i in range(4)]
    with pytest.raises(ValueError, match=r"Wire ID 4 falls outside the range \[0, 4\)."):
        c._validate_wire_ids(wire_ids=[4])
    with pytest.raises(ValueError, match="Wire ID 0 is specified more than once."):
        c._validate_wire_ids(wire_ids=[0, 0])
    c._wires[0].closed = True
    with pytest.raises(ValueError, match="Wire 0 is closed."):
        c._validate_wire_ids(wire_ids=[0])


def test_append_gates_and_states(jet):
    c = jet.Circuit(num_wires=4)
    h = jet.GateFactory.create("H")
    with pytest.raises(ValueError, match=r"Number of wire IDs \(2\) must match the number of "
                                         r"wires connected to the gate \(1\)."):
        c.append_gate(h, wire_ids=[0, 1])
    c.append_gate(h, wire_ids=[3])
    assert h.indices == ["3-1", "3-0"]
    cx = jet.GateFactory.create("CNOT")
    c.append_gate(cx, wire_ids=[2, 3])
    assert cx.indices == ["2-1", "3-2", "2-0", "3-1"]
    st = jet.QubitRegister(size=2)
    c.append_state(st, wire_ids=[0, 1])
    assert st.indices == ["0-0", "1-0"]
    assert [w.closed for w in c.wires] == [True, True, False, False]
    assert list(c.indices([2, 3])) == ["2-1", "3-2"]
    with pytest.raises(ValueError, match="States must have one index per wire"):
        jet.Qubit().indices = ["a", "b"]
    with pytest.raises(ValueError, match="Gates must have two indices per wire"):
        jet.GateFactory.create("X").indices = ["a"]


def test_registry_has_the_reference_names(jet):
    for name in REFERENCE_NAMES:
        assert name in jet.GateFactory.registry, name
    with pytest.raises(KeyError, match="does not exist in the gate registry"):
        jet.GateFactory.create("Nope")
    with pytest.raises(KeyError, match="already exist in the gate registry"):
        jet.GateFactory.register(["H"])(jet.PauliX)


def _params(cls):
    return {"PhaseShift": 1, "CPhaseShift": 1, "RX": 1, "RY": 1, "RZ": 1, "Rot": 3, "CRX": 1,
            "CRY": 1, "CRZ": 1, "CRot": 3, "U1": 1, "U2": 2, "U3": 3, "FSim": 2}.get(cls, 0)


def test_gate_matrices(jet):
    rng = np.random.default_rng(1)
    for name in set(type(g).__name__ for g in
                    (jet.GateFactory.registry[n]
                     (*rng.uniform(0, 2 * math.pi, _params(jet.GateFactory.registry[n].__name__)))
                     for n in jet.GateFactory.registry)):
        cls = getattr(jet, name)
        g = cls(*rng.uniform(0, 2 * math.pi, _params(name)))
        m = g._data()
        assert m.shape == (2 ** g.num_wires, 2 ** g.num_wires)
        assert np.allclose(m.conj().T @ m, np.eye(m.shape[0])), name
        adj = jet.Adjoint(g)._data()
        assert np.allclose(adj, m.conj().T)
        assert np.allclose(jet.Scale(g, 2.5)._data(), 2.5 * m)
    assert np.allclose(jet.RX(math.pi)._data(), -1j * jet.PauliX()._data())
    assert np.allclose(jet.CNOT()._data() if hasattr(jet, "CNOT") else jet.CX()._data(),
                       [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]])
    assert np.allclose(jet.U3(0.3, 0.0, 0.0)._data(), jet.RY(0.3)._data())
    assert np.allclose(jet.Toffoli()._data()[6:, 6:], [[0, 1], [1, 0]])
    g = jet.GateFactory.create("RZ", 0.7, adjoint=True, scalar=2)
    assert np.allclose(g._data(), 2 * jet.RZ(-0.7)._data())


def test_take_expected_value_structure(jet):
    c = jet.Circuit(num_wires=2)
    c.append_gate(jet.GateFactory.create("H"), [0])
    c.append_gate(jet.GateFactory.create("CNOT"), [0, 1])
    c.take_expected_value([jet.Operation(jet.GateFactory.create("Z"), [0])])
    ops = list(c.operations)
    assert len(ops) == 2 + 2 + 1 + 2 + 2
    assert all(w.closed for w in c.wires)
    tn = c.tensor_network(dtype="complex64")
    assert tn.num_tensors == len(ops)


def _statevector(n, ops):
    """numpy simulation: apply each (matrix, wires) to |0...0>."""
    psi = np.zeros([2] * n, dtype=np.complex128)
    psi[(0,) * n] = 1
    for m, wires in ops:
        k = len(wires)
        t = m.reshape([2] * (2 * k))
        psi = np.tensordot(t, psi, axes=(list(range(k, 2 * k)), wires))
        psi = np.moveaxis(psi, list(range(k)), wires)
    return psi


def _random_circuit(jet, n, depth, seed):
    rng = np.random.default_rng(seed)
    names = ["H", "X", "Y", "Z", "S", "T", "SX", "RX", "RY", "RZ", "Rot", "U2", "U3", "CNOT",
             "CY", "CZ", "SWAP", "ISWAP", "CRX", "CRot", "CPhaseShift", "Toffoli", "CSWAP",
             "SqrtY", "SqrtW", "FSim"]
    c = jet.Circuit(num_wires=n)
    sim = []
    for _ in range(depth):
        name = names[int(rng.integers(len(names)))]
        cls = jet.GateFactory.registry[name]
        g = jet.GateFactory.create(name, *rng.uniform(0, 2 * math.pi, _params(cls.__name__)))
        wires = [int(w) for w in rng.permutation(n)[:g.num_wires]]
        c.append_gate(g, wires)
        sim.append((g._data(), wires))
    return c, sim


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,tol", [("complex128", 1e-12), ("complex64", 1e-5)])
def test_circuit_amplitudes_on_gpu(cuda, jet, dtype, tol):
    n = 5
    c, sim = _random_circuit(jet, n, 40, 3)
    psi = _statevector(n, sim)
    bits = [1, 0, 1, 1, 0]
    for w, b in enumerate(bits):
        c.append_state(jet.Qubit(np.array([0, 1] if b else [1, 0])), [w])
    got = complex(c.tensor_network(dtype=dtype).contract().data[0])
    want = psi[tuple(bits)]
    assert abs(got - want) <= tol * max(abs(want), 1e-3)


@pytest.mark.gpu
def test_expected_value_on_gpu(cuda, jet):
    n = 4
    c, sim = _random_circuit(jet, n, 25, 4)
    psi = _statevector(n, sim)
    z = np.diag([1.0, -1.0])
    zz = np.tensordot(np.tensordot(psi, z, axes=([0], [1])), z, axes=([0], [1]))
    want = np.vdot(psi.reshape(-1), np.moveaxis(zz, [n - 2, n - 1], [0, 1]).reshape(-1))
    c.take_expected_value([jet.Operation(jet.GateFactory.create("Z"), [0]),
                           jet.Operation(jet.GateFactory.create("Z"), [1])])
    got = complex(c.tensor_network(dtype="complex128").contract().data[0])
    assert abs(got - want) <= 1e-12
