"""Quantum gates with the reference's Python gate API (python/jet/gate.py):
`Gate` (name, num_wires, dimension, params, indices, tensor(dtype)),
`GateFactory` (create / register / unregister by name), the `Adjoint` and
`Scale` decorators and the qubit gates, under the names the reference
registers. `tensor()` returns a GPU tensor of this package, so a circuit's
network (`Circuit.tensor_network`) contracts on the GPU.

The qubit gates are defined here from their standard matrices, one table row
each; the classes are generated from the table. Added beside the reference's
set: SqrtY, SqrtW and FSim (the benchmark circuits' gates). The reference's
continuous-variable Fock gates (Displacement, Squeezing, TwoModeSqueezing,
Beamsplitter) take their matrices from the thewalrus package, which this
build does not have; they are not provided.
"""
from __future__ import annotations

import cmath
import math
from abc import ABC, abstractmethod
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np

from . import circuits
from .factory import Tensor

_R2 = 1.0 / math.sqrt(2.0)


class Gate(ABC):
    """A quantum gate on `num_wires` wires of dimension `dim`.

    Its tensor has two indices per wire, outputs then inputs; its data is the
    gate's matrix, flattened row-major."""

    def __init__(self, name: str, num_wires: int, dim: int, params: Optional[List[float]] = None):
        self.name = name
        self._indices = None
        self._num_wires = num_wires
        self._params = params
        self._validate_dimension(dim)
        self._dim = dim

    @property
    def dimension(self) -> int:
        return self._dim

    @dimension.setter
    def dimension(self, dim: int) -> None:
        self._validate_dimension(dim)
        self._dim = dim

    @abstractmethod
    def _validate_dimension(self, dim: int) -> None:
        """Raises ValueError when `dim` is not a valid dimension."""

    @property
    def indices(self) -> Optional[Sequence[str]]:
        return self._indices

    @indices.setter
    def indices(self, indices: Optional[Sequence[str]]) -> None:
        if indices is not None:
            if (not isinstance(indices, Sequence) or not all(isinstance(i, str) for i in indices)
                    or len(set(indices)) != len(indices)):
                raise ValueError("Indices must be a sequence of unique strings.")
            if len(indices) != 2 * self._num_wires:
                raise ValueError(
                    f"Gates must have two indices per wire; received {len(indices)} "
                    f"indices for {self._num_wires} wires.")
        self._indices = indices

    @property
    def num_wires(self) -> int:
        return self._num_wires

    @property
    def params(self) -> Optional[List[float]]:
        return self._params

    @abstractmethod
    def _data(self) -> np.ndarray:
        """The gate's matrix."""

    def tensor(self, dtype=np.complex128):
        """The gate as a GPU tensor (indices: the set ones, else "0", "1", ...)."""
        data = np.asarray(self._data()).reshape(-1)
        indices = self.indices if self.indices is not None else [
            str(i) for i in range(2 * self._num_wires)]
        dim = int(round(len(data) ** (1.0 / len(indices))))
        return Tensor(indices=list(indices), shape=[dim] * len(indices), data=list(data),
                      dtype=dtype)


class GateFactory:
    """Gates by registered name: create("CNOT"), create("RX", 0.3, adjoint=True)."""

    registry: Dict[str, type] = {}

    @staticmethod
    def create(name: str, *params: float, adjoint: bool = False, scalar: float = 1,
               **kwargs) -> Gate:
        if name not in GateFactory.registry:
            raise KeyError(f"The name '{name}' does not exist in the gate registry.")
        gate = GateFactory.registry[name](*params, **kwargs)
        if adjoint:
            gate = Adjoint(gate=gate)
        if scalar != 1:
            gate = Scale(gate=gate, scalar=scalar)
        return gate

    @staticmethod
    def register(names: Sequence[str]) -> Callable[[type], type]:
        def wrapper(subclass: type) -> type:
            if not issubclass(subclass, Gate):
                raise ValueError(f"The type '{subclass.__name__}' is not a subclass of Gate.")
            taken = set(names) & set(GateFactory.registry)
            if taken:
                raise KeyError(f"The names {taken} already exist in the gate registry.")
            for n in set(names):
                GateFactory.registry[n] = subclass
            return subclass

        return wrapper

    @staticmethod
    def unregister(cls: type) -> None:
        for key in [k for k, v in GateFactory.registry.items() if v == cls]:
            del GateFactory.registry[key]


class Adjoint(Gate):
    """The conjugate transpose of another gate."""

    def __init__(self, gate: Gate):
        self._gate = gate
        super().__init__(name=gate.name, num_wires=gate.num_wires, dim=gate.dimension,
                         params=gate.params)

    def _data(self):
        return np.conj(np.asarray(self._gate._data())).T

    def _validate_dimension(self, dim):
        self._gate._validate_dimension(dim)


class Scale(Gate):
    """Another gate multiplied by a scalar."""

    def __init__(self, gate: Gate, scalar: float):
        self._gate = gate
        self._scalar = scalar
        super().__init__(name=gate.name, num_wires=gate.num_wires, dim=gate.dimension,
                         params=gate.params)

    def _data(self):
        return self._scalar * np.asarray(self._gate._data())

    def _validate_dimension(self, dim):
        self._gate._validate_dimension(dim)


class QubitGate(Gate):
    """A gate on qubits (dimension 2)."""

    def __init__(self, name: str, num_wires: int, params: Optional[List[float]] = None):
        super().__init__(name=name, num_wires=num_wires, dim=2, params=params)

    def _validate_dimension(self, dim):
        if dim != 2:
            raise ValueError("The dimension of a qubit gate must be exactly two.")


# ---------------------------------------------------------------------------
# Standard matrices.
# ---------------------------------------------------------------------------

def _rx(t):
    c, s = math.cos(t / 2), math.sin(t / 2)
    return np.array([[c, -1j * s], [-1j * s, c]])


def _ry(t):
    c, s = math.cos(t / 2), math.sin(t / 2)
    return np.array([[c, -s], [s, c]], dtype=complex)


def _rz(t):
    return np.diag([cmath.exp(-0.5j * t), cmath.exp(0.5j * t)])


def _phase(p):
    return np.diag([1, cmath.exp(1j * p)])


def _u3(t, p, lam):
    c, s = math.cos(t / 2), math.sin(t / 2)
    return np.array([[c, -cmath.exp(1j * lam) * s],
                     [cmath.exp(1j * p) * s, cmath.exp(1j * (p + lam)) * c]])


def _controlled(u, controls=1):
    """Block-diagonal (identity, u) with `controls` leading control qubits."""
    n = u.shape[0] * 2 ** controls
    m = np.eye(n, dtype=complex)
    m[n - u.shape[0]:, n - u.shape[0]:] = u
    return m


def _swap():
    m = np.zeros((4, 4), dtype=complex)
    for a in range(2):
        for b in range(2):
            m[2 * b + a, 2 * a + b] = 1
    return m


def _iswap():
    m = _swap()
    m[1, 2] = m[2, 1] = 1j
    return m


_X = np.array([[0, 1], [1, 0]], dtype=complex)

# (class name, registered names, wires, parameters, matrix of the parameters)
_QUBIT_GATES = [
    ("Hadamard", ["Hadamard", "hadamard", "H", "h"], 1, 0,
     lambda: _R2 * np.array([[1, 1], [1, -1]], dtype=complex)),
    ("PauliX", ["PauliX", "paulix", "X", "x", "NOT", "not"], 1, 0, lambda: _X),
    ("PauliY", ["PauliY", "pauliy", "Y", "y"], 1, 0, lambda: np.array([[0, -1j], [1j, 0]])),
    ("PauliZ", ["PauliZ", "pauliz", "Z", "z"], 1, 0, lambda: np.diag([1, -1]).astype(complex)),
    ("S", ["S", "s"], 1, 0, lambda: np.diag([1, 1j])),
    ("T", ["T", "t"], 1, 0, lambda: _phase(math.pi / 4)),
    ("SX", ["SX", "sx"], 1, 0, lambda: 0.5 * np.array([[1 + 1j, 1 - 1j], [1 - 1j, 1 + 1j]])),
    ("PhaseShift", ["PhaseShift", "phaseshift"], 1, 1, _phase),
    ("CPhaseShift", ["CPhaseShift", "cphaseshift"], 2, 1, lambda p: _controlled(_phase(p))),
    ("CX", ["CX", "cx", "CNOT", "cnot"], 2, 0, lambda: _controlled(_X)),
    ("CY", ["CY", "cy"], 2, 0, lambda: _controlled(np.array([[0, -1j], [1j, 0]]))),
    ("CZ", ["CZ", "cz"], 2, 0, lambda: _controlled(np.diag([1, -1]).astype(complex))),
    ("SWAP", ["SWAP", "swap"], 2, 0, _swap),
    ("ISWAP", ["ISWAP", "iswap"], 2, 0, _iswap),
    ("CSWAP", ["CSWAP", "cswap"], 3, 0, lambda: _controlled(_swap())),
    ("Toffoli", ["Toffoli", "toffoli"], 3, 0, lambda: _controlled(_X, controls=2)),
    ("RX", ["RX", "rx"], 1, 1, _rx),
    ("RY", ["RY", "ry"], 1, 1, _ry),
    ("RZ", ["RZ", "rz"], 1, 1, _rz),
    ("Rot", ["Rot", "rot"], 1, 3, lambda p, t, o: _rz(o) @ _ry(t) @ _rz(p)),
    ("CRX", ["CRX", "crx"], 2, 1, lambda t: _controlled(_rx(t))),
    ("CRY", ["CRY", "cry"], 2, 1, lambda t: _controlled(_ry(t))),
    ("CRZ", ["CRZ", "crz"], 2, 1, lambda t: _controlled(_rz(t))),
    ("CRot", ["CRot", "crot"], 2, 3, lambda p, t, o: _controlled(_rz(o) @ _ry(t) @ _rz(p))),
    ("U1", ["U1", "u1"], 1, 1, _phase),
    ("U2", ["U2", "u2"], 1, 2, lambda p, lam: _u3(math.pi / 2, p, lam)),
    ("U3", ["U3", "u3"], 1, 3, _u3),
    # Added: the gates of the benchmark circuits.
    ("SqrtY", ["SqrtY", "sqrty"], 1, 0, circuits.gate_sqrt_y),
    ("SqrtW", ["SqrtW", "sqrtw"], 1, 0, circuits.gate_sqrt_w),
    ("FSim", ["FSim", "fsim"], 2, 2, circuits.gate_fsim),
]


def _make_gate_class(cls_name, names, n_wires, n_params, matrix):
    def __init__(self, *params):
        if len(params) != n_params:
            raise TypeError(f"{cls_name} takes {n_params} parameters ({len(params)} given)")
        QubitGate.__init__(self, name=cls_name, num_wires=n_wires,
                           params=list(params) if n_params else None)

    def _data(self):
        return np.asarray(matrix(*(self.params or [])), dtype=complex)

    cls = type(cls_name, (QubitGate,), {"__init__": __init__, "_data": _data,
                                        "__doc__": f"{cls_name} ({n_wires}-qubit gate, "
                                                   f"{n_params} parameters)."})
    return GateFactory.register(names)(cls)


for _row in _QUBIT_GATES:
    globals()[_row[0]] = _make_gate_class(*_row)

__all__ = ["Gate", "GateFactory", "Adjoint", "Scale", "QubitGate"] + [r[0] for r in _QUBIT_GATES]
