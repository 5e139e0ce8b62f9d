"""Quantum circuits with the reference's Python circuit API
(python/jet/circuit.py:18-194): `Circuit(num_wires, dim)` starts every wire in
|0>, `append_gate` / `append_state` connect gates and states by index labels
"<wire>-<depth>", `take_expected_value` closes the circuit into <psi|O|psi>,
and `tensor_network(dtype)` returns the circuit as a network of this
package's GPU tensors, ready for TensorNetwork.contract, a
TaskBasedContractor or the sliced contractor.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Iterator, List, Sequence, Union

import numpy as np

from .factory import TensorNetwork
from .gate import Adjoint, Gate
from .state import Qudit, State


@dataclass(frozen=True)
class Operation:
    """A gate or state applied to the wires `wire_ids`."""

    part: Union[Gate, State]
    wire_ids: Sequence[int]


@dataclass
class Wire:
    """A wire: its position, the number of gates on it and whether a state
    has terminated it."""

    id_: int
    depth: int = 0
    closed: bool = False

    @property
    def index(self) -> str:
        """The wire's current index label."""
        return f"{self.id_}-{self.depth}"


class Circuit:
    """`num_wires` wires of dimension `dim`, each starting in |0>."""

    def __init__(self, num_wires: int, dim: int = 2):
        self._dim = dim
        self._wires: List[Wire] = [Wire(i) for i in range(num_wires)]
        self._ops: List[Operation] = []
        for w in self._wires:
            start = Qudit(dim=dim)
            start.indices = [w.index]
            self._ops.append(Operation(part=start, wire_ids=[w.id_]))

    @property
    def dimension(self) -> int:
        return self._dim

    @property
    def operations(self) -> Iterator[Operation]:
        """The starting qudits (one per wire), then the appended operations."""
        return iter(self._ops)

    @property
    def wires(self) -> Iterator[Wire]:
        return iter(self._wires)

    def append_gate(self, gate: Gate, wire_ids: Sequence[int]) -> None:
        """Applies `gate` to `wire_ids`: its indices become the wires' next
        labels (outputs) followed by their current ones (inputs)."""
        self._validate_wire_ids(wire_ids)
        if len(wire_ids) != gate.num_wires:
            raise ValueError(
                f"Number of wire IDs ({len(wire_ids)}) must match the number of wires "
                f"connected to the gate ({gate.num_wires}).")
        inputs = list(self.indices(wire_ids))
        for i in wire_ids:
            self._wires[i].depth += 1
        gate.indices = list(self.indices(wire_ids)) + inputs
        self._ops.append(Operation(part=gate, wire_ids=wire_ids))

    def append_state(self, state: State, wire_ids: Sequence[int]) -> None:
        """Terminates `wire_ids` with `state`."""
        self._validate_wire_ids(wire_ids)
        if len(wire_ids) != state.num_wires:
            raise ValueError(
                f"Number of wire IDs ({len(wire_ids)}) must match the number of wires "
                f"connected to the state ({state.num_wires}).")
        for i in wire_ids:
            self._wires[i].closed = True
        state.indices = list(self.indices(wire_ids))
        self._ops.append(Operation(part=state, wire_ids=wire_ids))

    def take_expected_value(self, observable: Iterator[Operation]) -> None:
        """Closes the circuit into <psi| O |psi>: the observable's gates, then
        the adjoints of the circuit's gates in reverse order, then |0> states
        (real, so no adjoint) on every wire. Nothing can be appended after."""
        first = len(self._wires)
        last = len(self._ops)
        for op in observable:
            self.append_gate(gate=op.part, wire_ids=op.wire_ids)
        for op in reversed(self._ops[first:last]):
            self.append_gate(gate=Adjoint(gate=op.part), wire_ids=op.wire_ids)
        for op in reversed(self._ops[:first]):
            self.append_state(state=Qudit(dim=self.dimension), wire_ids=op.wire_ids)

    def indices(self, wire_ids: Iterator[int]) -> Iterator[str]:
        """The current index label of each wire in `wire_ids`."""
        return (self._wires[i].index for i in wire_ids)

    def tensor_network(self, dtype=np.complex128):
        """The circuit as a GPU tensor network, one tensor per operation."""
        tn = TensorNetwork(dtype=dtype)
        for op in self._ops:
            tn.add_tensor(op.part.tensor(dtype=dtype))
        return tn

    def _validate_wire_ids(self, wire_ids: Sequence[int]) -> None:
        n = len(self._wires)
        for w in wire_ids:
            if not 0 <= w < n:
                raise ValueError(f"Wire ID {w} falls outside the range [0, {n}).")
            if list(wire_ids).count(w) > 1:
                raise ValueError(f"Wire ID {w} is specified more than once.")
            if self._wires[w].closed:
                raise ValueError(f"Wire {w} is closed.")
