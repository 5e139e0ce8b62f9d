"""Quantum states with the reference's Python state API (python/jet/state.py):
`State` (name, num_wires, indices, tensor(dtype)), `Qudit`, `QuditRegister`
and the qubit shorthands `Qubit`, `QubitRegister`. A state's tensor has one
index per wire and its state vector as data; `tensor()` returns a GPU tensor
of this package."""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import List, Optional, Sequence

import numpy as np

from .factory import Tensor


class State(ABC):
    """A quantum state on `num_wires` wires."""

    def __init__(self, name: str, num_wires: int):
        self.name = name
        self._indices = None
        self._num_wires = num_wires

    @property
    def indices(self) -> Optional[List[str]]:
        return self._indices

    @indices.setter
    def indices(self, indices: Optional[Sequence[str]]) -> None:
        if indices is not None:
            if (not isinstance(indices, Sequence) or not all(isinstance(i, str) for i in indices)
                    or len(set(indices)) != len(indices)):
                raise ValueError("Indices must be a sequence of unique strings.")
            if len(indices) != self.num_wires:
                raise ValueError(
                    f"States must have one index per wire. "
                    f"Received {len(indices)} indices for {self.num_wires} wires.")
        self._indices = indices

    @property
    def num_wires(self) -> int:
        return self._num_wires

    def __eq__(self, other) -> bool:
        return bool(np.all(self._data() == other._data()))

    def __ne__(self, other) -> bool:
        return not self == other

    @abstractmethod
    def _data(self) -> np.ndarray:
        """The state vector."""

    def tensor(self, dtype=np.complex128):
        """The state as a GPU tensor (indices: the set ones, else "0", "1", ...)."""
        data = np.asarray(self._data()).reshape(-1)
        indices = self.indices if self.indices is not None else [
            str(i) for i in range(self.num_wires)]
        dim = int(round(len(data) ** (1.0 / len(indices))))
        return Tensor(indices=list(indices), shape=[dim] * len(indices), data=list(data),
                      dtype=dtype)


class Qudit(State):
    """One qudit of dimension `dim`: |0> unless a state vector is given."""

    def __init__(self, dim: int, data: Optional[np.ndarray] = None):
        super().__init__(name="Qubit" if dim == 2 else f"Qudit(d={dim})", num_wires=1)
        self._vec = (np.arange(dim) == 0).astype(np.complex128) if data is None \
            else np.asarray(data).reshape(-1)

    def _data(self) -> np.ndarray:
        return self._vec


class QuditRegister(State):
    """`size` qudits of dimension `dim`: |0...0> unless a state vector is given."""

    def __init__(self, dim: int, size: int, data: Optional[np.ndarray] = None):
        super().__init__(name=f"Qubit[{size}]" if dim == 2 else f"Qudit(d={dim})[{size}]",
                         num_wires=size)
        self._vec = (np.arange(dim ** size) == 0).astype(np.complex128) if data is None \
            else np.asarray(data).reshape(-1)

    def _data(self) -> np.ndarray:
        return self._vec


def Qubit(data: Optional[np.ndarray] = None) -> Qudit:
    """A qubit (|0> unless a state vector is given)."""
    return Qudit(dim=2, data=data)


def QubitRegister(size: int, data: Optional[np.ndarray] = None) -> QuditRegister:
    """`size` qubits (|0...0> unless a state vector is given)."""
    return QuditRegister(dim=2, size=size, data=data)
