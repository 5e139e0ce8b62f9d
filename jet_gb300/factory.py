"""dtype-dispatching constructors, as in the reference's python/jet/factory.py:
Tensor(...), TensorNetwork(...) and TaskBasedContractor(...) return the C64 or
C128 class of the bindings; complex128 is the default."""
from __future__ import annotations

from typing import Union

import numpy as np

from ._jet_bindings import (
    TaskBasedContractorC64,
    TaskBasedContractorC128,
    TensorC64,
    TensorC128,
    TensorNetworkC64,
    TensorNetworkC128,
)

__all__ = ["TensorType", "TensorNetworkType", "TaskBasedContractorType", "Tensor",
           "TensorNetwork", "TaskBasedContractor"]

TensorType = Union[TensorC64, TensorC128]
TensorNetworkType = Union[TensorNetworkC64, TensorNetworkC128]
TaskBasedContractorType = Union[TaskBasedContractorC64, TaskBasedContractorC128]


def _pick(c64, c128, kwargs):
    dtype = np.dtype(kwargs.pop("dtype", np.complex128))
    if dtype == np.complex64:
        return c64
    if dtype == np.complex128:
        return c128
    raise TypeError(f"Data type '{dtype}' is not supported.")


def Tensor(*args, **kwargs) -> TensorType:
    cls = _pick(TensorC64, TensorC128, kwargs)
    if "data" in kwargs and not isinstance(kwargs["data"], list):
        kwargs["data"] = list(kwargs["data"])
    return cls(*args, **kwargs)


def TensorNetwork(*args, **kwargs) -> TensorNetworkType:
    return _pick(TensorNetworkC64, TensorNetworkC128, kwargs)(*args, **kwargs)


def TaskBasedContractor(*args, **kwargs) -> TaskBasedContractorType:
    return _pick(TaskBasedContractorC64, TaskBasedContractorC128, kwargs)(*args, **kwargs)
