"""Slice counts chosen against a device-memory budget.

The reference slices a network by hand: the caller lists the indices to slice
(TensorNetwork::SliceIndices, TensorNetwork.hpp:210-284) and PathInfo reports
each step's memory (PathInfo.hpp:211-239), so the caller can check that the
largest intermediate fits. Here the sliced contractor plans a whole chunk of
slices at once (its arena holds `batch` slices of every live intermediate),
so the budget is checked against the contractor's own plan: bonds are added in
the greedy slicer's order (circuits.choose_slices) until
SlicedContractor.estimate_device_bytes() at the requested batch size fits.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

from . import circuits


def choose_slices_for_memory(net: circuits.Network, path: Sequence[Tuple[int, int]], tn,
                             batch: int, budget_bytes: float, precision: int,
                             min_count: int = 0, max_count: int = 24,
                             dtype: str = "complex64") -> Tuple[List[str], int, int]:
    """(sliced labels, device bytes of one chunk's plan, batch size): the
    fewest bonds, at least `min_count`, that give at least `batch` slices and
    for which a chunk of `batch` slices fits `budget_bytes`. Raises
    ValueError when even `max_count` bonds do not fit."""
    from ._jet_bindings import SlicedContractorC64, SlicedContractorC128

    cls = SlicedContractorC64 if dtype == "complex64" else SlicedContractorC128
    for count in range(min_count, max_count + 1):
        sliced = circuits.choose_slices(net, path, count) if count else []
        sc = cls(tn, path, sliced, precision)
        sc.set_batch_size(batch)
        used = sc.batch_size
        need = sc.estimate_device_bytes()
        del sc
        if used == batch and need <= budget_bytes:
            return sliced, int(need), used
    raise ValueError("no slicing of up to %d bonds fits %.3g bytes at %d slices per batch"
                     % (max_count, budget_bytes, batch))
