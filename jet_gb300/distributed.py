"""Slices across GPUs: each rank contracts a contiguous, batch-aligned range
of slice values with its own SlicedContractor, then the FP64 partial results
are summed once across ranks. This is the only exchange of the sliced path;
the reference has no distributed backend, and its slices are independent
networks (TaskBasedContractor.hpp:162-248, AddReductionTask :258-280).
"""
from __future__ import annotations

from typing import Optional, Sequence, Tuple

import numpy as np


def shard_range(n_slices: int, batch: int, rank: int, world: int) -> Tuple[int, int]:
    """(first, count) of this rank's slices: chunks of `batch` slices are
    dealt out as evenly as possible, in order, so every count is a multiple
    of the batch size and the ranges tile [0, n_slices)."""
    if n_slices % batch:
        raise ValueError("slice count must be a multiple of the batch size")
    chunks = n_slices // batch
    base, extra = divmod(chunks, world)
    start_chunk = rank * base + min(rank, extra)
    my_chunks = base + (1 if rank < extra else 0)
    return start_chunk * batch, my_chunks * batch


def reduce_partials(partial: Sequence[complex], group=None) -> np.ndarray:
    """Sum of every rank's FP64 partial result (all ranks receive it)."""
    import torch
    import torch.distributed as dist

    arr = np.asarray(partial, dtype=np.complex128)
    t = torch.from_numpy(np.stack([arr.real, arr.imag], axis=-1).reshape(-1).copy())
    if dist.is_initialized() and dist.get_world_size(group) > 1:
        backend = dist.get_backend(group)
        if backend == "nccl":
            t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        t = t.cpu()
    v = t.numpy().reshape(-1, 2)
    return v[:, 0] + 1j * v[:, 1]


def contract_sharded(sliced_contractor, rank: int, world: int, group=None,
                     checkpoint: Optional[str] = None, **checkpoint_args) -> np.ndarray:
    """Contracts this rank's share of the slices and returns the total.

    With `checkpoint`, each rank keeps its own resumable partial sum in
    "<checkpoint>.rank<r>-of-<world>" (jet_gb300.checkpoint.contract_resumable;
    `checkpoint_args` go to it), so a restarted job redoes no finished chunk."""
    first, count = shard_range(sliced_contractor.num_slices, sliced_contractor.batch_size,
                               rank, world)
    if not count:
        part = [0j] * int(np.prod(sliced_contractor.result_shape or [1]))
    elif checkpoint is not None:
        from .checkpoint import contract_resumable

        path = "%s.rank%d-of-%d" % (checkpoint, rank, world)
        part = contract_resumable(sliced_contractor, path, first, count,
                                  **checkpoint_args).reshape(-1)
    else:
        part = sliced_contractor.contract(first, count)
    return reduce_partials(part, group)
