"""Checkpoint / resume of a sliced contraction.

A sliced network's result is a sum over independent slices. A long run keeps
that sum as it goes: the slices are contracted in chunks (a multiple of the
contractor's batch size), and after every chunk the FP64 running sum and the
slice cursor (slices done so far) are written to a checkpoint file. A run
that stops -- an exception, a lost process, a job time limit -- is resumed by
calling the same function with the same checkpoint path: it reloads the sum
and continues at the cursor, so no finished slice is contracted again.

The reference has no checkpointing; its sliced runs (examples/
jet_sliced_subset.cpp) contract every slice in one go and sum the results
(TaskBasedContractor::AddReductionTask, TaskBasedContractor.hpp:258-280).
The summation order here is fixed by the chunking: a resumed run returns
bit for bit what an uninterrupted run with the same chunk size returns.

The file is an .npz holding the sum (complex128) and a JSON header (the
slice range, batch size, chunk size, result shape and an optional caller
fingerprint). It is written to a temporary name, flushed and renamed over
the old one, so a run killed mid-write leaves the previous checkpoint intact.
A checkpoint whose header does not match the requested run raises ValueError
instead of being overwritten.
"""
from __future__ import annotations

import json
import os
from typing import Callable, Optional

import numpy as np

FORMAT_VERSION = 1


def _header(num_slices, batch, first, count, chunk, shape, fingerprint):
    return {
        "format": "jet_gb300.sliced_checkpoint",
        "version": FORMAT_VERSION,
        "num_slices": int(num_slices),
        "batch_size": int(batch),
        "first": int(first),
        "count": int(count),
        "chunk_slices": int(chunk),
        "result_shape": [int(d) for d in shape],
        "fingerprint": fingerprint,
    }


def save_checkpoint(path: str, header: dict, done: int, total: np.ndarray) -> None:
    """Atomically writes the running sum and the cursor to `path`."""
    meta = dict(header, done=int(done))
    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        np.savez(f, sum=np.asarray(total, dtype=np.complex128),
                 header=np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8))
        f.flush()
        os.fsync(f.fileno())
    os.replace(tmp, path)


def load_checkpoint(path: str):
    """(header, done, running sum) of a checkpoint file."""
    with np.load(path) as z:
        meta = json.loads(bytes(z["header"]).decode())
        total = np.array(z["sum"], dtype=np.complex128)
    if meta.get("format") != "jet_gb300.sliced_checkpoint":
        raise ValueError("%s is not a sliced-contraction checkpoint" % path)
    if meta.get("version") != FORMAT_VERSION:
        raise ValueError("checkpoint format version %r is not supported" % meta.get("version"))
    done = int(meta.pop("done"))
    return meta, done, total


def contract_resumable(sliced_contractor, checkpoint: str, first: int = 0,
                       count: Optional[int] = None, chunk_slices: Optional[int] = None,
                       fingerprint: Optional[str] = None,
                       on_chunk: Optional[Callable[[int, int], None]] = None) -> np.ndarray:
    """Sum over slices [first, first + count) of `sliced_contractor` (a
    SlicedContractor, or any object with num_slices, batch_size, result_shape
    and contract(first, count)), checkpointed to `checkpoint` after every
    chunk and resumed from it when it exists.

    chunk_slices: slices per checkpoint, rounded down to a multiple of the
    batch size (default: 16 batches). `fingerprint` is stored and must match
    on resume (e.g. a hash of the network and path). `on_chunk(done, count)`
    runs after each checkpoint is written. Returns the FP64 sum, shaped as
    the contractor's result; the checkpoint file is left in place, complete.
    """
    sc = sliced_contractor
    n, batch = int(sc.num_slices), int(sc.batch_size)
    if count is None:
        count = n - first
    if first < 0 or count < 0 or first + count > n:
        raise ValueError("slice range [%d, %d) is out of bounds (%d slices)"
                         % (first, first + count, n))
    if count % batch:
        raise ValueError("slice count must be a multiple of the batch size")
    if chunk_slices is None:
        chunk_slices = 16 * batch
    chunk = max(batch, int(chunk_slices) // batch * batch)
    shape = list(sc.result_shape)
    header = _header(n, batch, first, count, chunk, shape, fingerprint)
    size = int(np.prod(shape)) if shape else 1

    if os.path.exists(checkpoint):
        meta, done, total = load_checkpoint(checkpoint)
        if meta != header:
            diff = sorted(k for k in set(meta) | set(header) if meta.get(k) != header.get(k))
            raise ValueError("checkpoint %s belongs to another run (differs in %s)"
                             % (checkpoint, ", ".join(diff)))
        if total.size != size or not 0 <= done <= count or done % batch:
            raise ValueError("checkpoint %s is inconsistent" % checkpoint)
    else:
        done, total = 0, np.zeros(size, dtype=np.complex128)
        save_checkpoint(checkpoint, header, done, total)

    while done < count:
        step = min(chunk, count - done)
        part = np.asarray(sc.contract(first + done, step), dtype=np.complex128).reshape(-1)
        total = total + part
        done += step
        save_checkpoint(checkpoint, header, done, total)
        if on_chunk is not None:
            on_chunk(done, count)
    return total.reshape(shape) if shape else total
