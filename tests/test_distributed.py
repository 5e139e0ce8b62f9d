"""Host logic of the multi-GPU path on CPU ranks (gloo, world size 2): slice
ranges tile the slice space in batch-aligned pieces, and the FP64 partial
sums combine exactly. No GPU is involved."""
import os
import socket

import numpy as np
import pytest


def test_shard_ranges_tile_the_slices():
    from jet_gb300.distributed import shard_range

    for n, b, w in [(4096, 64, 2), (4096, 2, 8), (64, 16, 3), (16, 16, 4), (1, 1, 2)]:
        covered = []
        for r in range(w):
            first, count = shard_range(n, b, r, w)
            assert count % b == 0
            covered.extend(range(first, first + count))
        assert covered == list(range(n))
    with pytest.raises(ValueError):
        shard_range(10, 4, 0, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from jet_gb300.distributed import reduce_partials, shard_range

    # Stand-in per-slice values: rank r sums its own range in FP64.
    vals = np.exp(1j * np.arange(256)) * (1.0 + np.arange(256)) * 1e-3
    first, count = shard_range(256, 16, rank, world)
    part = [vals[first:first + count].sum()]
    total = reduce_partials(part)
    out[rank] = (complex(total[0]), complex(vals.sum()))
    dist.destroy_process_group()


def test_partial_sums_all_reduce_gloo():
    import torch.multiprocessing as mp

    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        got, want = out[r]
        assert abs(got - want) <= 1e-12 * abs(want)
