"""Checkpoint / resume of a sliced contraction (jet_gb300.checkpoint).

CPU: a stand-in contractor with known per-slice values. A run stopped by an
exception after some chunks resumes at its cursor, contracts no finished
slice again and returns bit for bit the uninterrupted result; mismatched or
foreign checkpoints are refused; the write is atomic. Two gloo ranks, one of
which fails mid-run, finish from their own checkpoints after a restart.

GPU: the same on a real SlicedContractor (a 4x4 random-circuit network,
4 sliced indices), within 1e-12 of the one-shot slice sum."""
import os
import socket

import numpy as np
import pytest


class FakeSliced:
    """num_slices slices of a 2x3 result; slice v's value is a fixed array."""

    def __init__(self, num_slices=64, batch=4, shape=(2, 3), seed=0):
        self.num_slices, self.batch_size, self.result_shape = num_slices, batch, list(shape)
        rng = np.random.default_rng(seed)
        size = int(np.prod(shape))
        self.values = rng.standard_normal((num_slices, size)) + 1j * rng.standard_normal(
            (num_slices, size))
        self.calls = []

    def contract(self, first=0, count=None):
        if count is None:
            count = self.num_slices - first
        assert count % self.batch_size == 0
        self.calls.append((first, count))
        return list(self.values[first:first + count].sum(axis=0))


class Stop(Exception):
    pass


def _stop_after(n_chunks):
    seen = []

    def cb(done, count):
        seen.append(done)
        if len(seen) == n_chunks:
            raise Stop()

    return cb


def test_resume_continues_at_the_cursor(tmp_path):
    from jet_gb300.checkpoint import contract_resumable, load_checkpoint

    ck = str(tmp_path / "run.ckpt")
    ref = FakeSliced()
    want = contract_resumable(ref, str(tmp_path / "ref.ckpt"), chunk_slices=8)
    assert want.shape == (2, 3)
    assert np.allclose(want.reshape(-1), ref.values.sum(axis=0), rtol=1e-13)

    sc = FakeSliced()
    with pytest.raises(Stop):
        contract_resumable(sc, ck, chunk_slices=8, on_chunk=_stop_after(3))
    meta, done, _ = load_checkpoint(ck)
    assert done == 24 and meta["chunk_slices"] == 8
    assert sc.calls == [(0, 8), (8, 8), (16, 8)]

    sc2 = FakeSliced()
    got = contract_resumable(sc2, ck, chunk_slices=8)
    assert sc2.calls == [(s, 8) for s in range(24, 64, 8)]
    assert np.array_equal(got, want)
    # A finished checkpoint returns its sum without contracting anything.
    sc3 = FakeSliced()
    assert np.array_equal(contract_resumable(sc3, ck, chunk_slices=8), want)
    assert sc3.calls == []
    assert not os.path.exists(ck + ".tmp")


def test_sub_range_and_chunk_rounding(tmp_path):
    from jet_gb300.checkpoint import contract_resumable

    sc = FakeSliced(num_slices=64, batch=4)
    got = contract_resumable(sc, str(tmp_path / "c"), first=16, count=32, chunk_slices=10)
    # 10 rounds down to 8 (a multiple of the batch size).
    assert sc.calls == [(16, 8), (24, 8), (32, 8), (40, 8)]
    assert np.allclose(got.reshape(-1), sc.values[16:48].sum(axis=0), rtol=1e-13)


def test_checkpoint_of_another_run_is_refused(tmp_path):
    from jet_gb300.checkpoint import contract_resumable

    ck = str(tmp_path / "c")
    with pytest.raises(Stop):
        contract_resumable(FakeSliced(), ck, chunk_slices=8, fingerprint="net-A",
                           on_chunk=_stop_after(1))
    for kwargs in [dict(fingerprint="net-B"), dict(fingerprint="net-A", chunk_slices=16),
                   dict(fingerprint="net-A", first=8, count=32)]:
        args = dict(chunk_slices=8)
        args.update(kwargs)
        with pytest.raises(ValueError, match="another run"):
            contract_resumable(FakeSliced(), ck, **args)
    with pytest.raises(ValueError, match="another run"):
        contract_resumable(FakeSliced(batch=8), ck, chunk_slices=8, fingerprint="net-A")
    bad = str(tmp_path / "bad")
    np.savez(open(bad, "wb"), sum=np.zeros(6, np.complex128),
             header=np.frombuffer(b'{"format": "other"}', dtype=np.uint8))
    with pytest.raises(ValueError, match="not a sliced-contraction checkpoint"):
        contract_resumable(FakeSliced(), bad)


def test_range_and_batch_errors(tmp_path):
    from jet_gb300.checkpoint import contract_resumable

    with pytest.raises(ValueError, match="out of bounds"):
        contract_resumable(FakeSliced(), str(tmp_path / "a"), first=60, count=8)
    with pytest.raises(ValueError, match="multiple of the batch size"):
        contract_resumable(FakeSliced(), str(tmp_path / "b"), count=6)


def test_a_failed_write_keeps_the_previous_checkpoint(tmp_path, monkeypatch):
    from jet_gb300 import checkpoint

    ck = str(tmp_path / "c")
    with pytest.raises(Stop):
        checkpoint.contract_resumable(FakeSliced(), ck, chunk_slices=8, on_chunk=_stop_after(2))
    before = open(ck, "rb").read()

    def broken_replace(src, dst):
        raise OSError("disk went away")

    monkeypatch.setattr(checkpoint.os, "replace", broken_replace)
    with pytest.raises(OSError):
        checkpoint.contract_resumable(FakeSliced(), ck, chunk_slices=8)
    monkeypatch.undo()
    assert open(ck, "rb").read() == before
    _, done, _ = checkpoint.load_checkpoint(ck)
    assert done == 16


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, ck, fail_rank, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from jet_gb300.distributed import contract_sharded

    sc = FakeSliced(num_slices=64, batch=4)
    try:
        cb = _stop_after(2) if rank == fail_rank else None
        total = contract_sharded(sc, rank, world, checkpoint=ck, chunk_slices=8, on_chunk=cb)
        out[rank] = ("ok", list(total), sc.calls)
    except Stop:
        out[rank] = ("stopped", None, sc.calls)
    dist.destroy_process_group()


def _single(rank, world, ck, fail_rank, out):
    """A rank that contracts its share with a checkpoint and no collective."""
    from jet_gb300.checkpoint import contract_resumable
    from jet_gb300.distributed import shard_range

    sc = FakeSliced(num_slices=64, batch=4)
    first, count = shard_range(64, 4, rank, world)
    try:
        cb = _stop_after(2) if rank == fail_rank else None
        part = contract_resumable(sc, "%s.rank%d-of-%d" % (ck, rank, world), first, count,
                                  chunk_slices=8, on_chunk=cb)
        out[rank] = ("ok", list(part.reshape(-1)), sc.calls)
    except Stop:
        out[rank] = ("stopped", None, sc.calls)


def test_sharded_restart_after_a_rank_fails(tmp_path):
    """Rank 1 stops after two chunks (before the all-reduce), the job ends; a
    restart of both ranks reduces the same total as an uninterrupted run, and
    rank 1 contracts only the chunks it had not finished."""
    import torch.multiprocessing as mp

    world, ck = 2, str(tmp_path / "job")
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    # First attempt: every rank works on its own checkpoint; rank 1 fails.
    procs = [ctx.Process(target=_single, args=(r, world, ck, 1, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0][0] == "ok" and out[1][0] == "stopped"
    assert out[1][2] == [(32, 8), (40, 8)]
    # Restart: both ranks resume and all-reduce over gloo.
    port = _free_port()
    out2 = mgr.dict()
    procs = [ctx.Process(target=_worker, args=(r, world, port, ck, -1, out2))
             for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    want = FakeSliced(num_slices=64, batch=4).values.sum(axis=0)
    for r in range(world):
        status, total, calls = out2[r]
        assert status == "ok"
        assert np.allclose(np.array(total), want, rtol=1e-12)
    assert out2[0][2] == []  # rank 0 had finished: nothing contracted again
    assert out2[1][2] == [(48, 8), (56, 8)]


@pytest.mark.gpu
def test_resume_on_the_gpu_sliced_contractor(tmp_path, cuda):
    import jet_gb300 as jet
    from jet_gb300 import circuits
    from jet_gb300.checkpoint import contract_resumable

    net = circuits.random_circuit_network(4, 4, 8, seed=21, dtype=np.dtype("complex64"))
    path = circuits.find_path(net, restarts=2, seed=21)
    sliced = circuits.choose_slices(net, path, 4)

    def make():
        tn = jet.TensorNetwork(dtype="complex64")
        for lab, sh, d in net.tensors:
            tn.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype="complex64"))
        sc = jet.SlicedContractorC64(tn, path, sliced, 0)
        sc.set_batch_size(2)
        return sc

    one_shot = np.asarray(make().contract())
    ref = contract_resumable(make(), str(tmp_path / "ref"), chunk_slices=4)
    ck = str(tmp_path / "run")
    with pytest.raises(Stop):
        contract_resumable(make(), ck, chunk_slices=4, on_chunk=_stop_after(2))
    got = contract_resumable(make(), ck, chunk_slices=4)
    assert np.array_equal(got, ref)
    scale = max(abs(one_shot).max(), 1e-30)
    assert abs(got.reshape(-1) - one_shot).max() <= 1e-12 * scale * 16
