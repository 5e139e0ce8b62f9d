"""Grouped launch of small contractions (jetgpu_contract_group): every task
of a group, each with its own shapes, axis order and batch placement read
through offset tables, matches the complex128 product of the same views
(1e-5 relative in complex64, 1e-12 in complex128); the sliced contractor's
grouped tiny steps give the amplitude of one launch per step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _task(rng, cuda, dtype, batch, m, n, k, shared_b=False):
    """Operands as random tensors whose axes (batch, rows, k / k, columns, as
    powers of two and odd extents) sit in a random order."""
    import torch

    from jet_gb300 import capi

    def tensor(groups):
        # groups: list of extents per view group; split each into 1-2 axes.
        axes, owner = [], []
        for gi, ext in enumerate(groups):
            parts = [ext] if ext < 4 or ext % 2 else [ext // 2, 2]
            for p in parts:
                axes.append(p)
                owner.append(gi)
        order = rng.permutation(len(axes))
        shape = [axes[i] for i in order]
        pos = {int(i): j for j, i in enumerate(order)}  # original axis -> layout position
        view = [[pos[i] for i in range(len(axes)) if owner[i] == gi] for gi in range(len(groups))]
        size = int(np.prod(shape))
        host = (rng.standard_normal(size) + 1j * rng.standard_normal(size)).astype(dtype)
        return host, shape, view

    ha, sa, va = tensor([batch, m, k])
    hb, sb, vb = tensor([1 if shared_b else batch, k, n])
    A = torch.from_numpy(ha).to(cuda)
    B = torch.from_numpy(hb).to(cuda)
    C = torch.empty(batch * m * n, dtype=A.dtype, device=cuda)
    tab = {}
    for name, shape, view in (("a", sa, va), ("b", sb, vb)):
        for slot, axes in zip(("bat", "row", "col"), view):
            tab[name + "_" + slot] = torch.from_numpy(capi.view_offsets(shape, axes)).to(cuda)
    if shared_b:
        tab["b_bat"] = torch.zeros(batch, dtype=torch.int64, device=cuda)
    # The complex128 reference of the same views.
    def mats(host, shape, view, lead):
        t = host.astype(np.complex128).reshape(shape)
        t = np.transpose(t, view[0] + view[1] + view[2])
        return t.reshape(lead, int(np.prod([shape[i] for i in view[1]] or [1])),
                         int(np.prod([shape[i] for i in view[2]] or [1])))
    am = mats(ha, sa, va, batch)
    bm = mats(hb, sb, vb, 1 if shared_b else batch)
    want = am @ bm
    task = dict(A=A, B=B, C=C, batch=batch, m=m, n=n, k=k, **tab)
    return task, want


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_group_matches_each_product(cuda, dtype):
    import torch

    from jet_gb300 import capi

    rng = np.random.default_rng(11 if dtype == np.complex64 else 12)
    shapes = [(1, 5, 7, 9, False), (4, 16, 8, 32, False), (3, 33, 1, 70, True),
              (2, 1, 40, 24, False), (1, 64, 64, 3, True), (8, 12, 10, 1, False),
              (5, 2, 2, 200, False)]
    tasks, wants = [], []
    for b, m, n, k, shared in shapes:
        t, w = _task(rng, cuda, dtype, b, m, n, k, shared)
        tasks.append(t)
        wants.append(w)
    keep = capi.contract_group(tasks)
    torch.cuda.synchronize()
    tol = 1e-5 if dtype == np.complex64 else 1e-12
    for t, w in zip(tasks, wants):
        got = t["C"].cpu().numpy().reshape(w.shape)
        assert np.linalg.norm(got - w) <= tol * max(np.linalg.norm(w), 1e-300)
    del keep


def test_group_rejects_too_many_tasks(cuda):
    from jet_gb300 import capi

    rc = capi.lib.jetgpu_contract_group(None, 257, 1, capi.C64, None)
    assert rc == capi.ERR_INVALID


@pytest.mark.parametrize("precision", [0, 2, 5])
def test_sliced_grouping_keeps_the_amplitude(cuda, precision):
    import jet_gb300 as jet
    from jet_gb300 import circuits

    net = circuits.random_circuit_network(5, 6, 10, seed=3)
    best = None
    for s in range(4):
        p = circuits.greedy_path(net, seed=s, score="gain")
        f, _ = circuits.path_cost(net, p)
        if best is None or f < best[0]:
            best = (f, p)
    path = best[1]
    sliced = circuits.choose_slices(net, path, 3)

    def tn(dtype):
        t = jet.TensorNetwork(dtype=dtype)
        for lab, sh, d in net.tensors:
            t.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype=dtype))
        return t

    ref = jet.SlicedContractorC128(tn("complex128"), path, sliced, 0).contract()[0]
    sc = jet.SlicedContractorC64(tn("complex64"), path, sliced, precision)
    sc.set_batch_size(4)
    grouped = sc.contract()[0]
    kinds = [e["kind"] for e in sc.profile_chunk(0)]
    assert "group" in kinds
    sc.set_grouping(False)
    single = sc.contract()[0]
    assert "group" not in [e["kind"] for e in sc.profile_chunk(0)]
    assert abs(grouped - ref) <= 1e-5 * abs(ref)
    assert abs(single - ref) <= 1e-5 * abs(ref)
