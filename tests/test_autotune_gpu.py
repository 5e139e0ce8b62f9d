"""The contraction autotuner (JETGPU_PREC_TUNED).

Each tuned contraction must match the complex128 oracle product within 1e-5
like the forms it picks from; the first contraction with a key makes one
table entry with a measured time for the chosen form, later ones with the
same key reuse it; small steps and keys first met inside a stream capture
take AUTO's rule without an entry; a sliced network contracted TUNED stays
within 1e-5 of FP64 (the eager chunk tunes, the captured graph replays the
choices)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture()
def tuner(cuda):
    from jet_gb300 import capi

    capi.autotune_clear()
    capi.set_autotune_min_work(1 << 20)
    yield capi
    capi.autotune_clear()
    capi.set_autotune_min_work(1 << 20)


def _operands(cuda, lm, lk, ln, seed):
    import torch

    g = torch.Generator(device=cuda)
    g.manual_seed(seed)
    a = torch.randn(2 ** (lm + lk), dtype=torch.complex64, device=cuda, generator=g)
    b = torch.randn(2 ** (lk + ln), dtype=torch.complex64, device=cuda, generator=g)
    rng = np.random.default_rng(seed)
    a_perm = list(rng.permutation(lm + lk))
    b_perm = list(rng.permutation(lk + ln))
    return a, [2] * (lm + lk), a_perm, b, [2] * (lk + ln), b_perm


def _want(capi, a, a_shape, a_perm, b, b_shape, b_perm, m, n, k):
    at = capi.permute(a, a_shape, a_perm).view(m, k).cpu().numpy().astype(np.complex128)
    bt = capi.permute(b, b_shape, b_perm).view(k, n).cpu().numpy().astype(np.complex128)
    return at @ bt


@pytest.mark.parametrize("lm,lk,ln", [(10, 10, 10), (12, 8, 6), (6, 12, 10), (12, 9, 0)])
def test_tuned_matches_fp64_and_tunes_once(tuner, cuda, lm, lk, ln):
    capi = tuner
    a, sa, pa, b, sb, pb = _operands(cuda, lm, lk, ln, seed=lm * 100 + lk * 10 + ln)
    m, k, n = 2 ** lm, 2 ** lk, 2 ** ln
    want = _want(capi, a, sa, pa, b, sb, pb, m, n, k)
    for _ in range(2):
        c = capi.contract(a, sa, pa, b, sb, pb, m, n, k, precision=capi.PREC_TUNED)
        got = c.view(m, n).cpu().numpy()
        assert np.linalg.norm(got - want) <= 1e-5 * np.linalg.norm(want)
    table = capi.autotune_table()
    if n < 2:
        assert table == []  # vector shapes are not tuned
        return
    assert len(table) == 1
    e = table[0]
    assert (e["batch"], e["m"], e["n"], e["k"]) == (1, m, n, k)
    assert e["choice"] in capi.AUTOTUNE_CANDIDATES
    assert e["ms"][e["choice"]] is not None and e["ms"][e["choice"]] > 0
    timed = [v for v in e["ms"].values() if v is not None]
    assert e["ms"][e["choice"]] == min(timed)
    assert capi.take_device_status() == 0


def test_small_steps_take_auto_without_an_entry(tuner, cuda):
    capi = tuner
    a, sa, pa, b, sb, pb = _operands(cuda, 6, 6, 6, seed=5)
    c = capi.contract(a, sa, pa, b, sb, pb, 64, 64, 64, precision=capi.PREC_TUNED)
    want = _want(capi, a, sa, pa, b, sb, pb, 64, 64, 64)
    assert np.linalg.norm(c.view(64, 64).cpu().numpy() - want) <= 1e-5 * np.linalg.norm(want)
    assert capi.autotune_table() == []
    capi.set_autotune_min_work(0)
    capi.contract(a, sa, pa, b, sb, pb, 64, 64, 64, precision=capi.PREC_TUNED)
    assert len(capi.autotune_table()) == 1


def test_batched_keys_differ_by_batch(tuner, cuda):
    import torch

    capi = tuner
    lm, lk, ln = 8, 8, 8
    m = n = k = 256
    g = torch.Generator(device=cuda)
    g.manual_seed(9)
    for batch in (4, 8):
        a = torch.randn(batch * m * k, dtype=torch.complex64, device=cuda, generator=g)
        b = torch.randn(batch * k * n, dtype=torch.complex64, device=cuda, generator=g)
        c = capi.contract_batched(batch, a, [2] * (lm + lk), list(range(lm + lk)), 1, b,
                                  [2] * (lk + ln), list(range(lk + ln)), 1, m, n, k,
                                  precision=capi.PREC_TUNED)
        at = a.view(batch, m, k).cpu().numpy().astype(np.complex128)
        bt = b.view(batch, k, n).cpu().numpy().astype(np.complex128)
        want = at @ bt
        got = c.view(batch, m, n).cpu().numpy()
        assert np.linalg.norm(got - want) <= 1e-5 * np.linalg.norm(want)
    table = capi.autotune_table()
    assert [(e["batch"], e["m"]) for e in table] == [(4, 256), (8, 256)]


def test_sliced_network_tuned_within_1e5_of_fp64(tuner, cuda):
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
    sliced = circuits.choose_slices(net, path, 2)

    def tn(dtype):
        t = jet.TensorNetwork(dtype=dtype)
        for lab, sh, d in net.tensors:
            t.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype=dtype))
        return t

    ref = jet.SlicedContractorC128(tn("complex128"), path, sliced, 0).contract()[0]
    tuner.set_autotune_min_work(1 << 16)
    sc = jet.SlicedContractorC64(tn("complex64"), path, sliced, jet.PREC_TUNED)
    sc.set_batch_size(2)
    got = sc.contract()[0]
    again = sc.contract()[0]
    assert abs(got - ref) <= 1e-5 * abs(ref)
    assert got == again  # the graph replays the same forms
    assert len(tuner.autotune_table()) > 0


def test_key_first_met_in_a_capture_takes_auto(tuner, cuda):
    """No timing inside a stream capture: a new key runs AUTO's form there and
    makes no entry; the replayed graph gives the right product."""
    import torch

    capi = tuner
    a, sa, pa, b, sb, pb = _operands(cuda, 9, 9, 9, seed=11)
    m = n = k = 512
    need = capi.contract_workspace_size(sa, pa, sb, pb, m, n, k, capi.C64, capi.PREC_TUNED)
    out = torch.empty(m * n, dtype=torch.complex64, device=cuda)
    ws = torch.empty(need, dtype=torch.uint8, device=cuda)
    # First launches configure kernels: keep them out of the capture.
    capi.contract(a, sa, pa, b, sb, pb, m, n, k, precision=capi.PREC_AUTO, out=out, workspace=ws)
    torch.cuda.synchronize()
    out.zero_()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        capi.contract(a, sa, pa, b, sb, pb, m, n, k, precision=capi.PREC_TUNED, out=out,
                      workspace=ws)
    assert capi.autotune_table() == []
    g.replay()
    torch.cuda.synchronize()
    want = _want(capi, a, sa, pa, b, sb, pb, m, n, k)
    got = out.view(m, n).cpu().numpy()
    assert np.linalg.norm(got - want) <= 1e-5 * np.linalg.norm(want)
