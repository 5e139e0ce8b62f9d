"""Gradients of Re<psi|Z_i Z_j|psi> with respect to gate angles through the
hand-written adjoint (jet_gb300.autograd on the GPU), checked against
complex128 torch.einsum autograd on the CPU along the same path and against
complex128 central finite differences (h = 1e-4) of the oracle contraction.
Tolerance: 1e-4 absolute against finite differences (complex64 GPU run),
1e-10 against einsum for the complex128 GPU run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _einsum_value(leaves, labels, path):
    """Pairwise torch.einsum contraction along `path` (CPU reference)."""
    import torch

    vals = list(leaves)
    labs = [list(l) for l in labels]
    for a, b in path:
        la, lb = labs[a], labs[b]
        letters = {}
        for x in la + lb:
            if x not in letters:
                letters[x] = chr(ord("a") + len(letters)) if len(letters) < 26 else chr(
                    ord("A") + len(letters) - 26)
        out = [x for x in la if x not in lb] + [x for x in lb if x not in la]
        eq = "%s,%s->%s" % ("".join(letters[x] for x in la), "".join(letters[x] for x in lb),
                            "".join(letters[x] for x in out))
        vals.append(torch.einsum(eq, vals[a], vals[b]))
        labs.append(out)
    return vals[-1]


def _setup(rows, cols, layers, seed):
    from jet_gb300 import circuits, expectation as ex

    rng = np.random.default_rng(seed)
    th = rng.uniform(0, 2 * np.pi, (layers, rows * cols))
    ph = rng.uniform(0, 2 * np.pi, (layers, rows * cols))
    pair = ex.default_pair(rows, cols, seed)
    leaves = ex.zz_network(rows, cols, layers, pair)
    net = ex.numeric_network(leaves, th, ph)
    path = circuits.find_path(net, restarts=2, seed=seed)
    return leaves, path, th, ph


def _oracle_loss(leaves, path, th, ph):
    from jet_gb300 import expectation as ex
    from oracle import jet_oracle as jo

    net = ex.numeric_network(leaves, th, ph)
    tn = jo.OTensorNetwork()
    for lab, sh, d in net.tensors:
        tn.add_tensor(jo.OTensor.make(lab, sh, d, np.complex128))
    return tn.contract(path).data[0].real


@pytest.mark.parametrize("dtype,precision,tol_einsum", [("complex64", 2, 1e-4),
                                                        ("complex128", 0, 1e-10)])
def test_adjoint_matches_einsum_and_finite_differences(cuda, dtype, precision, tol_einsum):
    import torch

    from jet_gb300 import autograd, expectation as ex

    rows, cols, layers = 3, 3, 4
    leaves, path, th, ph = _setup(rows, cols, layers, 3)
    tdt = getattr(torch, dtype)
    real = torch.float32 if dtype == "complex64" else torch.float64
    t = torch.tensor(th, dtype=real, device=cuda, requires_grad=True)
    p = torch.tensor(ph, dtype=real, device=cuda, requires_grad=True)
    lv = ex.build_leaves(leaves, t, p, dtype=tdt, device=cuda)
    val = autograd.contract_network(lv, [l.labels for l in leaves], path, precision=precision)
    loss = val.real
    loss.backward()
    g_t = t.grad.double().cpu().numpy()
    g_p = p.grad.double().cpu().numpy()
    # complex128 einsum autograd on the CPU.
    t64 = torch.tensor(th, dtype=torch.float64, requires_grad=True)
    p64 = torch.tensor(ph, dtype=torch.float64, requires_grad=True)
    lv64 = ex.build_leaves(leaves, t64, p64, dtype=torch.complex128)
    ref = _einsum_value(lv64, [l.labels for l in leaves], path).real
    ref.backward()
    assert abs(float(loss.item()) - float(ref.item())) <= max(tol_einsum, 1e-5)
    assert np.max(np.abs(g_t - t64.grad.numpy())) <= tol_einsum
    assert np.max(np.abs(g_p - p64.grad.numpy())) <= tol_einsum
    # Central finite differences in complex128 on a few angles.
    h = 1e-4
    rng = np.random.default_rng(0)
    for _ in range(6):
        l, q = int(rng.integers(layers)), int(rng.integers(rows * cols))
        for which, grad in (("t", g_t), ("p", g_p)):
            tp, pp = th.copy(), ph.copy()
            tm, pm = th.copy(), ph.copy()
            if which == "t":
                tp[l, q] += h
                tm[l, q] -= h
            else:
                pp[l, q] += h
                pm[l, q] -= h
            fd = (_oracle_loss(leaves, path, tp, pp) - _oracle_loss(leaves, path, tm, pm)) / (2 * h)
            assert abs(fd - grad[l, q]) <= 1e-4, (which, l, q, fd, grad[l, q])


def test_graphed_step_matches_eager(cuda):
    """The gradient captured in one CUDA graph equals the eager gradient, and
    a replay after new parameter values gives the eager result at those."""
    import torch

    from jet_gb300 import autograd, circuits
    from jet_gb300 import expectation as ex

    rows, cols, layers = 3, 3, 3
    rng = np.random.default_rng(5)
    pair = ex.default_pair(rows, cols, 5)
    spec = ex.zz_network(rows, cols, layers, pair)
    th = rng.uniform(0, 2 * np.pi, (layers, rows * cols))
    ph = rng.uniform(0, 2 * np.pi, (layers, rows * cols))
    path = circuits.find_path(ex.numeric_network(spec, th, ph), restarts=2, seed=5)
    labels = [l.labels for l in spec]
    plan = autograd.ContractionPlan(labels, [l.shape for l in spec], path)
    t = torch.tensor(th, dtype=torch.float32, device=cuda, requires_grad=True)
    p = torch.tensor(ph, dtype=torch.float32, device=cuda, requires_grad=True)

    consts = {}

    def loss_fn():
        lv = ex.build_leaves(spec, t, p, dtype=torch.complex64, device=cuda, const_cache=consts)
        return autograd.contract_network(lv, labels, path, precision=2, plan=plan).real

    def eager():
        t.grad = None
        p.grad = None
        val = loss_fn()
        val.backward()
        return float(val.item()), t.grad.clone(), p.grad.clone()

    v0, gt0, gp0 = eager()
    step = autograd.GraphedStep(loss_fn, [t, p])
    v1 = float(step.step().item())
    assert abs(v1 - v0) <= 1e-6 * max(abs(v0), 1e-30)
    assert torch.allclose(step.grads[0], gt0, rtol=1e-5, atol=1e-7)
    assert torch.allclose(step.grads[1], gp0, rtol=1e-5, atol=1e-7)
    with torch.no_grad():
        t.add_(0.1)
    v2 = float(step.step().item())
    g2t, g2p = step.grads[0].clone(), step.grads[1].clone()
    v3, gt3, gp3 = eager()
    assert abs(v2 - v3) <= 1e-6 * max(abs(v3), 1e-30)
    assert torch.allclose(g2t, gt3, rtol=1e-5, atol=1e-7)
    assert torch.allclose(g2p, gp3, rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("dtype,precision,tol", [("complex128", 0, 1e-11), ("complex64", 2, 1e-4)])
def test_sliced_adjoint_matches_unsliced_and_einsum(cuda, dtype, precision, tol):
    """Forward and backward run slice by slice over 3 sliced bonds (8 slices,
    each recomputed from the leaves): the value and every angle's gradient
    equal the unsliced adjoint's and complex128 einsum autograd's on the CPU.
    The sliced leaves' gradients come back through jetgpu_slice_scatter_add."""
    import torch

    from jet_gb300 import autograd, circuits, expectation as ex

    rows, cols, layers = 3, 3, 4
    leaves, path, th, ph = _setup(rows, cols, layers, 7)
    labels = [l.labels for l in leaves]
    net = ex.numeric_network(leaves, th, ph)
    sliced = circuits.choose_slices(net, path, 3)
    tdt = getattr(torch, dtype)
    real = torch.float32 if dtype == "complex64" else torch.float64

    def run(**kw):
        t = torch.tensor(th, dtype=real, device=cuda, requires_grad=True)
        p = torch.tensor(ph, dtype=real, device=cuda, requires_grad=True)
        lv = ex.build_leaves(leaves, t, p, dtype=tdt, device=cuda)
        val = autograd.contract_network(lv, labels, path, precision=precision, **kw).real
        val.backward()
        return float(val.item()), t.grad.double().cpu().numpy(), p.grad.double().cpu().numpy()

    v0, gt0, gp0 = run()
    v1, gt1, gp1 = run(sliced=sliced)
    t64 = torch.tensor(th, dtype=torch.float64, requires_grad=True)
    p64 = torch.tensor(ph, dtype=torch.float64, requires_grad=True)
    ref = _einsum_value(ex.build_leaves(leaves, t64, p64, dtype=torch.complex128), labels,
                        path).real
    ref.backward()
    assert abs(v1 - float(ref.item())) <= tol and abs(v1 - v0) <= tol
    for g, want in ((gt1, t64.grad.numpy()), (gp1, p64.grad.numpy()), (gt1, gt0), (gp1, gp0)):
        assert np.max(np.abs(g - want)) <= tol


def test_memory_budget_picks_slices(cuda):
    """memory_budget slices the network until one slice's checkpointed
    backward fits: a budget below the unsliced need gives sliced bonds, and
    the gradient is unchanged (complex128)."""
    import torch

    from jet_gb300 import autograd, expectation as ex

    from jet_gb300 import circuits

    rows, cols, layers = 3, 3, 4
    leaves, path, th, ph = _setup(rows, cols, layers, 8)
    labels = [l.labels for l in leaves]
    shapes = [l.shape for l in leaves]
    plan = autograd.ContractionPlan(labels, shapes, path)
    leaf_bytes = 16 * sum(int(np.prod(s)) for s in shapes)
    net = ex.numeric_network(leaves, th, ph)

    def need(count):
        sub = autograd.SlicedPlan(plan, path, circuits.choose_slices(net, path, count)).sub \
            if count else plan
        return autograd.checkpoint_bytes(sub, 16) + leaf_bytes

    needs = [need(c) for c in range(4)]
    budget = min(needs[1:])
    assert budget < needs[0]
    sliced = autograd.slices_for_budget(labels, shapes, path, budget, 16)
    assert 1 <= len(sliced) <= 3 and needs[len(sliced)] <= budget

    def grads(**kw):
        t = torch.tensor(th, dtype=torch.float64, device=cuda, requires_grad=True)
        p = torch.tensor(ph, dtype=torch.float64, device=cuda, requires_grad=True)
        lv = ex.build_leaves(leaves, t, p, dtype=torch.complex128, device=cuda)
        autograd.contract_network(lv, labels, path, precision=0, **kw).real.backward()
        return t.grad.cpu().numpy(), p.grad.cpu().numpy()

    a = grads()
    b = grads(memory_budget=budget)
    assert np.max(np.abs(a[0] - b[0])) <= 1e-11 and np.max(np.abs(a[1] - b[1])) <= 1e-11
