"""The adjoint's host logic (jet_gb300/autograd.py) on the CPU: the reverse
sweep over conjugated gradients, the operand orders it picks to avoid
transposes, the leaves' gradients gathered in one flat buffer, operands that
need no gradient skipped, and the sliced forward and backward. The library
calls it makes (contract, permute, conj, add, slice gather and scatter-add)
are replaced here by complex128 torch stand-ins of their documented
semantics, and the gradients are checked against torch autograd through
einsum of the same network. The GPU tests run the same code on the library."""
import collections

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _into(r, out):
    if out is None:
        return r
    out.reshape(-1)[: r.numel()].copy_(r.reshape(-1))
    return out


class _Stand:
    """CPU stand-ins of the capi calls the adjoint makes, counting calls."""

    def __init__(self):
        self.calls = collections.Counter()

    def contract(self, a, a_shape, a_perm, b, b_shape, b_perm, m, n, k, precision=0, out=None,
                 **kw):
        self.calls["contract"] += 1
        A = a.reshape(a_shape).permute(a_perm).reshape(m, k)
        B = b.reshape(b_shape).permute(b_perm).reshape(k, n)
        return _into((A @ B).reshape(-1), out)

    def permute(self, x, shape, perm, out=None, **kw):
        self.calls["permute"] += 1
        return _into(x.reshape(shape).permute(perm).reshape(-1).contiguous(), out)

    def conj(self, x, out=None, **kw):
        self.calls["conj"] += 1
        return _into(torch.conj(x).resolve_conj(), out)

    def add(self, a, b, out=None, **kw):
        self.calls["add"] += 1
        return _into(a + b, out)

    def launch_group(self, group):
        """jetgpu_contract_group: out[i, j] = sum_c x[a_row[i] + a_col[c]]
        y[b_row[c] + b_col[j]] for every task, read through its tables."""
        self.calls["group"] += 1
        self.calls["grouped_tasks"] += len(group.tasks)
        for t in group.tasks:
            op = t["op"]
            ar, ac, br, bc = (torch.as_tensor(x) for x in t["tables"])
            x, y = group.view(op.x), group.view(op.y)
            X = x[ar[:, None] + ac[None, :]]
            Y = y[br[:, None] + bc[None, :]]
            group.view(op.out)[: op.m * op.n] = (X @ Y).reshape(-1)

    @staticmethod
    def _index(shape, axes, strides, v):
        idx = [slice(None)] * len(shape)
        for a, s in zip(axes, strides):
            idx[a] = (v // s) % shape[a]
        return tuple(idx)

    def slice_gather(self, x, shape, axes, value_strides, first_value, n_values, out=None, **kw):
        self.calls["slice_gather"] += 1
        r = x.reshape(shape)[self._index(shape, axes, value_strides, first_value)]
        return _into(r.reshape(-1).contiguous(), out)

    def slice_scatter_add(self, sliced, shape, axes, value_strides, value, full, **kw):
        self.calls["slice_scatter_add"] += 1
        view = full.view(shape)[self._index(shape, axes, value_strides, value)]
        view += sliced.reshape(view.shape)
        return full


@pytest.fixture
def stand(monkeypatch):
    from jet_gb300 import capi, grouped

    s = _Stand()
    for name in ("contract", "permute", "conj", "add", "slice_gather", "slice_scatter_add"):
        monkeypatch.setattr(capi, name, getattr(s, name))
    monkeypatch.setattr(grouped, "launch_group", s.launch_group)
    return s


def _network(rows, cols, layers, seed):
    from jet_gb300 import circuits, expectation as ex

    rng = np.random.default_rng(seed)
    th = rng.uniform(0, 2 * np.pi, (layers, rows * cols))
    ph = rng.uniform(0, 2 * np.pi, (layers, rows * cols))
    spec = ex.zz_network(rows, cols, layers, ex.default_pair(rows, cols, seed))
    path = circuits.find_path(ex.numeric_network(spec, th, ph), restarts=2, seed=seed)
    return spec, path, th, ph


def _einsum_loss(leaves, labels, path):
    vals, labs = list(leaves), [list(l) for l in labels]
    for i, j in path:
        la, lb = labs[i], labs[j]
        out = [x for x in la if x not in lb] + [x for x in lb if x not in la]
        sym = {x: chr(97 + q) for q, x in enumerate(dict.fromkeys(la + lb))}
        eq = "".join(sym[x] for x in la) + "," + "".join(sym[x] for x in lb) + "->" + "".join(
            sym[x] for x in out)
        vals.append(torch.einsum(eq, vals[i], vals[j]))
        labs.append(out)
    return vals[-1].real.reshape(())


def _grads(spec, path, th, ph, via, grouping=False, **kw):
    from jet_gb300 import autograd, expectation as ex

    t = torch.tensor(th, requires_grad=True)
    p = torch.tensor(ph, requires_grad=True)
    lv = ex.build_leaves(spec, t, p, dtype=torch.complex128)
    labels = [l.labels for l in spec]
    if via == "adjoint":
        if "plan" not in kw and "sliced" not in kw:
            plan = autograd.ContractionPlan(labels, [l.shape for l in spec], path)
            plan.grouping = grouping
            kw["plan"] = plan
        loss = autograd.contract_network(lv, labels, path, precision=0, **kw).real
    else:
        loss = _einsum_loss(lv, labels, path)
    loss.backward()
    return float(loss.detach()), t.grad, p.grad


@pytest.mark.parametrize("shape", [(2, 3, 3), (3, 3, 4)])
def test_adjoint_matches_einsum_autograd(stand, shape):
    spec, path, th, ph = _network(*shape, seed=11)
    loss, gt, gp = _grads(spec, path, th, ph, "adjoint")
    calls = dict(stand.calls)
    want, wt, wp = _grads(spec, path, th, ph, "einsum")
    assert abs(loss - want) <= 1e-14
    torch.testing.assert_close(gt, wt, rtol=0, atol=1e-13)
    torch.testing.assert_close(gp, wp, rtol=0, atol=1e-13)
    # One conjugation of the incoming gradient and one of all the leaves'
    # gradients; the forward once and its recomputation once; no gradient
    # for the constant leaves (states, CZ, Z): fewer than two adjoint
    # contractions per step.
    steps = len(path)
    assert calls["conj"] == 2
    assert calls["contract"] < 2 * steps + 2 * steps
    assert calls["contract"] >= 2 * steps + sum(1 for l in spec if l.kind != "const")


@pytest.mark.parametrize("grouping", [True, False])
def test_sliced_adjoint_matches_einsum_autograd(stand, grouping):
    """Slice by slice, the sliced network's plan grouped (its forward and the
    recomputation in grouped launches) or not."""
    from jet_gb300 import autograd, circuits, expectation as ex

    spec, path, th, ph = _network(2, 3, 3, seed=4)
    net = ex.numeric_network(spec, th, ph)
    sliced = circuits.choose_slices(net, path, 2)
    assert sliced
    plan = autograd.ContractionPlan([l.labels for l in spec], [l.shape for l in spec], path)
    plan.grouping = grouping
    sp = autograd.SlicedPlan(plan, path, sliced)
    loss, gt, gp = _grads(spec, path, th, ph, "adjoint", sliced=sliced, plan=sp)
    assert stand.calls["slice_scatter_add"] > 0
    assert (stand.calls["group"] > 0) == grouping
    want, wt, wp = _grads(spec, path, th, ph, "einsum")
    assert abs(loss - want) <= 1e-14
    torch.testing.assert_close(gt, wt, rtol=0, atol=1e-13)
    torch.testing.assert_close(gp, wp, rtol=0, atol=1e-13)


def test_leaves_without_grad_get_none(stand):
    from jet_gb300 import autograd

    rng = np.random.default_rng(3)
    labels = [["i", "j"], ["j", "k"], ["k", "i"]]
    shapes = [[2, 3], [3, 4], [4, 2]]
    leaves = [torch.tensor(rng.standard_normal(s) + 1j * rng.standard_normal(s),
                           requires_grad=(q != 1)) for q, s in enumerate(shapes)]
    out = autograd.contract_network(leaves, labels, [(0, 1), (2, 3)], precision=0)
    out.real.backward()
    assert leaves[1].grad is None
    ref = [x.detach().clone().requires_grad_(x.requires_grad) for x in leaves]
    torch.einsum("ij,jk,ki->", *ref).real.backward()
    for x, r in zip(leaves, ref):
        if x.requires_grad:
            torch.testing.assert_close(x.grad, r.grad, rtol=0, atol=1e-13)


@pytest.mark.parametrize("shape", [(2, 3, 3), (3, 3, 4)])
def test_grouped_levels_match_einsum_autograd(stand, shape):
    """The tiny steps of each dependency level in one grouped launch (tables
    read through by the stand-in), forward and reverse sweep; the same plan
    evaluated twice reuses its arenas and task tables."""
    from jet_gb300 import autograd, expectation as ex

    spec, path, th, ph = _network(*shape, seed=11)
    labels = [l.labels for l in spec]
    plan = autograd.ContractionPlan(labels, [l.shape for l in spec], path)
    want, wt, wp = _grads(spec, path, th, ph, "einsum")
    for rep in range(2):
        stand.calls.clear()
        t = torch.tensor(th, requires_grad=True)
        p = torch.tensor(ph, requires_grad=True)
        lv = ex.build_leaves(spec, t, p, dtype=torch.complex128)
        loss = autograd.contract_network(lv, labels, path, precision=0, plan=plan).real
        loss.backward()
        assert abs(float(loss.detach()) - want) <= 1e-14
        torch.testing.assert_close(t.grad, wt, rtol=0, atol=1e-13)
        torch.testing.assert_close(p.grad, wp, rtol=0, atol=1e-13)
        calls = dict(stand.calls)
        steps = len(path)
        # Forward, recomputation and the adjoint's contractions nearly all
        # grouped: far fewer launches than steps.
        assert calls["group"] > 0 and calls["grouped_tasks"] > steps
        assert calls.get("contract", 0) + calls["group"] < steps
        assert calls["conj"] == 2
    g = plan._grouped[(torch.complex128, "cpu")]
    assert g is not None and len(g.backward_schedules) == 1


def test_grouping_off_runs_step_by_step(stand):
    spec, path, th, ph = _network(2, 3, 3, seed=2)
    _grads(spec, path, th, ph, "adjoint", grouping=False)
    assert stand.calls["group"] == 0
    want = _grads(spec, path, th, ph, "einsum")
    stand.calls.clear()
    got = _grads(spec, path, th, ph, "adjoint", grouping=True)
    assert stand.calls["group"] > 0
    assert abs(got[0] - want[0]) <= 1e-14
    torch.testing.assert_close(got[1], want[1], rtol=0, atol=1e-13)


def test_schedule_refuses_tables_outside_their_regions():
    """A grouped task whose offset tables or output would leave its arena
    region is refused on the host (NoGroup) before anything is uploaded."""
    from jet_gb300 import grouped

    arenas = {"val": torch.zeros(64, dtype=torch.complex128)}
    # x: a 2 x 4 tensor, y: 4 x 3, out: 2 x 3 -> m 2, n 3, k 4 (tiny).
    good = [grouped.Op(("val", 0, 8), ["i", "c"], [2, 4], ("val", 8, 12), ["c", "j"], [4, 3],
                       ("val", 20, 6)),
            grouped.Op(("val", 26, 8), ["i", "c"], [2, 4], ("val", 34, 12), ["c", "j"], [4, 3],
                       ("val", 46, 6))]
    s = grouped.Schedule([good], arenas, torch.complex128, torch.device("cpu"))
    assert [k for k, _ in s.items] == ["group"] and len(s.groups[0].tasks) == 2
    for bad_x, bad_out in ((("val", 0, 7), ("val", 20, 6)),   # x region one short
                           (("val", 0, 8), ("val", 20, 5)),   # out region one short
                           (("val", 0, 8), ("val", 60, 6))):  # out past the arena
        ops = [grouped.Op(bad_x, ["i", "c"], [2, 4], ("val", 8, 12), ["c", "j"], [4, 3],
                          bad_out), good[1]]
        with pytest.raises(grouped.NoGroup):
            grouped.Schedule([ops], arenas, torch.complex128, torch.device("cpu"))
