"""expectation.build_leaves on the CPU: the batched construction of the
RX / RZ gate leaves (one gather, cos, sin and complex tensor per gate kind)
against the gate matrices of expectation.numeric_network (numpy complex128)
and against a construction one gate at a time, for values and for the
gradients it carries back to the angles; and the angle-independent leaves
and gather indices are served from const_cache on repeated calls."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _spec(rows=3, cols=3, layers=4, seed=5):
    from jet_gb300 import expectation as ex

    rng = np.random.default_rng(seed)
    th = rng.uniform(0, 2 * np.pi, (layers, rows * cols))
    ph = rng.uniform(0, 2 * np.pi, (layers, rows * cols))
    spec = ex.zz_network(rows, cols, layers, ex.default_pair(rows, cols, seed))
    return spec, th, ph


def _one_by_one(spec, t, p):
    """Each gate leaf from its own angle, as plain torch operations."""
    out = []
    for lf in spec:
        if lf.kind == "const":
            out.append(torch.as_tensor(lf.data, dtype=torch.complex128).reshape(lf.shape))
            continue
        a = (t if lf.kind == "rx" else p)[lf.layer, lf.qubit]
        c, s = torch.cos(a / 2), torch.sin(a / 2)
        z = torch.zeros_like(c)
        if lf.kind == "rx":
            g = torch.complex(torch.stack([c, z, z, c]), torch.stack([z, -s, -s, z]))
        else:
            g = torch.complex(torch.stack([c, z, z, c]), torch.stack([-s, z, z, s]))
        g = g.reshape(2, 2)
        out.append(torch.conj(g).resolve_conj() if lf.conj else g)
    return out


def test_leaves_equal_gate_matrices():
    from jet_gb300 import expectation as ex

    spec, th, ph = _spec()
    lv = ex.build_leaves(spec, torch.tensor(th), torch.tensor(ph), dtype=torch.complex128)
    net = ex.numeric_network(spec, th, ph)
    assert len(lv) == len(spec) == len(net.tensors)
    for (lab, sh, d), lf, x in zip(net.tensors, spec, lv):
        assert list(x.shape) == list(sh) == lf.shape
        np.testing.assert_allclose(x.detach().numpy().reshape(-1), d, rtol=0, atol=1e-15)


@pytest.mark.parametrize("dtype", [torch.complex64, torch.complex128])
def test_values_and_gradients_equal_one_by_one(dtype):
    from jet_gb300 import expectation as ex

    spec, th, ph = _spec(seed=9)
    real = torch.float32 if dtype == torch.complex64 else torch.float64
    rng = np.random.default_rng(1)
    weights = [torch.tensor(rng.standard_normal(lf.shape) + 1j * rng.standard_normal(lf.shape),
                            dtype=dtype) for lf in spec]
    got, want = [], []
    for build, sink in ((lambda s, t, p: ex.build_leaves(s, t, p, dtype=dtype), got),
                        (lambda s, t, p: [x.to(dtype) for x in _one_by_one(s, t, p)], want)):
        t = torch.tensor(th, dtype=real, requires_grad=True)
        p = torch.tensor(ph, dtype=real, requires_grad=True)
        lv = build(spec, t, p)
        loss = sum((w * x).sum().real for w, x in zip(weights, lv))
        loss.backward()
        sink.append([x.detach() for x in lv])
        sink.append((t.grad.clone(), p.grad.clone()))
    for a, b in zip(got[0], want[0]):
        assert torch.equal(a, b)
    tol = 1e-6 if dtype == torch.complex64 else 1e-14
    for a, b in zip(got[1], want[1]):
        torch.testing.assert_close(a, b, rtol=tol, atol=tol)


def test_const_cache_reused():
    from jet_gb300 import expectation as ex

    spec, th, ph = _spec()
    cache = {}
    t, p = torch.tensor(th), torch.tensor(ph)
    first = ex.build_leaves(spec, t, p, dtype=torch.complex128, const_cache=cache)
    n = len(cache)
    second = ex.build_leaves(spec, t, p, dtype=torch.complex128, const_cache=cache)
    assert len(cache) == n
    for lf, a, b in zip(spec, first, second):
        if lf.kind == "const":
            assert a is b
        assert torch.equal(a, b)
