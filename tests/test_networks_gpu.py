"""Full-size networks on the GPU against golden fixtures made on the CPU
(tests/golden/make_network_fixtures.py):

  * m10: the reference's own 53-qubit, depth-10 benchmark network
    (examples/paper_benchmarks/data_files/m10.json) rebuilt as JSON text of
    the reference's schema, loaded through jet_gb300.io (the
    TensorNetworkSerializer counterpart) and contracted on its stored path by
    a TaskBasedContractor, as the reference's GPU/jet_gpu_m10/jet_full.cpp
    does. Checked against the reference headers compiled on the CPU
    (complex<float> and complex<double>) and the complex128 oracle.
  * m12: slices 0, 1, 2 of the reference's 9-index slicing
    (GPU/jet_gpu_m12/jet_sliced_subset.cpp:53-54) through the sliced
    contractor, against the complex128 oracle and, for slice 0, the compiled
    reference in complex<float>.
  * config 4: two slices of the 53-qubit 6 x 9 x 12 circuit (1011 steps,
    3.6e12 PathInfo flops each) in AUTO, TUNED and plain FP32 against the
    complex128 oracle.
  * config 3: loss and all 720 gradient entries of the 6 x 6 x 10
    parameterised circuit through the hand-written adjoint, against
    complex128 torch.einsum autograd on the CPU.

Tolerances (complex64): 1e-5 relative for amplitudes against complex128, and
against the reference's own complex<float> result 1e-5 plus that result's
own distance from complex128 (two complex64 evaluations; m10: 7.5e-6); gradients within 1e-4
absolute (the bound set for adjoint gradients); the loss, an
expectation value in [-1, 1] that here cancels down to about 8e-4, within
1e-6 absolute. complex128 runs: 1e-12 relative (amplitudes), 1e-10 absolute
(gradients), 1e-12 absolute (loss).
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


@pytest.fixture(scope="module")
def jet(cuda):
    import jet_gb300

    return jet_gb300


@pytest.fixture(scope="module")
def amps():
    with open(os.path.join(GOLDEN, "network_amplitudes.json")) as f:
        return json.load(f)


def _c(pair):
    return complex(pair[0], pair[1])


def _rel(got, want):
    return abs(got - want) / abs(want)


def _load(name, dtype):
    import make_network_fixtures as mk

    import jet_gb300 as jet

    tensors, path = mk.load_network_npz(os.path.join(GOLDEN, name + "_network.npz"))
    text = mk.network_json_text(tensors, path)
    return jet.TensorNetworkSerializer(dtype=dtype)(text), tensors, path


@pytest.mark.parametrize("dtype,precision", [("complex64", 0), ("complex64", 2),
                                             ("complex128", 0)])
def test_m10_full_amplitude_through_serializer(jet, amps, dtype, precision):
    ent = amps["m10"]
    tnf, tensors, path = _load("m10", dtype)
    assert tnf.tensors.num_tensors == ent["tensors"] == len(tensors)
    assert len(tnf.path.path) == ent["path_steps"]
    assert tnf.path.total_flops() == ent["pathinfo_flops"]
    old = jet.get_precision()
    jet.set_precision(precision)
    try:
        tbc = jet.TaskBasedContractor(dtype=dtype)
        tbc.add_contraction_tasks(tnf.tensors, tnf.path)
        tbc.add_deletion_tasks()
        tbc.contract()
        got = complex(tbc.results[0].data[0])
    finally:
        jet.set_precision(old)
    if dtype == "complex64":
        assert _rel(got, _c(ent["ref_c128"])) <= 1e-5, _rel(got, _c(ent["ref_c128"]))
        # Two complex64 evaluations: within 1e-5 plus the reference's own
        # complex<float> distance from complex128 (7.5e-6 on m10).
        ref_err = _rel(_c(ent["ref_c64"]), _c(ent["ref_c128"]))
        assert _rel(got, _c(ent["ref_c64"])) <= 1e-5 + ref_err, _rel(got, _c(ent["ref_c64"]))
    else:
        assert _rel(got, _c(ent["ref_c128"])) <= 1e-12
        assert _rel(got, _c(ent["oracle_c128"])) <= 1e-12


@pytest.mark.parametrize("precision", [0, 2])
def test_m12_reference_slices(jet, amps, precision):
    ent = amps["m12"]
    tnf, _, path = _load("m12", "complex64")
    sc = jet.SlicedContractorC64(tnf.tensors, path, ent["sliced"], precision)
    assert sc.num_slices == 2 ** 9
    sc.set_batch_size(1)
    vals = []
    for v in (0, 1, 2):
        got = sc.contract(v, 1)[0]
        want = _c(ent["slices"][str(v)]["oracle_c128"])
        assert _rel(got, want) <= 1e-5, (v, _rel(got, want))
        vals.append(got)
    ref0 = _c(ent["slices"]["0"]["ref_c64"])
    ref_err = _rel(ref0, _c(ent["slices"]["0"]["oracle_c128"]))
    assert _rel(vals[0], ref0) <= 1e-5 + ref_err, _rel(vals[0], ref0)
    # Slices 0 and 1 in one batch, summed in FP64 on the device.
    sc2 = jet.SlicedContractorC64(tnf.tensors, path, ent["sliced"], precision)
    sc2.set_batch_size(2)
    total = sc2.contract(0, 2)[0]
    want = sum(_c(ent["slices"][str(v)]["oracle_c128"]) for v in (0, 1))
    scale = sum(abs(_c(ent["slices"][str(v)]["oracle_c128"])) for v in (0, 1))
    assert abs(total - want) <= 1e-5 * scale


def _config4_network(jet, ent):
    from jet_gb300 import circuits

    net = circuits.random_circuit_network(ent["rows"], ent["cols"], ent["cycles"],
                                          seed=ent["seed"], removed=tuple(ent["removed"]))
    tn = jet.TensorNetwork(dtype="complex64")
    for lab, sh, d in net.tensors:
        tn.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype="complex64"))
    return tn, [tuple(p) for p in ent["path"]]


@pytest.mark.parametrize("precision", [2, 5, 0])
def test_config4_slices_match_oracle(jet, amps, precision):
    """AUTO and TUNED (tensor-core products on the large steps) within 1e-5 of
    complex128. Plain FP32 -- complex64 with FP32 FMA, the arithmetic of the
    reference's own complex<float> path -- within 1e-5, or where the
    reference's own complex<float> result (compiled reference, golden) is
    further than that from complex128, no further than it: on slice 37 the
    reference's error is 2.05e-5 (the slice's amplitude is a quarter of slice
    0's, with more cancellation)."""
    ent = amps["config4"]
    tn, path = _config4_network(jet, ent)
    sc = jet.SlicedContractorC64(tn, path, ent["sliced"], precision)
    assert sc.num_slices == 2 ** len(ent["sliced"])
    sc.set_batch_size(1)
    for v, rec in ent["slices"].items():
        got = sc.contract(int(v), 1)[0]
        want = _c(rec["oracle_c128"])
        tol = 1e-5
        if precision == 0:
            tol = max(tol, _rel(_c(rec["ref_c64"]), want))
        assert _rel(got, want) <= tol, (v, _rel(got, want), tol)
    from jet_gb300 import capi

    assert capi.take_device_status() == 0


@pytest.fixture(scope="module")
def config3():
    with open(os.path.join(GOLDEN, "config3_gradient.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("grouping", [True, False])
@pytest.mark.parametrize("dtype,precision,tol_grad,tol_loss", [
    ("complex64", 2, 1e-4, 1e-6), ("complex128", 0, 1e-10, 1e-12)])
def test_config3_gradient_matches_einsum(jet, config3, dtype, precision, tol_grad, tol_loss,
                                         grouping):
    """Through a plan, with the tiny steps of each dependency level in
    grouped launches and step by step."""
    import torch

    from jet_gb300 import autograd, expectation as ex

    g = config3
    dev = torch.device("cuda:0")
    spec = ex.zz_network(g["rows"], g["cols"], g["layers"], tuple(g["pair"]))
    assert len(spec) == g["tensors"]
    path = [tuple(p) for p in g["path"]]
    real = torch.float32 if dtype == "complex64" else torch.float64
    t = torch.tensor(g["thetas"], dtype=real, device=dev, requires_grad=True)
    p = torch.tensor(g["phis"], dtype=real, device=dev, requires_grad=True)
    lv = ex.build_leaves(spec, t, p, dtype=getattr(torch, dtype), device=dev)
    labels = [lf.labels for lf in spec]
    plan = autograd.ContractionPlan(labels, [lf.shape for lf in spec], path)
    plan.grouping = grouping
    loss = autograd.contract_network(lv, labels, path, precision=precision, plan=plan).real
    loss.backward()
    assert abs(float(loss.item()) - g["loss"]) <= tol_loss
    gt = t.grad.double().cpu().numpy()
    gp = p.grad.double().cpu().numpy()
    err = max(np.abs(gt - np.array(g["grad_thetas"])).max(),
              np.abs(gp - np.array(g["grad_phis"])).max())
    assert err <= tol_grad, err
