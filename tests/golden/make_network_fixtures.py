"""Golden fixtures of full-size networks for the GPU parity tests.

Writes into tests/golden/:

  m10_network.npz, m12_network.npz
      The reference's paper-benchmark networks
      (examples/paper_benchmarks/data_files/m10.json and m12.json: 53-qubit
      Sycamore circuits of depth 10 and 12, rank-3 tensors, with a stored
      contraction path) in a compact binary form: per tensor its tags, index
      labels, shape and complex64 data, plus the path. The GPU tests rebuild
      the JSON text of the reference's schema from it and load it through
      jet_gb300.io, the TensorNetworkSerializer counterpart.

  network_amplitudes.json
      m10:     the full amplitude <0|C|0> along the stored path, from the
               reference headers compiled in this container
               (TensorNetwork::Contract, TensorNetwork.hpp:301-328, in
               complex<float> and complex<double>) and from the complex128
               oracle;
      m12:     slices 0, 1 and 2 of the reference's own 9-index slicing
               (GPU/jet_gpu_m12/jet_sliced_subset.cpp:53-54, slices
               0 .. num_slices_to_contract - 1 = 2), complex128 oracle, and
               the compiled reference in complex<float> for slice 0;
      config4: the 53-qubit circuit (6 x 9 grid minus site 5, 12 cycles,
               seed 20240601) with its greedy path and 6 sliced bonds, and
               the amplitudes of slices 0 and 37 from the complex128 oracle
               and from the compiled reference in complex<float>;
      config2: the 49-qubit circuit (7 x 7 grid, 14 cycles) with its greedy
               path and 12 sliced bonds (4096 slices).

  config3_gradient.json
      The 36-qubit parameterised circuit (6 x 6, 10 layers, 720 angles):
      its path, the loss Re<psi|Z_i Z_j|psi> and the full gradient with
      respect to all 720 angles, from complex128 torch.einsum autograd on
      the CPU along that path.

Usage (in a container with the reference tree; JET_REF overrides its
location):

  make -C oracle/ref_build
  python tests/golden/make_network_fixtures.py [--only m10,m12,config4,config2,config3]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

SEED = 20240601
M12_SLICED = ["h5", "m", "H10", "w", "y", "J", "S", "G10", "P0"]
C4 = dict(rows=6, cols=9, cycles=12, removed=[5], n_sliced=6, restarts=48, slices=[0, 37])
C3 = dict(rows=6, cols=6, layers=10, restarts=8)
C2 = dict(rows=7, cols=7, cycles=14, removed=[], n_sliced=12, restarts=48)


def reference_root() -> str:
    """The reference tree: $JET_REF, else where this container holds it."""
    return os.environ.get("JET_REF", "/root/reference")


def save_network_npz(path_out: str, js: dict) -> None:
    """The network of a reference JSON file as flat arrays (no pickled
    objects): tags and labels joined by ',' per tensor and '\\n' between
    tensors."""
    tensors = js["tensors"]
    ranks = np.array([len(t[1]) for t in tensors], dtype=np.int64)
    shapes = np.array([int(s) for t in tensors for s in t[2]], dtype=np.int64)
    sizes = np.array([len(t[3]) for t in tensors], dtype=np.int64)
    data = np.array([complex(x[0], x[1]) for t in tensors for x in t[3]], dtype=np.complex64)
    tags = "\n".join(",".join(t[0]) for t in tensors)
    labels = "\n".join(",".join(t[1]) for t in tensors)
    path = np.array(js.get("path", []), dtype=np.int64).reshape(-1, 2)
    np.savez_compressed(path_out, ranks=ranks, shapes=shapes, sizes=sizes, data=data,
                        tags=np.array(tags), labels=np.array(labels), path=path)


def load_network_npz(path_in: str):
    """(tensors [(tags, labels, shape, complex64 data)], path) of a file
    written by save_network_npz."""
    z = np.load(path_in)
    tags = str(z["tags"]).split("\n")
    labels = str(z["labels"]).split("\n")
    out = []
    so = do = 0
    for i, r in enumerate(z["ranks"]):
        sh = [int(v) for v in z["shapes"][so:so + r]]
        n = int(z["sizes"][i])
        out.append((tags[i].split(",") if tags[i] else [], labels[i].split(",") if r else [],
                    sh, z["data"][do:do + n]))
        so += r
        do += n
    return out, [tuple(int(v) for v in p) for p in z["path"]]


def network_json_text(tensors, path) -> str:
    """The reference's JSON schema (TensorNetworkIO.hpp:94-293) for a network
    read back from its npz form."""
    js = {"path": [list(p) for p in path],
          "tensors": [[list(tg), list(lb), list(sh),
                       [[float(x.real), float(x.imag)] for x in d]]
                      for tg, lb, sh, d in tensors]}
    return json.dumps(js)


def _oracle_amplitude(tensors, path, sliced=(), value=0):
    from oracle import jet_oracle as jo

    tn = jo.OTensorNetwork()
    for lb, sh, d in tensors:
        tn.add_tensor(jo.OTensor.make(lb, sh, np.asarray(d, dtype=np.complex128)))
    if sliced:
        tn.slice_indices(list(sliced), value)
    out = tn.contract(path, release=True)
    return complex(out.data.reshape(-1)[0])


def _ref_amplitude(tensors, path, dtype, sliced=(), value=0):
    from oracle import ref

    if not ref.available():
        raise SystemExit("oracle/_ref/libjetref.so missing: run make -C oracle/ref_build")
    ts = [(lb, sh, np.asarray(d, dtype=dtype)) for lb, sh, d in tensors]
    _, _, d, flops, mem = ref.network_contract(ts, path, sliced, value, out_cap=16)
    return complex(d.reshape(-1)[0]), flops, mem


def _pair(z: complex):
    return [z.real, z.imag]


def make_m10_m12(which, amps):
    root = os.path.join(reference_root(), "examples", "paper_benchmarks", "data_files")
    for name in ("m10", "m12"):
        if name not in which:
            continue
        with open(os.path.join(root, name + ".json")) as f:
            js = json.load(f)
        npz = os.path.join(HERE, name + "_network.npz")
        save_network_npz(npz, js)
        tensors, path = load_network_npz(npz)
        plain = [(lb, sh, d) for _, lb, sh, d in tensors]
        t0 = time.time()
        if name == "m10":
            r64, flops, mem = _ref_amplitude(plain, path, np.complex64)
            r128, _, _ = _ref_amplitude(plain, path, np.complex128)
            o128 = _oracle_amplitude(plain, path)
            amps["m10"] = {"tensors": len(plain), "path_steps": len(path),
                           "pathinfo_flops": flops, "pathinfo_memory": mem,
                           "ref_c64": _pair(r64), "ref_c128": _pair(r128),
                           "oracle_c128": _pair(o128)}
        else:
            ent = {"tensors": len(plain), "path_steps": len(path), "sliced": M12_SLICED,
                   "slices": {}}
            for v in (0, 1, 2):
                ent["slices"][str(v)] = {"oracle_c128": _pair(
                    _oracle_amplitude(plain, path, M12_SLICED, v))}
                print("m12 slice", v, "oracle", time.time() - t0, flush=True)
            r64, flops, mem = _ref_amplitude(plain, path, np.complex64, M12_SLICED, 0)
            ent["slices"]["0"]["ref_c64"] = _pair(r64)
            ent["pathinfo_flops_per_slice"] = flops
            ent["pathinfo_memory_per_slice"] = mem
            amps["m12"] = ent
        print(name, "done in %.1f s" % (time.time() - t0), flush=True)


def make_config4(amps):
    from jet_gb300 import circuits

    net = circuits.random_circuit_network(C4["rows"], C4["cols"], C4["cycles"], seed=SEED,
                                          removed=tuple(C4["removed"]))
    path = circuits.best_gain_path(net, C4["restarts"])
    sliced = circuits.choose_slices(net, path, C4["n_sliced"])
    flops, big = circuits.path_cost(net, path, sliced)
    ent = {k: C4[k] for k in ("rows", "cols", "cycles", "removed")}
    ent.update(seed=SEED, path=[list(p) for p in path], sliced=sliced,
               slice_pathinfo_flops=flops, log2_largest=big, slices={})
    plain = [(lb, sh, d) for lb, sh, d in net.tensors]
    for v in C4["slices"]:
        t0 = time.time()
        ent["slices"][str(v)] = {"oracle_c128": _pair(_oracle_amplitude(plain, path, sliced, v))}
        ent["slices"][str(v)]["ref_c64"] = _pair(
            _ref_amplitude(plain, path, np.complex64, sliced, v)[0])
        print("config4 slice", v, "%.1f s" % (time.time() - t0), flush=True)
    amps["config4"] = ent


def make_config2(amps):
    """The 49-qubit circuit's path and 12 sliced bonds (no amplitude: one
    slice is 3.6e13 PathInfo flops with intermediates of 2^30 elements, too
    large for the CPU oracle here)."""
    from jet_gb300 import circuits

    net = circuits.random_circuit_network(C2["rows"], C2["cols"], C2["cycles"], seed=SEED)
    path = circuits.best_gain_path(net, C2["restarts"])
    sliced = circuits.choose_slices(net, path, C2["n_sliced"])
    flops, big = circuits.path_cost(net, path, sliced)
    ent = {k: C2[k] for k in ("rows", "cols", "cycles", "removed")}
    ent.update(seed=SEED, path=[list(p) for p in path], sliced=sliced,
               slice_pathinfo_flops=flops, log2_largest=big, slices={})
    amps["config2"] = ent


def make_config3():
    import torch

    from jet_gb300 import circuits, expectation as ex

    rows, cols, layers = C3["rows"], C3["cols"], C3["layers"]
    rng = np.random.default_rng(SEED)
    th = rng.uniform(0, 2 * np.pi, (layers, rows * cols))
    ph = rng.uniform(0, 2 * np.pi, (layers, rows * cols))
    pair = ex.default_pair(rows, cols, SEED)
    spec = ex.zz_network(rows, cols, layers, pair)
    path = circuits.find_path(ex.numeric_network(spec, th, ph), restarts=C3["restarts"],
                              seed=SEED)
    t = torch.tensor(th, dtype=torch.float64, requires_grad=True)
    p = torch.tensor(ph, dtype=torch.float64, requires_grad=True)
    leaves = ex.build_leaves(spec, t, p, dtype=torch.complex128)
    t0 = time.time()
    val = einsum_along_path(leaves, [lf.labels for lf in spec], path)
    loss = val.real.reshape(())
    loss.backward()
    print("config3 loss and gradient in %.1f s" % (time.time() - t0), flush=True)
    out = {"rows": rows, "cols": cols, "layers": layers, "seed": SEED, "pair": list(pair),
           "tensors": len(spec), "path": [list(q) for q in path],
           "thetas": th.tolist(), "phis": ph.tolist(),
           "loss": float(loss.item()),
           "grad_thetas": t.grad.numpy().tolist(), "grad_phis": p.grad.numpy().tolist(),
           "how": "complex128 torch.einsum autograd on the CPU, pairwise along the path"}
    with open(os.path.join(HERE, "config3_gradient.json"), "w") as f:
        json.dump(out, f)


def einsum_along_path(leaves, labels, path):
    """Pairwise torch.einsum contraction along `path` (node ids as in
    TensorNetwork::Contract: each result appends a node)."""
    import torch

    vals = list(leaves)
    labs = [list(lb) for lb in labels]
    alphabet = [chr(c) for c in range(ord("a"), ord("z") + 1)] + \
               [chr(c) for c in range(ord("A"), ord("Z") + 1)]
    for a, b in path:
        la, lb = labs[a], labs[b]
        letters = {}
        for x in la + lb:
            if x not in letters:
                letters[x] = alphabet[len(letters)]
        out = [x for x in la if x not in lb] + [x for x in lb if x not in la]
        eq = "%s,%s->%s" % ("".join(letters[x] for x in la), "".join(letters[x] for x in lb),
                            "".join(letters[x] for x in out))
        vals.append(torch.einsum(eq, vals[a], vals[b]))
        vals[a] = vals[b] = None
        labs.append(out)
    return vals[-1]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default="m10,m12,config4,config2,config3")
    which = set(ap.parse_args().only.split(","))
    amp_path = os.path.join(HERE, "network_amplitudes.json")
    amps = {}
    if os.path.exists(amp_path):
        with open(amp_path) as f:
            amps = json.load(f)
    make_m10_m12(which, amps)
    if "config4" in which:
        make_config4(amps)
    if "config2" in which:
        make_config2(amps)
    with open(amp_path, "w") as f:
        json.dump(amps, f)
    if "config3" in which:
        make_config3()


if __name__ == "__main__":
    main()
