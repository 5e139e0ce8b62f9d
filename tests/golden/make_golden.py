"""Generates the golden fixtures in this directory from the reference Jet.

Run in a container that has the reference tree and its compiled headers
(oracle/ref_build/Makefile -> oracle/_ref/libjetref.so):

    make -C oracle/ref_build && python tests/golden/make_golden.py

Outputs (committed; nothing at test time reads the reference tree):
  permuter_vectors.json  -- the Permuter golden vectors of the reference's
                            test/Test_Permuter.cpp, parsed from the file as
                            text, each re-checked through the compiled
                            Permuter<DefaultPermuter> and Permuter<QFlexPermuter>.
  qflex_plans.json       -- accept / reject decisions of the compiled
                            QFlexPermuter<BLOCKSIZE, MIN_DIMS> plan on seeded
                            power-of-2 transposes (with the output hash when
                            accepted), for seven instantiations.
  ref_cases.json         -- seeded random cases run through the compiled
                            reference: Tensor::Transpose (SHA-256 of the
                            output bytes, bit-exact), ContractTensors
                            (outputs), SliceIndex, AddTensors, and
                            TensorNetwork::SliceIndices + Contract(path) +
                            PathInfo totals on small seeded circuit networks.
Inputs of the random cases are regenerated from their seeds by
tests/golden/cases.py, so the fixtures hold seeds and outputs only.
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from oracle import ref  # noqa: E402
import cases  # noqa: E402

REF_TEST = os.environ.get("JET_REF", "/root/reference") + "/test/Test_Permuter.cpp"


def parse_arrays(text: str):
    out = {}
    for m in re.finditer(r"static const std::vector<Data>\s+(\w+)\s*\{(.*?)\};", text, re.S):
        name, body = m.group(1), m.group(2)
        pairs = re.findall(r"\{\s*(-?\d+)\s*,\s*(-?\d+)\s*\}", body)
        out[name] = [[int(a), int(b)] for a, b in pairs]
    return out


# (array name, shape in current order, current labels, target labels),
# following the sections of Test_Permuter.cpp:182-519.
PERMUTER_CASES = [
    ("data_pow2_dbca", [2, 2, 2, 2], "dbca", "abcd"),
    ("data_pow2_cbad", [2, 2, 2, 2], "cbad", "abcd"),
    ("data_pow2_bacd", [2, 2, 2, 2], "bacd", "abcd"),
    ("data_pow2_badc", [2, 2, 2, 2], "badc", "abcd"),
    ("data_pow2_4x4_ba", [4, 4], "ba", "ab"),
    ("data_pow2_2x4x2_bac", [2, 4, 2], "bac", "abc"),
    ("data_pow2_2x4x2_acb", [2, 4, 2], "acb", "abc"),
    ("data_pow2_dbca", [2, 4, 2], "cba", "abc"),
    ("data_pow2_4x2x2_bac", [4, 2, 2], "bac", "abc"),
    ("data_pow2_4x2x2_acb", [4, 2, 2], "acb", "abc"),
    ("data_pow2_4x2x2_cba", [4, 2, 2], "cba", "abc"),
    ("data_pow2_bacd", [2, 2, 4], "bac", "abc"),
    ("data_pow2_2x2x4_acb", [2, 2, 4], "acb", "abc"),
    ("data_pow2_2x2x4_cba", [2, 2, 4], "cba", "abc"),
    ("data_non_pow2_bca", [3, 5, 2], "bca", "abc"),
    ("data_non_pow2_cba", [5, 3, 2], "cba", "abc"),
    ("data_non_pow2_cab", [5, 2, 3], "cab", "abc"),
    ("large_example", [2] * 9, "dghbiafce", "abcdefghi"),
]


def make_permuter_vectors():
    text = open(REF_TEST).read()
    arrays = parse_arrays(text)
    out = []
    for name, shape, old, new in PERMUTER_CASES:
        data = arrays[name]
        n = int(np.prod(shape))
        assert len(data) == n, (name, len(data), n)
        expected = [[i, i] for i in range(n)]  # FillArray(n): (i, i)
        x = np.array([complex(a, b) for a, b in data], dtype=np.complex64)
        backends = [0] + ([1] if (n & (n - 1)) == 0 else [])
        for be in backends:
            got = ref.permuter_transpose(be, x, shape, list(old), list(new))
            want = np.array([complex(a, b) for a, b in expected], dtype=np.complex64)
            assert np.array_equal(got, want), (name, be)
        out.append({"source": "test/Test_Permuter.cpp:" + name, "shape": shape,
                    "old": list(old), "new": list(new), "input": data, "expected": expected})
    # Exception messages of the Permuter front-end (Permuter.hpp:99-117) and
    # QFlex (QFlex.hpp:333-336, 517-519), as asserted by Test_Permuter.cpp:344-519.
    errors = []
    x30 = np.zeros(30, np.complex64)
    for be, shape, old, new, msg in [
        (1, [2, 3, 5, 2], "cab", "abc", "Tensor shape does not match number of indices."),
        (1, [2, 3, 5, 2], "cabd", "abcd", "Tensor shape does not match given tensor data."),
        (1, [3, 5, 2], "bca", "abc", "Fast transpose expects power-of-2 data"),
        (0, [2, 3, 5], "abb", "abc", "Duplicate existing indices found"),
        (0, [2, 3, 5], "abc", "abd", "New indices are an invalid permutation"),
    ]:
        try:
            ref.permuter_transpose(be, x30, shape, list(old), list(new))
            raise AssertionError("expected an exception")
        except ref.RefError as e:
            assert msg in str(e), (msg, str(e))
        errors.append({"shape": shape, "old": list(old), "new": list(new), "message": msg})
    big = np.array([complex(a, b) for a, b in arrays["large_example"]], np.complex64)
    try:
        ref.permuter_transpose(2, big, [2] * 9, list("dghbiafce"), list("abcdefghi"))
        raise AssertionError("expected an exception")
    except ref.RefError as e:
        assert "Consider increasing the BLOCKSIZE" in str(e)
    return {"cases": out, "errors": errors}


def sha(arr: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(arr).tobytes()).hexdigest()


def cplx_list(a: np.ndarray):
    return [[float(z.real), float(z.imag)] for z in a.reshape(-1)]


def make_ref_cases():
    res = {"transpose": [], "contract": [], "slice": [], "add": [], "network": []}
    for c in cases.transpose_cases():
        x = cases.tensor_data(c["seed"], c["shape"], c["dtype"])
        got = ref.tensor_transpose(x, c["shape"], c["old"], c["new"])
        res["transpose"].append(dict(c, sha256=sha(got)))
    for c in cases.contract_cases():
        a = cases.tensor_data(c["seed"], c["a_shape"], c["dtype"])
        b = cases.tensor_data(c["seed"] + 1, c["b_shape"], c["dtype"])
        lb, sh, d = ref.contract(c["a_labels"], c["a_shape"], a, c["b_labels"], c["b_shape"], b)
        res["contract"].append(dict(c, out_labels=lb, out_shape=sh, out=cplx_list(d)))
    for c in cases.slice_cases():
        x = cases.tensor_data(c["seed"], c["shape"], c["dtype"])
        lb, sh, d = ref.slice_index(c["labels"], c["shape"], x, c["index"], c["value"])
        res["slice"].append(dict(c, out_labels=lb, out_shape=sh, sha256=sha(d)))
    for c in cases.add_cases():
        a = cases.tensor_data(c["seed"], c["a_shape"], c["dtype"])
        b = cases.tensor_data(c["seed"] + 1, c["b_shape"], c["dtype"])
        lb, sh, d = ref.add_tensors(c["a_labels"], c["a_shape"], a, c["b_labels"], c["b_shape"], b)
        res["add"].append(dict(c, out_labels=lb, out_shape=sh, sha256=sha(d)))
    for c in cases.network_cases():
        tensors, path = cases.network(c)
        lb, sh, d, flops, mem = ref.network_contract(tensors, path, c["sliced"], c["slice_value"])
        res["network"].append(dict(c, out_labels=lb, out_shape=sh, out=cplx_list(d),
                                   flops=flops, memory=mem))
    return res


# QFlexPermuter instantiations of the reference wrapper (oracle/ref_build/ref_capi.cpp).
QFLEX_BACKENDS = {1: (1024, 32), 2: (64, 32), 3: (128, 64), 4: (256, 2), 5: (64, 2),
                  6: (2048, 1024), 7: (512, 32)}


def make_qflex_plans():
    """Accept / reject decisions of the reference's QFlexPermuter plan on
    seeded power-of-2 transposes (6 to 14 binary indices), for every
    instantiation above: per case the shape, labels, the output's SHA-256
    (DefaultPermuter; every accepting QFlexPermuter must match it) and, per
    "BLOCKSIZE,MIN_DIMS", true or the reference's error message."""
    rng = np.random.default_rng(2024)
    out = []
    for case in range(160):
        nbits = int(rng.integers(6, 15))
        dims = []
        left = nbits
        while left:
            k = int(rng.integers(1, min(3, left) + 1))
            dims.append(2 ** k)
            left -= k
        rank = len(dims)
        old = [chr(ord("a") + i) for i in range(rank)]
        new = [old[i] for i in rng.permutation(rank)]
        data = cases.tensor_data(7000 + case, [2 ** nbits], np.complex64)
        want = ref.permuter_transpose(0, data, dims, old, new)
        decisions = {}
        for backend, (block, min_dims) in QFLEX_BACKENDS.items():
            try:
                got = ref.permuter_transpose(backend, data, dims, old, new)
                assert np.array_equal(got, want)
                decisions["%d,%d" % (block, min_dims)] = True
            except ref.RefError as e:
                # Keep the message only (the text after "Error in Jet: ").
                decisions["%d,%d" % (block, min_dims)] = str(e).split("Error in Jet: ")[-1]
        out.append({"case": case, "seed": 7000 + case, "shape": dims, "old": old, "new": new,
                    "sha256": sha(want), "decisions": decisions})
    return out


def main():
    assert ref.available(), "build oracle/_ref first: make -C oracle/ref_build"
    with open(os.path.join(HERE, "qflex_plans.json"), "w") as f:
        json.dump(make_qflex_plans(), f)
    with open(os.path.join(HERE, "permuter_vectors.json"), "w") as f:
        json.dump(make_permuter_vectors(), f)
    with open(os.path.join(HERE, "ref_cases.json"), "w") as f:
        json.dump(make_ref_cases(), f)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
