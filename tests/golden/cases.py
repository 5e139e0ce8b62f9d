"""Seeded case definitions shared by the fixture generator and the tests.

Inputs come from a self-contained splitmix64 generator (not numpy's
distributions), so they regenerate bit-identically on any machine and numpy
version. Real and imaginary parts are multiples of 2^-24 in [-0.5, 0.5):
exactly representable in complex64, so complex64 and complex128 runs see the
same inputs.
"""
from __future__ import annotations

from typing import Dict, List

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(seed: int, n: int) -> np.ndarray:
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, n: int) -> np.ndarray:
    """n values in [-0.5, 0.5), multiples of 2^-24 (float64)."""
    z = _splitmix64(seed, n)
    return (z >> np.uint64(40)).astype(np.float64) / float(1 << 24) - 0.5


def tensor_data(seed: int, shape, dtype) -> np.ndarray:
    n = int(np.prod(shape)) if len(shape) else 1
    u = uniform(seed, 2 * n)
    return (u[0::2] + 1j * u[1::2]).astype(dtype)


def permutation(seed: int, r: int) -> List[int]:
    keys = _splitmix64(seed * 7919 + 17, r)
    return [int(i) for i in np.argsort(keys, kind="stable")]


def labels(r: int, offset: int = 0) -> List[str]:
    return ["x%d" % (i + offset) for i in range(r)]


def transpose_cases() -> List[Dict]:
    out = []
    seed = 1000
    # Power-of-2 tensors, ranks 1..14 (tiled kernel from 2^12 elements).
    for r in range(1, 15):
        shape = [2] * r
        old = labels(r)
        for rep in range(2):
            seed += 1
            p = permutation(seed, r)
            out.append({"seed": seed, "shape": shape, "old": old,
                        "new": [old[i] for i in p], "dtype": "complex64"})
    # Mixed power-of-2 dims.
    for shape in ([4, 8, 2, 16, 4], [32, 2, 64], [2, 128, 4, 8], [16, 16, 16, 4]):
        seed += 1
        old = labels(len(shape))
        p = permutation(seed, len(shape))
        out.append({"seed": seed, "shape": shape, "old": old,
                    "new": [old[i] for i in p], "dtype": "complex64"})
    # complex128.
    for shape in ([2] * 6, [2] * 13, [8, 4, 2, 16, 4]):
        seed += 1
        old = labels(len(shape))
        p = permutation(seed, len(shape))
        out.append({"seed": seed, "shape": shape, "old": old,
                    "new": [old[i] for i in p], "dtype": "complex128"})
    # Non-power-of-2 (qutrit-like) tensors; the reference's Default permuter
    # is exact up to 65536 elements.
    for shape in ([3] * 5, [3] * 9, [3, 2, 5], [6, 3, 4, 5], [3] * 10, [5, 7, 3, 2]):
        for dt in ("complex64", "complex128"):
            seed += 1
            old = labels(len(shape))
            p = permutation(seed, len(shape))
            out.append({"seed": seed, "shape": shape, "old": old,
                        "new": [old[i] for i in p], "dtype": dt})
    return out


def _rand_int(seed: int, lo: int, hi: int) -> int:
    return lo + int(_splitmix64(seed, 1)[0] % np.uint64(hi - lo + 1))


def contract_cases() -> List[Dict]:
    out = []
    seed = 5000
    specs = [
        # (n_left, n_common, n_right, dim)
        (1, 1, 1, 2), (2, 1, 0, 2), (0, 1, 2, 2), (0, 2, 0, 2), (2, 0, 2, 2),
        (3, 3, 3, 2), (4, 5, 3, 2), (5, 4, 6, 2), (2, 2, 2, 3), (3, 2, 1, 3),
        (6, 6, 5, 2), (6, 4, 6, 2), (1, 9, 1, 2), (8, 1, 0, 2), (0, 1, 8, 2),
    ]
    for dt in ("complex64", "complex128"):
        for nl, nc, nr, d in specs:
            seed += 1
            left = ["l%d" % i for i in range(nl)]
            common = ["c%d" % i for i in range(nc)]
            right = ["r%d" % i for i in range(nr)]
            a = left + common
            b = common + right
            pa = permutation(seed, len(a))
            pb = permutation(seed + 500, len(b))
            a = [a[i] for i in pa]
            b = [b[i] for i in pb]
            out.append({"seed": seed, "a_labels": a, "a_shape": [d] * len(a),
                        "b_labels": b, "b_shape": [d] * len(b), "dtype": dt})
    return out


def slice_cases() -> List[Dict]:
    out = []
    seed = 8000
    for shape, idx, val in (([2, 3, 4], 0, 1), ([2, 3, 4], 1, 2), ([2, 3, 4], 2, 3),
                            ([2] * 10, 4, 1), ([3] * 6, 5, 2), ([2] * 13, 0, 1)):
        seed += 1
        lab = labels(len(shape))
        out.append({"seed": seed, "shape": shape, "labels": lab, "index": lab[idx],
                    "value": val, "dtype": "complex64"})
    return out


def add_cases() -> List[Dict]:
    out = []
    seed = 9000
    for shape, swap in (([2, 2], False), ([2, 2], True), ([3, 4, 2], True), ([2] * 12, True)):
        seed += 1
        lab = labels(len(shape))
        p = permutation(seed, len(shape)) if swap else list(range(len(shape)))
        out.append({"seed": seed, "a_labels": lab, "a_shape": shape,
                    "b_labels": [lab[i] for i in p], "b_shape": [shape[i] for i in p],
                    "dtype": "complex64"})
    return out


def network_cases() -> List[Dict]:
    """Small seeded circuit networks (see jet_gb300.circuits)."""
    return [
        {"rows": 2, "cols": 2, "cycles": 4, "seed": 11, "sliced": [], "slice_value": 0,
         "dtype": "complex64"},
        {"rows": 3, "cols": 2, "cycles": 4, "seed": 12, "sliced": [], "slice_value": 0,
         "dtype": "complex128"},
        {"rows": 3, "cols": 3, "cycles": 4, "seed": 13, "n_sliced": 2, "slice_value": 3,
         "dtype": "complex64"},
        {"rows": 4, "cols": 4, "cycles": 8, "seed": 14, "sliced": [], "slice_value": 0,
         "dtype": "complex64"},
    ]


def network(case: Dict):
    """(tensors, path) of a network case; fills case['sliced'] when the case
    asks for n_sliced bonds (chosen by the slicer)."""
    import jet_gb300.circuits as circuits

    net = circuits.random_circuit_network(case["rows"], case["cols"], case["cycles"],
                                          seed=case["seed"], dtype=np.dtype(case["dtype"]))
    path = circuits.greedy_path(net, seed=case["seed"])
    if case.get("n_sliced"):
        case["sliced"] = circuits.choose_slices(net, path, case["n_sliced"])
    return net.tensors, path
