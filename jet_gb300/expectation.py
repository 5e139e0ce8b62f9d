"""Expectation values of parameterised circuits as doubled (bra-ket)
networks, with light-cone pruning, for gradient computations.

Circuit: a rows x cols grid, `layers` layers; each layer applies RX(theta)
then RZ(phi) on every qubit, then CZ on one of four alternating
nearest-neighbour coupler patterns (A B C D ... as in circuits.couplers).
Observable: Z_i Z_j. The network of <psi| Z_i Z_j |psi> keeps only the gates
in the backward light cone of {i, j}: a gate later than the moment its
qubits enter the cone cancels against its conjugate (U^dagger U = 1), so the
ket and bra wires of such a qubit are joined directly.

Leaves are described symbolically (`Leaf`), so that `build_leaves` can
create them from angle tensors that require gradients: the gates are torch
functions of the angles and the bra gates their conjugates, and
jet_gb300.autograd.contract_network carries the gradient from the contracted
value back to every angle.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Sequence, Tuple

import numpy as np

from . import circuits


@dataclasses.dataclass
class Leaf:
    labels: List[str]
    shape: List[int]
    kind: str  # "const", "rx", "rz"
    layer: int = -1
    qubit: int = -1
    conj: bool = False
    data: np.ndarray = None


def zz_network(rows: int, cols: int, layers: int, pair: Tuple[int, int],
               lightcone: bool = True) -> List[Leaf]:
    n = rows * cols
    pats = circuits.couplers(rows, cols)
    # Backward light cone: the set of qubits whose gates matter at each layer.
    keep_cz = [[] for _ in range(layers)]
    keep_1q = [set() for _ in range(layers)]
    cone = set(pair)
    for layer in reversed(range(layers)):
        for a, b in pats["ABCD"[layer % 4]]:
            if not lightcone or a in cone or b in cone:
                keep_cz[layer].append((a, b))
        for a, b in keep_cz[layer]:
            cone |= {a, b}
        keep_1q[layer] = set(range(n)) if not lightcone else set(cone)
    active = set(range(n)) if not lightcone else cone
    ver = {q: 0 for q in range(n)}
    leaves: List[Leaf] = []
    ket = lambda q: "k%d_%d" % (q, ver[q])  # noqa: E731
    bra = lambda q: "b%d_%d" % (q, ver[q])  # noqa: E731
    zero = np.array([1, 0], dtype=np.complex128)
    for q in sorted(active):
        leaves.append(Leaf([ket(q)], [2], "const", data=zero))
        leaves.append(Leaf([bra(q)], [2], "const", data=zero))
    cz = circuits.gate_cz().reshape(-1)
    for layer in range(layers):
        for kind in ("rx", "rz"):
            for q in sorted(keep_1q[layer]):
                ki, bi = ket(q), bra(q)
                ver[q] += 1
                leaves.append(Leaf([ket(q), ki], [2, 2], kind, layer, q, False))
                leaves.append(Leaf([bra(q), bi], [2, 2], kind, layer, q, True))
        for a, b in keep_cz[layer]:
            ka, kb, ba, bb = ket(a), ket(b), bra(a), bra(b)
            ver[a] += 1
            ver[b] += 1
            leaves.append(Leaf([ket(a), ket(b), ka, kb], [2, 2, 2, 2], "const", data=cz))
            leaves.append(Leaf([bra(a), bra(b), ba, bb], [2, 2, 2, 2], "const", data=cz.conj()))
    # Close the wires: Z on the pair, identity (shared label) elsewhere.
    zmat = np.diag([1.0, -1.0]).astype(np.complex128).reshape(-1)
    rename = {}
    for q in sorted(active):
        if q in pair:
            leaves.append(Leaf([bra(q), ket(q)], [2, 2], "const", data=zmat))
        else:
            rename[bra(q)] = ket(q)
    for lf in leaves:
        lf.labels = [rename.get(x, x) for x in lf.labels]
    return leaves


def numeric_network(leaves: Sequence[Leaf], thetas: np.ndarray, phis: np.ndarray,
                    dtype=np.complex128) -> circuits.Network:
    """The network with every gate evaluated at the given angles (numpy)."""
    out = []
    for lf in leaves:
        if lf.kind == "const":
            d = lf.data
        elif lf.kind == "rx":
            d = circuits.gate_rx(thetas[lf.layer, lf.qubit]).reshape(-1)
        else:
            d = circuits.gate_rz(phis[lf.layer, lf.qubit]).reshape(-1)
        if lf.conj and lf.kind != "const":
            d = np.conj(d)
        out.append((list(lf.labels), list(lf.shape), np.asarray(d, dtype=dtype)))
    return circuits.Network(out)


def build_leaves(leaves: Sequence[Leaf], thetas, phis, dtype=None, device=None,
                 const_cache=None):
    """torch leaves as differentiable functions of the angle tensors.

    The gates of one kind (RX, RZ) are built together: one gather of their
    angles, one cos and one sin, one complex tensor of all their matrices and
    one of its conjugates; each leaf is a row of those (torch.unbind, whose
    backward is one stack). Built one by one, the gates of the 6 x 6, 10-layer
    network took about 9,000 torch operations forward and as many backward.

    const_cache (a dict, optional) keeps the angle-independent leaves and the
    gathers' index tensors on the device between calls, so a call makes no
    host-to-device copy (required inside a CUDA graph capture)."""
    import torch

    dtype = dtype or torch.complex64
    real = torch.float32 if dtype == torch.complex64 else torch.float64
    out = [None] * len(leaves)
    rows = {"rx": {}, "rz": {}}  # (layer, qubit) -> row of that kind's gates
    for i, lf in enumerate(leaves):
        if lf.kind == "const":
            key = (i, str(dtype), str(device))
            t = None if const_cache is None else const_cache.get(key)
            if t is None:
                t = torch.as_tensor(lf.data, dtype=dtype, device=device).reshape(lf.shape)
                if const_cache is not None:
                    const_cache[key] = t
            out[i] = t
        else:
            rows[lf.kind].setdefault((lf.layer, lf.qubit), len(rows[lf.kind]))
    for kind, at in rows.items():
        if not at:
            continue
        src = thetas if kind == "rx" else phis
        key = ("index", kind, tuple(at), str(src.device))
        idx = None if const_cache is None else const_cache.get(key)
        if idx is None:
            lq = torch.as_tensor(list(at.keys()), dtype=torch.long, device=src.device)
            idx = (lq[:, 0].contiguous(), lq[:, 1].contiguous())
            if const_cache is not None:
                const_cache[key] = idx
        ang = src[idx].to(real)
        c, s = torch.cos(ang / 2), torch.sin(ang / 2)
        z = torch.zeros_like(c)
        re = torch.stack([c, z, z, c], dim=1)
        if kind == "rx":  # [[c, -i s], [-i s, c]]
            ns = -s
            im = torch.stack([z, ns, ns, z], dim=1)
        else:  # diag(e^{-i phi/2}, e^{i phi/2})
            im = torch.stack([-s, z, z, s], dim=1)
        g = torch.complex(re, im).to(dtype).reshape(-1, 2, 2)
        if device is not None:
            g = g.to(device)
        kets = torch.unbind(g)
        bras = None
        for i, lf in enumerate(leaves):
            if lf.kind != kind:
                continue
            r = at[(lf.layer, lf.qubit)]
            if lf.conj:
                if bras is None:
                    bras = torch.unbind(torch.conj(g).resolve_conj())
                out[i] = bras[r]
            else:
                out[i] = kets[r]
    return out


def default_pair(rows: int, cols: int, seed: int = 0) -> Tuple[int, int]:
    """A seeded horizontal nearest-neighbour pair."""
    rng = np.random.default_rng(seed)
    r = int(rng.integers(rows))
    c = int(rng.integers(cols - 1))
    return (r * cols + c, r * cols + c + 1)
