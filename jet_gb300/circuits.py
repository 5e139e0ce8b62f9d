"""Random-circuit tensor networks, a greedy contraction path and a slicer.

The reference builds circuit networks in Python (python/jet/circuit.py:181-194:
one tensor per operation, gate tensors hold the flattened matrix with indices
outputs ++ inputs, circuit.py:113-118 / gate.py:176-191) and samples random
paths (python/jet/interpreter.py:533-618). This module generates the seeded
Sycamore-style circuits of the benchmark configurations directly:

  * a rows x cols grid of qubits, each capped with |0> at both ends, so the
    network evaluates the amplitude <0...0| C |0...0>;
  * per cycle, one single-qubit gate per qubit drawn from {sqrtX, sqrtY,
    sqrtW} (never the gate that qubit had in the previous cycle), then
    fSim(theta, phi) on one of four alternating nearest-neighbour coupler
    patterns, in the order A B C D A B ... (A: horizontal couplers starting
    at an even column, B: odd column, C: vertical couplers starting at an
    even row, D: odd row).

sqrtY, sqrtW and fSim are not in the reference's gate set; they are defined
here from their standard matrices.

Paths use the reference's node-id convention (TensorNetwork.hpp:301-328,
PathInfo.hpp:80-113): contracting (i, j) appends a node whose id is the
current number of nodes.
"""
from __future__ import annotations

import dataclasses
import heapq
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

SQ2 = 1.0 / math.sqrt(2.0)


def gate_sqrt_x() -> np.ndarray:
    return SQ2 * np.array([[1, -1j], [-1j, 1]], dtype=np.complex128)


def gate_sqrt_y() -> np.ndarray:
    return SQ2 * np.array([[1, -1], [1, 1]], dtype=np.complex128)


def gate_sqrt_w() -> np.ndarray:
    # W = (X + Y) / sqrt(2); sqrt(W) = (I - i W) / sqrt(2).
    w = np.array([[0, np.exp(-1j * np.pi / 4)], [np.exp(1j * np.pi / 4), 0]])
    return SQ2 * (np.eye(2) - 1j * w)


def gate_fsim(theta: float, phi: float) -> np.ndarray:
    c, s = math.cos(theta), math.sin(theta)
    return np.array([[1, 0, 0, 0], [0, c, -1j * s, 0], [0, -1j * s, c, 0],
                     [0, 0, 0, np.exp(-1j * phi)]], dtype=np.complex128)


def gate_rx(theta: float) -> np.ndarray:
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return np.array([[c, -1j * s], [-1j * s, c]], dtype=np.complex128)


def gate_rz(phi: float) -> np.ndarray:
    return np.array([[np.exp(-0.5j * phi), 0], [0, np.exp(0.5j * phi)]], dtype=np.complex128)


def gate_cz() -> np.ndarray:
    return np.diag([1, 1, 1, -1]).astype(np.complex128)


@dataclasses.dataclass
class Network:
    """Leaf tensors as (labels, shape, flat row-major data)."""

    tensors: List[Tuple[List[str], List[int], np.ndarray]]
    open_labels: List[str] = dataclasses.field(default_factory=list)

    def index_dims(self) -> Dict[str, int]:
        d: Dict[str, int] = {}
        for lab, sh, _ in self.tensors:
            for x, s in zip(lab, sh):
                d[x] = s
        return d


def couplers(rows: int, cols: int) -> Dict[str, List[Tuple[int, int]]]:
    q = lambda r, c: r * cols + c  # noqa: E731
    pats: Dict[str, List[Tuple[int, int]]] = {"A": [], "B": [], "C": [], "D": []}
    for r in range(rows):
        for c in range(cols - 1):
            pats["A" if c % 2 == 0 else "B"].append((q(r, c), q(r, c + 1)))
    for r in range(rows - 1):
        for c in range(cols):
            pats["C" if r % 2 == 0 else "D"].append((q(r, c), q(r + 1, c)))
    return pats


class _Wires:
    def __init__(self, n: int):
        self.version = [0] * n

    def cur(self, q: int) -> str:
        return "q%d_%d" % (q, self.version[q])

    def advance(self, q: int) -> str:
        self.version[q] += 1
        return self.cur(q)


def random_circuit_network(rows: int, cols: int, cycles: int, seed: int = 0,
                           dtype=np.complex64, theta: float = math.pi / 2,
                           phi: float = math.pi / 6, removed: Sequence[int] = (),
                           bitstring: Optional[Sequence[int]] = None) -> Network:
    """Amplitude network <bitstring| C |0...0> of the seeded random circuit.

    `removed` lists grid sites without a qubit (the 53-qubit configuration
    removes one site of a 6x9 grid)."""
    rng = np.random.default_rng(seed)
    n = rows * cols
    present = [q not in set(removed) for q in range(n)]
    pats = couplers(rows, cols)
    singles = [gate_sqrt_x(), gate_sqrt_y(), gate_sqrt_w()]
    fsim = gate_fsim(theta, phi).reshape(2, 2, 2, 2)
    wires = _Wires(n)
    tensors: List[Tuple[List[str], List[int], np.ndarray]] = []
    zero = np.array([1, 0], dtype=np.complex128)
    for q in range(n):
        if present[q]:
            tensors.append(([wires.cur(q)], [2], zero.copy()))
    prev = [-1] * n
    for cyc in range(cycles):
        for q in range(n):
            if not present[q]:
                continue
            choices = [g for g in range(3) if g != prev[q]]
            g = choices[int(rng.integers(len(choices)))]
            prev[q] = g
            i = wires.cur(q)
            o = wires.advance(q)
            tensors.append(([o, i], [2, 2], singles[g].reshape(-1)))
        for a, b in pats["ABCD"[cyc % 4]]:
            if not (present[a] and present[b]):
                continue
            ia, ib = wires.cur(a), wires.cur(b)
            oa, ob = wires.advance(a), wires.advance(b)
            tensors.append(([oa, ob, ia, ib], [2, 2, 2, 2], fsim.reshape(-1)))
    for q in range(n):
        if present[q]:
            bit = 0 if bitstring is None else int(bitstring[q])
            cap = np.array([1, 0] if bit == 0 else [0, 1], dtype=np.complex128)
            tensors.append(([wires.cur(q)], [2], cap))
    return Network([(l, s, d.astype(dtype)) for l, s, d in tensors])


def haar_unitary(d: int, rng: np.random.Generator) -> np.ndarray:
    """Haar-random d x d unitary: QR of a complex Gaussian matrix with the
    phases of R's diagonal folded back into Q (Mezzadri, 2007)."""
    z = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / math.sqrt(2.0)
    q, r = np.linalg.qr(z)
    ph = np.diag(r) / np.abs(np.diag(r))
    return q * ph


def qudit_circuit_network(rows: int, cols: int, layers: int, d: int = 3, seed: int = 0,
                          dtype=np.complex64) -> Network:
    """<0...0| C |0...0> of a qudit circuit (local dimension d): per layer a
    seeded Haar-random d x d unitary on every site, then a Haar-random
    d^2 x d^2 unitary on one of the four alternating nearest-neighbour
    coupler patterns."""
    rng = np.random.default_rng(seed)
    n = rows * cols
    pats = couplers(rows, cols)
    wires = _Wires(n)
    e0 = np.zeros(d, dtype=np.complex128)
    e0[0] = 1
    tensors: List[Tuple[List[str], List[int], np.ndarray]] = []
    for q in range(n):
        tensors.append(([wires.cur(q)], [d], e0.copy()))
    for layer in range(layers):
        for q in range(n):
            i = wires.cur(q)
            o = wires.advance(q)
            tensors.append(([o, i], [d, d], haar_unitary(d, rng).reshape(-1)))
        for a, b in pats["ABCD"[layer % 4]]:
            ia, ib = wires.cur(a), wires.cur(b)
            oa, ob = wires.advance(a), wires.advance(b)
            tensors.append(([oa, ob, ia, ib], [d, d, d, d], haar_unitary(d * d, rng).reshape(-1)))
    for q in range(n):
        tensors.append(([wires.cur(q)], [d], e0.copy()))
    return Network([(l, s, x.astype(dtype)) for l, s, x in tensors])


def parameterised_layers_network(rows: int, cols: int, layers: int,
                                 thetas: np.ndarray, phis: np.ndarray,
                                 dtype=np.complex64) -> Tuple[Network, List[Tuple[int, str]]]:
    """|psi> = prod_layers [CZ(alternating couplers) RZ(phi) RX(theta)] |0...0>.

    Returns the open-output network and, for every parameterised gate, its
    (tensor position, parameter kind) so that callers can rebuild gates."""
    n = rows * cols
    pats = couplers(rows, cols)
    wires = _Wires(n)
    tensors: List[Tuple[List[str], List[int], np.ndarray]] = []
    where: List[Tuple[int, str]] = []
    zero = np.array([1, 0], dtype=np.complex128)
    for q in range(n):
        tensors.append(([wires.cur(q)], [2], zero.copy()))
    cz = gate_cz().reshape(-1)
    for layer in range(layers):
        for q in range(n):
            i = wires.cur(q)
            o = wires.advance(q)
            where.append((len(tensors), "rx"))
            tensors.append(([o, i], [2, 2], gate_rx(thetas[layer, q]).reshape(-1)))
            i = wires.cur(q)
            o = wires.advance(q)
            where.append((len(tensors), "rz"))
            tensors.append(([o, i], [2, 2], gate_rz(phis[layer, q]).reshape(-1)))
        for a, b in pats["ABCD"[layer % 4]]:
            ia, ib = wires.cur(a), wires.cur(b)
            oa, ob = wires.advance(a), wires.advance(b)
            tensors.append(([oa, ob, ia, ib], [2, 2, 2, 2], cz.copy()))
    net = Network([(l, s, d.astype(dtype)) for l, s, d in tensors],
                  open_labels=[wires.cur(q) for q in range(n)])
    return net, where


# ---------------------------------------------------------------------------
# Greedy path
# ---------------------------------------------------------------------------


def _size(labels, dims) -> float:
    s = 1.0
    for x in labels:
        s *= dims[x]
    return s


def greedy_path(net: Network, seed: int = 0, sliced: Sequence[str] = (),
                temperature: float = 0.0, score: str = "size") -> List[Tuple[int, int]]:
    """Seeded greedy path.

    Repeatedly contracts the connected pair of nodes with the lowest score:
    score "size" is log2 of the result's size (the min-intermediate-size
    heuristic); score "gain" is size(result) - size(a) - size(b), the
    memory a contraction adds (as in opt_einsum's greedy), signed-log2
    compressed. Ties -- and with temperature > 0 near-ties, through Gumbel
    noise -temperature * log(-log u) -- are broken by a seeded random key.
    Disconnected remainders are then contracted smallest first. Sliced
    indices count as dimension 1."""
    rng = np.random.default_rng(seed)
    score_kind = score
    dims = dict(net.index_dims())
    for x in sliced:
        dims[x] = 1
    nodes: Dict[int, List[str]] = {}
    where: Dict[str, List[int]] = {}
    for i, (lab, _, _) in enumerate(net.tensors):
        nodes[i] = list(lab)
        for x in lab:
            where.setdefault(x, []).append(i)
    next_id = len(net.tensors)
    open_set = set(net.open_labels)

    def out_labels(a: int, b: int) -> List[str]:
        la, lb = nodes[a], nodes[b]
        sb = set(lb)
        sa = set(la)
        res = [x for x in la if x not in sb or x in open_set]
        res += [x for x in lb if x not in sa]
        return res

    def score(a: int, b: int) -> float:
        if score_kind == "gain":
            g = (_size(out_labels(a, b), dims) - _size(nodes[a], dims) - _size(nodes[b], dims))
            s = math.copysign(math.log2(abs(g) + 1.0), g)
        else:
            s = math.log2(max(_size(out_labels(a, b), dims), 1.0))
        noise = float(rng.random())
        if temperature > 0:
            s -= temperature * math.log(-math.log(max(noise, 1e-300)))
            return s
        return s + 1e-6 * noise

    heap: List[Tuple[float, int, int]] = []
    seen = set()
    for x, ids in where.items():
        if len(ids) == 2:
            a, b = sorted(ids)
            if (a, b) not in seen:
                seen.add((a, b))
                heapq.heappush(heap, (score(a, b), a, b))
    path: List[Tuple[int, int]] = []
    while heap:
        _, a, b = heapq.heappop(heap)
        if a not in nodes or b not in nodes:
            continue
        lab = out_labels(a, b)
        for x in nodes[a] + nodes[b]:
            ids = where.get(x, [])
            where[x] = [i for i in ids if i not in (a, b)]
        del nodes[a]
        del nodes[b]
        c = next_id
        next_id += 1
        nodes[c] = lab
        path.append((a, b))
        for x in lab:
            where.setdefault(x, []).append(c)
        nbrs = set()
        for x in lab:
            for i in where[x]:
                if i != c:
                    nbrs.add(i)
        for i in nbrs:
            heapq.heappush(heap, (score(min(i, c), max(i, c)), min(i, c), max(i, c)))
    # Disconnected components (scalars or outer products).
    rest = sorted(nodes.keys(), key=lambda i: (_size(nodes[i], dims), i))
    while len(rest) > 1:
        a, b = rest[0], rest[1]
        lab = nodes[a] + nodes[b]
        del nodes[a]
        del nodes[b]
        c = next_id
        next_id += 1
        nodes[c] = lab
        path.append((a, b))
        rest = sorted(nodes.keys(), key=lambda i: (_size(nodes[i], dims), i))
    return path


def find_path(net: Network, restarts: int = 16, seed: int = 0,
              sliced: Sequence[str] = ()) -> List[Tuple[int, int]]:
    """Best of `restarts` seeded greedy runs (both scores, with and without
    noise) by total flops, then by the largest intermediate."""
    best = None
    for r in range(restarts):
        for score, temp in (("gain", 0.0), ("gain", 0.3), ("size", 0.0)):
            p = greedy_path(net, seed=seed * 1000 + r, sliced=sliced, temperature=temp, score=score)
            flops, big = path_cost(net, p, sliced)
            if best is None or (flops, big) < best[0]:
                best = ((flops, big), p)
    return best[1]


def best_gain_path(net: Network, restarts: int) -> List[Tuple[int, int]]:
    """Best (total flops, then largest intermediate) of the "gain"-score
    greedy runs with seeds 0 .. restarts-1, each without and with Gumbel
    noise at temperature 0.2: the path of the sliced benchmark circuits."""
    best = None
    for s in range(restarts):
        for temp in (0.0, 0.2):
            p = greedy_path(net, seed=s, temperature=temp, score="gain")
            f, big = path_cost(net, p)
            if best is None or (f, big) < best[0]:
                best = ((f, big), p)
    return best[1]


def path_cost(net: Network, path: Sequence[Tuple[int, int]], sliced: Sequence[str] = ()):
    """(total flops as PathInfo counts them, log2 of the largest intermediate)
    with the sliced indices at dimension 1 (PathInfo.hpp:157-224)."""
    dims = dict(net.index_dims())
    for x in sliced:
        dims[x] = 1
    open_set = set(net.open_labels)
    nodes = {i: list(l) for i, (l, _, _) in enumerate(net.tensors)}
    nid = len(nodes)
    flops = 0.0
    biggest = 0.0
    for a, b in path:
        la, lb = nodes.pop(a), nodes.pop(b)
        sa, sb = set(la), set(lb)
        common = [x for x in la if x in sb and x not in open_set]
        out = [x for x in la if x not in sb or x in open_set] + [x for x in lb if x not in sa]
        size = _size(out, dims)
        flops += size * 2 * _size(common, dims)
        biggest = max(biggest, size)
        nodes[nid] = out
        nid += 1
    return flops, math.log2(max(biggest, 1.0))


def _largest_intermediates(net: Network, path, sliced, top: int = 4):
    """Label sets of the `top` largest intermediates of the path."""
    dims = dict(net.index_dims())
    for x in sliced:
        dims[x] = 1
    open_set = set(net.open_labels)
    nodes = {i: list(l) for i, (l, _, _) in enumerate(net.tensors)}
    nid = len(nodes)
    sizes = []
    for a, b in path:
        la, lb = nodes.pop(a), nodes.pop(b)
        sa, sb = set(la), set(lb)
        out = [x for x in la if x not in sb or x in open_set] + [x for x in lb if x not in sa]
        sizes.append((_size(out, dims), out))
        nodes[nid] = out
        nid += 1
    sizes.sort(key=lambda t: -t[0])
    return [lab for _, lab in sizes[:top]]


def choose_slices(net: Network, path: Sequence[Tuple[int, int]], count: int,
                  seed: int = 0) -> List[str]:
    """Greedy slicer: `count` times, slice the bond that most reduces
    (largest intermediate, total flops); seeded tie-break. Only bonds of the
    largest intermediates can shrink the largest intermediate, so the
    candidates are the labels of the few largest ones. Open and
    already-sliced indices are excluded."""
    rng = np.random.default_rng(seed)
    dims = net.index_dims()
    open_set = set(net.open_labels)
    chosen: List[str] = []
    for _ in range(count):
        cands = set()
        for lab in _largest_intermediates(net, path, chosen):
            cands.update(x for x in lab if dims[x] > 1 and x not in open_set and x not in chosen)
        if not cands:
            cands = {x for x, d in dims.items() if d > 1 and x not in open_set and x not in chosen}
        order = sorted(cands)
        rng.shuffle(order)
        best = None
        for x in order:
            flops, big = path_cost(net, path, chosen + [x])
            key = (big, flops)
            if best is None or key < best[0]:
                best = (key, x)
        chosen.append(best[1])
    return chosen
