"""CPU oracle: a numpy restatement of Jet's contraction hot path.

TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg may import this module, and only as the checker or the timed
CPU baseline -- never as the thing measured or shipped. The product path
(jet_gb300) never imports it and fails loudly when its CUDA library is missing.

Parity is pinned two ways (tests/test_oracle.py):
  * against the golden vectors of the reference's own tests
    (test/Test_Permuter.cpp, Test_Tensor.cpp, Test_TensorNetwork.cpp,
    Test_PathInfo.cpp, python/tests/test_task_based_contractor.py), committed
    under tests/golden/;
  * against the reference headers compiled in this container
    (oracle/ref_build -> oracle/_ref/libjetref.so) on seeded random inputs.

Every function cites the reference file:line it restates (paths relative to
the reference project root).
"""
from __future__ import annotations

import dataclasses
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

# ---------------------------------------------------------------------------
# Label algebra: include/jet/Utilities.hpp
# ---------------------------------------------------------------------------

_ALPHABET = [chr(c) for c in range(ord("a"), ord("z") + 1)] + [
    chr(c) for c in range(ord("A"), ord("Z") + 1)
]


def generate_string_index(i: int) -> str:
    """Utilities.hpp:86-97: a..z A..Z, then a0..Z0, a1.. ."""
    div = i // len(_ALPHABET)
    return _ALPHABET[i % len(_ALPHABET)] + ("" if div == 0 else str(div - 1))


def vector_intersection(v1: Sequence[str], v2: Sequence[str]) -> List[str]:
    """Utilities.hpp:316-327: elements of v1 also in v2, in v1's order."""
    s2 = set(v2)
    return [x for x in v1 if x in s2]


def vector_union(v1: Sequence[str], v2: Sequence[str]) -> List[str]:
    """Utilities.hpp:337-348: v1 followed by the elements of v2 not in v1."""
    s1 = set(v1)
    return list(v1) + [x for x in v2 if x not in s1]


def vector_subtraction(v1: Sequence[str], v2: Sequence[str]) -> List[str]:
    """Utilities.hpp:358-369: elements of v1 not in v2, in v1's order."""
    s2 = set(v2)
    return [x for x in v1 if x not in s2]


def vector_disjunctive_union(v1: Sequence[str], v2: Sequence[str]) -> List[str]:
    """Utilities.hpp:379-384: union minus intersection."""
    return vector_subtraction(vector_union(v1, v2), vector_intersection(v1, v2))


def shape_to_size(shape: Sequence[int]) -> int:
    """Utilities.hpp:438-445."""
    n = 1
    for d in shape:
        n *= int(d)
    return n


def unravel_index(index: int, shape: Sequence[int]) -> List[int]:
    """Utilities.hpp:463-475 (row-major; raises if the index does not fit)."""
    if shape_to_size(shape) <= index:
        raise ValueError("Linear index does not fit in the shape.")
    out = [0] * len(shape)
    for i in range(len(shape) - 1, -1, -1):
        out[i] = index % shape[i]
        index //= shape[i]
    return out


# ---------------------------------------------------------------------------
# Tensor: include/jet/Tensor.hpp
# ---------------------------------------------------------------------------


@dataclasses.dataclass
class OTensor:
    """Row-major labelled complex tensor (Tensor.hpp:30-776)."""

    indices: List[str]
    shape: List[int]
    data: np.ndarray  # flat, row-major

    @staticmethod
    def make(indices, shape, data=None, dtype=np.complex128) -> "OTensor":
        n = shape_to_size(shape)
        if data is None:
            arr = np.zeros(n, dtype=dtype)
        else:
            arr = np.asarray(data, dtype=dtype).reshape(-1).copy()
            assert arr.size == n
        return OTensor(list(indices), [int(s) for s in shape], arr)

    @property
    def size(self) -> int:
        return int(self.data.size)

    def index_to_dimension(self) -> Dict[str, int]:
        return dict(zip(self.indices, self.shape))

    def nd(self) -> np.ndarray:
        return self.data.reshape(self.shape) if self.shape else self.data.reshape(())


def transpose(a: OTensor, new_indices: Sequence[str]) -> OTensor:
    """Tensor.hpp:578-612. The permuter backends (QFlex.hpp, Default.hpp)
    compute the exact index permutation; numpy's transpose does the same copy.

    Note: Default.hpp:85-86 stores output positions in `unsigned short`, so
    the reference's non-power-of-2 path truncates positions >= 65536; the
    oracle gives the mathematically exact permutation (what QFlex and the
    Default permuter agree on below that size)."""
    new_indices = list(new_indices)
    if list(a.indices) == new_indices:
        return OTensor(list(a.indices), list(a.shape), a.data.copy())
    if len(a.indices) == 0:
        raise ValueError("Number of indices cannot be zero.")
    pos = {lab: i for i, lab in enumerate(a.indices)}
    perm = [pos[lab] for lab in new_indices]
    out = np.ascontiguousarray(np.transpose(a.nd(), perm)).reshape(-1)
    return OTensor(new_indices, [a.shape[p] for p in perm], out)


def contract_tensors(a: OTensor, b: OTensor, dtype=None) -> OTensor:
    """Tensor.hpp:708-752 + TensorHelpers.hpp:128-168.

    left = A\\B (A order), right = B\\A (B order), common = A∩B (A order);
    A is transposed to left++common, B to common++right, then one
    GEMM/GEMV/dot with alpha=1, beta=0. `dtype` selects the arithmetic type
    (complex128 by default: the FP64 oracle)."""
    dt = np.dtype(dtype) if dtype is not None else np.result_type(a.data, b.data)
    left = vector_subtraction(a.indices, b.indices)
    right = vector_subtraction(b.indices, a.indices)
    common = vector_intersection(a.indices, b.indices)
    a_dims, b_dims = a.index_to_dimension(), b.index_to_dimension()
    m = shape_to_size([a_dims[x] for x in left])
    n = shape_to_size([b_dims[x] for x in right])
    k = shape_to_size([a_dims[x] for x in common])
    at = transpose(a, vector_union(left, common))
    bt = transpose(b, vector_union(common, right))
    am = at.data.astype(dt, copy=False).reshape(m, k)
    bm = bt.data.astype(dt, copy=False).reshape(k, n)
    c = (am @ bm).reshape(-1)
    c_indices = vector_union(left, right)
    c_shape = [a_dims[x] for x in left] + [b_dims[x] for x in right]
    return OTensor(c_indices, c_shape, c)


def slice_index(t: OTensor, index: str, value: int) -> OTensor:
    """Tensor.hpp:493-526: move `index` to the front, keep block `value`."""
    order = [index] + [x for x in t.indices if x != index]
    tt = transpose(t, order)
    rest = tt.shape[1:]
    block = shape_to_size(rest)
    return OTensor(order[1:], list(rest), tt.data[block * value: block * (value + 1)].copy())


def reshape(t: OTensor, new_shape: Sequence[int]) -> OTensor:
    """Tensor.hpp:546-558: same data, default labels ?a, ?b, ..."""
    if t.size != shape_to_size(new_shape):
        raise ValueError("Size is inconsistent between tensors.")
    labels = ["?" + generate_string_index(i) for i in range(len(new_shape))]
    return OTensor(labels, list(new_shape), t.data.copy())


def conj(t: OTensor) -> OTensor:
    """Tensor.hpp:668-675."""
    return OTensor(list(t.indices), list(t.shape), np.conj(t.data))


def _is_zero_sentinel(t: OTensor) -> bool:
    # Tensor.hpp:415-424 compares against a default Tensor: no indices, no
    # shape, one zero datum.
    return not t.indices and not t.shape and t.size == 1 and t.data[0] == 0


def add_tensors(a: OTensor, b: OTensor) -> OTensor:
    """Tensor.hpp:412-454: zero-sentinel shortcut, B transposed to A's order."""
    if _is_zero_sentinel(a):
        return OTensor(list(b.indices), list(b.shape), b.data.copy())
    if _is_zero_sentinel(b):
        return OTensor(list(a.indices), list(a.shape), a.data.copy())
    if vector_disjunctive_union(a.indices, b.indices):
        raise ValueError("Tensor addition with disjoint indices is not supported.")
    bt = transpose(b, a.indices)
    return OTensor(list(a.indices), list(a.shape), a.data + bt.data)


# ---------------------------------------------------------------------------
# TensorNetwork: include/jet/TensorNetwork.hpp
# ---------------------------------------------------------------------------


@dataclasses.dataclass
class ONode:
    id: int
    name: str
    indices: List[str]
    tags: List[str]
    contracted: bool
    tensor: OTensor


def _node_name(indices: Sequence[str]) -> str:
    """TensorNetwork.hpp:548-552 (DeriveNodeName_)."""
    return "".join(indices) if indices else "_"


class OTensorNetwork:
    """TensorNetwork.hpp:58-556 (explicit-path subset)."""

    def __init__(self):
        self.nodes: List[ONode] = []
        # index -> [dim, node_ids]
        self.edges: Dict[str, List] = {}

    def add_tensor(self, t: OTensor, tags: Sequence[str] = ()) -> int:
        """TensorNetwork.hpp:167-184; edges skip dims < 2 (:356-358)."""
        nid = len(self.nodes)
        self.nodes.append(ONode(nid, _node_name(t.indices), list(t.indices), list(tags), False, t))
        for lab, dim in zip(t.indices, t.shape):
            if dim < 2:
                continue
            if lab in self.edges:
                self.edges[lab][1].append(nid)
            else:
                self.edges[lab] = [dim, [nid]]
        return nid

    def slice_indices(self, indices: Sequence[str], value: int) -> None:
        """TensorNetwork.hpp:210-284: row-major unravel of `value` over the
        sliced dims, per node slice (+ transpose back + reshape), annotate
        node labels as `label(v)`, drop the sliced edges."""
        node_to_idx: Dict[int, List[int]] = {}
        sizes = []
        for i, lab in enumerate(indices):
            if lab not in self.edges:
                raise ValueError("Sliced index does not exist.")
            dim, ids = self.edges[lab]
            sizes.append(dim)
            for nid in ids:
                node_to_idx.setdefault(nid, []).append(i)
        values = unravel_index(value, sizes)
        for nid, idxs in node_to_idx.items():
            node = self.nodes[nid]
            for i in idxs:
                lab, v = indices[i], values[i]
                t = node.tensor
                keep = [x for x in t.indices if x != lab]
                keep_shape = [d for x, d in zip(t.indices, t.shape) if x != lab]
                t = slice_index(t, lab, v)
                if t.indices != keep:
                    t = transpose(t, keep)
                node.tensor = OTensor(keep, keep_shape, t.data)
                node.indices = [x + f"({v})" if x == lab else x for x in node.indices]
            node.name = _node_name(node.indices)
        for lab in indices:
            self.edges.pop(lab, None)

    def contract(self, path: Sequence[Tuple[int, int]], dtype=None,
                 release: bool = False) -> OTensor:
        """TensorNetwork.hpp:301-328 -> ContractNodes_ :394-421.

        release=True drops each node's tensor once it has been contracted
        (the reference keeps every intermediate in nodes_); the arithmetic
        and the result are the same, only the memory held differs, which
        lets large networks (53-qubit slices, m12) run in host memory."""
        if not self.nodes:
            raise ValueError("An empty tensor network cannot be contracted.")
        for a, b in path:
            if a >= len(self.nodes):
                raise ValueError("Node ID 1 in contraction pair is invalid.")
            if b >= len(self.nodes):
                raise ValueError("Node ID 2 in contraction pair is invalid.")
            n1, n2 = self.nodes[a], self.nodes[b]
            t3 = contract_tensors(n1.tensor, n2.tensor, dtype=dtype)
            n1.contracted = n2.contracted = True
            if release:
                n1.tensor = OTensor(list(n1.tensor.indices), list(n1.tensor.shape),
                                    np.zeros(0, dtype=t3.data.dtype))
                n2.tensor = OTensor(list(n2.tensor.indices), list(n2.tensor.shape),
                                    np.zeros(0, dtype=t3.data.dtype))
            idx3 = vector_disjunctive_union(n1.indices, n2.indices)
            n3 = ONode(len(self.nodes), _node_name(idx3), idx3,
                       vector_union(n1.tags, n2.tags), False, t3)
            self.nodes.append(n3)
            # UpdateIndexMapAfterContraction_ :431-453
            for lab in n3.indices:
                if lab in self.edges:
                    self.edges[lab][1] = [n3.id if x in (n1.id, n2.id) else x
                                          for x in self.edges[lab][1]]
            for lab in vector_intersection(n1.tensor.indices, n2.tensor.indices):
                self.edges.pop(lab, None)
        return self.nodes[-1].tensor


# ---------------------------------------------------------------------------
# PathInfo: include/jet/PathInfo.hpp
# ---------------------------------------------------------------------------


@dataclasses.dataclass
class OStep:
    id: int
    parent: Optional[int]
    children: Tuple[Optional[int], Optional[int]]
    name: str
    node_indices: List[str]
    tensor_indices: List[str]
    tags: List[str]
    contracted_indices: List[str]


class OPathInfo:
    """PathInfo.hpp:52-298."""

    def __init__(self, tn: OTensorNetwork, path: Sequence[Tuple[int, int]]):
        self.path = [tuple(p) for p in path]
        self.steps: List[OStep] = []
        for node in tn.nodes:
            self.steps.append(OStep(node.id, None, (None, None), node.name, list(node.indices),
                                    list(node.tensor.indices), list(node.tags), []))
        self.num_leaves = len(tn.nodes)
        self.index_sizes = {lab: e[0] for lab, e in tn.edges.items()}
        for a, b in self.path:
            if a >= len(self.steps):
                raise ValueError("Node ID 1 in contraction path pair is invalid.")
            if b >= len(self.steps):
                raise ValueError("Node ID 2 in contraction path pair is invalid.")
            self._contract_steps(a, b)

    def _contract_steps(self, a: int, b: int) -> None:
        """PathInfo.hpp:262-297."""
        s1, s2 = self.steps[a], self.steps[b]
        sid = len(self.steps)
        contracted = vector_intersection(s1.tensor_indices, s2.tensor_indices)
        node_idx = vector_subtraction(s1.node_indices + s2.node_indices, contracted)
        s1.parent = s2.parent = sid
        self.steps.append(OStep(sid, None, (a, b), _node_name(node_idx), node_idx,
                                vector_disjunctive_union(s1.tensor_indices, s2.tensor_indices),
                                vector_union(s1.tags, s2.tags), contracted))

    def step_flops(self, i: int) -> float:
        """PathInfo.hpp:157-183: size(out) * 2 * prod(contracted dims)."""
        if i < self.num_leaves:
            return 0.0
        st = self.steps[i]
        muls = 1.0
        for x in st.contracted_indices:
            muls *= self.index_sizes.get(x, 1)
        size = 1.0
        for x in st.tensor_indices:
            size *= self.index_sizes.get(x, 1)
        return size * (muls + muls)

    def total_flops(self) -> float:
        return sum(self.step_flops(i) for i in range(self.num_leaves, len(self.steps)))

    def step_memory(self, i: int) -> float:
        """PathInfo.hpp:211-224."""
        m = 1.0
        for x in self.steps[i].tensor_indices:
            m *= self.index_sizes.get(x, 1)
        return m

    def total_memory(self) -> float:
        return sum(self.step_memory(i) for i in range(len(self.steps)))


def task_name(step: OStep) -> str:
    """TaskBasedContractor.hpp:367-370: "<step id>:<step name>"."""
    return f"{step.id}:{step.name}"
