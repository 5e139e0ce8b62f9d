"""Differentiable network contraction with a hand-written adjoint.

`contract_network(leaves, labels, path)` contracts a tensor network on the
GPU along `path` (the reference's node-id convention, TensorNetwork.hpp:
301-328) and returns the result as a torch tensor that carries gradients back
to every leaf.

Each pairwise step is the reference's Tensor::ContractTensors
(Tensor.hpp:708-752): labels left = A\\B, right = B\\A, common = A∩B (A
order), C[left ++ right] = sum_common A B. Its adjoint is two conjugate
contractions, replayed along the path in reverse:

    grad_A[left, common] = sum_right grad_C[left, right] conj(B[common, right])
    grad_B[common, right] = sum_left conj(A[left, common]) grad_C[left, right]

(PyTorch's convention for complex gradients: grad = dL/d(conj z)), each
followed by a transpose back to the operand's own label order. The reverse
sweep carries the conjugated gradients H = conj(grad) instead:

    H_A[left, common] = sum_right H_C[left, right] B[common, right]
    H_B[common, right] = sum_left A[left, common] H_C[left, right]

are plain contractions of the forward values (term by term the conjugates
of the products above), and only the leaves' gradients are conjugated at the
end, instead of every operand of every step. Operands whose subtree
holds no leaf that needs a gradient get none. The forward keeps only the
leaves: backward recomputes the intermediates (checkpointing), so memory
stays at one forward's worth plus the gradients. Every contraction,
conjugation and transpose runs in libjetgpu.so (jetgpu_contract,
jetgpu_conj, jetgpu_permute).

Sliced networks (`sliced` labels, TensorNetwork::SliceIndices semantics,
TensorNetwork.hpp:210-284): the value is the sum over every slice value of
the network with those bonds fixed. Forward and backward both run slice by
slice, recomputing each slice's intermediates from the leaves, so the memory
held is one slice's forward and gradients, not the whole network's. A
slice's leaf gradients are added into the full leaves' gradients at that
slice's positions (jetgpu_slice_scatter_add, the adjoint of the device
SliceIndex gather). `memory_budget` (bytes) picks the sliced bonds: the
greedy slicer's bonds are added until one slice's checkpointed forward plus
the gradients fits.
"""
from __future__ import annotations

import dataclasses
from typing import List, Sequence, Tuple

import numpy as np
import torch

from . import capi, grouped


@dataclasses.dataclass
class _Step:
    a: int
    b: int
    out_labels: List[str]
    a_perm: List[int]
    b_perm: List[int]
    m: int
    n: int
    k: int


class ContractionPlan:
    """Label bookkeeping of a path: per step, the operand orders and the
    product dimensions ContractTensors derives (left, right, common)."""

    def __init__(self, labels: Sequence[Sequence[str]], shapes: Sequence[Sequence[int]],
                 path: Sequence[Tuple[int, int]]):
        self.labels: List[List[str]] = [list(l) for l in labels]
        self.shapes: List[List[int]] = [list(s) for s in shapes]
        self.num_leaves = len(self.labels)
        self.dims = {}
        for lab, sh in zip(self.labels, self.shapes):
            for x, d in zip(lab, sh):
                self.dims[x] = int(d)
        self.steps: List[_Step] = []
        # Grouped launches of tiny steps (jet_gb300.grouped), per (dtype,
        # device): on by default; off runs every step as its own launch.
        self.grouping = True
        self._grouped = {}
        for a, b in path:
            la, lb = self.labels[a], self.labels[b]
            sb, sa = set(lb), set(la)
            left = [x for x in la if x not in sb]
            right = [x for x in lb if x not in sa]
            common = [x for x in la if x in sb]
            step = _Step(a, b, left + right, [la.index(x) for x in left + common],
                         [lb.index(x) for x in common + right], self._prod(left),
                         self._prod(right), self._prod(common))
            self.steps.append(step)
            self.labels.append(step.out_labels)
            self.shapes.append([self.dims[x] for x in step.out_labels])

    def _prod(self, labels) -> int:
        p = 1
        for x in labels:
            p *= self.dims[x]
        return p

    @property
    def out_labels(self) -> List[str]:
        return self.labels[-1]

    @property
    def out_shape(self) -> List[int]:
        return self.shapes[-1]


def _contract(a, a_labels, a_shape, b, b_labels, b_shape, precision, out=None):
    """ContractTensors on device tensors; returns (C, C labels, C shape)."""
    sb, sa = set(b_labels), set(a_labels)
    left = [x for x in a_labels if x not in sb]
    right = [x for x in b_labels if x not in sa]
    common = [x for x in a_labels if x in sb]
    dims = dict(zip(a_labels, a_shape))
    dims.update(zip(b_labels, b_shape))
    m = n = k = 1
    for x in left:
        m *= dims[x]
    for x in right:
        n *= dims[x]
    for x in common:
        k *= dims[x]
    out = capi.contract(a, list(a_shape), [a_labels.index(x) for x in left + common], b,
                        list(b_shape), [b_labels.index(x) for x in common + right], m, n, k,
                        precision=precision, out=out)
    return out[: m * n], left + right, [dims[x] for x in left + right]


def _out_labels(a_labels, b_labels):
    sa, sb = set(a_labels), set(b_labels)
    return [x for x in a_labels if x not in sb] + [x for x in b_labels if x not in sa]


def _to_order(x, labels, shape, target, out=None):
    if labels == target:
        return x
    return capi.permute(x, list(shape), [labels.index(t) for t in target], out=out)


def _operand_h(x, x_labels, x_shape, y, y_labels, y_shape, target, precision, slot):
    """The contraction of x and y in `target`'s label order, written into
    `slot` (a leaf's place in one flat buffer) when given. Of contract(x, y)
    and contract(y, x), one whose labels come out in that order needs no
    transpose."""
    for p, lp, sp, q, lq, sq in ((x, x_labels, x_shape, y, y_labels, y_shape),
                                 (y, y_labels, y_shape, x, x_labels, x_shape)):
        if _out_labels(lp, lq) == target:
            return _contract(p, lp, sp, q, lq, sq, precision, out=slot)[0]
    h, lh, sh = _contract(x, x_labels, x_shape, y, y_labels, y_shape, precision)
    return _to_order(h, lh, sh, target, out=slot)


def _grouped_for(plan: ContractionPlan, like, precision: int):
    """The plan's grouped evaluation for tensors like `like`, or None (not
    in the plain forms, grouping off, the plan unsuited, or first asked
    inside a CUDA graph capture, where it cannot be built)."""
    if (not plan.grouping or precision not in (capi.PREC_FP32, capi.PREC_AUTO)
            or like.dtype not in (torch.complex64, torch.complex128)):
        return None
    key = (like.dtype, str(like.device))
    if key in plan._grouped:
        return plan._grouped[key]
    if grouped.capturing(like.device):
        return None
    try:
        g = grouped.Grouped(plan, like.dtype, like.device)
    except grouped.NoGroup:
        g = None
    plan._grouped[key] = g
    return g


def _forward(plan: ContractionPlan, leaves, precision: int, keep: bool):
    g = _grouped_for(plan, leaves[0], precision)
    if g is not None:
        vals = g.run_forward(leaves, precision)
        if not keep:  # the arena is overwritten by the next evaluation
            vals[-1] = vals[-1].clone()
        return vals
    vals = list(leaves)
    for st in plan.steps:
        out = capi.contract(vals[st.a], plan.shapes[st.a], st.a_perm, vals[st.b],
                            plan.shapes[st.b], st.b_perm, st.m, st.n, st.k,
                            precision=precision)[: st.m * st.n]
        vals.append(out)
        if not keep:
            # Release operands that are intermediates (each is used once).
            for i in (st.a, st.b):
                if i >= plan.num_leaves:
                    vals[i] = None
    return vals


def _needs(plan: ContractionPlan, leaf_needs) -> List[bool]:
    """Per node of the path: whether a leaf of its subtree needs a gradient."""
    need = [bool(x) for x in leaf_needs]
    for st in plan.steps:
        need.append(need[st.a] or need[st.b])
    return need


def _backward_conj(plan: ContractionPlan, vals, h_out, precision: int, need, slots=None):
    """The reverse sweep over conjugated gradients: H of every leaf (None
    where no gradient is needed), from H of the result. A leaf's H comes in
    the leaf's label order (into `slots[leaf]` when given: one contribution
    per leaf, as the path consumes each node once); an intermediate's H stays
    in the label order its contraction produced, since it is only read again
    as an operand of contractions, which take any axis order."""
    slots = slots or {}
    hs = [None] * len(vals)  # (tensor, labels, shape)
    hs[-1] = (h_out, plan.labels[-1], plan.shapes[-1])
    for idx in range(len(plan.steps) - 1, -1, -1):
        st = plan.steps[idx]
        c_id = plan.num_leaves + idx
        if hs[c_id] is None:
            continue
        hc, lc, sc = hs[c_id]
        la, lb = plan.labels[st.a], plan.labels[st.b]
        sa, sb = plan.shapes[st.a], plan.shapes[st.b]
        # H_A = contract(H_C, B) and H_B = contract(A, H_C).
        for i, x, lx, sx, y, ly, sy in ((st.a, hc, lc, sc, vals[st.b], lb, sb),
                                        (st.b, vals[st.a], la, sa, hc, lc, sc)):
            if not need[i]:
                continue
            first = hs[i] is None
            if i < plan.num_leaves:
                target = plan.labels[i]
                h = _operand_h(x, lx, sx, y, ly, sy, target, precision,
                               slots.get(i) if first else None)
                lh, sh = target, plan.shapes[i]
            else:
                h, lh, sh = _contract(x, lx, sx, y, ly, sy, precision)
            if first:
                hs[i] = (h, lh, sh)
                continue
            prev, lp, sp = hs[i]
            h = capi.add(prev, _to_order(h, lh, sh, lp))
            if i in slots:
                slots[i].copy_(h)
                h = slots[i]
            hs[i] = (h, lp, sp)
        hs[c_id] = None
        vals[c_id] = None
    return [None if h is None else h[0] for h in hs[: plan.num_leaves]]


def _backward(plan: ContractionPlan, vals, grad_out, precision: int, leaf_needs=None):
    """Leaf gradients (None where `leaf_needs` is false) from the result's.
    The leaves' conjugated gradients are written into one flat buffer and
    conjugated by one launch."""
    if leaf_needs is None:
        leaf_needs = [True] * plan.num_leaves
    g = _grouped_for(plan, grad_out, precision)
    if g is not None:  # `vals` are then the values run_forward left in its arena
        try:
            return g.run_backward(grad_out, _needs(plan, leaf_needs), precision)
        except grouped.NoGroup:
            pass
    sizes = [int(np.prod(plan.shapes[i])) if len(plan.shapes[i]) else 1
             for i in range(plan.num_leaves)]
    at, total = {}, 0
    for i in range(plan.num_leaves):
        if leaf_needs[i]:
            at[i] = total
            total += sizes[i]
    flat = torch.empty(max(total, 1), dtype=grad_out.dtype, device=grad_out.device)
    slots = {i: flat[o: o + sizes[i]] for i, o in at.items()}
    hs = _backward_conj(plan, vals, capi.conj(grad_out), precision, _needs(plan, leaf_needs),
                        slots)
    grads = capi.conj(flat)
    return [None if h is None else grads[at[i]: at[i] + sizes[i]] for i, h in enumerate(hs)]


class SlicedPlan:
    """A path over the leaves with the `sliced` bonds fixed: per leaf the
    sliced axes (jetgpu_slice_gather's value strides: row-major over the
    sliced bonds, as SliceIndices unravels a slice value) and the plan of the
    sliced network (each leaf keeps its other axes in their order)."""

    def __init__(self, plan: ContractionPlan, path: Sequence[Tuple[int, int]],
                 sliced: Sequence[str]):
        self.full = plan
        self.sliced = list(sliced)
        dims = [plan.dims[x] for x in self.sliced]
        strides = [1] * len(dims)
        for j in range(len(dims) - 2, -1, -1):
            strides[j] = strides[j + 1] * dims[j + 1]
        self.num_slices = 1
        for d in dims:
            self.num_slices *= d
        pos = {x: j for j, x in enumerate(self.sliced)}
        self.leaf_axes: List[List[int]] = []
        self.leaf_strides: List[List[int]] = []
        labels, shapes = [], []
        for i in range(plan.num_leaves):
            lab, sh = plan.labels[i], plan.shapes[i]
            axes = [a for a, x in enumerate(lab) if x in pos]
            self.leaf_axes.append(axes)
            self.leaf_strides.append([strides[pos[lab[a]]] for a in axes])
            labels.append([x for x in lab if x not in pos])
            shapes.append([d for x, d in zip(lab, sh) if x not in pos])
        self.sub = ContractionPlan(labels, shapes, path)
        self.sub.grouping = plan.grouping

    def gather(self, leaves, v: int):
        """The leaves of slice value v (flat device tensors)."""
        out = []
        for i, x in enumerate(leaves):
            axes = self.leaf_axes[i]
            if not axes:
                out.append(x)
                continue
            out.append(capi.slice_gather(x, self.full.shapes[i], axes, self.leaf_strides[i], v,
                                         1))
        return out


def checkpoint_bytes(plan: ContractionPlan, itemsize: int) -> int:
    """Device bytes of one recomputing backward over `plan`: every node of
    the forward kept for the reverse sweep, the largest intermediate's
    gradient twice over (the gradient in flight and its transpose) and one
    gradient per leaf."""
    sizes = [1] * len(plan.shapes)
    for i, sh in enumerate(plan.shapes):
        for d in sh:
            sizes[i] *= d
    leaves = sum(sizes[: plan.num_leaves])
    inter = sizes[plan.num_leaves:]
    return itemsize * (sum(sizes) + 2 * (max(inter) if inter else 0) + leaves)


def slices_for_budget(labels, shapes, path, budget_bytes: float, itemsize: int = 8,
                      max_count: int = 24) -> List[str]:
    """The fewest bonds, in the greedy slicer's order
    (circuits.choose_slices), for which one slice's checkpointed backward fits
    `budget_bytes` (checkpoint_bytes of the sliced plan, plus the full leaves'
    gradients). Raises ValueError when `max_count` bonds do not fit."""
    from . import circuits

    net = circuits.Network([(list(l), list(s), None) for l, s in zip(labels, shapes)])
    full = ContractionPlan(labels, shapes, path)
    leaf_bytes = itemsize * sum(int(np.prod(s)) if len(s) else 1 for s in shapes)
    for count in range(0, max_count + 1):
        sliced = circuits.choose_slices(net, path, count) if count else []
        sub = SlicedPlan(full, path, sliced).sub if sliced else full
        if checkpoint_bytes(sub, itemsize) + leaf_bytes <= budget_bytes:
            return sliced
    raise ValueError("no slicing of up to %d bonds fits %.3g bytes" % (max_count, budget_bytes))


def _sliced_forward(sp: SlicedPlan, leaves, precision: int):
    total = None
    for v in range(sp.num_slices):
        out = _forward(sp.sub, sp.gather(leaves, v), precision, keep=False)[-1]
        total = out if total is None else capi.add(total, out)
    return total


def _sliced_backward(sp: SlicedPlan, leaves, grad_out, precision: int, leaf_needs=None):
    """Per slice the conjugated leaf gradients, summed over the slices (into
    the full leaves' positions), then conjugated once."""
    if leaf_needs is None:
        leaf_needs = [True] * sp.full.num_leaves
    need = _needs(sp.sub, leaf_needs)
    h_out = capi.conj(grad_out)
    hs = [None] * sp.full.num_leaves
    for v in range(sp.num_slices):
        vals = _forward(sp.sub, sp.gather(leaves, v), precision, keep=True)
        h = _backward_conj(sp.sub, vals, h_out, precision, need)
        for i, hi in enumerate(h):
            if hi is None:
                continue
            if not sp.leaf_axes[i]:
                hs[i] = hi if hs[i] is None else capi.add(hs[i], hi)
                continue
            if hs[i] is None:
                hs[i] = torch.zeros_like(leaves[i])
            capi.slice_scatter_add(hi, sp.full.shapes[i], sp.leaf_axes[i], sp.leaf_strides[i], v,
                                   hs[i])
    return [None if h is None else capi.conj(h) for h in hs]


class _NetworkContraction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, plan, precision: int, *leaves):
        flat = [l.contiguous().reshape(-1) for l in leaves]
        if isinstance(plan, SlicedPlan):
            res = _sliced_forward(plan, flat, precision)
            out_shape = plan.sub.out_shape
        else:
            res = _forward(plan, flat, precision, keep=False)[-1]
            out_shape = plan.out_shape
        ctx.plan = plan
        ctx.precision = precision
        ctx.leaf_shapes = [tuple(l.shape) for l in leaves]
        ctx.save_for_backward(*leaves)
        return res.reshape(out_shape)

    @staticmethod
    def backward(ctx, grad_out):
        leaves = [l.contiguous().reshape(-1) for l in ctx.saved_tensors]
        g = grad_out.contiguous().reshape(-1).to(leaves[0].dtype)
        needs = ctx.needs_input_grad[2:]
        if isinstance(ctx.plan, SlicedPlan):
            grads = _sliced_backward(ctx.plan, leaves, g, ctx.precision, needs)
        else:
            vals = _forward(ctx.plan, leaves, ctx.precision, keep=True)
            grads = _backward(ctx.plan, vals, g, ctx.precision, needs)
        out = [None if gr is None else gr.reshape(s) for gr, s in zip(grads, ctx.leaf_shapes)]
        return (None, None, *out)


def contract_network(leaves: Sequence[torch.Tensor], labels: Sequence[Sequence[str]],
                     path: Sequence[Tuple[int, int]], precision: int = capi.PREC_AUTO,
                     plan=None, sliced: Sequence[str] = None,
                     memory_budget: float = None) -> torch.Tensor:
    """Contracts CUDA complex tensors `leaves` (labels[i] per leaf) along
    `path`; differentiable with respect to every leaf.

    sliced: bonds to slice; the value is the sum over their slice values,
    and forward and backward run (and recompute) one slice at a time.
    memory_budget: device bytes for one slice's checkpointed backward; picks
    `sliced` (slices_for_budget) when `sliced` is not given. `plan` (a
    ContractionPlan, or the SlicedPlan these build) skips the bookkeeping;
    reused across calls in a plain form (FP32, AUTO), it also runs the tiny
    steps of each dependency level as one grouped launch (jet_gb300.grouped)
    over device arenas it owns, so its evaluations must not overlap in time.
    A call without a plan runs every step as its own launch."""
    if plan is None:
        shapes = [list(l.shape) for l in leaves]
        if sliced is None and memory_budget is not None:
            sliced = slices_for_budget(labels, shapes, path, memory_budget,
                                       leaves[0].element_size())
        plan = ContractionPlan(labels, shapes, path)
        plan.grouping = False  # made for this call: a grouped schedule would not be reused
        if sliced:
            plan = SlicedPlan(plan, path, sliced)
    return _NetworkContraction.apply(plan, precision, *leaves)


class GraphedStep:
    """A loss-and-gradient evaluation captured once in a CUDA graph and
    replayed: `loss_fn()` must build its inputs from fixed tensors (the
    parameters) and return a real scalar; `params` are the leaf tensors whose
    `.grad` the backward fills.

    Every contraction, conjugation and transpose of the network (and torch's
    own kernels around it) is a node of one graph, so a replay costs no
    per-step host work: the per-step Python and launch overhead of the eager
    path (several launches per contraction, hundreds of steps) disappears.
    Shapes and the path are fixed at capture; to evaluate at new parameter
    values, copy them into `params` (in place) before `step()`.

    Capture happens after `warmup` eager evaluations on a side stream (the
    first launches of each kernel configure it, which must not happen inside
    a capture)."""

    def __init__(self, loss_fn, params: Sequence[torch.Tensor], warmup: int = 2):
        self.loss_fn = loss_fn
        self.params = list(params)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(max(1, warmup)):
                for p in self.params:
                    p.grad = None
                loss_fn().backward()
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        for p in self.params:
            p.grad = None
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.loss = loss_fn()
            self.loss.backward()
        self.grads = [p.grad for p in self.params]

    def step(self):
        """Replays the graph: returns the loss tensor; the gradients are in
        `self.grads` (the params' `.grad`, overwritten by every replay)."""
        self.graph.replay()
        return self.loss
