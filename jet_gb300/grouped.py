"""Grouped launches for the differentiable contraction (jet_gb300.autograd).

A light-cone expectation network such as <Z_i Z_j> of a 6 x 6, 10-layer
RX-RZ-CZ circuit (679 steps, 668 of them tiny) has few dependency levels
(23): the steps of one level read only values of lower levels. Launched one by one, each step costs a launch of a few microseconds
of device time, which is nearly all of its time. Here the tiny steps of a
level (m n k below 131,072 and k <= 64, the bound by which the
TaskBasedContractor's replay groups) share one jetgpu_contract_group launch,
which reads every operand through offset tables (any axis order) and adds
the k products in order with the plain form's FMAs. Larger steps keep their
own jetgpu_contract call.

The values live in one device arena owned by the evaluation (leaves first,
copied in by one torch.cat, then every step's output), so that the task
tables, whose entries hold arena addresses, are built and uploaded once, on
the first evaluation, outside any CUDA graph capture: a captured evaluation
then makes no host-to-device copy. The reverse sweep over conjugated
gradients (see jet_gb300.autograd) groups the adjoint contractions of a
level the same way, in a second arena. Evaluations of one plan share these
arenas, so they must not overlap in time (one stream, or synchronised).
"""
from __future__ import annotations

import ctypes
from typing import Dict, List, Tuple

import numpy as np
import torch

from . import capi

TINY_WORK = 131072  # m n k below this, with k <= TINY_K: a task of a grouped launch
TINY_K = 64
GROUP_TASKS = 256  # tasks per jetgpu_contract_group launch
ARENA_MAX_BYTES = 1 << 30  # plans whose values need more are evaluated step by step

Region = Tuple[str, int, int]  # (arena, element offset, elements)


def tiny(m: int, n: int, k: int) -> bool:
    return k <= TINY_K and m * n * k < TINY_WORK


def layout(a_labels, a_shape, b_labels, b_shape):
    """ContractTensors' view of a pairwise contraction (Tensor.hpp:708-752):
    (a_perm, b_perm, m, n, k, left count, common count, C labels, C shape)."""
    pa, pb = {}, {}  # first position of each label
    for i, x in enumerate(a_labels):
        pa.setdefault(x, i)
    for i, x in enumerate(b_labels):
        pb.setdefault(x, i)
    left = [x for x in a_labels if x not in pb]
    right = [x for x in b_labels if x not in pa]
    common = [x for x in a_labels if x in pb]
    dims = dict(zip(a_labels, a_shape))
    dims.update(zip(b_labels, b_shape))
    m = n = k = 1
    for x in left:
        m *= dims[x]
    for x in right:
        n *= dims[x]
    for x in common:
        k *= dims[x]
    return ([pa[x] for x in left + common], [pb[x] for x in common + right], m, n, k,
            len(left), len(common), left + right, [dims[x] for x in left + right])


class NoGroup(Exception):
    """The evaluation runs step by step instead."""


def capturing(device) -> bool:
    return torch.device(device).type == "cuda" and torch.cuda.is_current_stream_capturing()


class Op:
    """One contraction: out[m x n] = x[m x k] y[k x n] over arena regions
    (operand axes in the orders x_perm, y_perm), then, when `dst` is set, a
    transpose of out (shape out_shape) by dst_perm into dst."""

    def __init__(self, x: Region, x_labels, x_shape, y: Region, y_labels, y_shape, out: Region):
        (self.x_perm, self.y_perm, self.m, self.n, self.k, self.nl, self.nc, self.out_labels,
         self.out_shape) = layout(x_labels, x_shape, y_labels, y_shape)
        self.x, self.x_shape = x, list(x_shape)
        self.y, self.y_shape = y, list(y_shape)
        self.out = out
        self.dst = None
        self.dst_perm = None

    @property
    def tiny(self) -> bool:
        return tiny(self.m, self.n, self.k)


class Group:
    """One grouped launch: the device address of its task array, and per task
    the Op and its four offset tables (for readers without the device)."""

    def __init__(self, ptr: int, tasks: List[dict], tiles: int, dtype_code: int, view):
        self.ptr, self.tasks, self.tiles, self.dtype_code, self.view = (ptr, tasks, tiles,
                                                                        dtype_code, view)


def launch_group(group: Group) -> None:
    capi.contract_group_at(group.ptr, len(group.tasks), group.tiles, group.dtype_code)


class Schedule:
    """The launches of one evaluation in order: per level, its tiny ops in
    grouped launches (a lone tiny op runs as a single), then its other ops,
    then the transposes of ops that have a `dst`. Builds and uploads the
    offset tables and task array, checking every table against its region."""

    def __init__(self, levels: List[List[Op]], arenas: Dict[str, torch.Tensor], dtype, device):
        self.arenas = arenas
        self.items: List[Tuple[str, object]] = []
        tables = [np.zeros(1, dtype=np.int64)]  # entry 0: the batch offset
        at = 1
        specs = []  # (op, [(table start, table)] x 4)
        chunks = []  # (first spec, ops)
        for level in levels:
            tiny_ops = [op for op in level if op.tiny]
            for first in range(0, len(tiny_ops), GROUP_TASKS):
                chunk = tiny_ops[first: first + GROUP_TASKS]
                if len(chunk) < 2:
                    self.items.extend(("single", op) for op in chunk)
                    continue
                chunks.append((len(specs), chunk))
                self.items.append(("group", len(chunks) - 1))
                for op in chunk:
                    offs = []
                    for shape, axes in ((op.x_shape, op.x_perm[: op.nl]),
                                        (op.x_shape, op.x_perm[op.nl:]),
                                        (op.y_shape, op.y_perm[: op.nc]),
                                        (op.y_shape, op.y_perm[op.nc:])):
                        t = capi.view_offsets(shape, axes)
                        offs.append((at, t))
                        tables.append(t)
                        at += len(t)
                    ar, ac, br, bc = (t for _, t in offs)
                    if (len(ar) != op.m or len(ac) != op.k or len(br) != op.k or len(bc) != op.n
                            or int(ar.max()) + int(ac.max()) >= op.x[2]
                            or int(br.max()) + int(bc.max()) >= op.y[2]
                            or op.m * op.n > op.out[2]):
                        raise NoGroup("an offset table leaves its operand")
                    specs.append((op, offs))
            self.items.extend(("single", op) for op in level if not op.tiny)
            self.items.extend(("permute", op) for op in level if op.dst is not None)
        esize = torch.empty(0, dtype=dtype).element_size()
        for op in (o for lv in levels for o in lv):
            for r in (op.x, op.y, op.out) + ((op.dst,) if op.dst is not None else ()):
                if r[1] < 0 or r[1] + r[2] > arenas[r[0]].numel():
                    raise NoGroup("a region leaves its arena")
        table = np.concatenate(tables)
        table_bytes = (table.nbytes + 255) // 256 * 256
        task_size = ctypes.sizeof(capi.GroupTask)
        self.buffer = torch.empty(table_bytes + len(specs) * task_size, dtype=torch.uint8,
                                  device=device)
        base = self.buffer.data_ptr()
        arr = (capi.GroupTask * max(len(specs), 1))()
        for q, (op, offs) in zip(arr, specs):
            q.A, q.B, q.C = (arenas[r[0]].data_ptr() + r[1] * esize for r in (op.x, op.y, op.out))
            q.batch, q.m, q.n, q.k = 1, op.m, op.n, op.k
            q.a_bat = q.b_bat = base
            q.a_row, q.a_col, q.b_row, q.b_col = (base + 8 * o for o, _ in offs)
        host = bytearray(table_bytes + len(specs) * task_size)
        host[: table.nbytes] = table.tobytes()
        host[table_bytes:] = bytes(arr)[: len(specs) * task_size]
        self.buffer.copy_(torch.frombuffer(host, dtype=torch.uint8))
        dc = capi.dtype_code(dtype)
        self.groups = []
        for first, chunk in chunks:
            tiles = sum(int(capi.lib.jetgpu_group_tiles(1, op.m, op.n)) for op in chunk)
            tasks = [{"op": op, "tables": [t for _, t in specs[first + j][1]]}
                     for j, op in enumerate(chunk)]
            self.groups.append(Group(base + table_bytes + first * task_size, tasks, tiles, dc,
                                     self.view))

    def view(self, region: Region) -> torch.Tensor:
        name, off, n = region
        return self.arenas[name][off: off + n]

    def run(self, precision: int) -> None:
        v = self.view
        for kind, it in self.items:
            if kind == "group":
                launch_group(self.groups[it])
            elif kind == "single":
                capi.contract(v(it.x), it.x_shape, it.x_perm, v(it.y), it.y_shape, it.y_perm,
                              it.m, it.n, it.k, precision=precision, out=v(it.out))
            else:
                capi.permute(v(it.out), it.out_shape, it.dst_perm, out=v(it.dst))


class Grouped:
    """Grouped evaluation of an autograd.ContractionPlan (no slicing) on one
    device and dtype: the forward, and per pattern of leaves that need
    gradients, the reverse sweep."""

    def __init__(self, plan, dtype, device):
        if capturing(device):
            raise NoGroup("built outside captures only")
        L = plan.num_leaves
        used = [0] * len(plan.shapes)
        for st in plan.steps:
            used[st.a] += 1
            used[st.b] += 1
        if any(u > 1 for u in used):
            raise NoGroup("a node is read twice")
        self.plan, self.dtype, self.device = plan, dtype, device
        self.size = [int(np.prod(s)) if len(s) else 1 for s in plan.shapes]
        self.depth = [0] * L
        for st in plan.steps:
            self.depth.append(max(self.depth[st.a], self.depth[st.b]) + 1)
        off = np.concatenate([[0], np.cumsum(self.size)]).astype(np.int64)
        self.val_off = [int(x) for x in off]
        self.esize = torch.empty(0, dtype=dtype).element_size()
        if self.val_off[-1] * self.esize > ARENA_MAX_BYTES:
            raise NoGroup("the values need more than the arena limit")
        self.arenas: Dict[str, torch.Tensor] = {
            "val": torch.empty(max(self.val_off[-1], 1), dtype=dtype, device=device)}
        levels: Dict[int, List[Op]] = {}
        for idx, st in enumerate(plan.steps):
            c = L + idx
            op = Op(self.val(st.a), plan.labels[st.a], plan.shapes[st.a], self.val(st.b),
                    plan.labels[st.b], plan.shapes[st.b], self.val(c))
            levels.setdefault(self.depth[c], []).append(op)
        self.forward_schedule = Schedule([levels[d] for d in sorted(levels)], self.arenas, dtype,
                                         device)
        self.backward_schedules: Dict[tuple, tuple] = {}

    def val(self, node: int) -> Region:
        return ("val", self.val_off[node], self.size[node])

    def run_forward(self, leaves, precision: int) -> List[torch.Tensor]:
        """Every node's value (views of the arena), the leaves copied in first."""
        L = self.plan.num_leaves
        torch.cat([l.reshape(-1) for l in leaves], out=self.arenas["val"][: self.val_off[L]])
        self.forward_schedule.run(precision)
        return [self.forward_schedule.view(self.val(i)) for i in range(len(self.size))]

    def _backward_schedule(self, need: List[bool]):
        key = tuple(need)
        if key in self.backward_schedules:
            return self.backward_schedules[key]
        if capturing(self.device):
            raise NoGroup("built outside captures only")
        plan, L = self.plan, self.plan.num_leaves
        # Conjugated gradients: the needed leaves' first and contiguous (one
        # conjugation at the end), then every other node that needs one, then
        # room for the leaves' transposes.
        h_off, at = {}, 0
        for i in range(L):
            if need[i]:
                h_off[i] = at
                at += self.size[i]
        leaf_end = at
        for i in range(L, len(self.size)):
            if need[i]:
                h_off[i] = at
                at += self.size[i]
        tmp_off, tmp_at = {}, at
        for i in range(L):
            if need[i]:
                tmp_off[i] = tmp_at
                tmp_at += self.size[i]
        if tmp_at * self.esize > ARENA_MAX_BYTES:
            raise NoGroup("the gradients need more than the arena limit")
        name = "h%d" % len(self.backward_schedules)  # one arena per pattern
        self.arenas[name] = torch.empty(max(tmp_at, 1), dtype=self.dtype, device=self.device)

        def h(i):
            return (name, h_off[i], self.size[i])

        hl = {len(self.size) - 1: (plan.labels[-1], plan.shapes[-1])}
        levels: Dict[int, List[Op]] = {}
        for idx in range(len(plan.steps) - 1, -1, -1):
            st = plan.steps[idx]
            c = L + idx
            if not need[c]:
                continue
            lc, sc = hl[c]
            la, sa, lb, sb = plan.labels[st.a], plan.shapes[st.a], plan.labels[st.b], plan.shapes[st.b]
            for i, x, lx, sx, y, ly, sy in ((st.a, h(c), lc, sc, self.val(st.b), lb, sb),
                                            (st.b, self.val(st.a), la, sa, h(c), lc, sc)):
                if not need[i]:
                    continue
                if i >= L:  # an intermediate: its H in the order its contraction gives
                    op = Op(x, lx, sx, y, ly, sy, h(i))
                    hl[i] = (op.out_labels, op.out_shape)
                else:  # a leaf: in its own order, transposed only if neither order gives it
                    target = plan.labels[i]
                    op = Op(x, lx, sx, y, ly, sy, h(i))
                    if op.out_labels != target:
                        op = Op(y, ly, sy, x, lx, sx, h(i))
                    if op.out_labels != target:
                        op = Op(x, lx, sx, y, ly, sy, (name, tmp_off[i], self.size[i]))
                        op.dst = h(i)
                        op.dst_perm = [op.out_labels.index(t) for t in target]
                levels.setdefault(self.depth[c], []).append(op)
        sched = Schedule([levels[d] for d in sorted(levels, reverse=True)], self.arenas,
                         self.dtype, self.device)
        self.backward_schedules[key] = (sched, h(len(self.size) - 1), (name, 0, leaf_end), h_off)
        return self.backward_schedules[key]

    def run_backward(self, grad_out, need: List[bool], precision: int) -> List[torch.Tensor]:
        """Leaf gradients (None where not needed) from the result's gradient;
        the values must be in the arena (run_forward just before)."""
        sched, root, leaves, h_off = self._backward_schedule(need)
        capi.conj(grad_out, out=sched.view(root))
        sched.run(precision)
        if not h_off or leaves[2] == 0:
            return [None] * self.plan.num_leaves
        flat = capi.conj(sched.view(leaves))
        out = []
        for i in range(self.plan.num_leaves):
            if i in h_off:
                out.append(flat[h_off[i]: h_off[i] + self.size[i]])
            else:
                out.append(None)
        return out
