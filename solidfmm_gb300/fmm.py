"""Uniform-octree FMM pass over the translation operators.

The reference ships no tree code; its documentation describes the intended
use (doc/solidfmm.tex:660-690): multipoles move up the tree by M2M, across
by M2L over interaction lists, and down by L2L, each level a batch of
independent translations (multithreaded_translator, one call per level).
This module is that driver for a uniform octree on the unit cube, with every
batch kept on the GPU:

* level l has 2^l boxes per side, box (i, j, k) has index (i 2^l + j) 2^l + k
  and centre ((i, j, k) + 1/2) 2^-l; expansions of all levels live in one
  array (level offsets ``offset[l]``), multipoles and locals separately;
* arbitrary particles in the unit cube are binned into the leaves on the
  device (``bin_particles``: leaf index, stable sort, counts -> offsets), so
  leaves hold any number of particles, none included;
* P2M at the leaves (``sfmm_p2x_device``, or ``sfmm_p2x_ragged_device`` over
  each leaf's range of the sorted particles), then one execution plan
  (``sfmm_plan_*``) with the stages M2M depth -> 2 (one per level, targets
  repeat), M2L at levels 2..depth (interaction lists: children of the
  parent's neighbours that are not neighbours, at most 189 per box; targets
  repeat) and L2L 2 -> depth (one per level);
* L2P of the leaf locals at the particles (``sfmm_eval_device``) gives the
  far field; the near field (the 27 neighbour leaves) is direct summation and
  is not part of this module.

Tree construction uses torch on whatever device the tensors live on, so the
index arithmetic is testable on the CPU.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def level_offsets(depth: int):
    """Start of every level's boxes in the all-levels expansion array."""
    off = [0]
    for l in range(depth + 1):
        off.append(off[-1] + 8 ** l)
    return off


def box_coords(level: int, device="cpu"):
    import torch

    n = 2 ** level
    idx = torch.arange(n ** 3, device=device)
    return torch.stack((idx // (n * n), (idx // n) % n, idx % n), dim=1)


def box_centres(level: int, device="cpu"):
    import torch

    return (box_coords(level, device).to(torch.float64) + 0.5) / 2 ** level


def interaction_list(level: int, device="cpu"):
    """(source, target) box indices at one level (level >= 2): sources are the
    children of the target parent's neighbours (itself included) that are not
    neighbours of the target."""
    import torch

    n = 2 ** level
    c = box_coords(level, device)
    r = torch.arange(-3, 4, device=device)
    off = torch.stack(torch.meshgrid(r, r, r, indexing="ij"), dim=-1).reshape(-1, 3)
    off = off[off.abs().amax(1) >= 2]                      # not a neighbour
    cand = c[:, None, :] + off[None, :, :]                 # (boxes, offsets, 3)
    inside = ((cand >= 0) & (cand < n)).all(-1)
    same_parent_nbr = ((cand.div(2, rounding_mode="floor") - c[:, None, :].div(2, rounding_mode="floor")).abs()
                       .amax(-1) <= 1)
    ok = inside & same_parent_nbr
    tgt, k = torch.nonzero(ok, as_tuple=True)
    s = cand[tgt, k]
    src = (s[:, 0] * n + s[:, 1]) * n + s[:, 2]
    return src, tgt


def neighbours(level: int, device="cpu"):
    """(source, target) pairs of adjacent boxes (target itself included)."""
    import torch

    n = 2 ** level
    c = box_coords(level, device)
    r = torch.arange(-1, 2, device=device)
    off = torch.stack(torch.meshgrid(r, r, r, indexing="ij"), dim=-1).reshape(-1, 3)
    cand = c[:, None, :] + off[None, :, :]
    ok = ((cand >= 0) & (cand < n)).all(-1)
    tgt, k = torch.nonzero(ok, as_tuple=True)
    s = cand[tgt, k]
    return (s[:, 0] * n + s[:, 1]) * n + s[:, 2], tgt


@dataclass
class Stage:
    op: str
    src_index: object      # indices into the all-levels multipole (M2M, M2L) or local (L2L) array
    dst_index: object      # indices into the all-levels multipole (M2M) or local array
    shift: object          # new centre - old centre
    repeat: bool


def pass_stages(depth: int, device="cpu"):
    """The translation batches of one FMM pass, in execution order."""
    import torch

    assert depth >= 2
    off = level_offsets(depth)
    stages = []
    for l in range(depth, 2, -1):  # M2M: children at level l -> parents at l-1
        nb = 8 ** l
        child = torch.arange(nb, device=device)
        c = box_coords(l, device)
        parent = ((c[:, 0] // 2) * 2 ** (l - 1) + c[:, 1] // 2) * 2 ** (l - 1) + c[:, 2] // 2
        sh = box_centres(l - 1, device)[parent] - box_centres(l, device)[child]
        stages.append(Stage("m2m", child + off[l], parent + off[l - 1], sh, True))
    srcs, tgts, shs = [], [], []
    for l in range(2, depth + 1):  # M2L at every level from 2
        s, t = interaction_list(l, device)
        cen = box_centres(l, device)
        srcs.append(s + off[l])
        tgts.append(t + off[l])
        shs.append(cen[t] - cen[s])
    stages.append(Stage("m2l", torch.cat(srcs), torch.cat(tgts), torch.cat(shs), True))
    for l in range(2, depth):  # L2L: parents at level l -> children at l+1
        nb = 8 ** (l + 1)
        child = torch.arange(nb, device=device)
        c = box_coords(l + 1, device)
        parent = ((c[:, 0] // 2) * 2 ** l + c[:, 1] // 2) * 2 ** l + c[:, 2] // 2
        sh = box_centres(l + 1, device)[child] - box_centres(l, device)[parent]
        stages.append(Stage("l2l", parent + off[l], child + off[l + 1], sh, False))
    return stages


class UniformFMM:
    """One FMM pass on a uniform octree of the given depth at order P:
    leaf multipoles from particles, the translation plan, leaf locals.

    ``particles_per_leaf`` positions per leaf are given leaf by leaf (leaf
    index order) with their charges; ``run`` returns nothing and leaves the
    results in ``M`` and ``L`` (all levels, ``offsets`` per level)."""

    def __init__(self, ctx, depth: int, precision: int, device, tune: bool = False):
        import torch

        from . import _native

        self.ctx = ctx
        self.depth = depth
        self.P = P = ctx.P
        self.S = S = P * (P + 1)
        self.device = device
        self.offsets = off = level_offsets(depth)
        nbox = off[-1]
        self.M = torch.zeros(nbox, S, dtype=torch.float64, device=device)
        self.L = torch.zeros(nbox, S, dtype=torch.float64, device=device)
        self.leaf_centres = box_centres(depth, device).contiguous()
        self.stages = pass_stages(depth, device)
        self.plan = _native.Plan(ctx)
        self._keep = []
        for st in self.stages:
            n = len(st.src_index)
            order = torch.full((n,), P, dtype=torch.int32, device=device)
            si = st.src_index.to(torch.int32).contiguous()
            ti = st.dst_index.to(torch.int32).contiguous()
            sh = st.shift.to(torch.float64).contiguous()
            src = self.L if st.op == "l2l" else self.M
            dst = self.M if st.op == "m2m" else self.L
            self._keep += [order, si, ti, sh]
            self.plan.add(st.op, precision, n, src, S, nbox, dst, S, nbox, order, order, sh, src_index=si,
                          dst_index=ti, repeat=st.repeat)
        if tune:  # launch shapes measured per (operator, order bound) at finalize
            self.plan.options(tune=True)
        self.plan.finalize()

    @property
    def translations(self):
        return {op: sum(len(s.src_index) for s in self.stages if s.op == op) for op in ("m2m", "m2l", "l2l")}

    def run(self, charges, positions):
        """charges (leaves, q), positions (leaves, q, 3), leaf by leaf."""
        nleaf, nq = charges.shape
        self.M.zero_()
        self.L.zero_()
        lo = self.offsets[self.depth]
        self.ctx.p2x(0, nleaf, nq, charges, positions, self.leaf_centres, self.M[lo:], self.S)
        self.plan.run()

    def run_particles(self, charges, positions):
        """One pass for arbitrary particles in the unit cube (charges (n,),
        positions (n, 3)): bin them into the leaves (``bin_particles``), P2M
        of every leaf over its own particles, then the plan.  Returns the
        charges and positions sorted by leaf and keeps the binning in
        ``order`` and ``leaf_offsets``; ``leaf_of_sorted()`` gives each sorted
        particle's leaf (the box index for L2P)."""
        order, off = bin_particles(positions, self.depth)
        self.order, self.leaf_offsets = order, off
        q = charges[order].contiguous()
        p = positions[order].contiguous()
        self._sorted = (q, p)  # alive until the next pass (the kernels run asynchronously)
        self.M.zero_()
        self.L.zero_()
        lo = self.offsets[self.depth]
        self.ctx.p2x_ragged(0, 8 ** self.depth, off, q, p, self.leaf_centres, self.M[lo:], self.S)
        self.plan.run()
        return q, p

    def leaf_of_sorted(self):
        """Leaf of every particle of the last ``run_particles``, in sorted order (int32)."""
        import torch

        counts = (self.leaf_offsets[1:] - self.leaf_offsets[:-1]).to(torch.int64)
        leaves = torch.arange(len(counts), dtype=torch.int32, device=counts.device)
        return torch.repeat_interleave(leaves, counts)

    def leaf_locals(self):
        return self.L[self.offsets[self.depth]:]


def bin_particles(positions, depth: int):
    """Octree build for arbitrary particles in the unit cube: every particle
    goes to the leaf box (i, j, k) = floor(x 2^depth) (the face x = 1 to the
    last box), and the particles are ordered by leaf, stably.  Returns
    (order, offsets): ``positions[order]`` lists leaf 0's particles first and
    leaf b's are ``order[offsets[b]:offsets[b+1]]`` (int32, 8^depth + 1
    entries).  Positions outside [0, 1]^3 raise ValueError."""
    import torch

    n = 2 ** depth
    if positions.numel() and (bool((positions < 0).any()) or bool((positions > 1).any())):
        raise ValueError("particles must lie in the unit cube [0, 1]^3")
    ijk = (positions * n).floor().to(torch.int64).clamp_(0, n - 1)
    leaf = (ijk[:, 0] * n + ijk[:, 1]) * n + ijk[:, 2]
    order = torch.argsort(leaf, stable=True)
    offsets = torch.zeros(n ** 3 + 1, dtype=torch.int64, device=positions.device)
    offsets[1:] = torch.cumsum(torch.bincount(leaf, minlength=n ** 3), 0)
    return order, offsets.to(torch.int32)


def random_particles(depth: int, per_leaf: int, seed: int, device):
    """per_leaf particles uniform in every leaf, charges U[-1, 1]."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    nleaf = 8 ** depth
    lo = box_coords(depth, device).to(torch.float64) / 2 ** depth
    pos = lo[:, None, :] + torch.rand(nleaf, per_leaf, 3, dtype=torch.float64, device=device, generator=g) / 2 ** depth
    q = torch.rand(nleaf, per_leaf, dtype=torch.float64, device=device, generator=g) * 2 - 1
    return q.contiguous(), pos.contiguous()
