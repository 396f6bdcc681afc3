"""Splitting one translation batch across ranks by target.

The reference's multithreaded_translator gives each host thread a partition
of the targets, so that no two threads update one expansion
(solidfmm/multithreaded_translator.cpp:261-330).  Across GPUs the same
partition needs no collective: rank r owns the targets [lo_r, hi_r) and runs
exactly the batch entries whose target lies there, in their original order,
reading its own copy of the sources.  Every target then receives the same
contributions in the same order as on one GPU, so the union of the ranks'
targets is bit-identical to the single-GPU result.

    pos = shard_by_target(dst_index, n_targets, world, rank)
    ctx.translate_device(op, prec, len(pos), src, S, nsrc, dst, S, n_targets,
                         p_in[pos], p_out[pos], shift[pos],
                         src_index=src_index[pos], dst_index=dst_index[pos])

Each rank's targets outside its range stay untouched; gathering them (for
example with an all-gather of the owned ranges) is the caller's choice.
"""
from __future__ import annotations

import numpy as np


def target_range(n_targets: int, world: int, rank: int) -> tuple[int, int]:
    """The contiguous target range [lo, hi) owned by a rank: n_targets split
    as evenly as possible, the first n_targets % world ranks one larger."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    base, extra = divmod(int(n_targets), world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_by_target(dst_index, n_targets: int, world: int, rank: int):
    """Positions, in batch order, of the entries whose target lies in this
    rank's range.  dst_index None means entry i targets expansion i (a batch
    of n_targets entries).  numpy arrays give a numpy int64 array, torch
    tensors a tensor on the same device."""
    lo, hi = target_range(n_targets, world, rank)
    if dst_index is None:
        return np.arange(lo, hi, dtype=np.int64)
    if isinstance(dst_index, np.ndarray):
        t = dst_index.astype(np.int64, copy=False)
        return np.nonzero((t >= lo) & (t < hi))[0].astype(np.int64)
    import torch

    t = dst_index.to(torch.int64)
    return torch.nonzero((t >= lo) & (t < hi)).flatten()
