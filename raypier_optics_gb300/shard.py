"""Ray sharding across GPUs.

Within a generation every ray is independent and a child depends only on its
parent, so a trace splits into contiguous ray shards, one per rank, with no
exchange inside the hot path.  The only global quantity is the position of a
shard's rays in the concatenated generation: the single-GPU (and reference)
order is "shard 0's rays, then shard 1's, ...", because children are appended
in ascending parent index (raypier/core/ctracer.pyx:2083-2117) and contiguous
parent ranges produce contiguous child ranges.  Merging therefore needs, per
generation, an exclusive scan of the per-shard ray counts to rebase
``parent_idx`` -- one small all-gather of integers per trace, done after the
trace, off the data path.
"""
from __future__ import annotations

import numpy as np


def shard_bounds(n: int, world: int, rank: int):
    """Contiguous [lo, hi) slice of n rays owned by `rank`."""
    base, rem = divmod(n, world)
    lo = rank * base + min(rank, rem)
    return lo, lo + base + (1 if rank < rem else 0)


def merge_generations(per_shard):
    """Concatenate per-shard generations into the single-trace order.

    per_shard[r][g] is shard r's generation g (a ray_dtype array); generation
    0 is the shard's input slice.  Returns the merged list of generations with
    parent_idx rebased to the merged parent generation.
    """
    n_gens = max((len(s) for s in per_shard), default=0)
    merged = []
    for g in range(n_gens):
        parts = []
        parent_offset = 0
        for s in per_shard:
            part = s[g].copy() if g < len(s) else None
            if part is not None and g > 0:
                part['parent_idx'] += np.uint32(parent_offset)
            if g > 0:
                parent_offset += len(s[g - 1]) if g - 1 < len(s) else 0
            if part is not None:
                parts.append(part)
        merged.append(np.concatenate(parts) if parts else np.zeros(0, dtype=per_shard[0][0].dtype))
    # the reference stops at the first empty generation
    while merged and len(merged[-1]) == 0:
        merged.pop()
    return merged


def generation_offsets(counts_per_rank):
    """Exclusive scan over ranks of per-generation ray counts.

    counts_per_rank[r][g] -> offsets[r][g] = sum of counts of ranks < r in g.
    """
    c = np.asarray(counts_per_rank, dtype=np.int64)
    return np.cumsum(c, axis=0) - c


def gather_counts(local_counts, max_gens, group=None):
    """All-gather each rank's per-generation counts (torch.distributed)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    t = torch.zeros(max_gens, dtype=torch.int64)
    t[:len(local_counts)] = torch.tensor(local_counts, dtype=torch.int64)
    out = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(out, t, group=group)
    return np.stack([o.numpy() for o in out])


def rebase_local(local_gens, rank, counts_all):
    """Rebase this rank's generations into global indices in place of a full
    merge: parent_idx of generation g >= 1 is shifted by the number of rays
    lower ranks hold in generation g-1.  Returns (rebased gens, global start
    of this rank's slice in each generation)."""
    offs = generation_offsets(counts_all)[rank]
    out = []
    for g, gen in enumerate(local_gens):
        a = gen.copy()
        if g > 0:
            a['parent_idx'] += np.uint32(offs[g - 1])
        out.append(a)
    return out, offs
