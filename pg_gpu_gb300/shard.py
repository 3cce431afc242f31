"""Sharding the distance-binned LD sums across ranks (one GPU per rank).

The binned sums of moments_ld._compute_ld_sums (moments_ld.py:248-343) are a
sum over SNP pairs (i < j, pos[j] - pos[i] <= max_dist), so they partition by
the first SNP of a pair: rank r takes the anchors [start, stop) -- contiguous
ranges balanced by their pair counts -- and reads the SNPs up to the halo end
(the last SNP within max_dist of stop - 1).  Its partial is the binned sum
over the pairs whose first SNP lies in [start, stop), computed once
(pgld_hap_binned_sums_range); the one exchange is a sum of the
(n_bins x n_stats) float64 partials and the pair counts over the ranks.

The packed panel is replicated on every rank (at 2,000 haplotypes a SNP packs
to 504 bytes).  The planning and combination here are host code; the per-shard
compute is any callable (start, stop) -> (sums, counts) over the pairs
anchored in [start, stop), normally ``range_binned_sums`` on the device.
"""
from __future__ import annotations

import numpy as np


class Shard:
    """Anchors [start, stop) of one rank and the end of their halo."""

    __slots__ = ("rank", "start", "stop", "halo")

    def __init__(self, rank, start, stop, halo):
        self.rank, self.start, self.stop, self.halo = int(rank), int(start), int(stop), int(halo)

    def __repr__(self):
        return f"Shard(rank={self.rank}, start={self.start}, stop={self.stop}, halo={self.halo})"


def plan_shards(positions, max_dist, world):
    """Contiguous anchor ranges for `world` ranks, balanced by pair count.

    positions: sorted SNP coordinates (host array); a pair (i, j) belongs to
    the rank owning i.  Returns one Shard per rank (empty ranges allowed)."""
    pos = np.asarray(positions, dtype=np.float64)
    if world < 1:
        raise ValueError("world must be at least 1")
    if pos.ndim != 1:
        raise ValueError("positions must be 1-D")
    if pos.size > 1 and np.any(np.diff(pos) < 0):
        raise ValueError("positions must be sorted")
    n = pos.size
    jend = np.searchsorted(pos, pos + float(max_dist), side="right")  # one past the last partner
    per = np.maximum(jend - np.arange(n) - 1, 0).astype(np.int64)
    cum = np.concatenate([[0], np.cumsum(per)])
    total = int(cum[-1])
    cuts = [0]
    for r in range(1, world):
        # first anchor whose cumulative pairs reach r / world of the total
        cuts.append(int(np.searchsorted(cum, total * r / world, side="left")) if total else
                    (n * r) // world)
    cuts.append(n)
    for r in range(1, len(cuts)):
        cuts[r] = min(max(cuts[r], cuts[r - 1]), n)
    shards = []
    for r in range(world):
        s, e = cuts[r], cuts[r + 1]
        halo = int(jend[e - 1]) if e > s else e
        shards.append(Shard(r, s, e, max(halo, e)))
    return shards


def shard_partial(compute, shard):
    """(sums, counts) of the pairs whose first SNP lies in the shard:
    compute(start, stop) over the shard's anchor range, or None for an empty
    shard."""
    if shard.stop <= shard.start:
        return None
    return compute(shard.start, shard.stop)


def reduce_partials(sums, counts, group=None):
    """Sum the ranks' partials in place over torch.distributed (gloo on CPU
    tensors, nccl on device tensors); every rank gets the total."""
    import torch.distributed as dist
    backend = dist.get_backend(group)
    moved = backend == "gloo" and sums.is_cuda
    s = sums.cpu() if moved else sums
    c = counts.cpu() if moved else counts
    dist.all_reduce(s, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(c, op=dist.ReduceOp.SUM, group=group)
    if moved:
        sums.copy_(s)
        counts.copy_(c)
    return sums, counts


def range_binned_sums(pops, pos_d, bins, max_dist=None, bin_coord=None, form="auto"):
    """The device compute of one anchor range: compute(start, stop) -> the
    binned sums of the pairs whose first SNP lies in [start, stop), on the
    whole replicated panel (the kernels read the anchors and their halo)."""
    from . import _ops

    def compute(s, e):
        return _ops.binned_sums(pops, pos_d, bins, max_dist=max_dist, bin_coord=bin_coord,
                                form=form, anchors=(s, e))
    return compute


def binned_sums_distributed(pops, pos_d, bins, positions_host, max_dist=None, bin_coord=None,
                            form="auto", group=None):
    """Binned sums of the whole panel computed by all ranks of the process
    group, each on its shard; returns the total (sums, counts) on every rank."""
    import torch
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    bins_np = np.asarray(bins, dtype=np.float64)
    md = float(bins_np[-1]) if max_dist is None else float(max_dist)
    shards = plan_shards(positions_host, md, world)
    part = shard_partial(range_binned_sums(pops, pos_d, bins, md, bin_coord, form), shards[rank])
    n_bins = len(bins_np) - 1
    n_stats = {1: 3, 2: 15, 3: 45, 4: 105}[len(pops)]
    if part is None:
        sums = torch.zeros((n_bins, n_stats), dtype=torch.float64, device=pos_d.device)
        cnt = torch.zeros(n_bins, dtype=torch.int64, device=pos_d.device)
    else:
        sums, cnt = part
    return reduce_partials(sums, cnt, group)
