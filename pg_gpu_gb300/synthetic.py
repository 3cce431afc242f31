"""Seeded synthetic haplotype panels of the measured LD workloads.

The copying model: F founder haplotypes draw each SNP's allele as
Bernoulli(p) with p ~ Beta(0.3, 0.3); every sampled haplotype copies one
founder, switches to another at rate ``switch`` per SNP, and flips an allele
with probability ``flip``; missing entries (-1) are set completely at random.
Positions are sorted uniform draws without replacement over the chromosome.

Panels are generated on the device with torch's generator (seeded), so the
benchmark and the full-size parity tests of the same workload see the same
panel within one process.
"""
from __future__ import annotations

import numpy as np

# two populations sharing a 40-founder pool, each flipping 10 % of the
# founders' alleles: 2 x 1,000 haplotypes x 200,000 SNPs over 20 Mb, 2 %
# missing, 20 log-spaced distance bins from 1 kb to 1 Mb
BINNED2POP = dict(pops=2, hap_per_pop=1000, n_snp=200_000, length=20_000_000, founders=40,
                  switch=1e-3, pop_flip=0.10, flip=1e-3, missing=0.02,
                  bins=np.logspace(3, 6, 21), seed=20261503)
# the same model at a tenth of the SNPs and chromosome length
BINNED2POP_SMALL = dict(BINNED2POP, n_snp=20_000, length=2_000_000)


def shared_founder_panel(cfg, device):
    """(int8 (pops * H, M) device panel, sorted int64 positions on the host)
    of the shared-founder multi-population model described by cfg."""
    import torch
    rng = np.random.default_rng(cfg["seed"])
    M, F, H = cfg["n_snp"], cfg["founders"], cfg["hap_per_pop"]
    pos = np.sort(rng.choice(cfg["length"], M, replace=False)).astype(np.int64)
    p = torch.as_tensor(rng.beta(0.3, 0.3, size=M), dtype=torch.float32, device=device)
    g = torch.Generator(device=device)
    g.manual_seed(cfg["seed"])
    founders = (torch.rand((F, M), generator=g, device=device) < p).to(torch.int8)
    pops = []
    for _ in range(cfg["pops"]):
        fp = founders ^ (torch.rand((F, M), generator=g, device=device) < cfg["pop_flip"]).to(torch.int8)
        sw = torch.rand((H, M), generator=g, device=device) < cfg["switch"]
        seg = torch.cumsum(sw, dim=1, dtype=torch.int32)
        del sw
        choice = torch.randint(0, F, (H, int(seg.max()) + 1), generator=g, device=device,
                               dtype=torch.int64)
        idx = torch.gather(choice, 1, seg.to(torch.int64))
        del seg, choice
        hap = torch.gather(fp, 0, idx)
        del idx
        hap ^= (torch.rand((H, M), generator=g, device=device) < cfg["flip"]).to(torch.int8)
        hap[torch.rand((H, M), generator=g, device=device) < cfg["missing"]] = -1
        pops.append(hap)
    panel = torch.cat(pops, 0).contiguous()
    torch.cuda.synchronize(device)
    return panel, pos


def copying_panel(gen, H, M, F, switch, flip, missing, device):
    """int8 (H, M) device panel of one population of the copying model: the
    founders' Beta(0.3, 0.3) allele frequencies come from torch's global
    generator (seed it first), everything else from the generator gen."""
    import torch
    p = torch.distributions.Beta(0.3, 0.3).sample((M,)).to(device)
    founders = (torch.rand((F, M), generator=gen, device=device) < p).to(torch.int8)
    sw = torch.rand((H, M), generator=gen, device=device) < switch
    seg = torch.cumsum(sw, dim=1, dtype=torch.int32)
    choice = torch.randint(0, F, (H, int(seg.max()) + 1), generator=gen, device=device)
    hap = torch.gather(founders, 0, torch.gather(choice, 1, seg.to(torch.int64)))
    hap ^= (torch.rand((H, M), generator=gen, device=device) < flip).to(torch.int8)
    if missing:
        hap[torch.rand((H, M), generator=gen, device=device) < missing] = -1
    return hap


def anchors_per_pairs(pos, max_dist, first, n_pairs):
    """End of the anchor block starting at `first` that holds at least
    n_pairs pairs within max_dist (or the last anchor)."""
    pos = np.asarray(pos, np.float64)
    jend = np.searchsorted(pos, pos[first:] + max_dist, side="right")
    per = np.maximum(jend - np.arange(first, len(pos)) - 1, 0)
    cum = np.cumsum(per)
    k = int(np.searchsorted(cum, n_pairs, side="left"))
    return min(first + k + 1, len(pos)), int(cum[min(k, len(cum) - 1)])
