"""Drop-in for pg_gpu.moments_ld.compute_ld_statistics (moments format).

The reference loops over chunks of banded pairs (count gathers, float64
statistic kernels, cp.add.at into the bins; moments_ld.py:248-343).  Here one
libpgld call per population set walks the whole distance band on the device
and returns the (n_bins, n_stats) float64 sums: the haplotype path on the
tensor cores where they apply, the genotype path on dosage bit planes.
"""
from __future__ import annotations

import numpy as np

from . import _lib as L
from . import _ops
from .genotype_matrix import GenotypeMatrix
from .haplotype_matrix import HaplotypeMatrix, PackedVcf, read_vcf_packed
from .ld_pipeline import het_names as _het_names
from .ld_pipeline import ld_names as _ld_names


def _accessible(mat, accessible_bed):
    """The variants at accessible positions of the BED file (all of its
    chromosomes, as the reference's set_accessible_mask(path) without a
    chromosome; moments_ld.py:136-137, 159-160)."""
    if accessible_bed is None:
        return mat
    from .accessible import accessible_variants
    if isinstance(mat, PackedVcf):
        return mat.subset(accessible_variants(mat.positions, accessible_bed))
    keep = accessible_variants(mat._pos_np(), accessible_bed)
    return mat.get_subset(np.nonzero(keep)[0])


def _packed_vcf(vcf_file, pop_file, pops, ac_filter):
    """The populations packed straight from the VCF's GT text (no int8
    haplotype matrix), biallelic sites only with ac_filter; None when a
    population holds alleles >= 2 that are kept (ac_filter False), whose
    values the heterozygosity sums need."""
    pv = read_vcf_packed(vcf_file, pop_file, pops)
    if ac_filter:
        return pv.subset(pv.biallelic_sites())
    if any(pk.has_other for pk in pv.packs.values()):
        return None
    return pv


def compute_ld_statistics(vcf_file=None, rec_map_file=None, pop_file=None, pops=None,
                          r_bins=None, bp_bins=None, use_genotypes=False, report=True,
                          ac_filter=True, haplotype_matrix=None, genotype_matrix=None,
                          accessible_bed=None):
    """Binned moments LD statistics; returns {'bins', 'sums', 'stats', 'pops'}
    (moments_ld.py:40-206)."""
    if pops is None:
        pops = ["pop0", "pop1"]
    num_pops = len(pops)
    if num_pops < 1 or num_pops > 4:
        raise ValueError("1-4 populations supported")
    if r_bins is None and bp_bins is None:
        raise ValueError("Either r_bins or bp_bins must be provided")

    if use_genotypes:
        if genotype_matrix is not None:
            mat = genotype_matrix
        elif haplotype_matrix is not None:
            mat = GenotypeMatrix.from_haplotype_matrix(haplotype_matrix)
        else:
            if vcf_file is None:
                raise ValueError("vcf_file or genotype_matrix required")
            if pop_file is None:
                raise ValueError("pop_file is required when loading from VCF")
            if report:
                print(f"Loading {vcf_file} (genotypes) ...")
            mat = GenotypeMatrix.from_vcf(vcf_file)
            mat.load_pop_file(pop_file, pops=pops)
            if ac_filter:
                mat = mat.apply_biallelic_filter()
        mat = _accessible(mat, accessible_bed)
        mat.transfer_to_gpu()
        if report:
            print(f"  {mat.num_individuals} individuals, {mat.num_variants:,} variants")
    else:
        if haplotype_matrix is not None:
            mat = haplotype_matrix
        else:
            if vcf_file is None:
                raise ValueError("vcf_file or haplotype_matrix is required")
            if pop_file is None:
                raise ValueError("pop_file is required when loading from VCF")
            if report:
                print(f"Loading {vcf_file} ...")
            mat = _packed_vcf(vcf_file, pop_file, pops, ac_filter)
            if mat is None:
                mat = HaplotypeMatrix.from_vcf(vcf_file)
                mat.load_pop_file(pop_file, pops=pops)
                if ac_filter:
                    mat = mat.apply_biallelic_filter()
        mat = _accessible(mat, accessible_bed)
        if isinstance(mat, HaplotypeMatrix):
            mat.transfer_to_gpu()
            if report:
                print(f"  {mat.num_haplotypes} hap, {mat.num_variants:,} variants")
        elif report:
            print(f"  {sum(len(r) for r in mat.sample_sets.values())} hap, "
                  f"{mat.num_variants:,} variants")

    pos_np = (mat.positions if isinstance(mat, PackedVcf) else mat._pos_np()).astype(np.float64)
    if r_bins is not None:
        if rec_map_file is None:
            raise ValueError("rec_map_file required with r_bins")
        bins = np.asarray(r_bins, dtype=np.float64)
        gen = _interpolate_genetic_distances(pos_np, rec_map_file)
        max_bp = _max_bp_for_r_dist(pos_np, gen, float(bins[-1]))
    else:
        bins = np.asarray(bp_bins, dtype=np.float64)
        gen = None
        max_bp = float(bins[-1])
    n_bins = len(bins) - 1
    if report:
        print(f"  Computing LD ({n_bins} bins, {num_pops} pops) ...")
    ld_sums = _compute_ld_sums(mat, pops, bins, gen, max_bp, use_genotypes)
    het = _compute_heterozygosity(mat, pops, use_genotypes)
    if report:
        print("  Done.")
    bin_tuples = [(float(bins[i]), float(bins[i + 1])) for i in range(n_bins)]
    sums = [ld_sums[i] for i in range(n_bins)]
    sums.append(np.array([het[h] for h in _het_names(num_pops)]))
    return {"bins": bin_tuples, "sums": sums,
            "stats": (_ld_names(num_pops), _het_names(num_pops)), "pops": pops}


def _interpolate_genetic_distances(positions, rec_map_file):
    """Per-variant map positions in Morgans from a pos / cM map (moments_ld.py:214-227)."""
    mp, mv = [], []
    with open(rec_map_file) as f:
        for line in f:
            parts = line.strip().split()
            if len(parts) >= 2:
                try:
                    mp.append(float(parts[0]))
                    mv.append(float(parts[1]) / 100.0)
                except ValueError:
                    continue
    return np.interp(positions, np.array(mp), np.array(mv))


def _max_bp_for_r_dist(positions, gen_dists, max_r):
    """Physical distance bound for a recombination distance (moments_ld.py:230-245)."""
    chrom_len = float(positions[-1] - positions[0])
    if len(positions) < 2:
        return chrom_len
    bp = np.diff(positions).astype(np.float64)
    rd = np.diff(gen_dists)
    ok = bp > 0
    if not np.any(ok):
        return chrom_len
    rates = rd[ok] / bp[ok]
    min_rate = np.min(rates[rates > 0]) if np.any(rates > 0) else max_r / chrom_len
    return min(max_r / min_rate * 1.1, chrom_len)


def _compute_ld_sums(mat, pops, bins, gen_dists, max_bp, use_genotypes=False):
    """(n_bins, n_stats) float64 numpy sums (moments_ld.py:248-343)."""
    import torch
    if use_genotypes:
        # variants polymorphic across the union of the populations (moments_ld.py:256-280)
        g = mat.genotypes
        rows = sorted(set(i for p in pops for i in mat.sample_sets[p]))
        sub = g[torch.as_tensor(rows, device=g.device)]
        v = sub >= 0
        alt = torch.where(v, sub, torch.zeros_like(sub)).to(torch.int64).sum(0)
        nv = v.to(torch.int64).sum(0)
        keep = ((alt > 0) & (alt < 2 * nv) & (nv >= 2)).nonzero().flatten()
        data = g[:, keep].contiguous()
        pos_d = L.as_device(mat.positions, np.float64)[keep].contiguous()
        bc = None if gen_dists is None else L.as_device(gen_dists, np.float64)[keep].contiguous()
        packs = [_ops.pack_geno(data, mat.sample_sets[p]) for p in pops]
        sums, _ = _ops.geno_binned_sums(packs, pos_d, bins, max_dist=max_bp, bin_coord=bc)
    else:
        pos_d = L.as_device(mat.positions, np.float64)
        bc = None if gen_dists is None else L.as_device(gen_dists, np.float64)
        packs = [mat.packs[p] if isinstance(mat, PackedVcf) else mat.packed(p) for p in pops]
        sums, _ = _ops.binned_sums(packs, pos_d, bins, max_dist=max_bp, bin_coord=bc)
    return sums.cpu().numpy()


def _compute_heterozygosity(mat, pops, use_genotypes=False):
    """H_i_j of the moments convention (moments_ld.py:346-388)."""
    import torch
    alt, ref, nh = [], [], []
    for p in pops:
        rows = torch.as_tensor(mat.sample_sets[p], device="cuda")
        if use_genotypes:
            d = mat.genotypes[rows]
            v = d >= 0
            a = torch.where(v, d, torch.zeros_like(d)).to(torch.float64).sum(0)
            n = 2.0 * v.to(torch.float64).sum(0)
        elif isinstance(mat, PackedVcf):
            # biallelic alleles: the carriers of allele 1
            a = mat.alt_counts(p)
            n = torch.full_like(a, float(len(mat.sample_sets[p])))
        else:
            a = mat.haplotypes[rows].clamp(min=0).to(torch.float64).sum(0)
            n = torch.full_like(a, float(len(mat.sample_sets[p])))
        alt.append(a)
        ref.append(n - a)
        nh.append(n)
    out = {}
    P = len(pops)
    for i in range(P):
        for j in range(i, P):
            if i == j:
                val = (2.0 * ref[i] * alt[i] / (nh[i] * (nh[i] - 1))).sum()
            else:
                val = ((ref[i] * alt[j] + alt[i] * ref[j]) / (nh[i] * nh[j])).sum()
            out[f"H_{i}_{j}"] = float(val)
    return out
