"""Genotype-path helpers behind the drop-in modules: 9-way counts, the
genotype case selection of the moments tables, Rogers-Huff r."""
from __future__ import annotations

import numpy as np

from . import _lib as L
from . import _ops


def counts_pairs(genotypes, idx_i, idx_j, pop_indices=None):
    """ld_pipeline.compute_genotype_counts_for_pairs (ld_pipeline.py:220-263)."""
    pk = _ops.pack_geno(genotypes, pop_indices)
    return _ops.geno_counts_pairs(pk, idx_i, idx_j)


def case_of(kind, pp):
    """Genotype kernel case of one (kind, populations) call, as the grouping of
    compute_all_{dd,dz,pi2}_geno (genotype_kernels.py:560-886)."""
    pp = tuple(int(x) for x in pp)
    if kind == "dd":
        a, b = pp
        return (L.G_DD_II, (a,)) if a == b else (L.G_DD_IJ, (a, b))
    if kind == "dz":
        i, j, k = pp
        if i == j == k:
            return L.G_DZ_III, (i,)
        if i == j:
            return L.G_DZ_IIJ, (i, k)
        if i == k:
            return L.G_DZ_IJI, (i, j)
        if j == k:
            return L.G_DZ_IJJ, (i, j)
        return L.G_DZ_IJK, (i, j, k)
    i, j, k, l = pp
    cnt = {}
    for p in pp:
        cnt[p] = cnt.get(p, 0) + 1
    nu, mc = len(cnt), max(cnt.values())
    if nu == 1:
        return L.G_PI2_IIII, (i,)
    if mc == 3:
        t = [p for p, v in cnt.items() if v == 3][0]
        s = [p for p, v in cnt.items() if v == 1][0]
        return (L.G_PI2_IIIJ if (i == t and j == t) else L.G_PI2_IJII), (t, s)
    if i == j and k == l:
        return L.G_PI2_IIKK, (i, k)
    if i == j:
        return L.G_PI2_IIKL, (i, k, l)
    if k == l:
        return L.G_PI2_IJKK, (i, j, k)
    if (i == k and j == l) or (i == l and j == k):
        return L.G_PI2_IJIJ, (i, j)
    if nu == 3:
        if i == k:
            return L.G_PI2_SHARED, (i, j, l)
        if i == l:
            return L.G_PI2_SHARED, (i, j, k)
        if j == k:
            return L.G_PI2_SHARED, (j, i, l)
        return L.G_PI2_SHARED, (j, i, k)
    return L.G_PI2_ALLDIFF, (i, j, k, l)


def specs_to_terms(stat_specs):
    terms = []
    for s, (_, calls) in enumerate(stat_specs):
        for w, kind, pp in calls:
            k, roles = case_of(kind, pp)
            terms.append((s, k, roles, float(w)))
    return terms


def dosage(matrix):
    """(n_individuals, n_variants) int8 dosage tensor of a Genotype- or
    HaplotypeMatrix (adjacent haplotypes paired, as _dosage_from_matrix,
    ld_statistics.py:346-390); raises ValueError on missing values."""
    from .genotype_matrix import GenotypeMatrix
    from .haplotype_matrix import HaplotypeMatrix
    if isinstance(matrix, HaplotypeMatrix):
        hap = L.as_device(matrix.haplotypes, np.int8)
        if bool((hap < 0).any()):
            raise ValueError("rogers_huff_r: input HaplotypeMatrix contains missing values (-1)")
        if hap.shape[0] % 2:
            raise ValueError(f"rogers_huff_r: HaplotypeMatrix has an odd number of haplotypes "
                             f"({hap.shape[0]}); cannot pair into diploids.")
        return (hap[0::2] + hap[1::2]).contiguous()
    if isinstance(matrix, GenotypeMatrix):
        g = L.as_device(matrix.genotypes, np.int8)
        if bool((g < 0).any()):
            raise ValueError("rogers_huff_r: input GenotypeMatrix contains missing values (-1)")
        return g
    raise TypeError(f"rogers_huff_r: expected HaplotypeMatrix or GenotypeMatrix; "
                    f"got {type(matrix).__name__}")


def rh_pairs(genotypes, idx_i, idx_j, square=False, dtype="f64"):
    """Rogers-Huff r (or r^2) of listed pairs over the individuals valid at both
    SNPs (equal to the reference's rogers_huff_r where nothing is missing)."""
    pk = _ops.pack_geno(genotypes)
    c, _ = _ops.geno_counts_pairs(pk, idx_i, idx_j)
    kind = L.G_RH_R2 if square else L.G_RH_R
    return _ops.stats([c], [None], [(0, kind, (0,), 1.0)], 1, dtype=dtype, geno=True)[:, 0]


def rogers_huff_r(matrix):
    """Condensed upper-triangle Rogers-Huff r (ld_statistics.py:492-521)."""
    import torch
    g = dosage(matrix)
    m = g.shape[1]
    ii, jj = torch.triu_indices(m, m, offset=1, device=g.device)
    return rh_pairs(g, ii.to(torch.int32), jj.to(torch.int32))
