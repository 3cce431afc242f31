"""Drop-in for pg_gpu.ld_statistics_genotype.sigma_d2_geno (the per-pair
DD / pi2 ratio of the moments genotype estimators)."""
from __future__ import annotations

import numpy as np

from . import _lib as L
from . import _ops


def sigma_d2_geno(matrix, idx_i=None, idx_j=None):
    """Per-pair sigma_D^2 (ld_statistics_genotype.py:1518-1598).

    NaN where pi^2 is not positive or fewer than 4 individuals; ValueError on
    missing values, TypeError for other inputs, as the reference.
    """
    import torch
    from .genotype_matrix import GenotypeMatrix
    from .haplotype_matrix import HaplotypeMatrix
    if isinstance(matrix, GenotypeMatrix):
        g = L.as_device(matrix.genotypes, np.int8)
    elif isinstance(matrix, HaplotypeMatrix):
        g = L.as_device(GenotypeMatrix.from_haplotype_matrix(matrix).genotypes, np.int8)
    else:
        raise TypeError(f"matrix must be a GenotypeMatrix or HaplotypeMatrix, "
                        f"got {type(matrix).__name__}")
    if bool((g < 0).any()):
        raise ValueError("sigma_d2_geno does not support missing values (-1); "
                         "filter or impute before calling")
    m = g.shape[1]
    if idx_i is None and idx_j is None:
        ii, jj = torch.triu_indices(m, m, offset=1, device=g.device)
        ii, jj = ii.to(torch.int32), jj.to(torch.int32)
    elif idx_i is None or idx_j is None:
        raise ValueError("idx_i and idx_j must be provided together")
    else:
        ii, jj = L.as_device(idx_i, np.int32), L.as_device(idx_j, np.int32)
        if ii.shape != jj.shape:
            raise ValueError("idx_i and idx_j must have the same shape")
    pk = _ops.pack_geno(g)
    c, _ = _ops.geno_counts_pairs(pk, ii, jj)
    return _ops.stats([c], [None], [(0, L.G_SIGMA_D2, (0,), 1.0)], 1, geno=True)[:, 0]
