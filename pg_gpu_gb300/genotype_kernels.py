"""Drop-in for pg_gpu.genotype_kernels.compute_multi_pop_statistics_batch_geno.

The reference runs one float64 RawKernel per case group on per-population
feature arrays (genotype_kernels.py:412-936); here the whole (N, n_stats)
table is one libpgld launch over exact 64-bit integer numerators, each
divided once.
"""
from __future__ import annotations

import numpy as np

from . import _geno
from . import _lib as L
from . import _ops


def compute_multi_pop_statistics_batch_geno(counts_per_pop, n_valid_per_pop, _=None,
                                            stat_specs=None):
    """(N, n_stats) float64 for 1..4 populations from (N, 9) genotype counts
    in the reference's n00..n22 column order (genotype_kernels.py:889-936)."""
    from .ld_pipeline import generate_stat_specs
    P = len(counts_per_pop)
    if not 1 <= P <= L.MAX_POPS:
        raise ValueError(f"1 to {L.MAX_POPS} populations supported, got {P}")
    specs = generate_stat_specs(P) if stat_specs is None else stat_specs
    cs = [L.as_device(c, np.int32) for c in counts_per_pop]
    for c in cs:
        if c.dim() != 2 or c.shape[1] < 9:
            raise ValueError("genotype counts must have shape (n_pairs, 9)")
    nvs = [None if v is None else L.as_device(v, np.int32) for v in n_valid_per_pop]
    return _ops.stats(cs, nvs, _geno.specs_to_terms(specs), len(specs), geno=True)
