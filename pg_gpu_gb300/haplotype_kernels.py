"""Drop-in for pg_gpu.haplotype_kernels.compute_multi_pop_statistics_batch_hap.

The reference dispatches each moments statistic to case-grouped float64
kernels (haplotype_kernels.py:335-640); here the whole (N, n_stats) table is
one libpgld launch over exact integer case formulas.
"""
from __future__ import annotations

import numpy as np

from . import _lib as L
from . import _ops
from .ld_pipeline import specs_to_terms


def compute_multi_pop_statistics_batch_hap(counts_per_pop, n_valid_per_pop,
                                           ld_statistics_module=None, stat_specs=None):
    """(N, n_stats) float64 for 1..4 populations (haplotype_kernels.py:584-640)."""
    from .ld_pipeline import generate_stat_specs
    P = len(counts_per_pop)
    if not 1 <= P <= L.MAX_POPS:
        raise ValueError(f"1 to {L.MAX_POPS} populations supported, got {P}")
    specs = generate_stat_specs(P) if stat_specs is None else stat_specs
    cs = [L.as_device(c, np.int32) for c in counts_per_pop]
    nvs = [None if v is None else L.as_device(v, np.int32) for v in n_valid_per_pop]
    return _ops.stats(cs, nvs, specs_to_terms(specs), len(specs))
