"""Drop-in for pg_gpu.ld_pipeline (ld_pipeline.py:1-482) on libpgld.

Same function names, arguments, return shapes and orders.  Arrays come back
as CUDA torch tensors (the reference returns CuPy arrays); inputs may be
torch tensors, CuPy arrays (``__cuda_array_interface__``) or NumPy arrays.
"""
from __future__ import annotations

import numpy as np

from . import _lib as L
from . import _ops

__all__ = ["estimate_ld_chunk_size", "iter_pairs_within_distance", "compute_counts_for_pairs",
           "compute_genotype_counts_for_pairs", "compute_two_pop_statistics_batch",
           "compute_single_pop_statistics_batch", "ld_names", "het_names",
           "generate_stat_specs", "PopData", "pairs_within_distance_statistics",
           "genotype_pairs_within_distance_statistics"]


def estimate_ld_chunk_size(n_haplotypes_per_pop, available_memory_bytes=None, num_pops=2):
    """Pairs per chunk from free device memory (ld_pipeline.py:16-49).

    Kept for callers that size their own loops; the library's band kernels
    do not chunk at all (they walk a tile work list in one launch).
    """
    if available_memory_bytes is None:
        import torch
        available_memory_bytes = int(torch.cuda.mem_get_info()[0] * 0.5)
    bytes_per_pair = (4 * n_haplotypes_per_pop * num_pops + 150 * num_pops) * 3
    chunk_size = available_memory_bytes // bytes_per_pair
    return max(100_000, min(chunk_size, 10_000_000))


def iter_pairs_within_distance(positions, max_dist, chunk_size):
    """Yield (idx_i, idx_j) int32 chunks of the pairs with pos[j]-pos[i] <= max_dist.

    Chunks are the reference's anchor blocks (ld_pipeline.py:94-122): block
    k ends at the first anchor whose cumulative pair count reaches
    k * chunk_size, so chunk contents match the reference exactly.
    """
    pos_d = _ops.positions_f64(positions)
    n = pos_d.numel()
    if n < 2:
        return
    off_d, total = _ops.band_offsets(pos_d, max_dist)
    if total == 0:
        return
    cum = off_d[1:].cpu().numpy()  # inclusive cumulative pairs per anchor
    chunk_size = max(1, int(chunk_size))
    n_chunks = (total + chunk_size - 1) // chunk_size
    targets = np.minimum(np.arange(1, n_chunks + 1, dtype=np.int64) * chunk_size, total)
    v_his = np.minimum(np.searchsorted(cum, targets, side="left") + 1, n)
    off = np.concatenate([[0], cum])
    v_lo = 0
    for v_hi in v_his:
        v_hi = int(v_hi)
        if v_hi <= v_lo:
            continue
        npairs = int(off[v_hi] - off[v_lo])
        if npairs == 0:
            v_lo = v_hi
            continue
        yield _ops.pairs_range(pos_d, max_dist, v_lo, v_hi, npairs)
        v_lo = v_hi


def compute_counts_for_pairs(haplotypes, idx_i, idx_j, pop_indices=None):
    """Counts [n11, n10, n01, n00] (N,4) int32 and n_valid (N,) or None.

    ld_pipeline.py:130-175: ==1 / ==0 allele semantics, n_valid returned only
    when the (population) matrix holds a -1.
    """
    pk = _ops.pack(haplotypes, pop_indices)
    return _ops.counts_pairs(pk, idx_i, idx_j)


def compute_genotype_counts_for_pairs(genotypes, idx_i, idx_j, pop_indices=None):
    """9-way genotype counts (N,9) (n00..n22) and n_valid or None (ld_pipeline.py:220-263)."""
    from . import _geno
    return _geno.counts_pairs(genotypes, idx_i, idx_j, pop_indices)


def _pc(counts):
    c = L.as_device(counts, np.int32)
    if c.dim() != 2 or c.shape[1] < 4:
        raise ValueError("counts must have shape (n_pairs, 4*P)")
    return c


def _nv(n_valid):
    return None if n_valid is None else L.as_device(n_valid, np.int32)


def pairs_within_distance_statistics(haplotypes, positions, max_dist, pop_indices=None,
                                     with_stats=True):
    """Every pair (i < j, pos[j] - pos[i] <= max_dist) of one population, fused
    on the device: the loop of iter_pairs_within_distance +
    compute_counts_for_pairs + compute_ld_statistics (ld_pipeline.py:57-175,
    ld_statistics.py:13-246) in one call, pairs in iter_pairs_within_distance
    order.  Returns (counts (N,4) int32, n_valid (N,) int32, stats (N,4)
    float32 = r^2, DD, Dz, pi2, or None)."""
    pk = _ops.pack(haplotypes, pop_indices)
    return _ops.band_pairs(pk, _ops.positions_f64(positions), float(max_dist),
                           with_stats=with_stats)


def genotype_pairs_within_distance_statistics(genotypes, positions, max_dist, pop_indices=None,
                                              statistics=("r2", "dd", "dz", "pi2"),
                                              with_counts=True):
    """Every pair (i < j, pos[j] - pos[i] <= max_dist) of one population of
    dosages, fused on the device: the loop of iter_pairs_within_distance +
    compute_genotype_counts_for_pairs + the single-population genotype DD /
    Dz / pi2 (genotype_kernels.py:27-71, 235-279, 364-398) and Rogers-Huff
    r^2 over the pairwise-valid individuals, pairs in
    iter_pairs_within_distance order.  Returns (counts (N,9) int32 or None,
    n_valid (N,) int32, stats (N,4) float32 = r^2, DD, Dz, pi2; columns not
    in `statistics` hold 0)."""
    pk = _ops.pack_geno(genotypes, pop_indices)
    return _ops.geno_band_pairs(pk, _ops.positions_f64(positions), float(max_dist),
                                with_counts=with_counts, columns=tuple(statistics))


def compute_two_pop_statistics_batch(counts_pop1, counts_pop2, n_valid1, n_valid2,
                                     ld_statistics=None):
    """The 15 two-population statistics, (N,15) float64 (ld_pipeline.py:271-322).

    Computed exactly (64-bit integer numerators, one float64 division).  The
    reference's fast path forms its polynomials in int32 and wraps once a
    population has more than ~215 valid haplotypes; this does not.
    """
    c1, c2 = _pc(counts_pop1), _pc(counts_pop2)
    n1, n2 = _nv(n_valid1), _nv(n_valid2)
    terms = spec_terms(2)
    return _ops.stats([c1, c2], [n1, n2], terms, 15)


def compute_single_pop_statistics_batch(counts, n_valid, ld_statistics=None):
    """(N,3) float64 columns DD, Dz, pi2 (ld_pipeline.py:330-349)."""
    c = _pc(counts)
    terms = [(0, L.DD_II, (0,), 1.0), (1, L.DZ_III, (0,), 1.0), (2, L.PI2_IIII, (0,), 1.0)]
    return _ops.stats([c], [_nv(n_valid)], terms, 3)


# --------------------------------------------------------------------------
# moments statistic names and specs (ld_pipeline.py:357-457)
# --------------------------------------------------------------------------
def ld_names(num_pops):
    """Names of moments.LD.Util.ld_names (ld_pipeline.py:357-376)."""
    P = int(num_pops)
    out = [f"DD_{i}_{j}" for i in range(P) for j in range(i, P)]
    out += [f"Dz_{i}_{j}_{k}" for i in range(P) for j in range(P) for k in range(j, P)]
    for i in range(P):
        for j in range(i, P):
            for k in range(i, P):
                for l in range(k, P):
                    if k == i == l and j != i:
                        continue
                    if i == k and l < j:
                        continue
                    out.append(f"pi2_{i}_{j}_{k}_{l}")
    return out


def het_names(num_pops):
    P = int(num_pops)
    return [f"H_{i}_{j}" for i in range(P) for j in range(i, P)]


def generate_stat_specs(num_pops):
    """(name, [(weight, 'dd'|'dz'|'pi2', pops)]) averaging of moments' _call_sgc."""
    specs = []
    for name in ld_names(num_pops):
        parts = name.split("_")
        kind, pp = parts[0], tuple(int(v) for v in parts[1:])
        if kind == "DD":
            specs.append((name, [(1.0, "dd", pp)]))
        elif kind == "Dz":
            i, j, k = pp
            specs.append((name, [(1.0, "dz", pp)] if j == k else
                          [(0.5, "dz", (i, j, k)), (0.5, "dz", (i, k, j))]))
        else:
            i, j, k, l = pp
            if i == j and k == l:
                calls = ([(1.0, "pi2", pp)] if i == k else
                         [(0.5, "pi2", (i, j, k, l)), (0.5, "pi2", (k, l, i, j))])
            elif i == j:
                calls = [(0.25, "pi2", t) for t in
                         ((i, j, k, l), (i, j, l, k), (k, l, i, j), (l, k, i, j))]
            elif k == l:
                calls = [(0.25, "pi2", t) for t in
                         ((i, j, k, l), (j, i, k, l), (k, l, i, j), (k, l, j, i))]
            else:
                calls = [(0.125, "pi2", t) for t in
                         ((i, j, k, l), (i, j, l, k), (j, i, k, l), (j, i, l, k),
                          (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i))]
            specs.append((name, calls))
    return specs


def _pi2_case(pp, symmetric_iikk):
    i, j, k, l = pp
    cnt = {}
    for p in pp:
        cnt[p] = cnt.get(p, 0) + 1
    nu, mc = len(cnt), max(cnt.values())
    if nu == 1:
        return L.PI2_IIII, (i,)
    if mc == 3:
        t = [p for p, v in cnt.items() if v == 3][0]
        s = [p for p, v in cnt.items() if v == 1][0]
        return L.PI2_TRIPLE, (t, s)
    if i == j and k == l:
        return (L.PI2_IIKK_SYM if symmetric_iikk else L.PI2_IIKK), (i, k)
    if i == j:
        return L.PI2_IIKL, (i, k, l)
    if k == l:
        return L.PI2_IJKK, (i, j, k)
    if (i == k and j == l) or (i == l and j == k):
        return L.PI2_IJIJ, (i, j)
    if nu == 3:
        if i == k:
            return L.PI2_SHARED, (i, j, l)
        if i == l:
            return L.PI2_SHARED, (i, j, k)
        if j == k:
            return L.PI2_SHARED, (j, i, l)
        return L.PI2_SHARED, (j, i, k)
    return L.PI2_ALLDIFF, (i, j, k, l)


def _dz_case(pp):
    i, j, k = pp
    if i == j == k:
        return L.DZ_III, (i,)
    if i == j:
        return L.DZ_IIJ, (i, k)
    if i == k:
        return L.DZ_IJI, (i, j)
    if j == k:
        return L.DZ_IJJ, (i, j)
    return L.DZ_IJK, (i, j, k)


def _dd_case(pp):
    a, b = pp
    return (L.DD_II, (a,)) if a == b else (L.DD_IJ, (a, b))


def case_of(kind, pops, symmetric_iikk=False):
    if kind == "dd":
        return _dd_case(pops)
    if kind == "dz":
        return _dz_case(pops)
    return _pi2_case(pops, symmetric_iikk)


def specs_to_terms(stat_specs):
    """Term list of the fused-kernel dispatch (haplotype_kernels.py:584-640)."""
    terms = []
    for s, (_, calls) in enumerate(stat_specs):
        for w, kind, pp in calls:
            k, roles = case_of(kind, tuple(pp))
            terms.append((s, k, roles, float(w)))
    return terms


def spec_terms(num_pops):
    return specs_to_terms(generate_stat_specs(num_pops))


class PopData:
    """Per-population float64 features (ld_pipeline.py:465-482), as tensors."""
    __slots__ = ("c1", "c2", "c3", "c4", "n", "D", "pA", "qA", "pB", "qB")

    def __init__(self, counts, n_valid):
        import torch
        c = L.as_device(counts).to(torch.float64)
        self.c1, self.c2, self.c3, self.c4 = c[:, 0], c[:, 1], c[:, 2], c[:, 3]
        self.n = (L.as_device(n_valid).to(torch.float64) if n_valid is not None
                  else self.c1 + self.c2 + self.c3 + self.c4)
        self.D = self.c2 * self.c3 - self.c1 * self.c4
        self.pA = self.c1 + self.c2
        self.qA = self.c3 + self.c4
        self.pB = self.c1 + self.c3
        self.qB = self.c2 + self.c4
