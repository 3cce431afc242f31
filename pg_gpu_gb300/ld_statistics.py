"""Drop-in for the LD-statistic functions of pg_gpu.ld_statistics.

dd / dz / pi2 / r / r_squared / d_prime / compute_ld_statistics keep the
reference signatures (ld_statistics.py:13-246, 1030-1079) and population /
n_valid conventions (ld_statistics.py:1082-1113); the arithmetic runs in
libpgld with exact 64-bit integer numerators and a single float64 division,
so results equal the reference's float64 values wherever its own evaluation
is exact, and stay exact where its int32 fast path would wrap.
"""
from __future__ import annotations

from typing import Dict, List, Optional, Tuple, Union

import numpy as np

from . import _lib as L
from . import _ops
from .ld_pipeline import case_of

__all__ = ["mu_ld", "dd", "dz", "pi2", "dd_within", "dd_between", "r", "r_squared", "d_prime",
           "compute_ld_statistics", "rogers_huff_r", "rogers_huff_r_squared", "zns",
           "windowed_zns", "omega", "windowed_omega", "zns_diploid", "omega_diploid"]


def _counts(counts):
    c = L.as_device(counts, np.int32)
    if c.dim() != 2 or c.shape[1] % 4 != 0 or c.shape[1] == 0:
        raise ValueError("counts must have shape (N, 4*P)")
    return c


def _nv_tensor(x):
    return None if x is None else L.as_device(x, np.int32)


def _pop_views(c, n_valid, pops_needed):
    """Per-population (counts view, n_valid view or None), as _get_pop_data."""
    P = c.shape[1] // 4
    views, nvs = [], []
    nv2d = None
    if n_valid is not None and not isinstance(n_valid, tuple):
        nv2d = _nv_tensor(n_valid)
    tup = None
    if isinstance(n_valid, tuple):
        tup = [(_nv_tensor(x) if x is not None else None) for x in n_valid]
    for p in range(P):
        views.append(c[:, 4 * p:4 * p + 4])
        if n_valid is None:
            nvs.append(None)
        elif tup is not None:
            nvs.append(tup[p] if p < len(tup) else None)
        elif nv2d.dim() == 2:
            nvs.append(nv2d[:, p])
        else:
            nvs.append(nv2d)
    return views, nvs


def _one(counts, n_valid, kind, roles, views=None, nvs=None):
    c = _counts(counts)
    if views is None:
        views, nvs = _pop_views(c, n_valid, None)
    out = _ops.stats(views, nvs, [(0, kind, roles, 1.0)], 1)
    return out[:, 0]


def dd(counts, populations: Optional[Union[Tuple[int, int], int]] = None,
       n_valid=None):
    """D^2 for one population or between two (ld_statistics.py:13-65)."""
    c = _counts(counts)
    if populations is None:
        if c.shape[1] == 4:
            return _one(c, n_valid, L.DD_II, (0,))
        nv = n_valid
        if nv is not None and not isinstance(nv, tuple):
            t = _nv_tensor(nv)
            nv = t[:, 0] if t.dim() == 2 else t
        return _one(c[:, :4], nv, L.DD_II, (0,))
    a, b = populations
    if a == b:
        return _one(c, n_valid, L.DD_II, (a,))
    views, nvs = _pop_views(c, n_valid, None)
    if isinstance(n_valid, tuple):
        # _dd_between reads the tuple by position (ld_statistics.py:1145-1147)
        nvs = list(nvs)
        t0 = _nv_tensor(n_valid[0]) if len(n_valid) > 0 else None
        t1 = _nv_tensor(n_valid[1]) if len(n_valid) > 1 else None
        nvs[a], nvs[b] = t0, t1
    return _one(c, n_valid, L.DD_IJ, (a, b), views, nvs)


def dz(counts, populations: Optional[Tuple[int, int, int]] = None, n_valid=None):
    """Dz for any population triple (ld_statistics.py:68-97)."""
    c = _counts(counts)
    if populations is None:
        if c.shape[1] == 4:
            return _one(c, n_valid, L.DZ_III, (0,))
        populations = (0, 0, 0)
    kind, roles = case_of("dz", tuple(populations))
    return _one(c, n_valid, kind, roles)


def pi2(counts, populations: Optional[Tuple[int, int, int, int]] = None, n_valid=None):
    """pi2 for any population quadruple (ld_statistics.py:100-129, 1299-1412)."""
    c = _counts(counts)
    if populations is None:
        if c.shape[1] == 4:
            return _one(c, n_valid, L.PI2_IIII, (0,))
        populations = (0, 0, 0, 0)
    kind, roles = case_of("pi2", tuple(populations), symmetric_iikk=True)
    return _one(c, n_valid, kind, roles)


def dd_within(counts, n_valid=None):
    return dd(counts, None, n_valid)


def dd_between(counts, pop1_idx: int, pop2_idx: int, n_valid=None):
    return dd(counts, (pop1_idx, pop2_idx), n_valid)


def _r_family(counts, n_valid, kind):
    c = _counts(counts)[:, :4]
    nv = _nv_tensor(n_valid)
    out = _ops.stats([c], [nv], [(0, kind, (0,), 1.0)], 1)
    return out[:, 0]


def r(counts, n_valid=None):
    """Signed r from counts, NaN where undefined (ld_statistics.py:167-191)."""
    return _r_family(counts, n_valid, L.R)


def r_squared(counts, n_valid=None):
    """r^2 from counts, NaN where undefined (ld_statistics.py:194-217)."""
    return _r_family(counts, n_valid, L.R2)


def d_prime(counts, n_valid=None):
    """Lewontin's D', NaN where undefined (ld_statistics.py:220-246)."""
    return _r_family(counts, n_valid, L.DPRIME)


def compute_ld_statistics(counts, statistics: List[str] = ("dd", "dz", "pi2"),
                          populations: Optional[Dict[str, Union[Tuple, None]]] = None,
                          n_valid=None) -> Dict:
    """Several statistics in one call (ld_statistics.py:1030-1079)."""
    populations = populations or {}
    out = {}
    for stat in statistics:
        if stat == "dd":
            out["dd"] = dd(counts, populations.get("dd"), n_valid)
        elif stat == "dz":
            out["dz"] = dz(counts, populations.get("dz"), n_valid)
        elif stat == "pi2":
            out["pi2"] = pi2(counts, populations.get("pi2"), n_valid)
        elif stat == "r":
            out["r"] = r(counts, n_valid)
        elif stat == "r_squared":
            out["r_squared"] = r_squared(counts, n_valid)
        else:
            raise ValueError(f"Unknown statistic: {stat}")
    return out


def rogers_huff_r(matrix, tile_size=None):
    """Condensed Rogers-Huff r of all variant pairs (ld_statistics.py:492-521)."""
    from . import _geno
    return _geno.rogers_huff_r(matrix)


def rogers_huff_r_squared(matrix, tile_size=None):
    return rogers_huff_r(matrix) ** 2


# --------------------------------------------------------------------------
# ZnS over windows (ld_statistics.py:534-735, windowed_analysis.py:2013-2062)
# --------------------------------------------------------------------------
def _segregating_index(hap):
    """Indices of the sites with 0 < derived count < valid count (ld_statistics.py:250-277)."""
    import torch
    h = L.as_device(hap, np.int8)
    dac = h.clamp(min=0).to(torch.int32).sum(0)
    nv = (h >= 0).to(torch.int32).sum(0)
    return ((dac > 0) & (dac < nv)).nonzero().flatten().to(torch.int32)


def _zns_windows(matrix, win_start, win_stop, estimator):
    """ZnS of each SNP window [win_start[w], win_stop[w]) over its segregating
    sites (_zns_from_precomputed, ld_statistics.py:595-676), all windows in
    one launch; 0.0 where a window has fewer than 2 segregating sites."""
    if estimator not in ("sigma_d2", "r2"):
        raise ValueError(f"unknown estimator {estimator!r}")
    matrix.transfer_to_gpu()
    ws = np.asarray(win_start, np.int64)
    we = np.asarray(win_stop, np.int64)
    if ws.shape != we.shape:
        raise ValueError("win_start and win_stop must have the same shape")
    seg = _segregating_index(matrix.haplotypes)
    seg_np = seg.cpu().numpy()
    b = np.searchsorted(seg_np, ws, side="left").astype(np.int64)
    e = np.searchsorted(seg_np, we, side="left").astype(np.int64)
    sums, cnt = _ops.window_sums(matrix.packed(None), seg, b, e)
    s, c = sums.cpu().numpy(), cnt.cpu().numpy()
    out = np.zeros(len(ws))
    for w in range(len(ws)):
        if e[w] - b[w] < 2:
            continue
        if estimator == "sigma_d2":
            out[w] = s[w, 1] / c[w, 2] if c[w, 2] > 0 else 0.0
        else:
            out[w] = s[w, 5] / c[w, 0]
    return out


def windowed_zns(matrix, win_start, win_stop, estimator="sigma_d2"):
    """Per-window ZnS for SNP windows [win_start[w], win_stop[w]) in one launch:
    the zns loop of windowed_analysis (windowed_analysis.py:2013-2062), where
    windows of fewer than 4 SNPs are NaN and the estimator defaults to the
    unbiased sigma_D^2 (estimator "r2": mean naive r^2)."""
    out = _zns_windows(matrix, win_start, win_stop, estimator)
    short = (np.asarray(win_stop, np.int64) - np.asarray(win_start, np.int64)) < 4
    out[short] = np.nan
    return out


def zns(r2_matrix_or_matrix, missing_data="include", estimator="auto"):
    """Kelly's ZnS (ld_statistics.py:679-731).

    A HaplotypeMatrix takes the unbiased sigma_D^2 estimator by default
    ("auto"), or naive r^2 ("r2"), over its segregating sites (missing_data
    "exclude" first drops sites with missing calls), in one device pass; a
    GenotypeMatrix the squared dosage correlation of all its sites
    (_r2_matrix_diploid, ld_statistics.py:973-1020) from the 9-way joint
    genotype counts; a precomputed square r^2 matrix gives its mean
    off-diagonal value.
    """
    from .haplotype_matrix import HaplotypeMatrix
    is_hm = isinstance(r2_matrix_or_matrix, HaplotypeMatrix)
    if estimator == "auto":
        estimator = "sigma_d2" if is_hm else "r2"
    if estimator not in ("r2", "sigma_d2"):
        raise ValueError(f"unknown estimator {estimator!r}")
    if is_hm:
        hm = r2_matrix_or_matrix
        hm.transfer_to_gpu()
        if missing_data == "exclude":
            keep = ((hm.haplotypes < 0).sum(0) == 0).nonzero().flatten()
            hm = hm.get_subset(keep)
        return float(_zns_windows(hm, [0], [hm.num_variants], estimator)[0])
    if estimator == "sigma_d2":
        raise ValueError("estimator='sigma_d2' requires a HaplotypeMatrix, "
                         "not a pre-computed r² array")
    if _is_genotype_matrix(r2_matrix_or_matrix):
        row, _ = _diploid_row_col_sums(r2_matrix_or_matrix, missing_data)
        m = row.size
        return float(2.0 * row.sum() / (m * (m - 1))) if m >= 2 else 0.0
    import torch
    r2 = L.as_device(r2_matrix_or_matrix, np.float64)
    m = r2.shape[0]
    if m < 2:
        return 0.0
    return float((r2.sum() - torch.trace(r2)) / (m * (m - 1)))


# --------------------------------------------------------------------------
# diploid dosage r^2 of a GenotypeMatrix (ld_statistics.py:973-1020)
# --------------------------------------------------------------------------
def _cluster_labels(h):
    """Cluster labels of the rows of an int8 host matrix: identical rows
    without missing data; with missing data each row joins the first cluster
    whose representative (first member) matches it wherever both are called
    (diversity.py:1310-1360), compared against all representatives at once."""
    if not np.any(h < 0):
        _, inv = np.unique(h, axis=0, return_inverse=True)
        return inv.reshape(-1)
    n = h.shape[0]
    reps = np.empty((n, h.shape[1]), dtype=h.dtype)
    reps[0] = h[0]
    k = 1
    labels = np.zeros(n, dtype=np.int64)
    for i in range(1, n):
        r = reps[:k]
        ok = np.all((r == h[i]) | (r < 0) | (h[i] < 0), axis=1)
        j = int(np.argmax(ok)) if ok.any() else -1
        if j < 0:
            reps[k] = h[i]
            labels[i] = k
            k += 1
        else:
            labels[i] = j
    return labels


def mu_ld(haplotype_matrix, missing_data="include"):
    """mu_LD: how exclusively the haplotype patterns of the left half of the
    variants pair with those of the right half (RAiSD; ld_statistics.py:
    865-918).  A host computation over the haplotype patterns, as in the
    reference."""
    h = haplotype_matrix.haplotypes
    h = np.asarray(h.cpu().numpy() if hasattr(h, "cpu") else h).astype(np.int8, copy=False)
    if missing_data == "exclude":
        h = h[:, ~np.any(h < 0, axis=0)]
    n_hap, n_var = h.shape
    if n_var < 2:
        return 0.0
    mid = n_var // 2
    left = _cluster_labels(np.ascontiguousarray(h[:, :mid]))
    right = _cluster_labels(np.ascontiguousarray(h[:, mid:]))
    pairs = np.unique(np.stack([left, right], axis=1), axis=0)
    if pairs.size == 0:
        return 0.0
    # a left pattern is exclusive when it pairs with one right pattern only
    _, n_right_per_left = np.unique(pairs[:, 0], return_counts=True)
    _, n_left_per_right = np.unique(pairs[:, 1], return_counts=True)
    return float((np.mean(n_right_per_left == 1) + np.mean(n_left_per_right == 1)) / 2.0)


def _is_genotype_matrix(x):
    from .genotype_matrix import GenotypeMatrix
    return isinstance(x, GenotypeMatrix)


def _diploid_row_col_sums(gm, missing_data="include", chunk_pairs=1 << 24):
    """Per-site row and column sums of the upper triangle of the squared
    dosage-correlation matrix of _r2_matrix_diploid, from the 9-way joint
    genotype counts of every site pair (pgld_geno_counts_pairs): with per-site
    means mu and variances var over the valid individuals, the covariance of
    centred dosages with missing entries zeroed is sum_ab (a - mu_i)(b - mu_j)
    n_ab over the jointly valid individuals.  Returns (row, col) float64 on the
    host; pairs are processed in chunks of about chunk_pairs."""
    import torch
    gm.transfer_to_gpu()
    g = L.as_device(gm.genotypes, np.int8)
    if missing_data == "exclude":
        keep = ((g < 0).sum(0) == 0).nonzero().flatten()
        gm = gm.get_subset(keep)
        g = L.as_device(gm.genotypes, np.int8)
    m = g.shape[1]
    dev = g.device
    row = torch.zeros(m, dtype=torch.float64, device=dev)
    col = torch.zeros(m, dtype=torch.float64, device=dev)
    if m < 2:
        return row.cpu().numpy(), col.cpu().numpy()
    pk = gm.packed(None)
    if pk.has_other:
        raise NotImplementedError("diploid r^2 of dosages above 2")
    valid = g >= 0
    gc = torch.where(valid, g, torch.zeros_like(g)).to(torch.float64)
    nvs = valid.sum(0).to(torch.float64)
    mu = torch.where(nvs > 0, gc.sum(0) / torch.where(nvs > 0, nvs, 1.0), 0.0)
    var = (((gc - mu[None, :]) * valid) ** 2).sum(0)
    av = torch.tensor([0., 0., 0., 1., 1., 1., 2., 2., 2.], dtype=torch.float64, device=dev)
    bv = torch.tensor([0., 1., 2.] * 3, dtype=torch.float64, device=dev)
    per_row = (m - 1 - torch.arange(m, device=dev)).cpu().numpy()
    r0 = 0
    while r0 < m - 1:
        # rows [r0, r1) with about chunk_pairs pairs
        cum = np.cumsum(per_row[r0:])
        r1 = r0 + max(1, int(np.searchsorted(cum, chunk_pairs, side="right")))
        r1 = min(r1, m - 1)
        cnt = torch.as_tensor(per_row[r0:r1], device=dev)
        ii = torch.repeat_interleave(torch.arange(r0, r1, device=dev), cnt)
        start = torch.cumsum(cnt, 0) - cnt
        k = torch.arange(ii.numel(), device=dev)
        jj = ii + 1 + (k - torch.repeat_interleave(start, cnt))
        c, _ = _ops.geno_counts_pairs(pk, ii.to(torch.int32), jj.to(torch.int32))
        c = c.to(torch.float64)
        s_ab = c @ (av * bv)
        s_a = c @ av
        s_b = c @ bv
        n_ij = c.sum(1)
        mi, mj = mu[ii], mu[jj]
        cov = s_ab - mj * s_a - mi * s_b + mi * mj * n_ij
        den = var[ii] * var[jj]
        r2 = torch.where(den > 0, cov * cov / torch.where(den > 0, den, 1.0), 0.0)
        row.index_add_(0, ii, r2)
        col.index_add_(0, jj, r2)
        r0 = r1
    return row.cpu().numpy(), col.cpu().numpy()


# --------------------------------------------------------------------------
# Kim and Nielsen's omega (ld_statistics.py:734-862, windowed_analysis.py:2051)
# --------------------------------------------------------------------------
def _omega_estimator(estimator, is_hm):
    """'auto' -> sigma_d2 for a HaplotypeMatrix (ld_statistics.py:344-363)."""
    if estimator == "auto":
        return "sigma_d2" if is_hm else "rogers_huff"
    if estimator not in ("r2", "sigma_d2", "rogers_huff"):
        raise ValueError(f"Unknown estimator: {estimator!r} "
                         "(expected one of 'auto', 'r2', 'sigma_d2', 'rogers_huff')")
    return estimator


def _omega_windows(hm, win_start, win_stop, column):
    """omega of each SNP window [win_start[w], win_stop[w]) of hm over its
    segregating sites, one launch for all windows: the per-site row and
    column sums of the pair statistic (window column `column`) give every
    split point's block sums."""
    hm.transfer_to_gpu()
    seg = _segregating_index(hm.haplotypes)
    seg_np = seg.cpu().numpy()
    b = np.searchsorted(seg_np, np.asarray(win_start, np.int64), side="left").astype(np.int64)
    e = np.searchsorted(seg_np, np.asarray(win_stop, np.int64), side="left").astype(np.int64)
    rows, cols, off = _ops.window_snp_sums(hm.packed(None), seg, b, e, column)
    rows, cols = rows.cpu().numpy(), cols.cpu().numpy()
    return np.array([_ops.omega_from_sums(rows[off[w]:off[w + 1]], cols[off[w]:off[w + 1]])
                     for w in range(len(b))])


def omega(r2_matrix_or_matrix, missing_data="include", estimator="auto"):
    """Kim and Nielsen's omega: the largest ratio of the mean LD within the two
    blocks of a split of the sites to the mean LD across them, over splits
    l = 3 .. m-2 of the upper triangle (ld_statistics.py:761-862).

    A HaplotypeMatrix uses its segregating sites (after dropping sites with
    missing calls for missing_data="exclude") and the unbiased sigma_D^2 =
    DD / pi2 numerators by default ("auto"), or naive r^2 ("r2",
    "rogers_huff"); the pair statistics are reduced on the device to per-site
    row and column sums (no m x m matrix).  A GenotypeMatrix uses the squared
    dosage correlation of all its sites (as zns).  A precomputed square r^2
    matrix is used as given.  0.0 below 5 sites."""
    from .haplotype_matrix import HaplotypeMatrix
    is_hm = isinstance(r2_matrix_or_matrix, HaplotypeMatrix)
    estimator = _omega_estimator(estimator, is_hm)
    if estimator == "sigma_d2" and not is_hm:
        raise ValueError("estimator='sigma_d2' requires a HaplotypeMatrix")
    if is_hm:
        hm = r2_matrix_or_matrix
        hm.transfer_to_gpu()
        if missing_data == "exclude":
            keep = ((hm.haplotypes < 0).sum(0) == 0).nonzero().flatten()
            hm = hm.get_subset(keep)
        column = 1 if estimator == "sigma_d2" else 5
        return float(_omega_windows(hm, [0], [hm.num_variants], column)[0])
    if _is_genotype_matrix(r2_matrix_or_matrix):
        return _ops.omega_from_sums(*_diploid_row_col_sums(r2_matrix_or_matrix, missing_data))
    import torch
    r2 = L.as_device(r2_matrix_or_matrix, np.float64)
    if r2.dim() != 2 or r2.shape[0] != r2.shape[1]:
        raise ValueError("omega needs a square r^2 matrix")
    up = torch.triu(r2, diagonal=1)
    return _ops.omega_from_sums(up.sum(1).cpu().numpy(), up.sum(0).cpu().numpy())


def windowed_omega(matrix, win_start, win_stop, missing_data="include", estimator="auto"):
    """Per-window omega of SNP windows [win_start[w], win_stop[w]) of a
    HaplotypeMatrix in one launch: the omega column of windowed_analysis
    (windowed_analysis.py:2014-2062), NaN for windows of fewer than 4 SNPs."""
    estimator = _omega_estimator(estimator, True)
    hm = matrix
    ws = np.asarray(win_start, np.int64)
    we = np.asarray(win_stop, np.int64)
    if ws.shape != we.shape:
        raise ValueError("win_start and win_stop must have the same shape")
    if missing_data == "exclude":
        hm.transfer_to_gpu()
        keep = ((hm.haplotypes < 0).sum(0) == 0).nonzero().flatten()
        keep_np = keep.cpu().numpy()
        ws2 = np.searchsorted(keep_np, ws, side="left")
        we2 = np.searchsorted(keep_np, we, side="left")
        hm = hm.get_subset(keep)
    else:
        ws2, we2 = ws, we
    out = _omega_windows(hm, ws2, we2, 1 if estimator == "sigma_d2" else 5)
    out[(we - ws) < 4] = np.nan
    return out


# the reference's diploid names are aliases (ld_statistics.py:1026-1027)
zns_diploid = zns
omega_diploid = omega
