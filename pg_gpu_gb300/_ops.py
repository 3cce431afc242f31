"""Device operations behind the reference-shaped API: packing, counting,
statistic finalisation and distance-binned sums, all through libpgld.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as L


def _torch():
    import torch
    return torch


# --------------------------------------------------------------------------
# packed haplotype planes
# --------------------------------------------------------------------------
class PackedPop:
    """Bit planes of one population (carrier / reference, optional validity).

    ``has_missing`` mirrors the reference's ``cp.any(haplotypes == -1)`` over
    the population's rows (ld_pipeline.py:158); ``has_other`` flags values
    outside {-1, 0, 1}, for which the validity plane is kept.
    """

    def __init__(self, planes, valid, n_words, n_rows, n_snp, has_missing, has_other):
        self.planes = planes
        self.valid = valid
        self.n_words = n_words
        self.n_rows = n_rows
        self.n_snp = n_snp
        self._flags = None
        self._missing = has_missing
        self._other = has_other

    @classmethod
    def pending(cls, planes, valid, n_words, n_rows, n_snp, flags):
        """Planes whose flags (a device int32[2] written by the packing kernel)
        are read on first use, so that packing does not synchronise."""
        pk = cls(planes, valid, n_words, n_rows, n_snp, None, None)
        pk._flags = flags
        return pk

    def _resolve(self):
        if self._flags is not None:
            f = self._flags.cpu().numpy()
            self._missing, self._other = bool(f[0]), bool(f[1])
            self._flags = None

    @property
    def has_missing(self):
        self._resolve()
        return self._missing

    @property
    def has_other(self):
        self._resolve()
        return self._other

    @property
    def valid_for_n(self):
        """Validity plane when the pairwise n differs from n11+n10+n01+n00."""
        return self.valid if (self.has_other and self.has_missing) else None


def _check_rows(rows, n_total):
    """Population row indices as a device int32 tensor, checked against
    n_total (on the host for host indices, one device read otherwise)."""
    torch = _torch()
    if isinstance(rows, torch.Tensor) and rows.is_cuda:
        rows_t = L.as_device(rows, np.int32)
        if rows_t.numel():
            # a device tensor passed again unmodified (same version counter)
            # keeps the range its last check found: no device read per call
            seen = getattr(rows_t, "_pgld_range", None)
            if seen is not None and seen[0] == rows_t._version:
                lo, hi = seen[1], seen[2]
            else:
                lo, hi = (int(v) for v in torch.aminmax(rows_t))
                rows_t._pgld_range = (rows_t._version, lo, hi)
            if lo < 0 or hi >= n_total:
                raise IndexError("population row index out of range")
        return rows_t
    r = np.asarray(rows.numpy() if isinstance(rows, torch.Tensor) else rows)
    if r.size and (int(r.min()) < 0 or int(r.max()) >= n_total):
        raise IndexError("population row index out of range")
    return L.as_device(r.astype(np.int32, copy=False), np.int32)


def _host_readable(hap):
    """True for a contiguous int8 CPU tensor in pinned (page-locked) memory:
    the packing kernel reads it in place over the host link."""
    torch = _torch()
    return (isinstance(hap, torch.Tensor) and not hap.is_cuda and hap.dtype == torch.int8
            and hap.dim() == 2 and hap.stride(1) == 1 and hap.is_pinned())


def pack(hap, rows=None):
    """Pack the rows of an int8 (H x M) matrix into bit planes on the device.

    hap is a device matrix (or anything as_device accepts, copied first); an
    int8 CPU tensor in pinned memory is read in place by the packing kernel,
    so only the packed planes are written to device memory (the call then
    returns once the kernel is done with the host matrix)."""
    torch = _torch()
    if not _host_readable(hap):
        hap = L.as_device(hap, np.int8)
    if hap.dim() != 2:
        raise ValueError("haplotypes must be 2-D (n_haplotypes, n_variants)")
    n_total, n_snp = hap.shape
    if rows is not None:
        rows_t = _check_rows(rows, n_total)
        n_rows = rows_t.numel()
    else:
        rows_t = None
        n_rows = n_total
    W = max(1, (n_rows + 31) // 32)
    dev = hap.device if hap.is_cuda else torch.device("cuda", torch.cuda.current_device())
    planes = torch.empty((n_snp, 2 * W), dtype=torch.int32, device=dev)
    valid = torch.empty((n_snp, W), dtype=torch.int32, device=dev)
    flags = torch.zeros(2, dtype=torch.int32, device=dev)
    if n_rows == 0:
        planes.zero_()
        valid.zero_()
    else:
        h = L.handle()
        L.check(L.lib().pgld_pack_haplotypes(h, L.ptr(hap), hap.stride(0), n_snp, L.ptr(rows_t),
                                             n_rows, L.ptr(planes), L.ptr(valid), L.ptr(flags),
                                             L.stream_ptr()), h)
    pk = PackedPop.pending(planes, valid, W, n_rows, n_snp, flags)
    if not hap.is_cuda:
        pk._resolve()  # the host matrix is read in place: finish before returning
    return pk


def panel(pops):
    pn = L.HapPanel()
    pn.n_pops = len(pops)
    for p, pk in enumerate(pops):
        pn.n_words[p] = pk.n_words
        pn.planes[p] = pk.planes.data_ptr()
        v = pk.valid_for_n
        pn.valid[p] = v.data_ptr() if v is not None else None
    pn.n_snp = pops[0].n_snp
    return pn


# --------------------------------------------------------------------------
# counts
# --------------------------------------------------------------------------
def counts_pairs(pk, idx_i, idx_j):
    """(counts int32 (N,4), n_valid int32 (N,) or None) for listed pairs."""
    torch = _torch()
    ii = L.as_device(idx_i, np.int32)
    jj = L.as_device(idx_j, np.int32)
    if ii.shape != jj.shape:
        raise ValueError("idx_i and idx_j must have the same shape")
    n = ii.numel()
    counts = torch.empty((n, 4), dtype=torch.int32, device=ii.device)
    nv = torch.empty(n, dtype=torch.int32, device=ii.device) if pk.has_missing else None
    if n:
        h = L.handle()
        v = pk.valid_for_n
        L.check(L.lib().pgld_hap_counts_pairs(h, L.ptr(pk.planes), L.ptr(v), pk.n_words, pk.n_snp,
                                              L.ptr(ii), L.ptr(jj), n, L.ptr(counts), 4,
                                              L.ptr(nv), L.stream_ptr()), h)
        st = torch.zeros(1, dtype=torch.int32)
        L.check(L.lib().pgld_device_status(h, ctypes.cast(st.data_ptr(), ctypes.POINTER(
            ctypes.c_int32)), L.stream_ptr()), h)
        if int(st[0]):
            raise IndexError("pair index out of range of the variant axis")
    return counts, nv


def tally(pk):
    torch = _torch()
    m = pk.n_snp
    n = m * (m - 1) // 2
    counts = torch.empty((n, 4), dtype=torch.int32, device=pk.planes.device)
    nv = torch.empty(n, dtype=torch.int32, device=pk.planes.device) if pk.has_missing else None
    if n:
        h = L.handle()
        # tally_gpu_haplotypes counts validity as != -1 (haplotype_matrix.py:1398-1418)
        L.check(L.lib().pgld_hap_tally(h, L.ptr(pk.planes), L.ptr(pk.valid_for_n), pk.n_words, m,
                                       L.ptr(counts), L.ptr(nv), L.stream_ptr()), h)
    return counts, nv


# --------------------------------------------------------------------------
# statistics
# --------------------------------------------------------------------------
def make_terms(term_list):
    """[(stat, kind, pops, weight)] -> ctypes array of Term."""
    arr = (L.Term * len(term_list))()
    for k, (stat, kind, pops, w) in enumerate(term_list):
        arr[k].stat = stat
        arr[k].kind = kind
        pp = list(pops) + [0] * (4 - len(pops))
        for q in range(4):
            arr[k].pops[q] = pp[q]
        arr[k].weight = w
    return arr


def stats(pop_counts, pop_nvalid, term_list, n_stats, dtype="f64", geno=False):
    """Statistic columns (N, n_stats) from per-pop counts views.

    pop_counts[p]: int32 CUDA tensor view with shape (N, >=4) (haplotype
    counts) or (N, >=9) (genotype counts, geno=True) and unit inner stride;
    pop_nvalid[p]: int32 CUDA tensor (N,) (any stride) or None.
    """
    torch = _torch()
    n = pop_counts[0].shape[0]
    out = torch.empty((n, n_stats), dtype=torch.float64 if dtype == "f64" else torch.float32,
                      device=pop_counts[0].device)
    if n == 0:
        return out
    pc = L.PairCounts()
    pc.n_pops = len(pop_counts)
    for p, c in enumerate(pop_counts):
        if c.dtype != torch.int32 or c.stride(1) != 1:
            raise ValueError("counts must be int32 with unit column stride")
        pc.counts[p] = c.data_ptr()
        pc.counts_ld[p] = c.stride(0)
        nv = pop_nvalid[p]
        if nv is not None:
            if nv.dtype != torch.int32:
                raise ValueError("n_valid must be int32")
            pc.n_valid[p] = nv.data_ptr()
            pc.nvalid_ld[p] = nv.stride(0)
    terms = make_terms(term_list)
    h = L.handle()
    fn = L.lib().pgld_geno_stats if geno else L.lib().pgld_hap_stats
    L.check(fn(h, ctypes.byref(pc), n, terms, len(term_list), n_stats, L.ptr(out),
               L.F64 if dtype == "f64" else L.F32, n_stats, L.stream_ptr()), h)
    return out


# --------------------------------------------------------------------------
# distance band
# --------------------------------------------------------------------------
def band_offsets(pos_d, max_dist):
    torch = _torch()
    m = pos_d.numel()
    off = torch.empty(m + 1, dtype=torch.int64, device=pos_d.device)
    tot = ctypes.c_int64()
    h = L.handle()
    L.check(L.lib().pgld_count_pairs_within(h, L.ptr(pos_d), m, float(max_dist), ctypes.byref(tot),
                                            L.ptr(off), L.stream_ptr()), h)
    return off, int(tot.value)


def band_pair_count(pos_d, max_dist):
    """Pairs within max_dist of sorted device positions.  The count is kept
    with the positions tensor (keyed by its version counter and max_dist), so
    a call repeated on unchanged positions reads nothing from the device."""
    key = float(max_dist)
    cache = getattr(pos_d, "_pgld_npairs", None)
    if cache is not None and cache[0] == pos_d._version and key in cache[1]:
        return cache[1][key]
    _, n = band_offsets(pos_d, max_dist)
    if cache is None or cache[0] != pos_d._version:
        cache = (pos_d._version, {})
        pos_d._pgld_npairs = cache
    cache[1][key] = n
    return n


def pairs_range(pos_d, max_dist, i_begin, i_end, n_pairs):
    torch = _torch()
    ii = torch.empty(n_pairs, dtype=torch.int32, device=pos_d.device)
    jj = torch.empty(n_pairs, dtype=torch.int32, device=pos_d.device)
    h = L.handle()
    L.check(L.lib().pgld_pairs_within(h, L.ptr(pos_d), pos_d.numel(), float(max_dist), i_begin,
                                      i_end, L.ptr(ii), L.ptr(jj), n_pairs, L.stream_ptr()), h)
    return ii, jj


def positions_f64(positions):
    return L.as_device(positions, np.float64)


def band_pairs(pk, pos_d, max_dist, with_stats=True, form="auto", _tuning=False):
    """Fused per-pair outputs of one population over the distance band.

    Returns (counts (N,4) int32, n_valid (N,) int32, stats (N,4) float32 =
    r^2, DD, Dz, pi2 or None).  form: "tc" (tcgen05 tensor cores), "plain"
    (AND + popcount) or "auto" (tensor cores whenever they apply).
    """
    if form == "auto":
        form = "tc" if tc_applies([pk]) else "plain"
    if form == "tc" and not _tuning:
        from . import autotune
        autotune.apply("pairs", [pk.n_words])
    torch = _torch()
    n = band_pair_count(pos_d, max_dist)
    dev = pos_d.device
    counts = torch.empty((n, 4), dtype=torch.int32, device=dev)
    nv = torch.empty(n, dtype=torch.int32, device=dev)
    st = torch.empty((n, 4), dtype=torch.float32, device=dev) if with_stats else None
    h = L.handle()
    L.check(L.lib().pgld_hap_band_pairs(h, ctypes.byref(panel([pk])), L.ptr(pos_d),
                                        float(max_dist), L.ptr(counts), L.ptr(nv), L.ptr(st), n,
                                        L.FORM_TC if form == "tc" else L.FORM_PLAIN,
                                        L.stream_ptr()), h)
    return counts, nv, st


WINDOW_COLUMNS = ("r2", "sigma_d2", "dd", "dz", "pi2", "r2_naive")


def window_sums(pk, idx, win_begin, win_end, form="auto", _tuning=False):
    """Per-window sums (n_win, 6) float64 and counts (n_win, 3) int64 over
    every pair inside each window (one launch for all windows).

    idx: int32 SNP indices (None: identity); window w covers
    idx[win_begin[w]:win_end[w]].  Columns: WINDOW_COLUMNS; counts: pairs,
    pairs with r^2 defined, pairs with n >= 4.  form: "tc", "plain" or
    "auto" (tensor cores whenever they apply)."""
    if form == "auto":
        form = "tc" if tc_applies([pk]) else "plain"
    if form == "tc" and not _tuning:
        from . import autotune
        autotune.apply("windows", [pk.n_words])
    torch = _torch()
    dev = pk.planes.device
    wb = L.as_device(win_begin, np.int64)
    we = L.as_device(win_end, np.int64)
    if wb.shape != we.shape:
        raise ValueError("win_begin and win_end must have the same shape")
    n_win = wb.numel()
    sums = torch.empty((max(n_win, 0), 6), dtype=torch.float64, device=dev)
    cnt = torch.empty((max(n_win, 0), 3), dtype=torch.int64, device=dev)
    if n_win <= 0:
        return sums, cnt
    ii = None if idx is None else L.as_device(idx, np.int32)
    n_idx = pk.n_snp if ii is None else ii.numel()
    h = L.handle()
    L.check(L.lib().pgld_hap_window_sums(h, ctypes.byref(panel([pk])), L.ptr(ii), n_idx, L.ptr(wb),
                                         L.ptr(we), n_win, L.ptr(sums), L.ptr(cnt),
                                         L.FORM_TC if form == "tc" else L.FORM_PLAIN,
                                         L.stream_ptr()), h)
    st = torch.zeros(1, dtype=torch.int32)
    L.check(L.lib().pgld_device_status(h, ctypes.cast(st.data_ptr(), ctypes.POINTER(
        ctypes.c_int32)), L.stream_ptr()), h)
    if int(st[0]):
        raise IndexError(f"window or SNP index out of range (device status {int(st[0])})")
    return sums, cnt


def window_snp_sums(pk, idx, win_begin, win_end, stat):
    """Per-SNP row and column sums (float64, one entry per list position of
    each window, windows concatenated) of window statistic column stat
    (WINDOW_COLUMNS) over the pairs a < b of each window, and the offsets of
    the windows' entries (host int64, n_win + 1)."""
    torch = _torch()
    dev = pk.planes.device
    wb_h = np.asarray(win_begin, np.int64)
    we_h = np.asarray(win_end, np.int64)
    if wb_h.shape != we_h.shape:
        raise ValueError("win_begin and win_end must have the same shape")
    n_win = wb_h.size
    lens = np.maximum(we_h - wb_h, 0)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    n_out = int(off[-1])
    rows = torch.empty(max(n_out, 1), dtype=torch.float64, device=dev)
    cols = torch.empty(max(n_out, 1), dtype=torch.float64, device=dev)
    if n_win == 0:
        return rows[:0], cols[:0], off
    ii = None if idx is None else L.as_device(idx, np.int32)
    n_idx = pk.n_snp if ii is None else ii.numel()
    wb, we = L.as_device(wb_h, np.int64), L.as_device(we_h, np.int64)
    off_d = L.as_device(off[:-1].copy(), np.int64)
    h = L.handle()
    L.check(L.lib().pgld_hap_window_snp_sums(h, ctypes.byref(panel([pk])), L.ptr(ii), n_idx,
                                             L.ptr(wb), L.ptr(we), n_win, L.ptr(off_d), int(stat),
                                             L.ptr(rows), L.ptr(cols), n_out, L.stream_ptr()), h)
    st = torch.zeros(1, dtype=torch.int32)
    L.check(L.lib().pgld_device_status(h, ctypes.cast(st.data_ptr(), ctypes.POINTER(
        ctypes.c_int32)), L.stream_ptr()), h)
    if int(st[0]):
        raise IndexError(f"window or SNP index out of range (device status {int(st[0])})")
    return rows[:n_out], cols[:n_out], off


def omega_from_sums(row, col):
    """Kim and Nielsen's omega of m sites from the row sums row[i] = sum over
    j > i and column sums col[j] = sum over i < j of the pair statistic (the
    upper triangle): for every split l = 3 .. m-2 the mean within the blocks
    [0, l) and [l, m) over the mean across them (ld_statistics.py:810-862);
    0.0 below 5 sites or where no split is defined."""
    row = np.asarray(row, np.float64)
    col = np.asarray(col, np.float64)
    m = row.size
    if m < 5:
        return 0.0
    A = np.cumsum(row)          # pairs with i < l: A[l - 1]
    left_all = np.cumsum(col)   # pairs with j < l: left_all[l - 1]
    total = A[-1]
    l = np.arange(3, m - 1)
    left = left_all[l - 1]
    cross = A[l - 1] - left
    right = total - A[l - 1]
    n_left = l * (l - 1) // 2
    n_right = (m - l) * (m - l - 1) // 2
    n_cross = l * (m - l)
    n_within = n_left + n_right
    valid = (n_within > 0) & (n_cross > 0) & (cross > 0)
    within = np.where(n_within > 0, (left + right) / np.maximum(n_within, 1), 0.0)
    across = np.where(n_cross > 0, cross / np.maximum(n_cross, 1), 1.0)
    vals = np.where(valid, within / np.where(valid, across, 1.0), 0.0)
    return float(vals.max()) if vals.size else 0.0


def tc_applies(pops):
    """The tensor-core form takes 1-2 populations of <= 2048 haplotypes (0/1/-1 codes)."""
    return len(pops) <= 2 and all(pk.n_words <= 64 and pk.valid_for_n is None for pk in pops)


def binned_sums(pops, pos_d, bins, max_dist=None, bin_coord=None, form="auto", anchors=None,
                _tuning=False):
    """(sums (n_bins, n_stats) float64 tensor, pair counts (n_bins,) int64).

    form: "tc" (tcgen05 tensor cores), "plain" (AND + popcount) or "auto"
    (tensor cores whenever they apply).  anchors: optional (begin, end) --
    only the pairs whose first SNP lies in [begin, end) are summed."""
    if form == "auto":
        form = "tc" if tc_applies(pops) else "plain"
    if form == "tc" and not _tuning:
        from . import autotune
        autotune.apply("binned2" if len(pops) == 2 else "binned1", [pk.n_words for pk in pops])
    torch = _torch()
    bins_np = np.asarray(bins, dtype=np.float64)
    if bins_np.ndim != 1 or len(bins_np) < 2:
        raise ValueError("bins must hold at least two edges")
    if np.any(np.diff(bins_np) <= 0):
        raise ValueError("bins must be strictly increasing")
    n_bins = len(bins_np) - 1
    P = len(pops)
    n_stats = {1: 3, 2: 15, 3: 45, 4: 105}[P]
    dev = pos_d.device
    bins_d = torch.as_tensor(bins_np, device=dev)
    sums = torch.empty((n_bins, n_stats), dtype=torch.float64, device=dev)
    cnt = torch.empty(n_bins, dtype=torch.int64, device=dev)
    md = float(bins_np[-1]) if max_dist is None else float(max_dist)
    bc = None if bin_coord is None else L.as_device(bin_coord, np.float64)
    h = L.handle()
    fm = L.FORM_TC if form == "tc" else L.FORM_PLAIN
    if anchors is None:
        L.check(L.lib().pgld_hap_binned_sums(h, ctypes.byref(panel(pops)), L.ptr(pos_d), md,
                                             L.ptr(bc), L.ptr(bins_d), n_bins, L.ptr(sums),
                                             L.ptr(cnt), fm, L.stream_ptr()), h)
    else:
        a0, a1 = (int(v) for v in anchors)
        L.check(L.lib().pgld_hap_binned_sums_range(h, ctypes.byref(panel(pops)), L.ptr(pos_d), md,
                                                   L.ptr(bc), L.ptr(bins_d), n_bins, a0, a1,
                                                   L.ptr(sums), L.ptr(cnt), fm, L.stream_ptr()), h)
    return sums, cnt


# --------------------------------------------------------------------------
# genotype (unphased diploid dosage) path
# --------------------------------------------------------------------------
MAX_GENO_N = 8192


class PackedGeno:
    """Dosage bit planes (g == 0, 1, 2) of one population.

    ``has_missing`` mirrors the reference's ``cp.any(g < 0)`` over the
    population's rows (ld_pipeline.py:253); ``has_other`` flags dosages above
    2, for which the validity plane and the planes of the values 3..8 (``ext``,
    folded into classes like the reference's counting kernel) are kept.
    """

    def __init__(self, planes, valid, n_words, n_rows, n_snp, has_missing, has_other, ext=None):
        self.planes = planes
        self.valid = valid
        self.ext = ext
        self.n_words = n_words
        self.n_rows = n_rows
        self.n_snp = n_snp
        self.has_missing = has_missing
        self.has_other = has_other

    @property
    def valid_for_n(self):
        """Validity plane when the pairwise n differs from the sum of the 9
        counts: dosages above 2 and missing data (with no missing data the
        reference's n is the sum of the counts, ld_pipeline.py:253-263)."""
        return self.valid if (self.has_other and self.has_missing) else None

    @property
    def ext_planes(self):
        return self.ext if self.has_other else None


def pack_geno(geno, rows=None):
    """Pack the rows of an int8 (n_individuals x M) device dosage matrix."""
    torch = _torch()
    g = L.as_device(geno, np.int8)
    if g.dim() != 2:
        raise ValueError("genotypes must be 2-D (n_individuals, n_variants)")
    n_total, n_snp = g.shape
    if rows is not None:
        rows_t = L.as_device(rows, np.int32)
        if rows_t.numel() and (int(rows_t.min()) < 0 or int(rows_t.max()) >= n_total):
            raise IndexError("population row index out of range")
        n_rows = rows_t.numel()
    else:
        rows_t = None
        n_rows = n_total
    if n_rows > MAX_GENO_N:
        raise ValueError(f"{n_rows} individuals exceed {MAX_GENO_N} per population")
    W = max(1, (n_rows + 31) // 32)
    planes = torch.empty((n_snp, 3 * W), dtype=torch.int32, device=g.device)
    valid = torch.empty((n_snp, W), dtype=torch.int32, device=g.device)
    flags = torch.zeros(2, dtype=torch.int32, device=g.device)
    ext = None
    if n_rows == 0:
        planes.zero_()
        valid.zero_()
    else:
        h = L.handle()
        L.check(L.lib().pgld_pack_genotypes(h, L.ptr(g), g.stride(0), n_snp, L.ptr(rows_t), n_rows,
                                            L.ptr(planes), L.ptr(valid), None, L.ptr(flags),
                                            L.stream_ptr()), h)
        if int(flags[1]):
            # dosages above 2: the planes of the values 3..8 as well
            ext = torch.empty((n_snp, 6 * W), dtype=torch.int32, device=g.device)
            L.check(L.lib().pgld_pack_genotypes(h, L.ptr(g), g.stride(0), n_snp, L.ptr(rows_t),
                                                n_rows, L.ptr(planes), L.ptr(valid), L.ptr(ext),
                                                L.ptr(flags), L.stream_ptr()), h)
    f = flags.cpu().numpy()
    return PackedGeno(planes, valid, W, n_rows, n_snp, bool(f[0]), bool(f[1]), ext)


def geno_panel(pops):
    pn = L.GenoPanel()
    pn.n_pops = len(pops)
    for p, pk in enumerate(pops):
        pn.n_words[p] = pk.n_words
        pn.planes[p] = pk.planes.data_ptr()
        v = pk.valid_for_n
        pn.valid[p] = v.data_ptr() if v is not None else None
        x = pk.ext_planes
        pn.ext[p] = x.data_ptr() if x is not None else None
    pn.n_snp = pops[0].n_snp
    return pn


def geno_counts_pairs(pk, idx_i, idx_j):
    """(counts int32 (N,9) n00..n22, n_valid int32 (N,) or None) for listed pairs."""
    torch = _torch()
    ii = L.as_device(idx_i, np.int32)
    jj = L.as_device(idx_j, np.int32)
    if ii.shape != jj.shape:
        raise ValueError("idx_i and idx_j must have the same shape")
    n = ii.numel()
    counts = torch.empty((n, 9), dtype=torch.int32, device=ii.device)
    nv = torch.empty(n, dtype=torch.int32, device=ii.device) if pk.has_missing else None
    if n:
        h = L.handle()
        L.check(L.lib().pgld_geno_counts_pairs(h, L.ptr(pk.planes), L.ptr(pk.valid_for_n),
                                               L.ptr(pk.ext_planes), pk.n_words, pk.n_snp, L.ptr(ii), L.ptr(jj), n,
                                               L.ptr(counts), 9, L.ptr(nv), L.stream_ptr()), h)
        st = torch.zeros(1, dtype=torch.int32)
        L.check(L.lib().pgld_device_status(h, ctypes.cast(st.data_ptr(), ctypes.POINTER(
            ctypes.c_int32)), L.stream_ptr()), h)
        if int(st[0]):
            raise IndexError("pair index out of range of the variant axis")
    return counts, nv


def geno_spec_terms(P):
    """[(stat, kind, pops, weight)] of the moments genotype table of P populations."""
    n_terms, n_stats = ctypes.c_int32(), ctypes.c_int32()
    L.check(L.lib().pgld_geno_stat_terms(P, None, 0, ctypes.byref(n_terms), ctypes.byref(n_stats)))
    arr = (L.Term * n_terms.value)()
    L.check(L.lib().pgld_geno_stat_terms(P, arr, n_terms.value, ctypes.byref(n_terms),
                                         ctypes.byref(n_stats)))
    return [(t.stat, t.kind, tuple(t.pops), t.weight) for t in arr], n_stats.value


GENO_BAND_COLUMNS = ("r2", "dd", "dz", "pi2")


def geno_band_pairs(pk, pos_d, max_dist, with_counts=True, with_stats=True,
                    columns=GENO_BAND_COLUMNS, form="auto"):
    """Fused per-pair genotype outputs over the distance band.

    Returns (counts (N,9) int32 or None, n_valid (N,) int32, stats (N,4)
    float32 = Rogers-Huff r^2, DD, Dz, pi2 or None); only the named columns
    are evaluated, the others hold 0.  form: "tc" (tensor-core counts),
    "plain" (AND + popcount) or "auto" (tensor cores unless a dosage above 2
    needs the extra planes)."""
    if form == "auto":
        form = "plain" if pk.has_other else "tc"
    mask = 0
    for c in columns:
        if c not in GENO_BAND_COLUMNS:
            raise ValueError(f"unknown column {c!r}")
        mask |= 1 << GENO_BAND_COLUMNS.index(c)
    torch = _torch()
    n = band_pair_count(pos_d, max_dist)
    dev = pos_d.device
    counts = torch.empty((n, 9), dtype=torch.int32, device=dev) if with_counts else None
    nv = torch.empty(n, dtype=torch.int32, device=dev)
    st = torch.empty((n, 4), dtype=torch.float32, device=dev) if with_stats else None
    h = L.handle()
    L.check(L.lib().pgld_geno_band_pairs(h, ctypes.byref(geno_panel([pk])), L.ptr(pos_d),
                                         float(max_dist), L.ptr(counts), L.ptr(nv), L.ptr(st),
                                         mask, n, L.FORM_TC if form == "tc" else L.FORM_PLAIN,
                                         L.stream_ptr()), h)
    return counts, nv, st


def geno_tc_applies(pops):
    """The genotype tensor-core forms take dosages 0/1/2 with missing data
    (no values above 2) of 1-4 populations."""
    return 1 <= len(pops) <= 4 and all(pk.ext_planes is None for pk in pops)


def geno_binned_sums(pops, pos_d, bins, max_dist=None, bin_coord=None, form="auto"):
    """(sums (n_bins, n_stats) float64, pair counts (n_bins,) int64), genotype statistics.

    form: "tc" (moments from tcgen05 MMAs), "plain" (AND + popcount) or
    "auto" (tensor cores whenever they apply)."""
    if form == "auto":
        # several populations: the exact per-pair term table dominates
        # either form, and the popcount one measured slightly faster
        form = "tc" if len(pops) == 1 and geno_tc_applies(pops) else "plain"
    if form not in ("tc", "plain"):
        raise ValueError("form must be 'tc', 'plain' or 'auto'")
    torch = _torch()
    bins_np = np.asarray(bins, dtype=np.float64)
    if bins_np.ndim != 1 or len(bins_np) < 2:
        raise ValueError("bins must hold at least two edges")
    if np.any(np.diff(bins_np) <= 0):
        raise ValueError("bins must be strictly increasing")
    n_bins = len(bins_np) - 1
    n_stats = {1: 3, 2: 15, 3: 45, 4: 105}[len(pops)]
    dev = pos_d.device
    bins_d = torch.as_tensor(bins_np, device=dev)
    sums = torch.empty((n_bins, n_stats), dtype=torch.float64, device=dev)
    cnt = torch.empty(n_bins, dtype=torch.int64, device=dev)
    md = float(bins_np[-1]) if max_dist is None else float(max_dist)
    bc = None if bin_coord is None else L.as_device(bin_coord, np.float64)
    h = L.handle()
    L.check(L.lib().pgld_geno_binned_sums_form(h, ctypes.byref(geno_panel(pops)), L.ptr(pos_d), md,
                                               L.ptr(bc), L.ptr(bins_d), n_bins, L.ptr(sums),
                                               L.ptr(cnt), 1 if form == "tc" else 0,
                                               L.stream_ptr()), h)
    return sums, cnt


# --------------------------------------------------------------------------
# dense all-pairs outputs and distance-binned percentiles
# --------------------------------------------------------------------------
def pairwise_ld(pk, want_D=True, want_r2=True):
    """(D, r2) float64 (m, m) device matrices of one population (either None
    when not wanted): pgld_hap_pairwise_ld."""
    torch = _torch()
    m = pk.n_snp
    dev = pk.planes.device
    D = torch.empty((m, m), dtype=torch.float64, device=dev) if want_D else None
    r2 = torch.empty((m, m), dtype=torch.float64, device=dev) if want_r2 else None
    if m:
        h = L.handle()
        L.check(L.lib().pgld_hap_pairwise_ld(h, L.ptr(pk.planes), pk.n_words, m, L.ptr(D),
                                             L.ptr(r2), m, L.stream_ptr()), h)
    return D, r2


def pairs_by_bin(pos_d, bins, pk=None, pair_values=None):
    """(values grouped by bin: float64 device tensor, counts: host int64
    (n_bins,)) of every pair i < j with a non-NaN value -- its r^2 from the
    packed population pk, or pair_values (condensed upper triangle, device
    float64) -- binned by pos[j] - pos[i] (right-open bins)."""
    torch = _torch()
    bins_np = np.asarray(bins, dtype=np.float64)
    if bins_np.ndim != 1 or len(bins_np) < 2:
        raise ValueError("bins must hold at least two edges")
    n_bins = len(bins_np) - 1
    m = pos_d.numel()
    dev = pos_d.device
    bins_d = torch.as_tensor(bins_np, device=dev)
    pv = None if pair_values is None else L.as_device(pair_values, np.float64)
    if pv is not None and pv.numel() != m * (m - 1) // 2:
        raise ValueError("pair_values must hold the m (m - 1) / 2 pairs of the upper triangle")
    counts = np.zeros(n_bins, np.int64)
    h = L.handle()
    planes = None if pk is None else pk.planes
    W = 1 if pk is None else pk.n_words
    c_ptr = counts.ctypes.data_as(ctypes.c_void_p)
    L.check(L.lib().pgld_pairs_by_bin(h, L.ptr(planes), W, L.ptr(pv), m, L.ptr(pos_d),
                                      L.ptr(bins_d), n_bins, c_ptr, None, L.stream_ptr()), h)
    vals = torch.empty(max(int(counts.sum()), 1), dtype=torch.float64, device=dev)
    if counts.sum():
        L.check(L.lib().pgld_pairs_by_bin(h, L.ptr(planes), W, L.ptr(pv), m, L.ptr(pos_d),
                                          L.ptr(bins_d), n_bins, c_ptr, L.ptr(vals),
                                          L.stream_ptr()), h)
        st = torch.zeros(1, dtype=torch.int32)
        L.check(L.lib().pgld_device_status(h, ctypes.cast(st.data_ptr(), ctypes.POINTER(
            ctypes.c_int32)), L.stream_ptr()), h)
        if int(st[0]):
            raise RuntimeError(f"pairs changed between counting and filling (status {int(st[0])})")
    return vals[:int(counts.sum())], counts


def segment_kth(values, counts, targets):
    """Host float64 order statistics: targets = [(segment, rank), ...] of the
    segments of `values` whose lengths are `counts` (pgld_segment_kth)."""
    off = np.concatenate([[0], np.cumsum(np.asarray(counts, np.int64))]).astype(np.int64)
    tg = np.ascontiguousarray(np.asarray(targets, np.int64).reshape(-1, 2))
    out = np.zeros(len(tg), np.float64)
    if len(tg):
        h = L.handle()
        L.check(L.lib().pgld_segment_kth(h, L.ptr(values), off.ctypes.data_as(ctypes.c_void_p),
                                         len(off) - 1, tg.ctypes.data_as(ctypes.c_void_p),
                                         len(tg), out.ctypes.data_as(ctypes.c_void_p),
                                         L.stream_ptr()), h)
    return out


def percentiles_from_order_stats(counts, percentile, kth):
    """numpy.percentile (method 'linear') of segments of sizes `counts`,
    computed from the order statistics kth([(segment, rank), ...]) -> values,
    with numpy's own float64 steps: virtual index (n - 1) q, its floor and the
    next rank (both the last one at or above n - 1), and the interpolation
    a + (b - a) g, or b - (b - a)(1 - g) where g >= 0.5.  NaN where a segment
    is empty.  Returns (n_seg, n_pct)."""
    counts = np.asarray(counts, np.int64)
    q = np.true_divide(np.atleast_1d(np.asarray(percentile, np.float64)), 100)
    res = np.full((len(counts), len(q)), np.nan)
    plan, targets = [], {}
    for s, n in enumerate(counts):
        if n <= 0:
            continue
        for k, qq in enumerate(q):
            v = np.float64(n - 1) * qq
            prev = np.floor(v)
            if v >= n - 1:
                lo = hi = int(n - 1)
                g = v - np.float64(-1.0)
            elif v < 0:
                lo = hi = 0
                g = v - prev
            else:
                lo, hi = int(prev), int(prev) + 1
                g = v - prev
            plan.append((s, k, lo, hi, g))
            targets.setdefault((s, lo), None)
            targets.setdefault((s, hi), None)
    keys = list(targets)
    vals = kth(keys) if keys else []
    got = dict(zip(keys, vals))
    for s, k, lo, hi, g in plan:
        a, b = np.float64(got[(s, lo)]), np.float64(got[(s, hi)])
        d = b - a
        res[s, k] = (b - d * (1 - g)) if g >= 0.5 else (a + d * g)
    return res
