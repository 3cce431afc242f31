"""HaplotypeMatrix: the reference container and its LD methods on libpgld.

Mirrors pg_gpu.haplotype_matrix.HaplotypeMatrix (haplotype_matrix.py:34-170)
for the data it holds (an int8 (n_haplotypes, n_variants) matrix with 1 / 0 /
-1, sorted positions, named sample sets) and re-implements its two-locus LD
methods (haplotype_matrix.py:1092-1866).  'GPU' storage is a CUDA torch
tensor; packed bit planes of each population are cached after first use.
"""
from __future__ import annotations

import ctypes
import gzip
from collections import OrderedDict

import numpy as np

from . import _lib as L
from . import _ops


def _is_torch(x):
    try:
        import torch
        return isinstance(x, torch.Tensor)
    except ImportError:
        return False


def _parse_region(region):
    """('chrom', start or None, end or None) of 'chrom[:start[-end]]'."""
    chrom, _, rng = region.partition(":")
    lo = hi = None
    if rng:
        a, _, b = rng.partition("-")
        lo = int(a.replace(",", "")) if a else None
        hi = int(b.replace(",", "")) if b else None
    return chrom, lo, hi


def _vcf_region(data, region):
    """The VCF text with only the header lines and the records of region."""
    chrom, lo, hi = _parse_region(region)
    c = chrom.encode()
    keep = []
    for line in data.split(b"\n"):
        if line.startswith(b"#"):
            keep.append(line)
            continue
        f = line.split(b"\t", 2)
        if len(f) < 2 or f[0] != c:
            continue
        p = int(f[1])
        if (lo is None or p >= lo) and (hi is None or p <= hi):
            keep.append(line)
    return b"\n".join(keep)


def vcf_first_chrom(path):
    """CHROM of the first data record of a plain or gzipped VCF (or None)."""
    with open(path, "rb") as f:
        gz = f.read(2) == b"\x1f\x8b"
    opener = gzip.open if gz else open
    with opener(path, "rb") as f:
        for line in f:
            if not line.startswith(b"#") and line.strip():
                return line.split(b"\t", 1)[0].decode()
    return None


def _vcf_sample_names(data):
    """Sample names of the #CHROM header line."""
    i = data.find(b"#CHROM")
    line = data[i:data.find(b"\n", i) if data.find(b"\n", i) >= 0 else len(data)]
    return [x.decode() for x in line.rstrip(b"\r").split(b"\t")[9:]]


def read_vcf_gt(path, region=None, samples=None):
    """(sample names, int8 haplotypes (2 n, M), int64 POS) of a plain or
    gzipped VCF through the native GT reader (pgld_vcf_scan /
    pgld_vcf_parse_gt): row k = first allele of sample k, row n + k its
    second, -1 = missing (the calldata/GT layout of allel.read_vcf that
    haplotype_matrix.py:317-328 reshapes)."""
    data = _read_vcf_text(path, region)
    ns, nr = ctypes.c_int32(0), ctypes.c_int64(0)
    L.check(L.lib().pgld_vcf_scan(data, len(data), ctypes.byref(ns), ctypes.byref(nr)))
    names = _vcf_sample_names(data)
    if nr.value == 0:
        raise ValueError(f"No variants found in {path}"
                         + (f" for region {region}" if region else ""))
    cols = None
    if samples is not None:
        missing = [s for s in samples if s not in names]
        if missing:
            raise ValueError(f"samples not in {path}: {missing}")
        cols = np.ascontiguousarray([names.index(s) for s in samples], np.int32)
        names = list(samples)
    n_sel = len(names)
    hap = np.empty((2 * n_sel, nr.value), np.int8)
    pos = np.empty(nr.value, np.int64)
    L.check(L.lib().pgld_vcf_parse_gt(
        data, len(data), ns.value, nr.value,
        None if cols is None else cols.ctypes.data_as(ctypes.c_void_p), n_sel,
        hap.ctypes.data_as(ctypes.c_void_p), pos.ctypes.data_as(ctypes.c_void_p)))
    return names, hap, pos


def _read_vcf_text(path, region=None):
    with open(path, "rb") as f:
        data = f.read()
    if data[:2] == b"\x1f\x8b":
        data = gzip.decompress(data)
    if region is not None:
        data = _vcf_region(data, region)
    return data


def pop_file_sets(pop_file, names, pops=None):
    """{pop: haplotype rows} of a sample / pop file over the VCF samples
    `names`: sample i owns rows i and i + len(names), in the order of
    HaplotypeMatrix.load_pop_file (haplotype_matrix.py:475-512)."""
    n = len(names)
    pop_map = {}
    with open(pop_file) as f:
        for line in f:
            parts = line.strip().split()
            if len(parts) >= 2 and parts[0] != "sample":
                pop_map[parts[0]] = parts[1]
    if pops is None:
        pops = sorted(set(pop_map.values()))
    sets = {p: [] for p in pops}
    for i, name in enumerate(names):
        p = pop_map.get(name)
        if p in sets:
            sets[p].append(i)
            sets[p].append(i + n)
    return sets


class PackedVcf:
    """Populations of a VCF packed straight from the GT text into bit planes
    (pgld_vcf_pack_gt), without the int8 haplotype matrix.

    ``packs``: {pop: PackedPop} on the device; ``positions``: int64 POS;
    ``site_flags``: uint8 per site over every haplotype of the VCF (bit 0 an
    allele 0, bit 1 an allele 1, bit 2 an allele >= 2, bit 3 missing);
    ``pop_flags``: uint8 (n_sites, n_pops) (bit 0 missing, bit 1 an allele
    outside {0, 1}); ``sample_sets``: {pop: rows}."""

    def __init__(self, names, sample_sets, packs, positions, site_flags, pop_flags):
        self.samples = names
        self.sample_sets = sample_sets
        self.packs = packs
        self.positions = positions
        self.site_flags = site_flags
        self.pop_flags = pop_flags

    @property
    def num_variants(self):
        return len(self.positions)

    def biallelic_sites(self):
        """Sites with an allele 0, an allele 1 and no allele >= 2 over every
        haplotype (HaplotypeMatrix.apply_biallelic_filter,
        haplotype_matrix.py:724-789)."""
        f = self.site_flags
        return ((f & 4) == 0) & ((f & 1) != 0) & ((f & 2) != 0)

    def subset(self, keep):
        """The sites where the boolean mask keep is True (planes gathered on
        the device; population flags recomputed over the kept sites)."""
        import torch
        idx = np.nonzero(np.asarray(keep, bool))[0]
        idx_d = torch.as_tensor(idx, dtype=torch.int64, device="cuda")
        packs = {}
        pf = self.pop_flags[idx]
        for k, (p, pk) in enumerate(self.packs.items()):
            f = np.bitwise_or.reduce(pf[:, k]) if len(idx) else 0
            packs[p] = _ops.PackedPop(pk.planes.index_select(0, idx_d).contiguous(),
                                      pk.valid.index_select(0, idx_d).contiguous(), pk.n_words,
                                      pk.n_rows, len(idx), bool(f & 1), bool(f & 2))
        return PackedVcf(self.samples, self.sample_sets, packs, self.positions[idx],
                         self.site_flags[idx], pf)

    def alt_counts(self, pop):
        """float64 device (n_sites,): carriers of allele 1 among the
        population's haplotypes (popcount of its carrier plane)."""
        import torch
        pk = self.packs[pop]
        words = pk.planes[:, :pk.n_words].contiguous()
        b = words.view(torch.uint8).to(torch.int64)
        table = torch.tensor([bin(v).count("1") for v in range(256)], dtype=torch.int64,
                             device=b.device)
        return table[b].sum(1).to(torch.float64)


def read_vcf_packed(path, pop_file, pops=None, region=None):
    """PackedVcf of a plain or gzipped VCF: the populations of pop_file
    (rows as load_pop_file gives them) packed on the host threads straight
    from the GT text into carrier / reference / validity planes (no int8
    haplotype matrix), then copied to the device."""
    import torch
    data = _read_vcf_text(path, region)
    ns, nr = ctypes.c_int32(0), ctypes.c_int64(0)
    L.check(L.lib().pgld_vcf_scan(data, len(data), ctypes.byref(ns), ctypes.byref(nr)))
    if nr.value == 0:
        raise ValueError(f"No variants found in {path}"
                         + (f" for region {region}" if region else ""))
    names = _vcf_sample_names(data)
    sets = pop_file_sets(pop_file, names, pops)
    order = list(sets)
    rows = np.ascontiguousarray(np.concatenate(
        [np.asarray(sets[p], np.int32) for p in order] or [np.zeros(0, np.int32)]), np.int32)
    off = np.zeros(len(order) + 1, np.int32)
    off[1:] = np.cumsum([len(sets[p]) for p in order])
    Ws = [max(1, (len(sets[p]) + 31) // 32) for p in order]
    n_rec = nr.value
    planes = np.empty(2 * n_rec * max(1, sum(Ws)), np.uint32)
    valid = np.empty(n_rec * max(1, sum(Ws)), np.uint32)
    site = np.empty(n_rec, np.uint8)
    popf = np.empty((n_rec, max(1, len(order))), np.uint8)
    pos = np.empty(n_rec, np.int64)
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    L.check(L.lib().pgld_vcf_pack_gt(data, len(data), ns.value, n_rec, vp(rows), vp(off),
                                     len(order), vp(planes), vp(valid), vp(site), vp(popf),
                                     vp(pos)))
    packs = OrderedDict()
    wb = 0
    for k, p in enumerate(order):
        W = Ws[k]
        pl = torch.from_numpy(planes[2 * n_rec * wb:2 * n_rec * (wb + W)].view(np.int32))
        va = torch.from_numpy(valid[n_rec * wb:n_rec * (wb + W)].view(np.int32))
        f = np.bitwise_or.reduce(popf[:, k])
        packs[p] = _ops.PackedPop(pl.view(n_rec, 2 * W).to("cuda"), va.view(n_rec, W).to("cuda"),
                                  W, len(sets[p]), n_rec, bool(f & 1), bool(f & 2))
        wb += W
    return PackedVcf(names, sets, packs, pos, site, popf[:, :len(order)])


class HaplotypeMatrix:
    def __init__(self, genotypes, positions, chrom_start=None, chrom_end=None,
                 sample_sets=None, n_total_sites=None, samples=None, accessible_mask=None):
        g_dev = _is_torch(genotypes) or hasattr(genotypes, "__cuda_array_interface__")
        if not g_dev and not isinstance(genotypes, np.ndarray):
            raise ValueError("genotypes must be a numpy array or a CUDA array")
        size = genotypes.numel() if _is_torch(genotypes) else np.asarray(genotypes).size \
            if not g_dev else int(np.prod(genotypes.shape))
        if size == 0:
            raise ValueError("genotypes cannot be empty")
        if len(positions) == 0:
            raise ValueError("positions cannot be empty")
        # a pinned int8 CPU tensor stays on the host: the LD methods pack it in
        # place (the packing kernel reads it over the host link); other
        # methods copy it to the device on first use, like a numpy matrix
        self._pinned = genotypes if _ops._host_readable(genotypes) else None
        if self._pinned is not None:
            self._device = "CPU"
            self._haplotypes = genotypes.numpy()
            self._positions = np.asarray(positions.cpu().numpy() if _is_torch(positions)
                                         else positions)
        elif g_dev:
            self._device = "GPU"
            self._haplotypes = L.as_device(genotypes, np.int8)
            self._positions = L.as_device(positions)
        else:
            self._device = "CPU"
            self._haplotypes = np.asarray(genotypes)
            self._positions = np.asarray(positions.cpu().numpy() if _is_torch(positions)
                                         else positions)
        self.chrom_start = chrom_start
        self.chrom_end = chrom_end
        self._sample_sets = None
        if sample_sets is not None:
            self.sample_sets = sample_sets
        self.n_total_sites = n_total_sites
        self.samples = samples
        self.accessible_mask = accessible_mask
        self._packed = {}

    # ------------------------------------------------------------------ data
    @property
    def haplotypes(self):
        return self._haplotypes

    @haplotypes.setter
    def haplotypes(self, value):
        self._haplotypes = value
        self._pinned = None
        self._packed = {}

    @property
    def positions(self):
        return self._positions

    @positions.setter
    def positions(self, value):
        self._positions = value

    @property
    def device(self):
        return self._device

    @property
    def num_haplotypes(self):
        return int(self._haplotypes.shape[0])

    @property
    def num_variants(self):
        return int(self._haplotypes.shape[1])

    @property
    def shape(self):
        return tuple(self._haplotypes.shape)

    @property
    def sample_sets(self):
        if self._sample_sets is None:
            return {"all": list(range(self.num_haplotypes))}
        return self._sample_sets

    @sample_sets.setter
    def sample_sets(self, sample_sets):
        if not isinstance(sample_sets, dict):
            raise ValueError("sample_sets must be a dictionary")
        for v in sample_sets.values():
            if not isinstance(v, list):
                raise ValueError("values in sample_sets must be lists")
        self._sample_sets = sample_sets
        self._packed = {}

    def transfer_to_gpu(self):
        if self._device == "CPU":
            self._haplotypes = L.as_device(self._haplotypes, np.int8)
            self._positions = L.as_device(self._positions)
            self._device = "GPU"

    def transfer_to_cpu(self):
        if self._device == "GPU":
            self._haplotypes = self._haplotypes.cpu().numpy()
            self._positions = self._positions.cpu().numpy()
            self._device = "CPU"
            self._packed = {}

    def _pos_np(self):
        p = self._positions
        return p.cpu().numpy() if _is_torch(p) else np.asarray(p)

    def get_subset(self, positions_idx):
        idx = np.asarray(positions_idx.cpu().numpy() if _is_torch(positions_idx)
                         else positions_idx)
        if self._device == "GPU":
            import torch
            ti = torch.as_tensor(idx, device=self._haplotypes.device, dtype=torch.int64)
            hap = self._haplotypes.index_select(1, ti)
            pos = self._positions.index_select(0, ti)
        else:
            hap = self._haplotypes[:, idx]
            pos = self._positions[idx]
        return HaplotypeMatrix(hap, pos, self.chrom_start, self.chrom_end, self._sample_sets,
                               self.n_total_sites, self.samples)

    def apply_biallelic_filter(self):
        """Keep sites with both 0 and 1 and no value >= 2 (haplotype_matrix.py:724-789)."""
        if self._device == "GPU":
            h = self._haplotypes
            keep = ((h >= 2).sum(0) == 0) & ((h == 0).sum(0) > 0) & ((h == 1).sum(0) > 0)
            idx = keep.nonzero().flatten()
        else:
            h = self._haplotypes
            keep = (np.sum(h >= 2, 0) == 0) & (np.sum(h == 0, 0) > 0) & (np.sum(h == 1, 0) > 0)
            idx = np.where(keep)[0]
        out = self.get_subset(idx)
        if len(idx):
            pos = out._pos_np()
            out.chrom_start, out.chrom_end = int(pos[0]), int(pos[-1])
        return out

    @classmethod
    def from_vcf(cls, path, region=None, samples=None, include_invariant=False,
                 accessible_bed=None):
        """GT of a plain or gzipped VCF through the native reader; rows = all
        hap-0 then all hap-1 (haplotype_matrix.py:293-356).

        ``region`` ('chrom', 'chrom:start-end', 1-based inclusive) keeps the
        records inside it by a linear scan (no tabix index needed) and sets
        chrom_start / chrom_end from its bounds, as the reference does."""
        names, hap, pos = read_vcf_gt(path, region, samples)
        start, end = int(pos[0]), int(pos[-1])
        if region is not None:
            _, lo, hi = _parse_region(region)
            start = lo if lo is not None else start
            end = hi if hi is not None else end
        hm = cls(hap, pos, start, end, samples=names,
                 n_total_sites=len(pos) if include_invariant else None)
        if accessible_bed is not None:
            # variants at inaccessible positions are dropped (the reference
            # hides them behind a mask of the region's chromosome)
            from .accessible import accessible_variants
            chrom = _parse_region(region)[0] if region is not None else vcf_first_chrom(path)
            keep = accessible_variants(pos, accessible_bed, chrom or None)
            cs, ce = hm.chrom_start, hm.chrom_end
            hm = hm.get_subset(np.nonzero(keep)[0])
            # the per-base denominator: the BED's accessible bases in the range
            from .accessible import accessible_base_count
            hm.chrom_start, hm.chrom_end = cs, ce
            hm.n_total_sites = accessible_base_count(accessible_bed, chrom or None, cs, ce)
        return hm

    def load_pop_file(self, pop_file, pops=None):
        """Sample sets from a sample / pop file; sample i owns haplotype rows i and
        i + n_samples (haplotype_matrix.py:475-512)."""
        if self.samples is None:
            raise ValueError("No sample names stored. Use from_vcf() to load data.")
        self.sample_sets = pop_file_sets(pop_file, self.samples, pops)

    # ------------------------------------------------------------- packing
    def _pop_rows(self, pop):
        if pop is None:
            return None
        if self._sample_sets is None:
            raise ValueError("sample_sets must be defined to use pop parameter")
        if pop not in self._sample_sets:
            raise KeyError(f"Population key {pop} must exist in sample_sets")
        return self._sample_sets[pop]

    def packed(self, pop=None):
        """Cached bit planes of a population (None: every haplotype)."""
        src = self._pinned if (self._device == "CPU" and self._pinned is not None) else None
        if src is None:
            self.transfer_to_gpu()
            src = self._haplotypes
        key = pop
        if key not in self._packed:
            rows = self._pop_rows(pop)
            self._packed[key] = _ops.pack(src, rows)
        return self._packed[key]

    # ------------------------------------------------------------ LD methods
    def tally_gpu_haplotypes(self, pop=None):
        """All-pairs [n11,n10,n01,n00] and n_valid or None (haplotype_matrix.py:1320-1434).

        Exact at any sample size (the reference's no-missing int8 X.T@X wraps
        at 128 haplotypes)."""
        return _ops.tally(self.packed(pop))

    def tally_gpu_haplotypes_two_pops(self, pop1, pop2):
        """(counts (N,8), n_valid1, n_valid2) (haplotype_matrix.py:1518-1589)."""
        import torch
        if self._sample_sets is None:
            raise ValueError("sample_sets must be defined to use this function")
        if pop1 not in self._sample_sets or pop2 not in self._sample_sets:
            raise KeyError(f"Population keys {pop1} and {pop2} must exist in sample_sets")
        c1, nv1 = _ops.tally(self.packed(pop1))
        c2, nv2 = _ops.tally(self.packed(pop2))
        any_missing = bool((self._haplotypes == -1).any())
        if any_missing:
            nv1 = nv1 if nv1 is not None else c1.sum(1, dtype=torch.int32)
            nv2 = nv2 if nv2 is not None else c2.sum(1, dtype=torch.int32)
            return torch.cat([c1, c2], 1), nv1, nv2
        return torch.cat([c1, c2], 1), None, None

    def _binned(self, bp_bins, pops):
        bins = np.asarray(bp_bins, dtype=np.float64)
        packs = [self.packed(p) for p in pops]
        sums, cnt = _ops.binned_sums(packs, _ops.positions_f64(self._positions), bins)
        return bins, sums.cpu().numpy(), cnt.cpu().numpy()

    def compute_ld_statistics_gpu_single_pop(self, bp_bins, raw=False, ac_filter=True,
                                             chunk_size="auto"):
        """{(lo, hi): (DD, Dz, pi2)} sums or means per bin (haplotype_matrix.py:1592-1716)."""
        if ac_filter:
            return self.apply_biallelic_filter().compute_ld_statistics_gpu_single_pop(
                bp_bins, raw=raw, ac_filter=False, chunk_size=chunk_size)
        bins, sums, cnt = self._binned(bp_bins, [None])
        out = {}
        for i in range(len(bins) - 1):
            key = (float(bins[i]), float(bins[i + 1]))
            if raw:
                out[key] = tuple(float(v) for v in sums[i])
            elif cnt[i] > 0:
                out[key] = tuple(float(v) for v in sums[i] / cnt[i])
            else:
                out[key] = (0.0, 0.0, 0.0)
        return out

    def compute_ld_statistics_gpu_two_pops(self, bp_bins, pop1, pop2, raw=False,
                                           ac_filter=True, chunk_size="auto"):
        """{(lo, hi): OrderedDict of the 15 statistics} (haplotype_matrix.py:1719-1866)."""
        if ac_filter:
            return self.apply_biallelic_filter().compute_ld_statistics_gpu_two_pops(
                bp_bins, pop1, pop2, raw=raw, ac_filter=False, chunk_size=chunk_size)
        from .ld_pipeline import ld_names
        names = ld_names(2)
        bins, sums, cnt = self._binned(bp_bins, [pop1, pop2])
        out = {}
        for i in range(len(bins) - 1):
            key = (float(bins[i]), float(bins[i + 1]))
            if raw:
                out[key] = OrderedDict((n, float(v)) for n, v in zip(names, sums[i]))
            elif cnt[i] > 0:
                out[key] = OrderedDict((n, float(v) / cnt[i]) for n, v in zip(names, sums[i]))
            else:
                out[key] = OrderedDict((n, 0.0) for n in names)
        return out

    def windowed_r_squared(self, bp_bins, percentile=50, pop=None, estimator="r2"):
        """Percentiles of r^2 per distance bin and pair counts
        (haplotype_matrix.py:1235-1317).  The pairs' r^2 are grouped by bin on
        the device (pgld_pairs_by_bin) and each percentile is interpolated, as
        numpy.percentile does, between two order statistics found on the
        device (pgld_segment_kth); nothing per pair reaches the host."""
        if estimator == "rogers_huff":
            if pop is not None:
                raise NotImplementedError(
                    "windowed_r_squared(estimator='rogers_huff', pop=...) is not implemented; "
                    "subset the haplotypes first")
            from .ld_statistics import rogers_huff_r
            r = rogers_huff_r(self)
            vals, cnt = _ops.pairs_by_bin(_ops.positions_f64(self._positions), bp_bins,
                                          pair_values=r * r)
        elif estimator == "r2":
            pk = self.packed(pop)
            if pk.has_other:
                raise NotImplementedError("windowed_r_squared of non-biallelic codes")
            vals, cnt = _ops.pairs_by_bin(_ops.positions_f64(self._positions), bp_bins, pk=pk)
        else:
            raise ValueError(f"Unknown estimator: {estimator!r} (expected 'r2' or 'rogers_huff')")
        res = _ops.percentiles_from_order_stats(
            cnt, percentile, lambda keys: _ops.segment_kth(vals, cnt, keys))
        return (res[:, 0] if res.shape[1] == 1 else res), cnt.astype(int)

    def pairwise_r2(self, estimator="r2"):
        """(m, m) float64 r^2 with a zero diagonal (haplotype_matrix.py:1138-1170):
        'r2' from the joint and per-site frequencies on the device
        (pgld_hap_pairwise_ld); 'rogers_huff' the squared Rogers-Huff r of
        adjacent-haplotype dosages, NaN set to 0."""
        import torch
        if estimator == "rogers_huff":
            from .ld_statistics import rogers_huff_r
            r = rogers_huff_r(self)
            m = self.num_variants
            out = torch.zeros((m, m), dtype=torch.float64, device=r.device)
            ii, jj = torch.triu_indices(m, m, 1, device=r.device)
            r2 = torch.nan_to_num(r * r, nan=0.0)
            out[ii, jj] = r2
            out[jj, ii] = r2
            return out
        if estimator != "r2":
            raise ValueError(f"Unknown estimator: {estimator!r} (expected 'r2' or 'rogers_huff')")
        _, r2 = _ops.pairwise_ld(self._dense_packed(), want_D=False, want_r2=True)
        return r2

    def locate_unlinked(self, size=100, step=20, threshold=0.1):
        """Variants in approximate linkage equilibrium (haplotype_matrix.py:1172-1233):
        windows of `size` variants advanced by `step`; within a window an
        active variant j is dropped when its naive r^2 with an earlier active
        variant i exceeds threshold.  The naive r^2 of every pair closer than
        `size` variants comes from one band-pair call on the device (D =
        n11 / n - p_i p_j over the pair's valid haplotypes, p per site); the
        greedy pruning runs on the host, as in the reference."""
        import ctypes
        import torch
        size, step = int(size), int(step)
        if size < 1 or step < 1:
            raise ValueError("size and step must be positive")
        m = self.num_variants
        pk = self.packed(None)
        if pk.has_other:
            raise NotImplementedError("locate_unlinked of non-biallelic codes")
        dev = pk.planes.device
        pos_d = torch.arange(m, dtype=torch.float64, device=dev)
        off, n = _ops.band_offsets(pos_d, size - 1)
        counts, nv, _ = _ops.band_pairs(pk, pos_d, size - 1, with_stats=False)
        h = self._pinned if (self._device == "CPU" and self._pinned is not None) else None
        h = L.as_device(self._haplotypes if h is None else h, np.int8)
        dac = (h == 1).sum(0).to(torch.float64)
        nvs = (h >= 0).sum(0).to(torch.float64)
        p = torch.where(nvs > 0, dac / torch.where(nvs > 0, nvs, 1.0), 0.0)
        rows = torch.repeat_interleave(torch.arange(m, device=dev), off[1:] - off[:-1])
        k = torch.arange(n, device=dev)
        cols = rows + 1 + (k - off[:-1][rows])
        c = counts.to(torch.float64)
        nn = nv.to(torch.float64) if pk.has_missing else c.sum(1)
        D = torch.where(nn > 0, c[:, 0] / torch.where(nn > 0, nn, 1.0), 0.0) - p[rows] * p[cols]
        den = p[rows] * (1 - p[rows]) * p[cols] * (1 - p[cols])
        r2 = torch.where(den > 0, D * D / torch.where(den > 0, den, 1.0), 0.0)
        r2_h = np.ascontiguousarray(r2.cpu().numpy())
        off_h = np.ascontiguousarray(off.cpu().numpy())
        loc = np.zeros(m, dtype=np.uint8)
        hd = L.handle()
        L.check(L.lib().pgld_prune_unlinked(hd, r2_h.ctypes.data_as(ctypes.c_void_p),
                                            off_h.ctypes.data_as(ctypes.c_void_p), m, size, step,
                                            float(threshold),
                                            loc.ctypes.data_as(ctypes.c_void_p)), hd)
        return loc.astype(bool)

    def pairwise_LD_v(self):
        """(m, m) float64 D = pAB - pA pB with a zero diagonal
        (haplotype_matrix.py:1092-1136), on the device (pgld_hap_pairwise_ld)."""
        D, _ = _ops.pairwise_ld(self._dense_packed(), want_D=True, want_r2=False)
        return D

    def _dense_packed(self):
        pk = self.packed(None)
        if pk.has_other:
            raise NotImplementedError("pairwise LD of non-biallelic codes (apply the biallelic "
                                      "filter first)")
        return pk
