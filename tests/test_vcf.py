"""Native VCF GT reader (pgld_vcf_scan / pgld_vcf_parse_gt) against the oracle's
restatement of allel.read_vcf's GT layout, and HaplotypeMatrix.from_vcf end to
end (haplotype_matrix.py:293-356).  Host code only: no GPU."""
import gzip
import os

import numpy as np
import pytest

from oracle import ld_oracle as O

pytest.importorskip("torch")
from pg_gpu_gb300 import _lib as L  # noqa: E402

pytestmark = pytest.mark.skipif(not os.path.exists(L.LIB_PATH), reason="libpgld.so not built")

HEADER = "##fileformat=VCFv4.2\n##contig=<ID=chr1>\n"
COLS = "#CHROM\tPOS\tID\tREF\tALT\tQUAL\tFILTER\tINFO\tFORMAT"


def _vcf(names, records, eol="\n"):
    lines = HEADER.rstrip("\n").split("\n") + [COLS + "".join("\t" + n for n in names)]
    for chrom, pos, fmt, gts in records:
        lines.append("\t".join([chrom, str(pos), ".", "A", "T", ".", "PASS", ".", fmt] + gts))
    return eol.join(lines) + eol


def _edge_text(eol="\n"):
    names = ["s0", "s1", "s2", "s3"]
    recs = [
        ("chr1", 100, "GT", ["0|1", "1|1", "0|0", "1|0"]),
        ("chr1", 250, "GT:DP:GQ", ["0/1:12:99", "./.:0:0", "1/1:3:20", "0|.:4:5"]),
        ("chr1", 300, "GT", [".|.", "0", "1", "."]),         # missing and haploid calls
        ("chr1", 1000, "GT:AD", ["2|0:1,2", "0|3:4,5", "12|1:0,0", "0|200:1,1"]),
        ("chr2", 50, "GT", ["1|1", "0|0", "1|0", "0|1"]),
    ]
    return names, _vcf(names, recs, eol)


def _native(text, samples=None):
    import ctypes
    data = text.encode()
    ns, nr = ctypes.c_int32(0), ctypes.c_int64(0)
    L.check(L.lib().pgld_vcf_scan(data, len(data), ctypes.byref(ns), ctypes.byref(nr)))
    from pg_gpu_gb300.haplotype_matrix import _vcf_sample_names
    names = _vcf_sample_names(data)
    cols = None if samples is None else np.array([names.index(s) for s in samples], np.int32)
    n_sel = ns.value if cols is None else len(cols)
    hap = np.full((2 * n_sel, nr.value), 99, np.int8)
    pos = np.zeros(nr.value, np.int64)
    rc = L.lib().pgld_vcf_parse_gt(data, len(data), ns.value, nr.value,
                                   None if cols is None else cols.ctypes.data_as(ctypes.c_void_p),
                                   n_sel, hap.ctypes.data_as(ctypes.c_void_p),
                                   pos.ctypes.data_as(ctypes.c_void_p))
    L.check(rc)
    return hap, pos


@pytest.mark.parametrize("eol", ["\n", "\r\n"])
def test_native_gt_matches_oracle_edge_cases(eol):
    names, text = _edge_text(eol)
    ref_names, ref_hap, ref_pos = O.read_vcf_gt(text)
    hap, pos = _native(text)
    assert ref_names == names
    assert np.array_equal(hap, ref_hap) and np.array_equal(pos, ref_pos)
    # spot values: missing, haploid, multi-digit and clipped alleles
    assert hap[1, 1] == -1 and hap[5, 1] == -1          # "./."
    assert hap[1, 2] == 0 and hap[5, 2] == -1           # "0" (haploid)
    assert hap[2, 3] == 12 and hap[7, 3] == 127         # "12|1", "0|200"


def test_native_sample_subset_matches_oracle():
    _, text = _edge_text()
    sub = ["s3", "s0"]
    ref_names, ref_hap, _ = O.read_vcf_gt(text, samples=sub)
    hap, _ = _native(text, samples=sub)
    assert ref_names == sub and np.array_equal(hap, ref_hap)


def test_native_rejects_malformed_text():
    import ctypes
    ns, nr = ctypes.c_int32(0), ctypes.c_int64(0)
    data = b"##fileformat=VCFv4.2\nchr1\t1\t.\tA\tT\t.\t.\t.\tGT\t0|1\n"   # no #CHROM line
    assert L.lib().pgld_vcf_scan(data, len(data), ctypes.byref(ns), ctypes.byref(nr)) != 0
    names, text = _edge_text()
    short = text.replace("\t1|0\n", "\n", 1).encode()                     # a record short a sample
    L.check(L.lib().pgld_vcf_scan(short, len(short), ctypes.byref(ns), ctypes.byref(nr)))
    hap = np.zeros((2 * ns.value, nr.value), np.int8)
    pos = np.zeros(nr.value, np.int64)
    assert L.lib().pgld_vcf_parse_gt(short, len(short), ns.value, nr.value, None, ns.value,
                                     hap.ctypes.data_as(ctypes.c_void_p),
                                     pos.ctypes.data_as(ctypes.c_void_p)) != 0
    bad = np.array([7], np.int32)                                          # sample out of range
    assert L.lib().pgld_vcf_parse_gt(short, len(short), ns.value, nr.value,
                                     bad.ctypes.data_as(ctypes.c_void_p), 1,
                                     hap.ctypes.data_as(ctypes.c_void_p),
                                     pos.ctypes.data_as(ctypes.c_void_p)) != 0


def test_from_vcf_gzip_region_and_samples(tmp_path):
    from pg_gpu_gb300 import HaplotypeMatrix
    names, text = _edge_text()
    p = tmp_path / "edge.vcf.gz"
    with gzip.open(p, "wt") as f:
        f.write(text)
    hm = HaplotypeMatrix.from_vcf(str(p))
    _, ref_hap, ref_pos = O.read_vcf_gt(text)
    assert np.array_equal(np.asarray(hm.haplotypes), ref_hap)
    assert np.array_equal(np.asarray(hm.positions), ref_pos) and hm.samples == names
    assert (hm.chrom_start, hm.chrom_end) == (100, 50)    # first and last record
    # region: chr1 records in [200, 1000], bounds from the region string
    hm = HaplotypeMatrix.from_vcf(str(p), region="chr1:200-1,000", samples=["s2", "s1"])
    _, ref_hap, ref_pos = O.read_vcf_gt(text, samples=["s2", "s1"])
    keep = np.array([False, True, True, True, False])
    assert np.array_equal(np.asarray(hm.haplotypes), ref_hap[:, keep])
    assert np.array_equal(np.asarray(hm.positions), ref_pos[keep])
    assert (hm.chrom_start, hm.chrom_end) == (200, 1000) and hm.samples == ["s2", "s1"]
    with pytest.raises(ValueError):
        HaplotypeMatrix.from_vcf(str(p), region="chr3")
    with pytest.raises(ValueError):
        HaplotypeMatrix.from_vcf(str(p), samples=["nope"])


def test_from_vcf_round_trips_moments_im_haplotypes(golden, tmp_path):
    """The im-parsing-example haplotypes of the moments golden fixture written
    back as phased VCF text read back identically."""
    from pg_gpu_gb300 import HaplotypeMatrix
    z = golden("moments_im")
    hap, pos = z["hap"], z["pos"]
    n = hap.shape[0] // 2
    names = [f"tsk_{k}" for k in range(n)]
    al = lambda a: "." if a < 0 else str(int(a))  # noqa: E731
    recs = [("1", int(pos[j]), "GT", [al(hap[k, j]) + "|" + al(hap[n + k, j]) for k in range(n)])
            for j in range(hap.shape[1])]
    p = tmp_path / "im.vcf"
    p.write_text(_vcf(names, recs))
    hm = HaplotypeMatrix.from_vcf(str(p))
    assert np.array_equal(np.asarray(hm.haplotypes), hap)
    assert np.array_equal(np.asarray(hm.positions), pos) and hm.samples == names


def test_genotype_from_vcf_matches_oracle(tmp_path):
    from pg_gpu_gb300 import GenotypeMatrix
    names, text = _edge_text()
    # add a monomorphic site, an all-missing site and a biallelic site with a missing call
    extra = _vcf(names, [("chr2", 60, "GT", ["0|0", "0/0", "0|0", "0|0"]),
                         ("chr2", 70, "GT", [".|.", "./.", ".", ".|."]),
                         ("chr2", 80, "GT", ["0|1", "./1", "1|1", "0"])])
    text += extra.split(COLS)[1].split("\n", 1)[1]
    p = tmp_path / "g.vcf"
    p.write_text(text)
    gm = GenotypeMatrix.from_vcf(str(p))
    ref_names, ref_g, ref_pos = O.vcf_dosages(text)
    assert gm.samples == ref_names
    assert np.array_equal(np.asarray(gm.genotypes), ref_g)
    assert np.array_equal(np.asarray(gm.positions), ref_pos)
    assert list(ref_pos) == [100, 250, 300, 50, 80]   # 1000 (alleles 2..), 60, 70 dropped


def _accessible_loop(pos, intervals, chrom=None):
    """Direct restatement of the reference's BED mask (accessible.py:167-197):
    (start, end) covers the 1-based positions start + 1 .. end."""
    out = []
    for p in pos:
        out.append(any(s + 1 <= p <= e for c, s, e in intervals if chrom is None or c == chrom))
    return np.array(out, bool)


def test_accessible_filter_matches_loop(tmp_path):
    from pg_gpu_gb300 import accessible as A
    rng = np.random.default_rng(3)
    bed = tmp_path / "acc.bed"
    iv = []
    for c in ("chr1", "chr2"):
        starts = np.sort(rng.choice(10_000, 40, replace=False))
        for s in starts:
            iv.append((c, int(s), int(s + rng.integers(0, 300))))
    with open(bed, "w") as f:
        f.write("track name=acc\n# comment\n")
        for c, s, e in iv:
            f.write(f"{c}\t{s}\t{e}\textra\n")
    assert A.parse_bed(str(bed)) == iv
    pos = np.sort(rng.choice(np.arange(1, 10_500), 2_000, replace=False))
    for chrom in (None, "chr1", "chr2"):
        assert np.array_equal(A.accessible_variants(pos, str(bed), chrom),
                              _accessible_loop(pos, iv, chrom))
        # the interval list form gives the same mask
        assert np.array_equal(A.accessible_variants(pos, iv, chrom),
                              _accessible_loop(pos, iv, chrom))
    # no interval for the chromosome: an error for a file (the reference's
    # resolve_accessible_mask), an empty mask for an interval list
    with pytest.raises(ValueError):
        A.accessible_variants(pos, str(bed), "chr9")
    assert not A.accessible_variants(pos, iv, "chr9").any()


def test_from_vcf_accessible_bed(tmp_path):
    from pg_gpu_gb300 import GenotypeMatrix, HaplotypeMatrix
    names, text = _edge_text()
    p = tmp_path / "e.vcf"
    p.write_text(text)
    bed = tmp_path / "a.bed"
    bed.write_text("chr1\t99\t100\nchr1\t299\t1000\nchr2\t0\t60\n")
    hm = HaplotypeMatrix.from_vcf(str(p), accessible_bed=str(bed))
    # the mask is built from the intervals of the first record's chromosome
    # (chr1): POS 100, 300 and 1000 are accessible, 250 is not, and the chr2
    # record at POS 50 is not covered by a chr1 interval
    assert list(np.asarray(hm.positions)) == [100, 300, 1000]
    gm = GenotypeMatrix.from_vcf(str(p), accessible_bed=str(bed))
    assert list(np.asarray(gm.positions)) == [100, 300]  # 1000 is multi-allelic
    hm = HaplotypeMatrix.from_vcf(str(p), region="chr2", accessible_bed=str(bed))
    assert list(np.asarray(hm.positions)) == [50]
    # n_total_sites: the BED-accessible bases of the analysis range
    # [chrom_start, chrom_end] (haplotype_matrix.py:196-205), counted directly
    for m, chrom, iv in ((HaplotypeMatrix.from_vcf(str(p), accessible_bed=str(bed)), "chr1",
                          [(99, 100), (299, 1000)]),
                         (GenotypeMatrix.from_vcf(str(p), accessible_bed=str(bed)), "chr1",
                          [(99, 100), (299, 1000)]),
                         (HaplotypeMatrix.from_vcf(str(p), region="chr2",
                                                   accessible_bed=str(bed)), "chr2", [(0, 60)])):
        cs, ce = m.chrom_start, m.chrom_end
        want = sum(1 for x in range(cs, ce + 1) if any(s < x <= e for s, e in iv))
        assert m.n_total_sites == want, (chrom, cs, ce)
    # a BED without intervals for the chromosome is an error, as in the
    # reference (accessible.py:232-235), not an empty mask
    other = tmp_path / "b.bed"
    other.write_text("chr3\t0\t1000\n")
    with pytest.raises(ValueError, match="No BED intervals"):
        HaplotypeMatrix.from_vcf(str(p), accessible_bed=str(other))
    with pytest.raises(ValueError, match="No BED intervals"):
        GenotypeMatrix.from_vcf(str(p), accessible_bed=str(other))


def _pack_native(text, sets):
    """pgld_vcf_pack_gt of text for the row lists sets (list of lists)."""
    import ctypes
    data = text.encode()
    ns, nr = ctypes.c_int32(0), ctypes.c_int64(0)
    L.check(L.lib().pgld_vcf_scan(data, len(data), ctypes.byref(ns), ctypes.byref(nr)))
    rows = np.ascontiguousarray(np.concatenate([np.asarray(r, np.int32) for r in sets]
                                               or [np.zeros(0, np.int32)]), np.int32)
    off = np.zeros(len(sets) + 1, np.int32)
    off[1:] = np.cumsum([len(r) for r in sets])
    Ws = [max(1, (len(r) + 31) // 32) for r in sets]
    n = nr.value
    planes = np.full(2 * n * sum(Ws), 0xDEADBEEF, np.uint32)
    valid = np.full(n * sum(Ws), 0xDEADBEEF, np.uint32)
    site = np.zeros(n, np.uint8)
    popf = np.zeros((n, len(sets)), np.uint8)
    pos = np.zeros(n, np.int64)
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    rc = L.lib().pgld_vcf_pack_gt(data, len(data), ns.value, n, vp(rows), vp(off), len(sets),
                                  vp(planes), vp(valid), vp(site), vp(popf), vp(pos))
    L.check(rc)
    out, wb = [], 0
    for k, W in enumerate(Ws):
        out.append((planes[2 * n * wb:2 * n * (wb + W)].reshape(n, 2 * W),
                    valid[n * wb:n * (wb + W)].reshape(n, W)))
        wb += W
    return out, site, popf, pos


def _planes_of(hap, rows):
    """Carrier / reference / validity words of hap's rows (bit k of word w: row 32 w + k)."""
    sub = hap[np.asarray(rows, np.int64)] if len(rows) else np.zeros((0, hap.shape[1]), np.int8)
    M = hap.shape[1]
    W = max(1, (len(rows) + 31) // 32)
    c, z, v = (np.zeros((M, W), np.uint32) for _ in range(3))
    for k in range(len(rows)):
        w, b = divmod(k, 32)
        c[:, w] |= (sub[k] == 1).astype(np.uint32) << np.uint32(b)
        z[:, w] |= (sub[k] == 0).astype(np.uint32) << np.uint32(b)
        v[:, w] |= (sub[k] >= 0).astype(np.uint32) << np.uint32(b)
    flags = (np.any(sub == -1, 0).astype(np.uint8)
             | (np.any((sub != -1) & (sub != 0) & (sub != 1), 0).astype(np.uint8) << 1))
    return np.concatenate([c, z], 1), v, flags


def _random_vcf(rng, n_samples, n_records):
    names = [f"ind{k}" for k in range(n_samples)]
    alle = lambda: rng.choice(["0", "1", ".", "2", "13"], p=[0.45, 0.4, 0.08, 0.05, 0.02])  # noqa: E731
    recs = []
    for j in range(n_records):
        gts = []
        for _ in range(n_samples):
            u = rng.random()
            if u < 0.03:
                gts.append(alle())                       # haploid call
            else:
                gts.append(alle() + ("|" if u < 0.6 else "/") + alle() + (":7" if u > 0.9 else ""))
        recs.append(("chr1", 10 * j + 5, "GT:DP" if j % 3 == 0 else "GT", gts))
    return names, _vcf(names, recs)


@pytest.mark.parametrize("case", ["edge", "random"])
def test_pack_gt_matches_packing_of_the_int8_matrix(case):
    """Packing straight from the GT text equals packing the int8 matrix the
    text parses to: carrier / reference / validity words of every population
    (overlapping, empty, more than 32 rows, any row order), the per-site and
    per-population flags and POS."""
    rng = np.random.default_rng(11)
    if case == "edge":
        names, text = _edge_text()
    else:
        names, text = _random_vcf(rng, 45, 70)
    n = len(names)
    hap, pos = _native(text)
    sets = [list(range(0, 2 * n, 2)), [], list(rng.permutation(2 * n)[:37]), [2 * n - 1, 0, n],
            list(range(2 * n))]
    got, site, popf, gpos = _pack_native(text, sets)
    assert np.array_equal(gpos, pos)
    for k, rows in enumerate(sets):
        pl, va, fl = _planes_of(hap, rows)
        assert np.array_equal(got[k][0], pl), k
        assert np.array_equal(got[k][1], va), k
        assert np.array_equal(popf[:, k], fl), k
    want_site = ((np.any(hap == 0, 0).astype(np.uint8)) | (np.any(hap == 1, 0).astype(np.uint8) << 1)
                 | (np.any(hap >= 2, 0).astype(np.uint8) << 2)
                 | (np.any(hap < 0, 0).astype(np.uint8) << 3))
    assert np.array_equal(site, want_site)


def test_pack_gt_rejects_bad_rows_and_records():
    import ctypes
    names, text = _edge_text()
    with pytest.raises(Exception):
        _pack_native(text, [[0, 2 * len(names)]])      # a haplotype index past the samples
    bad = text.replace("0|1\t1|1\t0|0\t1|0", "0|1\t1|1", 1)  # a record with too few fields
    with pytest.raises(Exception):
        _pack_native(bad, [[0, 1]])
    data = text.encode()
    z = np.zeros(4, np.int32)
    assert L.lib().pgld_vcf_pack_gt(data, len(data), 4, 5, None, None, 1, None, None, None,
                                    None, z.ctypes.data_as(ctypes.c_void_p)) != 0
