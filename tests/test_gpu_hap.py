"""GPU parity of the haplotype LD path against the reference fixtures and the oracle.

Counts are compared bit-for-bit.  float64 statistics come from exact integer
numerators divided once, so they match the reference to 1e-13 relative.
float32 per-pair statistics are held to 1e-6 relative of the float64 oracle.
Binned sums are held to |gpu - oracle| <= 2e-6 * sum|x| per bin and
statistic (float32 per-pair values, float64 accumulation).
"""
import itertools

import numpy as np
import pytest

from oracle import ld_oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

from pg_gpu_gb300 import _ops, haplotype_kernels, ld_pipeline, ld_statistics  # noqa: E402
from pg_gpu_gb300._lib import PgldError  # noqa: E402



def np_(t):
    return None if t is None else t.cpu().numpy()


def _close(a, b, rtol=1e-13, atol=0.0):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    assert np.array_equal(np.isnan(a), np.isnan(b))
    m = ~np.isnan(a)
    np.testing.assert_allclose(a[m], b[m], rtol=rtol, atol=atol)


def copying_model(rng, H, M, F, switch, missing=0.0, flip=1e-3):
    p = rng.beta(0.3, 0.3, size=M)
    f = (rng.random((F, M)) < p).astype(np.int8)
    sw = rng.random((H, M)) < switch
    seg = np.cumsum(sw, axis=1)
    choice = rng.integers(0, F, size=(H, seg.max() + 1))
    hap = f[np.take_along_axis(choice, seg, axis=1), np.arange(M)[None, :]]
    hap ^= (rng.random(hap.shape) < flip).astype(np.int8)
    if missing:
        hap[rng.random(hap.shape) < missing] = -1
    return hap.astype(np.int8)


# --------------------------------------------------------------------------
# reference fixtures
# --------------------------------------------------------------------------
def test_counts_match_reference(golden):
    z = golden("hap_counts")
    for tag, rows in (("all", None), ("a", z["rows_a"]), ("b", z["rows_b"])):
        c, nv = ld_pipeline.compute_counts_for_pairs(z["hap"], z["idx_i"], z["idx_j"], rows)
        assert np.array_equal(np_(c), z[f"counts_{tag}"])
        assert np.array_equal(np_(nv), z[f"nvalid_{tag}"])
    c, nv = ld_pipeline.compute_counts_for_pairs(z["hap_nomiss"], z["idx_i"], z["idx_j"])
    assert nv is None and np.array_equal(np_(c), z["counts_nomiss"])


def test_pair_chunks_match_reference(golden):
    z = golden("hap_counts")
    chunks = list(ld_pipeline.iter_pairs_within_distance(z["pos"], float(z["max_dist"]),
                                                         int(z["chunk_size"])))
    assert [len(c[0]) for c in chunks] == list(z["chunk_len"])
    assert np.array_equal(np.concatenate([np_(c[0]) for c in chunks]), z["idx_i"])
    assert np.array_equal(np.concatenate([np_(c[1]) for c in chunks]), z["idx_j"])
    for cs, md in ((1, 2000.0), (10_000, 60_000.0), (50, 0.0)):
        key = f"chunks_{cs}_{int(md)}"
        ch = list(ld_pipeline.iter_pairs_within_distance(z["pos"], md, cs))
        assert [len(c[0]) for c in ch] == list(z[key + "_len"])
        if ch:
            assert np.array_equal(np.concatenate([np_(c[0]) for c in ch]), z[key + "_i"])
            assert np.array_equal(np.concatenate([np_(c[1]) for c in ch]), z[key + "_j"])
    assert list(ld_pipeline.iter_pairs_within_distance(np.array([5.0]), 10, 10)) == []


def test_public_statistics_match_reference(golden):
    z = golden("hap_stats")
    c, nv = z["counts"], z["nvalid"]
    for pp in itertools.product(range(4), repeat=2):
        _close(np_(ld_statistics.dd(c, pp, nv)), z["dd_" + "".join(map(str, pp))])
    for pp in itertools.product(range(4), repeat=3):
        _close(np_(ld_statistics.dz(c, pp, nv)), z["dz_" + "".join(map(str, pp))])
    for pp in itertools.product(range(4), repeat=4):
        _close(np_(ld_statistics.pi2(c, pp, nv)), z["pi2_" + "".join(map(str, pp))])
    c4 = c[:, :4]
    _close(np_(ld_statistics.dd(c4)), z["dd_single_nonv"])
    _close(np_(ld_statistics.dz(c4)), z["dz_single_nonv"])
    _close(np_(ld_statistics.pi2(c4)), z["pi2_single_nonv"])
    for f in ("r", "r_squared", "d_prime"):
        _close(np_(getattr(ld_statistics, f)(c4, nv[:, 0])), z[f + "_nv"], rtol=1e-12)
        _close(np_(getattr(ld_statistics, f)(c4)), z[f + "_nonv"], rtol=1e-12)


def test_batches_match_reference(golden):
    z = golden("hap_stats")
    c, nv = z["counts"], z["nvalid"]
    for p in range(1, 5):
        cs = [c[:, 4 * q:4 * q + 4] for q in range(p)]
        got = haplotype_kernels.compute_multi_pop_statistics_batch_hap(
            cs, [nv[:, q] for q in range(p)], None, ld_pipeline.generate_stat_specs(p))
        _close(np_(got), z[f"multi_{p}"])
        got = haplotype_kernels.compute_multi_pop_statistics_batch_hap(
            cs, [None] * p, None, ld_pipeline.generate_stat_specs(p))
        _close(np_(got), z[f"multi_{p}_nonv"])
    _close(np_(ld_pipeline.compute_two_pop_statistics_batch(c[:, :4], c[:, 4:8], nv[:, 0],
                                                            nv[:, 1])), z["two_pop"], rtol=1e-14)
    _close(np_(ld_pipeline.compute_two_pop_statistics_batch(c[:, :4], c[:, 4:8], None, None)),
           z["two_pop_nonv"], rtol=1e-14)
    _close(np_(ld_pipeline.compute_single_pop_statistics_batch(c[:, :4], nv[:, 0])),
           z["single_pop"])


# binned sums: within RTOL of each bin value; a bin whose terms cancel to
# below FLOOR of their sum of |x| is held to RTOL of that share instead
RTOL = 1e-6
FLOOR = 0.05


def _binned_check(hap, pos, rows, bins, form="plain", floor=FLOOR):
    hap_d = torch.as_tensor(hap, device="cuda")
    pops = [_ops.pack(hap_d, r) for r in rows]
    sums, cnt = _ops.binned_sums(pops, _ops.positions_f64(pos), bins, form=form)
    ref, ref_cnt, ref_abs = O.binned_sums(hap, pos, rows, bins, abs_sums=True)
    assert np.array_equal(np_(cnt), ref_cnt)
    rel = O.bin_errors(np_(sums), ref, ref_abs, floor)
    assert rel.max() <= RTOL, float(rel.max())
    return np_(sums), ref_abs


def _near(got, want, scale, floor=FLOOR):
    # against the reference's own fixture (its float64 sums)
    assert O.bin_errors(got, want, scale, floor).max() <= RTOL


def test_binned_sums_match_reference(golden):
    z = golden("binned")
    rows = [z["rows0"], z["rows1"]]
    s2, a2 = _binned_check(z["hap"], z["pos"], rows, z["bins"])
    _near(s2, z["sums_2pop"], a2)
    s1, a1 = _binned_check(z["hap"], z["pos"], rows[:1], z["bins"])
    _near(s1, z["sums_1pop"], a1)
    s3, a3 = _binned_check(z["hap"], z["pos"],
                           [np.arange(0, 16), np.arange(16, 32), np.arange(32, 48)], z["bins"])
    _near(s3, z["sums_3pop"], a3)


def test_binned_sums_match_moments_golden(golden):
    z = golden("moments_im")
    keep = O.biallelic_keep(z["hap"])
    # the reference's criterion for moments' sums: 1e-6 of each value
    s, a = _binned_check(z["hap"][:, keep], z["pos"][keep], [z["rows0"], z["rows1"]], z["bins"],
                         floor=0.0)
    _near(s, z["ld_sums"], a, floor=0.0)


def _planes_oracle(hap, rows):
    """Carrier / reference / validity words of the rows (bit r of word w: row 32w + r)."""
    sub = hap[rows]
    H, M = sub.shape
    W = (H + 31) // 32
    cw = np.zeros((M, W), np.uint32)
    zw = np.zeros((M, W), np.uint32)
    vw = np.zeros((M, W), np.uint32)
    for r in range(H):
        w, b = divmod(r, 32)
        cw[:, w] |= (sub[r] == 1).astype(np.uint32) << np.uint32(b)
        zw[:, w] |= (sub[r] == 0).astype(np.uint32) << np.uint32(b)
        vw[:, w] |= (sub[r] >= 0).astype(np.uint32) << np.uint32(b)
    return np.concatenate([cw, zw], 1), vw, bool((sub == -1).any()), \
        bool(((sub != -1) & (sub != 0) & (sub != 1)).any())


@pytest.mark.parametrize("M", [1040, 1037, 511])
def test_pack_tiles_and_pinned_host(M):
    """Packing: full 512-SNP tiles with 16-byte loads (row stride a multiple of
    16), byte loads otherwise, ragged row subsets, other codes; a pinned host
    matrix is read in place and gives the same planes."""
    rng = np.random.default_rng(M)
    hap = rng.choice(np.array([-1, 0, 1, 2], np.int8), size=(70, M), p=[0.05, 0.5, 0.44, 0.01])
    rows = np.sort(rng.choice(70, 45, replace=False)).astype(np.int32)
    want_p, want_v, miss, other = _planes_oracle(hap, rows)
    host = torch.as_tensor(hap).pin_memory()
    for src in (torch.as_tensor(hap, device="cuda"), host):
        pk = _ops.pack(src, rows)
        assert np.array_equal(np_(pk.planes).view(np.uint32), want_p)
        assert np.array_equal(np_(pk.valid).view(np.uint32), want_v)
        assert (pk.has_missing, pk.has_other) == (miss, other)


def test_pinned_host_matrix_binned_equals_device():
    from pg_gpu_gb300.haplotype_matrix import HaplotypeMatrix
    rng = np.random.default_rng(17)
    hap = copying_model(rng, 96, 1200, 8, 2e-3, missing=0.02)
    pos = np.sort(rng.choice(600_000, 1200, replace=False)).astype(np.int64)
    bins = np.logspace(3, 5, 9)
    sets = {"a": list(range(48)), "b": list(range(48, 96))}
    host = torch.as_tensor(hap).pin_memory()
    hm_h = HaplotypeMatrix(host, pos, sample_sets=sets)
    assert hm_h.device == "CPU"
    got = hm_h.compute_ld_statistics_gpu_two_pops(bins, "a", "b", raw=True, ac_filter=False)
    assert hm_h.device == "CPU"  # packed in place, not copied
    hm_d = HaplotypeMatrix(torch.as_tensor(hap, device="cuda"), pos, sample_sets=sets)
    want = hm_d.compute_ld_statistics_gpu_two_pops(bins, "a", "b", raw=True, ac_filter=False)
    assert got == want


# --------------------------------------------------------------------------
# oracle comparisons: sizes, ragged word counts, large samples
# --------------------------------------------------------------------------
@pytest.mark.parametrize("H", [1, 31, 32, 33, 63, 64, 65, 127, 128, 129, 700])
def test_counts_ragged_sizes(H):
    rng = np.random.default_rng(H)
    M = 70
    hap = copying_model(rng, H, M, 5, 0.05, missing=0.03)
    pos = np.sort(rng.choice(10_000, M, replace=False))
    ii, jj = O.pairs_within_distance(pos, 3000)
    c, nv = ld_pipeline.compute_counts_for_pairs(hap, ii, jj)
    rc, rnv = O.counts_for_pairs(hap, ii, jj)
    assert np.array_equal(np_(c), rc)
    assert (nv is None) == (rnv is None)
    if rnv is not None:
        assert np.array_equal(np_(nv), rnv)
    # tally: every pair, correct where the reference's int8 X.T@X wraps (H >= 128)
    pk = _ops.pack(torch.as_tensor(hap, device="cuda"))
    tc, tnv = _ops.tally(pk)
    oc, onv = O.tally(hap)
    assert np.array_equal(np_(tc), oc)
    if onv is not None:
        assert np.array_equal(np_(tnv), onv)


def test_large_sample_statistics_are_exact():
    # 1000 haplotypes per population: the reference's int32 fast path wraps here
    rng = np.random.default_rng(3)
    hap = copying_model(rng, 2000, 120, 40, 1e-3, missing=0.02)
    pos = np.sort(rng.choice(50_000, 120, replace=False))
    ii, jj = O.pairs_within_distance(pos, 20_000)
    rows = [np.arange(1000), np.arange(1000, 2000)]
    c1, nv1 = ld_pipeline.compute_counts_for_pairs(hap, ii, jj, rows[0])
    c2, nv2 = ld_pipeline.compute_counts_for_pairs(hap, ii, jj, rows[1])
    got = np_(ld_pipeline.compute_two_pop_statistics_batch(c1, c2, nv1, nv2))
    ref = O.two_pop_stats(np_(c1), np_(c2), np_(nv1), np_(nv2))
    _close(got, ref, rtol=1e-15)


@pytest.mark.parametrize("layout", [1, 2])
def test_band_pairs_fp32_outputs(layout, tc_layout):
    # layout: 1 = 64 x 64 tiles, 2 = 64 x 128 tiles
    rng = np.random.default_rng(11)
    H, M = 2000, 600
    hap = copying_model(rng, H, M, 50, 5e-4, missing=0.02)
    pos = np.sort(rng.choice(200_000, M, replace=False)).astype(np.int64)
    pk = _ops.pack(torch.as_tensor(hap, device="cuda"))
    with tc_layout(layout):
        counts, nv, st = _ops.band_pairs(pk, _ops.positions_f64(pos), 20_000)
    ii, jj = O.pairs_within_distance(pos, 20_000)
    rc, rnv = O.counts_for_pairs(hap, ii, jj)
    assert np.array_equal(np_(counts), rc) and np.array_equal(np_(nv), rnv)
    st = np_(st).astype(np.float64)
    ref = np.stack([O.r_squared(rc, rnv), O.dd(rc, None, rnv), O.dz(rc, None, rnv),
                    O.pi2(rc, None, rnv)], axis=1)
    assert np.array_equal(np.isnan(st), np.isnan(ref))
    m = ~np.isnan(ref) & (np.abs(ref) > 1e-30)
    rel = np.abs(st[m] - ref[m]) / np.abs(ref[m])
    assert rel.max() <= 1e-6, rel.max()


def test_binned_sums_two_pops_large_h():
    rng = np.random.default_rng(5)
    hap = copying_model(rng, 2000, 400, 40, 1e-3, missing=0.02)
    pos = np.sort(rng.choice(400_000, 400, replace=False)).astype(np.int64)
    bins = np.logspace(3, 5, 11)
    _binned_check(hap, pos, [np.arange(1000), np.arange(1000, 2000)], bins)


def test_binned_sums_genetic_distance():
    rng = np.random.default_rng(9)
    hap = copying_model(rng, 64, 300, 8, 5e-3, missing=0.01)
    pos = np.sort(rng.choice(100_000, 300, replace=False)).astype(np.int64)
    gmap = np.cumsum(rng.random(300)) * 1e-5
    bins = np.array([0.0, 1e-4, 3e-4, 1e-3])
    rows = [np.arange(32), np.arange(32, 64)]
    hap_d = torch.as_tensor(hap, device="cuda")
    pops = [_ops.pack(hap_d, r) for r in rows]
    sums, cnt = _ops.binned_sums(pops, _ops.positions_f64(pos), bins, max_dist=40_000,
                                 bin_coord=gmap)
    ref, ref_cnt, ref_abs = O.binned_sums(hap, pos, rows, bins, coords=gmap, max_dist=40_000,
                                          abs_sums=True)
    assert np.array_equal(np_(cnt), ref_cnt)
    assert O.bin_errors(np_(sums), ref, ref_abs, FLOOR).max() <= RTOL


def test_edge_cases_and_errors():
    hap = np.zeros((4, 1), np.int8)
    c, nv = ld_pipeline.compute_counts_for_pairs(hap, np.zeros(0, np.int32), np.zeros(0, np.int32))
    assert c.shape == (0, 4) and nv is None
    with pytest.raises(IndexError):
        ld_pipeline.compute_counts_for_pairs(np.zeros((4, 3), np.int8), [0], [5])
    with pytest.raises(ValueError):
        _ops.binned_sums([_ops.pack(np.zeros((4, 3), np.int8))], _ops.positions_f64([1.0, 2, 3]),
                         [10.0, 5.0])
    # one SNP: no pairs, zero sums
    pk = _ops.pack(np.ones((8, 1), np.int8))
    s, n = _ops.binned_sums([pk], _ops.positions_f64([1.0]), [0.0, 10.0])
    assert float(s.abs().sum()) == 0.0 and int(n.sum()) == 0
    with pytest.raises(PgldError):
        _ops.binned_sums([pk], _ops.positions_f64([1.0]), np.linspace(0, 1, 200))


def test_device_rows_checked_again_after_a_change():
    # the range of a device row tensor is read once and kept with the tensor;
    # an in-place change (a new version) is checked again before packing
    hap = torch.zeros((8, 5), dtype=torch.int8, device="cuda")
    rows = torch.arange(4, dtype=torch.int32, device="cuda")
    for _ in range(2):
        pk = _ops.pack(hap, rows)
        assert pk.n_rows == 4
    rows[2] = 8
    with pytest.raises(IndexError):
        _ops.pack(hap, rows)
    rows[2] = -1
    with pytest.raises(IndexError):
        _ops.pack(hap, rows)
    rows[2] = 7
    assert _ops.pack(hap, rows).n_rows == 4


def test_band_pair_count_follows_position_changes():
    # the pair count kept with a positions tensor is read again after an
    # in-place change of the positions, and per distance
    pos_d = _ops.positions_f64(np.arange(0, 1000, 10, dtype=np.float64))
    assert _ops.band_pair_count(pos_d, 25) == 99 + 98
    assert _ops.band_pair_count(pos_d, 25) == 99 + 98
    assert _ops.band_pair_count(pos_d, 5) == 0
    pos_d.mul_(0.5)  # spacing 5
    assert _ops.band_pair_count(pos_d, 5) == 99
    assert _ops.band_pair_count(pos_d, 25) == 99 + 98 + 97 + 96 + 95


def _block_copies(rng, n, M, F, block):
    """n haplotypes copying one of F founders per block of SNPs (a coarse
    copying model that generates full-size panels quickly)."""
    p = rng.beta(0.3, 0.3, size=M)
    f = (rng.random((F, M)) < p).astype(np.int8)
    nb = (M + block - 1) // block
    pick = rng.integers(0, F, size=(n, nb))
    out = np.empty((n, M), np.int8)
    for b in range(nb):
        s, e = b * block, min(M, (b + 1) * block)
        out[:, s:e] = f[pick[:, b], s:e]
    return out


@pytest.mark.parametrize("H,M,D", [(33, 700, 3_000), (400, 1_300, 40_000), (2000, 900, 1e9),
                                   (64, 129, 1e9), (96, 2, 1e9)])
def test_band_pairs_layouts_agree(H, M, D, tc_layout):
    # 64 x 64 tiles (eight epilogue warps) and 64 x 128 tiles (twelve) run the
    # same per-pair arithmetic: equal outputs bit for bit, every band pair
    # written once (including bands wider than the panel and ragged ends)
    rng = np.random.default_rng(H + M)
    hap = copying_model(rng, H, M, 12, 2e-3, missing=0.03)
    pos = np.sort(rng.choice(100 * M, M, replace=False)).astype(np.int64)
    pk = _ops.pack(torch.as_tensor(hap, device="cuda"))
    pos_d = _ops.positions_f64(pos)
    out = {}
    for layout in (1, 2):
        with tc_layout(layout):
            c, nv, st = _ops.band_pairs(pk, pos_d, D, form="tc")
        out[layout] = (np_(c), np_(nv), np_(st))
    for a, b in zip(out[1], out[2]):
        assert np.array_equal(a.view(np.int32), b.view(np.int32))
    ii, jj = O.pairs_within_distance(pos, D)
    rc, rnv = O.counts_for_pairs(hap, ii, jj)
    assert np.array_equal(out[2][0], rc) and np.array_equal(out[2][1], rnv)


def test_full_size_band_pairs():
    # the per-pair workload at full size: 2,000 haplotypes x 100,000 SNPs over
    # 10 Mb, 2 % missing, every pair within 100 kb (~1e8 pairs).  On all pairs:
    # the pair count equals the one from the positions, n = n11+n10+n01+n00,
    # r^2 in [0, 1] or NaN; the first ~1e6 pairs equal the oracle's
    rng = np.random.default_rng(20261502)
    H, M, D = 2000, 100_000, 100_000
    hap = _block_copies(rng, H, M, 50, 2_000)
    hap[rng.random(hap.shape) < 0.02] = -1
    pos = np.sort(rng.choice(10_000_000, M, replace=False)).astype(np.int64)
    pk = _ops.pack(torch.as_tensor(hap, device="cuda"))
    counts, nv, st = _ops.band_pairs(pk, _ops.positions_f64(pos), D, form="tc")
    pf = pos.astype(np.float64)
    n_exact = int((np.searchsorted(pf, pf + D, side="right") - np.arange(M) - 1).sum())
    assert counts.shape[0] == n_exact
    assert torch.equal(counts.sum(1, dtype=torch.int32), nv)
    r2 = st[:, 0]
    ok = torch.isnan(r2) | ((r2 >= 0) & (r2 <= 1 + 1e-6))
    assert bool(ok.all())
    A = 1000  # anchors of the sampled pairs (~1e6 pairs)
    ext = np.searchsorted(pf, pf[:A] + D, side="right")
    ii, jj = O.pairs_within_distance(pos[:int(ext.max())], D)
    sel = ii < A
    ii, jj = ii[sel], jj[sel]
    parts = [O.counts_for_pairs(hap, ii[s:s + 200_000], jj[s:s + 200_000])
             for s in range(0, len(ii), 200_000)]
    rc = np.concatenate([p[0] for p in parts])
    rnv = np.concatenate([p[1] for p in parts])
    assert np.array_equal(np_(counts[:len(ii)]), rc) and np.array_equal(np_(nv[:len(ii)]), rnv)
    ref = np.stack([O.r_squared(rc, rnv), O.dd(rc, None, rnv), O.dz(rc, None, rnv),
                    O.pi2(rc, None, rnv)], axis=1)
    got = np_(st[:len(ii)]).astype(np.float64)
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    m = ~np.isnan(ref) & (np.abs(ref) > 1e-30)
    assert (np.abs(got[m] - ref[m]) / np.abs(ref[m])).max() <= 1e-6


def test_moments_ld_vcf_packs_straight_from_the_gt_text(golden, tmp_path):
    """moments_ld.compute_ld_statistics(vcf_file, pop_file): the populations
    are packed from the GT text into bit planes (no int8 haplotype matrix);
    the sums equal the matrix path's (from_vcf, load_pop_file,
    apply_biallelic_filter) and the moments golden within 1e-6 of each
    value; heterozygosity from the carrier planes."""
    from pg_gpu_gb300 import moments_ld
    from pg_gpu_gb300.haplotype_matrix import HaplotypeMatrix, PackedVcf
    z = golden("moments_im")
    hap, pos = z["hap"], z["pos"]
    n = hap.shape[0] // 2
    names = [f"tsk_{k}" for k in range(n)]
    r0 = set(int(r) for r in z["rows0"])
    al = lambda a: "." if a < 0 else str(int(a))  # noqa: E731
    lines = ["##fileformat=VCFv4.2",
             "#CHROM\tPOS\tID\tREF\tALT\tQUAL\tFILTER\tINFO\tFORMAT\t" + "\t".join(names)]
    for j in range(hap.shape[1]):
        lines.append("\t".join(["1", str(int(pos[j])), ".", "A", "T", ".", "PASS", ".", "GT"]
                               + [al(hap[k, j]) + "|" + al(hap[n + k, j]) for k in range(n)]))
    vcf = tmp_path / "im.vcf"
    vcf.write_text("\n".join(lines) + "\n")
    popf = tmp_path / "pops.txt"
    popf.write_text("sample\tpop\n" + "".join(f"{names[k]}\t{'deme0' if k in r0 else 'deme1'}\n"
                                              for k in range(n)))
    pops = ["deme0", "deme1"]
    assert isinstance(moments_ld._packed_vcf(str(vcf), str(popf), pops, True), PackedVcf)
    res = moments_ld.compute_ld_statistics(vcf_file=str(vcf), pop_file=str(popf), pops=pops,
                                           bp_bins=z["bins"], report=False)
    hm = HaplotypeMatrix.from_vcf(str(vcf))
    hm.load_pop_file(str(popf), pops=pops)
    ref = moments_ld.compute_ld_statistics(haplotype_matrix=hm.apply_biallelic_filter(),
                                           pops=pops, bp_bins=z["bins"], report=False)
    np.testing.assert_allclose(np.array(res["sums"][:-1]), np.array(ref["sums"][:-1]),
                               rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(res["sums"][-1], ref["sums"][-1], rtol=1e-14)
    np.testing.assert_allclose(res["sums"][-1], z["het_sums"], rtol=1e-12)
    keep = O.biallelic_keep(hap)
    _, _, a = O.binned_sums(hap[:, keep], pos[keep], [z["rows0"], z["rows1"]], z["bins"],
                            abs_sums=True)
    _near(np.array(res["sums"][:-1]), z["ld_sums"], a, floor=0.0)
    # with an accessible mask (sites subset on the device) as the matrix path
    lo, hi = int(pos[len(pos) // 4]), int(pos[3 * len(pos) // 4])
    bed = tmp_path / "acc.bed"
    bed.write_text(f"1\t{lo}\t{hi}\n")
    res_b = moments_ld.compute_ld_statistics(vcf_file=str(vcf), pop_file=str(popf), pops=pops,
                                             bp_bins=z["bins"], report=False,
                                             accessible_bed=str(bed))
    ref_b = moments_ld.compute_ld_statistics(haplotype_matrix=hm.apply_biallelic_filter(),
                                             pops=pops, bp_bins=z["bins"], report=False,
                                             accessible_bed=str(bed))
    np.testing.assert_allclose(np.array(res_b["sums"][:-1]), np.array(ref_b["sums"][:-1]),
                               rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(res_b["sums"][-1], ref_b["sums"][-1], rtol=1e-14)
