"""GPU parity of the genotype (unphased diploid) LD path.

9-way counts are compared bit-for-bit with the reference's counting kernel;
float64 statistics (exact 64-bit integer numerators, one division) with the
reference's float64 kernels at 1e-13 relative (same NaN / inf pattern);
float32 per-pair statistics within 1e-6 relative of the float64 oracle; binned
sums within |gpu - oracle| <= 2e-6 * sum|x| per bin and statistic.
"""
import numpy as np
import pytest

from oracle import ld_oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

from pg_gpu_gb300 import (_geno, _ops, genotype_kernels, ld_pipeline,  # noqa: E402
                          ld_statistics, ld_statistics_genotype, moments_ld)
from pg_gpu_gb300._lib import PgldError  # noqa: E402
from pg_gpu_gb300.genotype_matrix import GenotypeMatrix  # noqa: E402
from pg_gpu_gb300.haplotype_matrix import HaplotypeMatrix  # noqa: E402

SUM_TOL = 2e-6


def np_(t):
    return None if t is None else t.cpu().numpy()


def _ieee(got, ref, rtol):
    got, ref = np.asarray(got), np.asarray(ref)
    assert got.shape == ref.shape
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    inf = np.isinf(ref)
    assert np.array_equal(np.isinf(got), inf) and np.array_equal(got[inf], ref[inf])
    f = np.isfinite(ref)
    np.testing.assert_allclose(got[f], ref[f], rtol=rtol, atol=0)


def dosages(rng, n_ind, M, F, switch, missing=0.0):
    p = rng.beta(0.3, 0.3, size=M)
    f = (rng.random((F, M)) < p).astype(np.int8)
    H = 2 * n_ind
    sw = rng.random((H, M)) < switch
    seg = np.cumsum(sw, axis=1)
    choice = rng.integers(0, F, size=(H, seg.max() + 1))
    hap = f[np.take_along_axis(choice, seg, axis=1), np.arange(M)[None, :]]
    hap ^= (rng.random(hap.shape) < 1e-3).astype(np.int8)
    g = (hap[0::2] + hap[1::2]).astype(np.int8)
    if missing:
        g[rng.random(g.shape) < missing] = -1
    return g


def test_genotype_counts_match_reference(golden):
    z = golden("geno")
    c, nv = ld_pipeline.compute_genotype_counts_for_pairs(z["geno_miss"], z["idx_i"], z["idx_j"])
    assert np.array_equal(np_(c), z["counts9_miss"]) and np.array_equal(np_(nv), z["nvalid_miss"])
    c, nv = ld_pipeline.compute_genotype_counts_for_pairs(z["geno"], z["idx_i"], z["idx_j"])
    assert nv is None and np.array_equal(np_(c), z["counts9"])
    c, _ = ld_pipeline.compute_genotype_counts_for_pairs(z["geno_miss"], z["idx_i"], z["idx_j"],
                                                         list(z["rows"]))
    assert np.array_equal(np_(c), z["counts9_rows"])
    # dosages above 2 fold into classes like the reference kernel (3 g_i + g_j)
    c, nv = ld_pipeline.compute_genotype_counts_for_pairs(z["geno_odd"], z["idx_i"], z["idx_j"])
    assert np.array_equal(np_(c), z["counts9_odd"]) and np.array_equal(np_(nv), z["nvalid_odd"])
    pk = _ops.pack_geno(z["geno_odd"])
    cb, nvb, _ = _ops.geno_band_pairs(pk, _ops.positions_f64(z["pos"]), 15_000, with_stats=False)
    assert np.array_equal(np_(cb), z["counts9_odd"]) and np.array_equal(np_(nvb), z["nvalid_odd"])


def test_dd_and_sigma_d2_match_reference_kernels(golden):
    z = golden("geno")
    for tag in ("", "_miss"):
        c = torch.as_tensor(z["counts9" + tag], device="cuda")
        import pg_gpu_gb300._lib as L
        out = _ops.stats([c], [None], [(0, L.G_DD_II, (0,), 1.0), (1, L.G_SIGMA_D2, (0,), 1.0)],
                         2, geno=True)
        _ieee(np_(out[:, 0]), z["dd_geno" + tag], 1e-13)
        _ieee(np_(out[:, 1]), z["sigma_d2" + tag], 1e-13)
    gm = GenotypeMatrix(z["geno"], z["pos"])
    s = ld_statistics_genotype.sigma_d2_geno(gm, z["idx_i"], z["idx_j"])
    _ieee(np_(s), z["sigma_d2"], 1e-13)
    with pytest.raises(ValueError):
        ld_statistics_genotype.sigma_d2_geno(GenotypeMatrix(z["geno_miss"], z["pos"]))
    with pytest.raises(TypeError):
        ld_statistics_genotype.sigma_d2_geno(z["geno"])


@pytest.mark.parametrize("P", [1, 2, 3, 4])
def test_multi_pop_statistics_match_reference(golden, P):
    z = golden("geno_stats")
    cs = [z[f"counts_{q}"] for q in range(P)]
    got = genotype_kernels.compute_multi_pop_statistics_batch_geno(
        cs, [c.sum(1).astype(np.int32) for c in cs], None, ld_pipeline.generate_stat_specs(P))
    _ieee(np_(got), z[f"multi_{P}"], 1e-13)
    got0 = genotype_kernels.compute_multi_pop_statistics_batch_geno(cs, [None] * P)
    _ieee(np_(got0), z[f"multi_{P}_nonv"], 1e-13)


def test_rogers_huff_matches_reference(golden):
    z = golden("geno")
    gm = GenotypeMatrix(z["geno"], z["pos"])
    r = np_(ld_statistics.rogers_huff_r(gm))
    ref = z["rh_r_condensed"]
    assert np.array_equal(np.isnan(r), np.isnan(ref))
    m = ~np.isnan(ref)
    np.testing.assert_allclose(r[m], ref[m], rtol=1e-9, atol=1e-12)
    r2 = np_(ld_statistics.rogers_huff_r_squared(gm))
    np.testing.assert_allclose(r2[m], ref[m] ** 2, rtol=1e-9, atol=1e-12)
    with pytest.raises(ValueError):
        ld_statistics.rogers_huff_r(GenotypeMatrix(z["geno_miss"], z["pos"]))
    # with missing data: pairwise-complete moments, exact against the oracle
    rp = _geno.rh_pairs(z["geno_miss"], z["idx_i"], z["idx_j"])
    np.testing.assert_allclose(np_(rp), O.rogers_huff_r_pairs(z["geno_miss"], z["idx_i"],
                                                              z["idx_j"]), rtol=1e-14)


def test_band_pairs_fp32_outputs():
    # unphased-genotype workload shape: 1,000 diploids, 3 % missing
    rng = np.random.default_rng(21)
    g = dosages(rng, 1000, 500, 60, 5e-4, missing=0.03)
    pos = np.sort(rng.choice(500_000, 500, replace=False)).astype(np.int64)
    pk = _ops.pack_geno(torch.as_tensor(g, device="cuda"))
    counts, nv, st = _ops.geno_band_pairs(pk, _ops.positions_f64(pos), 200_000)
    ii, jj = O.pairs_within_distance(pos, 200_000)
    rc, rnv = O.genotype_counts_for_pairs(g, ii, jj)
    assert np.array_equal(np_(counts), rc) and np.array_equal(np_(nv), rnv)
    st = np_(st).astype(np.float64)
    ref = np.stack([O.rogers_huff_r_counts(rc) ** 2,
                    O.geno_dd((0, 0), [O.GenoPop(rc, rnv)]),
                    O.geno_dz((0, 0, 0), [O.GenoPop(rc, rnv)]),
                    O.geno_pi2((0, 0, 0, 0), [O.GenoPop(rc, rnv)])], axis=1)
    assert np.array_equal(np.isnan(st), np.isnan(ref))
    m = ~np.isnan(ref) & (np.abs(ref) > 1e-30)
    rel = np.abs(st[m] - ref[m]) / np.abs(ref[m])
    assert rel.max() <= 1e-6, rel.max()
    # a column subset evaluates only those columns, bit-identical
    _, _, st2 = _ops.geno_band_pairs(pk, _ops.positions_f64(pos), 200_000, with_counts=False,
                                     columns=("r2", "dd"))
    st2 = np_(st2).astype(np.float64)
    assert np.array_equal(st2[:, :2], st[:, :2], equal_nan=True)
    assert np.all(st2[:, 2:] == 0)


@pytest.mark.parametrize("n_ind,M", [(1, 90), (31, 200), (33, 333), (130, 257), (1000, 300),
                                     (1281, 200), (3000, 150)])
def test_tc_band_pairs_match_plain_and_oracle(n_ind, M):
    # the tensor-core genotype form: counts bit-exact, statistics bit-identical
    # to the plain form (the same float32 epilogue on the same counts)
    rng = np.random.default_rng(n_ind * 7 + M)
    g = dosages(rng, n_ind, M, 12, 2e-3, missing=0.03)
    pos = np.sort(rng.choice(100_000, M, replace=False)).astype(np.int64)
    pk = _ops.pack_geno(torch.as_tensor(g, device="cuda"))
    pos_d = _ops.positions_f64(pos)
    c_tc, nv_tc, st_tc = _ops.geno_band_pairs(pk, pos_d, 30_000, form="tc")
    c_pl, nv_pl, st_pl = _ops.geno_band_pairs(pk, pos_d, 30_000, form="plain")
    ii, jj = O.pairs_within_distance(pos, 30_000)
    rc, rnv = O.genotype_counts_for_pairs(g, ii, jj)
    assert np.array_equal(np_(c_tc), rc) and np.array_equal(np_(c_pl), rc)
    assert np.array_equal(np_(nv_tc), np_(nv_pl))
    assert np.array_equal(np_(st_tc), np_(st_pl), equal_nan=True)


@pytest.mark.parametrize("P", [2, 3])
def test_binned_sums_match_reference(golden, P):
    z = golden("geno_binned")
    rows = [z[f"rows{q}"] for q in range(P)]
    keep = z[f"keep_{P}"]
    g = torch.as_tensor(np.ascontiguousarray(z["geno"][:, keep]), device="cuda")
    pops = [_ops.pack_geno(g, r) for r in rows]
    sums, cnt = _ops.geno_binned_sums(pops, _ops.positions_f64(z["pos"][keep]), z["bins"])
    ref, ref_cnt, ref_abs = O.geno_binned_sums(z["geno"][:, keep], z["pos"][keep], rows,
                                               z["bins"], abs_sums=True)
    np.testing.assert_allclose(ref, z[f"sums_{P}"], rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    assert np.array_equal(np_(cnt), ref_cnt)
    assert np.all(np.abs(np_(sums) - z[f"sums_{P}"]) <= SUM_TOL * ref_abs + 1e-300)


@pytest.mark.parametrize("sizes,missing,coords", [([300], 0.03, False), ([120, 77], 0.02, False),
                                                  ([40, 33, 65], 0.0, True),
                                                  ([20, 31, 50, 9], 0.05, False)])
def test_tc_binned_sums_match_plain_and_oracle(sizes, missing, coords):
    """The tensor-core genotype binned form (moments from tcgen05 MMAs, one
    chain per population) against the popcount form and the oracle: 1-4
    populations of uneven sizes, missing dosages, a partial last tile,
    pairs below the first bin, binning by a second coordinate."""
    P = len(sizes)
    rng = np.random.default_rng(700 + P)
    M = 1_037
    g = dosages(rng, sum(sizes), M, 6, 0.01, missing)
    edges = np.concatenate([[0], np.cumsum(sizes)])
    rows = [np.arange(edges[q], edges[q + 1], dtype=np.int32) for q in range(P)]
    pos = np.sort(rng.choice(2_000_000, M, replace=False)).astype(np.int64)
    pos_d = _ops.positions_f64(pos)
    gt = torch.as_tensor(g, device="cuda")
    pops = [_ops.pack_geno(gt, r) for r in rows]
    if coords:
        rate = np.cumsum(rng.uniform(0.2, 2.0, M)) * 1e-6      # Morgans, uneven local rates
        bins = np.linspace(0.0, rate[-1] / 8, 7)
        max_dist = 400_000.0
        bc = torch.as_tensor(rate, device="cuda")
    else:
        bins = np.logspace(2.5, 5.3, 9)
        max_dist, bc, rate = None, None, None
    s_tc, c_tc = _ops.geno_binned_sums(pops, pos_d, bins, max_dist=max_dist, bin_coord=bc,
                                       form="tc")
    s_pl, c_pl = _ops.geno_binned_sums(pops, pos_d, bins, max_dist=max_dist, bin_coord=bc,
                                       form="plain")
    ref, ref_cnt, ref_abs = O.geno_binned_sums(g, pos, rows, bins, coords=rate,
                                               max_dist=max_dist, abs_sums=True)
    assert np.array_equal(np_(c_tc), ref_cnt) and np.array_equal(np_(c_pl), ref_cnt)
    assert ref_cnt.sum() > 10_000
    assert np.all(np.abs(np_(s_tc) - ref) <= SUM_TOL * ref_abs + 1e-300)
    assert np.all(np.abs(np_(s_tc) - np_(s_pl)) <= SUM_TOL * ref_abs + 1e-300)


def test_tc_binned_rejects_dosages_above_two():
    rng = np.random.default_rng(5)
    g = dosages(rng, 40, 200, 4, 0.01)
    g[3, 17] = 3
    pos = np.sort(rng.choice(100_000, 200, replace=False)).astype(np.int64)
    pk = _ops.pack_geno(torch.as_tensor(g, device="cuda"))
    with pytest.raises(PgldError):
        _ops.geno_binned_sums([pk], _ops.positions_f64(pos), np.logspace(2, 4, 5), form="tc")
    # auto takes the popcount form for such panels
    s, c = _ops.geno_binned_sums([pk], _ops.positions_f64(pos), np.logspace(2, 4, 5))
    ref, ref_cnt = O.geno_binned_sums(g, pos, [np.arange(40)], np.logspace(2, 4, 5))
    assert np.array_equal(np_(c), ref_cnt)


def test_moments_ld_genotype_and_haplotype_paths(golden):
    z = golden("moments_im")
    sets = {"deme0": list(map(int, z["rows0"])), "deme1": list(map(int, z["rows1"]))}
    keep = O.biallelic_keep(z["hap"])
    hm = HaplotypeMatrix(z["hap"][:, keep], z["pos"][keep], sample_sets=sets)
    res = moments_ld.compute_ld_statistics(haplotype_matrix=hm, pops=["deme0", "deme1"],
                                           bp_bins=z["bins"], report=False)
    assert res["stats"][0] == list(z["ld_names"]) and res["stats"][1] == list(z["het_names"])
    ld = np.array(res["sums"][:-1])
    _, _, a = O.binned_sums(z["hap"][:, keep], z["pos"][keep], [z["rows0"], z["rows1"]], z["bins"],
                            abs_sums=True)
    assert np.all(np.abs(ld - z["ld_sums"]) <= SUM_TOL * a + 1e-12 * np.abs(z["ld_sums"]))
    np.testing.assert_allclose(res["sums"][-1], z["het_sums"], rtol=1e-12)
    # genotype path on the paired haplotypes of the same data
    gm = GenotypeMatrix.from_haplotype_matrix(HaplotypeMatrix(z["hap"], z["pos"], sample_sets=sets))
    res_g = moments_ld.compute_ld_statistics(genotype_matrix=gm, pops=["deme0", "deme1"],
                                             bp_bins=z["bins"], use_genotypes=True, report=False)
    g = np_(gm.genotypes) if hasattr(gm.genotypes, "cpu") else gm.genotypes
    rows = [np.array(gm.sample_sets["deme0"]), np.array(gm.sample_sets["deme1"])]
    k = O.union_polymorphic(g, rows)
    ref, _, ref_abs = O.geno_binned_sums(g[:, k], z["pos"][k], rows, z["bins"], abs_sums=True)
    assert np.all(np.abs(np.array(res_g["sums"][:-1]) - ref) <= SUM_TOL * ref_abs + 1e-300)
    het = O.geno_heterozygosity(g, rows)
    np.testing.assert_allclose(res_g["sums"][-1], [het[h] for h in res_g["stats"][1]], rtol=1e-12)


def test_moments_ld_accessible_bed(golden, tmp_path):
    # accessible_bed: the variants outside the BED intervals are dropped
    # before the statistics (moments_ld.py:99-101, 159-160)
    z = golden("moments_im")
    sets = {"deme0": list(map(int, z["rows0"])), "deme1": list(map(int, z["rows1"]))}
    pos = z["pos"]
    lo, hi = int(pos[len(pos) // 4]), int(pos[3 * len(pos) // 4])
    bed = tmp_path / "acc.bed"
    bed.write_text(f"1\t{lo}\t{hi}\n")
    hm = HaplotypeMatrix(z["hap"], pos, sample_sets=sets)
    res = moments_ld.compute_ld_statistics(haplotype_matrix=hm, pops=["deme0", "deme1"],
                                           bp_bins=z["bins"], report=False,
                                           accessible_bed=str(bed))
    inside = np.nonzero((pos > lo) & (pos <= hi))[0]
    ref = moments_ld.compute_ld_statistics(
        haplotype_matrix=HaplotypeMatrix(z["hap"][:, inside], pos[inside], sample_sets=sets),
        pops=["deme0", "deme1"], bp_bins=z["bins"], report=False)
    np.testing.assert_array_equal(np.array(res["sums"][:-1]), np.array(ref["sums"][:-1]))
    np.testing.assert_allclose(res["sums"][-1], ref["sums"][-1], rtol=1e-12)


def test_edge_cases_and_errors():
    c, nv = ld_pipeline.compute_genotype_counts_for_pairs(np.zeros((4, 1), np.int8),
                                                          np.zeros(0, np.int32),
                                                          np.zeros(0, np.int32))
    assert c.shape == (0, 9) and nv is None
    with pytest.raises(IndexError):
        ld_pipeline.compute_genotype_counts_for_pairs(np.zeros((4, 3), np.int8), [0], [7])
    with pytest.raises(ValueError):
        _ops.pack_geno(np.zeros((8193, 2), np.int8))
    # ragged population sizes around word boundaries, counts exact
    rng = np.random.default_rng(3)
    for n_ind in (1, 31, 33, 64, 95):
        g = dosages(rng, n_ind, 70, 4, 0.05, missing=0.05)
        pos = np.sort(rng.choice(10_000, 70, replace=False)).astype(np.int64)
        pk = _ops.pack_geno(g)
        counts, nv, _ = _ops.geno_band_pairs(pk, _ops.positions_f64(pos), 3_000, with_stats=False)
        ii, jj = O.pairs_within_distance(pos, 3_000)
        rc, rnv = O.genotype_counts_for_pairs(g, ii, jj)
        assert np.array_equal(np_(counts), rc)
    with pytest.raises(PgldError):
        _ops.geno_binned_sums([pk], _ops.positions_f64(pos), np.linspace(0, 1, 200))


def test_public_fused_pair_statistics_match_the_chunked_loop():
    # ld_pipeline's fused band calls give the reference loop's pairs, in its order
    from pg_gpu_gb300 import ld_pipeline as LP
    rng = np.random.default_rng(31)
    g = dosages(rng, 200, 400, 12, 2e-3, missing=0.03)
    hap = (rng.random((64, 400)) < 0.4).astype(np.int8)
    hap[rng.random(hap.shape) < 0.02] = -1
    pos = np.sort(rng.choice(200_000, 400, replace=False)).astype(np.int64)
    ii, jj = O.pairs_within_distance(pos, 20_000)
    c, nv, st = LP.genotype_pairs_within_distance_statistics(
        torch.as_tensor(g, device="cuda"), pos, 20_000, statistics=("r2", "dd"))
    rc, rnv = O.genotype_counts_for_pairs(g, ii, jj)
    assert np.array_equal(np_(c), rc) and np.array_equal(np_(nv), rnv)
    ref = O.geno_dd((0, 0), [O.GenoPop(rc, rnv)])
    got = np_(st)[:, 1].astype(np.float64)
    m = np.abs(ref) > 1e-30
    assert np.all(np.abs(got[m] - ref[m]) <= 1e-6 * np.abs(ref[m])) and np.all(np_(st)[:, 2:] == 0)
    c4, nv4, st4 = LP.pairs_within_distance_statistics(torch.as_tensor(hap, device="cuda"), pos,
                                                       20_000)
    rc4 = O.counts_for_pairs(hap, ii, jj)[0]
    assert np.array_equal(np_(c4), rc4) and st4.shape == (len(ii), 4)


def test_full_size_geno_band():
    # the unphased-genotype workload at full size: 1,000 diploids x 500,000
    # SNPs over 50 Mb, 3 % missing, every pair within 200 kb (~1e9 pairs; the
    # n / r^2 / DD outputs, 20 GB).  On all pairs: the pair count equals the
    # one from the positions, 4 <= n <= 1,000 where DD is nonzero, r^2 in
    # [0, 1] or NaN; the first ~1e6 pairs equal the oracle's
    rng = np.random.default_rng(20261505)
    N, M, D = 1000, 500_000, 200_000
    p = rng.beta(0.3, 0.3, size=M)
    f = (rng.random((60, M)) < p).astype(np.int8)
    g = np.zeros((N, M), np.int8)
    for b in range(0, M, 2_000):  # each haplotype copies a founder per 2,000-SNP block
        for _ in range(2):
            g[:, b:b + 2_000] += f[rng.integers(0, 60, N), b:b + 2_000]
    g[rng.random(g.shape) < 0.03] = -1
    pos = np.sort(rng.choice(50_000_000, M, replace=False)).astype(np.int64)
    g_d = torch.as_tensor(g, device="cuda")
    pk = _ops.pack_geno(g_d)
    pos_d = _ops.positions_f64(pos)
    _, nv, st = _ops.geno_band_pairs(pk, pos_d, D, with_counts=False, columns=("r2", "dd"))
    pf = pos.astype(np.float64)
    n_exact = int((np.searchsorted(pf, pf + D, side="right") - np.arange(M) - 1).sum())
    assert nv.shape[0] == n_exact
    assert int(nv.max()) <= N and int(nv.min()) >= 0
    r2 = st[:, 0]
    assert bool((torch.isnan(r2) | ((r2 >= 0) & (r2 <= 1 + 1e-6))).all())
    assert bool(((st[:, 1] == 0) | (nv >= 4)).all()) and bool((st[:, 2:] == 0).all())
    del st
    A = 500  # anchors of the sampled pairs (~1e6 pairs)
    ext = np.searchsorted(pf, pf[:A] + D, side="right")
    ii, jj = O.pairs_within_distance(pos[:int(ext.max())], D)
    sel = ii < A
    ii, jj = ii[sel], jj[sel]
    parts = [O.genotype_counts_for_pairs(g, ii[s:s + 200_000], jj[s:s + 200_000])
             for s in range(0, len(ii), 200_000)]
    rc = np.concatenate([q[0] for q in parts])
    rnv = np.concatenate([q[1] for q in parts])
    c_gpu, _ = ld_pipeline.compute_genotype_counts_for_pairs(g_d, ii, jj)
    assert np.array_equal(np_(c_gpu), rc) and np.array_equal(np_(nv[:len(ii)]), rnv)
    _, _, st = _ops.geno_band_pairs(pk, pos_d, D, with_counts=False, columns=("r2", "dd"))
    got = np_(st[:len(ii), :2]).astype(np.float64)
    ref = np.stack([O.rogers_huff_r_counts(rc) ** 2, O.geno_dd((0, 0), [O.GenoPop(rc, rnv)])], 1)
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    m = ~np.isnan(ref) & (np.abs(ref) > 1e-30)
    assert (np.abs(got[m] - ref[m]) / np.abs(ref[m])).max() <= 1e-6
