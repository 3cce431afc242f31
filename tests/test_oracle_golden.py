"""The CPU oracle against fixtures produced by the reference pg_gpu itself.

Fixtures come from tests/golden/make_golden.py (reference code run through a
numpy stand-in for CuPy) and from the moments result the reference caches in
its own test suite (tests/test_ld_validation_full.py:38-67).
"""
import itertools

import numpy as np
import pytest

from oracle import ld_oracle as O


def test_pair_enumeration_matches_reference_chunks(golden):
    z = golden("hap_counts")
    ii, jj = O.pairs_within_distance(z["pos"], float(z["max_dist"]))
    assert np.array_equal(ii, z["idx_i"]) and np.array_equal(jj, z["idx_j"])
    lens = [b[2] for b in O.chunk_bounds(z["pos"], float(z["max_dist"]), int(z["chunk_size"]))]
    assert np.array_equal(lens, z["chunk_len"])
    for cs, md in ((1, 2000.0), (10_000, 60_000.0), (50, 0.0)):
        key = f"chunks_{cs}_{int(md)}"
        ii, jj = O.pairs_within_distance(z["pos"], md)
        assert np.array_equal(ii, z[key + "_i"]) and np.array_equal(jj, z[key + "_j"])
        lens = [b[2] for b in O.chunk_bounds(z["pos"], md, cs)]
        assert np.array_equal(lens, z[key + "_len"])


def test_pair_enumeration_edge_cases():
    # tests/test_ld_pair_iteration.py:21-115: empty, single SNP, max_dist 0 / inf
    assert len(O.pairs_within_distance(np.array([], np.int64), 10)[0]) == 0
    assert len(O.pairs_within_distance(np.array([5]), 10)[0]) == 0
    ii, jj = O.pairs_within_distance(np.array([1, 2, 2, 3]), 0)
    assert list(zip(ii, jj)) == [(1, 2)]
    ii, jj = O.pairs_within_distance(np.arange(6) * 10, np.inf)
    assert len(ii) == 15


def test_counts_match_reference(golden):
    z = golden("hap_counts")
    for tag, rows in (("all", None), ("a", z["rows_a"]), ("b", z["rows_b"])):
        c, nv = O.counts_for_pairs(z["hap"], z["idx_i"], z["idx_j"], rows)
        assert np.array_equal(c, z[f"counts_{tag}"])
        assert np.array_equal(nv, z[f"nvalid_{tag}"])
    c, nv = O.counts_for_pairs(z["hap_nomiss"], z["idx_i"], z["idx_j"])
    assert nv is None and np.array_equal(c, z["counts_nomiss"])


def test_counts_known_answers():
    # tests/test_haplotype_counting.py:22-52: ind0 = 1|1 , 1|0 ; ind1 = 0|1 , 1|0
    h = np.empty((4, 2), np.int8)
    h[0], h[1] = [1, 1], [0, 1]      # hap-0 of ind0, ind1
    h[2], h[3] = [1, 0], [1, 0]      # hap-1 of ind0, ind1
    c, nv = O.counts_for_pairs(h, np.array([0]), np.array([1]))
    assert c.tolist() == [[1, 2, 1, 0]] and nv is None


def _close(a, b, rtol=1e-13, atol=1e-300):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    assert np.array_equal(np.isnan(a), np.isnan(b))
    m = ~np.isnan(a)
    np.testing.assert_allclose(a[m], b[m], rtol=rtol, atol=atol)


def test_public_statistics_match_reference(golden):
    z = golden("hap_stats")
    c, nv = z["counts"], z["nvalid"]
    for pp in itertools.product(range(4), repeat=2):
        _close(O.dd(c, pp, nv), z["dd_" + "".join(map(str, pp))])
    for pp in itertools.product(range(4), repeat=3):
        _close(O.dz(c, pp, nv), z["dz_" + "".join(map(str, pp))])
    for pp in itertools.product(range(4), repeat=4):
        _close(O.pi2(c, pp, nv), z["pi2_" + "".join(map(str, pp))])
    c4 = c[:, :4]
    _close(O.dd(c4), z["dd_single_nonv"])
    _close(O.dz(c4), z["dz_single_nonv"])
    _close(O.pi2(c4), z["pi2_single_nonv"])


def test_r_family_matches_reference(golden):
    z = golden("hap_stats")
    c4, nv = z["counts"][:, :4], z["nvalid"][:, 0]
    for f in ("r", "r_squared", "d_prime"):
        _close(getattr(O, f)(c4, nv), z[f + "_nv"], rtol=1e-12)
        _close(getattr(O, f)(c4), z[f + "_nonv"], rtol=1e-12)


def test_r_known_answers():
    # tests/test_ld_r_squared.py:15-57, 171-190; tests/test_haplotype_kernels_rsq.py:90-126
    c = np.array([[5, 0, 0, 5], [25, 25, 25, 25], [0, 5, 5, 0], [5, 5, 0, 0]])
    r2 = O.r_squared(c)
    assert r2[0] == 1.0 and r2[1] == 0.0 and r2[2] == 1.0 and np.isnan(r2[3])
    assert O.r(c)[2] == -1.0
    dp = O.d_prime(c)
    assert dp[0] == 1.0 and dp[1] == 0.0 and dp[2] == -1.0 and np.isnan(dp[3])


def test_batches_match_reference(golden):
    z = golden("hap_stats")
    c, nv = z["counts"], z["nvalid"]
    for p in range(1, 5):
        cs = [c[:, 4 * q:4 * q + 4] for q in range(p)]
        _close(O.multi_pop_stats(cs, [nv[:, q] for q in range(p)]), z[f"multi_{p}"])
        _close(O.multi_pop_stats(cs, [None] * p), z[f"multi_{p}_nonv"])
    _close(O.two_pop_stats(c[:, :4], c[:, 4:8], nv[:, 0], nv[:, 1]), z["two_pop"], rtol=1e-14)
    _close(O.two_pop_stats(c[:, :4], c[:, 4:8], None, None), z["two_pop_nonv"], rtol=1e-14)
    _close(O.single_pop_stats(c[:, :4], nv[:, 0]), z["single_pop"])


def test_names_and_specs_match_reference():
    import os
    from tests.conftest import GOLDEN
    with open(os.path.join(GOLDEN, "ld_names.txt")) as f:
        lines = f.read().splitlines()
    for p in range(1, 5):
        assert lines[2 * (p - 1)].split()[1:] == O.ld_names(p)
        assert lines[2 * (p - 1) + 1].split()[1:] == O.het_names(p)
    assert [len(O.stat_specs(p)) for p in (1, 2, 3, 4)] == [3, 15, 45, 105]


def test_binned_sums_match_reference(golden):
    z = golden("binned")
    rows = [z["rows0"], z["rows1"]]
    for P, key in ((2, "sums_2pop"), (1, "sums_1pop")):
        s, _ = O.binned_sums(z["hap"], z["pos"], rows[:P], z["bins"])
        np.testing.assert_allclose(s, z[key], rtol=1e-13, atol=1e-300)
    s, _ = O.binned_sums(z["hap"], z["pos"], [np.arange(0, 16), np.arange(16, 32),
                                              np.arange(32, 48)], z["bins"])
    np.testing.assert_allclose(s, z["sums_3pop"], rtol=1e-13, atol=1e-300)


def test_binned_sums_match_moments_golden(golden):
    """moments.LD.Parsing on im-parsing-example.vcf, 2 demes, logspace(2,5,4) bins."""
    z = golden("moments_im")
    keep = O.biallelic_keep(z["hap"])
    rows = [z["rows0"], z["rows1"]]
    s, _ = O.binned_sums(z["hap"][:, keep], z["pos"][keep], rows, z["bins"])
    assert list(z["ld_names"]) == O.ld_names(2)
    np.testing.assert_allclose(s, z["ld_sums"], rtol=1e-10)
    het = O.heterozygosity(z["hap"][:, keep], rows)
    np.testing.assert_allclose([het[h] for h in z["het_names"]], z["het_sums"], rtol=1e-12)


def test_genotype_counts_match_reference(golden):
    z = golden("geno")
    c, nv = O.genotype_counts_for_pairs(z["geno_miss"], z["idx_i"], z["idx_j"])
    assert np.array_equal(c, z["counts9_miss"]) and np.array_equal(nv, z["nvalid_miss"])
    c, nv = O.genotype_counts_for_pairs(z["geno"], z["idx_i"], z["idx_j"])
    assert nv is None and np.array_equal(c, z["counts9"])
    c, _ = O.genotype_counts_for_pairs(z["geno_miss"], z["idx_i"], z["idx_j"], z["rows"])
    assert np.array_equal(c, z["counts9_rows"])


def test_rogers_huff_matches_reference(golden):
    z = golden("geno")
    # the reference centres in float64 (rounding noise ~1e-15 where r is 0)
    _close(O.rogers_huff_r(z["geno"]), z["rh_r_condensed"], rtol=1e-9, atol=1e-12)
    _close(O.rogers_huff_r_pairs(z["geno"], z["idx_i"], z["idx_j"]), z["rh_r_pairs"],
           rtol=1e-9, atol=1e-12)
    with pytest.raises(ValueError):
        O.rogers_huff_r(z["geno_miss"])


def _same_ieee(got, ref, rtol):
    """Equal NaN / inf pattern, finite values within rtol."""
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    inf = np.isinf(ref)
    assert np.array_equal(np.isinf(got), inf) and np.array_equal(got[inf], ref[inf])
    f = np.isfinite(ref)
    np.testing.assert_allclose(got[f], ref[f], rtol=rtol, atol=0)


def test_genotype_dd_and_sigma_d2_match_reference_kernels(golden):
    z = golden("geno")
    for tag in ("", "_miss"):
        c = z["counts9" + tag]
        # _DD_GENO_SINGLE_KERN and _SIGMA_D2_GENO_KERN run as host C++
        _same_ieee(O.dd_geno_single(c), z["dd_geno" + tag], 1e-12)
        _same_ieee(O.sigma_d2_geno(c), z["sigma_d2" + tag], 1e-12)


def test_rogers_huff_from_counts_matches_reference(golden):
    z = golden("geno")
    _close(O.rogers_huff_r_counts(z["counts9"]), z["rh_r_pairs"], rtol=1e-9, atol=1e-12)
    # with missing data the reference raises; the pairwise-complete definition
    # equals the dosage-level restatement
    c, _ = O.genotype_counts_for_pairs(z["geno_miss"], z["idx_i"], z["idx_j"])
    _close(O.rogers_huff_r_counts(c),
           O.rogers_huff_r_pairs(z["geno_miss"], z["idx_i"], z["idx_j"]), rtol=1e-12, atol=0)


@pytest.mark.parametrize("P", [1, 2, 3, 4])
def test_genotype_multi_pop_stats_match_reference(golden, P):
    # compute_multi_pop_statistics_batch_geno (genotype_kernels.py:889-936),
    # every dd / dz / pi2 case of 1-4 populations, with and without n_valid
    z = golden("geno_stats")
    cs = [z[f"counts_{q}"] for q in range(P)]
    with np.errstate(divide="ignore", invalid="ignore"):
        got = O.geno_multi_pop_stats(cs, [c.sum(1) for c in cs])
        got0 = O.geno_multi_pop_stats(cs, [None] * P)
    _same_ieee(got, z[f"multi_{P}"], 1e-13)
    _same_ieee(got0, z[f"multi_{P}_nonv"], 1e-13)


@pytest.mark.parametrize("P", [2, 3])
def test_genotype_binned_sums_match_reference(golden, P):
    # the genotype loop of moments_ld._compute_ld_sums run through the
    # reference's own pair iterator, counter and statistics
    z = golden("geno_binned")
    rows = [z[f"rows{q}"] for q in range(P)]
    keep = np.where(O.union_polymorphic(z["geno"], rows))[0]
    assert np.array_equal(keep, z[f"keep_{P}"])
    s, _ = O.geno_binned_sums(z["geno"][:, keep], z["pos"][keep], rows, z["bins"])
    np.testing.assert_allclose(s, z[f"sums_{P}"], rtol=1e-12, atol=1e-12 * np.abs(s).max())


def test_genotype_counts_fold_dosages_above_two(golden):
    # the reference kernel's class index 3 g_i + g_j folds the values 3..8
    z = golden("geno")
    c, nv = O.genotype_counts_for_pairs(z["geno_odd"], z["idx_i"], z["idx_j"])
    assert np.array_equal(c, z["counts9_odd"]) and np.array_equal(nv, z["nvalid_odd"])


def test_window_zns_matches_reference(golden):
    # _zns_from_precomputed (ld_statistics.py:595-676) per window, both estimators
    z = golden("windows")
    b = z["bounds"]
    for k, (s, e) in enumerate(zip(b[:-1], b[1:])):
        assert O.zns_window(z["hap"], s, e, True) == pytest.approx(z["zns_proj"][k], rel=1e-12)
        assert O.zns_window(z["hap"], s, e, False) == pytest.approx(z["zns_naive"][k], rel=1e-12)


def test_omega_matches_reference(golden):
    """Kim and Nielsen's omega (ld_statistics.py:761-862): sigma_D^2 and naive
    r^2 over segregating sites, missing_data 'exclude', and a precomputed r^2
    matrix, against the reference's own results."""
    z = golden("omega")
    for k in range(3):
        h = z[f"hap{k}"]
        np.testing.assert_allclose(O.omega_hap(h), z[f"omega_sd2_{k}"], rtol=1e-12)
        np.testing.assert_allclose(O.omega_hap(h, "r2"), z[f"omega_r2_{k}"], rtol=1e-12)
        np.testing.assert_allclose(O.omega_hap(h, missing_data="exclude"),
                                   z[f"omega_sd2_excl_{k}"], rtol=1e-12)
        np.testing.assert_allclose(O.omega_matrix(z[f"r2_{k}"]), z[f"omega_arr_{k}"], rtol=1e-12)


def test_locate_unlinked_matches_reference(golden):
    z = golden("unlinked")
    for k in range(3):
        size, step = (int(v) for v in z[f"args{k}"])
        got = O.locate_unlinked(z[f"hap{k}"], size, step, float(z[f"thr{k}"]))
        assert np.array_equal(got, z[f"loc{k}"])


def test_diploid_zns_omega_match_reference(golden):
    z = golden("diploid_ld")
    for k in range(3):
        g = z[f"geno{k}"]
        np.testing.assert_allclose(O.r2_matrix_diploid(g), z[f"r2_{k}"], rtol=1e-12, atol=1e-15)
        np.testing.assert_allclose(O.zns_diploid(g), z[f"zns_{k}"], rtol=1e-12)
        np.testing.assert_allclose(O.omega_diploid(g), z[f"omega_{k}"], rtol=1e-12)
        np.testing.assert_allclose(O.zns_diploid(g, "exclude"), z[f"zns_excl_{k}"], rtol=1e-12,
                                   atol=1e-15)
        np.testing.assert_allclose(O.omega_diploid(g, "exclude"), z[f"omega_excl_{k}"],
                                   rtol=1e-12)


def test_mu_ld_matches_reference(golden):
    """mu_LD (ld_statistics.py:865-918) of the reference, with and without
    missing data and with missing_data='exclude': oracle and package."""
    from pg_gpu_gb300 import ld_statistics as LS
    from pg_gpu_gb300.haplotype_matrix import HaplotypeMatrix
    z = golden("mu_ld")
    k = 0
    while f"hap{k}" in z.files:
        hap = z[f"hap{k}"]
        pos = np.arange(1, hap.shape[1] + 1, dtype=np.int64) * 100
        assert O.mu_ld(hap) == pytest.approx(float(z[f"mu_{k}"]), abs=1e-15)
        assert O.mu_ld(hap, "exclude") == pytest.approx(float(z[f"mu_excl_{k}"]), abs=1e-15)
        hm = HaplotypeMatrix(hap.copy(), pos)
        assert LS.mu_ld(hm) == pytest.approx(float(z[f"mu_{k}"]), abs=1e-15)
        assert LS.mu_ld(hm, missing_data="exclude") == pytest.approx(float(z[f"mu_excl_{k}"]),
                                                                     abs=1e-15)
        k += 1
    assert k >= 7


def test_naive_r2_equals_r2_where_valid_sets_agree():
    # the identity the tensor-core window kernel uses for pairs whose two SNPs
    # have the same valid haplotypes (every pair of a panel without missing
    # data): the naive r^2 from per-site frequencies equals the pairwise r^2,
    # x^2 / (p_A q_A p_B q_B) = x^2 u_i u_j with u = 1 / (dac (nv - dac));
    # with missing data the two differ
    rng = np.random.default_rng(41)
    H, M = 64, 300
    hap = (rng.random((H, M)) < rng.beta(0.3, 0.3, M)).astype(np.int8)
    idx = np.arange(M)
    b, e = np.array([0, 17, 100]), np.array([M, 90, 300])
    sums, cnt = O.window_sums(hap, idx, b, e)
    np.testing.assert_allclose(sums[:, 5], sums[:, 0], rtol=1e-12)
    assert np.array_equal(cnt[:, 0], cnt[:, 2])  # n = H >= 4 for every pair
    hap[rng.random(hap.shape) < 0.05] = -1
    sums2, _ = O.window_sums(hap, idx, b, e)
    assert np.all(np.abs(sums2[:, 5] - sums2[:, 0]) > 1e-9 * np.abs(sums2[:, 0]))


def test_bin_vote_equals_bisection():
    # the warp-vote bin of a distance (thresholds at or below it, less one:
    # the tensor-core kernels' unit classification) against a bisection over
    # the same right-open integer thresholds (ceil of the bin edges, as the
    # reference's np.digitize bins integer distances), with equal thresholds
    # (bin edges closer than 1 bp) and the range ends
    rng = np.random.default_rng(5)

    def bisect(thr, d):
        n = len(thr) - 1
        if d < thr[0] or d >= thr[n]:
            return -1
        lo, hi = 0, n
        while hi - lo > 1:
            mid = (lo + hi) // 2
            if thr[mid] <= d:
                lo = mid
            else:
                hi = mid
        return lo

    def vote(thr, d):
        n = len(thr) - 1
        c = int(np.sum(thr[: n + 1] <= d))
        return -1 if c == 0 or c > n else c - 1

    for n_bins in (1, 2, 20, 31, 32, 33, 63, 64):
        edges = np.sort(rng.uniform(0, 5_000, n_bins + 1))
        edges[n_bins // 2] = edges[max(0, n_bins // 2 - 1)] + 0.3  # two edges within 1 bp
        edges = np.sort(edges)
        thr = np.ceil(edges).astype(np.int64)
        for d in list(rng.integers(-10, 5_010, 400)) + list(thr) + list(thr - 1):
            assert vote(thr, int(d)) == bisect(thr, int(d)), (n_bins, d)
