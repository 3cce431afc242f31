"""GPU parity of the dense all-pairs outputs and of the recombination-map
binning of moments_ld.

* pairwise_LD_v / pairwise_r2 ('r2'): equal to the reference's float64
  matrices (fixtures from the reference's HaplotypeMatrix, rtol 1e-13);
  'rogers_huff' within 1e-12.
* windowed_r_squared: pair counts per bin exact; each percentile within
  1e-12 of the reference's (its r^2 are rounded float expressions, this
  library's are exact quotients of the joint counts), both estimators.
* moments_ld with r_bins and a recombination map: bins and heterozygosity
  as the reference; LD sums within 1e-6 of each value (5 % of the bin's sum
  of |x| for bins whose terms cancel), haplotype and genotype paths.
"""
import numpy as np
import pytest

from oracle import ld_oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

from pg_gpu_gb300 import moments_ld  # noqa: E402
from pg_gpu_gb300.haplotype_matrix import HaplotypeMatrix  # noqa: E402

RTOL = 1e-6
FLOOR = 0.05


def np_(t):
    return t.cpu().numpy() if hasattr(t, "cpu") else np.asarray(t)


def _nan_close(got, want, rtol):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    assert got.shape == want.shape
    assert np.array_equal(np.isnan(got), np.isnan(want))
    m = ~np.isnan(want)
    np.testing.assert_allclose(got[m], want[m], rtol=rtol, atol=0)


@pytest.mark.parametrize("k", range(4))
def test_pairwise_matrices_match_reference(golden, k):
    z = golden("dense")
    hap, pos = z[f"hap{k}"], z[f"pos{k}"]
    D = np_(HaplotypeMatrix(hap, pos).pairwise_LD_v())
    np.testing.assert_allclose(D, z[f"ldv{k}"], rtol=1e-13, atol=1e-16)
    r2 = np_(HaplotypeMatrix(hap, pos).pairwise_r2())
    np.testing.assert_allclose(r2, z[f"r2_{k}"], rtol=1e-13, atol=1e-16)
    if f"rh_{k}" in z.files:
        rh = np_(HaplotypeMatrix(hap, pos).pairwise_r2(estimator="rogers_huff"))
        np.testing.assert_allclose(rh, z[f"rh_{k}"], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("k", range(4))
def test_windowed_r_squared_matches_reference(golden, k):
    z = golden("dense")
    hap, pos, bins = z[f"hap{k}"], z[f"pos{k}"], z[f"wbins{k}"]
    res, cnt = HaplotypeMatrix(hap, pos).windowed_r_squared(bins, percentile=[5, 50, 95])
    assert np.array_equal(cnt, z[f"wcnt{k}"])
    _nan_close(res, z[f"wr2_{k}"], 1e-12)
    med, cnt1 = HaplotypeMatrix(hap, pos).windowed_r_squared(bins, percentile=50)
    assert med.shape == (len(bins) - 1,) and np.array_equal(cnt1, z[f"wcnt{k}"])
    _nan_close(med, z[f"wr2med_{k}"], 1e-12)
    if f"wrh_{k}" in z.files:
        rr, rc = HaplotypeMatrix(hap, pos).windowed_r_squared(bins, percentile=[25, 75],
                                                              estimator="rogers_huff")
        assert np.array_equal(rc, z[f"wrhcnt{k}"])
        _nan_close(rr, z[f"wrh_{k}"], 1e-12)


def test_dense_larger_panel_against_oracle():
    # 700 haplotypes (K padding, 22 words) x 1,100 SNPs (partial tiles), 3 %
    # missing: the full matrices and the percentiles of 10 bins with some
    # empty, against the oracle
    rng = np.random.default_rng(44)
    H, M = 700, 1_100
    hap = (rng.random((H, M)) < rng.beta(0.3, 0.3, M)).astype(np.int8)
    hap[rng.random(hap.shape) < 0.03] = -1
    hap[:, 17] = 0  # a monomorphic site (zero denominators)
    pos = np.sort(rng.choice(2_000_000, M, replace=False)).astype(np.int64)
    hm = HaplotypeMatrix(hap, pos)
    np.testing.assert_allclose(np_(hm.pairwise_LD_v()), O.pairwise_ld_v(hap), rtol=1e-13,
                               atol=1e-16)
    np.testing.assert_allclose(np_(hm.pairwise_r2()), O.pairwise_r2(hap), rtol=1e-13, atol=1e-16)
    bins = np.array([0.0, 100.0, 1e3, 1e4, 3e4, 1e5, 3e5, 1e6, 2e6, 3e6, 4e6])
    res, cnt = hm.windowed_r_squared(bins, percentile=[0, 1, 33.3, 50, 99.9, 100])
    ref, ref_cnt = O.windowed_r_squared(hap, pos, bins, [0, 1, 33.3, 50, 99.9, 100])
    assert np.array_equal(cnt, ref_cnt)
    assert cnt[-1] == 0 and np.all(np.isnan(res[-1]))
    _nan_close(res, ref, 1e-12)


def test_rbins_match_reference(golden):
    # moments_ld.compute_ld_statistics with recombination-distance bins: the
    # genetic map interpolated at the variants (moments_ld.py:211-224), the
    # physical search radius from the smallest local rate (:227-245), pairs
    # binned by genetic distance
    import os
    z = golden("rbins")
    im = golden("moments_im")
    rec = os.path.join(os.path.dirname(__file__), "golden", "rec_map_im.txt")
    sets = {"deme0": list(map(int, im["rows0"])), "deme1": list(map(int, im["rows1"]))}
    for tag, geno in (("hap", False), ("geno", True)):
        hm = HaplotypeMatrix(im["hap"], im["pos"], sample_sets=sets)
        res = moments_ld.compute_ld_statistics(haplotype_matrix=hm, rec_map_file=rec,
                                               pops=["deme0", "deme1"], r_bins=z["r_bins"],
                                               use_genotypes=geno, report=False)
        np.testing.assert_array_equal(np.asarray(res["bins"], np.float64), z[f"{tag}_bins"])
        np.testing.assert_allclose(res["sums"][-1], z[f"{tag}_het"], rtol=1e-12)
        got = np.array(res["sums"][:-1])
        want = z[f"{tag}_ld"]
        if not geno:
            keep = O.biallelic_keep(im["hap"])
            gmap = moments_ld._interpolate_genetic_distances(im["pos"][keep], rec)
            _, _, scale = O.binned_sums(im["hap"][:, keep], im["pos"][keep],
                                        [im["rows0"], im["rows1"]], z["r_bins"], coords=gmap,
                                        max_dist=moments_ld._max_bp_for_r_dist(
                                            im["pos"][keep], gmap, float(z["r_bins"][-1])),
                                        abs_sums=True)
            rel = O.bin_errors(got, want, scale, FLOOR)
        else:
            rel = O.bin_errors(got, want)
        print(f"{tag}: max error relative to the bin value {rel.max():.3g}")
        assert rel.max() <= RTOL, rel.max()
