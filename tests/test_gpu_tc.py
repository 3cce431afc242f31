"""GPU parity of the tcgen05 tensor-core binned-sum form.

Same bar as the plain form: pair counts per bin equal the oracle's exactly,
and every bin sum is within 2e-6 * sum|x| of the float64 oracle.  Cases cover
one and two populations, SNP counts that leave partial 64-SNP tiles, sample
sizes that are not multiples of 128 (K padding), 1,000 haplotypes per
population, genetic-map distances and non-integer positions.
"""
import numpy as np
import pytest

from oracle import ld_oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

from pg_gpu_gb300 import _ops  # noqa: E402

SUM_TOL = 2e-6


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


def check(hap, pos, rows, bins, **kw):
    hap_d = torch.as_tensor(hap, device="cuda")
    pops = [_ops.pack(hap_d, r) for r in rows]
    sums, cnt = _ops.binned_sums(pops, _ops.positions_f64(pos), bins, form="tc", **kw)
    okw = {}
    if "bin_coord" in kw:
        okw["coords"] = kw["bin_coord"]
    if "max_dist" in kw:
        okw["max_dist"] = kw["max_dist"]
    ref, ref_cnt, ref_abs = O.binned_sums(hap, pos, rows, bins, abs_sums=True, **okw)
    assert np.array_equal(cnt.cpu().numpy(), ref_cnt)
    err = np.abs(sums.cpu().numpy() - ref)
    worst = float((err / np.maximum(ref_abs, 1e-300)).max())
    assert np.all(err <= SUM_TOL * ref_abs + 1e-300), worst
    return worst


@pytest.mark.parametrize("P", [1, 2])
def test_tc_matches_reference_fixture(golden, P):
    z = golden("binned")
    check(z["hap"], z["pos"], [z["rows0"], z["rows1"]][:P], z["bins"])


def test_tc_matches_moments_golden(golden):
    z = golden("moments_im")
    keep = O.biallelic_keep(z["hap"])
    check(z["hap"][:, keep], z["pos"][keep], [z["rows0"], z["rows1"]], z["bins"])


@pytest.mark.parametrize("H,M", [(40, 65), (130, 129), (300, 191), (257, 640)])
def test_tc_ragged_sizes(H, M):
    rng = np.random.default_rng(H * 1000 + M)
    hap = copying_model(rng, H, M, 6, 0.02, missing=0.03)
    pos = np.sort(rng.choice(M * 300, M, replace=False)).astype(np.int64)
    bins = np.logspace(2, np.log10(M * 150), 8)
    h2 = H // 2
    check(hap, pos, [np.arange(h2)], bins)
    check(hap, pos, [np.arange(h2), np.arange(h2, H)], bins)


def test_tc_large_populations():
    rng = np.random.default_rng(12)
    hap = copying_model(rng, 2000, 700, 40, 1e-3, missing=0.02)
    pos = np.sort(rng.choice(700_000, 700, replace=False)).astype(np.int64)
    check(hap, pos, [np.arange(1000), np.arange(1000, 2000)], np.logspace(3, 5.3, 13))


def test_tc_genetic_distance_and_fractional_positions():
    rng = np.random.default_rng(21)
    hap = copying_model(rng, 96, 400, 8, 5e-3, missing=0.01)
    pos = np.sort(rng.choice(200_000, 400, replace=False)).astype(np.float64) + 0.25
    gmap = np.cumsum(rng.random(400)) * 1e-5
    rows = [np.arange(48), np.arange(48, 96)]
    check(hap, pos, rows, np.array([0.0, 1e-4, 3e-4, 1e-3]), max_dist=60_000, bin_coord=gmap)
    check(hap, pos, rows, np.logspace(2, 4.7, 9))


@pytest.mark.parametrize("H,M", [(2000, 600), (130, 700), (33, 257)])
def test_tc_band_pairs_match_oracle(H, M):
    # per-pair counts, n and float32 r^2 / DD / Dz / pi2 of the tensor-core
    # form: counts bit-exact, statistics within 1e-6 of the float64 oracle,
    # and equal to the plain form's output
    rng = np.random.default_rng(H + M)
    hap = (rng.random((H, M)) < rng.beta(0.3, 0.3, M)).astype(np.int8)
    hap[rng.random(hap.shape) < 0.02] = -1
    pos = np.sort(rng.choice(200_000, M, replace=False)).astype(np.int64)
    pk = _ops.pack(torch.as_tensor(hap, device="cuda"))
    pos_d = _ops.positions_f64(pos)
    c_tc, nv_tc, st_tc = _ops.band_pairs(pk, pos_d, 20_000, form="tc")
    c_pl, nv_pl, st_pl = _ops.band_pairs(pk, pos_d, 20_000, form="plain")
    ii, jj = O.pairs_within_distance(pos, 20_000)
    rc, rnv = O.counts_for_pairs(hap, ii, jj)
    assert np.array_equal(c_tc.cpu().numpy(), rc) and np.array_equal(nv_tc.cpu().numpy(), rnv)
    assert np.array_equal(c_pl.cpu().numpy(), rc)
    st = st_tc.cpu().numpy().astype(np.float64)
    ref = np.stack([O.r_squared(rc, rnv), O.dd(rc, None, rnv), O.dz(rc, None, rnv),
                    O.pi2(rc, None, rnv)], axis=1)
    assert np.array_equal(np.isnan(st), np.isnan(ref))
    m = ~np.isnan(ref) & (np.abs(ref) > 1e-30)
    assert (np.abs(st[m] - ref[m]) / np.abs(ref[m])).max() <= 1e-6
    z = ref == 0
    assert np.all(st[z] == 0)


@pytest.mark.parametrize("form", ["tc", "plain"])
def test_sharded_binned_sums_add_up(form):
    # the multi-rank partition (pg_gpu_gb300/shard.py) run as three shards on
    # one device: the partials' sum is the oracle's whole-panel result
    from pg_gpu_gb300 import shard as S
    rng = np.random.default_rng(77)
    H, M = 300, 2_500
    hap = copying_model(rng, 2 * H, M, 20, 2e-3, missing=0.02)
    pos = np.sort(rng.choice(2_000_000, M, replace=False)).astype(np.int64)
    bins = np.array([0.0, 1e3, 1e4, 5e4, 1e5])
    rows = [np.arange(0, H), np.arange(H, 2 * H)]
    hap_d = torch.as_tensor(hap, device="cuda")
    pops = [_ops.pack(hap_d, r) for r in rows]
    pos_d = _ops.positions_f64(pos)
    compute = S.slice_binned_sums(pops, pos_d, bins, form=form)
    acc_s, acc_c = 0.0, 0
    for sh in S.plan_shards(pos, bins[-1], 3):
        part = S.shard_partial(compute, sh)
        acc_s = acc_s + part[0].cpu().numpy()
        acc_c = acc_c + part[1].cpu().numpy()
    ref, ref_cnt, ref_abs = O.binned_sums(hap, pos, rows, bins, abs_sums=True)
    assert np.array_equal(acc_c, ref_cnt)
    # each shard's sums carry the float32 per-pair error of the halo pairs twice
    assert np.all(np.abs(acc_s - ref) <= 3 * SUM_TOL * ref_abs + 1e-300)


def test_full_size_headline_panel():
    # the binned two-population workload at full size (2 x 1,000 haplotypes,
    # 200,000 SNPs over 20 Mb, 20 log bins up to 1 Mb; ~1.9e9 pairs):
    # per-bin pair counts equal the exact counts from the positions alone, the
    # tensor-core and popcount forms agree on them, and a 300-anchor sample of
    # the pairs (~1e6, computed as a shard) matches the oracle
    from pg_gpu_gb300 import shard as S
    rng = np.random.default_rng(20261203)
    M, H = 200_000, 1000
    hap = np.concatenate([copying_model(rng, H, M, 40, 1e-3, missing=0.0) for _ in range(2)])
    pos = np.sort(rng.choice(20_000_000, M, replace=False)).astype(np.int64)
    bins = np.concatenate([[0.0], np.logspace(3, 6, 20)])
    rows = [np.arange(0, H), np.arange(H, 2 * H)]
    hap_d = torch.as_tensor(hap, device="cuda")
    pops = [_ops.pack(hap_d, r) for r in rows]
    pos_d = _ops.positions_f64(pos)
    sums_tc, cnt_tc = _ops.binned_sums(pops, pos_d, bins, form="tc")
    _, cnt_pl = _ops.binned_sums(pops, pos_d, bins, form="plain")
    pf = pos.astype(np.float64)
    # pairs (i, j > i) with pos[j] - pos[i] < e, for every bin edge e
    below = [int(np.maximum(np.searchsorted(pf, pf + e, side="left") - np.arange(M) - 1, 0).sum())
             for e in bins]
    exact = np.diff(np.asarray(below, np.int64))
    assert np.array_equal(cnt_tc.cpu().numpy(), exact)
    assert np.array_equal(cnt_pl.cpu().numpy(), exact)
    assert np.all(np.isfinite(sums_tc.cpu().numpy()))
    A = 100
    sh = S.Shard(0, 0, A, int(np.searchsorted(pf, pf[A - 1] + bins[-1], side="right")))
    part_s, part_c = S.shard_partial(S.slice_binned_sums(pops, pos_d, bins, form="tc"), sh)
    ref, ref_cnt, ref_abs = O.binned_sums(hap, pos, rows, bins, abs_sums=True,
                                          anchor_stop=A, pair_block=100_000)
    assert np.array_equal(part_c.cpu().numpy(), ref_cnt)
    err = np.abs(part_s.cpu().numpy() - ref)
    assert np.all(err <= 3 * SUM_TOL * ref_abs + 1e-300)
