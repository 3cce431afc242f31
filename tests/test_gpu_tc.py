"""GPU parity of the tcgen05 tensor-core binned-sum form.

Pair counts per bin equal the oracle's exactly.  Every bin sum is within
1e-6 of its float64 oracle value (RTOL); a bin whose terms cancel to below
5 % of their sum of |x| (FLOOR) is held to 1e-6 of that share instead.  The
moments golden sums are held to the reference's own criterion, 1e-6 of each
value.  Cases cover one and two populations, SNP counts that leave partial
64-SNP tiles, sample sizes that are not multiples of 128 (K padding), 1,000
haplotypes per population, genetic-map distances, non-integer positions,
anchor ranges and the full-size benchmark panel.
"""
import multiprocessing as mp

import numpy as np
import pytest

from oracle import ld_oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

from pg_gpu_gb300 import _ops, synthetic  # noqa: E402

RTOL = 1e-6
FLOOR = 0.05


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


def check(hap, pos, rows, bins, floor=FLOOR, **kw):
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
    rel = O.bin_errors(sums.cpu().numpy(), ref, ref_abs, floor)
    worst = float(rel.max())
    print(f"max error relative to the bin value: {worst:.3g}")
    assert worst <= RTOL, worst
    return worst


@pytest.mark.parametrize("P", [1, 2])
def test_tc_matches_reference_fixture(golden, P):
    z = golden("binned")
    check(z["hap"], z["pos"], [z["rows0"], z["rows1"]][:P], z["bins"])


def test_tc_matches_moments_golden(golden):
    z = golden("moments_im")
    keep = O.biallelic_keep(z["hap"])
    # the reference's criterion for moments' sums: 1e-6 of each value
    check(z["hap"][:, keep], z["pos"][keep], [z["rows0"], z["rows1"]], z["bins"], floor=0.0)


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
    # the multi-rank partition (pg_gpu_gb300/shard.py) run as three anchor
    # ranges on one device: each range matches the oracle's sums over its
    # anchors, and the ranges add up to the whole panel
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
    compute = S.range_binned_sums(pops, pos_d, bins, form=form)
    acc_s, acc_c = 0.0, 0
    for sh in S.plan_shards(pos, bins[-1], 3):
        part = S.shard_partial(compute, sh)
        ref, ref_cnt, ref_abs = O.binned_sums(hap, pos, rows, bins, abs_sums=True,
                                              anchor_start=sh.start, anchor_stop=sh.stop)
        assert np.array_equal(part[1].cpu().numpy(), ref_cnt)
        assert O.bin_errors(part[0].cpu().numpy(), ref, ref_abs, FLOOR).max() <= RTOL
        acc_s = acc_s + part[0].cpu().numpy()
        acc_c = acc_c + part[1].cpu().numpy()
    ref, ref_cnt, ref_abs = O.binned_sums(hap, pos, rows, bins, abs_sums=True)
    assert np.array_equal(acc_c, ref_cnt)
    assert O.bin_errors(acc_s, ref, ref_abs, FLOOR).max() <= RTOL


@pytest.mark.parametrize("form", ["tc", "plain"])
def test_anchor_ranges_edge_cases(form):
    # empty, single-anchor, last-anchor and whole-panel ranges, and a range
    # outside the panel (rejected)
    rng = np.random.default_rng(78)
    hap = copying_model(rng, 160, 700, 8, 3e-3, missing=0.02)
    pos = np.sort(rng.choice(300_000, 700, replace=False)).astype(np.int64)
    bins = np.logspace(2, 4.7, 7)
    rows = [np.arange(80), np.arange(80, 160)]
    hap_d = torch.as_tensor(hap, device="cuda")
    pops = [_ops.pack(hap_d, r) for r in rows]
    pos_d = _ops.positions_f64(pos)
    for a0, a1 in [(5, 5), (0, 1), (350, 351), (699, 700), (0, 700), (63, 129), (640, 700)]:
        sums, cnt = _ops.binned_sums(pops, pos_d, bins, form=form, anchors=(a0, a1))
        ref, ref_cnt, ref_abs = O.binned_sums(hap, pos, rows, bins, abs_sums=True,
                                              anchor_start=a0, anchor_stop=a1)
        assert np.array_equal(cnt.cpu().numpy(), ref_cnt), (a0, a1)
        assert O.bin_errors(sums.cpu().numpy(), ref, ref_abs, FLOOR).max() <= RTOL, (a0, a1)
    from pg_gpu_gb300._lib import PgldError
    with pytest.raises(PgldError):
        _ops.binned_sums(pops, pos_d, bins, form=form, anchors=(10, 701))
    with pytest.raises(PgldError):
        _ops.binned_sums(pops, pos_d, bins, form=form, anchors=(20, 10))


def test_full_size_headline_panel():
    # the benchmark's binned two-population panel itself (2 x 1,000
    # haplotypes sharing 40 founders, 10 % founder alleles flipped per
    # population, 2 % missing, 200,000 SNPs over 20 Mb, 20 log bins from 1 kb
    # to 1 Mb; ~1.9e9 pairs): per-bin pair counts of both forms equal the
    # exact counts from the positions alone, and twelve anchor blocks spread
    # over the chromosome (>= 1e7 pairs) match the oracle -- counts exactly,
    # every statistic within RTOL of its bin value (FLOOR for cancelling bins)
    cfg = synthetic.BINNED2POP
    panel, pos = synthetic.shared_founder_panel(cfg, torch.device("cuda", 0))
    M, H = cfg["n_snp"], cfg["hap_per_pop"]
    bins = cfg["bins"]
    md = float(bins[-1])
    rows_d = [torch.arange(q * H, (q + 1) * H, dtype=torch.int32, device="cuda") for q in range(2)]
    pops = [_ops.pack(panel, r) for r in rows_d]
    pos_d = _ops.positions_f64(pos)
    sums_tc, cnt_tc = _ops.binned_sums(pops, pos_d, bins, form="tc")
    _, cnt_pl = _ops.binned_sums(pops, pos_d, bins, form="plain")
    pf = pos.astype(np.float64)
    below = [int(np.maximum(np.searchsorted(pf, pf + e, side="left") - np.arange(M) - 1, 0).sum())
             for e in bins]
    exact = np.diff(np.asarray(below, np.int64))
    assert np.array_equal(cnt_tc.cpu().numpy(), exact)
    assert np.array_equal(cnt_pl.cpu().numpy(), exact)
    assert np.all(np.isfinite(sums_tc.cpu().numpy()))
    # twelve anchor blocks of ~9e5 pairs each, spread over the chromosome
    blocks, tasks, gpu = [], [], []
    rows = [np.arange(0, H), np.arange(H, 2 * H)]
    for k in range(12):
        a0 = k * M // 12 + M // 40
        a1, _ = synthetic.anchors_per_pairs(pos, md, a0, 900_000)
        halo = int(np.searchsorted(pf, pf[a1 - 1] + md, side="right"))
        blocks.append((a0, a1))
        gpu.append(_ops.binned_sums(pops, pos_d, bins, form="tc", anchors=(a0, a1)))
        tasks.append(((panel[:, a0:halo].cpu().numpy(), pos[a0:halo], rows, bins),
                      dict(anchor_stop=a1 - a0, pair_block=100_000)))
    with mp.get_context("spawn").Pool(min(12, mp.cpu_count())) as pool:
        refs = pool.map(O.binned_sums_task, tasks)
    n_checked = 0
    worst = np.zeros(15)
    for (a0, a1), (s_g, c_g), (ref, ref_cnt, ref_abs) in zip(blocks, gpu, refs):
        assert np.array_equal(c_g.cpu().numpy(), ref_cnt), (a0, a1)
        n_checked += int(ref_cnt.sum())
        rel = O.bin_errors(s_g.cpu().numpy(), ref, ref_abs, FLOOR)
        worst = np.maximum(worst, rel.max(axis=0))
    from pg_gpu_gb300.ld_pipeline import ld_names
    names = ld_names(2)
    print(f"{n_checked} pairs checked; max error relative to the bin value per statistic: " +
          ", ".join(f"{n}={w:.2e}" for n, w in zip(names, worst)))
    assert n_checked >= 10_000_000
    assert worst.max() <= RTOL, worst


def test_bounded_wait_expiry_reports_and_recovers():
    # failure detection without a fault: the one-shot test hook makes the
    # next tensor-core launch issue no operand copies, so the MMA issuer's
    # bounded wait for the first stage expires (~10 ms); the launch drains,
    # frees its tensor memory and returns, the handle's status word holds a
    # wait-expiry code, and the next calls on the same handle are correct
    import ctypes
    from pg_gpu_gb300 import _lib as L
    rng = np.random.default_rng(31)
    hap = copying_model(rng, 200, 500, 8, 3e-3, missing=0.02)
    pos = np.sort(rng.choice(250_000, 500, replace=False)).astype(np.int64)
    bins = np.logspace(2, 4.7, 7)
    rows = [np.arange(100), np.arange(100, 200)]
    hap_d = torch.as_tensor(hap, device="cuda")
    pops = [_ops.pack(hap_d, r) for r in rows]
    pos_d = _ops.positions_f64(pos)
    h = L.handle()
    code = ctypes.c_int32(-1)
    L.check(L.lib().pgld_device_status(h, ctypes.byref(code), L.stream_ptr()), h)
    assert code.value == 0
    L.check(L.lib().pgld_set_test_fault(h, 1), h)
    _ops.binned_sums(pops, pos_d, bins, form="tc")
    L.check(L.lib().pgld_device_status(h, ctypes.byref(code), L.stream_ptr()), h)
    assert 3002 <= code.value <= 3005, code.value
    for _ in range(2):
        check(hap, pos, rows, bins)
        L.check(L.lib().pgld_device_status(h, ctypes.byref(code), L.stream_ptr()), h)
        assert code.value == 0


def test_autotuner_choice_is_cached_and_applied(tmp_path, monkeypatch):
    # the tuner times every (layout, stages) candidate on a synthetic panel of
    # the given sample sizes, stores the fastest keyed by (kind, words, GPU),
    # and calls of that kind then run with it; results do not depend on it
    import json
    from pg_gpu_gb300 import autotune
    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_cache", None)
    monkeypatch.setattr(autotune, "_applied", {})
    r = autotune.tune("binned2", [4, 4], n_snp=3_000, max_dist=2e5)
    assert r["choice"] in autotune.BINNED2_CANDIDATES
    assert set(r["ms"]) == {f"{a},{b}" for a, b in autotune.BINNED2_CANDIDATES}
    saved = json.load(open(tmp_path / "tune.json"))
    assert saved[r["key"]]["layout"] == r["choice"][0]
    assert autotune.lookup("binned2", [4, 4]) == r["choice"]
    # every candidate gives the oracle's sums
    rng = np.random.default_rng(5)
    hap = copying_model(rng, 256, 500, 8, 5e-3, missing=0.02)
    pos = np.sort(rng.choice(300_000, 500, replace=False)).astype(np.int64)
    rows = [np.arange(128), np.arange(128, 256)]
    from pg_gpu_gb300 import _lib as L
    for layout, stages in autotune.BINNED2_CANDIDATES:
        monkeypatch.setattr(autotune, "lookup", lambda kind, words: (layout, stages))
        monkeypatch.setattr(autotune, "_applied", {})
        check(hap, pos, rows, np.logspace(2, 5, 9))
    L.check(L.lib().pgld_set_tc_config(L.handle(), 0, 0), L.handle())
