"""GPU parity of the batched-window path (one launch over all windows).

Per-window sums of float32 per-pair statistics accumulate in float64; they are
held to |gpu - oracle| <= 2e-6 * sum|x| per window and statistic, pair counts
exactly, and ZnS to the reference's _zns_from_precomputed fixtures at 1e-5.
"""
import numpy as np
import pytest

from oracle import ld_oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

from pg_gpu_gb300 import _ops, ld_statistics  # noqa: E402
from pg_gpu_gb300.haplotype_matrix import HaplotypeMatrix  # noqa: E402


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


@pytest.mark.parametrize("H,form,layout", [(33, "plain", 0), (400, "plain", 0), (33, "tc", 1),
                                           (33, "tc", 2), (400, "tc", 1), (400, "tc", 2),
                                           (2000, "tc", 1), (2000, "tc", 2)])
def test_window_sums_match_oracle(H, form, layout, tc_layout):
    # layout (tensor cores): 1 = 64 x 64 tiles, 2 = 64 x 128 tiles
    with tc_layout(layout):
        _window_sums_check(H, form)


def _window_sums_check(H, form):
    rng = np.random.default_rng(H)
    M = 900
    hap = copying_model(rng, H, M, 12, 2e-3, missing=0.02)
    seg = np.where(O.segregating(hap))[0].astype(np.int32)
    # uneven and overlapping windows, including empty and one-SNP ones
    ns = len(seg)
    b = np.minimum(np.array([0, 0, 5, 5, 100, 131, 400, 700, 60], np.int64), ns)
    e = np.minimum(np.array([0, 1, 5, 37, 300, 131 + 64, 700, ns, 200], np.int64), ns)
    assert ns > 300
    pk = _ops.pack(torch.as_tensor(hap, device="cuda"))
    sums, cnt = _ops.window_sums(pk, torch.as_tensor(seg, device="cuda"), b, e, form=form)
    ref, rcnt = O.window_sums(hap, seg, b, e)
    assert np.array_equal(cnt.cpu().numpy(), rcnt)
    got = sums.cpu().numpy()
    # scale: per-pair magnitudes (the float32 per-pair values sum to these)
    for w in range(len(b)):
        sel = seg[b[w]:e[w]]
        if len(sel) < 2:
            assert np.all(got[w] == 0)
            continue
        a_, b_ = np.triu_indices(len(sel), 1)
        c, nv = O.counts_for_pairs(hap, sel[a_], sel[b_])
        n = c.astype(np.int64).sum(1)
        scale = np.array([np.nansum(np.abs(O.r_squared(c, nv))),
                          np.abs(ref[w, 1]) + 1e-12 * rcnt[w, 2],
                          np.abs(O.dd(c, None, n)).sum(), np.abs(O.dz(c, None, n)).sum(),
                          np.abs(O.pi2(c, None, n)).sum(), abs(ref[w, 5])])
        # sigma_D^2 terms can cancel: bound by the sum of |dd / pi2| per pair
        p = O.Pop(c, n)
        ddn, _ = O.dd_ii(p)
        pin, _ = O.pi2_iiii(p)
        ok = (n >= 4) & (pin != 0)
        scale[1] = np.abs(ddn[ok] / pin[ok]).sum()
        assert np.all(np.abs(got[w] - ref[w]) <= 2e-6 * scale + 1e-12), (w, got[w], ref[w])


def test_zns_matches_reference(golden):
    z = golden("windows")
    hm = HaplotypeMatrix(z["hap"], np.arange(z["hap"].shape[1]))
    bnd = z["bounds"]
    got = ld_statistics.windowed_zns(hm, bnd[:-1], bnd[1:])
    want = np.where(np.diff(bnd) < 4, np.nan, z["zns_proj"])
    assert np.array_equal(np.isnan(got), np.isnan(want))
    m = ~np.isnan(want)
    np.testing.assert_allclose(got[m], want[m], rtol=1e-5, atol=1e-9)
    got_r2 = ld_statistics.windowed_zns(hm, bnd[:-1], bnd[1:], estimator="r2")
    want_r2 = np.where(np.diff(bnd) < 4, np.nan, z["zns_naive"])
    np.testing.assert_allclose(got_r2[m], want_r2[m], rtol=1e-5, atol=1e-9)
    # whole-matrix ZnS: one window over every site
    full = O.zns_window(z["hap"], 0, z["hap"].shape[1], True)
    assert ld_statistics.zns(hm) == pytest.approx(full, rel=1e-5)
    assert ld_statistics.zns(hm, estimator="r2") == pytest.approx(
        O.zns_window(z["hap"], 0, z["hap"].shape[1], False), rel=1e-5)


@pytest.mark.parametrize("form", ["plain", "tc"])
def test_window_errors(form):
    pk = _ops.pack(np.zeros((8, 10), np.int8))
    with pytest.raises(IndexError):
        _ops.window_sums(pk, torch.arange(10, dtype=torch.int32, device="cuda"), [0], [11],
                         form=form)
    with pytest.raises(IndexError):
        _ops.window_sums(pk, torch.tensor([0, 3, 99], dtype=torch.int32, device="cuda"), [0], [3],
                         form=form)


def test_omega_matches_reference(golden):
    """omega of a HaplotypeMatrix from per-site row / column sums on the device
    equals the reference's omega (sigma_D^2, naive r^2, missing_data
    'exclude', precomputed r^2 matrix)."""
    z = golden("omega")
    for k in range(3):
        h = z[f"hap{k}"]
        pos = np.arange(h.shape[1], dtype=np.int64) * 1000
        hm = lambda: HaplotypeMatrix(h.copy(), pos.copy())  # noqa: E731
        np.testing.assert_allclose(ld_statistics.omega(hm()), z[f"omega_sd2_{k}"], rtol=1e-5)
        np.testing.assert_allclose(ld_statistics.omega(hm(), estimator="r2"), z[f"omega_r2_{k}"],
                                   rtol=1e-5)
        np.testing.assert_allclose(ld_statistics.omega(hm(), missing_data="exclude"),
                                   z[f"omega_sd2_excl_{k}"], rtol=1e-5, atol=1e-12)
        np.testing.assert_allclose(ld_statistics.omega(z[f"r2_{k}"]), z[f"omega_arr_{k}"],
                                   rtol=1e-12)
    with pytest.raises(ValueError, match="HaplotypeMatrix"):
        ld_statistics.omega(z["r2_0"], estimator="sigma_d2")
    with pytest.raises(ValueError, match="Unknown estimator"):
        ld_statistics.omega(z["r2_0"], estimator="nonsense")
    assert ld_statistics.omega(np.zeros((4, 4))) == 0.0


@pytest.mark.parametrize("H", [40, 300])
def test_windowed_omega_matches_oracle(H):
    rng = np.random.default_rng(H + 7)
    M = 400
    hap = copying_model(rng, H, M, 6, 0.01, missing=0.02)
    pos = np.arange(M, dtype=np.int64) * 100
    ws = np.array([0, 10, 50, 50, 200, 390, 100])
    we = np.array([3, 60, 130, 400, 330, 400, 102])
    hm = HaplotypeMatrix(hap, pos)
    for est in ("sigma_d2", "r2"):
        got = ld_statistics.windowed_omega(hm, ws, we, estimator=est)
        for w in range(len(ws)):
            if we[w] - ws[w] < 4:
                assert np.isnan(got[w])
                continue
            want = O.omega_hap(hap[:, ws[w]:we[w]], est)
            np.testing.assert_allclose(got[w], want, rtol=2e-5, atol=1e-12)
    # one window and the single-matrix call agree
    one = ld_statistics.windowed_omega(hm, [0], [M])[0]
    np.testing.assert_allclose(one, ld_statistics.omega(HaplotypeMatrix(hap, pos)), rtol=1e-12)


def test_locate_unlinked_matches_reference(golden):
    """Greedy pruning on naive r^2 of every pair closer than `size` variants
    (band pairs on the device, pruning on the host) equals the reference."""
    z = golden("unlinked")
    for k in range(3):
        size, step = (int(v) for v in z[f"args{k}"])
        h = z[f"hap{k}"]
        hm = HaplotypeMatrix(h, np.arange(h.shape[1], dtype=np.int64) * 100)
        got = hm.locate_unlinked(size=size, step=step, threshold=float(z[f"thr{k}"]))
        assert np.array_equal(got, z[f"loc{k}"])
    rng = np.random.default_rng(3)
    h = copying_model(rng, 300, 700, 5, 0.02, missing=0.02)
    hm = HaplotypeMatrix(h, np.arange(700, dtype=np.int64))
    assert np.array_equal(hm.locate_unlinked(64, 16, 0.3), O.locate_unlinked(h, 64, 16, 0.3))
    with pytest.raises(ValueError):
        hm.locate_unlinked(0, 1)


def test_diploid_zns_omega_match_reference(golden):
    """zns / omega of a GenotypeMatrix (squared dosage correlation from 9-way
    counts, pairs in chunks) equal the reference's zns_diploid / omega_diploid."""
    from pg_gpu_gb300.genotype_matrix import GenotypeMatrix
    z = golden("diploid_ld")
    for k in range(3):
        g = z[f"geno{k}"]
        pos = np.arange(g.shape[1], dtype=np.int64) * 100
        gm = lambda: GenotypeMatrix(g.copy(), pos.copy())  # noqa: E731
        np.testing.assert_allclose(ld_statistics.zns_diploid(gm()), z[f"zns_{k}"], rtol=1e-10)
        np.testing.assert_allclose(ld_statistics.omega_diploid(gm()), z[f"omega_{k}"], rtol=1e-10)
        np.testing.assert_allclose(ld_statistics.zns(gm(), missing_data="exclude"),
                                   z[f"zns_excl_{k}"], rtol=1e-10, atol=1e-15)
        np.testing.assert_allclose(ld_statistics.omega(gm(), missing_data="exclude"),
                                   z[f"omega_excl_{k}"], rtol=1e-10)
    # chunked pair enumeration gives the same sums as one chunk
    from pg_gpu_gb300.ld_statistics import _diploid_row_col_sums
    g = z["geno1"]
    a = _diploid_row_col_sums(GenotypeMatrix(g, np.arange(g.shape[1])), chunk_pairs=97)
    b = _diploid_row_col_sums(GenotypeMatrix(g, np.arange(g.shape[1])))
    np.testing.assert_allclose(a[0], b[0], rtol=1e-12)
    np.testing.assert_allclose(a[1], b[1], rtol=1e-12)


def test_full_size_windows():
    # the batched-window workload at full size: 400 haplotypes, 512 windows of
    # log-uniform 500..20,000 SNPs (each its own copying panel; 1.3e10 pairs).
    # On all windows: the pair counts are n (n - 1) / 2, every pair has n >= 4
    # (no missing data), and the tensor-core and popcount forms count alike;
    # the three smallest windows equal the oracle's sums
    rng = np.random.default_rng(20261504)
    H = 400
    sizes = np.exp(rng.uniform(np.log(500), np.log(20_000), 512)).astype(np.int64)
    we = np.cumsum(sizes)
    wb = we - sizes
    M = int(we[-1])
    hap = np.empty((H, M), np.int8)
    for w in range(len(sizes)):
        s, e = int(wb[w]), int(we[w])
        p = rng.beta(0.3, 0.3, size=e - s)
        f = (rng.random((40, e - s)) < p).astype(np.int8)
        for b in range(s, e, 1_000):  # a founder per haplotype per 1,000-SNP block
            hap[:, b:min(e, b + 1_000)] = f[rng.integers(0, 40, H), b - s:min(e, b + 1_000) - s]
    pk = _ops.pack(torch.as_tensor(hap, device="cuda"))
    sums, cnt = _ops.window_sums(pk, None, wb, we, form="tc")
    _, cnt_pl = _ops.window_sums(pk, None, wb, we, form="plain")
    c = cnt.cpu().numpy()
    assert np.array_equal(c[:, 0], sizes * (sizes - 1) // 2)
    assert np.array_equal(c[:, 2], c[:, 0]) and np.all(c[:, 1] <= c[:, 0])
    assert np.array_equal(c, cnt_pl.cpu().numpy())
    got = sums.cpu().numpy()
    assert np.all(np.isfinite(got))
    for w in np.argsort(sizes)[:3]:
        s, e = int(wb[w]), int(we[w])
        ref, rcnt = O.window_sums(hap[:, s:e], np.arange(e - s), [0], [e - s])
        assert np.array_equal(c[w], rcnt[0])
        sel = np.arange(s, e)
        a_, b_ = np.triu_indices(len(sel), 1)
        cc, nv = O.counts_for_pairs(hap, sel[a_], sel[b_])
        n = cc.astype(np.int64).sum(1)
        p_ = O.Pop(cc, n)
        ddn, _ = O.dd_ii(p_)
        pin, _ = O.pi2_iiii(p_)
        ok = (n >= 4) & (pin != 0)
        scale = np.array([np.nansum(np.abs(O.r_squared(cc, nv))), np.abs(ddn[ok] / pin[ok]).sum(),
                          np.abs(O.dd(cc, None, n)).sum(), np.abs(O.dz(cc, None, n)).sum(),
                          np.abs(O.pi2(cc, None, n)).sum(), abs(ref[0, 5])])
        assert np.all(np.abs(got[w] - ref[0]) <= 2e-6 * scale + 1e-12), (w, got[w], ref[0])
