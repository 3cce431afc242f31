"""Host logic of the dense outputs, no GPU: the percentile interpolation
from order statistics against numpy.percentile, and the oracle's dense
restatements against the reference's own results (tests/golden/dense.npz,
made by tests/golden/make_golden.py from the reference's HaplotypeMatrix)."""
import numpy as np
import pytest

from oracle import ld_oracle as O

pytest.importorskip("torch")
from pg_gpu_gb300 import _ops  # noqa: E402


@pytest.mark.parametrize("seed", range(6))
def test_percentiles_from_order_stats_equal_numpy(seed):
    rng = np.random.default_rng(seed)
    segs = [rng.random(n) ** 3 for n in (1, 2, 3, 7, 100, 1001, 0, 50)]
    segs.append(np.full(9, 0.25))
    counts = np.array([len(s) for s in segs])
    pct = [0, 0.1, 5, 12.5, 33.3, 50, 66.6, 95, 99.99, 100]

    def kth(keys):
        return [np.partition(segs[s], r)[r] for s, r in keys]

    got = _ops.percentiles_from_order_stats(counts, pct, kth)
    for s, v in enumerate(segs):
        if len(v) == 0:
            assert np.all(np.isnan(got[s]))
        else:
            assert np.array_equal(got[s], np.percentile(v, pct)), s
    one = _ops.percentiles_from_order_stats(counts, 50, kth)
    assert one.shape == (len(segs), 1)


@pytest.mark.parametrize("k", range(4))
def test_oracle_dense_pinned_to_reference(golden, k):
    z = golden("dense")
    hap, pos = z[f"hap{k}"], z[f"pos{k}"]
    assert np.array_equal(O.pairwise_ld_v(hap), z[f"ldv{k}"])
    assert np.array_equal(O.pairwise_r2(hap), z[f"r2_{k}"])
    res, cnt = O.windowed_r_squared(hap, pos, z[f"wbins{k}"], [5, 50, 95])
    assert np.array_equal(cnt, z[f"wcnt{k}"])
    want = z[f"wr2_{k}"]
    assert np.array_equal(np.isnan(res), np.isnan(want))
    m = ~np.isnan(want)
    np.testing.assert_allclose(res[m], want[m], rtol=1e-14)
