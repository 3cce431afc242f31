"""The allocation-free binned-sum entry point against the regular one.

pgld_hap_binned_sums_noalloc serves callers that cannot call cudaMalloc (a
host that owns all device memory through its own pool, or a loop that cannot
take cudaMalloc's device-wide synchronisation).  It is called here through the
C ABI, twice in a row on the same inputs, and each result must match
pgld_hap_binned_sums within the binned-sum tolerance of the other GPU tests
(|a - b| <= 2e-6 * sum|x| per bin and statistic), with identical pair counts.
The first call in a fresh process performs the per-device set-up.
"""
import ctypes

import numpy as np
import pytest

from oracle import ld_oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA device", allow_module_level=True)

from pg_gpu_gb300 import _lib as L  # noqa: E402
from pg_gpu_gb300 import _ops  # noqa: E402

SUM_TOL = 2e-6


def _inputs():
    rng = np.random.default_rng(20261231)
    H, M = 160, 900
    p = rng.beta(0.4, 0.4, M)
    hap = (rng.random((H, M)) < p).astype(np.int8)
    hap[rng.random(hap.shape) < 0.02] = -1
    pos = np.sort(rng.choice(400_000, M, replace=False)).astype(np.int64)
    rows = [np.arange(0, 70), np.arange(70, 160)]
    bins = np.logspace(2.5, 5, 9)
    return hap, pos, rows, bins


def _noalloc_call(panel, pos_d, bins_d, n_bins, sums, cnt):
    dev = torch.cuda.current_device()
    rc = L.lib().pgld_hap_binned_sums_noalloc(dev, ctypes.byref(panel), L.ptr(pos_d),
                                              float(bins_d[-1].item()), None, L.ptr(bins_d),
                                              n_bins, L.ptr(sums), L.ptr(cnt), L.stream_ptr())
    if rc:
        raise L.PgldError(rc, L.lib().pgld_last_error(None).decode())


def test_noalloc_matches_regular_entry_point():
    hap, pos, rows, bins = _inputs()
    hap_d = torch.as_tensor(hap, device="cuda")
    pops = [_ops.pack(hap_d, r) for r in rows]
    pos_d = _ops.positions_f64(pos)
    ref_sums, ref_cnt = _ops.binned_sums(pops, pos_d, bins)
    ref_sums, ref_cnt = ref_sums.cpu().numpy(), ref_cnt.cpu().numpy()
    _, oracle_cnt, scale = O.binned_sums(hap, pos, rows, bins, abs_sums=True)
    assert np.array_equal(ref_cnt, oracle_cnt)

    panel = _ops.panel(pops)
    bins_d = torch.as_tensor(bins, device="cuda")
    n_bins = len(bins) - 1
    for _ in range(2):
        # caller-owned outputs, filled with garbage the call must overwrite
        sums = torch.full((n_bins, 15), 7.0, dtype=torch.float64, device="cuda")
        cnt = torch.full((n_bins,), 7, dtype=torch.int64, device="cuda")
        _noalloc_call(panel, pos_d, bins_d, n_bins, sums, cnt)
        torch.cuda.synchronize()
        got, got_cnt = sums.cpu().numpy(), cnt.cpu().numpy()
        assert np.array_equal(got_cnt, ref_cnt)
        assert np.all(np.abs(got - ref_sums) <= SUM_TOL * scale + 1e-300)


def test_noalloc_rejects_oversized_panels():
    pk = _ops.pack(np.zeros((32, 2), np.int8))
    panel = _ops.panel([pk])
    panel.n_snp = 20_000_000  # beyond the static scratch; rejected before any launch
    bins_d = torch.as_tensor([0.0, 10.0], dtype=torch.float64, device="cuda")
    pos_d = _ops.positions_f64([1.0, 2.0])
    sums = torch.zeros((1, 3), dtype=torch.float64, device="cuda")
    rc = L.lib().pgld_hap_binned_sums_noalloc(torch.cuda.current_device(), ctypes.byref(panel),
                                              L.ptr(pos_d), 10.0, None, L.ptr(bins_d), 1,
                                              L.ptr(sums), None, L.stream_ptr())
    assert rc == -3
    assert b"static scratch" in L.lib().pgld_last_error(None)
