"""The allocation-free binned-sum entry point against the regular one.

pgld_hap_binned_sums_noalloc serves callers that cannot call cudaMalloc (a
host that owns all device memory through its own pool, or a loop that cannot
take cudaMalloc's device-wide synchronisation).  It is called here through the
C ABI, twice in a row on the same inputs, and each result must match
pgld_hap_binned_sums within the binned-sum tolerance of the other GPU tests
(1e-6 of each bin value, or of 5 % of the bin's sum of |x| where its terms
cancel), with identical pair counts and a clear device status word.  One and
two populations run the float32-epilogue kernel, three populations the
general term-table kernel.  The first call in a fresh process performs the
per-device set-up.
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

RTOL = 1e-6
FLOOR = 0.05


def _inputs(missing=0.02, n_pops=2):
    rng = np.random.default_rng(20261231)
    H, M = 160, 900
    p = rng.beta(0.4, 0.4, M)
    hap = (rng.random((H, M)) < p).astype(np.int8)
    if missing:
        hap[rng.random(hap.shape) < missing] = -1
    pos = np.sort(rng.choice(400_000, M, replace=False)).astype(np.int64)
    rows = ([np.arange(0, 70), np.arange(70, 160)][:n_pops] if n_pops <= 2 else
            [np.arange(0, 50), np.arange(50, 110), np.arange(110, 160)])
    bins = np.logspace(2.5, 5, 9)
    return hap, pos, rows, bins


def _status():
    code = ctypes.c_int32(-1)
    assert L.lib().pgld_noalloc_status(torch.cuda.current_device(), ctypes.byref(code)) == 0
    return code.value


def _noalloc_call(panel, pos_d, bins_d, n_bins, sums, cnt):
    dev = torch.cuda.current_device()
    rc = L.lib().pgld_hap_binned_sums_noalloc(dev, ctypes.byref(panel), L.ptr(pos_d),
                                              float(bins_d[-1].item()), None, L.ptr(bins_d),
                                              n_bins, L.ptr(sums), L.ptr(cnt), L.stream_ptr())
    if rc:
        raise L.PgldError(rc, L.lib().pgld_last_error(None).decode())


@pytest.mark.parametrize("missing,n_pops", [(0.02, 2), (0.0, 2), (0.02, 1), (0.02, 3)])
def test_noalloc_matches_regular_entry_point(missing, n_pops):
    hap, pos, rows, bins = _inputs(missing, n_pops)
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
    S = {1: 3, 2: 15, 3: 45}[n_pops]
    for _ in range(2):
        # caller-owned outputs, filled with garbage the call must overwrite
        sums = torch.full((n_bins, S), 7.0, dtype=torch.float64, device="cuda")
        cnt = torch.full((n_bins,), 7, dtype=torch.int64, device="cuda")
        _noalloc_call(panel, pos_d, bins_d, n_bins, sums, cnt)
        torch.cuda.synchronize()
        got, got_cnt = sums.cpu().numpy(), cnt.cpu().numpy()
        assert np.array_equal(got_cnt, ref_cnt)
        assert O.bin_errors(got, ref_sums, scale, FLOOR).max() <= RTOL
        assert _status() == 0


def test_noalloc_single_snp_gives_zeros():
    # fewer than two SNPs: no pair, zeroed sums and counts, nothing launched
    pk = _ops.pack(np.zeros((32, 1), np.int8))
    panel = _ops.panel([pk])
    bins_d = torch.as_tensor([0.0, 10.0, 20.0], dtype=torch.float64, device="cuda")
    pos_d = _ops.positions_f64([1.0])
    sums = torch.full((2, 3), 5.0, dtype=torch.float64, device="cuda")
    cnt = torch.full((2,), 5, dtype=torch.int64, device="cuda")
    _noalloc_call(panel, pos_d, bins_d, 2, sums, cnt)
    torch.cuda.synchronize()
    assert np.all(sums.cpu().numpy() == 0.0) and np.all(cnt.cpu().numpy() == 0)
    assert _status() == 0


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
