"""Time the reference's own LD array code on the host cores (test
infrastructure: a measurement of the reference, never imported by the
library).

The reference (kr-colab/pg_gpu) is Python on CuPy; tests/golden/_ref_shim.py
runs its modules unmodified on NumPy (a numpy-backed stand-in for ``cupy``,
its RawKernel bodies compiled as host C++).  This script times that code path
-- the chain of moments_ld._compute_ld_sums (moments_ld.py:306-343):
iter_pairs_within_distance, compute_counts_for_pairs per population,
compute_two_pop_statistics_batch, digitize and np.add.at -- on

* the two-population binned workload (2 x 1,000 haplotypes sharing 40
  founders, 10 % founder alleles flipped per population, 2 % missing, one SNP
  per 100 bp, 20 log bins from 1 kb to 1 Mb): the pairs of a block of
  anchors, at least 1e7 pairs, on one core and on every core (one block per
  process);
* the small all-pairs workload (200 haplotypes x 2,000 SNPs over 1 Mb, 20
  founders, no missing data): counts, r^2, DD, Dz and pi2 of all 1,999,000
  pairs through ld_statistics, in full, on one core.

It needs the reference checkout (PGLD_REFERENCE or /root/reference) and runs
where that exists, not on the GPU host.  Usage:
    python oracle/time_reference_cpu.py [--pairs 10000000] [--procs N]
"""
import argparse
import json
import os
import sys
import time

os.environ.setdefault("OMP_NUM_THREADS", "1")
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def shared_founder_panel(seed, M, H=1000, F=40, length=None, switch=1e-3, pop_flip=0.10,
                         flip=1e-3, missing=0.02):
    rng = np.random.default_rng(seed)
    length = length or 100 * M
    pos = np.sort(rng.choice(length, M, replace=False)).astype(np.int64)
    p = rng.beta(0.3, 0.3, M)
    founders = (rng.random((F, M)) < p).astype(np.int8)
    pops = []
    for _ in range(2):
        fp = founders ^ (rng.random((F, M)) < pop_flip).astype(np.int8)
        seg = np.cumsum(rng.random((H, M)) < switch, axis=1)
        choice = rng.integers(0, F, size=(H, seg.max() + 1))
        hap = fp[np.take_along_axis(choice, seg, axis=1), np.arange(M)[None, :]]
        hap ^= (rng.random(hap.shape) < flip).astype(np.int8)
        hap[rng.random(hap.shape) < missing] = -1
        pops.append(hap)
    return np.concatenate(pops).astype(np.int8), pos


def binned_block(args):
    """The reference's binned-sum chain over the pairs anchored in [0, n_anchor)
    of a panel slice; returns (pairs, seconds)."""
    hap, pos, n_anchor, bins = args
    import _ref_shim as S
    M = S.load_reference_modules()
    lp, ls = M["ld_pipeline"], M["ld_statistics"]
    H = hap.shape[0] // 2
    rows = [list(range(H)), list(range(H, 2 * H))]
    n_bins = len(bins) - 1
    n_ld = len(lp.ld_names(2))
    sums = np.zeros((n_bins, n_ld))
    chunk = lp.estimate_ld_chunk_size(H, 16 << 30, num_pops=2)
    t0 = time.perf_counter()
    pairs = 0
    for ci, cj in lp.iter_pairs_within_distance(S.garr(pos), float(bins[-1]), chunk):
        ci, cj = np.asarray(ci), np.asarray(cj)
        keep = ci < n_anchor
        if not keep.any():
            break
        ci, cj = S.garr(ci[keep]), S.garr(cj[keep])
        pairs += len(ci)
        d = pos[np.asarray(cj)] - pos[np.asarray(ci)]
        cb = np.digitize(d, bins) - 1
        cl, nl = [], []
        for r in rows:
            c, nv = lp.compute_counts_for_pairs(S.garr(hap), ci, cj, r)
            cl.append(c)
            nl.append(nv)
        st = np.asarray(lp.compute_two_pop_statistics_batch(cl[0], cl[1], nl[0], nl[1], ls))
        ok = (cb >= 0) & (cb < n_bins)
        flat = cb[ok][:, None] * n_ld + np.arange(n_ld)[None, :]
        np.add.at(sums.ravel(), flat.ravel(), st[ok].ravel())
    return pairs, time.perf_counter() - t0


def all_pairs_small():
    """All 1,999,000 pairs of 200 haplotypes x 2,000 SNPs: counts, r^2, DD,
    Dz, pi2 through the reference's ld_pipeline / ld_statistics."""
    import _ref_shim as S
    M = S.load_reference_modules()
    lp, ls = M["ld_pipeline"], M["ld_statistics"]
    rng = np.random.default_rng(20261303)
    Hn, Mn, F = 200, 2000, 20
    p = rng.beta(0.3, 0.3, Mn)
    founders = (rng.random((F, Mn)) < p).astype(np.int8)
    seg = np.cumsum(rng.random((Hn, Mn)) < 1e-3, axis=1)
    choice = rng.integers(0, F, size=(Hn, seg.max() + 1))
    hap = founders[np.take_along_axis(choice, seg, axis=1), np.arange(Mn)[None, :]]
    hap ^= (rng.random(hap.shape) < 1e-3).astype(np.int8)
    ii, jj = np.triu_indices(Mn, k=1)
    t0 = time.perf_counter()
    c, nv = lp.compute_counts_for_pairs(S.garr(hap.astype(np.int8)), S.garr(ii.astype(np.int32)),
                                        S.garr(jj.astype(np.int32)))
    ls.r_squared(c, n_valid=nv)
    ls.dd(c, n_valid=nv)
    ls.dz(c, n_valid=nv)
    ls.pi2(c, n_valid=nv)
    return len(ii), time.perf_counter() - t0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=10_000_000)
    ap.add_argument("--procs", type=int, default=len(os.sched_getaffinity(0)))
    args = ap.parse_args()
    bins = np.logspace(3, 6, 21)
    out = {"host": os.uname().machine, "cores": len(os.sched_getaffinity(0))}
    try:
        import cpuinfo  # noqa: F401
        out["cpu"] = cpuinfo.get_cpu_info().get("brand_raw")
    except Exception:
        pass
    # one SNP per 100 bp: ~10,000 partners per anchor within 1 Mb
    n_anchor = max(1, args.pairs // 9_900)
    M = n_anchor + 11_000
    hap, pos = shared_founder_panel(20261503, M)
    pairs, sec = binned_block((hap, pos, n_anchor, bins))
    out["binned2pop_one_core"] = {"pairs": pairs, "seconds": sec, "pairs_per_s": pairs / sec}
    # every core: one anchor block per process (spawned)
    import multiprocessing as mp
    blocks = [(hap, pos, max(1, n_anchor // 4), bins) for _ in range(args.procs)]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(args.procs) as pool:
        res = pool.map(binned_block, blocks)
    wall = time.perf_counter() - t0
    tot = sum(r[0] for r in res)
    out["binned2pop_all_cores"] = {"procs": args.procs, "pairs": tot, "seconds": wall,
                                   "pairs_per_s": tot / wall}
    n, sec = all_pairs_small()
    out["all_pairs_200x2000_one_core"] = {"pairs": n, "seconds": sec, "pairs_per_s": n / sec}
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
