"""Benchmark of the two-locus LD hot path on GB300.

Workload (default): two populations of 1,000 haplotypes each x 200,000 SNPs
over 20 Mb, sharing a 40-founder pool (each population flips 10 % of founder
alleles; copying model with founder switches at rate 1e-3 per SNP, allele
flips 1e-3, 2 % entries missing), moments DD/Dz/pi2 (15 statistics) summed
into 20 log-spaced distance bins from 1 kb to 1 Mb over every pair within
1 Mb.  One step = pack both populations' bit planes from the resident int8
panel + one binned-sum launch.  Metric: SNP pairs per second.

  python bench.py [--gpus N --steps K --warmup W] [--form plain|tc]
  python bench.py --impl reference      # the reference path on host cores

Under torchrun (N > 1) every rank runs an independent replica (weak
scaling); rank 0 prints the max-over-ranks time.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LD SNP-pairs/s at 2k haps, int8-TC vs plain popcount; % INT8 TC peak; 1×GB300"

from pg_gpu_gb300 import synthetic  # noqa: E402

WORKLOADS = {
    # two-population binned moments statistics (the headline)
    "binned2pop": synthetic.BINNED2POP,
    # reduced size of the same workload, for profiling captures
    "binned2pop_small": synthetic.BINNED2POP_SMALL,
}


def rank_info():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    return r, w, lr


def make_panel(cfg, device):
    """int8 (2*H, M) panel on the device, sorted int64 positions (host)."""
    return synthetic.shared_founder_panel(cfg, device)


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        if self.proc is not None:
            # wait (up to 3 s) for the first sample, so that the sampler is
            # running when the timed region starts; that sample is not kept
            import select
            ready, _, _ = select.select([self.proc.stdout], [], [], 3.0)
            if ready:
                self.proc.stdout.readline()
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d, "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# --------------------------------------------------------------------------
# the tensor-pipe peak: tcgen05 E4M3 MMA throughput measured on this device
# --------------------------------------------------------------------------
_PEAK = {}


def tc_mma_peak(gpu_index, launch_ms=20.0, sustained_s=3.0):
    """E4M3 tcgen05.mma (M = 128, N = 128, K = 32) rate of this GPU, TFLOP/s:
    every SM issues MMAs back to back from operands resident in shared memory
    (pgld_tc_mma_rate), in launches of about launch_ms; "burst" = ten
    launches, "sustained" = sustained_s seconds of them, each with the SM
    clocks sampled while it ran.  Measured once per process."""
    if "burst" in _PEAK:
        return _PEAK
    import ctypes
    from pg_gpu_gb300 import _lib as L
    h = L.handle()
    ms, fl = ctypes.c_float(), ctypes.c_double()

    def run(n_cols, mmas, launches):
        L.check(L.lib().pgld_tc_mma_rate(h, n_cols, int(mmas), int(launches), ctypes.byref(ms),
                                         ctypes.byref(fl), L.stream_ptr()), h)
        return fl.value / (ms.value / 1e3) / 1e12, ms.value

    run(128, 1 << 16, 3)
    _, m = run(128, 1 << 18, 1)
    mmas = int(min(1 << 24, max(1 << 12, (1 << 18) * launch_ms / max(m, 1e-3))))
    run(128, mmas, 3)
    with ClockSampler(gpu_index) as c1:
        burst, bms = run(128, mmas, 10)
    with ClockSampler(gpu_index) as c2:
        sust, sms = run(128, mmas, max(10, int(sustained_s * 1e3 / launch_ms)))
    n256, _ = run(256, mmas // 2, 10)
    _PEAK.update({"burst": burst, "burst_clocks": c1.summary(), "sustained": sust,
                  "sustained_clocks": c2.summary(), "n256_burst": n256,
                  "mmas_per_sm_per_launch": mmas, "launch_ms": bms / 10})
    return _PEAK


def tc_roofline(pairs_per_s, ops_per_pair, basis, gpu_index=0, sm_mhz=None):
    """Tensor-pipe roofline of a tensor-core workload: ops_per_pair int8-
    equivalent operations per pair (the algorithmic contraction) per second,
    against the measured E4M3 tcgen05 burst rate of this GPU; basis names the
    timed region.  frac_clock_normalised divides each rate by the median SM
    clock it ran at."""
    pk = tc_mma_peak(gpu_index)
    peak = pk["burst"]
    achieved = pairs_per_s * ops_per_pair / 1e12
    out = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
           "frac": achieved / peak, "traffic": None, "ops_per_pair": ops_per_pair,
           "peak_source": "measured on this GPU: tcgen05 kind::f8f6f4 M128 N128 K32 from "
                          "shared memory on every SM (pgld_tc_mma_rate), burst of ten ~20 ms "
                          "launches",
           "peak_sm_mhz": pk["burst_clocks"].get("sm_mhz"),
           "peak_sustained": pk["sustained"],
           "peak_sustained_sm_mhz": pk["sustained_clocks"].get("sm_mhz"),
           "timed": basis}
    pm = pk["burst_clocks"].get("sm_mhz")
    if sm_mhz and pm:
        out["frac_clock_normalised"] = (achieved / sm_mhz) / (peak / pm)
    return out


def kernel_times(enable):
    """Turn per-launch timing of the library's dominant kernels on (and clear
    it) or read and clear the times (ms) timed since."""
    import ctypes
    from pg_gpu_gb300 import _lib as L
    h = L.handle()
    if enable:
        L.check(L.lib().pgld_set_kernel_timing(h, 1), h)
        return []
    buf = (ctypes.c_float * 4096)()
    n = ctypes.c_int32()
    L.check(L.lib().pgld_kernel_times(h, buf, 4096, ctypes.byref(n)), h)
    L.check(L.lib().pgld_set_kernel_timing(h, 0), h)
    return [float(buf[k]) for k in range(min(n.value, 4096))]


# --------------------------------------------------------------------------
# parity of the timed configuration: one anchor block against the oracle
# --------------------------------------------------------------------------
def _oracle_block(args):
    hap, pos, rows, bins, n_anchor = args
    from oracle import ld_oracle as O
    sums, cnt, asum = O.binned_sums(hap, pos, rows, bins, abs_sums=True, anchor_stop=n_anchor,
                                    pair_block=100_000)
    return sums, cnt, asum


def parity_block(pool, panel, pos, cfg, pops, pos_d, form, first, n_pairs):
    """The binned sums of the pairs anchored in one block of the panel (from
    SNP `first`, about n_pairs pairs), this library against the oracle: exact
    pair counts, and the largest error of every statistic relative to its bin
    value and to the bin's sum of |x|."""
    from pg_gpu_gb300 import _ops
    bins = cfg["bins"]
    md = float(bins[-1])
    a1, npairs = synthetic.anchors_per_pairs(pos, md, first, n_pairs)
    sums, cnt = _ops.binned_sums(pops, pos_d, bins, form=form, anchors=(first, a1))
    halo = int(np.searchsorted(pos, pos[a1 - 1] + md, side="right"))
    H = cfg["hap_per_pop"]
    rows = [np.arange(q * H, (q + 1) * H) for q in range(cfg["pops"])]
    args = (panel[:, first:halo].cpu().numpy(), pos[first:halo], rows, bins, a1 - first)
    ref, ref_cnt, ref_abs = pool.apply(_oracle_block, (args,)) if pool else _oracle_block(args)
    got = sums.cpu().numpy()
    err = np.abs(got - ref)
    nz = np.abs(ref) > 0
    rel = np.where(nz, err / np.where(nz, np.abs(ref), 1.0), 0.0)
    return {"anchors": [int(first), int(a1)], "pairs": int(npairs),
            "counts_equal": bool(np.array_equal(cnt.cpu().numpy(), ref_cnt)),
            "max_rel_err_of_value_by_stat": [float(x) for x in rel.max(axis=0)],
            "max_err_of_sum_abs": float((err / np.maximum(ref_abs, 1e-300)).max())}


def profile_traffic(form, workload):
    """dram bytes per launch of the dominant kernel from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    try:
        with open(path) as f:
            for line in f:
                parts = dict(kv.split("=", 1) for kv in line.split() if "=" in kv)
                if parts.get("form") == form and parts.get("workload") == workload:
                    return float(parts["traffic_bytes_per_launch"])
    except (OSError, ValueError, KeyError):
        pass
    return None


# --------------------------------------------------------------------------
# CPU baseline: the oracle (a restatement of the reference's NumPy path)
# --------------------------------------------------------------------------
def _cpu_worker(args):
    hap, pos, rows, bins, max_dist, a0, a1 = args
    from oracle import ld_oracle as O
    t = time.perf_counter()
    # the pairs of anchors a0..a1 (pair enumeration as ld_pipeline.py:85-121)
    jmax = np.searchsorted(pos, pos[a0:a1] + max_dist, side="right")
    per = np.maximum(0, jmax - np.arange(a0, a1) - 1)
    ii = np.repeat(np.arange(a0, a1), per)
    jj = ii + 1 + (np.arange(per.sum()) - np.repeat(np.cumsum(per) - per, per))
    n_sel = len(ii)
    d = (pos[jj] - pos[ii]).astype(np.float64)
    b = O.bin_index(d, bins)
    ok = (b >= 0) & (b < len(bins) - 1)
    ii, jj, b = ii[ok], jj[ok], b[ok]
    sums = np.zeros((len(bins) - 1, 15))
    for s0 in range(0, len(ii), 250_000):
        cs, nvs = [], []
        for r in rows:
            c, nv = O.counts_for_pairs(hap[r], ii[s0:s0 + 250_000], jj[s0:s0 + 250_000])
            cs.append(c)
            nvs.append(nv)
        st = O.multi_pop_stats(cs, nvs)
        for k in range(st.shape[1]):
            sums[:, k] += np.bincount(b[s0:s0 + 250_000], weights=st[:, k], minlength=len(bins) - 1)
    return int(n_sel), time.perf_counter() - t


def cpu_sample_inputs(panel, pos, cfg, n_workers, pairs_per_worker):
    """Contiguous sample: anchors 0..A split over workers, each with its window."""
    max_dist = float(cfg["bins"][-1])
    jmax = np.searchsorted(pos, pos + max_dist, side="right")
    per = np.maximum(0, jmax - np.arange(len(pos)) - 1)
    tasks = []
    a = 0
    H = cfg["hap_per_pop"]
    rows = [np.arange(q * H, (q + 1) * H) for q in range(cfg["pops"])]
    for _ in range(n_workers):
        cum = np.cumsum(per[a:])
        a1 = a + int(np.searchsorted(cum, pairs_per_worker)) + 1
        hi = int(jmax[a1 - 1])
        win = panel[:, a:hi].cpu().numpy()
        tasks.append((win, pos[a:hi], rows, cfg["bins"], max_dist, 0, a1 - a))
        a = a1
    return tasks


def run_cpu_baseline(pool, tasks, cores):
    t = time.perf_counter()
    res = pool.map(_cpu_worker, tasks)
    wall = time.perf_counter() - t
    pairs = sum(r[0] for r in res)
    return pairs / wall, pairs, wall


def make_pool(cores):
    import multiprocessing as mp
    return mp.get_context("spawn").Pool(cores)


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def run_gpu(args, pool, cores):
    import torch
    import torch.distributed as dist
    from pg_gpu_gb300 import _ops
    from pg_gpu_gb300.haplotype_matrix import HaplotypeMatrix

    rank, world, lrank = rank_info()
    torch.cuda.set_device(lrank)
    if world > 1:
        dist.init_process_group("nccl")
    cfg = WORKLOADS[args.workload]
    dev = torch.device("cuda", lrank)
    panel, pos = make_panel(cfg, dev)
    H = cfg["hap_per_pop"]
    rows = [torch.arange(q * H, (q + 1) * H, dtype=torch.int32, device=dev)
            for q in range(cfg["pops"])]
    bins = cfg["bins"]
    pos_d = _ops.positions_f64(pos)
    _, n_pairs = _ops.band_offsets(pos_d, float(bins[-1]))
    stream = torch.cuda.current_stream()
    # the tensor-core tile layout and pipeline depth for these sample sizes
    tuned = None
    if args.form == "tc" and not args.kernel_only:
        from pg_gpu_gb300 import autotune
        W = (H + 31) // 32
        tuned = autotune.tune("binned2" if cfg["pops"] == 2 else "binned1", [W] * cfg["pops"])
    flush = torch.empty(256 << 20, dtype=torch.int8, device=dev)

    def step():
        packs = [_ops.pack(panel, r) for r in rows]
        return _ops.binned_sums(packs, pos_d, bins, form=args.form)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # parity of the timed configuration (outside the timed region): the pairs
    # anchored in one block in the middle of the chromosome against the oracle
    parity = None
    if rank == 0 and not args.no_parity:
        packs = [_ops.pack(panel, r) for r in rows]
        parity = parity_block(pool, panel, pos, cfg, packs, pos_d, args.form,
                              len(pos) // 2, args.parity_pairs)
        del packs

    # ---- timed region: device-resident inputs ----
    def timed(form):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        for _ in range(args.warmup):
            packs = [_ops.pack(panel, r) for r in rows]
            _ops.binned_sums(packs, pos_d, bins, form=form)
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        kernel_times(True)
        with ClockSampler(lrank) as clk:
            for s in range(args.steps):
                flush.fill_(s & 0x7F)  # L2 flush between steps (outside the events)
                ev[s][0].record(stream)
                packs = [_ops.pack(panel, r) for r in rows]
                kev[s][0].record(stream)
                _ops.binned_sums(packs, pos_d, bins, form=form)
                kev[s][1].record(stream)
                ev[s][1].record(stream)
            torch.cuda.synchronize()
        step_ms = [a.elapsed_time(b) for a, b in ev]
        # the binned-sum call (operand expansion, work list, band kernel) and,
        # timed inside the library on the same stream, the band kernel alone
        call_ms = [a.elapsed_time(b) for a, b in kev]
        band_ms = kernel_times(False)
        kern_ms = (call_ms, band_ms)
        total = sum(step_ms) / 1e3
        if world > 1:
            t = torch.tensor([total], device=dev, dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            total = float(t.item())
        return world * n_pairs * args.steps / total, step_ms, kern_ms, clk

    value, step_ms, kern_ms, clk = timed(args.form)
    if args.kernel_only:
        # profiling runs: the timed steps only (no peak probe, comparison,
        # end-to-end leg or CPU baseline around the captured launches)
        if rank == 0:
            print(json.dumps({"workload": args.workload, "form": args.form, "value": value,
                              "unit": "pairs/s", "ms_per_step": float(np.mean(step_ms)),
                              "kernel_ms": float(np.mean(kern_ms[1] or kern_ms[0]))}), flush=True)
        return
    compare = None
    if not args.no_compare:
        other = "plain" if args.form == "tc" else "tc"
        v2, s2, k2, c2 = timed(other)
        compare = {"form": other, "value": v2, "unit": "pairs/s",
                   "ms_per_step": float(np.mean(s2)), "call_ms": float(np.mean(k2[0])),
                   "band_kernel_ms": float(np.mean(k2[1])) if k2[1] else None,
                   "clocks": c2.summary(), "ratio_this_over_other": value / v2}

    # ---- end to end through the public API, host buffers ----
    host = panel.cpu().pin_memory()
    sets = {f"pop{q}": list(range(q * H, (q + 1) * H)) for q in range(cfg["pops"])}
    e2e_ms = []
    for s in range(args.warmup + args.steps):
        flush.fill_(s & 0x7F)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hm = HaplotypeMatrix(host, pos, sample_sets=sets)
        out = hm.compute_ld_statistics_gpu_two_pops(bins, "pop0", "pop1", raw=True,
                                                    ac_filter=False)
        torch.cuda.synchronize()
        if s >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
        del hm
    e2e_s = sum(e2e_ms) / 1e3
    if world > 1:
        t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * n_pairs * args.steps / e2e_s
    h2d = host.numel() * host.element_size() + pos.nbytes
    d2h = (len(bins) - 1) * (15 + 1) * 8

    # ---- roofline of the band kernel (its launches timed on the call's stream) ----
    peaks, peak_src = measured_peaks()
    call_ms, band_ms = kern_ms
    k_s = float(np.mean(band_ms if band_ms else call_ms)) / 1e3
    W = (H + 31) // 32
    plane_bytes = cfg["n_snp"] * cfg["pops"] * 2 * W * 4
    traffic = profile_traffic(args.form, args.workload)
    basis = ("band kernel launches, CUDA events on the call's stream" if band_ms else
             "whole binned-sum call")
    if args.form == "plain":
        achieved = plane_bytes / k_s / 1e9
        peak = float(peaks.get("hbm_gbs", 6800.0))
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "peak_source": f"{peak_src} hbm_gbs", "timed": basis,
                "algorithmic_bytes_per_launch": plane_bytes,
                "note": "the plain form is bound by the integer (AND/POPC) pipe, not HBM; "
                        "int_ops_per_launch / time is reported as int_tops"}
        roof["int_tops"] = n_pairs * cfg["pops"] * 4 * W * 3 / k_s / 1e12
    else:
        ops_per_pair = 8 * H * cfg["pops"]
        roof = tc_roofline(n_pairs / k_s, ops_per_pair, basis, lrank, clk.summary().get("sm_mhz"))
        roof["traffic"] = traffic
        roof["algorithmic_ops_per_launch"] = n_pairs * ops_per_pair

    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(step_ms)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32" if args.form == "plain" else "e4m3",
        "data": "synthetic (seeded copying model, generated on device)",
        "config": {"workload": args.workload, "form": args.form, "pops": cfg["pops"],
                   "haplotypes_per_pop": H, "n_snp": cfg["n_snp"], "max_dist_bp": float(bins[-1]),
                   "bins": "20 log bins 1e3..1e6", "pairs_per_step": n_pairs,
                   "l2": "256 MB buffer written between steps; int8 panel 400 MB > L2",
                   "parallelism": f"replicas x{world}"},
        "clocks": clk.summary(),
        "e2e": {"value": e2e_value, "unit": "pairs/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "api": "HaplotypeMatrix(host int8).compute_ld_statistics_gpu_two_pops(raw=True)"},
        # per step: one pack per population, then the binned call: tile counts,
        # 3 scan launches and the band kernel; tc: also the integer-position
        # copy and the operand expansion -- one launch for both populations in
        # the combined 64 x 128 layout, one per population in the 64 x 64 one
        "gpu_launches": args.steps * (cfg["pops"] + 5 + (
            0 if args.form != "tc" else
            1 + (1 if (cfg["pops"] == 2 and (tuned is None or tuned["choice"][0] != 1))
                 else cfg["pops"]))),
        "call_ms": float(np.mean(call_ms)),
        "kernel_ms": k_s * 1e3,
        "roofline": roof,
        "parity": parity,
        "autotune": None if tuned is None else {
            "choice": {"layout": tuned["choice"][0], "stages": tuned["choice"][1]},
            "kernel_ms_by_layout_stages": tuned["ms"], "key": tuned["key"]},
        "compare": compare,
    }
    if pool is not None and rank == 0:
        tasks = cpu_sample_inputs(panel, pos, cfg, cores, args.cpu_pairs_per_worker)
        rate, pairs, wall = run_cpu_baseline(pool, tasks, cores)
        line["cpu_baseline"] = {"value": rate, "unit": "pairs/s", "cores": cores, "kind": "port",
                                "sample": f"first {pairs} pairs of the workload (anchors from "
                                          f"SNP 0), {cores} spawn workers, {wall:.1f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_reference(args, pool, cores):
    """The reference's CPU path (the oracle port) on every host core."""
    import torch
    rank, world, _ = rank_info()
    if rank != 0:
        return
    cfg = WORKLOADS[args.workload]
    dev = torch.device("cuda", 0) if torch.cuda.is_available() else None
    if dev is None:
        print(json.dumps({"impl": "reference", "unavailable": "needs the device panel generator"}))
        return
    panel, pos = make_panel(cfg, dev)
    tasks = cpu_sample_inputs(panel, pos, cfg, cores, args.cpu_pairs_per_worker)
    for _ in range(args.warmup):
        run_cpu_baseline(pool, tasks[:1], 1)
    rates, walls, pairs = [], [], 0
    for _ in range(args.steps):
        r, p, w = run_cpu_baseline(pool, tasks, cores)
        rates.append(r)
        walls.append(w)
        pairs = p
    value = float(np.sum([pairs] * len(walls)) / np.sum(walls))
    line = {"metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean(walls) * 1e3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "pops": cfg["pops"],
                       "haplotypes_per_pop": cfg["hap_per_pop"], "n_snp": cfg["n_snp"]},
            "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": cores, "kind": "port",
                             "sample": f"{pairs} pairs per step (contiguous from SNP 0)"},
            "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# secondary workloads (measurement of the other paths; not the headline line)
# --------------------------------------------------------------------------
def run_windows(args):
    """Batched uneven windows: 400 haplotypes, 512 windows of log-uniform
    500..20,000 SNPs (own seed each), every within-window pair; one launch over
    all windows against one launch per window."""
    import torch
    from pg_gpu_gb300 import _ops
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    rng = np.random.default_rng(20261504)
    sizes = np.exp(rng.uniform(np.log(500), np.log(20_000), 512)).astype(np.int64)
    sizes = sizes[:args.windows]  # a smaller case for profiler captures: the first windows
    torch.manual_seed(20261504)
    parts = []
    for w, m in enumerate(sizes):
        g = torch.Generator(device=dev)
        g.manual_seed(20261504 + w)
        parts.append(synthetic.copying_panel(g, 400, int(m), 20, 1e-3, 1e-3, 0.0, dev))
    panel = torch.cat(parts, 1).contiguous()
    del parts
    ends = np.cumsum(sizes)
    begins = ends - sizes
    n_pairs = int((sizes * (sizes - 1) // 2).sum())
    pk = _ops.pack(panel)
    wb = torch.as_tensor(begins, device=dev)
    we = torch.as_tensor(ends, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.int8, device=dev)

    def one():
        return _ops.window_sums(pk, None, wb, we, form="tc")

    def one_plain():
        return _ops.window_sums(pk, None, wb, we, form="plain")

    def per_window():
        for w in range(len(sizes)):
            _ops.window_sums(pk, None, wb[w:w + 1], we[w:w + 1], form="plain")

    def timeit(fn, steps):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ms = []
        for s in range(steps):
            flush.fill_(s & 0x7F)
            torch.cuda.synchronize()
            t = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ms.append((time.perf_counter() - t) * 1e3)
        return float(np.mean(ms))

    kernel_times(True)
    t_one = timeit(one, args.steps)
    k_one = kernel_times(False)
    k_ms = float(np.median(k_one[-args.steps:])) if k_one else t_one
    t_plain = timeit(one_plain, args.steps)
    t_per = timeit(per_window, max(1, args.steps // 2))
    sums, cnt = one()
    assert int(cnt[:, 0].sum()) == n_pairs
    s_pl, c_pl = one_plain()
    assert torch.equal(cnt, c_pl)
    print(json.dumps({
        "metric": f"within-window SNP-pairs/s, {len(sizes)} uneven windows, 400 haplotypes",
        "value": n_pairs / (t_one / 1e3), "unit": "pairs/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_one, "higher_is_better": True,
        "dtype": "e4m3", "data": "synthetic (copying model, seed per window)",
        "config": {"workload": "windows512", "haplotypes": 400, "windows": int(len(sizes)),
                   "n_snp": int(sizes.sum()), "pairs": n_pairs, "form": "tc"},
        "kernel_ms": k_ms,
        "roofline": tc_roofline(n_pairs / (k_ms / 1e3), 8 * 400,
                                "window kernel launches, CUDA events on the call's stream"),
        "plain_one_launch": {"ms_per_step": t_plain, "value": n_pairs / (t_plain / 1e3)},
        "plain_per_window_launches": {"ms_per_step": t_per, "value": n_pairs / (t_per / 1e3),
                                      "ratio_tc_one_launch_over_this": t_per / t_one}}),
          flush=True)


def run_geno_band(args):
    """Unphased genotype LD: 1,000 diploids x 500,000 SNPs over 50 Mb (dosage =
    sum of two copying-model haplotypes, 60 founders, switch 5e-4, 3 % missing);
    per-pair 9-way counts, Rogers-Huff r^2 and DD / Dz / pi2 for every pair
    within 200 kb."""
    import torch
    from pg_gpu_gb300 import _ops
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    g = torch.Generator(device=dev)
    g.manual_seed(20261505)
    M = args.geno_snps
    hap = synthetic.copying_panel(g, 2000, M, 60, 5e-4, 1e-3, 0.0, dev)
    geno = (hap[0::2] + hap[1::2]).to(torch.int8)
    del hap
    geno[torch.rand(geno.shape, generator=g, device=dev) < 0.03] = -1
    rng = np.random.default_rng(20261505)
    pos = np.sort(rng.choice(int(50_000_000 * M / 500_000), M, replace=False)).astype(np.int64)
    pos_d = _ops.positions_f64(pos)
    _, n_pairs = _ops.band_offsets(pos_d, 200_000)
    flush = torch.empty(256 << 20, dtype=torch.int8, device=dev)
    res = {}
    for form in ("tc", "plain"):
        def step():
            pk = _ops.pack_geno(geno)
            # the workload's outputs: genotype DD and Rogers-Huff r^2 per pair
            return _ops.geno_band_pairs(pk, pos_d, 200_000, with_counts=args.geno_counts,
                                        columns=("r2", "dd"), form=form)

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        ev = []
        for s_ in range(args.steps):
            flush.fill_(s_ & 0x7F)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            out = step()
            b.record()
            ev.append((a, b))
            del out
        torch.cuda.synchronize()
        res[form] = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    ms = res["tc"]
    print(json.dumps({
        "metric": "genotype LD SNP-pairs/s (n, Rogers-Huff r^2 and genotype DD per pair)",
        "value": n_pairs / (ms / 1e3), "unit": "pairs/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "dtype": "e4m3",
        "data": "synthetic (copying-model dosages, 3 % missing)",
        "config": {"workload": "geno_band", "individuals": 1000, "n_snp": M,
                   "max_dist_bp": 200_000, "pairs": n_pairs, "form": "tc",
                   "per_pair_bytes_written": (36 if args.geno_counts else 0) + 4 + 16},
        "roofline": tc_roofline(n_pairs / (ms / 1e3), 9 * 2 * 1000, "whole call, wall clock"),
        "compare": {"form": "plain", "ms_per_step": res["plain"],
                    "value": n_pairs / (res["plain"] / 1e3),
                    "ratio_tc_over_plain": res["plain"] / ms}}), flush=True)


def run_geno_binned(args):
    """Genotype moments LD in distance bins (moments_ld with use_genotypes):
    the 1,000 diploids x 500,000 SNPs over 50 Mb of the genotype band
    workload split into --geno-pops equal populations; the 3 / 15 / 45 / 105
    statistics of every pair within 200 kb summed in 12 log bins from 100 bp
    to 200 kb; the tensor-core form against the popcount form."""
    import torch
    from pg_gpu_gb300 import _ops
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    g = torch.Generator(device=dev)
    g.manual_seed(20261505)
    M = args.geno_snps
    hap = synthetic.copying_panel(g, 2000, M, 60, 5e-4, 1e-3, 0.0, dev)
    geno = (hap[0::2] + hap[1::2]).to(torch.int8)
    del hap
    geno[torch.rand(geno.shape, generator=g, device=dev) < 0.03] = -1
    rng = np.random.default_rng(20261505)
    pos = np.sort(rng.choice(int(50_000_000 * M / 500_000), M, replace=False)).astype(np.int64)
    pos_d = _ops.positions_f64(pos)
    P = args.geno_pops
    bins = np.logspace(2, np.log10(200_000), 13)
    _, n_pairs = _ops.band_offsets(pos_d, float(bins[-1]))
    per = 1000 // P
    rows = [torch.arange(q * per, (q + 1) * per, dtype=torch.int32, device=dev) for q in range(P)]
    flush = torch.empty(256 << 20, dtype=torch.int8, device=dev)
    res = {}
    for form in ("tc", "plain"):
        def step():
            pops = [_ops.pack_geno(geno, r) for r in rows]
            return _ops.geno_binned_sums(pops, pos_d, bins, form=form)

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        ev = []
        for s_ in range(args.steps):
            flush.fill_(s_ & 0x7F)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            out = step()
            b.record()
            ev.append((a, b))
            del out
        torch.cuda.synchronize()
        res[form] = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    ms = res["tc"]
    print(json.dumps({
        "metric": "genotype binned moments LD SNP-pairs/s",
        "value": n_pairs / (ms / 1e3), "unit": "pairs/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "dtype": "e4m3",
        "data": "synthetic (copying-model dosages, 3 % missing)",
        "config": {"workload": "geno_binned", "pops": P, "individuals_per_pop": per,
                   "n_snp": M, "max_dist_bp": 200_000, "bins": "12 log bins 1e2..2e5",
                   "pairs": n_pairs, "form": "tc"},
        "roofline": tc_roofline(n_pairs / (ms / 1e3), 9 * 2 * 1000, "whole call, wall clock"),
        "compare": {"form": "plain", "ms_per_step": res["plain"],
                    "value": n_pairs / (res["plain"] / 1e3),
                    "ratio_tc_over_plain": res["plain"] / ms}}), flush=True)


def run_hap_band(args):
    """Haplotype LD with missing data, per-pair outputs: 2,000 haplotypes x
    100,000 SNPs over 10 Mb (50 founders, switch 5e-4, 2 % missing), every pair
    within 100 kb: int32 counts, n and float32 r^2 / DD / Dz / pi2 per pair;
    the tensor-core form against the plain popcount form."""
    import torch
    from pg_gpu_gb300 import _ops
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    g = torch.Generator(device=dev)
    g.manual_seed(20261502)
    M = args.hap_snps
    hap = synthetic.copying_panel(g, 2000, M, 50, 5e-4, 1e-3, 0.02, dev)
    rng = np.random.default_rng(20261502)
    # 100 bp per SNP on average (10 Mb for the 100,000 SNPs of the workload)
    pos = np.sort(rng.choice(100 * M, M, replace=False)).astype(np.int64)
    pos_d = _ops.positions_f64(pos)
    _, n_pairs = _ops.band_offsets(pos_d, 100_000)
    flush = torch.empty(256 << 20, dtype=torch.int8, device=dev)
    res, kms = {}, {}
    for form in ("tc", "plain"):
        def step():
            pk = _ops.pack(hap)
            return _ops.band_pairs(pk, pos_d, 100_000, form=form)
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        ev = []
        kernel_times(True)
        for s_ in range(args.steps):
            flush.fill_(s_ & 0x7F)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            out = step()
            b.record()
            ev.append((a, b))
            del out
        torch.cuda.synchronize()
        kms[form] = kernel_times(False)
        res[form] = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    # the band kernel alone (library CUDA events on the call's stream): its
    # roofline is the HBM write of the 36 B of outputs per pair
    k_ms = float(np.median(kms["tc"])) if kms["tc"] else res["tc"]
    peaks, peak_src = measured_peaks()
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    out_bytes = 36 * n_pairs
    print(json.dumps({
        "metric": "haplotype LD SNP-pairs/s with per-pair outputs (counts, n, r^2, DD, Dz, pi2)",
        "value": n_pairs / (res["tc"] / 1e3), "unit": "pairs/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["tc"],
        "higher_is_better": True, "dtype": "e4m3",
        "data": "synthetic (copying model, 2 % missing)",
        "config": {"workload": "hap_band", "haplotypes": 2000, "n_snp": M,
                   "max_dist_bp": 100_000, "pairs": n_pairs, "per_pair_bytes_written": 36},
        "kernel_ms": k_ms,
        "roofline": {"bound": "hbm", "achieved": out_bytes / (k_ms / 1e3) / 1e9, "peak": hbm_peak,
                     "unit": "GB/s", "frac": out_bytes / (k_ms / 1e3) / 1e9 / hbm_peak,
                     "traffic": None, "algorithmic_bytes_per_launch": out_bytes,
                     "peak_source": f"{peak_src} hbm_gbs",
                     "timed": "band kernel launches, CUDA events on the call's stream"},
        "roofline_tensor": tc_roofline(n_pairs / (k_ms / 1e3), 8 * 2000,
                                       "band kernel launches, CUDA events on the call's stream"),
        "compare": {"form": "plain", "ms_per_step": res["plain"],
                    "value": n_pairs / (res["plain"] / 1e3),
                    "ratio_tc_over_plain": res["plain"] / res["tc"]}}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="tc", choices=["plain", "tc"])
    ap.add_argument("--no-compare", action="store_true", help="skip timing the other form")
    ap.add_argument("--workload", default="binned2pop",
                    choices=sorted(WORKLOADS) + ["windows512", "geno_band", "geno_binned",
                                                 "hap_band"])
    ap.add_argument("--geno-snps", type=int, default=500_000)
    ap.add_argument("--hap-snps", type=int, default=100_000,
                    help="hap_band: SNPs (same density; smaller cases for profiler captures)")
    ap.add_argument("--geno-pops", type=int, default=2, choices=[1, 2, 3, 4])
    ap.add_argument("--windows", type=int, default=512,
                    help="windows512: time the first N of the 512 windows (profiler captures)")
    ap.add_argument("--geno-counts", action="store_true", help="also write the 9-way counts")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-pairs-per-worker", type=int, default=400_000)
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle check of one block")
    ap.add_argument("--kernel-only", action="store_true",
                    help="time the steps only (for profiler captures); implies --no-cpu --no-parity")
    ap.add_argument("--parity-pairs", type=int, default=200_000)
    args = ap.parse_args()
    if args.kernel_only:
        args.no_cpu = args.no_parity = args.no_compare = True
    rank, world, _ = rank_info()
    cores = host_cores()
    # the oracle's process pool starts before the first GPU call (spawn)
    pool = None
    if args.workload in ("windows512", "geno_band", "geno_binned", "hap_band"):
        args.no_cpu = True
    if rank == 0 and (args.impl == "reference" or not args.no_cpu):
        pool = make_pool(cores)
    try:
        if args.impl == "reference":
            run_reference(args, pool, cores)
        elif args.workload == "windows512":
            run_windows(args)
        elif args.workload == "geno_band":
            run_geno_band(args)
        elif args.workload == "geno_binned":
            run_geno_binned(args)
        elif args.workload == "hap_band":
            run_hap_band(args)
        else:
            run_gpu(args, pool, cores)
    finally:
        if pool is not None:
            pool.close()
            pool.join()


if __name__ == "__main__":
    main()
