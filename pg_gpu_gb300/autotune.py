"""Per-sample-size choice of the tensor-core kernels' tile layout and pipeline
depth.

The reference sizes its work from free device memory
(ld_pipeline.estimate_ld_chunk_size, ld_pipeline.py:16-49; _memutil.py:6-52);
here the knobs are those of the tcgen05 band kernels, and the best setting
depends on the haplotypes per population (the K of every MMA), the kind of
call and the GPU:

* layout of the binned two-population form: 1 = tiles of 64 x 64 SNPs with
  one accumulator per population (M = N = 128 MMAs), 2 = tiles of 64 x 128
  SNPs with both populations in one accumulator (M = 128, N = 256 MMAs);
  of the one-population per-pair and window forms: 1 = 64 x 64 tiles with
  eight epilogue warps, 2 = 64 x 128 tiles with twelve;
* stages: pipeline stages of the TMA ring (0 = as many as shared memory
  holds).  A K chunk is one 128-byte swizzle row of the operand; it is not
  a knob.

``tune`` times every candidate on a synthetic panel of the caller's sample
sizes (the kernel alone, CUDA events on its stream, median of three launches)
and stores the fastest in ``tc_tuning.json`` beside the library, keyed by
(kind, words per population, GPU name, SM count).  ``apply`` sets a call's
configuration from that cache (the library's automatic choice when the key
is missing; with PGLD_AUTOTUNE=1 a missing key is tuned first).
"""
from __future__ import annotations

import json
import os
import threading

import numpy as np

from . import _lib as L

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tc_tuning.json")
_lock = threading.RLock()
_cache = None
_applied = {}

BINNED2_CANDIDATES = [(layout, stages) for layout in (2, 1) for stages in (0, 4, 3, 2)]
# per-pair outputs and window sums of one population: 64 x 128 (2) or 64 x 64 (1) tiles
ONE_POP_CANDIDATES = [(layout, stages) for layout in (2, 1) for stages in (0, 4, 3, 2)]
OTHER_CANDIDATES = [(0, stages) for stages in (0, 4, 3, 2)]


def _device_key():
    import torch
    dev = torch.cuda.current_device()
    p = torch.cuda.get_device_properties(dev)
    return f"{p.name}|{p.multi_processor_count}"


def key(kind, words):
    return f"{kind}|{','.join(str(int(w)) for w in words)}|{_device_key()}"


def _load():
    global _cache
    if _cache is None:
        with _lock:
            if _cache is None:
                try:
                    with open(CACHE) as f:
                        _cache = json.load(f)
                except (OSError, ValueError):
                    _cache = {}
    return _cache


def lookup(kind, words):
    """The cached (layout, stages) of a call, or None."""
    v = _load().get(key(kind, words))
    return None if v is None else (int(v["layout"]), int(v["stages"]))


def apply(kind, words):
    """Set the handle's tensor-core configuration for a call of `kind` on
    populations of `words` 32-haplotype words (tuning first when
    PGLD_AUTOTUNE=1 and nothing is cached)."""
    cfg = lookup(kind, words)
    if cfg is None and os.environ.get("PGLD_AUTOTUNE") == "1":
        cfg = tune(kind, words)["choice"]
    cfg = cfg or (0, 0)
    h = L.handle()
    if _applied.get(h) != cfg:
        L.check(L.lib().pgld_set_tc_config(h, int(cfg[0]), int(cfg[1])), h)
        _applied[h] = cfg
    return cfg


def _synthetic(words, n_snp, seed):
    """Device int8 panel of sum(32 w) haplotypes and sorted positions (one
    SNP per 100 bp on average): allele frequencies Beta(0.3, 0.3), 2 %
    missing."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    H = sum(32 * int(w) for w in words)
    p = torch.rand((n_snp,), generator=g, device="cuda") ** 2
    hap = (torch.rand((H, n_snp), generator=g, device="cuda") < p).to(torch.int8)
    hap[torch.rand((H, n_snp), generator=g, device="cuda") < 0.02] = -1
    rng = np.random.default_rng(seed)
    pos = np.sort(rng.choice(100 * n_snp, n_snp, replace=False)).astype(np.int64)
    return hap, pos


def _time_call(fn, reps=3):
    import ctypes
    h = L.handle()
    fn()
    L.check(L.lib().pgld_set_kernel_timing(h, 1), h)
    for _ in range(reps):
        fn()
    buf = (ctypes.c_float * 64)()
    n = ctypes.c_int32()
    L.check(L.lib().pgld_kernel_times(h, buf, 64, ctypes.byref(n)), h)
    L.check(L.lib().pgld_set_kernel_timing(h, 0), h)
    ms = sorted(buf[k] for k in range(min(n.value, 64)))
    return ms[len(ms) // 2] if ms else float("inf")


def tune(kind, words, n_snp=24_000, max_dist=1e6, save=True):
    """Time every candidate configuration of a `kind` call ("binned2",
    "binned1", "pairs", "windows") on populations of `words` words and cache
    the fastest.  Returns {"choice": (layout, stages), "ms": {...}}."""
    import torch
    from . import _ops
    words = [int(w) for w in words]
    hap, pos = _synthetic(words, n_snp, 20261207 + sum(words))
    pos_d = _ops.positions_f64(pos)
    rows, start = [], 0
    for w in words:
        rows.append(torch.arange(start, start + 32 * w, dtype=torch.int32, device="cuda"))
        start += 32 * w
    pops = [_ops.pack(hap, r) for r in rows]
    bins = np.logspace(3, np.log10(max_dist), 21)
    if kind in ("binned2", "binned1"):
        def call():
            _ops.binned_sums(pops, pos_d, bins, form="tc", _tuning=True)
        cands = BINNED2_CANDIDATES if kind == "binned2" else OTHER_CANDIDATES
    elif kind == "pairs":
        md = float(max_dist) / 10

        def call():
            _ops.band_pairs(pops[0], pos_d, md, form="tc", _tuning=True)
        cands = ONE_POP_CANDIDATES
    elif kind == "windows":
        sizes = np.full(max(1, n_snp // 2_000), 2_000)
        ends = np.cumsum(sizes)
        ends[-1] = n_snp
        begins = np.concatenate([[0], ends[:-1]])

        def call():
            _ops.window_sums(pops[0], None, begins, ends, form="tc", _tuning=True)
        cands = ONE_POP_CANDIDATES
    else:
        raise ValueError(f"unknown call kind {kind!r}")
    h = L.handle()
    ms = {}
    for layout, stages in cands:
        L.check(L.lib().pgld_set_tc_config(h, layout, stages), h)
        ms[f"{layout},{stages}"] = _time_call(call)
    best = min(ms, key=ms.get)
    choice = tuple(int(x) for x in best.split(","))
    _applied.pop(h, None)
    L.check(L.lib().pgld_set_tc_config(h, 0, 0), h)
    if save:
        with _lock:
            c = _load()
            c[key(kind, words)] = {"layout": choice[0], "stages": choice[1], "ms": ms}
            tmp = CACHE + ".tmp"
            with open(tmp, "w") as f:
                json.dump(c, f, indent=1, sort_keys=True)
            os.replace(tmp, CACHE)
    return {"choice": choice, "ms": ms, "key": key(kind, words)}
