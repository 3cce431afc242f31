"""Generate the golden fixtures in this folder from the reference pg_gpu.

Run here, where the reference checkout exists:

    python tests/golden/make_golden.py        # PGLD_REFERENCE=<checkout> to override

Every expected value is produced by the reference's own code (through the
numpy stand-in for CuPy in ``_ref_shim.py``; RawKernel bodies compiled as
host C++), or read from data the reference ships:

* ``hap_counts.npz``  -- ld_pipeline.iter_pairs_within_distance chunks and
  compute_counts_for_pairs on a seeded matrix with missing data and
  population subsets (ld_pipeline.py:57-175).
* ``hap_stats.npz``   -- ld_statistics.dd/dz/pi2 for every population tuple
  of a 4-population count table, compute_multi_pop_statistics_batch_hap for
  1..4 populations, compute_two_pop_statistics_batch,
  compute_single_pop_statistics_batch and r / r_squared / d_prime.
* ``binned.npz``      -- the binned-sum loop of moments_ld._compute_ld_sums
  (moments_ld.py:306-343) driven by the reference's own pair iterator,
  counter and statistics, for 1 and 2 populations.
* ``moments_im.npz``  -- the haplotypes of examples/data/im-parsing-example.vcf
  (parsed as text, from_vcf layout haplotype_matrix.py:324-328), the deme
  rows of im_pop.txt, and the moments binned sums cached by the reference in
  tests/cache/moments_ld_test_im_4bins_deme0-deme1.pkl (read with a
  restricted unpickler that only accepts numpy array reconstruction).
* ``mu_ld.npz``       -- ld_statistics.mu_ld (ld_statistics.py:865-918) with
  the reference's haplotype clustering (diversity.py:1310-1360).
* ``geno.npz``        -- 9-way genotype counts from the reference counting
  kernel (ld_pipeline.py:183-217), single-population genotype DD from
  _DD_GENO_SINGLE_KERN (genotype_kernels.py:27-71), sigma_D^2 from
  _SIGMA_D2_GENO_KERN (genotype_kernels.py:91-169) and Rogers-Huff r from
  ld_statistics._tile_rogers_huff_r (ld_statistics.py:410-443).
"""
import io
import itertools
import os
import pickle
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import _ref_shim as S  # noqa: E402


def copying_model(rng, n_hap, n_snp, n_founders, switch, flip=1e-3, missing=0.0):
    p = rng.beta(0.3, 0.3, size=n_snp)
    founders = (rng.random((n_founders, n_snp)) < p).astype(np.int8)
    out = np.empty((n_hap, n_snp), np.int8)
    for h in range(n_hap):
        f = rng.integers(n_founders)
        sw = rng.random(n_snp) < switch
        seg = np.cumsum(sw)
        choice = rng.integers(0, n_founders, size=seg[-1] + 1)
        choice[0] = f
        out[h] = founders[choice[seg], np.arange(n_snp)]
    out ^= (rng.random(out.shape) < flip).astype(np.int8)
    if missing > 0:
        out[rng.random(out.shape) < missing] = -1
    return out


def gen_hap_counts(M):
    lp = M["ld_pipeline"]
    rng = np.random.default_rng(20261203)
    hap = copying_model(rng, 70, 120, 8, 0.05, missing=0.04)
    pos = np.sort(rng.choice(60_000, 120, replace=False)).astype(np.int64)
    max_dist = 9_000.0
    chunks = list(lp.iter_pairs_within_distance(S.garr(pos), max_dist, 97))
    ci = np.concatenate([np.asarray(c[0]) for c in chunks])
    cj = np.concatenate([np.asarray(c[1]) for c in chunks])
    chunk_len = np.array([len(c[0]) for c in chunks])
    rows_a = np.arange(0, 33)
    rows_b = np.arange(33, 70)[::2]
    out = dict(hap=hap, pos=pos, max_dist=max_dist, chunk_size=97, idx_i=ci, idx_j=cj,
               chunk_len=chunk_len, rows_a=rows_a, rows_b=rows_b)
    for tag, rows in (("all", None), ("a", rows_a), ("b", rows_b)):
        c, nv = lp.compute_counts_for_pairs(S.garr(hap), S.garr(ci), S.garr(cj),
                                            None if rows is None else list(rows))
        out[f"counts_{tag}"] = np.asarray(c)
        out[f"nvalid_{tag}"] = np.asarray(nv)
    # no-missing matrix: n_valid must come back as None
    hap0 = np.where(hap < 0, 0, hap).astype(np.int8)
    c0, nv0 = lp.compute_counts_for_pairs(S.garr(hap0), S.garr(ci), S.garr(cj))
    assert nv0 is None
    out["hap_nomiss"] = hap0
    out["counts_nomiss"] = np.asarray(c0)
    # pair chunking for other chunk sizes / distances
    for cs, md in ((1, 2000.0), (10_000, 60_000.0), (50, 0.0)):
        ch = list(lp.iter_pairs_within_distance(S.garr(pos), md, cs))
        out[f"chunks_{cs}_{int(md)}_len"] = np.array([len(c[0]) for c in ch], np.int64)
        if ch:
            out[f"chunks_{cs}_{int(md)}_i"] = np.concatenate([np.asarray(c[0]) for c in ch])
            out[f"chunks_{cs}_{int(md)}_j"] = np.concatenate([np.asarray(c[1]) for c in ch])
        else:
            out[f"chunks_{cs}_{int(md)}_i"] = np.zeros(0, np.int32)
            out[f"chunks_{cs}_{int(md)}_j"] = np.zeros(0, np.int32)
    np.savez_compressed(os.path.join(HERE, "hap_counts.npz"), **out)


def gen_hap_stats(M):
    lp, ls, hk = M["ld_pipeline"], M["ld_statistics"], M["haplotype_kernels"]
    rng = np.random.default_rng(20261204)
    N, P = 150, 4
    counts = rng.integers(0, 24, size=(N, 4 * P)).astype(np.int32)
    counts[:7, :4] = [[0, 0, 5, 5], [5, 5, 0, 0], [3, 0, 0, 3], [0, 4, 4, 0],
                      [1, 0, 0, 1], [2, 0, 1, 0], [0, 0, 0, 0]]
    nv = np.stack([counts[:, 4 * p:4 * p + 4].sum(1) + rng.integers(0, 3, N)
                   for p in range(P)], 1).astype(np.int32)
    out = dict(counts=counts, nvalid=nv)
    for pp in itertools.product(range(P), repeat=2):
        out["dd_" + "".join(map(str, pp))] = np.asarray(ls.dd(S.garr(counts), pp, S.garr(nv)))
    for pp in itertools.product(range(P), repeat=3):
        out["dz_" + "".join(map(str, pp))] = np.asarray(ls.dz(S.garr(counts), pp, S.garr(nv)))
    for pp in itertools.product(range(P), repeat=4):
        out["pi2_" + "".join(map(str, pp))] = np.asarray(ls.pi2(S.garr(counts), pp, S.garr(nv)))
    c4 = counts[:, :4]
    out["dd_single_nonv"] = np.asarray(ls.dd(S.garr(c4)))
    out["dz_single_nonv"] = np.asarray(ls.dz(S.garr(c4)))
    out["pi2_single_nonv"] = np.asarray(ls.pi2(S.garr(c4)))
    for f in ("r", "r_squared", "d_prime"):
        out[f + "_nv"] = np.asarray(getattr(ls, f)(S.garr(c4), S.garr(nv[:, 0])))
        out[f + "_nonv"] = np.asarray(getattr(ls, f)(S.garr(c4)))
    for p in range(1, P + 1):
        cs = [S.garr(counts[:, 4 * q:4 * q + 4]) for q in range(p)]
        nvs = [S.garr(nv[:, q]) for q in range(p)]
        out[f"multi_{p}"] = np.asarray(hk.compute_multi_pop_statistics_batch_hap(
            cs, nvs, ls, lp.generate_stat_specs(p)))
        out[f"multi_{p}_nonv"] = np.asarray(hk.compute_multi_pop_statistics_batch_hap(
            cs, [None] * p, ls, lp.generate_stat_specs(p)))
    out["two_pop"] = np.asarray(lp.compute_two_pop_statistics_batch(
        S.garr(counts[:, :4]), S.garr(counts[:, 4:8]), S.garr(nv[:, 0]), S.garr(nv[:, 1]), ls))
    out["two_pop_nonv"] = np.asarray(lp.compute_two_pop_statistics_batch(
        S.garr(counts[:, :4]), S.garr(counts[:, 4:8]), None, None, ls))
    out["single_pop"] = np.asarray(lp.compute_single_pop_statistics_batch(
        S.garr(c4), S.garr(nv[:, 0]), ls))
    np.savez_compressed(os.path.join(HERE, "hap_stats.npz"), **out)
    names = {p: lp.ld_names(p) for p in range(1, 5)}
    with open(os.path.join(HERE, "ld_names.txt"), "w") as f:
        for p in range(1, 5):
            f.write(f"{p} " + " ".join(names[p]) + "\n")
            f.write(f"H{p} " + " ".join(lp.het_names(p)) + "\n")


def ref_binned_sums(M, hap, pos, pop_rows, bins, chunk):
    """moments_ld._compute_ld_sums (moments_ld.py:306-343), haplotype mode."""
    lp, ls, hk = M["ld_pipeline"], M["ld_statistics"], M["haplotype_kernels"]
    n_bins = len(bins) - 1
    P = len(pop_rows)
    n_ld = len(lp.ld_names(P))
    sums = np.zeros((n_bins, n_ld))
    specs = lp.generate_stat_specs(P) if P != 2 else None
    for ci, cj in lp.iter_pairs_within_distance(S.garr(pos), float(bins[-1]), chunk):
        d = pos[np.asarray(cj)] - pos[np.asarray(ci)]
        cb = np.digitize(d, bins) - 1
        cl, nl = [], []
        for rows in pop_rows:
            c, nv = lp.compute_counts_for_pairs(S.garr(hap), ci, cj, list(rows))
            cl.append(c)
            nl.append(nv)
        if P == 2:
            st = lp.compute_two_pop_statistics_batch(cl[0], cl[1], nl[0], nl[1], ls)
        else:
            st = hk.compute_multi_pop_statistics_batch_hap(cl, nl, ls, specs)
        st = np.asarray(st)
        ok = (cb >= 0) & (cb < n_bins)
        flat = cb[ok][:, None] * n_ld + np.arange(n_ld)[None, :]
        np.add.at(sums.ravel(), flat.ravel(), st[ok].ravel())
    return sums


def gen_binned(M):
    rng = np.random.default_rng(20261205)
    hap = copying_model(rng, 48, 400, 10, 0.01, missing=0.02)
    pos = np.sort(rng.choice(200_000, 400, replace=False)).astype(np.int64)
    bins = np.logspace(2, np.log10(50_000), 9)
    pops = [np.arange(0, 24), np.arange(24, 48)]
    out = dict(hap=hap, pos=pos, bins=bins, rows0=pops[0], rows1=pops[1])
    out["sums_2pop"] = ref_binned_sums(M, hap, pos, pops, bins, 5000)
    out["sums_1pop"] = ref_binned_sums(M, hap, pos, pops[:1], bins, 5000)
    out["sums_3pop"] = ref_binned_sums(M, hap, pos, [np.arange(0, 16), np.arange(16, 32),
                                                     np.arange(32, 48)], bins, 5000)
    np.savez_compressed(os.path.join(HERE, "binned.npz"), **out)


class _NumpyOnly(pickle.Unpickler):
    _OK = {("numpy.core.multiarray", "scalar"), ("numpy.core.multiarray", "_reconstruct"),
           ("numpy", "dtype"), ("numpy", "ndarray")}

    def find_class(self, module, name):
        if (module, name) not in self._OK:
            raise pickle.UnpicklingError(f"refusing {module}.{name}")
        if module == "numpy.core.multiarray":
            import numpy._core.multiarray as mm
            return getattr(mm, name)
        return getattr(np, name)


def parse_vcf_haplotypes(path):
    samples, gts, pos = None, [], []
    with open(path) as f:
        for line in f:
            if line.startswith("##"):
                continue
            parts = line.rstrip("\n").split("\t")
            if line.startswith("#CHROM"):
                samples = parts[9:]
                continue
            pos.append(int(parts[1]))
            row = []
            for g in parts[9:]:
                a, b = g.split(":")[0].replace("/", "|").split("|")
                row.append((-1 if a == "." else int(a), -1 if b == "." else int(b)))
            gts.append(row)
    gt = np.array(gts, np.int8)  # (M, n, 2)
    n = gt.shape[1]
    hap = np.empty((gt.shape[0], 2 * n), np.int8)
    hap[:, :n] = gt[:, :, 0]
    hap[:, n:] = gt[:, :, 1]
    return hap.T.copy(), np.array(pos, np.int64), samples


def gen_moments(M):
    ref = S.REF_ROOT
    hap, pos, samples = parse_vcf_haplotypes(os.path.join(ref, "examples/data/im-parsing-example.vcf"))
    assign = {}
    with open(os.path.join(ref, "examples/data/im_pop.txt")) as f:
        next(f)
        for line in f:
            s, p = line.split()
            assign[s] = p
    n = len(samples)
    rows = {"deme0": [], "deme1": []}
    for i, s in enumerate(samples):
        if assign.get(s) in rows:
            rows[assign[s]] += [i, i + n]
    with open(os.path.join(ref, "tests/cache/moments_ld_test_im_4bins_deme0-deme1.pkl"), "rb") as f:
        res = _NumpyOnly(io.BytesIO(f.read())).load()
    bins = np.array([res["bins"][0][0]] + [b[1] for b in res["bins"]], np.float64)
    ld = np.stack([np.asarray(s, np.float64) for s in res["sums"][:-1]])
    het = np.asarray(res["sums"][-1], np.float64)
    names = np.array(res["stats"][0])
    hnames = np.array(res["stats"][1])
    np.savez_compressed(os.path.join(HERE, "moments_im.npz"), hap=hap, pos=pos,
                        rows0=np.array(rows["deme0"]), rows1=np.array(rows["deme1"]),
                        bins=bins, ld_sums=ld, het_sums=het, ld_names=names, het_names=hnames)


def gen_geno(M):
    lp, ls, gk = M["ld_pipeline"], M["ld_statistics"], M["genotype_kernels"]
    rng = np.random.default_rng(20261206)
    h = copying_model(rng, 80, 150, 8, 0.03)
    g = (h[0::2] + h[1::2]).astype(np.int8)  # 40 diploids
    gm = g.copy()
    gm[rng.random(g.shape) < 0.04] = -1
    pos = np.sort(rng.choice(80_000, 150, replace=False)).astype(np.int64)
    ci, cj = [np.concatenate(x) for x in zip(*[(np.asarray(a), np.asarray(b)) for a, b in
                                               lp.iter_pairs_within_distance(S.garr(pos), 15_000, 10**6)])]
    out = dict(geno=g, geno_miss=gm, pos=pos, idx_i=ci, idx_j=cj)
    c, nv = lp.compute_genotype_counts_for_pairs(S.garr(gm), S.garr(ci), S.garr(cj))
    out["counts9_miss"], out["nvalid_miss"] = np.asarray(c), np.asarray(nv)
    c0, nv0 = lp.compute_genotype_counts_for_pairs(S.garr(g), S.garr(ci), S.garr(cj))
    assert nv0 is None
    out["counts9"] = np.asarray(c0)
    # dosages above 2 (multi-allelic codes summed): the kernel folds 3 g_i + g_j
    godd = gm.copy()
    mask = rng.random(g.shape) < 0.05
    godd[mask] = rng.integers(3, 10, size=int(mask.sum()))
    co, nvo = lp.compute_genotype_counts_for_pairs(S.garr(godd), S.garr(ci), S.garr(cj))
    out["geno_odd"], out["counts9_odd"], out["nvalid_odd"] = godd, np.asarray(co), np.asarray(nvo)
    rows = np.arange(5, 37, 2)
    cr, _ = lp.compute_genotype_counts_for_pairs(S.garr(gm), S.garr(ci), S.garr(cj), list(rows))
    out["rows"], out["counts9_rows"] = rows, np.asarray(cr)
    for tag, cc in (("", np.asarray(c0)), ("_miss", np.asarray(c))):
        rev = np.ascontiguousarray(cc[:, ::-1].astype(np.float64))
        o = np.empty(len(rev))
        gk._DD_GENO_SINGLE_KERN(((len(rev) + 255) // 256,), (256,), (rev, o, len(rev)))
        out["dd_geno" + tag] = o
        o2 = np.empty(len(rev))
        gk._SIGMA_D2_GENO_KERN(((len(rev) + 255) // 256,), (256,), (rev, o2, len(rev)))
        out["sigma_d2" + tag] = o2
    gf = g.astype(np.float64)
    mu = gf.mean(axis=0)
    ssd = ((gf - mu) ** 2).sum(axis=0)
    rfull = np.asarray(ls._tile_rogers_huff_r(S.garr(gf), S.garr(gf), S.garr(mu), S.garr(mu),
                                              S.garr(ssd), S.garr(ssd), gf.shape[0]))
    out["rh_r_pairs"] = rfull[ci, cj]
    iu = np.triu_indices(g.shape[1], k=1)
    out["rh_r_condensed"] = rfull[iu]
    np.savez_compressed(os.path.join(HERE, "geno.npz"), **out)


def gen_geno_stats(M):
    """Genotype moments statistics of 1-4 populations from the reference's
    compute_multi_pop_statistics_batch_geno (genotype_kernels.py:889-936)."""
    lp, gk = M["ld_pipeline"], M["genotype_kernels"]
    rng = np.random.default_rng(20261207)
    sizes = (14, 9, 22, 6)
    N = 240
    out = {}
    cs, nvs = [], []
    for q, n_ind in enumerate(sizes):
        # random 9-way tables with a few edge rows (tiny and monomorphic samples)
        n = rng.integers(4, n_ind + 1, size=N)
        c = np.stack([rng.multinomial(k, rng.dirichlet([0.4] * 9)) for k in n]).astype(np.int32)
        c[:4] = [[0] * 9, [1, 0, 0, 0, 1, 0, 0, 0, 1], [0, 0, 0, 0, 5, 0, 0, 0, 0],
                 [2, 0, 0, 0, 0, 0, 0, 0, 2]]
        cs.append(c)
        nvs.append(c.sum(1).astype(np.int32))
        out[f"counts_{q}"] = c
    for p in range(1, 5):
        specs = lp.generate_stat_specs(p)
        out[f"multi_{p}"] = np.asarray(gk.compute_multi_pop_statistics_batch_geno(
            [S.garr(cs[q]) for q in range(p)], [S.garr(nvs[q]) for q in range(p)], None, specs))
        out[f"multi_{p}_nonv"] = np.asarray(gk.compute_multi_pop_statistics_batch_geno(
            [S.garr(cs[q]) for q in range(p)], [None] * p, None, specs))
    np.savez_compressed(os.path.join(HERE, "geno_stats.npz"), **out)


def gen_geno_binned(M):
    """Genotype-mode binned sums: the loop of moments_ld._compute_ld_sums
    (moments_ld.py:248-343, use_genotypes=True) driven through the reference's
    own iter_pairs_within_distance, compute_genotype_counts_for_pairs and
    compute_multi_pop_statistics_batch_geno, with 2 and 3 populations."""
    lp, gk = M["ld_pipeline"], M["genotype_kernels"]
    rng = np.random.default_rng(20261208)
    h = copying_model(rng, 96, 360, 10, 0.02, missing=0.0)
    g = (h[0::2] + h[1::2]).astype(np.int8)  # 48 diploids
    g[rng.random(g.shape) < 0.03] = -1
    pos = np.sort(rng.choice(400_000, 360, replace=False)).astype(np.int64)
    bins = np.array([0.0, 2e3, 5e3, 1e4, 2.5e4, 5e4, 1e5], np.float64)
    rows = [np.arange(0, 16), np.arange(16, 34), np.arange(34, 48)]
    out = dict(geno=g, pos=pos, bins=bins, rows0=rows[0], rows1=rows[1], rows2=rows[2])
    for P in (2, 3):
        sel = sorted(set(int(i) for r in rows[:P] for i in r))
        sub = g[sel].astype(np.int64)
        v = sub >= 0
        alt = np.where(v, sub, 0).sum(0)
        nv = v.sum(0)
        keep = np.where((alt > 0) & (alt < 2 * nv) & (nv >= 2))[0]
        gk_ = g[:, keep]
        pk = pos[keep].astype(np.float64)
        specs = lp.generate_stat_specs(P)
        sums = np.zeros((len(bins) - 1, len(specs)))
        for ci, cj in lp.iter_pairs_within_distance(S.garr(pk), float(bins[-1]), 10_000):
            ci, cj = np.asarray(ci), np.asarray(cj)
            cb = np.digitize(pk[cj] - pk[ci], bins) - 1
            cs, nvs = [], []
            for r in rows[:P]:
                c, nvv = lp.compute_genotype_counts_for_pairs(S.garr(gk_), S.garr(ci), S.garr(cj),
                                                              list(r))
                cs.append(c)
                nvs.append(nvv)
            st = np.asarray(gk.compute_multi_pop_statistics_batch_geno(cs, nvs, None, specs))
            ok = (cb >= 0) & (cb < len(bins) - 1)
            np.add.at(sums, (cb[ok][:, None], np.arange(len(specs))[None, :]), st[ok])
        out[f"keep_{P}"] = keep
        out[f"sums_{P}"] = sums
    np.savez_compressed(os.path.join(HERE, "geno_binned.npz"), **out)


def gen_windows(M):
    """Per-window ZnS from the reference's _zns_from_precomputed
    (ld_statistics.py:595-676), projection (sigma_D^2) and naive r^2."""
    ls = M["ld_statistics"]
    rng = np.random.default_rng(20261209)
    hap = copying_model(rng, 60, 700, 8, 0.01, missing=0.03)
    bounds = np.array([0, 3, 40, 41, 130, 300, 301, 520, 700])
    hc = np.where(hap >= 0, hap, 0).astype(np.float64)
    vm = (hap >= 0).astype(np.float64)
    zp, zn = [], []
    for s, e in zip(bounds[:-1], bounds[1:]):
        zp.append(ls._zns_from_precomputed(S.garr(hc), S.garr(vm), int(s), int(e), tile_size=64,
                                            use_projection=True))
        zn.append(ls._zns_from_precomputed(S.garr(hc), S.garr(vm), int(s), int(e), tile_size=64,
                                            use_projection=False))
    np.savez_compressed(os.path.join(HERE, "windows.npz"), hap=hap, bounds=bounds,
                        zns_proj=np.array(zp, np.float64), zns_naive=np.array(zn, np.float64))


def gen_omega(M):
    """Kim and Nielsen's omega from the reference (ld_statistics.omega,
    ld_statistics.py:761-862) on HaplotypeMatrix inputs: the default sigma_D^2
    estimator, naive r^2, missing_data 'exclude'; and on a precomputed r^2
    matrix (the reference's own pairwise_r2)."""
    ls = M["ld_statistics"]
    HM = S.load_haplotype_matrix()
    out = {}
    for k, (H, m, F, sw, miss) in enumerate([(40, 100, 6, 0.02, 0.0), (64, 180, 8, 0.01, 0.03),
                                             (30, 60, 4, 0.05, 0.05)]):
        rng = np.random.default_rng(20261210 + k)
        hap = copying_model(rng, H, m, F, sw, missing=miss)
        pos = np.arange(m, dtype=np.int64) * 1000
        out[f"hap{k}"] = hap
        out[f"omega_sd2_{k}"] = ls.omega(HM(hap.copy(), pos.copy()))
        out[f"omega_r2_{k}"] = ls.omega(HM(hap.copy(), pos.copy()), estimator="r2")
        out[f"omega_sd2_excl_{k}"] = ls.omega(HM(hap.copy(), pos.copy()), missing_data="exclude")
        r2 = np.asarray(HM(hap.copy(), pos.copy()).pairwise_r2())
        out[f"r2_{k}"] = r2
        out[f"omega_arr_{k}"] = ls.omega(S.garr(r2))
    np.savez_compressed(os.path.join(HERE, "omega.npz"), **out)


def gen_unlinked(M):
    """HaplotypeMatrix.locate_unlinked (haplotype_matrix.py:1172-1233) from the
    reference: sliding windows, greedy pruning on naive r^2."""
    HM = S.load_haplotype_matrix()
    out = {}
    for k, (H, m, F, sw, miss, size, step, thr) in enumerate(
            [(40, 300, 6, 0.05, 0.0, 100, 20, 0.1), (64, 500, 8, 0.02, 0.03, 50, 10, 0.2),
             (30, 120, 3, 0.2, 0.05, 7, 3, 0.05)]):
        rng = np.random.default_rng(20261211 + k)
        hap = copying_model(rng, H, m, F, sw, missing=miss)
        pos = np.arange(m, dtype=np.int64) * 100
        loc = HM(hap.copy(), pos.copy()).locate_unlinked(size=size, step=step, threshold=thr)
        out[f"hap{k}"] = hap
        out[f"args{k}"] = np.array([size, step], np.int64)
        out[f"thr{k}"] = np.float64(thr)
        out[f"loc{k}"] = np.asarray(loc, bool)
    np.savez_compressed(os.path.join(HERE, "unlinked.npz"), **out)


def gen_diploid_ld(M):
    """ZnS and omega of a GenotypeMatrix (zns_diploid / omega_diploid: the
    dosage-correlation r^2 matrix of _r2_matrix_diploid, ld_statistics.py:
    973-1020, then zns / omega of it), from the reference."""
    ls = M["ld_statistics"]
    S.load_haplotype_matrix()
    GM = sys.modules["pg_gpu.genotype_matrix"].GenotypeMatrix
    out = {}
    for k, (n, m, miss) in enumerate([(30, 80, 0.0), (50, 120, 0.03), (20, 9, 0.1)]):
        rng = np.random.default_rng(20261212 + k)
        h = copying_model(rng, 2 * n, m, 6, 0.02)
        g = (h[0::2] + h[1::2]).astype(np.int8)
        g[rng.random(g.shape) < miss] = -1
        pos = np.arange(m, dtype=np.int64) * 100
        out[f"geno{k}"] = g
        out[f"r2_{k}"] = np.asarray(ls._r2_matrix_diploid(S.garr(g)))
        out[f"zns_{k}"] = ls.zns(GM(g.copy(), pos.copy()))
        out[f"omega_{k}"] = ls.omega(GM(g.copy(), pos.copy()))
        out[f"zns_excl_{k}"] = ls.zns(GM(g.copy(), pos.copy()), missing_data="exclude")
        out[f"omega_excl_{k}"] = ls.omega(GM(g.copy(), pos.copy()), missing_data="exclude")
    np.savez_compressed(os.path.join(HERE, "diploid_ld.npz"), **out)


def gen_mu_ld(M):
    """mu_LD (ld_statistics.mu_ld, ld_statistics.py:865-918) from the
    reference, with its haplotype clustering (diversity.py:1310-1360, loaded
    through the shim): matrices without missing data, with missing data (the
    wildcard clustering), missing_data 'exclude', and one- / two-variant
    edges."""
    import importlib.util
    ls = M["ld_statistics"]
    HM = S.load_haplotype_matrix()
    pkg = sys.modules["pg_gpu"]
    for mod in ("_utils", "diversity"):
        if hasattr(pkg, mod):
            continue
        path = os.path.join(S.REF_ROOT, "pg_gpu", mod + ".py")
        spec = importlib.util.spec_from_file_location("pg_gpu." + mod, path)
        m = importlib.util.module_from_spec(spec)
        sys.modules["pg_gpu." + mod] = m
        spec.loader.exec_module(m)
        setattr(pkg, mod, m)
    out = {}
    cases = [(40, 30, 4, 0.05, 0.0), (64, 51, 6, 0.02, 0.0), (50, 40, 3, 0.1, 0.04),
             (32, 25, 5, 0.05, 0.1), (20, 1, 2, 0.0, 0.0), (20, 2, 2, 0.5, 0.0),
             (200, 120, 10, 0.01, 0.01)]
    for k, (H, m, F, sw, miss) in enumerate(cases):
        rng = np.random.default_rng(20261220 + k)
        hap = copying_model(rng, H, m, F, sw, missing=miss)
        pos = np.arange(1, m + 1, dtype=np.int64) * 100
        out[f"hap{k}"] = hap
        out[f"mu_{k}"] = ls.mu_ld(HM(hap.copy(), pos.copy()))
        out[f"mu_excl_{k}"] = ls.mu_ld(HM(hap.copy(), pos.copy()), missing_data="exclude")
    np.savez_compressed(os.path.join(HERE, "mu_ld.npz"), **out)


def _load_ref_module(mod):
    """A further reference module under the stub package (after
    load_haplotype_matrix)."""
    import importlib.util
    pkg = sys.modules["pg_gpu"]
    if hasattr(pkg, mod):
        return getattr(pkg, mod)
    path = os.path.join(S.REF_ROOT, "pg_gpu", mod + ".py")
    spec = importlib.util.spec_from_file_location("pg_gpu." + mod, path)
    m = importlib.util.module_from_spec(spec)
    sys.modules["pg_gpu." + mod] = m
    spec.loader.exec_module(m)
    setattr(pkg, mod, m)
    return m


def gen_dense(M):
    """The dense M x M outputs of the reference's HaplotypeMatrix:
    pairwise_LD_v, pairwise_r2 (estimators 'r2' and 'rogers_huff') and
    windowed_r_squared (haplotype_matrix.py:1092-1170, 1235-1317), on
    copying-model panels with and without missing data."""
    HM = S.load_haplotype_matrix()
    out = {}
    cases = [(40, 90, 6, 0.03, 0.0), (64, 150, 8, 0.02, 0.03), (33, 70, 4, 0.05, 0.05),
             (130, 200, 10, 0.01, 0.0)]
    for k, (H, m, F, sw, miss) in enumerate(cases):
        rng = np.random.default_rng(20261230 + k)
        hap = copying_model(rng, H, m, F, sw, missing=miss)
        pos = np.sort(rng.choice(50_000, m, replace=False)).astype(np.int64) + 1
        hm = HM(hap.copy(), pos.copy())
        out[f"hap{k}"] = hap
        out[f"pos{k}"] = pos
        out[f"ldv{k}"] = np.asarray(hm.pairwise_LD_v())
        out[f"r2_{k}"] = np.asarray(HM(hap.copy(), pos.copy()).pairwise_r2())
        if H % 2 == 0 and not miss:
            out[f"rh_{k}"] = np.asarray(HM(hap.copy(), pos.copy()).pairwise_r2(estimator="rogers_huff"))
        bins = np.array([0.0, 500.0, 2_000.0, 5_000.0, 15_000.0, 40_000.0])
        res, cnt = HM(hap.copy(), pos.copy()).windowed_r_squared(bins, percentile=[5, 50, 95])
        out[f"wbins{k}"] = bins
        out[f"wr2_{k}"] = np.asarray(res)
        out[f"wcnt{k}"] = np.asarray(cnt)
        res1, cnt1 = HM(hap.copy(), pos.copy()).windowed_r_squared(bins, percentile=50)
        out[f"wr2med_{k}"] = np.asarray(res1)
        if H % 2 == 0 and not miss:
            resr, cntr = HM(hap.copy(), pos.copy()).windowed_r_squared(
                bins, percentile=[25, 75], estimator="rogers_huff")
            out[f"wrh_{k}"] = np.asarray(resr)
            out[f"wrhcnt{k}"] = np.asarray(cntr)
    np.savez_compressed(os.path.join(HERE, "dense.npz"), **out)


def gen_rbins(M):
    """moments_ld.compute_ld_statistics with recombination-distance bins
    (r_bins and rec_map_file, moments_ld.py:164-175, 211-245) from the
    reference, haplotype and genotype paths, on the IM example panel with a
    piecewise-linear genetic map (tests/golden/rec_map_im.txt, written here)."""
    HM = S.load_haplotype_matrix()
    mld = _load_ref_module("moments_ld")
    z = np.load(os.path.join(HERE, "moments_im.npz"))
    hap, pos = z["hap"], z["pos"]
    rng = np.random.default_rng(20261231)
    knots = np.arange(0, 1_050_001, 50_000)
    rates = rng.uniform(0.3, 3.0, len(knots) - 1)  # cM per Mb
    cm = np.concatenate([[0.0], np.cumsum(rates * np.diff(knots) / 1e6)])
    path = os.path.join(HERE, "rec_map_im.txt")
    with open(path, "w") as f:
        f.write("pos\tMap(cM)\n")
        for p_, c in zip(knots, cm):
            f.write(f"{int(p_)}\t{c:.10f}\n")
    r_bins = np.array([0.0, 1e-6, 3e-6, 1e-5, 3e-5, 1e-4, 3e-4])
    sets = {"deme0": list(map(int, z["rows0"])), "deme1": list(map(int, z["rows1"]))}
    out = {"r_bins": r_bins}
    for tag, geno in (("hap", False), ("geno", True)):
        hm = HM(hap.copy(), pos.copy(), sample_sets={k: list(v) for k, v in sets.items()})
        res = mld.compute_ld_statistics(haplotype_matrix=hm, rec_map_file=path,
                                        pops=["deme0", "deme1"], r_bins=r_bins,
                                        use_genotypes=geno, report=False)
        out[f"{tag}_ld"] = np.stack([np.asarray(x, np.float64) for x in res["sums"][:-1]])
        out[f"{tag}_het"] = np.asarray(res["sums"][-1], np.float64)
        out[f"{tag}_bins"] = np.asarray(res["bins"], np.float64)
    np.savez_compressed(os.path.join(HERE, "rbins.npz"), **out)


def main():
    M = S.load_reference_modules()
    gen_hap_counts(M)
    gen_hap_stats(M)
    gen_binned(M)
    gen_moments(M)
    gen_geno(M)
    gen_geno_stats(M)
    gen_geno_binned(M)
    gen_windows(M)
    gen_omega(M)
    gen_unlinked(M)
    gen_diploid_ld(M)
    gen_mu_ld(M)
    gen_dense(M)
    gen_rbins(M)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz") or f.endswith(".txt"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
