"""CPU oracle for the two-locus LD path -- TEST INFRASTRUCTURE ONLY.

This module restates, in plain numpy, the arithmetic of the reference
pg_gpu LD path (kr-colab/pg_gpu).  It is the checker the CUDA library is
compared against; nothing in the shipped package imports it.  Only
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` may use it.

Every statistic is formed as an exact integer numerator over an exact
integer denominator (numpy int64) and divided once in float64, which is
exactly what the reference's float64 kernels compute whenever their
intermediate terms stay below 2**53 (they do for the sample sizes here).

Parity is pinned by ``tests/test_oracle_golden.py`` against fixtures that
``tests/golden/make_golden.py`` produced by running the reference's own code,
and against the moments result shipped with the reference's tests.
"""
from __future__ import annotations

import numpy as np

I64 = np.int64


# ---------------------------------------------------------------------------
# pair enumeration  (ld_pipeline.py:57-122)
# ---------------------------------------------------------------------------
def pairs_within_distance(positions, max_dist):
    """All (i<j) with pos[j]-pos[i] <= max_dist, i-major then j ascending.

    Same pair set and order as concatenating every chunk yielded by
    ``ld_pipeline.iter_pairs_within_distance`` (ld_pipeline.py:57-122).
    """
    pos = np.asarray(positions)
    n = len(pos)
    if n < 2:
        return np.zeros(0, np.int32), np.zeros(0, np.int32)
    jmax = np.searchsorted(pos, pos + max_dist, side="right")
    per = np.maximum(0, jmax - np.arange(n) - 1)
    total = int(per.sum())
    idx_i = np.repeat(np.arange(n, dtype=np.int64), per)
    start = np.cumsum(per) - per
    within = np.arange(total, dtype=np.int64) - np.repeat(start, per)
    idx_j = idx_i + 1 + within
    return idx_i.astype(np.int32), idx_j.astype(np.int32)


def chunk_bounds(positions, max_dist, chunk_size):
    """Anchor-block chunking of the pair list (ld_pipeline.py:94-122).

    Returns a list of (v_lo, v_hi, n_pairs) for the non-empty chunks: chunk k
    holds every pair whose first index lies in [v_lo, v_hi).
    """
    pos = np.asarray(positions)
    n = len(pos)
    if n < 2:
        return []
    jmax = np.searchsorted(pos, pos + max_dist, side="right")
    per = np.maximum(0, jmax - np.arange(n) - 1)
    cum = np.cumsum(per)
    total = int(cum[-1])
    if total == 0:
        return []
    chunk_size = max(1, int(chunk_size))
    n_chunks = (total + chunk_size - 1) // chunk_size
    targets = np.minimum(np.arange(1, n_chunks + 1, dtype=np.int64) * chunk_size, total)
    v_his = np.minimum(np.searchsorted(cum, targets, side="left") + 1, n)
    out = []
    v_lo = 0
    for v_hi in v_his:
        v_hi = int(v_hi)
        if v_hi <= v_lo:
            continue
        npairs = int(per[v_lo:v_hi].sum())
        if npairs:
            out.append((v_lo, v_hi, npairs))
        v_lo = v_hi
    return out


# ---------------------------------------------------------------------------
# joint counts  (ld_pipeline.py:130-175, 183-263)
# ---------------------------------------------------------------------------
def counts_for_pairs(hap, idx_i, idx_j, rows=None):
    """[n11, n10, n01, n00] int32 per pair, plus n_valid (or None).

    ``==1`` / ``==0`` allele semantics and ``>=0`` validity; n_valid is None
    unless the (row-subset) matrix holds a -1 somewhere (ld_pipeline.py:158).
    """
    h = np.asarray(hap)
    if rows is not None:
        h = h[np.asarray(rows), :]
    hi = h[:, idx_i]
    hj = h[:, idx_j]
    has_missing = bool(np.any(h == -1))
    v = (hi >= 0) & (hj >= 0)
    c = np.stack([
        np.sum((hi == 1) & (hj == 1) & v, axis=0, dtype=np.int32),
        np.sum((hi == 1) & (hj == 0) & v, axis=0, dtype=np.int32),
        np.sum((hi == 0) & (hj == 1) & v, axis=0, dtype=np.int32),
        np.sum((hi == 0) & (hj == 0) & v, axis=0, dtype=np.int32),
    ], axis=1)
    nv = np.sum(v, axis=0, dtype=np.int32) if has_missing else None
    return c, nv


def genotype_counts_for_pairs(geno, idx_i, idx_j, rows=None):
    """9-way counts ordered n00,n01,n02,n10,...,n22 plus n_valid (or None).

    Follows the reference counting kernel (ld_pipeline.py:183-217): an
    individual contributes when both dosages are >= 0; n_valid is returned
    only when the matrix holds a negative entry (ld_pipeline.py:253).
    """
    g = np.asarray(geno).astype(np.int8)
    if rows is not None:
        g = g[np.asarray(rows), :]
    gi = g[:, idx_i].astype(np.int32)
    gj = g[:, idx_j].astype(np.int32)
    ok = (gi >= 0) & (gj >= 0)
    combo = gi * 3 + gj
    out = np.zeros((len(idx_i), 9), np.int32)
    for k in range(9):
        out[:, k] = np.sum(ok & (combo == k), axis=0)
    nv = np.sum(ok, axis=0, dtype=np.int32)
    return out, (nv if bool(np.any(g < 0)) else None)


# ---------------------------------------------------------------------------
# per-population integer features
# ---------------------------------------------------------------------------
class Pop:
    """Integer per-pair features of one population (cf. ld_pipeline.py:465-482)."""

    def __init__(self, c4, n):
        c = np.asarray(c4).astype(I64)
        self.c1, self.c2, self.c3, self.c4 = c[:, 0], c[:, 1], c[:, 2], c[:, 3]
        self.n = np.asarray(n).astype(I64)
        self.pA = self.c1 + self.c2
        self.qA = self.c3 + self.c4
        self.pB = self.c1 + self.c3
        self.qB = self.c2 + self.c4
        # x = c1*c4 - c2*c3 is minus the reference's D (ld_pipeline.py:478)
        self.x = self.c1 * self.c4 - self.c2 * self.c3


def _q(num, den):
    """num/den in float64 where den > 0, else 0 (the kernels' convention)."""
    num = np.asarray(num)
    den = np.asarray(den)
    out = np.zeros(np.broadcast(num, den).shape, np.float64)
    ok = den > 0
    out[ok] = num[ok].astype(np.float64) / den[ok].astype(np.float64)
    return out


def _d4(n):
    return n * (n - 1) * (n - 2) * (n - 3)


# --- DD (ld_statistics.py:1116-1169, haplotype_kernels.py:69-89) ----------
def dd_ii(p):
    c1, c2, c3, c4 = p.c1, p.c2, p.c3, p.c4
    num = c1 * (c1 - 1) * c4 * (c4 - 1) + c2 * (c2 - 1) * c3 * (c3 - 1) - 2 * c1 * c2 * c3 * c4
    return num, _d4(p.n)


def dd_ij(a, b):
    return a.x * b.x, a.n * (a.n - 1) * b.n * (b.n - 1)


# --- Dz (ld_statistics.py:1172-1272, haplotype_kernels.py:95-160) ---------
def dz_iii(p):
    c1, c2, c3, c4 = p.c1, p.c2, p.c3, p.c4
    num = (p.x * (p.qA - p.pA) * (p.qB - p.pB) + p.x * ((c2 + c3) - (c1 + c4))
           + 2 * (c2 * c3 + c1 * c4))
    return num, _d4(p.n)


def dz_iij(i, j):
    return (i.qA - i.pA) * i.x * (j.qB - j.pB), j.n * i.n * (i.n - 1) * (i.n - 2)


def dz_iji(i, j):
    return (i.qB - i.pB) * i.x * (j.qA - j.pA), j.n * i.n * (i.n - 1) * (i.n - 2)


def dz_ijj(i, j):
    num = i.x * ((j.c2 + j.c3) - (j.c1 + j.c4)) + i.x * (j.qB - j.pB) * (j.qA - j.pA)
    return num, i.n * (i.n - 1) * j.n * (j.n - 1)


def dz_ijk(i, j, k):
    return i.x * (j.pA - j.qA) * (k.pB - k.qB), i.n * (i.n - 1) * j.n * k.n


# --- pi2 (ld_statistics.py:1275-1617, haplotype_kernels.py:167-304) -------
def pi2_iiii(p):
    c1, c2, c3, c4 = p.c1, p.c2, p.c3, p.c4
    num = (p.pA * p.pB * p.qB * p.qA - c1 * c4 * (-1 + c1 + 3 * c2 + 3 * c3 + c4)
           - c2 * c3 * (-1 + 3 * c1 + c2 + c3 + 3 * c4))
    return num, _d4(p.n)


def pi2_triple(t, s):
    """pi2 with population t three times and s once; value = num / den."""
    num2 = (t.pA * t.qA * (t.qB * s.pB + t.pB * s.qB - 2 * s.qB)
            + (t.pA * t.c4 + t.c2 * t.qA) * (s.qB - s.pB))
    return num2, 2 * s.n * t.n * (t.n - 1) * (t.n - 2)


def pi2_iikk(i, k):
    """Kernel form (haplotype_kernels.py:180-190): not symmetrised."""
    return i.pA * i.qA * k.pB * k.qB, i.n * (i.n - 1) * k.n * (k.n - 1)


def pi2_iikk_sym(i, k):
    """ld_statistics form (ld_statistics.py:1327-1339): symmetrised."""
    num2 = i.pA * i.qA * k.pB * k.qB + k.pA * k.qA * i.pB * i.qB
    return num2, 2 * i.n * (i.n - 1) * k.n * (k.n - 1)


def pi2_iikl(i, k, l):
    num2 = i.pA * i.qA * (k.pB * l.qB + k.qB * l.pB)
    return num2, 2 * i.n * (i.n - 1) * k.n * l.n


def pi2_ijkk(i, j, k):
    num2 = k.pB * k.qB * (i.pA * j.qA + i.qA * j.pA)
    return num2, 2 * k.n * (k.n - 1) * i.n * j.n


def pi2_ijij(a, b):
    a1, a2, a3, a4 = a.c1, a.c2, a.c3, a.c4
    b1, b2, b3, b4 = b.c1, b.c2, b.c3, b.c4
    quart = (a.qB * a.qA * b.pA * b.pB + a.pB * a.qA * b.pA * b.qB
             + a.pA * a.qB * b.pB * b.qA + a.pA * a.pB * b.qB * b.qA)
    # cubic correction, grouped by the count of b it multiplies
    cub = (b1 * (a4 - a2 * a3 - a2 * a4 - a3 * a4 - a4 * a4 - a4 * b1)
           + b2 * (a3 - a1 * a3 - a3 * a3 - a1 * a4 - a3 * a4 - a3 * b1 - a4 * b1 - a3 * b2)
           + b3 * (a2 - a1 * a2 - a2 * a2 - a1 * a4 - a2 * a4 - a2 * b1 - a4 * b1
                   - a1 * b2 - a4 * b2 - a2 * b3)
           + b4 * (a1 - a1 * a1 - a1 * a2 - a1 * a3 - a2 * a3 - a2 * b1 - a3 * b1
                   - a1 * b2 - a3 * b2 - a1 * b3 - a2 * b3 - a1 * b4))
    return quart + cub, 4 * a.n * (a.n - 1) * b.n * (b.n - 1)


def pi2_shared(s, a, b):
    """s appears in both pairs, a in the first, b in the second (ld_statistics.py:1519-1589)."""
    s1, s2, s3, s4 = s.c1, s.c2, s.c3, s.c4
    a1, a2 = a.c1, a.c2
    b1, b2, b3, b4 = b.c1, b.c2, b.c3, b.c4
    inner = (s3 - 1) * b1 + s3 * b2 - b3 + s3 * b3 + s3 * b4 + s1 * b.qB
    num4 = (s4 * s4 * a.pA * b.pB + s2 * s2 * a.qA * b.pB
            + (s1 + s3 - 1) * (s3 * a.pA + s1 * a.qA) * b.qB
            + s4 * (s1 * a.qA * b.pB + (a1 + a2) * inner)
            + s2 * (s4 * (a.pA + a.qA) * b.pB + s3 * (a.pA * b.pB + a.qA * b.qB)
                    + a.qA * ((s1 - 1) * b1 - b3 + s1 * (b2 + b3 + b4))))
    return num4, 4 * s.n * (s.n - 1) * a.n * b.n


def pi2_alldiff(i, j, k, l):
    num4 = (i.qA * j.pA + i.pA * j.qA) * (k.qB * l.pB + k.pB * l.qB)
    return num4, 4 * i.n * j.n * k.n * l.n


# ---------------------------------------------------------------------------
# public-API dispatch  (ld_statistics.py:13-129, 1082-1113)
# ---------------------------------------------------------------------------
def _pop_n(counts, n_valid, p):
    """Valid n of population p, following _get_pop_data (ld_statistics.py:1082-1113)."""
    c = np.asarray(counts)[:, 4 * p:4 * p + 4].astype(I64)
    if n_valid is None:
        return c.sum(axis=1)
    if isinstance(n_valid, tuple):
        if p < len(n_valid) and n_valid[p] is not None:
            return np.asarray(n_valid[p]).astype(I64)
        return c.sum(axis=1)
    nv = np.asarray(n_valid)
    if nv.ndim == 2:
        return nv[:, p].astype(I64)
    return nv.astype(I64)


def _pop(counts, n_valid, p):
    return Pop(np.asarray(counts)[:, 4 * p:4 * p + 4], _pop_n(counts, n_valid, p))


def dd(counts, populations=None, n_valid=None):
    c = np.asarray(counts)
    if populations is None or populations[0] == populations[1]:
        p = 0 if populations is None else populations[0]
        if populations is None and isinstance(n_valid, np.ndarray) and n_valid.ndim == 2:
            n_valid = n_valid[:, 0]
        if populations is None and c.shape[1] == 4:
            return _q(*dd_ii(Pop(c, _pop_n(c, n_valid, 0))))
        return _q(*dd_ii(_pop(c, n_valid, p)))
    a, b = populations
    if isinstance(n_valid, np.ndarray) and n_valid.ndim == 1:
        na = nb = n_valid.astype(I64)
        pa = Pop(c[:, 4 * a:4 * a + 4], na)
        pb = Pop(c[:, 4 * b:4 * b + 4], nb)
    elif isinstance(n_valid, tuple):
        # _dd_between reads the tuple by position (0, 1), not by pop index
        pa = Pop(c[:, 4 * a:4 * a + 4], _pop_n(c[:, 4 * a:4 * a + 4], (n_valid[0],), 0))
        pb = Pop(c[:, 4 * b:4 * b + 4], _pop_n(c[:, 4 * b:4 * b + 4], (n_valid[1],), 0))
    else:
        pa = _pop(c, n_valid, a)
        pb = _pop(c, n_valid, b)
    return _q(*dd_ij(pa, pb))


def dz(counts, populations=None, n_valid=None):
    c = np.asarray(counts)
    if populations is None:
        if c.shape[1] == 4:
            return _q(*dz_iii(Pop(c, _pop_n(c, n_valid, 0))))
        populations = (0, 0, 0)
    i, j, k = populations
    P = lambda p: _pop(c, n_valid, p)  # noqa: E731
    if i == j == k:
        return _q(*dz_iii(P(i)))
    if i == j:
        return _q(*dz_iij(P(i), P(k)))
    if i == k:
        return _q(*dz_iji(P(i), P(j)))
    if j == k:
        return _q(*dz_ijj(P(i), P(j)))
    return _q(*dz_ijk(P(i), P(j), P(k)))


def pi2(counts, populations=None, n_valid=None):
    c = np.asarray(counts)
    if populations is None:
        if c.shape[1] == 4:
            return _q(*pi2_iiii(Pop(c, _pop_n(c, n_valid, 0))))
        populations = (0, 0, 0, 0)
    i, j, k, l = populations
    P = lambda p: _pop(c, n_valid, p)  # noqa: E731
    cnt = {}
    for p in populations:
        cnt[p] = cnt.get(p, 0) + 1
    nu, mc = len(cnt), max(cnt.values())
    if nu == 1:
        return _q(*pi2_iiii(P(i)))
    if mc == 3:
        t = [p for p, v in cnt.items() if v == 3][0]
        s = [p for p, v in cnt.items() if v == 1][0]
        return _q(*pi2_triple(P(t), P(s)))
    if i == j and k == l:
        return _q(*pi2_iikk_sym(P(i), P(k)))
    if i == j:
        return _q(*pi2_iikl(P(i), P(k), P(l)))
    if k == l:
        return _q(*pi2_ijkk(P(i), P(j), P(k)))
    if (i == k and j == l) or (i == l and j == k):
        return _q(*pi2_ijij(P(i), P(j)))
    if nu == 4:
        return _q(*pi2_alldiff(P(i), P(j), P(k), P(l)))
    s, a, b = _shared_roles(i, j, k, l)
    return _q(*pi2_shared(P(s), P(a), P(b)))


def _shared_roles(i, j, k, l):
    if i == k:
        return i, j, l
    if i == l:
        return i, j, k
    if j == k:
        return j, i, l
    return j, i, k


# ---------------------------------------------------------------------------
# r, r^2, D'  (haplotype_kernels.py:20-62, ld_statistics.py:153-246)
# ---------------------------------------------------------------------------
def _rsq_parts(counts, n_valid):
    c = np.asarray(counts).astype(I64)
    a, b, cc, d = c[:, 0], c[:, 1], c[:, 2], c[:, 3]
    n = c.sum(axis=1) if n_valid is None else np.asarray(n_valid).astype(I64)
    return a, b, cc, d, n


def r(counts, n_valid=None):
    a, b, c, d, n = _rsq_parts(counts, n_valid)
    den = (a + b) * (n - a - b) * (a + c) * (n - a - c)
    out = np.full(len(a), np.nan)
    ok = den > 0
    out[ok] = (a * d - b * c)[ok].astype(np.float64) / np.sqrt(den[ok].astype(np.float64))
    return out


def r_squared(counts, n_valid=None):
    a, b, c, d, n = _rsq_parts(counts, n_valid)
    den = (a + b) * (n - a - b) * (a + c) * (n - a - c)
    num = (a * d - b * c) ** 2
    out = np.full(len(a), np.nan)
    ok = den > 0
    out[ok] = num[ok].astype(np.float64) / den[ok].astype(np.float64)
    return out


def d_prime(counts, n_valid=None):
    a, b, c, d, n = _rsq_parts(counts, n_valid)
    x = a * d - b * c
    pos = np.minimum((a + b) * (n - a - c), (n - a - b) * (a + c))
    neg = np.minimum((a + b) * (a + c), (n - a - b) * (n - a - c))
    dmax = np.where(x >= 0, pos, neg)
    out = np.full(len(a), np.nan)
    ok = dmax > 0
    out[ok] = x[ok].astype(np.float64) / dmax[ok].astype(np.float64)
    return out


# ---------------------------------------------------------------------------
# moments statistic names / specs  (ld_pipeline.py:357-457)
# ---------------------------------------------------------------------------
def ld_names(P):
    names = [f"DD_{i}_{j}" for i in range(P) for j in range(i, P)]
    names += [f"Dz_{i}_{j}_{k}" for i in range(P) for j in range(P) for k in range(j, P)]
    for i in range(P):
        for j in range(i, P):
            for k in range(i, P):
                for l in range(k, P):
                    if k == i == l and j != i:
                        continue
                    if i == k and l < j:
                        continue
                    names.append(f"pi2_{i}_{j}_{k}_{l}")
    return names


def het_names(P):
    return [f"H_{i}_{j}" for i in range(P) for j in range(i, P)]


def stat_specs(P):
    """(name, [(weight, kind, pops)]) exactly as generate_stat_specs."""
    specs = []
    for name in ld_names(P):
        parts = name.split("_")
        kind, pp = parts[0], tuple(int(v) for v in parts[1:])
        if kind == "DD":
            specs.append((name, [(1.0, "dd", pp)]))
        elif kind == "Dz":
            i, j, k = pp
            if j == k:
                specs.append((name, [(1.0, "dz", pp)]))
            else:
                specs.append((name, [(0.5, "dz", (i, j, k)), (0.5, "dz", (i, k, j))]))
        else:
            i, j, k, l = pp
            if i == j and k == l:
                if i == k:
                    specs.append((name, [(1.0, "pi2", pp)]))
                else:
                    specs.append((name, [(0.5, "pi2", (i, j, k, l)), (0.5, "pi2", (k, l, i, j))]))
            elif i == j:
                specs.append((name, [(0.25, "pi2", t) for t in
                                     ((i, j, k, l), (i, j, l, k), (k, l, i, j), (l, k, i, j))]))
            elif k == l:
                specs.append((name, [(0.25, "pi2", t) for t in
                                     ((i, j, k, l), (j, i, k, l), (k, l, i, j), (k, l, j, i))]))
            else:
                specs.append((name, [(0.125, "pi2", t) for t in
                                     ((i, j, k, l), (i, j, l, k), (j, i, k, l), (j, i, l, k),
                                      (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i))]))
    return specs


def kernel_case_value(kind, pp, pops):
    """One case of the fused kernels (haplotype_kernels.py:335-581)."""
    if kind == "dd":
        a, b = pp
        return _q(*(dd_ii(pops[a]) if a == b else dd_ij(pops[a], pops[b])))
    if kind == "dz":
        i, j, k = pp
        if i == j == k:
            return _q(*dz_iii(pops[i]))
        if i == j:
            return _q(*dz_iij(pops[i], pops[k]))
        if i == k:
            return _q(*dz_iji(pops[i], pops[j]))
        if j == k:
            return _q(*dz_ijj(pops[i], pops[j]))
        return _q(*dz_ijk(pops[i], pops[j], pops[k]))
    i, j, k, l = pp
    cnt = {}
    for p in pp:
        cnt[p] = cnt.get(p, 0) + 1
    nu, mc = len(cnt), max(cnt.values())
    if nu == 1:
        return _q(*pi2_iiii(pops[i]))
    if mc == 3:
        t = [p for p, v in cnt.items() if v == 3][0]
        s = [p for p, v in cnt.items() if v == 1][0]
        return _q(*pi2_triple(pops[t], pops[s]))
    if i == j and k == l:
        return _q(*pi2_iikk(pops[i], pops[k]))
    if i == j:
        return _q(*pi2_iikl(pops[i], pops[k], pops[l]))
    if k == l:
        return _q(*pi2_ijkk(pops[i], pops[j], pops[k]))
    if (i == k and j == l) or (i == l and j == k):
        return _q(*pi2_ijij(pops[i], pops[j]))
    if nu == 3:
        s, a, b = _shared_roles(i, j, k, l)
        return _q(*pi2_shared(pops[s], pops[a], pops[b]))
    return _q(*pi2_alldiff(pops[i], pops[j], pops[k], pops[l]))


def multi_pop_stats(counts_per_pop, n_valid_per_pop, specs=None):
    """(N, n_stats) float64 as compute_multi_pop_statistics_batch_hap."""
    P = len(counts_per_pop)
    specs = stat_specs(P) if specs is None else specs
    pops = []
    for c, nv in zip(counts_per_pop, n_valid_per_pop):
        c = np.asarray(c)
        pops.append(Pop(c, c.astype(I64).sum(axis=1) if nv is None else nv))
    cache = {}
    out = np.zeros((len(np.asarray(counts_per_pop[0])), len(specs)), np.float64)
    for s, (_, calls) in enumerate(specs):
        acc = 0.0
        for w, kind, pp in calls:
            key = (kind, pp)
            if key not in cache:
                cache[key] = kernel_case_value(kind, pp, pops)
            acc = acc + (cache[key] if (w == 1.0 and len(calls) == 1) else w * cache[key])
        out[:, s] = acc
    return out


def two_pop_stats(c1, c2, nv1, nv2):
    """(N, 15) as ld_pipeline.compute_two_pop_statistics_batch, exact arithmetic."""
    return multi_pop_stats([c1, c2], [nv1, nv2])


def single_pop_stats(c, nv):
    """(N, 3) DD, Dz, pi2 as ld_pipeline.compute_single_pop_statistics_batch."""
    return np.stack([dd(c, n_valid=nv), dz(c, n_valid=nv), pi2(c, n_valid=nv)], axis=1)


# ---------------------------------------------------------------------------
# distance-binned sums  (moments_ld.py:248-343, haplotype_matrix.py:1592-1866)
# ---------------------------------------------------------------------------
def bin_index(distances, bins):
    """digitize(d, bins) - 1 with right-open bins; -1 / n_bins mark 'outside'."""
    return np.digitize(distances, np.asarray(bins, np.float64)) - 1


def binned_sums(hap, positions, pop_rows, bins, coords=None, max_dist=None,
                pair_block=2_000_000, abs_sums=False, anchor_stop=None, anchor_start=None,
                missing_flags=None):
    """(n_bins, n_stats) float64 sums of the per-pair statistics, plus pair counts.

    ``pop_rows``: list of row-index arrays, one per population (1..4).
    ``coords``: per-SNP coordinate used for the distance (positions when None;
    a genetic map in Morgans for the recombination-distance mode).
    With ``abs_sums`` the sums of |stat| are returned as a third value
    (the scale that bounds the float32 rounding of the GPU sums).
    ``anchor_start`` / ``anchor_stop``: only the pairs whose first SNP lies in
    [anchor_start, anchor_stop) (a sample of a large panel's pairs, or one
    rank's share).  ``missing_flags``: per population, whether its whole
    panel holds a -1 (the reference's n_valid switch, ld_pipeline.py:158);
    by default it is read from the SNPs the call looks at.
    """
    pos = np.asarray(positions)
    coord = pos.astype(np.float64) if coords is None else np.asarray(coords, np.float64)
    bins = np.asarray(bins, np.float64)
    n_bins = len(bins) - 1
    P = len(pop_rows)
    if max_dist is None:
        max_dist = float(bins[-1])
    n = len(pos)
    a0 = 0 if anchor_start is None else int(anchor_start)
    a1 = n if anchor_stop is None else min(int(anchor_stop), n)
    # the SNP slice [a0, halo): the anchors and their partners within max_dist
    halo = int(np.searchsorted(pos, pos[a1 - 1] + max_dist, side="right")) if a1 > a0 else a0
    pos = pos[a0:halo]
    coord = coord[a0:halo]
    ii, jj = pairs_within_distance(pos, max_dist)
    keep = ii < a1 - a0
    ii, jj = ii[keep], jj[keep]
    specs = stat_specs(P)
    sums = np.zeros((n_bins, len(specs)))
    asums = np.zeros((n_bins, len(specs)))
    npairs = np.zeros(n_bins, np.int64)
    h = np.asarray(hap)
    subs = [h[np.asarray(r), a0:halo] for r in pop_rows]
    miss = ([bool(np.any(s == -1)) for s in subs] if missing_flags is None
            else [bool(m) for m in missing_flags])
    for s0 in range(0, len(ii), pair_block):
        ci, cj = ii[s0:s0 + pair_block], jj[s0:s0 + pair_block]
        d = np.abs(coord[cj] - coord[ci]) if coords is not None else (coord[cj] - coord[ci])
        b = bin_index(d, bins)
        keep = (b >= 0) & (b < n_bins)
        if not np.any(keep):
            continue
        ci, cj, b = ci[keep], cj[keep], b[keep]
        cs, nvs = [], []
        for sub, m in zip(subs, miss):
            c, nv = counts_for_pairs(sub, ci, cj)
            cs.append(c)
            nvs.append(nv if m else None)
        st = multi_pop_stats(cs, nvs, specs)
        for k in range(len(specs)):
            sums[:, k] += np.bincount(b, weights=st[:, k], minlength=n_bins)
            if abs_sums:
                asums[:, k] += np.bincount(b, weights=np.abs(st[:, k]), minlength=n_bins)
        npairs += np.bincount(b, minlength=n_bins)
    if abs_sums:
        return sums, npairs, asums
    return sums, npairs


def bin_errors(got, ref, ref_abs=None, floor=0.0):
    """Errors of binned sums relative to the value: |got - ref| / max(|ref|,
    floor * ref_abs) per bin and statistic (0 where that scale is 0 and the
    sums agree, inf where it is 0 and they differ).  With floor > 0 a bin whose
    terms cancel to below floor * sum|x| is measured against that share of
    sum|x| (ref_abs, the oracle's sums of |x|) instead of its small value."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = np.abs(ref)
    if floor and ref_abs is not None:
        scale = np.maximum(scale, floor * np.asarray(ref_abs, np.float64))
    err = np.abs(got - ref)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(scale > 0, err / np.where(scale > 0, scale, 1.0),
                       np.where(err > 0, np.inf, 0.0))
    return rel


def binned_sums_task(args):
    """binned_sums(*args[0], **args[1]) with abs_sums; a picklable task for a
    process pool."""
    a, kw = args
    return binned_sums(*a, abs_sums=True, **kw)


def heterozygosity(hap, pop_rows):
    """H_i_j statistics (moments_ld.py:346-388), haplotype mode."""
    h = np.asarray(hap)
    alt, ref, size = [], [], []
    for rws in pop_rows:
        sub = h[np.asarray(rws), :]
        a = np.sum(np.maximum(sub, 0).astype(np.int64), axis=0).astype(np.float64)
        nh = float(len(rws)) * np.ones_like(a)
        alt.append(a)
        ref.append(nh - a)
        size.append(nh)
    out = {}
    P = len(pop_rows)
    for i in range(P):
        for j in range(i, P):
            if i == j:
                out[f"H_{i}_{j}"] = float(np.sum(2.0 * ref[i] * alt[i] / (size[i] * (size[i] - 1))))
            else:
                out[f"H_{i}_{j}"] = float(np.sum((ref[i] * alt[j] + alt[i] * ref[j])
                                                 / (size[i] * size[j])))
    return out


def biallelic_keep(hap):
    """Columns kept by HaplotypeMatrix.apply_biallelic_filter (haplotype_matrix.py:724-789)."""
    h = np.asarray(hap)
    return (np.sum(h >= 2, axis=0) == 0) & (np.sum(h == 0, axis=0) > 0) & (np.sum(h == 1, axis=0) > 0)


# ---------------------------------------------------------------------------
# all-pairs tally  (haplotype_matrix.py:1320-1589) -- correct at any H
# ---------------------------------------------------------------------------
def tally(hap, rows=None):
    h = np.asarray(hap)
    if rows is not None:
        h = h[np.asarray(rows), :]
    m = h.shape[1]
    ii, jj = np.triu_indices(m, k=1)
    c, _ = counts_for_pairs(h, ii, jj)
    if bool(np.any(h == -1)):
        valid = h != -1
        nv = np.sum(valid[:, ii] & valid[:, jj], axis=0, dtype=np.int32)
        return c, nv
    return c, None


# ---------------------------------------------------------------------------
# Rogers-Huff r  (ld_statistics.py:410-531)
# ---------------------------------------------------------------------------
def rogers_huff_r(geno):
    """Condensed upper-triangle Rogers-Huff r on a complete dosage matrix."""
    g = np.asarray(geno).astype(np.float64)
    if np.any(g < 0):
        raise ValueError("rogers_huff_r: missing values")
    n = g.shape[0]
    mu = g.mean(axis=0)
    ssd = ((g - mu) ** 2).sum(axis=0)
    cov = g.T @ g - n * np.outer(mu, mu)
    den = np.sqrt(np.outer(ssd, ssd))
    with np.errstate(invalid="ignore", divide="ignore"):
        rr = np.where(den > 0, cov / den, np.nan)
    iu = np.triu_indices(g.shape[1], k=1)
    return rr[iu]


def rogers_huff_r_pairs(geno, idx_i, idx_j):
    """Rogers-Huff r per listed pair with pairwise-complete individuals.

    With no missing dosage this equals the reference's rogers_huff_r on the
    same pairs; with missing data (where the reference raises) each pair
    uses the individuals valid at both loci -- the definition the CUDA
    path implements.  Exact integer moments, one float64 division.
    """
    g = np.asarray(geno).astype(np.int64)
    gi = g[:, idx_i]
    gj = g[:, idx_j]
    v = (gi >= 0) & (gj >= 0)
    gi = np.where(v, gi, 0)
    gj = np.where(v, gj, 0)
    n = v.sum(axis=0)
    si, sj = gi.sum(axis=0), gj.sum(axis=0)
    sii, sjj, sij = (gi * gi).sum(axis=0), (gj * gj).sum(axis=0), (gi * gj).sum(axis=0)
    cov = n * sij - si * sj
    vi = n * sii - si * si
    vj = n * sjj - sj * sj
    den = vi * vj
    out = np.full(len(idx_i), np.nan)
    ok = den > 0
    out[ok] = cov[ok].astype(np.float64) / np.sqrt(den[ok].astype(np.float64))
    return out


# ---------------------------------------------------------------------------
# genotype path: 9-way counts -> moments genotype statistics
# (genotype_kernels.py:27-936, ld_statistics_genotype.py:1518-1598)
# ---------------------------------------------------------------------------
def _geno_poly(table, g):
    """sum of coef * g[a] * g[b] * g[c] over a monomial table (g[9] = 1)."""
    acc = np.zeros(g.shape[1], I64)
    for coef, (a, b, c) in table:
        acc = acc + coef * g[a] * g[b] * g[c]
    return acc


class GenoPop:
    """Integer per-pair features of one population from 9-way counts.

    ``counts`` columns are the reference's n00, n01, ..., n22 (dosage at the
    first SNP times 3 plus dosage at the second, ld_pipeline.py:183-217); the
    features use moments order g1 = n22, ..., g9 = n00 (genotype_kernels.py:
    423-435).  Every half- or quarter-integer quantity of _PopDataGeno
    (genotype_kernels.py:437-521) is carried scaled to an integer:
    P2 = 2 pA, R2 = 2 qA, Q2 = 2 pB, S2 = 2 qB, X.. = 4 x.., D16 = 16 D_geno.
    """

    def __init__(self, counts, n_valid=None):
        c = np.asarray(counts).astype(I64)
        g = [c[:, 8 - k] for k in range(9)] + [np.ones(len(c), I64)]
        self.g = np.stack(g)
        g1, g2, g3, g4, g5, g6, g7, g8, g9 = g[:9]
        self.ns = c.sum(axis=1)
        self.n = self.ns if n_valid is None else np.asarray(n_valid).astype(I64)
        self.P2 = 2 * (g1 + g2 + g3) + g4 + g5 + g6
        self.R2 = g4 + g5 + g6 + 2 * (g7 + g8 + g9)
        self.Q2 = 2 * (g1 + g4 + g7) + g2 + g5 + g8
        self.S2 = g2 + g5 + g8 + 2 * (g3 + g6 + g9)
        self.X00 = 4 * g1 + 2 * g2 + 2 * g4 + g5
        self.X01 = 2 * g2 + 4 * g3 + g5 + 2 * g6
        self.X10 = 2 * g4 + g5 + 4 * g7 + 2 * g8
        self.X11 = g5 + 2 * g6 + 2 * g8 + 4 * g9
        self.D16 = self.X00 * self.X11 - self.X01 * self.X10
        self.a = -g1 + g3 - g4 + g6 - g7 + g9
        self.b = -g1 - g2 - g3 + g7 + g8 + g9
        cc = -g1 + g3 + g7 - g9
        # half of MA / MB of the Dz precompute (genotype_kernels.py:175-196)
        mah = g7 * (g2 + 2 * g3 + g5 + 2 * g6) + g8 * (g3 + g6 - g1 - g4) \
            - g9 * (2 * g1 + g2 + 2 * g4 + g5)
        mbh = g3 * (g4 + g5) - g6 * (g1 + g2) + (g7 + g8) * (2 * g3 + g6) \
            - g9 * (2 * g1 + 2 * g2 + g4 + g5)
        self.W = cc + self.a * self.b                   # Wjj
        self.U16 = self.D16 * (1 + self.b) + 8 * mah    # 16 Ucoef
        self.V16 = self.D16 * (1 + self.a) + 8 * mbh    # 16 Vcoef
        n = self.n
        self.m = np.maximum(4 * n * (n - 1), 1)         # B_L / C.. denominators
        self.BL = self.P2 * self.R2 - (g4 + g5 + g6)    # 4 n(n-1) B_L
        self.BR = self.Q2 * self.S2 - (g2 + g5 + g8)    # 4 n(n-1) B_R
        self.C00 = self.P2 * self.Q2 - self.X00         # 16 n(n-1) C00
        self.C01 = self.P2 * self.S2 - self.X01
        self.C10 = self.R2 * self.Q2 - self.X10
        self.C11 = self.R2 * self.S2 - self.X11
        self.Bs = self.X00 - self.X01 - self.X10 + self.X11  # 4 Bsgn
        # triple coefficients, times 16 (genotype_kernels.py:500-521)
        L0 = g5 + 2 * g6 + 2 * g8 + 4 * g9
        L1 = g5 + 2 * g6
        M1 = g5 + 2 * g8
        nR3 = 3 * (g4 + g5 + g6) + 4 * (g7 + g8 + g9)
        nR5 = 5 * (g4 + g5 + g6) + 8 * (g7 + g8 + g9)
        b5A = -2 * g2 - 4 * g3 + 4 * g4 + g5 - 2 * g6 + 8 * g7 + 4 * g8 + 4
        b6A = -g5 - 2 * g6 - 4 * g7 - 4 * g8 - 4 * g9
        nL3 = 3 * (g2 + g5 + g8) + 4 * (g3 + g6 + g9)
        nL5 = 5 * (g2 + g5 + g8) + 8 * (g3 + g6 + g9)
        b5B = 4 * g2 + 8 * g3 - 2 * g4 + g5 + 4 * g6 - 4 * g7 - 2 * g8 + 4
        b6B = -4 * g3 - g5 - 4 * g6 - 2 * g8 - 4 * g9
        P2, Q2, R2, S2 = self.P2, self.Q2, self.R2, self.S2
        self.AQ3 = -S2 * nR3 + P2 * S2 * R2 + R2 * L0 + 2 * L1 - P2 * L0
        self.AS3 = -Q2 * nR5 + P2 * Q2 * R2 + R2 * b5A + 2 * b6A + P2 * L0
        self.BP3 = -R2 * nL3 + Q2 * S2 * R2 + S2 * L0 + 2 * M1 - Q2 * L0
        self.BR3 = -P2 * nL5 + P2 * Q2 * S2 + S2 * b5B + 2 * b6B + Q2 * L0


def _fdiv(num, den):
    """num / den in float64 with IEEE results for den == 0 (no guard)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.asarray(num).astype(np.float64) / np.asarray(den).astype(np.float64)


def _gate(ok, num, den):
    out = np.zeros(np.broadcast(num, den).shape, np.float64)
    ok = np.asarray(ok) & (np.asarray(den) != 0)
    out[ok] = np.asarray(num)[ok].astype(np.float64) / np.asarray(den)[ok].astype(np.float64)
    return out


def geno_dd(pp, pops):
    """DD of _DD_GENO_SINGLE_KERN / _DD_GENO_BETWEEN_KERN (genotype_kernels.py:27-83)."""
    from oracle.geno_tables import DD_POLY
    a, b = pp
    if a == b:
        p = pops[a]
        num = 16 * _geno_poly(DD_POLY, p.g) + p.D16 * p.D16
        return _gate(p.ns >= 4, num, 64 * _d4(p.ns))
    A, B = pops[a], pops[b]
    den = A.n * (A.n - 1) * B.n * (B.n - 1)
    return _gate(den > 0, A.D16 * B.D16, 64 * den)


def geno_dz(pp, pops):
    """Dz cases of compute_all_dz_geno (genotype_kernels.py:614-713)."""
    from oracle.geno_tables import DZ_QUARTIC
    i, j, k = pp
    if i == j == k:
        p = pops[i]
        num = 4 * _geno_poly(DZ_QUARTIC, p.g) + p.a * p.b * p.D16
        return _gate(p.ns >= 4, num, 8 * _d4(p.ns))
    if i == j:    # Dz(i,i,k): repeated i, singleton k
        I, K = pops[i], pops[k]
        return _fdiv(I.U16 * K.a, 8 * K.n * I.n * (I.n - 1) * (I.n - 2))
    if i == k:    # Dz(i,j,i): repeated i, singleton j
        I, J = pops[i], pops[j]
        return _fdiv(I.V16 * J.b, 8 * J.n * I.n * (I.n - 1) * (I.n - 2))
    if j == k:    # Dz(i,j,j)
        I, J = pops[i], pops[j]
        return _fdiv(I.D16 * J.W, 8 * J.n * (J.n - 1) * I.n * (I.n - 1))
    I, J, K = pops[i], pops[j], pops[k]
    return _fdiv(I.D16 * J.b * K.a, 8 * I.n * (I.n - 1) * J.n * K.n)


def _geno_shared_roles(i, j, k, l):
    if i == k:
        return i, j, l
    if i == l:
        return i, j, k
    if j == k:
        return j, i, l
    if j == l:
        return j, i, k
    return 0, 0, 0


def geno_pi2(pp, pops):
    """pi2 cases of compute_all_pi2_geno (genotype_kernels.py:722-886)."""
    from oracle.geno_tables import PI2_CORR
    i, j, k, l = pp
    cnt = {}
    for q in pp:
        cnt[q] = cnt.get(q, 0) + 1
    nu, mc = len(cnt), max(cnt.values())
    if nu == 1:
        p = pops[i]
        num = p.P2 * p.Q2 * p.S2 * p.R2 + _geno_poly(PI2_CORR, p.g)
        return _gate(p.ns >= 4, num, 16 * _d4(p.ns))
    if mc == 3:
        t = [q for q, v in cnt.items() if v == 3][0]
        s = [q for q, v in cnt.items() if v == 1][0]
        T, Sg = pops[t], pops[s]
        d = T.n * (T.n - 1) * (T.n - 2) * Sg.n
        if i == t and j == t:
            num = T.AQ3 * Sg.Q2 + T.AS3 * Sg.S2
        else:
            num = T.BP3 * Sg.P2 + T.BR3 * Sg.R2
        return _gate(d > 0, num, 32 * d)
    if i == j and k == l:
        I, K = pops[i], pops[k]
        return _fdiv(I.BL * K.BR, I.m * K.m)
    if i == j:
        I, K, L = pops[i], pops[k], pops[l]
        return _fdiv(I.BL * (K.Q2 * L.S2 + K.S2 * L.Q2), I.m * 8 * K.n * L.n)
    if k == l:
        I, J, K = pops[i], pops[j], pops[k]
        return _fdiv((I.P2 * J.R2 + I.R2 * J.P2) * K.BR, 8 * I.n * J.n * K.m)
    if (i == k and j == l) or (i == l and j == k):
        A, B = pops[i], pops[j]
        PQa, RSa, PSa, QRa, PRa = (A.P2 * A.Q2, A.R2 * A.S2, A.P2 * A.S2, A.Q2 * A.R2,
                                   A.P2 * A.R2)
        PQb, RSb, PSb, QRb = B.P2 * B.Q2, B.R2 * B.S2, B.P2 * B.S2, B.Q2 * B.R2
        Ta = A.R2 * (4 + A.X01 - A.X10)
        Ua = A.S2 * (2 + A.R2)
        num = (-2 * RSa * B.Q2 - A.X11 * PQb + RSa * PQb - 2 * A.R2 * PSb
               - PQa * B.X11 - RSa * B.X11 + PSa * B.X11 + QRa * B.X11
               - 2 * PRa * B.S2 + Ta * B.S2 + A.X11 * PSb + QRa * PSb
               + 2 * Ua * B.R2 - A.X01 * QRb + PSa * QRb
               - 2 * PSa * B.R2 - 2 * A.P2 * RSb + A.X01 * RSb + PQa * RSb
               + A.X11 * B.Bs + A.Bs * B.X11 - 4 * A.X11 * B.X11)
        d = A.n * (A.n - 1) * B.n * (B.n - 1)
        return _gate(d > 0, num, 64 * d)
    if nu == 3:
        s, a, b = _geno_shared_roles(i, j, k, l)
        Sg, A, B = pops[s], pops[a], pops[b]
        num = A.R2 * (Sg.C00 * B.S2 + Sg.C01 * B.Q2) + A.P2 * (Sg.C10 * B.S2 + Sg.C11 * B.Q2)
        return _fdiv(num, 16 * Sg.m * A.n * B.n)
    I, J, K, L = pops[i], pops[j], pops[k], pops[l]
    return _fdiv((I.P2 * J.R2 + I.R2 * J.P2) * (K.Q2 * L.S2 + K.S2 * L.Q2),
                 64 * I.n * J.n * K.n * L.n)


def geno_case_value(kind, pp, pops):
    if kind == "dd":
        return geno_dd(pp, pops)
    if kind == "dz":
        return geno_dz(pp, pops)
    return geno_pi2(pp, pops)


def geno_multi_pop_stats(counts_per_pop, n_valid_per_pop, specs=None):
    """(N, n_stats) float64 as compute_multi_pop_statistics_batch_geno
    (genotype_kernels.py:889-936)."""
    P = len(counts_per_pop)
    specs = stat_specs(P) if specs is None else specs
    pops = [GenoPop(c, nv) for c, nv in zip(counts_per_pop, n_valid_per_pop)]
    cache = {}
    out = np.zeros((len(np.asarray(counts_per_pop[0])), len(specs)), np.float64)
    for s, (_, calls) in enumerate(specs):
        acc = 0.0
        for w, kind, pp in calls:
            key = (kind, pp)
            if key not in cache:
                cache[key] = geno_case_value(kind, pp, pops)
            acc = acc + (cache[key] if (w == 1.0 and len(calls) == 1) else w * cache[key])
        out[:, s] = acc
    return out


def dd_geno_single(counts):
    """_DD_GENO_SINGLE_KERN on reference-order 9-way counts."""
    return geno_dd((0, 0), [GenoPop(counts)])


def sigma_d2_geno(counts):
    """DD / pi2 ratio of _SIGMA_D2_GENO_KERN (genotype_kernels.py:91-169):
    NaN where fewer than 4 individuals or the pi2 numerator is not positive."""
    from oracle.geno_tables import DD_POLY, PI2_CORR
    p = GenoPop(counts)
    dd = 16 * _geno_poly(DD_POLY, p.g) + p.D16 * p.D16
    pi = p.P2 * p.Q2 * p.S2 * p.R2 + _geno_poly(PI2_CORR, p.g)
    out = np.full(len(dd), np.nan)
    ok = (p.ns >= 4) & (pi > 0)
    out[ok] = dd[ok].astype(np.float64) / (4.0 * pi[ok].astype(np.float64))
    return out


def rogers_huff_r_counts(counts):
    """Rogers-Huff r from reference-order 9-way counts: exact integer moments
    of the individuals valid at both SNPs, one float64 division."""
    c = np.asarray(counts).astype(I64)
    ga = np.array([0, 0, 0, 1, 1, 1, 2, 2, 2], I64)
    gb = np.array([0, 1, 2, 0, 1, 2, 0, 1, 2], I64)
    n = c.sum(axis=1)
    si, sj = c @ ga, c @ gb
    sii, sjj, sij = c @ (ga * ga), c @ (gb * gb), c @ (ga * gb)
    cov = n * sij - si * sj
    den = (n * sii - si * si) * (n * sjj - sj * sj)
    out = np.full(len(c), np.nan)
    ok = den > 0
    out[ok] = cov[ok].astype(np.float64) / np.sqrt(den[ok].astype(np.float64))
    return out


def geno_binned_sums(geno, positions, pop_rows, bins, coords=None, max_dist=None,
                     pair_block=1_000_000, abs_sums=False):
    """Genotype-mode binned sums (moments_ld.py:248-343 with use_genotypes=True),
    on an already union-filtered dosage matrix; returns (sums, pair counts[, abs])."""
    pos = np.asarray(positions)
    coord = pos.astype(np.float64) if coords is None else np.asarray(coords, np.float64)
    bins = np.asarray(bins, np.float64)
    n_bins = len(bins) - 1
    P = len(pop_rows)
    if max_dist is None:
        max_dist = float(bins[-1])
    ii, jj = pairs_within_distance(pos, max_dist)
    specs = stat_specs(P)
    sums = np.zeros((n_bins, len(specs)))
    asums = np.zeros((n_bins, len(specs)))
    npairs = np.zeros(n_bins, np.int64)
    g = np.asarray(geno)
    subs = [g[np.asarray(r), :] for r in pop_rows]
    for s0 in range(0, len(ii), pair_block):
        ci, cj = ii[s0:s0 + pair_block], jj[s0:s0 + pair_block]
        d = np.abs(coord[cj] - coord[ci]) if coords is not None else (coord[cj] - coord[ci])
        b = bin_index(d, bins)
        keep = (b >= 0) & (b < n_bins)
        if not np.any(keep):
            continue
        ci, cj, b = ci[keep], cj[keep], b[keep]
        cs, nvs = [], []
        for sub in subs:
            c, nv = genotype_counts_for_pairs(sub, ci, cj)
            cs.append(c)
            nvs.append(nv)
        with np.errstate(divide="ignore", invalid="ignore"):
            st = geno_multi_pop_stats(cs, nvs, specs)
        for k in range(len(specs)):
            sums[:, k] += np.bincount(b, weights=st[:, k], minlength=n_bins)
            if abs_sums:
                asums[:, k] += np.bincount(b, weights=np.abs(st[:, k]), minlength=n_bins)
        npairs += np.bincount(b, minlength=n_bins)
    if abs_sums:
        return sums, npairs, asums
    return sums, npairs


def union_polymorphic(geno, pop_rows):
    """Variants kept by the genotype path's union filter (moments_ld.py:256-280)."""
    rows = sorted(set(int(i) for r in pop_rows for i in r))
    sub = np.asarray(geno)[rows]
    v = sub >= 0
    alt = np.where(v, sub, 0).astype(np.int64).sum(0)
    nv = v.sum(0)
    return (alt > 0) & (alt < 2 * nv) & (nv >= 2)


def geno_heterozygosity(geno, pop_rows):
    """H_i_j statistics (moments_ld.py:346-388), genotype mode."""
    g = np.asarray(geno)
    alt, ref, size = [], [], []
    for rws in pop_rows:
        sub = g[np.asarray(rws), :]
        v = sub >= 0
        a = np.where(v, sub, 0).astype(np.int64).sum(0).astype(np.float64)
        nh = 2.0 * v.sum(0).astype(np.float64)
        alt.append(a)
        ref.append(nh - a)
        size.append(nh)
    out = {}
    P = len(pop_rows)
    for i in range(P):
        for j in range(i, P):
            if i == j:
                out[f"H_{i}_{j}"] = float(np.sum(2.0 * ref[i] * alt[i] / (size[i] * (size[i] - 1))))
            else:
                out[f"H_{i}_{j}"] = float(np.sum((ref[i] * alt[j] + alt[i] * ref[j])
                                                 / (size[i] * size[j])))
    return out


# ---------------------------------------------------------------------------
# per-window sums and ZnS  (ld_statistics.py:250-341, 534-676)
# ---------------------------------------------------------------------------
def segregating(hap):
    """Sites with 0 < derived count < valid count (ld_statistics.py:266-271)."""
    h = np.asarray(hap)
    dac = np.maximum(h, 0).astype(np.int64).sum(0)
    nv = (h >= 0).sum(0)
    return (dac > 0) & (dac < nv)


def window_sums(hap, idx, win_begin, win_end):
    """(sums [n_win][6], counts [n_win][3]) as pgld_hap_window_sums: r^2,
    sigma_D^2 (projection), DD, Dz, pi2, naive r^2; pairs, r^2-defined, n >= 4.
    Window w covers idx[win_begin[w]:win_end[w]]."""
    h = np.asarray(hap)
    idx = np.asarray(idx, np.int64)
    dac_all = (h == 1).sum(0).astype(np.int64)
    nv_all = (h >= 0).sum(0).astype(np.int64)
    n_win = len(win_begin)
    sums = np.zeros((n_win, 6))
    cnts = np.zeros((n_win, 3), np.int64)
    for w in range(n_win):
        sel = idx[win_begin[w]:win_end[w]]
        m = len(sel)
        if m < 2:
            continue
        a, b = np.triu_indices(m, 1)
        ii, jj = sel[a], sel[b]
        c, nv = counts_for_pairs(h, ii, jj)
        n = c.astype(I64).sum(1)
        cnts[w, 0] = len(ii)
        r2 = r_squared(c, nv)
        ok = ~np.isnan(r2)
        sums[w, 0] = r2[ok].sum()
        cnts[w, 1] = ok.sum()
        p = Pop(c, n)
        dd_n, _ = dd_ii(p)
        pi_n, _ = pi2_iiii(p)
        four = n >= 4
        cnts[w, 2] = four.sum()
        with np.errstate(divide="ignore", invalid="ignore"):
            sig = np.where(four & (pi_n != 0), dd_n / np.where(pi_n != 0, pi_n, 1), 0.0)
        sums[w, 1] = sig.sum()
        sums[w, 2] = dd(c, None, n).sum()
        sums[w, 3] = dz(c, None, n).sum()
        sums[w, 4] = pi2(c, None, n).sum()
        pi_ = dac_all[ii] / np.maximum(nv_all[ii], 1)
        pj_ = dac_all[jj] / np.maximum(nv_all[jj], 1)
        pab = np.where(n > 0, c[:, 0] / np.maximum(n, 1), 0.0)
        D = pab - pi_ * pj_
        den = pi_ * (1 - pi_) * pj_ * (1 - pj_)
        with np.errstate(divide="ignore", invalid="ignore"):
            sums[w, 5] = np.where(den > 0, D * D / np.where(den > 0, den, 1), 0.0).sum()
    return sums, cnts


def zns_window(hap, s, e, projection=True):
    """ZnS of the SNPs [s, e) as _zns_from_precomputed (ld_statistics.py:595-676)."""
    h = np.asarray(hap)[:, s:e]
    seg = np.where(segregating(h))[0]
    if len(seg) < 2:
        return 0.0
    sums, cnts = window_sums(h, seg, [0], [len(seg)])
    if projection:
        return sums[0, 1] / cnts[0, 2] if cnts[0, 2] > 0 else 0.0
    return sums[0, 5] / cnts[0, 0]


# ---------------------------------------------------------------------------
# Kim and Nielsen's omega  (ld_statistics.py:734-862)
# ---------------------------------------------------------------------------
def pair_stat_matrix(hap, stat):
    """Square matrix of one window statistic over all site pairs of hap
    (zero diagonal): stat 1 = sigma_D^2 = DD / pi2 numerators (n >= 4 and a
    nonzero pi2 numerator, else 0; _build_sigma_d2_matrix,
    ld_statistics.py:734-758), 5 = naive r^2 of per-site frequencies
    (HaplotypeMatrix.pairwise_r2, haplotype_matrix.py:1138-1170)."""
    h = np.asarray(hap)
    m = h.shape[1]
    out = np.zeros((m, m))
    if m < 2:
        return out
    a, b = np.triu_indices(m, 1)
    c, nv = counts_for_pairs(h, a, b)
    n = c.astype(I64).sum(1)
    if stat == 1:
        p = Pop(c, n)
        dd_n, _ = dd_ii(p)
        pi_n, _ = pi2_iiii(p)
        with np.errstate(divide="ignore", invalid="ignore"):
            v = np.where((n >= 4) & (pi_n != 0), dd_n / np.where(pi_n != 0, pi_n, 1), 0.0)
    elif stat == 5:
        dac = (h == 1).sum(0).astype(np.int64)
        nvs = (h >= 0).sum(0).astype(np.int64)
        pi_ = dac[a] / np.maximum(nvs[a], 1)
        pj_ = dac[b] / np.maximum(nvs[b], 1)
        pab = np.where(n > 0, c[:, 0] / np.maximum(n, 1), 0.0)
        D = pab - pi_ * pj_
        den = pi_ * (1 - pi_) * pj_ * (1 - pj_)
        with np.errstate(divide="ignore", invalid="ignore"):
            v = np.where(den > 0, D * D / np.where(den > 0, den, 1), 0.0)
    else:
        raise ValueError("stat 1 or 5")
    out[a, b] = v
    out[b, a] = v
    return out


def omega_matrix(r2):
    """omega of a square LD matrix: for splits l = 3 .. m-2 the mean of the
    upper triangle within [0, l) and [l, m) over the mean across, maximised
    (the 2-D prefix-sum form of ld_statistics.py:813-862); 0.0 below 5 sites."""
    r2 = np.asarray(r2, np.float64)
    m = r2.shape[0]
    if m < 5:
        return 0.0
    S = np.cumsum(np.cumsum(np.triu(r2, 1), axis=0), axis=1)
    l = np.arange(3, m - 1)
    left = S[l - 1, l - 1]
    total = S[m - 1, m - 1]
    cross = S[l - 1, m - 1] - left
    right = total - left - cross
    n_within = l * (l - 1) // 2 + (m - l) * (m - l - 1) // 2
    n_cross = l * (m - l)
    valid = (n_within > 0) & (n_cross > 0) & (cross > 0)
    with np.errstate(divide="ignore", invalid="ignore"):
        mw = np.where(n_within > 0, (left + right) / n_within, 0.0)
        mc = np.where(n_cross > 0, cross / n_cross, 1.0)
        vals = np.where(valid, mw / mc, 0.0)
    return float(vals.max()) if vals.size else 0.0


def omega_hap(hap, estimator="sigma_d2", missing_data="include"):
    """omega of a haplotype matrix over its segregating sites (after dropping
    sites with missing calls for missing_data 'exclude'), ld_statistics.py:761-862."""
    h = np.asarray(hap)
    if missing_data == "exclude":
        h = h[:, (h < 0).sum(0) == 0]
    h = h[:, segregating(h)]
    if h.shape[1] < 2:
        return 0.0
    return omega_matrix(pair_stat_matrix(h, 1 if estimator == "sigma_d2" else 5))


# ---------------------------------------------------------------------------
# locate_unlinked  (haplotype_matrix.py:1172-1233)
# ---------------------------------------------------------------------------
def locate_unlinked(hap, size=100, step=20, threshold=0.1):
    """Sliding windows of `size` variants advanced by `step`; within a window,
    for active variants i < j in order, j is dropped when naive r^2(i, j) >
    threshold (naive r^2 of pair_stat_matrix column 5 on the active subset)."""
    h = np.asarray(hap)
    m = h.shape[1]
    loc = np.ones(m, dtype=bool)
    for ws in range(0, m, step):
        we = min(ws + size, m)
        act = np.where(loc[ws:we])[0] + ws
        if len(act) <= 1:
            continue
        r2 = pair_stat_matrix(h[:, act], 5)
        for a in range(len(act)):
            if not loc[act[a]]:
                continue
            for b in range(a + 1, len(act)):
                if loc[act[b]] and r2[a, b] > threshold:
                    loc[act[b]] = False
    return loc


# ---------------------------------------------------------------------------
# diploid dosage r^2, ZnS and omega of a GenotypeMatrix  (ld_statistics.py:973-1020)
# ---------------------------------------------------------------------------
def r2_matrix_diploid(geno):
    """Squared dosage correlation: per-site means over valid individuals,
    centred dosages with missing entries zeroed, cov = gn^T gn over
    sqrt(var_i var_j) (0 where the denominator is 0), zero diagonal."""
    g = np.asarray(geno)
    valid = (g >= 0).astype(np.float64)
    gc = np.where(g >= 0, g, 0).astype(np.float64)
    nv = valid.sum(0)
    mean = np.where(nv > 0, gc.sum(0) / np.maximum(nv, 1), 0.0)
    gn = (gc - mean[None, :]) * valid
    var = (gn ** 2).sum(0)
    cov = gn.T @ gn
    den = np.sqrt(np.outer(var, var))
    with np.errstate(divide="ignore", invalid="ignore"):
        r2 = np.where(den > 0, (cov / np.where(den > 0, den, 1)) ** 2, 0.0)
    np.fill_diagonal(r2, 0.0)
    return r2


def zns_diploid(geno, missing_data="include"):
    g = np.asarray(geno)
    if missing_data == "exclude":
        g = g[:, (g < 0).sum(0) == 0]
    m = g.shape[1]
    if m < 2:
        return 0.0
    r2 = r2_matrix_diploid(g)
    return float((r2.sum() - np.trace(r2)) / (m * (m - 1)))


def omega_diploid(geno, missing_data="include"):
    g = np.asarray(geno)
    if missing_data == "exclude":
        g = g[:, (g < 0).sum(0) == 0]
    return omega_matrix(r2_matrix_diploid(g))


# ---------------------------------------------------------------------------
# VCF GT reading  (haplotype_matrix.py:293-404 through allel.read_vcf)
# ---------------------------------------------------------------------------
def read_vcf_gt(text, samples=None):
    """(sample names, int8 haplotypes (2 n, M), int64 POS) of a VCF text.

    The layout of HaplotypeMatrix.from_vcf (haplotype_matrix.py:324-328): row
    k is the first allele of sample k, row n + k its second.  GT semantics of
    allel.read_vcf's calldata/GT: the first ':' subfield, alleles split at
    '/' or '|', '.' or empty -> -1, a haploid call's second allele -1; allele
    numbers above 127 are clipped to 127 (int8)."""
    names, gts, pos = None, [], []
    for line in text.split("\n"):
        line = line.rstrip("\r")
        if not line or line.startswith("##"):
            continue
        parts = line.split("\t")
        if line.startswith("#CHROM"):
            names = parts[9:]
            continue
        if line.startswith("#"):
            continue
        pos.append(int(parts[1]))
        row = []
        for g in parts[9:9 + len(names)]:
            gt = g.split(":")[0].replace("/", "|").split("|")

            def al(s):
                return -1 if s in (".", "") else min(int(s), 127)
            row.append((al(gt[0]), al(gt[1]) if len(gt) > 1 else -1))
        gts.append(row)
    cols = list(range(len(names))) if samples is None else [names.index(s) for s in samples]
    gt = np.asarray(gts, np.int8).reshape(len(gts), len(names), 2)[:, cols, :]
    n = len(cols)
    hap = np.empty((2 * n, gt.shape[0]), np.int8)
    hap[:n] = gt[:, :, 0].T
    hap[n:] = gt[:, :, 1].T
    return [names[c] for c in cols], hap, np.asarray(pos, np.int64)


def vcf_dosages(text):
    """(names, int8 dosages (n, M'), POS) of GenotypeMatrix.from_vcf
    (genotype_matrix.py:359-380): alt-allele counts of the sites allel's
    count_alleles().is_biallelic_01() keeps (alleles 0 and 1 both observed,
    nothing above 1), -1 where either allele is missing."""
    names, hap, pos = read_vcf_gt(text)
    n = len(names)
    gt = np.stack([hap[:n].T, hap[n:].T], axis=2)          # (M, n, 2)
    keep = np.array([(0 in set(r.ravel())) and (1 in set(r.ravel())) and r.max() <= 1
                     for r in gt])
    gt = gt[keep]
    g = gt.sum(axis=2).astype(np.int8)
    g[(gt < 0).any(axis=2)] = -1
    return names, g.T.copy(), pos[keep]


# ---------------------------------------------------------------------------
# mu_LD  (ld_statistics.py:865-918, diversity.py:1310-1360)
# ---------------------------------------------------------------------------
def cluster_haplotypes(h):
    """Greedy clustering with -1 as a wildcard: each haplotype joins the first
    cluster whose representative (its first member) it matches at every site
    where both are called; without missing data, identical rows."""
    h = np.asarray(h)
    n = h.shape[0]
    if not np.any(h < 0):
        seen, labels = {}, []
        for row in h:
            key = row.tobytes()
            labels.append(seen.setdefault(key, len(seen)))
        return labels
    reps, labels = [0], [0]
    for i in range(1, n):
        for c, r in enumerate(reps):
            both = (h[i] >= 0) & (h[r] >= 0)
            if np.all(h[i][both] == h[r][both]):
                labels.append(c)
                break
        else:
            reps.append(i)
            labels.append(len(reps) - 1)
    return labels


def mu_ld(hap, missing_data="include"):
    """Exclusivity of the haplotype patterns of the left and right halves of
    the variants (RAiSD's mu_LD)."""
    h = np.asarray(hap)
    if missing_data == "exclude":
        h = h[:, ~np.any(h < 0, axis=0)]
    if h.shape[1] < 2:
        return 0.0
    mid = h.shape[1] // 2
    lab_l = cluster_haplotypes(h[:, :mid])
    lab_r = cluster_haplotypes(h[:, mid:])
    l2r, r2l = {}, {}
    for a, b in zip(lab_l, lab_r):
        l2r.setdefault(a, set()).add(b)
        r2l.setdefault(b, set()).add(a)
    if not l2r or not r2l:
        return 0.0
    el = sum(1 for v in l2r.values() if len(v) == 1)
    er = sum(1 for v in r2l.values() if len(v) == 1)
    return float((el / len(l2r) + er / len(r2l)) / 2.0)


# --------------------------------------------------------------------------
# dense all-pairs outputs (HaplotypeMatrix, haplotype_matrix.py:1092-1317)
# --------------------------------------------------------------------------
def pairwise_ld_core(hap):
    """(D, p): D = pAB - p_i p_j with pAB = joint_11 / joint_n over the pair's
    valid haplotypes and p per site (haplotype_matrix.py:1092-1128)."""
    h = np.asarray(hap)
    valid = (h >= 0).astype(np.float64)
    clean = np.where(h >= 0, h, 0).astype(np.float64)
    n_valid = valid.sum(axis=0)
    with np.errstate(divide="ignore", invalid="ignore"):
        p = np.where(n_valid > 0, clean.sum(axis=0) / n_valid, 0.0)
        joint_n = valid.T @ valid
        joint_11 = clean.T @ clean
        p_ab = np.where(joint_n > 0, joint_11 / joint_n, 0.0)
    return p_ab - np.outer(p, p), p


def pairwise_ld_v(hap):
    """pairwise_LD_v (haplotype_matrix.py:1130-1136): D, zero diagonal."""
    D, _ = pairwise_ld_core(hap)
    np.fill_diagonal(D, 0)
    return D


def pairwise_r2(hap):
    """pairwise_r2, estimator 'r2' (haplotype_matrix.py:1138-1170)."""
    D, p = pairwise_ld_core(hap)
    den = np.outer(p * (1 - p), p * (1 - p))
    with np.errstate(divide="ignore", invalid="ignore"):
        r2 = np.where(den > 0, (D ** 2) / den, 0)
    np.fill_diagonal(r2, 0)
    return r2


def windowed_r_squared(hap, positions, bins, percentile=50):
    """windowed_r_squared, estimator 'r2' (haplotype_matrix.py:1235-1317):
    r^2 of every pair i < j from its joint counts (NaN where undefined),
    binned by pos[j] - pos[i] (digitize, right-open), numpy percentiles per
    bin; (result, counts)."""
    h = np.asarray(hap)
    m = h.shape[1]
    ii, jj = np.triu_indices(m, k=1)
    c, nv = counts_for_pairs(h, ii, jj)
    r2 = r_squared(c, nv)
    pos = np.asarray(positions)
    d = pos[jj] - pos[ii]
    bins = np.asarray(bins, np.float64)
    nb = len(bins) - 1
    b = np.digitize(d, bins) - 1
    ok = (b >= 0) & (b < nb) & ~np.isnan(r2)
    pct = np.atleast_1d(percentile)
    res = np.full((nb, len(pct)), np.nan)
    cnt = np.zeros(nb, dtype=int)
    for k in range(nb):
        sel = r2[ok & (b == k)]
        cnt[k] = sel.size
        if sel.size:
            for q, pc in enumerate(pct):
                res[k, q] = np.percentile(sel, pc)
    return (res[:, 0] if res.shape[1] == 1 else res), cnt

