"""Accessible-region filtering of variants for the LD path.

The reference attaches an accessible mask built from a BED file and hides the
variants at inaccessible positions before computing LD statistics
(moments_ld.py:99-101, 136-137, 159-160; accessible.py:132-197 parses the BED).
Here the mask is applied as a variant filter: BED intervals are 0-based
half-open, so (start, end) covers the 1-based positions start + 1 .. end.
"""
from __future__ import annotations

import numpy as np


def parse_bed(path, chrom=None):
    """[(chrom, start, end)] of a BED file (tab- or space-separated; lines
    starting with '#', 'track' or 'browser' skipped), optionally one
    chromosome (accessible.py:132-164)."""
    out = []
    with open(path) as f:
        for line in f:
            line = line.strip()
            if not line or line.startswith(("#", "track", "browser")):
                continue
            fields = line.split("\t")
            if len(fields) < 3:
                fields = line.split()
            if len(fields) < 3:
                continue
            c, s, e = fields[0], int(fields[1]), int(fields[2])
            if chrom is None or c == chrom:
                out.append((c, s, e))
    return out


def _intervals(bed, chrom):
    """The BED file's (path) or interval list's intervals of chrom; a file
    without any for the chromosome raises ValueError, as the reference's
    resolve_accessible_mask does (accessible.py:232-235)."""
    if isinstance(bed, (str, bytes)) or hasattr(bed, "__fspath__"):
        iv = parse_bed(bed, chrom)
        if not iv:
            raise ValueError(f"No BED intervals found for chrom={chrom!r} in {bed}")
        return iv
    return [t for t in bed if chrom is None or t[0] == chrom]


def _merged(iv):
    """Merged 1-based closed intervals [s + 1, e] as (starts, ends) arrays."""
    se = np.array(sorted((s + 1, e) for _, s, e in iv if e > s), dtype=np.int64).reshape(-1, 2)
    if se.size == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    starts, ends = [se[0, 0]], [se[0, 1]]
    for s, e in se[1:]:
        if s <= ends[-1] + 1:
            ends[-1] = max(ends[-1], e)
        else:
            starts.append(s)
            ends.append(e)
    return np.asarray(starts), np.asarray(ends)


def accessible_variants(positions, bed, chrom=None):
    """Boolean array: True where a 1-based position lies in an interval of the
    BED file (path) or interval list [(chrom, start, end)]."""
    iv = _intervals(bed, chrom)
    pos = np.asarray(positions, dtype=np.int64)
    starts, ends = _merged(iv)
    if starts.size == 0 or pos.size == 0:
        return np.zeros(pos.shape, dtype=bool)
    k = np.searchsorted(starts, pos, side="right") - 1
    return (k >= 0) & (pos <= ends[np.maximum(k, 0)])


def accessible_base_count(bed, chrom=None, start=None, stop=None):
    """Number of accessible bases (1-based) in [start, stop] (both None: all
    of the BED's), the per-base denominator the reference's
    set_accessible_mask stores as n_total_sites (haplotype_matrix.py:
    196-205)."""
    starts, ends = _merged(_intervals(bed, chrom))
    if starts.size == 0:
        return 0
    lo = starts if start is None else np.maximum(starts, int(start))
    hi = ends if stop is None else np.minimum(ends, int(stop))
    return int(np.maximum(hi - lo + 1, 0).sum())
