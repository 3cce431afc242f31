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


def accessible_variants(positions, bed, chrom=None):
    """Boolean array: True where a 1-based position lies in an interval of the
    BED file (path) or interval list [(chrom, start, end)]."""
    iv = parse_bed(bed, chrom) if isinstance(bed, (str, bytes)) or hasattr(bed, "__fspath__") \
        else [t for t in bed if chrom is None or t[0] == chrom]
    pos = np.asarray(positions, dtype=np.int64)
    if not iv or pos.size == 0:
        return np.zeros(pos.shape, dtype=bool)
    # merge the intervals (as 1-based closed [s + 1, e]) and test membership
    se = np.array(sorted((s + 1, e) for _, s, e in iv if e > s), dtype=np.int64).reshape(-1, 2)
    if se.size == 0:
        return np.zeros(pos.shape, dtype=bool)
    starts, ends = [se[0, 0]], [se[0, 1]]
    for s, e in se[1:]:
        if s <= ends[-1] + 1:
            ends[-1] = max(ends[-1], e)
        else:
            starts.append(s)
            ends.append(e)
    starts = np.asarray(starts)
    ends = np.asarray(ends)
    k = np.searchsorted(starts, pos, side="right") - 1
    return (k >= 0) & (pos <= ends[np.maximum(k, 0)])
