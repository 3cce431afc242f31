"""The centred-moment form of the single-population genotype estimators
(pg_gpu_gb300/csrc/pgld_geno_mom.cuh), built for the host with g++: the int64
numerators of DD, Dz and pi2 must equal, exactly, the reference's polynomials
in the nine counts (the oracle's monomial tables of _DD_GENO_SINGLE_KERN,
_DZ_III_KERN and _PI2_IIII_KERN, genotype_kernels.py:27-71, 235-279,
364-398) scaled by 16, 4 and 1; the Rogers-Huff moments must equal the raw
dosage moments (ld_statistics.py:410-443); the counts must come back from the
moments unchanged."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle import ld_oracle as O
from oracle.geno_tables import DD_POLY, DZ_QUARTIC, PI2_CORR
from tests.conftest import ROOT

SRC = os.path.join(ROOT, "tests", "native", "geno_mom_check.cpp")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("gmom") / "gmom.so")
    subprocess.check_call(["g++", "-O2", "-shared", "-fPIC", "-o", so, SRC])
    L = ctypes.CDLL(so)
    L.pgld_check_geno_mom.argtypes = [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 3
    return L


def _counts(rng):
    rows = [rng.integers(0, 4, (4000, 9)), rng.integers(0, 60, (4000, 9)),
            rng.multinomial(1000, [0.3, 0.05, 0.02, 0.1, 0.2, 0.03, 0.05, 0.1, 0.15], 4000),
            rng.multinomial(32767, [1 / 9] * 9, 500),
            # one dosage class only, and the largest population: every individual 2/2
            np.array([[0] * 8 + [32767], [32767] + [0] * 8, [0, 0, 0, 0, 32767, 0, 0, 0, 0]]),
            np.zeros((1, 9), np.int64), np.eye(9, dtype=np.int64) * 3]
    return np.ascontiguousarray(np.concatenate(rows).astype(np.int32))


def test_moment_numerators_equal_reference_polynomials(lib):
    c = _counts(np.random.default_rng(11))
    N = len(c)
    mom = np.zeros((N, 9), np.int32)
    back = np.zeros((N, 9), np.int32)
    num = np.zeros((N, 6), np.int64)
    lib.pgld_check_geno_mom(c.ctypes.data, N, mom.ctypes.data, back.ctypes.data, num.ctypes.data)
    assert np.array_equal(back, c)
    p = O.GenoPop(c)
    g = p.g.astype(object)

    def poly(t):
        return sum(co * g[a] * g[b] * g[k] for co, (a, b, k) in t)
    D16 = p.D16.astype(object)
    ref_dd = 16 * poly(DD_POLY) + D16 * D16
    ref_dz = 4 * poly(DZ_QUARTIC) + p.a.astype(object) * p.b.astype(object) * D16
    ref_pi2 = (p.P2.astype(object) * p.Q2.astype(object) * p.S2.astype(object)
               * p.R2.astype(object) + poly(PI2_CORR))
    got = num.astype(object)
    assert all(ref_dd == 16 * got[:, 0])
    assert all(ref_dz == 4 * got[:, 1])
    assert all(ref_pi2 == got[:, 2])
    n = c.sum(1).astype(object)
    assert all(got[:, 3] == n * (n - 1) * (n - 2) * (n - 3))
    # Rogers-Huff from raw dosages
    a = np.repeat(np.arange(3), 3)
    b = np.tile(np.arange(3), 3)
    cc = c.astype(object)
    si, sj = cc @ a, cc @ b
    sij, sii, sjj = cc @ (a * b), cc @ (a * a), cc @ (b * b)
    cov = n * sij - si * sj
    assert all(got[:, 4] == cov * cov)
    assert all(got[:, 5] == (n * sii - si * si) * (n * sjj - sj * sj))


def test_moment_statistics_match_oracle_values(lib):
    """The float64 values num / den agree with the oracle's genotype DD / Dz /
    pi2 (which evaluate the reference polynomials) wherever n >= 4; rows up to
    8,000 individuals, where the oracle's own int64 D16^2 cannot overflow."""
    c = _counts(np.random.default_rng(12))
    c = np.ascontiguousarray(c[c.sum(1) <= 8000])
    N = len(c)
    mom = np.zeros((N, 9), np.int32)
    back = np.zeros((N, 9), np.int32)
    num = np.zeros((N, 6), np.int64)
    lib.pgld_check_geno_mom(c.ctypes.data, N, mom.ctypes.data, back.ctypes.data, num.ctypes.data)
    pops = [O.GenoPop(c)]
    ok = c.sum(1) >= 4
    d4 = num[:, 3].astype(np.float64)
    for k, (fn, pp, scale) in enumerate([(O.geno_dd, (0, 0), 4), (O.geno_dz, (0, 0, 0), 2),
                                         (O.geno_pi2, (0, 0, 0, 0), 16)]):
        ref = fn(pp, pops)
        val = np.where(ok, num[:, k].astype(np.float64) / np.where(ok, scale * d4, 1.0), 0.0)
        np.testing.assert_allclose(val, ref, rtol=1e-12, atol=0)
