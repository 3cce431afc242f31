"""The float32 statistic epilogue of the band kernels, built for the host.

pg_gpu_gb300/csrc/pgld_epilogue.cuh is compiled with g++ and evaluated on
count tables that cover empty and tiny populations, missing data (n below the
sum of the counts' planes) and 1,000 - 2,000 haplotypes per population; each
float32 statistic must lie within 1e-6 relative of the float64 oracle (where
the oracle value exceeds 1e-30 in magnitude) and be exactly 0 where the oracle
is 0 by the n thresholds.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle import ld_oracle as O
from tests.conftest import ROOT

SRC = os.path.join(ROOT, "tests", "native", "epilogue_check.cpp")


@pytest.fixture(scope="module")
def check_lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("epi") / "epi.so")
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-o", so, SRC])
    L = ctypes.CDLL(so)
    L.pgld_check_stats.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_int] * 2 + [ctypes.c_void_p]
    L.pgld_check_stats2.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_int] * 2 + [ctypes.c_void_p]
    return L


def _tables(rng, N, nmax):
    out = []
    for _ in range(N):
        row = []
        for _p in range(2):
            n = int(rng.integers(0, nmax + 1))
            pr = rng.dirichlet([0.3, 0.3, 0.3, 0.3])
            c = rng.multinomial(n, pr)
            row += list(c)
        out.append(row)
    c = np.array(out, np.int32)
    # a few edge rows: empty, tiny, monomorphic, perfect LD
    c[:6] = [[0] * 8, [1, 0, 0, 0, 1, 0, 0, 0], [2, 1, 0, 0, 1, 1, 1, 0],
             [0, 0, 500, 500, 300, 0, 0, 700], [500, 0, 0, 500, 0, 400, 600, 0],
             [3, 0, 0, 1, 0, 2, 1, 0]]
    return c


@pytest.mark.parametrize("nmax", [6, 60, 1000, 2048])
def test_fast_epilogue_within_1e6_of_oracle(check_lib, nmax):
    rng = np.random.default_rng(nmax)
    N = 20000
    c = _tables(rng, N, nmax)
    sums = np.stack([c[:, :4].sum(1), c[:, 4:].sum(1)], 1)
    # missing data: n_valid may exceed the allele counts' sum only with other codes;
    # with 0/1/-1 data n = sum of counts, which is what the band kernels use
    nvalid = sums.astype(np.int32)
    for P in (1, 2):
        out = np.zeros((N, 3 if P == 1 else 15), np.float32)
        check_lib.pgld_check_stats(c.ctypes.data, np.ascontiguousarray(nvalid).ctypes.data, N,
                                   P, out.ctypes.data)
        ref = O.multi_pop_stats([c[:, 4 * q:4 * q + 4] for q in range(P)],
                                [nvalid[:, q] for q in range(P)])
        got = out.astype(np.float64)
        zero = ref == 0
        assert np.all(got[zero] == 0)
        m = np.abs(ref) > 1e-30
        rel = np.abs(got[m] - ref[m]) / np.abs(ref[m])
        assert rel.max() <= 1e-6, (P, nmax, rel.max())


@pytest.mark.parametrize("nmax", [6, 1000, 2048])
def test_packed_epilogue_equals_scalar(check_lib, nmax):
    """The float2 (two pairs per instruction) epilogue is bit-identical per lane."""
    rng = np.random.default_rng(100 + nmax)
    N = 5000
    c = _tables(rng, N, nmax)
    nvalid = np.ascontiguousarray(np.stack([c[:, :4].sum(1), c[:, 4:].sum(1)], 1).astype(np.int32))
    for P in (1, 2):
        S = 3 if P == 1 else 15
        a = np.zeros((N, S), np.float32)
        b = np.zeros((N, S), np.float32)
        check_lib.pgld_check_stats(c.ctypes.data, nvalid.ctypes.data, N, P, a.ctypes.data)
        check_lib.pgld_check_stats2(c.ctypes.data, nvalid.ctypes.data, N, P, b.ctypes.data)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
