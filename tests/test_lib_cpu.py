"""Host-side checks of libpgld that need no GPU.

* the shared library loads and exports every entry point include/pgld.h
  declares;
* the C++ moments statistic table equals the Python host table and the
  oracle's restatement of generate_stat_specs;
* entry points fail with a status code (not a crash) on bad arguments and
  when no device is present.
"""
import ctypes
import os
import re

import pytest

from tests.conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from pg_gpu_gb300 import _build, _lib
    if not os.path.exists(_lib.LIB_PATH):
        _build.build()
    return _lib.lib()


def header_symbols():
    with open(os.path.join(ROOT, "include", "pgld.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(pgld_\w+)\(", text, re.M)))


def test_library_exports_every_declared_symbol(lib):
    syms = header_symbols()
    assert len(syms) >= 14
    for s in syms:
        assert hasattr(lib, s), f"{s} declared in include/pgld.h but not exported"
    from pg_gpu_gb300 import _lib
    assert set(syms) <= set(_lib.exported_symbols()), "binding lacks a declared entry point"


def _c_terms(lib, P):
    from pg_gpu_gb300 import _lib as L
    nt, ns = ctypes.c_int32(), ctypes.c_int32()
    assert lib.pgld_stat_terms(P, None, 0, ctypes.byref(nt), ctypes.byref(ns)) == 0
    arr = (L.Term * nt.value)()
    assert lib.pgld_stat_terms(P, arr, nt.value, ctypes.byref(nt), ctypes.byref(ns)) == 0
    return ns.value, [(t.stat, t.kind, tuple(t.pops), t.weight) for t in arr]


def test_stat_tables_agree(lib):
    from oracle import ld_oracle as O
    from pg_gpu_gb300 import ld_pipeline
    for P in (1, 2, 3, 4):
        ns, ct = _c_terms(lib, P)
        assert ns == len(O.ld_names(P)) == len(ld_pipeline.ld_names(P))
        assert ld_pipeline.ld_names(P) == O.ld_names(P)
        assert ld_pipeline.generate_stat_specs(P) == O.stat_specs(P)
        py = ld_pipeline.specs_to_terms(ld_pipeline.generate_stat_specs(P))
        assert len(py) == len(ct)
        for (s, k, roles, w), (cs, ck, cp, cw) in zip(py, ct):
            assert (s, k, w) == (cs, ck, cw)
            assert tuple(roles) == cp[:len(roles)]
    assert lib.pgld_stat_terms(5, None, 0, None, None) < 0


def test_genotype_stat_tables_agree(lib):
    from pg_gpu_gb300 import _geno, _lib as L, ld_pipeline
    for P in (1, 2, 3, 4):
        nt, ns = ctypes.c_int32(), ctypes.c_int32()
        assert lib.pgld_geno_stat_terms(P, None, 0, ctypes.byref(nt), ctypes.byref(ns)) == 0
        arr = (L.Term * nt.value)()
        assert lib.pgld_geno_stat_terms(P, arr, nt.value, ctypes.byref(nt), ctypes.byref(ns)) == 0
        ct = [(t.stat, t.kind, tuple(t.pops), t.weight) for t in arr]
        py = _geno.specs_to_terms(ld_pipeline.generate_stat_specs(P))
        assert ns.value == len(ld_pipeline.ld_names(P)) and len(py) == len(ct)
        for (s, k, roles, w), (cs, ck, cp, cw) in zip(py, ct):
            assert (s, k, w) == (cs, ck, cw) and tuple(roles) == cp[:len(roles)]
            assert L.G_DD_II <= ck <= L.G_PI2_ALLDIFF


def test_errors_are_status_codes(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("checks the no-device path")
    h = ctypes.c_void_p()
    rc = lib.pgld_create(0, ctypes.byref(h))
    assert rc < 0 and h.value is None
    assert lib.pgld_last_error(None)
    assert lib.pgld_create(0, None) < 0
    # NULL handle is rejected before any device work
    assert lib.pgld_hap_counts_pairs(None, None, None, 1, 1, None, None, 1, None, 4, None,
                                     None) < 0
    assert b"NULL handle" in lib.pgld_last_error(None)


def test_host_api_refuses_without_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("checks the no-device path")
    import numpy as np
    from pg_gpu_gb300 import ld_pipeline
    from pg_gpu_gb300._lib import PgldError
    with pytest.raises((PgldError, RuntimeError, AssertionError)):
        ld_pipeline.compute_counts_for_pairs(np.zeros((4, 3), np.int8), [0], [1])


def test_loader_lock_is_reentrant():
    """handle() loads the library while holding the loader lock."""
    import threading
    from pg_gpu_gb300 import _lib
    _lib.lib()
    saved = _lib._lib
    _lib._lib = None
    done = []

    def run():
        with _lib._lock:
            _lib.lib()
        done.append(True)

    t = threading.Thread(target=run, daemon=True)
    t.start()
    t.join(20)
    if not done:
        _lib._lib = saved
    assert done, "library loader deadlocked under its own lock"
