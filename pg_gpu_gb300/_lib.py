"""ctypes binding of libpgld (include/pgld.h) and device-array plumbing.

Device memory, streams and dtype handling come from PyTorch; the compute is
in libpgld.  There is no CPU fallback: every entry point raises
``PgldError`` when the library or a CUDA device is unavailable.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpgld.so")

MAX_POPS = 4
F64, F32 = 0, 1
FORM_PLAIN, FORM_TC = 0, 1

# enum pgld_kind
DD_II, DD_IJ, DZ_III, DZ_IIJ, DZ_IJI, DZ_IJJ, DZ_IJK = range(7)
(PI2_IIII, PI2_TRIPLE, PI2_IIKK, PI2_IIKK_SYM, PI2_IIKL, PI2_IJKK, PI2_IJIJ, PI2_SHARED,
 PI2_ALLDIFF) = range(7, 16)
R, R2, DPRIME = 16, 17, 18
# genotype kinds
(G_DD_II, G_DD_IJ, G_DZ_III, G_DZ_IIJ, G_DZ_IJI, G_DZ_IJJ, G_DZ_IJK, G_PI2_IIII, G_PI2_IIIJ,
 G_PI2_IJII, G_PI2_IIKK, G_PI2_IIKL, G_PI2_IJKK, G_PI2_IJIJ, G_PI2_SHARED, G_PI2_ALLDIFF,
 G_SIGMA_D2, G_RH_R, G_RH_R2) = range(32, 51)


class PgldError(RuntimeError):
    """A libpgld call failed (status code and message from the library)."""

    def __init__(self, code, msg):
        super().__init__(f"libpgld error {code}: {msg}")
        self.code = code


class HapPanel(ctypes.Structure):
    _fields_ = [("n_pops", ctypes.c_int32),
                ("n_words", ctypes.c_int32 * MAX_POPS),
                ("planes", ctypes.c_void_p * MAX_POPS),
                ("valid", ctypes.c_void_p * MAX_POPS),
                ("n_snp", ctypes.c_int64)]


class Term(ctypes.Structure):
    _fields_ = [("stat", ctypes.c_int32), ("kind", ctypes.c_int32),
                ("pops", ctypes.c_int32 * 4), ("weight", ctypes.c_double)]


class PairCounts(ctypes.Structure):
    _fields_ = [("n_pops", ctypes.c_int32),
                ("counts", ctypes.c_void_p * MAX_POPS),
                ("counts_ld", ctypes.c_int64 * MAX_POPS),
                ("n_valid", ctypes.c_void_p * MAX_POPS),
                ("nvalid_ld", ctypes.c_int64 * MAX_POPS)]


class GenoPanel(ctypes.Structure):
    _fields_ = [("n_pops", ctypes.c_int32),
                ("n_words", ctypes.c_int32 * MAX_POPS),
                ("planes", ctypes.c_void_p * MAX_POPS),
                ("valid", ctypes.c_void_p * MAX_POPS),
                ("ext", ctypes.c_void_p * MAX_POPS),
                ("n_snp", ctypes.c_int64)]


_P = ctypes.c_void_p
_I32, _I64, _D = ctypes.c_int32, ctypes.c_int64, ctypes.c_double

_SIGS = {
    "pgld_version": ([], ctypes.c_int),
    "pgld_create": ([ctypes.c_int, ctypes.POINTER(_P)], ctypes.c_int),
    "pgld_destroy": ([_P], ctypes.c_int),
    "pgld_last_error": ([_P], ctypes.c_char_p),
    "pgld_device_status": ([_P, ctypes.POINTER(_I32), _P], ctypes.c_int),
    "pgld_pack_haplotypes": ([_P, _P, _I64, _I64, _P, _I32, _P, _P, _P, _P], ctypes.c_int),
    "pgld_hap_counts_pairs": ([_P, _P, _P, _I32, _I64, _P, _P, _I64, _P, _I64, _P, _P],
                              ctypes.c_int),
    "pgld_hap_tally": ([_P, _P, _P, _I32, _I64, _P, _P, _P], ctypes.c_int),
    "pgld_stat_terms": ([_I32, _P, _I32, ctypes.POINTER(_I32), ctypes.POINTER(_I32)],
                        ctypes.c_int),
    "pgld_hap_stats": ([_P, ctypes.POINTER(PairCounts), _I64, ctypes.POINTER(Term), _I32, _I32,
                        _P, _I32, _I64, _P], ctypes.c_int),
    "pgld_count_pairs_within": ([_P, _P, _I64, _D, ctypes.POINTER(_I64), _P, _P], ctypes.c_int),
    "pgld_pairs_within": ([_P, _P, _I64, _D, _I64, _I64, _P, _P, _I64, _P], ctypes.c_int),
    "pgld_hap_band_pairs": ([_P, ctypes.POINTER(HapPanel), _P, _D, _P, _P, _P, _I64, _I32, _P],
                            ctypes.c_int),
    "pgld_hap_binned_sums": ([_P, ctypes.POINTER(HapPanel), _P, _D, _P, _P, _I32, _P, _P, _I32,
                              _P], ctypes.c_int),
    "pgld_hap_binned_sums_range": ([_P, ctypes.POINTER(HapPanel), _P, _D, _P, _P, _I32, _I64,
                                    _I64, _P, _P, _I32, _P], ctypes.c_int),
    "pgld_hap_pairwise_ld": ([_P, _P, _I32, _I64, _P, _P, _I64, _P], ctypes.c_int),
    "pgld_pairs_by_bin": ([_P, _P, _I32, _P, _I64, _P, _P, _I32, _P, _P, _P], ctypes.c_int),
    "pgld_segment_kth": ([_P, _P, _P, _I32, _P, _I32, _P, _P], ctypes.c_int),
    "pgld_pack_genotypes": ([_P, _P, _I64, _I64, _P, _I32, _P, _P, _P, _P, _P], ctypes.c_int),
    "pgld_geno_counts_pairs": ([_P, _P, _P, _P, _I32, _I64, _P, _P, _I64, _P, _I64, _P, _P],
                               ctypes.c_int),
    "pgld_geno_stat_terms": ([_I32, _P, _I32, ctypes.POINTER(_I32), ctypes.POINTER(_I32)],
                             ctypes.c_int),
    "pgld_geno_stats": ([_P, ctypes.POINTER(PairCounts), _I64, ctypes.POINTER(Term), _I32, _I32,
                         _P, _I32, _I64, _P], ctypes.c_int),
    "pgld_geno_band_pairs": ([_P, ctypes.POINTER(GenoPanel), _P, _D, _P, _P, _P, _I32, _I64, _I32,
                              _P],
                             ctypes.c_int),
    "pgld_geno_binned_sums": ([_P, ctypes.POINTER(GenoPanel), _P, _D, _P, _P, _I32, _P, _P, _P],
                              ctypes.c_int),
    "pgld_geno_binned_sums_form": ([_P, ctypes.POINTER(GenoPanel), _P, _D, _P, _P, _I32, _P, _P,
                                    _I32, _P], ctypes.c_int),
    "pgld_hap_window_sums": ([_P, ctypes.POINTER(HapPanel), _P, _I64, _P, _P, _I32, _P, _P, _I32,
                              _P],
                             ctypes.c_int),
    "pgld_hap_binned_sums_noalloc": ([ctypes.c_int, ctypes.POINTER(HapPanel), _P, _D, _P, _P, _I32,
                                      _P, _P, _P], ctypes.c_int),
    "pgld_noalloc_status": ([ctypes.c_int, ctypes.POINTER(_I32)], ctypes.c_int),
    "pgld_hap_window_snp_sums": ([_P, ctypes.POINTER(HapPanel), _P, _I64, _P, _P, _I32, _P, _I32,
                                  _P, _P, _I64, _P],
                                 ctypes.c_int),
    "pgld_prune_unlinked": ([_P, _P, _P, _I64, _I32, _I32, _D, _P], ctypes.c_int),
    "pgld_set_kernel_timing": ([_P, _I32], ctypes.c_int),
    "pgld_set_test_fault": ([_P, _I32], ctypes.c_int),
    "pgld_set_tc_config": ([_P, _I32, _I32], ctypes.c_int),
    "pgld_kernel_times": ([_P, _P, _I32, ctypes.POINTER(_I32)], ctypes.c_int),
    "pgld_tc_mma_rate": ([_P, _I32, _I64, _I32, ctypes.POINTER(ctypes.c_float),
                          ctypes.POINTER(_D), _P], ctypes.c_int),
    "pgld_vcf_scan": ([_P, _I64, _P, _P], ctypes.c_int),
    "pgld_vcf_parse_gt": ([_P, _I64, _I32, _I64, _P, _I32, _P, _P], ctypes.c_int),
    "pgld_vcf_pack_gt": ([_P, _I64, _I32, _I64, _P, _P, _I32, _P, _P, _P, _P, _P], ctypes.c_int),
}

_lib = None
_lock = threading.RLock()
_handles = {}


def lib():
    """The loaded libpgld (raises PgldError if it was not built)."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(LIB_PATH):
                    raise PgldError(-4, f"{LIB_PATH} is missing: run __graft_entry__.build() "
                                        "or python -m pg_gpu_gb300._build")
                L = ctypes.CDLL(LIB_PATH)
                for name, (args, res) in _SIGS.items():
                    f = getattr(L, name, None)
                    if f is None:
                        continue
                    f.argtypes = args
                    f.restype = res
                _lib = L
    return _lib


def exported_symbols():
    return [n for n in _SIGS]


def check(rc, h=None):
    if rc != 0:
        msg = lib().pgld_last_error(h)
        raise PgldError(rc, msg.decode() if msg else "")


def handle(device=None):
    """The per-device libpgld handle of this process."""
    import torch
    if not torch.cuda.is_available():
        raise PgldError(-2, "no CUDA device: libpgld has no CPU path")
    dev = torch.cuda.current_device() if device is None else int(device)
    h = _handles.get(dev)
    if h is None:
        lib()
        with _lock:
            h = _handles.get(dev)
            if h is None:
                p = ctypes.c_void_p()
                check(lib().pgld_create(dev, ctypes.byref(p)))
                h = p.value
                _handles[dev] = h
    return h


def stream_ptr():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


# --------------------------------------------------------------------------
# device arrays
# --------------------------------------------------------------------------
def as_device(x, dtype=None):
    """A contiguous CUDA torch tensor for x (torch, numpy, cupy, lists)."""
    import torch
    tdt = None
    if dtype is not None:
        tdt = {np.int8: torch.int8, np.int32: torch.int32, np.int64: torch.int64,
               np.float64: torch.float64, np.float32: torch.float32,
               np.uint32: torch.int32}[np.dtype(dtype).type]
    if isinstance(x, torch.Tensor):
        t = x
    elif hasattr(x, "__cuda_array_interface__"):
        t = torch.as_tensor(x, device="cuda")
    else:
        t = torch.as_tensor(np.asarray(x))
    if not t.is_cuda:
        t = t.to("cuda", non_blocking=False)
    if tdt is not None and t.dtype != tdt:
        t = t.to(tdt)
    return t.contiguous()
