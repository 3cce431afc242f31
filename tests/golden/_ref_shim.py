"""Run the reference pg_gpu LD modules on the CPU, for fixture generation only.

The reference (kr-colab/pg_gpu) is Python on CuPy.  This module provides a
numpy-backed stand-in for the ``cupy`` module so the reference's own array
code (``ld_pipeline.py``, ``ld_statistics.py``, ``haplotype_kernels.py``,
``genotype_kernels.py``, ``ld_statistics_genotype.py``) runs unmodified on
the host.  ``cupy.RawKernel`` bodies are plain CUDA C; they are compiled here
as host C++ (one loop iteration per CUDA thread) with g++ so the reference's
kernel-only cases produce real reference outputs too.

Only ``tests/golden/make_golden.py`` imports this, in a container where the
reference checkout exists (``PGLD_REFERENCE`` or ``/root/reference``).  Nothing
on the GPU path or in the committed tests reads the reference at run time.
"""
import ctypes
import hashlib
import importlib.util
import os
import re
import subprocess
import sys
import tempfile
import types

import numpy as np

REF_ROOT = os.environ.get("PGLD_REFERENCE", "/root/reference")


class GArr(np.ndarray):
    """ndarray with CuPy's ``.get()`` (device→host copy) as identity."""

    def get(self):
        return np.asarray(self)

    def __getitem__(self, key):
        r = super().__getitem__(key)
        if isinstance(r, np.generic):
            return np.asarray(r).view(GArr)
        return r

    def __array_wrap__(self, obj, context=None, return_scalar=False):
        r = super().__array_wrap__(obj, context, False)
        return r


def _wrap(x):
    if isinstance(x, np.generic):
        return np.asarray(x).view(GArr)
    if isinstance(x, np.ndarray) and not isinstance(x, GArr):
        return x.view(GArr)
    return x


def _wrapped(fn):
    def inner(*a, **k):
        return _wrap(fn(*a, **k))
    return inner


# --------------------------------------------------------------------------
# RawKernel -> host C++ loop
# --------------------------------------------------------------------------
_HOST_PRELUDE = r'''
#include <cmath>
#include <cstdint>
struct pgld_dim3 { long long x, y, z; };
static pgld_dim3 blockIdx = {0, 0, 0};
static pgld_dim3 threadIdx = {0, 0, 0};
static pgld_dim3 blockDim = {1, 1, 1};
#define __global__
#define __restrict__
#define __device__
#define nan(x) NAN
'''

_TYPE_MAP = {
    "int": ctypes.c_int,
    "long long": ctypes.c_longlong,
    "double": ctypes.c_double,
    "float": ctypes.c_float,
}


def _split_params(sig):
    params = []
    depth = 0
    cur = ""
    for ch in sig:
        if ch == "," and depth == 0:
            params.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        params.append(cur)
    return [p.strip() for p in params]


class RawKernel:
    _cache = {}

    def __init__(self, code, name, options=()):
        self.code = code
        self.name = name
        m = re.search(r"void\s+" + re.escape(name) + r"\s*\((.*?)\)\s*\{", code, re.S)
        if not m:
            raise RuntimeError("cannot parse kernel signature")
        params = _split_params(m.group(1))
        self.param_names = []
        self.argtypes = []
        for p in params:
            p = p.replace("__restrict__", "").replace("const", "").strip()
            is_ptr = "*" in p
            pname = re.split(r"[\s\*]+", p)[-1]
            ptype = p[: p.rfind(pname)].replace("*", "").strip()
            self.param_names.append(pname)
            if is_ptr:
                self.argtypes.append(ctypes.c_void_p)
            else:
                self.argtypes.append(_TYPE_MAP[" ".join(ptype.split())])
        self._fn = None

    def _compile(self):
        key = hashlib.sha1(self.code.encode()).hexdigest()[:16]
        if key in RawKernel._cache:
            return RawKernel._cache[key]
        src = _HOST_PRELUDE + self.code + "\n"
        src += 'extern "C" void pgld_host_launch(long long nthreads'
        m = re.search(r"void\s+" + re.escape(self.name) + r"\s*\((.*?)\)\s*\{", self.code, re.S)
        src += ", " + m.group(1) + ") {\n"
        src += "  for (long long t = 0; t < nthreads; ++t) { blockIdx.x = t; "
        src += self.name + "(" + ", ".join(self.param_names) + "); }\n}\n"
        d = tempfile.mkdtemp(prefix="pgld_rawk_")
        cpp = os.path.join(d, "k.cpp")
        so = os.path.join(d, "k.so")
        with open(cpp, "w") as f:
            f.write(src)
        subprocess.check_call(["g++", "-O1", "-shared", "-fPIC", "-o", so, cpp])
        lib = ctypes.CDLL(so)
        fn = lib.pgld_host_launch
        fn.argtypes = [ctypes.c_longlong] + self.argtypes
        fn.restype = None
        RawKernel._cache[key] = fn
        return fn

    def __call__(self, grid, block, args):
        fn = self._compile()
        nthreads = int(grid[0]) * int(block[0])
        cargs = []
        keep = []
        for a, t in zip(args, self.argtypes):
            if t is ctypes.c_void_p:
                arr = np.asarray(a)
                if not arr.flags.c_contiguous:
                    raise RuntimeError("non-contiguous kernel argument")
                keep.append(arr)
                cargs.append(arr.ctypes.data)
            else:
                cargs.append(t(a.item() if hasattr(a, "item") else a))
        fn(nthreads, *cargs)


# --------------------------------------------------------------------------
# fake cupy module
# --------------------------------------------------------------------------
def _make_cupy():
    cp = types.ModuleType("cupy")
    cp.ndarray = GArr
    for name in ("int8", "int32", "int64", "float64", "float32", "uint8", "bool_",
                 "nan", "inf", "newaxis", "float16"):
        setattr(cp, name, getattr(np, name))
    for name in ("array", "asarray", "zeros", "ones", "empty", "arange", "sum", "any",
                 "all", "stack", "concatenate", "where", "maximum", "minimum",
                 "searchsorted", "cumsum", "ascontiguousarray", "digitize", "outer",
                 "sqrt", "zeros_like", "ones_like", "empty_like", "isnan", "abs",
                 "triu_indices", "full", "mean", "diff", "unique", "clip", "log",
                 "exp", "isfinite", "column_stack", "vstack", "hstack", "repeat",
                 "tile", "nonzero", "argsort", "sort", "count_nonzero", "fill_diagonal",
                 "asnumpy", "nansum", "nanmean", "dot", "matmul", "einsum", "bincount",
                 "logical_and", "logical_or", "logical_not", "floor", "ceil", "round",
                 "minimum", "maximum", "prod", "cumprod", "max", "min", "float_", "triu",
                 "tril", "argmax", "trace"):
        if hasattr(np, name):
            fn = getattr(np, name)
            setattr(cp, name, _wrapped(fn) if callable(fn) else fn)
    cp.asnumpy = lambda a: np.asarray(a)
    cp.get_array_module = lambda *a: cp
    cp.add = types.SimpleNamespace(at=np.add.at)
    cp.RawKernel = RawKernel

    class _Dev:
        mem_info = (8 << 30, 16 << 30)

        def __init__(self, *a):
            pass

    class _Stream:
        def synchronize(self):
            pass

    cp.cuda = types.SimpleNamespace(
        Device=_Dev,
        Stream=types.SimpleNamespace(null=_Stream()),
        runtime=types.SimpleNamespace(getDeviceCount=lambda: 1),
    )
    cp.random = np.random
    return cp


_LOADED = {}


def load_reference_modules():
    """Import the reference's LD modules from REF_ROOT under a stub package."""
    if _LOADED:
        return _LOADED
    if not os.path.isdir(os.path.join(REF_ROOT, "pg_gpu")):
        raise RuntimeError(f"reference checkout not found at {REF_ROOT}")
    sys.modules["cupy"] = _make_cupy()
    pkg = types.ModuleType("pg_gpu")
    pkg.__path__ = [os.path.join(REF_ROOT, "pg_gpu")]
    sys.modules["pg_gpu"] = pkg
    for mod in ("ld_pipeline", "haplotype_kernels", "ld_statistics",
                "genotype_kernels", "ld_statistics_genotype"):
        path = os.path.join(REF_ROOT, "pg_gpu", mod + ".py")
        spec = importlib.util.spec_from_file_location("pg_gpu." + mod, path)
        m = importlib.util.module_from_spec(spec)
        sys.modules["pg_gpu." + mod] = m
        spec.loader.exec_module(m)
        setattr(pkg, mod, m)
        _LOADED[mod] = m
    return _LOADED


def load_haplotype_matrix():
    """The reference's HaplotypeMatrix class (haplotype_matrix.py), with empty
    stand-ins for its unused imports allel and tskit (absent here)."""
    if "haplotype_matrix" in _LOADED:
        return _LOADED["haplotype_matrix"].HaplotypeMatrix
    load_reference_modules()
    for name in ("allel", "tskit"):
        stub = sys.modules.setdefault(name, types.ModuleType(name))
        if name == "tskit" and not hasattr(stub, "TreeSequence"):
            stub.TreeSequence = type("TreeSequence", (), {})  # annotation only
    pkg = sys.modules["pg_gpu"]
    for mod in ("accessible", "haplotype_matrix", "genotype_matrix"):
        path = os.path.join(REF_ROOT, "pg_gpu", mod + ".py")
        spec = importlib.util.spec_from_file_location("pg_gpu." + mod, path)
        m = importlib.util.module_from_spec(spec)
        sys.modules["pg_gpu." + mod] = m
        spec.loader.exec_module(m)
        setattr(pkg, mod, m)
        _LOADED[mod] = m
    return _LOADED["haplotype_matrix"].HaplotypeMatrix


def garr(x):
    return np.ascontiguousarray(x).view(GArr)
