"""Expand the reference's three large genotype polynomials into monomial tables.

The unbiased genotype estimators of moments (Ragsdale & Gravel) that pg_gpu
evaluates for one population -- the DD numerator polynomial of
_DD_GENO_SINGLE_KERN (genotype_kernels.py:27-71), the Dz quartic of
_DZ_III_KERN (genotype_kernels.py:235-279) and the pi2 correction of
_PI2_IIII_KERN (genotype_kernels.py:364-398) -- are polynomials of degree 3 in
the nine genotype counts g1..g9 (moments order) with integer coefficients.
This script reads those expressions from the reference's kernel sources (run
through the CPU shim), expands each with sympy into canonical monomials, and
writes

  oracle/geno_tables.py                     (the oracle's exact evaluation)

The CUDA kernels evaluate the same numerators through the centred moments of
the pair (pg_gpu_gb300/csrc/pgld_geno_mom.cuh), checked against these tables
by tests/test_geno_mom_cpu.py.

The table is committed; this script runs only where the reference checkout
exists and is not needed to build or test.
"""
import os
import re
import sys

import sympy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)

import _ref_shim as S  # noqa: E402

SYMS = sympy.symbols("n1:10")


def _expr(code, var):
    m = re.search(r"double\s+" + var + r"\s*=(.*?);", code, re.S)
    if not m:
        raise RuntimeError(f"{var} not found")
    text = re.sub(r"//[^\n]*", "", m.group(1))
    text = text.replace("\n", " ")
    return sympy.sympify(text, locals={f"n{k}": SYMS[k - 1] for k in range(1, 10)},
                         rational=True)


def _monomials(expr):
    poly = sympy.Poly(sympy.expand(expr), *SYMS)
    out = []
    for exps, coef in sorted(poly.terms(), key=lambda t: (sum(t[0]), t[0])):
        if coef.q != 1:
            raise RuntimeError("non-integer coefficient")
        idx = []
        for k, e in enumerate(exps):
            idx += [k] * e
        if len(idx) > 3:
            raise RuntimeError("degree above 3")
        idx += [9] * (3 - len(idx))  # index 9 is the constant 1
        out.append((int(coef.p), tuple(sorted(idx))))
    return out


def main():
    M = S.load_reference_modules()
    gk = M["genotype_kernels"]
    tables = {
        "DD_POLY": _monomials(_expr(gk._DD_GENO_SINGLE_KERN.code, "poly")),
        "DZ_QUARTIC": _monomials(_expr(gk._DZ_III_KERN.code, "quartic")),
        # the kernel scales the bracket by 1/16 after the closing parenthesis
        "PI2_CORR": _monomials(_expr(gk._PI2_IIII_KERN.code, "corr") * 16),
    }
    py = ['"""Monomial tables of the single-population genotype estimators.',
          "",
          "Generated by tests/golden/make_geno_tables.py from the expressions of",
          "_DD_GENO_SINGLE_KERN, _DZ_III_KERN and _PI2_IIII_KERN",
          "(genotype_kernels.py:27-71, 235-279, 364-398).  Each entry is",
          "(coefficient, (a, b, c)): coefficient * g[a] * g[b] * g[c] with g the",
          "moments-order counts g1..g9 at indices 0..8 and g[9] = 1.",
          '"""', ""]
    for name, mono in tables.items():
        py.append(f"{name} = [")
        for c, (a, b, d) in mono:
            py.append(f"    ({c}, ({a}, {b}, {d})),")
        py.append("]")
        py.append("")
    with open(os.path.join(ROOT, "oracle", "geno_tables.py"), "w") as f:
        f.write("\n".join(py))
    for name, mono in tables.items():
        print(name, len(mono), "monomials, max |coef|", max(abs(c) for c, _ in mono))


if __name__ == "__main__":
    main()
