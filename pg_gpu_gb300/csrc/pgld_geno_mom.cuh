// The single-population genotype estimators of moments (DD, Dz, pi2 of
// _DD_GENO_SINGLE_KERN, _DZ_III_KERN and _PI2_IIII_KERN, genotype_kernels.py:
// 27-71, 235-279, 364-398) and the Rogers-Huff moments, written over the
// centred moments of a SNP pair instead of the nine counts.
//
// With c = dosage - 1 in {-1, 0, 1} for each individual valid at both SNPs I
// and J, the nine moments are m[3 i + j] = sum c_I^i c_J^j (i, j = 0..2;
// m0 = n, the pairwise-valid count).  The tensor-core kernel gets them
// straight from the MMA (operand planes 1, c and c^2 per SNP); from counts
// they are nine small linear forms.  Let
//   U = m1^2 - m2,  V = m3^2 - m6,  T = m1 m3 m4 - m1 m7 - m3 m5.
// As identities of polynomials in the nine counts (expanded with sympy and
// checked term by term against the reference's expressions):
//   16 dd_poly + D16^2      = 16 [(n-1)(n-2) m4^2 - n(n-1) m8 - 2(n-1) T + U V]
//   4 dz_quartic + a b D16  =  4 [(n+1) T - (n-1) m4^2 + 2 n m8 - U V]
//   P2 Q2 S2 R2 + pi2_corr  = n(n-1)(n-2)(n-3) - (n-2)(n-3)(U + V) + U V
//                             - 4 T + 2 m4^2 - 6 m8
// so DD = [..] / (4 d4), Dz = [..] / (2 d4), pi2 = [..] / (16 d4) with
// d4 = n(n-1)(n-2)(n-3), each gated on n >= 4 like the reference kernels.
// Rogers-Huff: cov = n m4 - m1 m3, var_I = n m6 - m3^2, var_J = n m2 - m1^2.
//
// Every |m| <= n < 2^15, so U, V, m4^2, m1 m3 and the polynomials in n are
// 32-bit integers, every product below is 32 x 32 -> 64 bits or a 64-bit
// value times a 16-bit one, and every partial sum stays below 2^62: the
// numerators are exact for populations below 32,768 individuals.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#include "pgld_internal.cuh"
#endif

#ifdef __CUDACC__
#define PGLD_GM_HD __host__ __device__ __forceinline__
#else
#define PGLD_GM_HD inline
#endif

namespace pgld {
namespace gmom {

typedef long long i64;

struct Mom {
  int m[9];  // m[3 i + j] = sum c_I^i c_J^j; m[0] = n
};

// from 9-way counts in the reference's order n00, n01, ..., n22 (dosage at I
// times 3 plus dosage at J)
PGLD_GM_HD Mom from_counts(const int* c) {
  // row sums over the dosage at J for each dosage at I, and the same weighted
  // by c_J and c_J^2
  Mom o;
  int r0[3], r1[3], r2[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int x0 = c[3 * a], x1 = c[3 * a + 1], x2 = c[3 * a + 2];
    r0[a] = x0 + x1 + x2;
    r1[a] = x2 - x0;
    r2[a] = x2 + x0;
  }
  // combine over the dosage at I: weights 1, c_I = a - 1, c_I^2
  o.m[0] = r0[0] + r0[1] + r0[2];
  o.m[1] = r1[0] + r1[1] + r1[2];
  o.m[2] = r2[0] + r2[1] + r2[2];
  o.m[3] = r0[2] - r0[0];
  o.m[4] = r1[2] - r1[0];
  o.m[5] = r2[2] - r2[0];
  o.m[6] = r0[2] + r0[0];
  o.m[7] = r1[2] + r1[0];
  o.m[8] = r2[2] + r2[0];
  return o;
}

// 9-way counts (reference order) back from the moments: the indicator of
// dosage 0, 1, 2 is (c^2 - c) / 2, 1 - c^2, (c^2 + c) / 2 over (1, c, c^2),
// so 4 n_ab = sum_x,y E_a[x] E_b[y] m[3 x + y] with E0 = (0, -1, 1),
// E1 = (2, 0, -2), E2 = (0, 1, 1); the division by 4 is exact
PGLD_GM_HD void to_counts(const Mom& o, int* c) {
  const int* m = o.m;
  int q[3][3];  // q[a][y] = sum_x E_a[x] m[3 x + y]
#pragma unroll
  for (int y = 0; y < 3; ++y) {
    q[0][y] = m[6 + y] - m[3 + y];
    q[1][y] = 2 * (m[y] - m[6 + y]);
    q[2][y] = m[6 + y] + m[3 + y];
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    c[3 * a + 0] = (q[a][2] - q[a][1]) / 4;
    c[3 * a + 1] = (2 * (q[a][0] - q[a][2])) / 4;
    c[3 * a + 2] = (q[a][2] + q[a][1]) / 4;
  }
}

struct Terms {
  i64 T;    // m1 m3 m4 - m1 m7 - m3 m5
  i64 UV;   // (m1^2 - m2)(m3^2 - m6)
  int UpV;  // (m1^2 - m2) + (m3^2 - m6)
  int m44;  // m4^2
};

PGLD_GM_HD Terms terms(const Mom& o) {
  const int* m = o.m;
  Terms t;
  const int U = m[1] * m[1] - m[2];
  const int V = m[3] * m[3] - m[6];
  t.T = (i64)(m[1] * m[3]) * m[4] - ((i64)(m[1] * m[7]) + (i64)(m[3] * m[5]));
  t.UV = (i64)U * V;
  t.UpV = U + V;
  t.m44 = m[4] * m[4];
  return t;
}

PGLD_GM_HD i64 d4(int n) { return (i64)(n * (n - 1)) * ((n - 2) * (n - 3)); }

// numerator over 4 d4
PGLD_GM_HD i64 dd_num(const Mom& o, const Terms& t) {
  const int n = o.m[0];
  return (i64)((n - 1) * (n - 2)) * t.m44 - (i64)(n * (n - 1)) * o.m[8] -
         2 * (i64)(n - 1) * t.T + t.UV;
}
// numerator over 2 d4
PGLD_GM_HD i64 dz_num(const Mom& o, const Terms& t) {
  const int n = o.m[0];
  return (i64)(n + 1) * t.T - (i64)(n - 1) * t.m44 + (i64)(2 * n) * o.m[8] - t.UV;
}
// numerator over 16 d4
PGLD_GM_HD i64 pi2_num(const Mom& o, const Terms& t) {
  const int n = o.m[0];
  return d4(n) - (i64)((n - 2) * (n - 3)) * t.UpV + t.UV - 4 * t.T + 2 * (i64)t.m44 -
         6 * (i64)o.m[8];
}

struct RHm {
  i64 cov2, den;  // cov^2 and var_I var_J
};
PGLD_GM_HD RHm rh(const Mom& o) {
  const int* m = o.m;
  const int n = m[0];
  const i64 cov = (i64)n * m[4] - (i64)m[1] * m[3];
  const i64 vi = (i64)n * m[6] - (i64)m[3] * m[3];
  const i64 vj = (i64)n * m[2] - (i64)m[1] * m[1];
  return {cov * cov, vi * vj};
}

#ifdef __CUDACC__
// float32 per-pair outputs of the band kernels: x = Rogers-Huff r^2 (NaN
// where a SNP has no variance among the pairwise-valid individuals), y, z, w
// = DD, Dz, pi2 (0 below 4 individuals); bit k of the mask selects component
// k, the others stay 0.  MASK >= 0 fixes the mask at compile time, -1 takes
// mask_rt; both evaluate the same operations, so the values are identical.
// Everything is computed unconditionally and the gates are selects (no
// divergent branches).  Populations up to 8,192 individuals: the
// Rogers-Huff moments n m4 - m1 m3, n m6 - m3^2, n m2 - m1^2 are then 32-bit
// integers below 2^27, converted once each (relative error 2^-24), so r^2
// carries at most 8 roundings; the 64-bit numerators convert with at most two
// roundings and share one reciprocal of d4 (__fdividef: 2 ulp): every output
// is within 1e-6 relative of its exact value.
template <int MASK>
__device__ __forceinline__ float4 stats_f32(const Mom& o, int mask_rt) {
  const int mask = MASK >= 0 ? MASK : mask_rt;
  float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
  const int* m = o.m;
  const int n = m[0];
  if (mask & 1) {
    const int cov = n * m[4] - m[1] * m[3];
    const int vi = n * m[6] - m[3] * m[3];
    const int vj = n * m[2] - m[1] * m[1];
    const float fc = (float)cov;
    const float v = __fdividef(fc * fc, (float)vi * (float)vj);
    out.x = (vi > 0 && vj > 0) ? v : __int_as_float(0x7fc00000);
  }
  if (mask & 14) {
    const Terms t = terms(o);
    const bool ok = n >= 4;
    const float r = __fdividef(1.0f, pgld::ll2f(d4(n)));  // unused where !ok
    if (mask & 2) out.y = ok ? pgld::ll2f(dd_num(o, t)) * (0.25f * r) : 0.f;
    if (mask & 4) out.z = ok ? pgld::ll2f(dz_num(o, t)) * (0.5f * r) : 0.f;
    if (mask & 8) out.w = ok ? pgld::ll2f(pi2_num(o, t)) * (0.0625f * r) : 0.f;
  }
  return out;
}
#endif

}  // namespace gmom
}  // namespace pgld
