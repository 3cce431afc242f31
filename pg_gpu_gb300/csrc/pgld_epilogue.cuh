// Fast float32 finalisation of the moments statistics for 1 and 2
// populations, shared by the plain and tensor-core band kernels.
//
// Counts arrive as exact float32 integers.  With at most 2048 haplotypes per
// population every feature below (marginals, c1*c4, x = c1c4 - c2c3,
// dA*dB + e, the quadratic cofactors of pi2(i,j,i,j), ...) is an integer of
// magnitude < 2^24, so it is formed exactly in float32 -- on the float32
// pipes, with no integer-to-float conversions.
//
// Every numerator is rewritten as (at most) two products of such exact
// integers -- e.g. DD: x (x + c2 + c3) - c1c4 n + (c1c4 + c2c3), pi2:
// c1c4 (n^2 - 4n + 2) + x (x + n - 1 - (n - 2)(c1 + c4)) -- and evaluated
// with Kahan's algorithm for a*b + c*d (the rounding error of c*d recovered
// exactly by an fma, one fma and one addition more), whose relative error is
// at most 2u even under cancellation (Jeannerod, Louvet and Muller, "Further
// analysis of Kahan's algorithm for the accurate computation of 2x2
// determinants", Math. Comp. 82, 2013).  The one numerator with three
// products, pi2(i,j,i,j), sums its two cubic products exactly as s + t
// (TwoProduct / TwoSum: the low parts are integers below 2^22 and add exactly)
// before one fma adds the quartic product, so it carries at most 3u (DD
// likewise, its exact integer remainder added last).
// 64-bit integer multiplies would run at the float64 rate on GB300.
// Denominators come from per-CTA tables of reciprocals indexed by the valid
// sample size n (1/n, 1/(n(n-1)), 1/(n(n-1)(n-2)), 1/(n(n-1)(n-2)(n-3)), each
// the IEEE reciprocal of the exact integer rounded once to float32), so each
// statistic is within 10u (< 6e-7) relative of its exact value.  The formulas
// are the case formulas of ld_statistics.py (1116-1617) for the population
// patterns of the moments tables of one and two populations
// (ld_pipeline.py:357-457).
#pragma once
#include <stdint.h>

#include <cmath>

#ifdef __CUDACC__
#define PGLD_HD __host__ __device__ __forceinline__
#else
#define PGLD_HD inline
#endif

namespace pgld {
namespace fast {

typedef long long i64;

constexpr int kMaxN = 2048;

// rounded-to-nearest float32 operations that the compiler may not fuse into
// fma (the error-free transformations depend on each rounding)
PGLD_HD float fadd(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
PGLD_HD float fsub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
PGLD_HD float fmul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}

// exact float32 integer in [0, 2^22) to int without the conversion pipe
PGLD_HD int f2i_small(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_int(f + 12582912.0f) - 0x4B400000;
#else
  return (int)f;
#endif
}

// an integer held exactly as s + e
struct X2 {
  float s, e;
};

PGLD_HD X2 x2_prod(float a, float b) {
  const float p = fmul(a, b);
  return {p, fmaf(a, b, -p)};
}

// acc += a * b, exactly (a, b integers of magnitude < 2^24)
PGLD_HD void x2_add_prod(X2& acc, float a, float b) {
  const float p = fmul(a, b);
  const float pe = fmaf(a, b, -p);
  const float s = fadd(acc.s, p);
  const float bb = fsub(s, acc.s);
  const float t = fadd(fsub(acc.s, fsub(s, bb)), fsub(p, bb));
  acc.s = s;
  acc.e = fadd(acc.e, fadd(pe, t));
}

PGLD_HD float x2_value(const X2& v) { return fadd(v.s, v.e); }

// a*b + c*d (exact float32 integers) with relative error <= 2u: Kahan's
// algorithm
PGLD_HD float dot2(float a, float b, float c, float d) {
  const float w = fmul(c, d);
  const float e = fmaf(c, d, -w);
  return fadd(fmaf(a, b, w), e);
}

// reciprocal tables, entries 0..nmax (0 where the integer is 0)
struct Recip {
  const float* inv;  // 1/n
  const float* r2;   // 1/(n(n-1))
  const float* r3;   // 1/(n(n-1)(n-2))
  const float* r4;   // 1/(n(n-1)(n-2)(n-3))
};

PGLD_HD void recip_entry(int n, float* inv, float* r2, float* r3, float* r4) {
  const i64 m1 = n, m2 = m1 * (n - 1), m3 = m2 * (n - 2), m4 = m3 * (n - 3);
  *inv = m1 > 0 ? 1.0f / (float)m1 : 0.0f;
  *r2 = m2 > 0 ? 1.0f / (float)m2 : 0.0f;
  *r3 = m3 > 0 ? 1.0f / (float)m3 : 0.0f;
  *r4 = m4 > 0 ? 1.0f / (float)m4 : 0.0f;
}

// exact per-population features as float32 integers
struct Pop {
  float c1, c2, c3, c4;
  float pA, qA, pB, qB;
  float a, b, x;    // c1c4, c2c3, c1c4 - c2c3
  float dA, dB, e;  // qA - pA, qB - pB, (c2+c3) - (c1+c4)
  float s, t, ns;   // c2 + c3, c1 + c4, c1 + c2 + c3 + c4
  int n;            // ns as an int (the pairwise valid n of 0/1/-1 data)
};

PGLD_HD Pop make(float c1, float c2, float c3, float c4) {
  Pop p;
  p.c1 = c1; p.c2 = c2; p.c3 = c3; p.c4 = c4;
  p.pA = c1 + c2; p.qA = c3 + c4; p.pB = c1 + c3; p.qB = c2 + c4;
  p.a = c1 * c4; p.b = c2 * c3; p.x = p.a - p.b;
  p.dA = p.qA - p.pA; p.dB = p.qB - p.pB;
  p.s = c2 + c3; p.t = c1 + c4; p.e = p.s - p.t;
  p.ns = p.pA + p.qA;
  p.n = f2i_small(p.ns);
  return p;
}

// c1(c1-1)c4(c4-1) + c2(c2-1)c3(c3-1) - 2c1c2c3c4
//   = x^2 - a(c1+c4-1) - b(c2+c3-1) = x (x + c2 + c3) - a n + (a + b)
// (n = the sum of the four counts; b = a - x).  With w = RN(a n) and its exact
// error e, x (x + c2 + c3) - w is an integer rounded once by the fma (exactly
// when below 2^24) and a + b - e is exact (< 2^23), so the value is within 3u.
PGLD_HD float dd_num(const Pop& p) {
  const float w = fmul(p.a, p.ns);
  const float e = fmaf(p.a, p.ns, -w);
  return fadd(fmaf(p.x, p.x + p.s, -w), (p.a + p.b) - e);
}
// x*(dA*dB + e) + 2(a+b): the fma rounds once, and whenever the two terms can
// cancel the product is below 2^24 and exact
PGLD_HD float dz_num(const Pop& p) { return fmaf(p.x, p.dA * p.dB + p.e, 2.0f * (p.a + p.b)); }
// pA pB qA qB - a(3c2 + 3c3 + c1 + c4 - 1) - b(3c1 + 3c4 + c2 + c3 - 1)
//   = a (n^2 - 4n + 2) + x (x + n - 1 - (n - 2)(c1 + c4))
// (pA pB = n c1 - x and qA qB = n c4 - x)
PGLD_HD float pi2_num(const Pop& p) {
  const float pn = fmaf(p.ns, p.ns - 4.0f, 2.0f);
  const float w = fmaf(2.0f - p.ns, p.t, p.x + (p.ns - 1.0f));
  return dot2(p.a, pn, p.x, w);
}
// pi2 with population t three times and s once, times 2
PGLD_HD float triple_num2(const Pop& t, const Pop& s) {
  return dot2(t.pA * t.qA, t.qB * s.pB + t.pB * s.qB - 2.0f * s.qB, t.pA * t.c4 + t.c2 * t.qA,
              s.qB - s.pB);
}
// pi2(i,j,i,j) times 4 (symmetric in the two populations).  The quartic and
// cubic polynomial of the reference (ld_statistics.py:1349-1402) equals
//   H_A H_B + (1 - n_A - n_B) K - x_A e_B - x_B e_A
//   = K m_A m_B + x_B (m_A e_A) + x_A (m_B e_B + 4 x_B)
// with H_A = qA_A pA_B + pA_A qA_B, H_B = qB_A pB_B + pB_A qB_B,
// K = c1_A c4_B + c2_A c3_B + c3_A c2_B + c4_A c1_B and m = n - 1 (algebraic
// identities, checked against the oracle in tests/test_epilogue_cpu.py).  The
// two cubic products are summed exactly as s + t; K m_A m_B + s rounds once in
// the fma and t (an integer below 2^22) is added last.
PGLD_HD float ijij_num4(const Pop& A, const Pop& B) {
  const float K = A.c1 * B.c4 + A.c2 * B.c3 + A.c3 * B.c2 + A.c4 * B.c1;
  const float mA = A.ns - 1.0f, mB = B.ns - 1.0f;
  const float y1 = mA * A.e, y2 = fmaf(mB, B.e, 4.0f * B.x);
  const float p1 = fmul(B.x, y1), e1 = fmaf(B.x, y1, -p1);
  const float p2 = fmul(A.x, y2), e2 = fmaf(A.x, y2, -p2);
  const float s = fadd(p1, p2);
  const float bb = fsub(s, p1);
  const float t = fadd(fadd(fsub(p1, fsub(s, bb)), fsub(p2, bb)), fadd(e1, e2));
  return fadd(fmaf(K, fmul(mA, mB), s), t);
}

// DD, Dz, pi2 of one population (moments order for one population)
PGLD_HD void stats1(const Pop& p, const Recip& T, float out[3]) {
  const float r4 = T.r4[p.n];
  out[0] = dd_num(p) * r4;
  out[1] = dz_num(p) * r4;
  out[2] = pi2_num(p) * r4;
}

// r^2 = x^2 / (pA (n-pA) pB (n-pB)), NaN where undefined
PGLD_HD float r2_of(const Pop& p) {
  const float num = x2_value(x2_prod(p.x, p.x));
  const float den = x2_value(x2_prod(p.pA * p.qA, p.pB * p.qB));
  return den > 0.0f ? num / den : NAN;
}

// the 15 two-population statistics in moments ld_names(2) order:
// DD_0_0 DD_0_1 DD_1_1 Dz_0_0_0 Dz_0_0_1 Dz_0_1_1 Dz_1_0_0 Dz_1_0_1 Dz_1_1_1
// pi2_0_0_0_0 pi2_0_0_0_1 pi2_0_0_1_1 pi2_0_1_0_1 pi2_0_1_1_1 pi2_1_1_1_1
PGLD_HD void stats2(const Pop& p, const Pop& q, const Recip& T, float o[15]) {
  const float r4p = T.r4[p.n], r4q = T.r4[q.n];
  const float r22 = T.r2[p.n] * T.r2[q.n];
  const float r31p = T.r3[p.n] * T.inv[q.n];  // 1 / (n_q * n_p(n_p-1)(n_p-2))
  const float r31q = T.r3[q.n] * T.inv[p.n];
  o[0] = dd_num(p) * r4p;
  o[1] = (p.x * q.x) * r22;
  o[2] = dd_num(q) * r4q;
  o[3] = dz_num(p) * r4p;
  o[4] = (p.x * (p.dA * q.dB + p.dB * q.dA)) * (0.5f * r31p);
  o[5] = (p.x * (q.e + q.dB * q.dA)) * r22;
  o[6] = (q.x * (p.e + p.dB * p.dA)) * r22;
  o[7] = (q.x * (q.dA * p.dB + q.dB * p.dA)) * (0.5f * r31q);
  o[8] = dz_num(q) * r4q;
  o[9] = pi2_num(p) * r4p;
  o[10] = triple_num2(p, q) * (0.5f * r31p);
  o[11] = fmaf(p.pA * p.qA, q.pB * q.qB, (q.pA * q.qA) * (p.pB * p.qB)) * (0.5f * r22);
  o[12] = ijij_num4(p, q) * (0.25f * r22);
  o[13] = triple_num2(q, p) * (0.5f * r31q);
  o[14] = pi2_num(q) * r4q;
}

}  // namespace fast
}  // namespace pgld
