// Fast float32 finalisation of the moments statistics for 1 and 2
// populations, shared by the plain and tensor-core band kernels.
//
// Every numerator is an exact integer (int32 where it fits, int64 where a
// sum can cancel) and is converted to float32 once; products of exact
// integers that cannot cancel are formed directly in float32.  Denominators
// are exact integers rounded once to float32 and inverted with an IEEE
// division, so each statistic carries at most four roundings (< 2.5e-7
// relative).  The formulas are the case formulas of ld_statistics.py
// (1116-1617) evaluated for the population patterns of the moments tables
// for one and two populations (ld_pipeline.py:357-457).
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

// int32 in [-2^22, 2^22) or int64 in [-2^44, 2^44) to float32, correctly
// rounded, without the conversion pipe: the exponent-bias trick places the
// integer in the mantissa of a known float and subtracts the bias.
PGLD_HD float small_i2f(int v) {
#ifdef __CUDA_ARCH__
  return __int_as_float(0x4B400000 + v) - 12582912.0f;
#else
  return (float)v;
#endif
}

PGLD_HD float i64_to_f32(i64 v) {
#ifdef __CUDA_ARCH__
  const int hi = (int)(v >> 22);
  if (hi >= -(1 << 22) && hi < (1 << 22)) {
    const int lo = (int)(v & 0x3FFFFF);
    const float fhi = __int_as_float(0x4B400000 + hi) - 12582912.0f;
    const float flo = __int_as_float(0x4B000000 | lo) - 8388608.0f;
    return fmaf(fhi, 4194304.0f, flo);  // one rounding
  }
  return __ll2float_rn(v);
#else
  return (float)v;
#endif
}

PGLD_HD float recip_or_zero(float d) { return d > 0.0f ? 1.0f / d : 0.0f; }

// exact per-population integer features
struct Pop {
  int c1, c2, c3, c4, n;
  int pA, qA, pB, qB;
  int a, b, x;  // c1c4, c2c3, c1c4 - c2c3
  int dA, dB, e;  // qA - pA, qB - pB, (c2+c3) - (c1+c4)
  float xf;
  float nn1f;     // n(n-1)
  float d4f;      // n(n-1)(n-2)(n-3) rounded once
  float t3f;      // n(n-1)(n-2) rounded once
};

PGLD_HD Pop make(int c1, int c2, int c3, int c4, int n) {
  Pop p;
  p.c1 = c1; p.c2 = c2; p.c3 = c3; p.c4 = c4; p.n = n;
  p.pA = c1 + c2; p.qA = c3 + c4; p.pB = c1 + c3; p.qB = c2 + c4;
  p.a = c1 * c4; p.b = c2 * c3; p.x = p.a - p.b;
  p.dA = p.qA - p.pA; p.dB = p.qB - p.pB; p.e = (c2 + c3) - (c1 + c4);
  p.xf = (float)p.x;
  const int nn1 = n * (n - 1);
  p.nn1f = (float)nn1;
  p.d4f = (n >= 4) ? p.nn1f * (float)((n - 2) * (n - 3)) : 0.0f;
  p.t3f = (n >= 3) ? p.nn1f * (float)(n - 2) : 0.0f;
  return p;
}

// numerators of the single-population cases (exact)
PGLD_HD i64 dd_num(const Pop& p) {
  return (i64)p.x * p.x - ((i64)p.a * (p.c1 + p.c4 - 1) + (i64)p.b * (p.c2 + p.c3 - 1));
}
PGLD_HD float dz_num_f(const Pop& p) {
  // x*(dA*dB + e) + 2(a+b): the fma rounds once, and whenever the two terms
  // can cancel the product is below 2^24 and exact
  return fmaf(p.xf, (float)(p.dA * p.dB + p.e), (float)(2 * (p.a + p.b)));
}
PGLD_HD i64 pi2_num(const Pop& p) {
  return (i64)(p.pA * p.pB) * (p.qB * p.qA) - (i64)p.a * (-1 + p.c1 + 3 * p.c2 + 3 * p.c3 + p.c4) -
         (i64)p.b * (-1 + 3 * p.c1 + p.c2 + p.c3 + 3 * p.c4);
}
// pi2 with population t three times and s once, times 2
PGLD_HD i64 triple_num2(const Pop& t, const Pop& s) {
  return (i64)(t.pA * t.qA) * (t.qB * s.pB + t.pB * s.qB - 2 * s.qB) +
         (i64)(t.pA * t.c4 + t.c2 * t.qA) * (s.qB - s.pB);
}
// pi2(i,j,i,j) times 4 (symmetric in the two populations)
PGLD_HD i64 ijij_num4(const Pop& A, const Pop& B) {
  const int a1 = A.c1, a2 = A.c2, a3 = A.c3, a4 = A.c4;
  const int b1 = B.c1, b2 = B.c2, b3 = B.c3, b4 = B.c4;
  i64 q = (i64)(A.qB * A.qA) * (B.pA * B.pB) + (i64)(A.pB * A.qA) * (B.pA * B.qB) +
          (i64)(A.pA * A.qB) * (B.pB * B.qA) + (i64)(A.pA * A.pB) * (B.qB * B.qA);
  const int g1 = a4 - a2 * a3 - a2 * a4 - a3 * a4 - a4 * a4 - a4 * b1;
  const int g2 = a3 - a1 * a3 - a3 * a3 - a1 * a4 - a3 * a4 - a3 * b1 - a4 * b1 - a3 * b2;
  const int g3 = a2 - a1 * a2 - a2 * a2 - a1 * a4 - a2 * a4 - a2 * b1 - a4 * b1 - a1 * b2 - a4 * b2 -
                 a2 * b3;
  const int g4 = a1 - a1 * a1 - a1 * a2 - a1 * a3 - a2 * a3 - a2 * b1 - a3 * b1 - a1 * b2 - a3 * b2 -
                 a1 * b3 - a2 * b3 - a1 * b4;
  return q + (i64)b1 * g1 + (i64)b2 * g2 + (i64)b3 * g3 + (i64)b4 * g4;
}

// DD, Dz, pi2 of one population (moments order for one population)
PGLD_HD void stats1(const Pop& p, float out[3]) {
  const float r4 = recip_or_zero(p.d4f);
  out[0] = i64_to_f32(dd_num(p)) * r4;
  out[1] = dz_num_f(p) * r4;
  out[2] = i64_to_f32(pi2_num(p)) * r4;
}

// the 15 two-population statistics in moments ld_names(2) order:
// DD_0_0 DD_0_1 DD_1_1 Dz_0_0_0 Dz_0_0_1 Dz_0_1_1 Dz_1_0_0 Dz_1_0_1 Dz_1_1_1
// pi2_0_0_0_0 pi2_0_0_0_1 pi2_0_0_1_1 pi2_0_1_0_1 pi2_0_1_1_1 pi2_1_1_1_1
PGLD_HD void stats2(const Pop& p, const Pop& q, float o[15]) {
  const float r4p = recip_or_zero(p.d4f), r4q = recip_or_zero(q.d4f);
  const float r22 = recip_or_zero(p.nn1f * q.nn1f);
  const float r31p = recip_or_zero((float)q.n * p.t3f);  // n_q * n_p(n_p-1)(n_p-2)
  const float r31q = recip_or_zero((float)p.n * q.t3f);
  o[0] = i64_to_f32(dd_num(p)) * r4p;
  o[1] = (p.xf * q.xf) * r22;
  o[2] = i64_to_f32(dd_num(q)) * r4q;
  o[3] = dz_num_f(p) * r4p;
  o[4] = (p.xf * (float)(p.dA * q.dB + p.dB * q.dA)) * (0.5f * r31p);
  o[5] = (p.xf * (float)(q.e + q.dB * q.dA)) * r22;
  o[6] = (q.xf * (float)(p.e + p.dB * p.dA)) * r22;
  o[7] = (q.xf * (float)(q.dA * p.dB + q.dB * p.dA)) * (0.5f * r31q);
  o[8] = dz_num_f(q) * r4q;
  o[9] = i64_to_f32(pi2_num(p)) * r4p;
  o[10] = i64_to_f32(triple_num2(p, q)) * (0.5f * r31p);
  o[11] = fmaf((float)(p.pA * p.qA), (float)(q.pB * q.qB), (float)(q.pA * q.qA) * (float)(p.pB * p.qB)) *
          (0.5f * r22);
  o[12] = i64_to_f32(ijij_num4(p, q)) * (0.25f * r22);
  o[13] = i64_to_f32(triple_num2(q, p)) * (0.5f * r31q);
  o[14] = i64_to_f32(pi2_num(q)) * r4q;
}

}  // namespace fast
}  // namespace pgld
