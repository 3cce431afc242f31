// Two pairs at a time: the float32 moments epilogue of pgld_epilogue.cuh on
// float2 operands, so that every addition, multiplication and fused
// multiply-add is one packed sm_100+ instruction (FADD2 / FMUL2 / FFMA2) for
// two SNP pairs.  The arithmetic of each lane is exactly that of the scalar
// code: the same exact integer features, the same two-product numerators
// (Kahan's algorithm, TwoProduct / TwoSum) and the same reciprocal-table
// divisions, so each lane's statistics equal the scalar epilogue's bit for bit.
#pragma once
#include "pgld_epilogue.cuh"

#ifndef __CUDACC__
struct float2 {
  float x, y;
};
inline float2 make_float2(float x, float y) { return {x, y}; }
struct alignas(16) float4 {
  float x, y, z, w;
};
inline float4 make_float4(float x, float y, float z, float w) { return {x, y, z, w}; }
#endif

namespace pgld {
namespace fast2 {

typedef float2 V;

#if defined(__CUDA_ARCH__)
PGLD_HD V vadd(V a, V b) { return __fadd2_rn(a, b); }
PGLD_HD V vmul(V a, V b) { return __fmul2_rn(a, b); }
PGLD_HD V vfma(V a, V b, V c) { return __ffma2_rn(a, b, c); }
#else
// host build (numerical tests): one rounded float operation per lane
PGLD_HD V vadd(V a, V b) { return make_float2(a.x + b.x, a.y + b.y); }
PGLD_HD V vmul(V a, V b) { return make_float2(a.x * b.x, a.y * b.y); }
PGLD_HD V vfma(V a, V b, V c) { return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y)); }
#endif
PGLD_HD V vneg(V a) { return make_float2(-a.x, -a.y); }
// one rounded product / fused multiply-add per lane, kept scalar (not paired
// into one packed instruction), for operands that live in unpaired registers
#if defined(__CUDA_ARCH__)
PGLD_HD float smul(float a, float b) {
  float r;
  asm("mul.rn.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
PGLD_HD float sfma(float a, float b, float c) {
  float r;
  asm("fma.rn.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
#else
PGLD_HD float smul(float a, float b) { return a * b; }
PGLD_HD float sfma(float a, float b, float c) { return fmaf(a, b, c); }
#endif
PGLD_HD V vmul_s(V a, V b) { return make_float2(smul(a.x, b.x), smul(a.y, b.y)); }
PGLD_HD V vfma_s(V a, V b, V c) { return make_float2(sfma(a.x, b.x, c.x), sfma(a.y, b.y, c.y)); }
// the scale products r22, h31 from unpaired table loads: scalar (1) or packed
#ifndef PGLD_F2_SSCALE
#define PGLD_F2_SSCALE 1
#endif
PGLD_HD V vs(float a) { return make_float2(a, a); }
// a - b: the negation is exact, so the sum rounds once, exactly like a
// correctly rounded subtraction
PGLD_HD V vsub(V a, V b) { return vadd(a, vneg(b)); }

// a*b + c*d with relative error <= 2u (Kahan's algorithm, as fast::dot2)
PGLD_HD V dot2(V a, V b, V c, V d) {
  const V w = vmul(c, d);
  const V e = vfma(c, d, vneg(w));
  return vadd(vfma(a, b, w), e);
}

struct Pop {
  V c1, c2, c3, c4;
  V pA, qA, pB, qB;
  V a, b, x;
  V dA, dB, e;
  V s, t, ns;
  V m1;        // ns - 1
  int n0, n1;  // valid n of each lane
};

PGLD_HD int f2i(float f) { return fast::f2i_small(f); }

PGLD_HD Pop make(V c1, V c2, V c3, V c4) {
  Pop p;
  p.c1 = c1; p.c2 = c2; p.c3 = c3; p.c4 = c4;
  p.pA = vadd(c1, c2); p.qA = vadd(c3, c4); p.pB = vadd(c1, c3); p.qB = vadd(c2, c4);
  p.a = vmul(c1, c4); p.b = vmul(c2, c3); p.x = vsub(p.a, p.b);
  p.dA = vsub(p.qA, p.pA); p.dB = vsub(p.qB, p.pB);
  p.s = vadd(c2, c3); p.t = vadd(c1, c4); p.e = vsub(p.s, p.t);
  p.ns = vadd(p.pA, p.qA);
  p.m1 = vsub(p.ns, vs(1.0f));
  p.n0 = f2i(p.ns.x);
  p.n1 = f2i(p.ns.y);
  return p;
}

PGLD_HD V dd_num(const Pop& p) {
  const V w = vmul(p.a, p.ns);
  const V e = vfma(p.a, p.ns, vneg(w));
  return vadd(vfma(p.x, vadd(p.x, p.s), vneg(w)), vsub(vadd(p.a, p.b), e));
}
// w = dA dB + e (exact), shared with the cross terms Dz(i,j,j)
PGLD_HD V dz_num(const Pop& p, V w) {
  const V ab = vadd(p.a, p.b);
  return vfma(p.x, w, vadd(ab, ab));
}
PGLD_HD V pi2_num(const Pop& p) {
  const V pn = vfma(p.ns, vsub(p.ns, vs(4.0f)), vs(2.0f));
  const V w = vfma(vsub(vs(2.0f), p.ns), p.t, vadd(p.x, p.m1));
  return dot2(p.a, pn, p.x, w);
}
// uA = pA qA of population t
PGLD_HD V triple_num2(const Pop& t, const Pop& s, V uA) {
  return dot2(uA, vsub(vfma(t.qB, s.pB, vmul(t.pB, s.qB)), vadd(s.qB, s.qB)),
              vfma(t.pA, t.c4, vmul(t.c2, t.qA)), vsub(s.qB, s.pB));
}
PGLD_HD V ijij_num4(const Pop& A, const Pop& B) {
  const V K = vfma(A.c1, B.c4, vfma(A.c2, B.c3, vfma(A.c3, B.c2, vmul(A.c4, B.c1))));
  const V mA = A.m1, mB = B.m1;
  const V x2 = vadd(B.x, B.x);
  const V y1 = vmul(mA, A.e), y2 = vfma(mB, B.e, vadd(x2, x2));
  const V p1 = vmul(B.x, y1), e1 = vfma(B.x, y1, vneg(p1));
  const V p2 = vmul(A.x, y2), e2 = vfma(A.x, y2, vneg(p2));
  const V s = vadd(p1, p2);
  const V bb = vsub(s, p1);
  const V t = vadd(vadd(vsub(p1, vsub(s, bb)), vsub(p2, bb)), vadd(e1, e2));
  return vadd(vfma(K, vmul(mA, mB), s), t);
}

// the reciprocal factors of the valid n of two lanes: 1/n, 1/(n(n-1)),
// 1/(2 n(n-1)(n-2)) (half the scalar table's r3: exact, and the factor the
// triple statistics need), 1/(n(n-1)(n-2)(n-3)), from one interleaved table
// of float4 (recip_entry4)
struct R2 {
  V inv, r2, r3h, r4;
};
PGLD_HD void recip_entry4(int n, float4* e) {
  float inv, r2, r3, r4;
  fast::recip_entry(n, &inv, &r2, &r3, &r4);
  *e = make_float4(inv, r2, 0.5f * r3, r4);
}
// statistics 11 (pi2_0_0_1_1) and 12 (pi2_0_1_0_1) leave stats2_to with the
// scale r22; their values are the num * r22 products (or sums of them) times
// these exact powers of two
constexpr float kPost11 = 0.5f, kPost12 = 0.25f;
PGLD_HD R2 recip(const float4* T4, int n0, int n1) {
  const float4 a = T4[n0], b = T4[n1];
  return {make_float2(a.x, b.x), make_float2(a.y, b.y), make_float2(a.z, b.z),
          make_float2(a.w, b.w)};
}

// the 15 two-population statistics in moments ld_names(2) order, two pairs:
// statistic k = num * scale goes to sink(k, num, scale) as soon as it is
// formed (a caller that accumulates fuses the product into its sums)
template <class Sink>
PGLD_HD void stats2_to(const Pop& p, const Pop& q, const float4* T4, Sink&& sink) {
  const R2 rp = recip(T4, p.n0, p.n1), rq = recip(T4, q.n0, q.n1);
#if PGLD_F2_SSCALE
  const V r22 = vmul_s(rp.r2, rq.r2);
#else
  const V r22 = vmul(rp.r2, rq.r2);
#endif
  const V wp = vfma(p.dA, p.dB, p.e), wq = vfma(q.dA, q.dB, q.e);
  sink(0, dd_num(p), rp.r4);
  sink(1, vmul(p.x, q.x), r22);
  sink(2, dd_num(q), rq.r4);
  sink(3, dz_num(p, wp), rp.r4);
  sink(8, dz_num(q, wq), rq.r4);
  sink(9, pi2_num(p), rp.r4);
  sink(14, pi2_num(q), rq.r4);
  sink(5, vmul(p.x, wq), r22);
  sink(6, vmul(q.x, wp), r22);
  const V uAp = vmul(p.pA, p.qA), uAq = vmul(q.pA, q.qA);
  sink(11, vfma(uAp, vmul(q.pB, q.qB), vmul(uAq, vmul(p.pB, p.qB))), r22);  // x kPost11
  sink(12, ijij_num4(p, q), r22);                                            // x kPost12
  const V dc = vfma(p.dA, q.dB, vmul(p.dB, q.dA));
#if PGLD_F2_SSCALE
  const V h31p = vmul_s(rp.r3h, rq.inv);
#else
  const V h31p = vmul(rp.r3h, rq.inv);
#endif
  sink(4, vmul(p.x, dc), h31p);
  sink(10, triple_num2(p, q, uAp), h31p);
#if PGLD_F2_SSCALE
  const V h31q = vmul_s(rq.r3h, rp.inv);
#else
  const V h31q = vmul(rq.r3h, rp.inv);
#endif
  sink(7, vmul(q.x, dc), h31q);
  sink(13, triple_num2(q, p, uAq), h31q);
}

// the sink's products, statistics 11 and 12 still without their post factors
PGLD_HD void stats2_raw(const Pop& p, const Pop& q, const float4* T4, V o[15]) {
  stats2_to(p, q, T4, [&](int k, V num, V sc) { o[k] = vmul(num, sc); });
}
PGLD_HD void stats2(const Pop& p, const Pop& q, const float4* T4, V o[15]) {
  stats2_raw(p, q, T4, o);
  o[11] = vmul(o[11], vs(kPost11));
  o[12] = vmul(o[12], vs(kPost12));
}
// the post factor of statistic k of the two-population list (scaling by a
// power of two commutes with every rounding of a sum of the sink's products)
PGLD_HD constexpr double post2(int k) { return k == 11 ? kPost11 : k == 12 ? kPost12 : 1.0; }

// a / b with b > 0: the CUDA fast division (within 2 ulp for b below 2^126)
PGLD_HD float fdiv(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdividef(a, b);
#else
  return a / b;
#endif
}

// the per-pair outputs of two pairs: r^2 (NaN where p_A q_A p_B q_B = 0), and
// DD, Dz, pi2 times r4 = 1/(n(n-1)(n-2)(n-3)) of each lane (0 below n = 4)
PGLD_HD void pair_outputs(const Pop& p, V r4, float4 (&st)[2]) {
  const V dd = vmul(dd_num(p), r4);
  const V dz = vmul(dz_num(p, vfma(p.dA, p.dB, p.e)), r4);
  const V pi = vmul(pi2_num(p), r4);
  const V num = vmul(p.x, p.x);
  const V den = vmul(vmul(p.pA, p.qA), vmul(p.pB, p.qB));
  st[0] = make_float4(den.x > 0.f ? fdiv(num.x, den.x) : NAN, dd.x, dz.x, pi.x);
  st[1] = make_float4(den.y > 0.f ? fdiv(num.y, den.y) : NAN, dd.y, dz.y, pi.y);
}

template <class Sink>
PGLD_HD void stats1_to(const Pop& p, const float4* T4, Sink&& sink) {
  const V r4 = recip(T4, p.n0, p.n1).r4;
  sink(0, dd_num(p), r4);
  sink(1, dz_num(p, vfma(p.dA, p.dB, p.e)), r4);
  sink(2, pi2_num(p), r4);
}

PGLD_HD void stats1(const Pop& p, const float4* T4, V o[3]) {
  stats1_to(p, T4, [&](int k, V num, V sc) { o[k] = vmul(num, sc); });
}

}  // namespace fast2
}  // namespace pgld
