// Per-pair statistics of the window sums, shared by the plain and the
// tensor-core window kernels.
//
// Per pair: r^2 on the pair's counts (where defined), sigma_D^2 = the DD over
// the pi2 numerator (n >= 4, 0 where the pi2 numerator is 0), the moments DD,
// Dz, pi2 (0 below n = 4) and the naive r^2 of _tile_r2_naive
// (ld_statistics.py:299-308) from per-site allele frequencies.  Numerators
// come from the exact float32 features of pgld_epilogue.cuh; the divisions
// use the fast reciprocal (relative error of a few ulp per pair, far inside
// the window sums' float32 accumulation), the moments denominators the
// per-n reciprocal tables.
#pragma once
#include "pgld_epilogue.cuh"
#include "pgld_epilogue2.cuh"

namespace pgld {
namespace win {

// per-site (dac, nv, 1 / nv, u) with u = 1 / (dac (nv - dac)); u is 0 where
// the site is monomorphic among its valid haplotypes or has none.  The naive
// r^2 of a pair is D^2 / (p_i q_i p_j q_j) with D = c1 / n - p_i p_j and
// p = dac / nv, i.e. E^2 u_i u_j with E = D nv_i nv_j = (c1 nv_i nv_j -
// n dac_i dac_j) / n (or -dac_i dac_j where n = 0)
__device__ __forceinline__ float4 site_freq(int dac, int nv) {
  if (nv <= 0) return make_float4(0.f, 0.f, 0.f, 0.f);
  const float d = (float)dac, v = (float)nv;
  const float pq_num = d * (v - d);  // exact: below 2^24 for nv <= 4096
  return make_float4(d, v, 1.0f / v, pq_num > 0.f ? 1.0f / pq_num : 0.f);
}

// accumulate one pair: acc = r^2, sigma_D^2, DD, Dz, pi2, naive r^2
__device__ __forceinline__ void window_pair(const fast::Pop& p, int n, float c1, float inv_n,
                                            float r4n, float4 si, float4 sj, float (&acc)[6],
                                            int& n_r2, int& n_four) {
  const float rden = fast::x2_value(fast::x2_prod(p.pA * p.qA, p.pB * p.qB));
  if (rden > 0.f) {
    acc[0] += __fdividef(fast::x2_value(fast::x2_prod(p.x, p.x)), rden);
    ++n_r2;
  }
  if (n >= 4) {
    const float dd = fast::dd_num(p), pi = fast::pi2_num(p);
    ++n_four;
    if (pi != 0.f) acc[1] += __fdividef(dd, pi);
    acc[2] += dd * r4n;
    acc[3] += fast::dz_num(p) * r4n;
    acc[4] += pi * r4n;
  }
  if (si.w > 0.f && sj.w > 0.f) {
    // E = D v_i v_j from the exact integer c1 v_i v_j - n d_i d_j, so that
    // the cancellation costs nothing (p_AB = 0 where n = 0)
    float E;
    if (n > 0) {
      fast::X2 num = fast::x2_prod(c1, si.y * sj.y);
      fast::x2_add_prod(num, -(float)n, si.x * sj.x);
      E = fast::x2_value(num) * inv_n;
    } else {
      E = -(si.x * sj.x);
    }
    acc[5] += (E * E) * (si.w * sj.w);
  }
}

// window_pair for two pairs (i, j0) and (i, j1) at once on packed float2
// features (the tensor-core window kernels): the same statistics, with the
// naive-r^2 numerator c1 v_i v_j - n d_i d_j by Kahan's two-product
// algorithm; live.x / live.y select the pairs that belong to the window.
// tab(n) gives (1/n, 1/(n(n-1)(n-2)(n-3))) of the reciprocal tables.
template <class Tab>
__device__ __forceinline__ void window_pair2(const fast2::Pop& p, float2 c1, Tab&& tab,
                                             float4 si, float4 sj0, float4 sj1, bool live0,
                                             bool live1, float2 (&acc)[6], int& n_pairs,
                                             int& n_r2, int& n_four) {
  using namespace fast2;
  const float2 t0 = tab(p.n0), t1 = tab(p.n1);
  n_pairs += (live0 ? 1 : 0) + (live1 ? 1 : 0);
  const V rden = vmul(vmul(p.pA, p.qA), vmul(p.pB, p.qB));
  const V xx = vmul(p.x, p.x);
  const bool r0 = live0 && rden.x > 0.f, r1 = live1 && rden.y > 0.f;
  n_r2 += (r0 ? 1 : 0) + (r1 ? 1 : 0);
  acc[0] = vadd(acc[0], make_float2(r0 ? __fdividef(xx.x, rden.x) : 0.f,
                                    r1 ? __fdividef(xx.y, rden.y) : 0.f));
  const bool f0 = live0 && p.n0 >= 4, f1 = live1 && p.n1 >= 4;
  n_four += (f0 ? 1 : 0) + (f1 ? 1 : 0);
  if (f0 || f1) {
    const V dd = dd_num(p), pi = pi2_num(p);
    const V dz = dz_num(p, vfma(p.dA, p.dB, p.e));
    const V r4 = make_float2(f0 ? t0.y : 0.f, f1 ? t1.y : 0.f);
    acc[1] = vadd(acc[1], make_float2(f0 && pi.x != 0.f ? __fdividef(dd.x, pi.x) : 0.f,
                                      f1 && pi.y != 0.f ? __fdividef(dd.y, pi.y) : 0.f));
    acc[2] = vfma(dd, r4, acc[2]);
    acc[3] = vfma(dz, r4, acc[3]);
    acc[4] = vfma(pi, r4, acc[4]);
  }
  const bool s0 = live0 && si.w > 0.f && sj0.w > 0.f, s1 = live1 && si.w > 0.f && sj1.w > 0.f;
  if (s0 || s1) {
    // E = D v_i v_j from the integer c1 v_i v_j - n d_i d_j
    const V ns = p.ns;
    const V vv = make_float2(si.y * sj0.y, si.y * sj1.y), dd2 = make_float2(si.x * sj0.x, si.x * sj1.x);
    const V num = dot2(c1, vv, vneg(ns), dd2);
    const V Ev = vmul(num, make_float2(t0.x, t1.x));
    const float E0 = p.n0 > 0 ? Ev.x : -dd2.x, E1 = p.n1 > 0 ? Ev.y : -dd2.y;
    const V ww = make_float2(s0 ? si.w * sj0.w : 0.f, s1 ? si.w * sj1.w : 0.f);
    acc[5] = vfma(vmul(make_float2(E0, E1), make_float2(E0, E1)), ww, acc[5]);
  }
}

// window_pair2 for pairs whose two SNPs have the same valid haplotypes (the
// pair's n equals nv of both sites: every pair of a panel without missing
// data).  Then p_A, q_A, p_B, q_B are the sites' own counts, r^2 =
// x^2 / (p_A q_A p_B q_B) = x^2 u_i u_j, and the naive r^2 equals it
// (E = x), so one product serves both; DD, Dz, pi2 and sigma_D^2 as above.
// n is the row SNP's nv for both pairs: four = (nv_i >= 4) and r4 =
// 1/(n(n-1)(n-2)(n-3)) come from the caller, once per row.
__device__ __forceinline__ void window_pair2_same(const fast2::Pop& p, bool four, float r4n,
                                                  float4 si, float4 sj0, float4 sj1, bool live0,
                                                  bool live1, float2 (&acc)[6], int& n_pairs,
                                                  int& n_r2, int& n_four) {
  using namespace fast2;
  n_pairs += (live0 ? 1 : 0) + (live1 ? 1 : 0);
  const V uu = vmul(vs(si.w), make_float2(sj0.w, sj1.w));
  const bool r0 = live0 && uu.x > 0.f, r1 = live1 && uu.y > 0.f;
  n_r2 += (r0 ? 1 : 0) + (r1 ? 1 : 0);
  const V r2 = vmul(vmul(p.x, p.x), make_float2(live0 ? uu.x : 0.f, live1 ? uu.y : 0.f));
  acc[0] = vadd(acc[0], r2);
  acc[5] = vadd(acc[5], r2);
  const bool f0 = live0 && four, f1 = live1 && four;
  n_four += (f0 ? 1 : 0) + (f1 ? 1 : 0);
  if (f0 || f1) {
    const V dd = dd_num(p), pi = pi2_num(p);
    const V dz = dz_num(p, vfma(p.dA, p.dB, p.e));
    const V r4 = make_float2(f0 ? r4n : 0.f, f1 ? r4n : 0.f);
    acc[1] = vadd(acc[1], make_float2(f0 && pi.x != 0.f ? __fdividef(dd.x, pi.x) : 0.f,
                                      f1 && pi.y != 0.f ? __fdividef(dd.y, pi.y) : 0.f));
    acc[2] = vfma(dd, r4, acc[2]);
    acc[3] = vfma(dz, r4, acc[3]);
    acc[4] = vfma(pi, r4, acc[4]);
  }
}

// the value of one statistic of a pair (column stat of window_pair, 0 where
// window_pair adds nothing), the same arithmetic as window_pair
__device__ __forceinline__ float pair_stat(int stat, const fast::Pop& p, int n, float c1,
                                           float inv_n, float r4n, float4 si, float4 sj) {
  if (stat == 0) {
    const float rden = fast::x2_value(fast::x2_prod(p.pA * p.qA, p.pB * p.qB));
    return rden > 0.f ? __fdividef(fast::x2_value(fast::x2_prod(p.x, p.x)), rden) : 0.f;
  }
  if (stat <= 4) {
    if (n < 4) return 0.f;
    if (stat == 1) {
      const float pi = fast::pi2_num(p);
      return pi != 0.f ? __fdividef(fast::dd_num(p), pi) : 0.f;
    }
    if (stat == 2) return fast::dd_num(p) * r4n;
    if (stat == 3) return fast::dz_num(p) * r4n;
    return fast::pi2_num(p) * r4n;
  }
  if (!(si.w > 0.f && sj.w > 0.f)) return 0.f;
  float E;
  if (n > 0) {
    fast::X2 num = fast::x2_prod(c1, si.y * sj.y);
    fast::x2_add_prod(num, -(float)n, si.x * sj.x);
    E = fast::x2_value(num) * inv_n;
  } else {
    E = -(si.x * sj.x);
  }
  return (E * E) * (si.w * sj.w);
}

}  // namespace win
}  // namespace pgld
