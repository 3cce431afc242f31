// Exact integer forms of the genotype (unphased diploid) two-locus statistics.
//
// Input per pair and population: the reference's 9-way counts n00 .. n22
// (dosage at the first SNP x 3 + dosage at the second, ld_pipeline.py:
// 183-217) and the pairwise-valid n.  The features use moments order
// g1 = n22, ..., g9 = n00 (genotype_kernels.py:423-435) and carry every half-
// or quarter-integer quantity of _PopDataGeno (genotype_kernels.py:437-521)
// scaled to a 64-bit integer, so each statistic is one exact integer
// numerator over one exact integer denominator, divided once:
//   P2 = 2 pA, R2 = 2 qA, Q2 = 2 pB, S2 = 2 qB,
//   X00, X01, X10, X11 = 4 x_AB, 4 x_Ab, 4 x_aB, 4 x_ab,  D16 = 16 D_geno.
// All numerators and denominators stay below 2^62 for populations of at most
// kMaxGenoN individuals.
#pragma once
#include <stdint.h>

#include "pgld_geno_mom.cuh"
#include "pgld_internal.cuh"

namespace pgld {
namespace geno {

constexpr int kMaxGenoN = 8192;

struct GPop {
  int g[10];  // g1..g9 and g[9] = 1
  i64 ns;     // sum of the 9 counts (single-population kernels gate on it)
  i64 n;      // valid n (n_valid when given, else ns)
  i64 P2, R2, Q2, S2;
  i64 X00, X01, X10, X11, D16;
  i64 a, b;  // fdA, fdB of the Dz precompute (genotype_kernels.py:176-197)
};

// c: the reference's column order n00, n01, ..., n22
__host__ __device__ __forceinline__ GPop make_gpop(const int* c, i64 n_valid) {
  GPop p;
#pragma unroll
  for (int k = 0; k < 9; ++k) p.g[k] = c[8 - k];
  p.g[9] = 1;
  const i64 g1 = p.g[0], g2 = p.g[1], g3 = p.g[2], g4 = p.g[3], g5 = p.g[4], g6 = p.g[5],
            g7 = p.g[6], g8 = p.g[7], g9 = p.g[8];
  p.ns = g1 + g2 + g3 + g4 + g5 + g6 + g7 + g8 + g9;
  p.n = n_valid >= 0 ? n_valid : p.ns;
  p.P2 = 2 * (g1 + g2 + g3) + g4 + g5 + g6;
  p.R2 = g4 + g5 + g6 + 2 * (g7 + g8 + g9);
  p.Q2 = 2 * (g1 + g4 + g7) + g2 + g5 + g8;
  p.S2 = g2 + g5 + g8 + 2 * (g3 + g6 + g9);
  p.X00 = 4 * g1 + 2 * g2 + 2 * g4 + g5;
  p.X01 = 2 * g2 + 4 * g3 + g5 + 2 * g6;
  p.X10 = 2 * g4 + g5 + 4 * g7 + 2 * g8;
  p.X11 = g5 + 2 * g6 + 2 * g8 + 4 * g9;
  p.D16 = p.X00 * p.X11 - p.X01 * p.X10;
  p.a = -g1 + g3 - g4 + g6 - g7 + g9;
  p.b = -g1 - g2 - g3 + g7 + g8 + g9;
  return p;
}

// 16 Ucoef / 16 Vcoef / Wjj of the Dz precompute (genotype_kernels.py:176-197)
__host__ __device__ __forceinline__ i64 u16(const GPop& p) {
  const i64 g1 = p.g[0], g2 = p.g[1], g3 = p.g[2], g4 = p.g[3], g5 = p.g[4], g6 = p.g[5],
            g7 = p.g[6], g8 = p.g[7], g9 = p.g[8];
  const i64 mah = g7 * (g2 + 2 * g3 + g5 + 2 * g6) + g8 * (g3 + g6 - g1 - g4) -
                  g9 * (2 * g1 + g2 + 2 * g4 + g5);
  return p.D16 * (1 + p.b) + 8 * mah;
}
__host__ __device__ __forceinline__ i64 v16(const GPop& p) {
  const i64 g1 = p.g[0], g2 = p.g[1], g3 = p.g[2], g4 = p.g[3], g5 = p.g[4], g6 = p.g[5],
            g7 = p.g[6], g8 = p.g[7], g9 = p.g[8];
  const i64 mbh = g3 * (g4 + g5) - g6 * (g1 + g2) + (g7 + g8) * (2 * g3 + g6) -
                  g9 * (2 * g1 + 2 * g2 + g4 + g5);
  return p.D16 * (1 + p.a) + 8 * mbh;
}
__host__ __device__ __forceinline__ i64 wjj(const GPop& p) {
  return (i64)(-p.g[0] + p.g[2] + p.g[6] - p.g[8]) + p.a * p.b;
}
// 4 n (n-1) B_L, 4 n (n-1) B_R, and their denominator max(4 n (n-1), 1)
__host__ __device__ __forceinline__ i64 bl4(const GPop& p) {
  return p.P2 * p.R2 - (i64)(p.g[3] + p.g[4] + p.g[5]);
}
__host__ __device__ __forceinline__ i64 br4(const GPop& p) {
  return p.Q2 * p.S2 - (i64)(p.g[1] + p.g[4] + p.g[7]);
}
__host__ __device__ __forceinline__ i64 mden(const GPop& p) {
  const i64 m = 4 * p.n * (p.n - 1);
  return m > 1 ? m : 1;
}

// A statistic value num / den.  gated: 0 unless `ok` (the reference's n
// thresholds); ungated values divide in IEEE arithmetic like the reference's
// unguarded kernels (den 0 gives +-inf or NaN).
struct GV {
  i64 num, den;
  bool ok, gated;
};

__host__ __device__ __forceinline__ GV gv(i64 num, i64 den, bool ok) { return {num, den, ok, true}; }
__host__ __device__ __forceinline__ GV gv_ieee(i64 num, i64 den) { return {num, den, true, false}; }

// The single-population DD, Dz and pi2 through the centred moments of the
// pair (pgld_geno_mom.cuh): the same exact numerators as the reference's
// degree-4 polynomials in the nine counts, in a few dozen integer operations.
__host__ __device__ __forceinline__ gmom::Mom mom_of(const GPop& p) {
  int c[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) c[k] = p.g[8 - k];
  return gmom::from_counts(c);
}

// ---- DD (genotype_kernels.py:27-83) ----
__host__ __device__ __forceinline__ GV dd_single(const GPop& p) {
  const gmom::Mom o = mom_of(p);
  return gv(gmom::dd_num(o, gmom::terms(o)), 4 * d4(p.ns), p.ns >= 4);
}
__host__ __device__ __forceinline__ GV dd_between(const GPop& A, const GPop& B) {
  const i64 den = A.n * (A.n - 1) * B.n * (B.n - 1);
  return gv(A.D16 * B.D16, 64 * den, den > 0);
}

// ---- Dz (genotype_kernels.py:176-276, cases of compute_all_dz_geno) ----
__host__ __device__ __forceinline__ GV dz_single(const GPop& p) {
  const gmom::Mom o = mom_of(p);
  return gv(gmom::dz_num(o, gmom::terms(o)), 2 * d4(p.ns), p.ns >= 4);
}
__host__ __device__ __forceinline__ GV dz_iik(const GPop& I, const GPop& K) {
  return gv_ieee(u16(I) * K.a, 8 * K.n * I.n * (I.n - 1) * (I.n - 2));
}
__host__ __device__ __forceinline__ GV dz_iji(const GPop& I, const GPop& J) {
  return gv_ieee(v16(I) * J.b, 8 * J.n * I.n * (I.n - 1) * (I.n - 2));
}
__host__ __device__ __forceinline__ GV dz_ijj(const GPop& I, const GPop& J) {
  return gv_ieee(I.D16 * wjj(J), 8 * J.n * (J.n - 1) * I.n * (I.n - 1));
}
__host__ __device__ __forceinline__ GV dz_ijk(const GPop& I, const GPop& J, const GPop& K) {
  return gv_ieee(I.D16 * J.b * K.a, 8 * I.n * (I.n - 1) * J.n * K.n);
}

// ---- pi2 (genotype_kernels.py:279-398, cases of compute_all_pi2_geno) ----
__host__ __device__ __forceinline__ i64 pi2_single_num(const GPop& p) {
  const gmom::Mom o = mom_of(p);
  return gmom::pi2_num(o, gmom::terms(o));
}
__host__ __device__ __forceinline__ GV pi2_single(const GPop& p) {
  return gv(pi2_single_num(p), 16 * d4(p.ns), p.ns >= 4);
}
// pi2 with population t three times and s once; first: the calls with
// (i, j) = (t, t) (AQ3 / AS3), otherwise BP3 / BR3 (genotype_kernels.py:500-521)
__host__ __device__ __forceinline__ GV pi2_triple(const GPop& T, const GPop& S, bool first) {
  const i64 g2 = T.g[1], g3 = T.g[2], g4 = T.g[3], g5 = T.g[4], g6 = T.g[5], g7 = T.g[6],
            g8 = T.g[7], g9 = T.g[8];
  const i64 L0 = g5 + 2 * g6 + 2 * g8 + 4 * g9;
  i64 num;
  if (first) {
    const i64 L1 = g5 + 2 * g6;
    const i64 nR3 = 3 * (g4 + g5 + g6) + 4 * (g7 + g8 + g9);
    const i64 nR5 = 5 * (g4 + g5 + g6) + 8 * (g7 + g8 + g9);
    const i64 b5 = -2 * g2 - 4 * g3 + 4 * g4 + g5 - 2 * g6 + 8 * g7 + 4 * g8 + 4;
    const i64 b6 = -g5 - 2 * g6 - 4 * g7 - 4 * g8 - 4 * g9;
    const i64 aq = -T.S2 * nR3 + T.P2 * T.S2 * T.R2 + T.R2 * L0 + 2 * L1 - T.P2 * L0;
    const i64 as = -T.Q2 * nR5 + T.P2 * T.Q2 * T.R2 + T.R2 * b5 + 2 * b6 + T.P2 * L0;
    num = aq * S.Q2 + as * S.S2;
  } else {
    const i64 M1 = g5 + 2 * g8;
    const i64 nL3 = 3 * (g2 + g5 + g8) + 4 * (g3 + g6 + g9);
    const i64 nL5 = 5 * (g2 + g5 + g8) + 8 * (g3 + g6 + g9);
    const i64 b5 = 4 * g2 + 8 * g3 - 2 * g4 + g5 + 4 * g6 - 4 * g7 - 2 * g8 + 4;
    const i64 b6 = -4 * g3 - g5 - 4 * g6 - 2 * g8 - 4 * g9;
    const i64 bp = -T.R2 * nL3 + T.Q2 * T.S2 * T.R2 + T.S2 * L0 + 2 * M1 - T.Q2 * L0;
    const i64 br = -T.P2 * nL5 + T.P2 * T.Q2 * T.S2 + T.S2 * b5 + 2 * b6 + T.Q2 * L0;
    num = bp * S.P2 + br * S.R2;
  }
  const i64 d = T.n * (T.n - 1) * (T.n - 2) * S.n;
  return gv(num, 32 * d, d > 0);
}
__host__ __device__ __forceinline__ GV pi2_iikk(const GPop& I, const GPop& K) {
  return gv_ieee(bl4(I) * br4(K), mden(I) * mden(K));
}
__host__ __device__ __forceinline__ GV pi2_iikl(const GPop& I, const GPop& K, const GPop& L) {
  return gv_ieee(bl4(I) * (K.Q2 * L.S2 + K.S2 * L.Q2), mden(I) * 8 * K.n * L.n);
}
__host__ __device__ __forceinline__ GV pi2_ijkk(const GPop& I, const GPop& J, const GPop& K) {
  return gv_ieee((I.P2 * J.R2 + I.R2 * J.P2) * br4(K), 8 * I.n * J.n * mden(K));
}
// 64 x the numerator of _PI2_IJIJ_KERN (genotype_kernels.py:341-361)
__host__ __device__ __forceinline__ GV pi2_ijij(const GPop& A, const GPop& B) {
  const i64 PQa = A.P2 * A.Q2, RSa = A.R2 * A.S2, PSa = A.P2 * A.S2, QRa = A.Q2 * A.R2,
            PRa = A.P2 * A.R2;
  const i64 PQb = B.P2 * B.Q2, RSb = B.R2 * B.S2, PSb = B.P2 * B.S2, QRb = B.Q2 * B.R2;
  const i64 Ta = A.R2 * (4 + A.X01 - A.X10), Ua = A.S2 * (2 + A.R2);
  const i64 Bsa = A.X00 - A.X01 - A.X10 + A.X11, Bsb = B.X00 - B.X01 - B.X10 + B.X11;
  const i64 num = -2 * RSa * B.Q2 - A.X11 * PQb + RSa * PQb - 2 * A.R2 * PSb -
                  PQa * B.X11 - RSa * B.X11 + PSa * B.X11 + QRa * B.X11 -
                  2 * PRa * B.S2 + Ta * B.S2 + A.X11 * PSb + QRa * PSb +
                  2 * Ua * B.R2 - A.X01 * QRb + PSa * QRb -
                  2 * PSa * B.R2 - 2 * A.P2 * RSb + A.X01 * RSb + PQa * RSb +
                  A.X11 * Bsb + Bsa * B.X11 - 4 * A.X11 * B.X11;
  const i64 d = A.n * (A.n - 1) * B.n * (B.n - 1);
  return gv(num, 64 * d, d > 0);
}
// pops = (shared s, a, b) as the shared-case role selection
__host__ __device__ __forceinline__ GV pi2_shared(const GPop& S, const GPop& A, const GPop& B) {
  const i64 c00 = S.P2 * S.Q2 - S.X00, c01 = S.P2 * S.S2 - S.X01;
  const i64 c10 = S.R2 * S.Q2 - S.X10, c11 = S.R2 * S.S2 - S.X11;
  const i64 num = A.R2 * (c00 * B.S2 + c01 * B.Q2) + A.P2 * (c10 * B.S2 + c11 * B.Q2);
  return gv_ieee(num, 16 * mden(S) * A.n * B.n);
}
__host__ __device__ __forceinline__ GV pi2_alldiff(const GPop& I, const GPop& J, const GPop& K,
                                                    const GPop& L) {
  return gv_ieee((I.P2 * J.R2 + I.R2 * J.P2) * (K.Q2 * L.S2 + K.S2 * L.Q2),
                 64 * I.n * J.n * K.n * L.n);
}

// DD / pi2 of one population (genotype_kernels.py:91-169): NaN unless n >= 4
// and the pi2 numerator is positive
__host__ __device__ __forceinline__ GV sigma_d2(const GPop& p) {
  const gmom::Mom o = mom_of(p);
  const gmom::Terms t = gmom::terms(o);
  const i64 pn = gmom::pi2_num(o, t);
  // DD / pi2 = [dd_num / (4 d4)] / [pn / (16 d4)] = 4 dd_num / pn
  return gv(4 * gmom::dd_num(o, t), pn, p.ns >= 4 && pn > 0);
}

// Rogers-Huff r: exact moments of the individuals valid at both SNPs; with no
// missing dosage this is the reference's rogers_huff_r (ld_statistics.py:410-443)
struct RH {
  i64 cov, vi, vj;
};
__host__ __device__ __forceinline__ RH rh_moments(const int* c) {
  i64 n = 0, si = 0, sj = 0, sii = 0, sjj = 0, sij = 0;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const i64 v = c[3 * a + b];
      n += v;
      si += a * v;
      sj += b * v;
      sii += a * a * v;
      sjj += b * b * v;
      sij += a * b * v;
    }
  return {n * sij - si * sj, n * sii - si * si, n * sjj - sj * sj};
}

#ifdef __CUDACC__
// float32 value of a statistic (at most five roundings: two per conversion)
__device__ __forceinline__ float gv_f32(const GV& v) {
  if (v.gated && !v.ok) return 0.f;
  return ll2f(v.num) / ll2f(v.den);
}
// Rogers-Huff r^2 in float32, NaN where a SNP has no variance among the valid
__device__ __forceinline__ float rh2_f32(const int* c) {
  const RH m = rh_moments(c);
  const i64 den = m.vi * m.vj;
  if (den <= 0) return __int_as_float(0x7fc00000);
  return ll2f(m.cov * m.cov) / ll2f(den);
}
#endif

// ---------------------------------------------------------------------------
// statistic terms
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ GV term_gv(int kind, const int32_t* pp, const GPop* P) {
  switch (kind) {
    case PGLD_G_DD_II: return dd_single(P[pp[0]]);
    case PGLD_G_DD_IJ: return dd_between(P[pp[0]], P[pp[1]]);
    case PGLD_G_DZ_III: return dz_single(P[pp[0]]);
    case PGLD_G_DZ_IIJ: return dz_iik(P[pp[0]], P[pp[1]]);
    case PGLD_G_DZ_IJI: return dz_iji(P[pp[0]], P[pp[1]]);
    case PGLD_G_DZ_IJJ: return dz_ijj(P[pp[0]], P[pp[1]]);
    case PGLD_G_DZ_IJK: return dz_ijk(P[pp[0]], P[pp[1]], P[pp[2]]);
    case PGLD_G_PI2_IIII: return pi2_single(P[pp[0]]);
    case PGLD_G_PI2_IIIJ: return pi2_triple(P[pp[0]], P[pp[1]], true);
    case PGLD_G_PI2_IJII: return pi2_triple(P[pp[0]], P[pp[1]], false);
    case PGLD_G_PI2_IIKK: return pi2_iikk(P[pp[0]], P[pp[1]]);
    case PGLD_G_PI2_IIKL: return pi2_iikl(P[pp[0]], P[pp[1]], P[pp[2]]);
    case PGLD_G_PI2_IJKK: return pi2_ijkk(P[pp[0]], P[pp[1]], P[pp[2]]);
    case PGLD_G_PI2_IJIJ: return pi2_ijij(P[pp[0]], P[pp[1]]);
    case PGLD_G_PI2_SHARED: return pi2_shared(P[pp[0]], P[pp[1]], P[pp[2]]);
    default: return pi2_alldiff(P[pp[0]], P[pp[1]], P[pp[2]], P[pp[3]]);
  }
}

__device__ __forceinline__ double gv_f64(const GV& v) {
  if (v.gated && !v.ok) return 0.0;
  return __ll2double_rn(v.num) / __ll2double_rn(v.den);
}

// r or r^2 of Rogers-Huff, NaN where a SNP has no variance among the valid
__device__ __forceinline__ double rh_f64(const int* c, bool square) {
  const RH m = rh_moments(c);
  const i64 den = m.vi * m.vj;
  if (den <= 0) return __longlong_as_double(0x7ff8000000000000ll);
  if (square) return __ll2double_rn(m.cov * m.cov) / __ll2double_rn(den);
  return __ll2double_rn(m.cov) / sqrt(__ll2double_rn(den));
}

template <typename T>
__device__ __forceinline__ T term_value(const pgld_term& tm, const GPop* P, const int* const* cc) {
  if (tm.kind == PGLD_G_SIGMA_D2) {
    const GV v = sigma_d2(P[tm.pops[0]]);
    if (!v.ok) return (T)__longlong_as_double(0x7ff8000000000000ll);
    return sizeof(T) == 8 ? (T)(__ll2double_rn(v.num) / __ll2double_rn(v.den))
                          : (T)(ll2f(v.num) / ll2f(v.den));
  }
  if (tm.kind == PGLD_G_RH_R || tm.kind == PGLD_G_RH_R2) {
    if (sizeof(T) == 4 && tm.kind == PGLD_G_RH_R2) return (T)rh2_f32(cc[tm.pops[0]]);
    return (T)rh_f64(cc[tm.pops[0]], tm.kind == PGLD_G_RH_R2);
  }
  const GV v = term_gv(tm.kind, tm.pops, P);
  return sizeof(T) == 8 ? (T)gv_f64(v) : (T)gv_f32(v);
}

}  // namespace geno
}  // namespace pgld
