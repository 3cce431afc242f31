// Internal declarations of libpgld: context, error plumbing, and the exact
// integer forms of the reference's two-locus statistics.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/pgld.h"

struct pgld_context {
  int device = 0;
  int n_sm = 0;
  void* ws = nullptr;       // device workspace owned by the handle
  size_t ws_bytes = 0;
  int32_t* dev_status = nullptr;  // device error word (bounded waits report here)
  std::string err;
  // device copies of the moments statistic term tables, one per population count
  pgld_term* spec_terms[PGLD_MAX_POPS + 1] = {nullptr};
  int spec_n_terms[PGLD_MAX_POPS + 1] = {0};
  int spec_n_stats[PGLD_MAX_POPS + 1] = {0};
  // the same tables with the genotype case kinds
  pgld_term* gspec_terms[PGLD_MAX_POPS + 1] = {nullptr};
  int gspec_n_terms[PGLD_MAX_POPS + 1] = {0};
  // per-launch timing of the dominant kernel of each call (off by default):
  // event pairs recorded around the launch on the call's stream
  int test_fault = 0;  // pgld_set_test_fault: one-shot hook of the next tensor-core launch
  // tensor-core configuration (pgld_set_tc_config): layout of the binned
  // two-population form (0 automatic, 1 64 x 64 tiles with one accumulator
  // per population, 2 64 x 128 tiles with one combined accumulator) and a cap
  // on the pipeline stages (0 = as many as shared memory holds)
  int tc_layout = 0;
  int tc_stages_cap = 0;
  bool timing = false;
  std::vector<cudaEvent_t> tev;
  int tev_used = 0;
  bool tev_overflow = false;
};

// --------------------------------------------------------------------------
// error plumbing (every entry point returns a status, never throws)
// --------------------------------------------------------------------------
int pgld_fail(pgld_context* h, int code, const char* fmt, ...);
int pgld_cuda_fail(pgld_context* h, cudaError_t e, const char* what);
int pgld_workspace(pgld_context* h, size_t bytes, void** out);
// event marks around the dominant kernel launch of a call (no-ops unless
// pgld_set_kernel_timing enabled timing on h)
void pgld_time_begin(pgld_context* h, cudaStream_t st);
void pgld_time_end(pgld_context* h, cudaStream_t st);

#define PGLD_CHECK_CUDA(h, expr)                              \
  do {                                                        \
    cudaError_t e_ = (expr);                                  \
    if (e_ != cudaSuccess) return pgld_cuda_fail((h), e_, #expr); \
  } while (0)

#define PGLD_REQUIRE(h, cond, ...)                                   \
  do {                                                               \
    if (!(cond)) return pgld_fail((h), PGLD_ERR_INVALID_ARG, __VA_ARGS__); \
  } while (0)

// moments statistic names / term tables (ld_pipeline.py:357-457)
int pgld_n_stats(int n_pops);
// geno: the genotype case kinds of compute_multi_pop_statistics_batch_geno
void pgld_build_spec_terms(int n_pops, std::vector<pgld_term>& out, bool geno = false);

// --------------------------------------------------------------------------
// exact integer per-population features and case formulas
// --------------------------------------------------------------------------
namespace pgld {

typedef long long i64;

struct PopC {
  i64 c1, c2, c3, c4, n;
  i64 pA, qA, pB, qB;
  i64 x;  // c1*c4 - c2*c3 (minus the reference's D, ld_pipeline.py:478)
};

__host__ __device__ __forceinline__ PopC make_pop(i64 c1, i64 c2, i64 c3, i64 c4, i64 n) {
  PopC p;
  p.c1 = c1; p.c2 = c2; p.c3 = c3; p.c4 = c4; p.n = n;
  p.pA = c1 + c2; p.qA = c3 + c4; p.pB = c1 + c3; p.qB = c2 + c4;
  p.x = c1 * c4 - c2 * c3;
  return p;
}

struct ND {
  i64 num, den;
};

__host__ __device__ __forceinline__ i64 d4(i64 n) { return n * (n - 1) * (n - 2) * (n - 3); }

// dd(i,i): c1(c1-1)c4(c4-1) + c2(c2-1)c3(c3-1) - 2 c1c2c3c4 written with
// a = c1c4, b = c2c3 so every product stays a 64-bit integer.
__host__ __device__ __forceinline__ ND dd_ii(const PopC& p) {
  i64 a = p.c1 * p.c4, b = p.c2 * p.c3;
  return {a * (a - p.c1 - p.c4 + 1) + b * (b - p.c2 - p.c3 + 1) - 2 * a * b, d4(p.n)};
}
__host__ __device__ __forceinline__ ND dd_ij(const PopC& a, const PopC& b) {
  return {a.x * b.x, a.n * (a.n - 1) * b.n * (b.n - 1)};
}
__host__ __device__ __forceinline__ ND dz_iii(const PopC& p) {
  i64 num = p.x * (p.qA - p.pA) * (p.qB - p.pB) + p.x * ((p.c2 + p.c3) - (p.c1 + p.c4)) +
            2 * (p.c2 * p.c3 + p.c1 * p.c4);
  return {num, d4(p.n)};
}
__host__ __device__ __forceinline__ ND dz_iij(const PopC& i, const PopC& j) {
  return {(i.qA - i.pA) * i.x * (j.qB - j.pB), j.n * i.n * (i.n - 1) * (i.n - 2)};
}
__host__ __device__ __forceinline__ ND dz_iji(const PopC& i, const PopC& j) {
  return {(i.qB - i.pB) * i.x * (j.qA - j.pA), j.n * i.n * (i.n - 1) * (i.n - 2)};
}
__host__ __device__ __forceinline__ ND dz_ijj(const PopC& i, const PopC& j) {
  i64 num = i.x * ((j.c2 + j.c3) - (j.c1 + j.c4)) + i.x * (j.qB - j.pB) * (j.qA - j.pA);
  return {num, i.n * (i.n - 1) * j.n * (j.n - 1)};
}
__host__ __device__ __forceinline__ ND dz_ijk(const PopC& i, const PopC& j, const PopC& k) {
  return {i.x * (j.pA - j.qA) * (k.pB - k.qB), i.n * (i.n - 1) * j.n * k.n};
}
__host__ __device__ __forceinline__ ND pi2_iiii(const PopC& p) {
  i64 num = p.pA * p.pB * p.qB * p.qA - p.c1 * p.c4 * (-1 + p.c1 + 3 * p.c2 + 3 * p.c3 + p.c4) -
            p.c2 * p.c3 * (-1 + 3 * p.c1 + p.c2 + p.c3 + 3 * p.c4);
  return {num, d4(p.n)};
}
// population t three times, s once
__host__ __device__ __forceinline__ ND pi2_triple(const PopC& t, const PopC& s) {
  i64 num = t.pA * t.qA * (t.qB * s.pB + t.pB * s.qB - 2 * s.qB) +
            (t.pA * t.c4 + t.c2 * t.qA) * (s.qB - s.pB);
  return {num, 2 * s.n * t.n * (t.n - 1) * (t.n - 2)};
}
__host__ __device__ __forceinline__ ND pi2_iikk(const PopC& i, const PopC& k) {
  return {i.pA * i.qA * k.pB * k.qB, i.n * (i.n - 1) * k.n * (k.n - 1)};
}
__host__ __device__ __forceinline__ ND pi2_iikk_sym(const PopC& i, const PopC& k) {
  return {i.pA * i.qA * k.pB * k.qB + k.pA * k.qA * i.pB * i.qB,
          2 * i.n * (i.n - 1) * k.n * (k.n - 1)};
}
__host__ __device__ __forceinline__ ND pi2_iikl(const PopC& i, const PopC& k, const PopC& l) {
  return {i.pA * i.qA * (k.pB * l.qB + k.qB * l.pB), 2 * i.n * (i.n - 1) * k.n * l.n};
}
__host__ __device__ __forceinline__ ND pi2_ijkk(const PopC& i, const PopC& j, const PopC& k) {
  return {k.pB * k.qB * (i.pA * j.qA + i.qA * j.pA), 2 * k.n * (k.n - 1) * i.n * j.n};
}
__host__ __device__ __forceinline__ ND pi2_ijij(const PopC& a, const PopC& b) {
  i64 a1 = a.c1, a2 = a.c2, a3 = a.c3, a4 = a.c4;
  i64 b1 = b.c1, b2 = b.c2, b3 = b.c3, b4 = b.c4;
  i64 quart = a.qB * a.qA * b.pA * b.pB + a.pB * a.qA * b.pA * b.qB + a.pA * a.qB * b.pB * b.qA +
              a.pA * a.pB * b.qB * b.qA;
  // cubic correction grouped by the b-count it multiplies
  i64 cub = b1 * (a4 - a2 * a3 - a2 * a4 - a3 * a4 - a4 * a4 - a4 * b1) +
            b2 * (a3 - a1 * a3 - a3 * a3 - a1 * a4 - a3 * a4 - a3 * b1 - a4 * b1 - a3 * b2) +
            b3 * (a2 - a1 * a2 - a2 * a2 - a1 * a4 - a2 * a4 - a2 * b1 - a4 * b1 - a1 * b2 -
                  a4 * b2 - a2 * b3) +
            b4 * (a1 - a1 * a1 - a1 * a2 - a1 * a3 - a2 * a3 - a2 * b1 - a3 * b1 - a1 * b2 -
                  a3 * b2 - a1 * b3 - a2 * b3 - a1 * b4);
  return {quart + cub, 4 * a.n * (a.n - 1) * b.n * (b.n - 1)};
}
// s in both pairs, a in the first pair, b in the second
__host__ __device__ __forceinline__ ND pi2_shared(const PopC& s, const PopC& a, const PopC& b) {
  i64 inner = (s.c3 - 1) * b.c1 + s.c3 * b.c2 - b.c3 + s.c3 * b.c3 + s.c3 * b.c4 + s.c1 * b.qB;
  i64 num = s.c4 * s.c4 * a.pA * b.pB + s.c2 * s.c2 * a.qA * b.pB +
            (s.c1 + s.c3 - 1) * (s.c3 * a.pA + s.c1 * a.qA) * b.qB +
            s.c4 * (s.c1 * a.qA * b.pB + (a.c1 + a.c2) * inner) +
            s.c2 * (s.c4 * (a.pA + a.qA) * b.pB + s.c3 * (a.pA * b.pB + a.qA * b.qB) +
                    a.qA * ((s.c1 - 1) * b.c1 - b.c3 + s.c1 * (b.c2 + b.c3 + b.c4)));
  return {num, 4 * s.n * (s.n - 1) * a.n * b.n};
}
__host__ __device__ __forceinline__ ND pi2_alldiff(const PopC& i, const PopC& j, const PopC& k,
                                                   const PopC& l) {
  return {(i.qA * j.pA + i.pA * j.qA) * (k.qB * l.pB + k.pB * l.qB), 4 * i.n * j.n * k.n * l.n};
}

// r family: exact forms of haplotype_kernels.py:20-62 (n is the valid n)
__host__ __device__ __forceinline__ i64 r_den(const PopC& p) {
  return p.pA * (p.n - p.pA) * p.pB * (p.n - p.pB);
}
__host__ __device__ __forceinline__ i64 dprime_den(const PopC& p) {
  i64 u, v;
  if (p.x >= 0) {
    u = p.pA * (p.n - p.pB);
    v = (p.n - p.pA) * p.pB;
  } else {
    u = p.pA * p.pB;
    v = (p.n - p.pA) * (p.n - p.pB);
  }
  return u < v ? u : v;
}

// case numerator / denominator of one term
__host__ __device__ __forceinline__ ND eval_case(int kind, const int* pp, const PopC* P) {
  switch (kind) {
    case PGLD_DD_II: return dd_ii(P[pp[0]]);
    case PGLD_DD_IJ: return dd_ij(P[pp[0]], P[pp[1]]);
    case PGLD_DZ_III: return dz_iii(P[pp[0]]);
    case PGLD_DZ_IIJ: return dz_iij(P[pp[0]], P[pp[1]]);
    case PGLD_DZ_IJI: return dz_iji(P[pp[0]], P[pp[1]]);
    case PGLD_DZ_IJJ: return dz_ijj(P[pp[0]], P[pp[1]]);
    case PGLD_DZ_IJK: return dz_ijk(P[pp[0]], P[pp[1]], P[pp[2]]);
    case PGLD_PI2_IIII: return pi2_iiii(P[pp[0]]);
    case PGLD_PI2_TRIPLE: return pi2_triple(P[pp[0]], P[pp[1]]);
    case PGLD_PI2_IIKK: return pi2_iikk(P[pp[0]], P[pp[1]]);
    case PGLD_PI2_IIKK_SYM: return pi2_iikk_sym(P[pp[0]], P[pp[1]]);
    case PGLD_PI2_IIKL: return pi2_iikl(P[pp[0]], P[pp[1]], P[pp[2]]);
    case PGLD_PI2_IJKK: return pi2_ijkk(P[pp[0]], P[pp[1]], P[pp[2]]);
    case PGLD_PI2_IJIJ: return pi2_ijij(P[pp[0]], P[pp[1]]);
    case PGLD_PI2_SHARED: return pi2_shared(P[pp[0]], P[pp[1]], P[pp[2]]);
    case PGLD_PI2_ALLDIFF: return pi2_alldiff(P[pp[0]], P[pp[1]], P[pp[2]], P[pp[3]]);
    default: return {0, 0};
  }
}

// value of one term in double: num/den, 0 when den <= 0; r family NaN
__device__ __forceinline__ double term_value_f64(int kind, const int* pp, const PopC* P) {
  if (kind >= PGLD_R) {
    const PopC& p = P[pp[0]];
    if (kind == PGLD_DPRIME) {
      i64 dm = dprime_den(p);
      return dm > 0 ? (double)p.x / (double)dm : __longlong_as_double(0x7ff8000000000000LL);
    }
    i64 den = r_den(p);
    if (den <= 0) return __longlong_as_double(0x7ff8000000000000LL);
    if (kind == PGLD_R) return (double)p.x / sqrt((double)den);
    return (double)(p.x * p.x) / (double)den;
  }
  ND v = eval_case(kind, pp, P);
  return v.den > 0 ? (double)v.num / (double)v.den : 0.0;
}

// 64-bit integer to float32 in two 32-bit conversions of the magnitude:
// |x| = hi * 2^31 + lo with 0 <= lo < 2^31; hi converts exactly while
// |x| < 2^55, lo and the fused sum round once each (at most two roundings, a
// relative error below 1.2e-7; no cancellation since both parts are
// non-negative).  The single-instruction 64-bit conversion runs at about two
// per SM per clock on GB300; this runs at the 32-bit conversion rate.
__device__ __forceinline__ float ll2f(i64 x) {
  const i64 ax = x < 0 ? -x : x;
  const int hi = (int)(ax >> 31);
  const int lo = (int)(ax & 0x7fffffffll);
  const float f = fmaf(__int2float_rn(hi), 2147483648.0f, __int2float_rn(lo));
  return x < 0 ? -f : f;
}

__device__ __forceinline__ float term_value_f32(int kind, const int* pp, const PopC* P) {
  if (kind >= PGLD_R) {
    const PopC& p = P[pp[0]];
    if (kind == PGLD_DPRIME) {
      i64 dm = dprime_den(p);
      return dm > 0 ? ll2f(p.x) / ll2f(dm) : __int_as_float(0x7fc00000);
    }
    i64 den = r_den(p);
    if (den <= 0) return __int_as_float(0x7fc00000);
    if (kind == PGLD_R) return ll2f(p.x) / sqrtf(ll2f(den));
    return ll2f(p.x * p.x) / ll2f(den);
  }
  ND v = eval_case(kind, pp, P);
  return v.den > 0 ? ll2f(v.num) / ll2f(v.den) : 0.0f;
}

}  // namespace pgld
