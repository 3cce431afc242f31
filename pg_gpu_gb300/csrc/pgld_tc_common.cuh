// Epilogue helpers shared by the tensor-core band kernels: warp reductions,
// distance-bin lookup and the per-warp bin slots.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pgld {
namespace tc {

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ int bin_of_int(const int* thr, int n_bins, int d) {
  if (d < thr[0] || d >= thr[n_bins]) return -1;
  int lo = 0, hi = n_bins;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (thr[mid] <= d) lo = mid; else hi = mid;
  }
  return lo;
}
// bin_of_int of a distance d that every lane of the warp passes alike: lane l
// compares d with thresholds l and 32 + l, and the bin is the number of
// thresholds at or below d, less one (n_bins <= 64)
__device__ __forceinline__ int bin_of_int_warp(const int* thr, int n_bins, int d, int lane) {
  const bool a = lane <= n_bins && thr[lane] <= d;
  const bool b = 32 + lane <= n_bins && thr[32 + lane] <= d;
  int c = __popc(__ballot_sync(0xffffffffu, a)) + __popc(__ballot_sync(0xffffffffu, b));
  if (n_bins >= 64 && thr[64] <= d) ++c;
  return (c == 0 || c > n_bins) ? -1 : c - 1;
}
__device__ __forceinline__ int bin_of_f64(const double* sb, int n_bins, double d) {
  if (!(d >= sb[0]) || !(d < sb[n_bins])) return -1;
  int lo = 0, hi = n_bins;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (sb[mid] <= d) lo = mid; else hi = mid;
  }
  return lo;
}


// warp totals of S <= 16 values by recursive halving (16 shuffles for S = 15
// where a butterfly per value takes 75): each step sends the half of the values
// that the partner lane keeps; lane l ends with the total of value
// l >> totals_shift<S>()
template <int S>
__host__ __device__ constexpr int totals_width() {
  return S <= 1 ? 1 : S <= 2 ? 2 : S <= 4 ? 4 : S <= 8 ? 8 : 16;
}
template <int S>
__host__ __device__ constexpr int totals_shift() {
  return totals_width<S>() == 16 ? 1 : totals_width<S>() == 8 ? 2 : totals_width<S>() == 4 ? 3
                                                               : totals_width<S>() == 2 ? 4 : 5;
}
template <int S>
__device__ __forceinline__ float warp_totals(const float (&v)[S], int lane) {
  constexpr int K = totals_width<S>();
  static_assert(S <= 16, "at most 16 values");
  float w[K];
#pragma unroll
  for (int k = 0; k < K; ++k) w[k] = k < S ? v[k] : 0.f;
  int off = 16;
#pragma unroll
  for (int h = K / 2; h >= 1; h >>= 1, off >>= 1) {
    const bool up = (lane & off) != 0;
#pragma unroll
    for (int k = 0; k < h; ++k) {
      const float send = up ? w[k] : w[k + h];
      const float keep = up ? w[k + h] : w[k];
      w[k] = keep + __shfl_xor_sync(0xffffffffu, send, off);
    }
  }
  float t = w[0];
#pragma unroll
  for (; off >= 1; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
  return t;
}
#ifndef PGLD_TC_SLOTS_F64
#define PGLD_TC_SLOTS_F64 1
#endif
#if PGLD_TC_SLOTS_F64
typedef double Slot;
__device__ __forceinline__ void slot_add(Slot* s, float v) { *s += (double)v; }
__device__ __forceinline__ double slot_value(const Slot& s) { return s; }
__device__ __forceinline__ Slot slot_zero() { return 0.0; }
#else
// compensated (Neumaier) float32 slot: x = sum, y = running correction
typedef float2 Slot;
__device__ __forceinline__ void slot_add(Slot* slot, float v) {
  const float s = slot->x;
  const float t = __fadd_rn(s, v);
  const float bp = __fsub_rn(t, s);
  const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(v, bp));
  slot->x = t;
  slot->y = __fadd_rn(slot->y, err);
}
__device__ __forceinline__ double slot_value(const Slot& s) { return (double)s.x + (double)s.y; }
__device__ __forceinline__ Slot slot_zero() { return make_float2(0.f, 0.f); }
#endif

// the warp's totals of v added to the bin slots slot[0..S) (one lane per value)
template <int S>
__device__ __forceinline__ void warp_totals_add(const float (&v)[S], int lane, Slot* slot) {
  const float tot = warp_totals<S>(v, lane);
  constexpr int sh = totals_shift<S>();
  const int k = lane >> sh;
  if ((lane & ((1 << sh) - 1)) == 0 && k < S) slot_add(slot + k, tot);
}

}  // namespace tc
}  // namespace pgld
