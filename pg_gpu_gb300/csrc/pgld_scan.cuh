// Exclusive prefix sum of int64 counts, in place, n -> n+1 entries
// (entry n receives the total).  Three launches: tile sums, scan of the
// tile sums in one block, then the per-tile scans.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pgld_internal.cuh"

namespace pgld {

constexpr int kScanThreads = 512;
constexpr int kScanPerThread = 8;
constexpr long long kScanTile = (long long)kScanThreads * kScanPerThread;

inline size_t scan_scratch_bytes(long long n) {
  long long tiles = (n + kScanTile - 1) / kScanTile;
  return (size_t)(tiles + 1) * 8 + 256;
}

static __device__ __forceinline__ long long block_excl_scan(long long v, long long* sh, long long* total) {
  // sh: kScanThreads/32 + 1 entries
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    long long s = lane < kScanThreads / 32 ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      long long y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kScanThreads / 32) sh[lane] = s;
  }
  __syncthreads();
  long long before = (wid > 0 ? sh[wid - 1] : 0) + x - v;
  *total = sh[kScanThreads / 32 - 1];
  __syncthreads();
  return before;
}

static __global__ void __launch_bounds__(kScanThreads) scan_tile_sums(const long long* __restrict__ a,
                                                              long long n, long long* __restrict__ part) {
  __shared__ long long sh[kScanThreads / 32 + 1];
  long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanPerThread;
  long long s = 0;
#pragma unroll
  for (int q = 0; q < kScanPerThread; ++q)
    if (base + q < n) s += a[base + q];
  long long tot;
  block_excl_scan(s, sh, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

static __global__ void __launch_bounds__(kScanThreads) scan_partials(long long* __restrict__ part, long long m) {
  __shared__ long long sh[kScanThreads / 32 + 1];
  long long carry = 0;
  for (long long b = 0; b < m; b += kScanThreads) {
    long long k = b + threadIdx.x;
    long long v = k < m ? part[k] : 0;
    long long tot;
    long long e = block_excl_scan(v, sh, &tot);
    if (k < m) part[k] = carry + e;
    carry += tot;
  }
  if (threadIdx.x == 0) part[m] = carry;
}

static __global__ void __launch_bounds__(kScanThreads) scan_apply(long long* __restrict__ a, long long n,
                                                          const long long* __restrict__ part,
                                                          long long m) {
  __shared__ long long sh[kScanThreads / 32 + 1];
  long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanPerThread;
  long long v[kScanPerThread];
  long long s = 0;
#pragma unroll
  for (int q = 0; q < kScanPerThread; ++q) {
    v[q] = base + q < n ? a[base + q] : 0;
    s += v[q];
  }
  long long tot;
  long long e = block_excl_scan(s, sh, &tot) + part[blockIdx.x];
#pragma unroll
  for (int q = 0; q < kScanPerThread; ++q) {
    if (base + q < n) a[base + q] = e;
    e += v[q];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) a[n] = part[m];
}

inline int exclusive_scan_i64(pgld_context* h, long long* a, long long n, void* scratch,
                              size_t scratch_bytes, cudaStream_t st) {
  long long tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 0) {
    cudaMemsetAsync(a, 0, 8, st);
    return PGLD_OK;
  }
  if (scratch_bytes < scan_scratch_bytes(n))
    return pgld_fail(h, PGLD_ERR_INVALID_ARG, "scan scratch too small");
  long long* part = (long long*)scratch;
  scan_tile_sums<<<(unsigned)tiles, kScanThreads, 0, st>>>(a, n, part);
  scan_partials<<<1, kScanThreads, 0, st>>>(part, tiles);
  scan_apply<<<(unsigned)tiles, kScanThreads, 0, st>>>(a, n, part, tiles);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "exclusive_scan_i64");
  return PGLD_OK;
}

}  // namespace pgld
