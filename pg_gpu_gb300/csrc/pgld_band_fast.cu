// Plain (AND + popcount) band kernel for one or two populations, with the
// float32 epilogue of pgld_epilogue.cuh.
//
// Per 32 x 32 SNP tile: the carrier / reference planes of both SNP blocks are
// staged in shared memory (transposed to [word][snp]), each thread counts four
// pairs (one j, four i) with AND + POPC, then finalises them in float32 from
// exact integer numerators.  Distances are exact integers when the positions
// are (the usual base-pair case): bins then use integer thresholds
// ceil(bins[k]), identical to digitize on float64.  A tile whose pairs all fall
// into one bin skips the per-pair bin search; each warp keeps private float64
// bin accumulators in shared memory (no atomics), merged once per CTA.
#include <cuda_runtime.h>

#include <algorithm>

#include "pgld_band.cuh"
#include "pgld_epilogue.cuh"
#include "pgld_internal.cuh"

namespace pgld {

namespace {

constexpr int kKW = 32;
constexpr int kPitch = 36;  // multiple of 4: 16-byte aligned rows for 4-SNP vector loads
constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;

struct __align__(16) FastSmem {
  uint32_t ci[kKW][kPitch], zi[kKW][kPitch], cj[kKW][kPitch], zj[kKW][kPitch];
  double bins[kMaxBins + 1];
  int thr[kMaxBins + 1];  // ceil(bins[k]) for integer distances
  int reli[kTile], relj[kTile];
  int tile_int;           // every position of the tile is an integer offset
  int tile_bin;           // the single bin of every pair, or -1
};

__device__ __forceinline__ void stage_t(uint32_t (*dst)[kPitch], const uint32_t* __restrict__ src,
                                        long long s0, long long n_snp, long long stride, int w0,
                                        int W) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kTile / kWarps; ++q) {
    const int sl = wid * (kTile / kWarps) + q;
    const long long s = s0 + sl;
    const int w = w0 + lane;
    uint32_t v = 0;
    if (s < n_snp && w < W) v = __ldg(src + s * stride + w);
    dst[lane][sl] = v;
  }
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

__device__ __forceinline__ int bin_of_f64(const double* sb, int n_bins, double d) {
  if (!(d >= sb[0]) || !(d < sb[n_bins])) return -1;
  int lo = 0, hi = n_bins;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (sb[mid] <= d) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// count (< 2^22) to float32 without the conversion pipe
__device__ __forceinline__ float cnt_f(int v) { return __int_as_float(0x4B400000 + v) - 12582912.0f; }

__device__ __forceinline__ fast::Pop pop_of(const int (&c)[4]) {
  return fast::make(cnt_f(c[0]), cnt_f(c[1]), cnt_f(c[2]), cnt_f(c[3]));
}

template <int P>
__device__ __forceinline__ void pair_stats(const int (&c)[P][4], const fast::Recip& T, float* s) {
  const fast::Pop p0 = pop_of(c[0]);
  if (P == 1) {
    fast::stats1(p0, T, s);
  } else {
    fast::stats2(p0, pop_of(c[P - 1]), T, s);
  }
}

// per-CTA reciprocal tables for n = 0..nmax, after the bin accumulators
__device__ __forceinline__ fast::Recip build_recip(float* base, int nmax, int tid, int nthreads) {
  fast::Recip T;
  float* inv = base;
  float* r2 = base + (nmax + 1);
  float* r3 = base + 2 * (nmax + 1);
  float* r4 = base + 3 * (nmax + 1);
  for (int n = tid; n <= nmax; n += nthreads) fast::recip_entry(n, inv + n, r2 + n, r3 + n, r4 + n);
  T.inv = inv;
  T.r2 = r2;
  T.r3 = r3;
  T.r4 = r4;
  return T;
}

template <int P, int MODE>
__global__ void __launch_bounds__(kThreads) band_fast_kernel(BandArgs a) {
  constexpr int S = (P == 1) ? 3 : 15;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FastSmem& sm = *reinterpret_cast<FastSmem*>(smem_raw);
  double* accw = reinterpret_cast<double*>(smem_raw + sizeof(FastSmem));  // [warp][bin][S]
  unsigned long long* cntw =
      reinterpret_cast<unsigned long long*>(accw + (MODE == kModeBinned ? kWarps * a.n_bins * S : 0));
  float* tables = reinterpret_cast<float*>(cntw + (MODE == kModeBinned ? kWarps * a.n_bins : 0));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int n_bins = a.n_bins;
  const fast::Recip T = build_recip(tables, a.nmax, threadIdx.x, kThreads);

  if (MODE == kModeBinned) {
    for (int x = threadIdx.x; x < kWarps * n_bins * S; x += kThreads) accw[x] = 0.0;
    for (int x = threadIdx.x; x < kWarps * n_bins; x += kThreads) cntw[x] = 0ull;
    for (int x = threadIdx.x; x <= n_bins; x += kThreads) {
      const double b = a.bins[x];
      sm.bins[x] = b;
      const double cb = ceil(b);
      sm.thr[x] = cb > 2147483647.0 ? 2147483647 : (cb < -2147483647.0 ? -2147483647 : (int)cb);
    }
  }
  __syncthreads();
  long long n_items = a.item_off[a.n_blocks];
  if (n_items < 0 || n_items > a.n_blocks * (a.n_blocks + 1) / 2) {
    if (threadIdx.x == 0 && a.status) atomicCAS(a.status, 0, 2001);
    n_items = 0;
  }
  // binned mode over an anchor range: the row blocks holding anchors only
  const long long n_anchor = MODE == kModeBinned ? anchors_of(a) : a.n_snp;
  if (n_items > 0 && n_anchor < a.n_snp) n_items = a.item_off[(n_anchor + kTile - 1) / kTile];
  const double maxd = a.max_dist;
  const int maxd_int = maxd >= 2147483647.0 ? 2147483647 : (int)floor(maxd);

  for (long long item = blockIdx.x; item < n_items; item += gridDim.x) {
    long long lo = 0, hi = a.n_blocks;
    while (hi - lo > 1) {
      const long long mid = (lo + hi) >> 1;
      if (a.item_off[mid] <= item) lo = mid; else hi = mid;
    }
    const long long bi = lo, bj = bi + (item - a.item_off[bi]);
    const long long i0 = bi * kTile, j0 = bj * kTile;
    __syncthreads();  // the previous tile's epilogue has read the tile metadata

    // tile coordinates: integer offsets from pos[i0] when exact
    bool is_int = true;
    if (threadIdx.x < 2 * kTile) {
      const int t = threadIdx.x & (kTile - 1);
      const long long s = (threadIdx.x < kTile ? i0 : j0) + t;
      int r = 0;
      if (s < a.n_snp) {
        const double rel = a.pos[s] - a.pos[i0];
        is_int = (rel == rint(rel)) && fabs(rel) < 1073741824.0;
        r = is_int ? (int)rel : 0;
      }
      if (threadIdx.x < kTile) sm.reli[t] = r; else sm.relj[t] = r;
    }
    const int all_int = __syncthreads_and(is_int ? 1 : 0) && (a.bcoord == nullptr);
    if (threadIdx.x == 0) {
      sm.tile_int = all_int;
      int tb = -1;
      if (MODE == kModeBinned && all_int && bj > bi && j0 + kTile <= a.n_snp &&
          i0 + kTile <= n_anchor) {
        const int dmin = sm.relj[0] - sm.reli[kTile - 1];
        const int dmax = sm.relj[kTile - 1] - sm.reli[0];
        if (dmax <= maxd_int) {
          const int b0 = bin_of_int(sm.thr, n_bins, dmin);
          if (b0 >= 0 && b0 == bin_of_int(sm.thr, n_bins, dmax)) tb = b0;
        }
      }
      sm.tile_bin = tb;
    }

    int c[P][4][4];
#pragma unroll
    for (int p = 0; p < P; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) c[p][q][0] = c[p][q][1] = c[p][q][2] = c[p][q][3] = 0;

#pragma unroll
    for (int p = 0; p < P; ++p) {
      const int W = a.W[p];
      const uint32_t* pl = a.planes[p];
      for (int w0 = 0; w0 < W; w0 += kKW) {
        __syncthreads();  // previous chunk consumed (and the tile metadata written)
        stage_t(sm.ci, pl, i0, a.n_snp, 2 * W, w0, W);
        stage_t(sm.zi, pl + W, i0, a.n_snp, 2 * W, w0, W);
        stage_t(sm.cj, pl, j0, a.n_snp, 2 * W, w0, W);
        stage_t(sm.zj, pl + W, j0, a.n_snp, 2 * W, w0, W);
        __syncthreads();
        const int nw = min(kKW, W - w0);
#pragma unroll 4
        for (int w = 0; w < nw; ++w) {
          const uint32_t cj = sm.cj[w][lane], zj = sm.zj[w][lane];
          const uint4 ci4 = *reinterpret_cast<const uint4*>(&sm.ci[w][wid * 4]);
          const uint4 zi4 = *reinterpret_cast<const uint4*>(&sm.zi[w][wid * 4]);
          const uint32_t ci[4] = {ci4.x, ci4.y, ci4.z, ci4.w};
          const uint32_t zi[4] = {zi4.x, zi4.y, zi4.z, zi4.w};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            c[p][q][0] += __popc(ci[q] & cj);
            c[p][q][1] += __popc(ci[q] & zj);
            c[p][q][2] += __popc(zi[q] & cj);
            c[p][q][3] += __popc(zi[q] & zj);
          }
        }
      }
    }

    // ---- epilogue: thread (wid, lane) owns pairs (i0 + 4*wid + q, j0 + lane) ----
    const int tile_bin = sm.tile_bin;
    if (MODE == kModeBinned && tile_bin >= 0) {
      float acc[S];
#pragma unroll
      for (int s = 0; s < S; ++s) acc[s] = 0.f;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int cq[P][4];
#pragma unroll
        for (int p = 0; p < P; ++p)
#pragma unroll
          for (int k = 0; k < 4; ++k) cq[p][k] = c[p][q][k];
        float st[S];
        pair_stats<P>(cq, T, st);
#pragma unroll
        for (int s = 0; s < S; ++s) acc[s] += st[s];
      }
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const float v = warp_sum(acc[s]);
        if (lane == 0) accw[(wid * n_bins + tile_bin) * S + s] += (double)v;
      }
      if (lane == 0) cntw[wid * n_bins + tile_bin] += 32ull * 4ull;
      continue;
    }
    const bool tint = sm.tile_int;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int il = wid * 4 + q;
      const long long i = i0 + il, j = j0 + lane;
      bool ok = (i < j) && (j < a.n_snp) && (i < n_anchor);
      int b = -1;
      if (tint) {
        const int d = sm.relj[lane] - sm.reli[il];
        ok = ok && d <= maxd_int;
        if (MODE == kModeBinned && ok) b = bin_of_int(sm.thr, n_bins, d);
      } else if (ok) {
        const double dp = a.pos[j] - a.pos[i];
        ok = dp <= maxd;
        if (MODE == kModeBinned && ok) {
          const double d = a.bcoord ? fabs(a.bcoord[j] - a.bcoord[i]) : dp;
          b = bin_of_f64(sm.bins, n_bins, d);
        }
      }
      int cq[P][4];
#pragma unroll
      for (int p = 0; p < P; ++p)
#pragma unroll
        for (int k = 0; k < 4; ++k) cq[p][k] = c[p][q][k];
      if (MODE == kModePairs) {
        // rows come from the band offsets: write exactly the pairs they list
        if (i < j && j < a.n_snp) ok = (j - i - 1) < (a.pair_off[i + 1] - a.pair_off[i]);
        if (ok) {
          const long long k = a.pair_off[i] + (j - i - 1);
          reinterpret_cast<int4*>(a.counts)[k] = make_int4(cq[0][0], cq[0][1], cq[0][2], cq[0][3]);
          const int n = cq[0][0] + cq[0][1] + cq[0][2] + cq[0][3];
          if (a.nvalid) a.nvalid[k] = n;
          if (a.stats) {
            const fast::Pop p0 = pop_of(cq[0]);
            float st[3];
            fast::stats1(p0, T, st);
            const float r2 = fast::r2_of(p0);
            reinterpret_cast<float4*>(a.stats)[k] = make_float4(r2, st[0], st[1], st[2]);
          }
        }
      } else {
        float st[S];
        pair_stats<P>(cq, T, st);
        unsigned pending = __ballot_sync(0xffffffffu, b >= 0);
        while (pending) {
          const int bb = __shfl_sync(0xffffffffu, b, __ffs(pending) - 1);
          const bool mine = (b == bb);
          const unsigned grp = __ballot_sync(0xffffffffu, mine);
#pragma unroll
          for (int s = 0; s < S; ++s) {
            const float v = warp_sum(mine ? st[s] : 0.f);
            if (lane == 0) accw[(wid * n_bins + bb) * S + s] += (double)v;
          }
          if (lane == 0) cntw[wid * n_bins + bb] += (unsigned long long)__popc(grp);
          pending &= ~grp;
        }
      }
    }
  }

  if (MODE == kModeBinned) {
    __syncthreads();
    for (int x = threadIdx.x; x < n_bins * S; x += kThreads) {
      double v = 0.0;
#pragma unroll
      for (int w = 0; w < kWarps; ++w) v += accw[w * n_bins * S + x];
      if (v != 0.0) atomicAdd(a.sums + x, v);
    }
    if (a.pair_counts)
      for (int x = threadIdx.x; x < n_bins; x += kThreads) {
        unsigned long long v = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) v += cntw[w * n_bins + x];
        if (v) atomicAdd(reinterpret_cast<unsigned long long*>(a.pair_counts) + x, v);
      }
  }
}

template <int P, int MODE>
int launch_fast_p(pgld_context* h, const BandArgs& a, cudaStream_t st) {
  constexpr int S = (P == 1) ? 3 : 15;
  size_t smem = sizeof(FastSmem);
  if (MODE == kModeBinned) smem += (size_t)kWarps * a.n_bins * (S + 1) * 8;
  smem += (size_t)4 * (a.nmax + 1) * sizeof(float);
  auto kern = band_fast_kernel<P, MODE>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_fast smem attribute");
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_fast occupancy");
  per_sm = std::max(1, per_sm);
  pgld_time_begin(h, st);
  kern<<<(unsigned)(h->n_sm * per_sm), kThreads, smem, st>>>(a);
  pgld_time_end(h, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_fast_kernel");
  return PGLD_OK;
}

}  // namespace

// one or two populations without validity planes take the fast kernel
bool band_fast_applies(const BandArgs& a, int mode) {
  // the float32 epilogue is exact for at most 2048 haplotypes per population
  if (mode == kModePairs) return a.n_pops == 1 && a.valid[0] == nullptr && a.W[0] <= 64;
  if (a.n_pops > 2) return false;
  for (int p = 0; p < a.n_pops; ++p)
    if (a.valid[p] != nullptr || a.W[p] > 64) return false;
  return true;
}

int launch_band_fast(pgld_context* h, const BandArgs& a, int mode, cudaStream_t st) {
  if (mode == kModePairs) return launch_fast_p<1, kModePairs>(h, a, st);
  return a.n_pops == 1 ? launch_fast_p<1, kModeBinned>(h, a, st)
                       : launch_fast_p<2, kModeBinned>(h, a, st);
}

}  // namespace pgld
