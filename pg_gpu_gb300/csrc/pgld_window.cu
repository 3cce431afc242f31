// Per-window LD sums over batched, uneven windows in one launch.
//
// A window is a range [win_begin[w], win_end[w]) of an index list of SNPs
// (e.g. the segregating sites of a position window); windows may overlap.  Its pairs a < b form an
// upper triangle of 32 x 32 tiles; the tiles of all windows are one work list
// (prefix sum of T_w (T_w + 1) / 2 over windows, T_w = ceil(m_w / 32)) that a
// persistent grid walks, recovering (window, tile row, tile column) by binary
// search.  Counts come from AND + popcount over the bit planes staged in
// shared memory; every statistic is an exact integer (or error-free float32)
// numerator over its denominator, and each warp adds its window's sums once
// per tile.  This replaces the per-window Python loop of
// _zns_from_precomputed / _zns_tiled (ld_statistics.py:534-676), which runs
// four float64 GEMMs per 512 x 512 tile with a host sync per tile.
#include <cuda_runtime.h>

#include <algorithm>

#include "pgld_band.cuh"
#include "pgld_epilogue.cuh"
#include "pgld_internal.cuh"
#include "pgld_scan.cuh"
#include "pgld_window.cuh"

using pgld::i64;

namespace pgld {
namespace win {

constexpr int kT = 32;
constexpr int kKW = 32;
constexpr int kPad = 33;
constexpr int kThreads = 256;
constexpr int kCols = 6;  // r2, sigma_D^2, DD, Dz, pi2, naive r2
constexpr int kCnts = 3;  // pairs, pairs with r2 defined, pairs with n >= 4

struct Args {
  const uint32_t* planes;
  const uint32_t* valid;
  int W;
  i64 n_snp;
  const int32_t* idx;      // SNP index list (NULL: identity)
  const i64* win_begin;    // [n_win] ranges of idx
  const i64* win_end;
  int n_win;
  const i64* tile_off;     // [n_win + 1] prefix of tiles per window
  const float4* site;      // per-SNP (dac, nv, 1 / nv, 1 / (dac (nv - dac))) of site_freq
  int nmax;                // largest valid n (reciprocal tables 0..nmax)
  double* sums;            // [n_win][kCols]
  unsigned long long* cnt; // [n_win][kCnts]
  int32_t* status;
  // per-SNP mode (window_kernel<true>): statistic snp_stat of every pair
  // (a, b), a < b list positions of window w, added to row_sums[snp_off[w] +
  // a - begin] and col_sums[snp_off[w] + b - begin]
  int snp_stat;
  const i64* snp_off;
  double* row_sums;
  double* col_sums;
};

// tiles per window; a window outside [0, n_idx] or with a negative length
// gets no tiles and sets the status word
__global__ void window_tiles_kernel(const i64* __restrict__ win_begin,
                                    const i64* __restrict__ win_end, int n_win, i64 n_idx,
                                    i64* __restrict__ tiles, int32_t* __restrict__ status) {
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < n_win; w += gridDim.x * blockDim.x) {
    const i64 lo = win_begin[w], hi = win_end[w];
    i64 T = 0;
    if (lo < 0 || hi < lo || hi > n_idx) {
      atomicCAS(status, 0, 3100);
    } else {
      T = (hi - lo + kT - 1) / kT;
    }
    tiles[w] = T * (T + 1) / 2;
  }
}

// per-SNP site_freq: carriers and valid haplotypes (carrier or reference)
__global__ void site_freq_kernel(const uint32_t* __restrict__ planes,
                                 const uint32_t* __restrict__ valid, int W, i64 n_snp,
                                 float4* __restrict__ site) {
  for (i64 s = (i64)blockIdx.x * blockDim.x + threadIdx.x; s < n_snp;
       s += (i64)gridDim.x * blockDim.x) {
    int d = 0, v = 0;
    for (int w = 0; w < W; ++w) {
      const uint32_t c = planes[s * 2 * W + w], z = planes[s * 2 * W + W + w];
      d += __popc(c);
      v += valid ? __popc(valid[s * W + w]) : __popc(c | z);
    }
    site[s] = site_freq(d, v);
  }
}

__device__ __forceinline__ void stage(uint32_t (*dst)[kPad], const uint32_t* __restrict__ src,
                                      const int32_t* __restrict__ idx, i64 a0, i64 a_end,
                                      i64 stride, int w0, int W, i64 n_snp, int32_t* status) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kT / (kThreads / 32); ++q) {
    const int sl = wid * (kT / (kThreads / 32)) + q;
    const i64 a = a0 + sl;
    const int w = w0 + lane;
    uint32_t v = 0;
    if (a < a_end && w < W) {
      const i64 s = idx ? (i64)idx[a] : a;
      if (s >= 0 && s < n_snp)
        v = __ldg(src + s * stride + w);
      else
        atomicCAS(status, 0, 3101);
    }
    dst[lane][sl] = v;
  }
}

struct __align__(16) Smem {
  uint32_t ci[kKW][kPad], zi[kKW][kPad], cj[kKW][kPad], zj[kKW][kPad];
  uint32_t vi[kKW][kPad], vj[kKW][kPad];
};

template <bool SNP>
__global__ void __launch_bounds__(kThreads) window_kernel(Args a) {
  __shared__ Smem sm;
  extern __shared__ float tabs[];  // 1/n and 1/(n(n-1)(n-2)(n-3)), n = 0..nmax
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float* tinv = tabs;
  float* tr4 = tabs + (a.nmax + 1);
  for (int x = threadIdx.x; x <= a.nmax; x += kThreads) {
    float r2, r3;
    fast::recip_entry(x, tinv + x, &r2, &r3, tr4 + x);
  }
  __syncthreads();
  i64 n_items = a.tile_off[a.n_win];
  for (i64 item = blockIdx.x; item < n_items; item += gridDim.x) {
    // window of the item, then its tile (bi, bj), bj >= bi, in row-major order
    int lo = 0, hi = a.n_win;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (a.tile_off[mid] <= item) lo = mid; else hi = mid;
    }
    const int w = lo;
    const i64 base = a.win_begin[w], m = a.win_end[w] - base;
    const i64 T = (m + kT - 1) / kT;
    const i64 t = item - a.tile_off[w];
    i64 rlo = 0, rhi = T;  // row bi starts at bi*T - bi(bi-1)/2
    while (rhi - rlo > 1) {
      const i64 mid = (rlo + rhi) >> 1;
      if (mid * T - mid * (mid - 1) / 2 <= t) rlo = mid; else rhi = mid;
    }
    const i64 bi = rlo, bj = bi + (t - (bi * T - bi * (bi - 1) / 2));
    const i64 a0 = base + bi * kT, b0 = base + bj * kT, end = base + m;

    int c[4][4], nv[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      c[q][0] = c[q][1] = c[q][2] = c[q][3] = 0;
      nv[q] = 0;
    }
    const int W = a.W;
    for (int w0 = 0; w0 < W; w0 += kKW) {
      stage(sm.ci, a.planes, a.idx, a0, end, 2 * W, w0, W, a.n_snp, a.status);
      stage(sm.zi, a.planes + W, a.idx, a0, end, 2 * W, w0, W, a.n_snp, a.status);
      stage(sm.cj, a.planes, a.idx, b0, end, 2 * W, w0, W, a.n_snp, a.status);
      stage(sm.zj, a.planes + W, a.idx, b0, end, 2 * W, w0, W, a.n_snp, a.status);
      if (a.valid) {
        stage(sm.vi, a.valid, a.idx, a0, end, W, w0, W, a.n_snp, a.status);
        stage(sm.vj, a.valid, a.idx, b0, end, W, w0, W, a.n_snp, a.status);
      }
      __syncthreads();
      const int nw = min(kKW, W - w0);
      for (int k = 0; k < nw; ++k) {
        const uint32_t cj = sm.cj[k][lane], zj = sm.zj[k][lane];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int r = wid + 8 * q;
          const uint32_t ci = sm.ci[k][r], zi = sm.zi[k][r];
          c[q][0] += __popc(ci & cj);
          c[q][1] += __popc(ci & zj);
          c[q][2] += __popc(zi & cj);
          c[q][3] += __popc(zi & zj);
        }
      }
      if (a.valid)
        for (int k = 0; k < nw; ++k) {
          const uint32_t vj = sm.vj[k][lane];
#pragma unroll
          for (int q = 0; q < 4; ++q) nv[q] += __popc(sm.vi[k][wid + 8 * q] & vj);
        }
      __syncthreads();
    }

    if constexpr (SNP) {
      // row totals of the warp's 4 rows, column totals of its lane's column
      float colv = 0.f;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const i64 ia = a0 + wid + 8 * q, jb = b0 + lane;
        float x = 0.f;
        if (ia < jb && jb < end) {
          const float c1 = (float)c[q][0], c2 = (float)c[q][1], c3 = (float)c[q][2],
                      c4 = (float)c[q][3];
          const fast::Pop p = fast::make(c1, c2, c3, c4);
          const int n = a.valid ? nv[q] : p.n;
          const i64 si = a.idx ? (i64)a.idx[ia] : ia, sj = a.idx ? (i64)a.idx[jb] : jb;
          const bool sok = si >= 0 && si < a.n_snp && sj >= 0 && sj < a.n_snp;
          const float4 fi = sok ? a.site[si] : make_float4(0.f, 0.f, 0.f, 0.f);
          const float4 fj = sok ? a.site[sj] : make_float4(0.f, 0.f, 0.f, 0.f);
          x = pair_stat(a.snp_stat, p, n, c1, tinv[n], tr4[n], fi, fj);
        }
        colv += x;
        float rv = x;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rv += __shfl_xor_sync(0xffffffffu, rv, o);
        if (lane == 0 && rv != 0.f && ia < end)
          atomicAdd(a.row_sums + a.snp_off[w] + (ia - base), (double)rv);
      }
      if (colv != 0.f && b0 + lane < end)
        atomicAdd(a.col_sums + a.snp_off[w] + (b0 + lane - base), (double)colv);
      continue;
    }

    float acc[kCols] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int n_pairs = 0, n_r2 = 0, n_four = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const i64 ia = a0 + wid + 8 * q, jb = b0 + lane;
      if (!(ia < jb && jb < end)) continue;
      const float c1 = (float)c[q][0], c2 = (float)c[q][1], c3 = (float)c[q][2],
                  c4 = (float)c[q][3];
      const fast::Pop p = fast::make(c1, c2, c3, c4);
      const int n = a.valid ? nv[q] : p.n;
      ++n_pairs;
      const i64 si = a.idx ? (i64)a.idx[ia] : ia, sj = a.idx ? (i64)a.idx[jb] : jb;
      const bool sok = si >= 0 && si < a.n_snp && sj >= 0 && sj < a.n_snp;
      const float4 fi = sok ? a.site[si] : make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 fj = sok ? a.site[sj] : make_float4(0.f, 0.f, 0.f, 0.f);
      window_pair(p, n, c1, tinv[n], tr4[n], fi, fj, acc, n_r2, n_four);
    }
    // warp totals, one atomic per statistic per warp
#pragma unroll
    for (int s = 0; s < kCols; ++s) {
      float v = acc[s];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0 && v != 0.f) atomicAdd(a.sums + (i64)w * kCols + s, (double)v);
    }
    const int tp = __reduce_add_sync(0xffffffffu, n_pairs);
    const int tr = __reduce_add_sync(0xffffffffu, n_r2);
    const int tf = __reduce_add_sync(0xffffffffu, n_four);
    if (lane == 0) {
      if (tp) atomicAdd(a.cnt + (i64)w * kCnts + 0, (unsigned long long)tp);
      if (tr) atomicAdd(a.cnt + (i64)w * kCnts + 1, (unsigned long long)tr);
      if (tf) atomicAdd(a.cnt + (i64)w * kCnts + 2, (unsigned long long)tf);
    }
  }
}

}  // namespace win
}  // namespace pgld

int pgld_site_freqs(pgld_context* h, const uint32_t* planes, const uint32_t* valid, int W,
                    long long n_snp, float4* site, cudaStream_t st) {
  const unsigned b = (unsigned)std::max<i64>(1, std::min<i64>((n_snp + 255) / 256, h->n_sm * 8));
  pgld::win::site_freq_kernel<<<b, 256, 0, st>>>(planes, valid, W, n_snp, site);
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  return PGLD_OK;
}

int pgld_tc_supported(pgld_context* h, const pgld_hap_panel* panel);
int pgld_tc_windows(pgld_context* h, const pgld_hap_panel* panel, const int32_t* idx,
                    long long n_idx, const long long* wb, const long long* we, int n_win,
                    double* sums, unsigned long long* counts, cudaStream_t st);

// the plain window kernel over windows [wb[w], we[w]) of the index list:
// window sums (snp_stat < 0) or per-SNP row / column sums of statistic
// snp_stat; synchronises (the workspace holds the tile list and site counts)
static int window_run(pgld_context* h, const pgld_hap_panel* panel, const int32_t* snp_idx,
                      i64 n_idx, const i64* wb, const i64* we, int n_win, double* sums,
                      unsigned long long* counts, int snp_stat, const i64* snp_off,
                      double* row_sums, double* col_sums, cudaStream_t st) {
  const i64 n = panel->n_snp;
  const int W = panel->n_words[0];
  const size_t sb = pgld::scan_scratch_bytes(n_win);
  const size_t tiles_b = ((size_t)(n_win + 1) * 8 + 255) & ~size_t(255);
  const size_t site_b = ((size_t)std::max<i64>(n, 1) * 16 + 255) & ~size_t(255);
  void* ws = nullptr;
  int rc = pgld_workspace(h, tiles_b + site_b + sb + 256, &ws);
  if (rc) return rc;
  char* wp = (char*)ws;
  i64* tiles = (i64*)wp;
  float4* site = (float4*)(wp + tiles_b);
  char* scratch = wp + tiles_b + site_b;
  const unsigned gb = (unsigned)std::max<i64>(1, std::min<i64>((n_win + 255) / 256, h->n_sm * 4));
  pgld::win::window_tiles_kernel<<<gb, 256, 0, st>>>(wb, we, n_win, n_idx, tiles,
                                                      h->dev_status);
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  rc = pgld::exclusive_scan_i64(h, tiles, n_win, scratch, sb, st);
  if (rc) return rc;
  if (n > 0) {
    const unsigned sbk = (unsigned)std::max<i64>(1, std::min<i64>((n + 255) / 256, h->n_sm * 8));
    pgld::win::site_freq_kernel<<<sbk, 256, 0, st>>>(panel->planes[0], panel->valid[0], W, n,
                                                      site);
    PGLD_CHECK_CUDA(h, cudaGetLastError());
  }
  pgld::win::Args a{};
  a.planes = panel->planes[0];
  a.valid = panel->valid[0];
  a.W = W;
  a.n_snp = n;
  a.idx = snp_idx;
  a.win_begin = wb;
  a.win_end = we;
  a.n_win = n_win;
  a.tile_off = tiles;
  a.site = site;
  a.nmax = 32 * W;
  a.sums = sums;
  a.cnt = counts;
  a.status = h->dev_status;
  a.snp_stat = snp_stat;
  a.snp_off = snp_off;
  a.row_sums = row_sums;
  a.col_sums = col_sums;
  const size_t tab_b = (size_t)2 * (a.nmax + 1) * sizeof(float);
  auto kern = snp_stat >= 0 ? pgld::win::window_kernel<true> : pgld::win::window_kernel<false>;
  PGLD_CHECK_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)tab_b));
  int per_sm = 0;
  PGLD_CHECK_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern,
                                                                   pgld::win::kThreads, tab_b));
  pgld_time_begin(h, st);
  kern<<<(unsigned)(h->n_sm * std::max(1, per_sm)), pgld::win::kThreads, tab_b, st>>>(a);
  pgld_time_end(h, st);
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  // the tile offsets and site counts live in the workspace: finish before reuse
  PGLD_CHECK_CUDA(h, cudaStreamSynchronize(st));
  return PGLD_OK;
}

extern "C" int pgld_hap_window_sums(pgld_handle h, const pgld_hap_panel* panel,
                                    const int32_t* snp_idx, int64_t n_idx,
                                    const int64_t* win_begin, const int64_t* win_end,
                                    int32_t n_win, double* sums, int64_t* counts, int32_t form,
                                    void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_hap_window_sums: NULL handle");
  PGLD_REQUIRE(h, panel != nullptr && panel->n_pops == 1,
               "pgld_hap_window_sums: one population per call");
  PGLD_REQUIRE(h, panel->n_words[0] >= 1 && panel->n_snp >= 0, "pgld_hap_window_sums: panel");
  PGLD_REQUIRE(h, n_win >= 0, "pgld_hap_window_sums: n_win < 0");
  PGLD_REQUIRE(h, snp_idx != nullptr || n_idx == panel->n_snp,
               "pgld_hap_window_sums: without an index list n_idx must be n_snp");
  PGLD_REQUIRE(h, n_idx >= 0, "pgld_hap_window_sums: n_idx < 0");
  PGLD_REQUIRE(h, form == PGLD_FORM_PLAIN || form == PGLD_FORM_TC, "pgld_hap_window_sums: form");
  if (form == PGLD_FORM_TC && !pgld_tc_supported(h, panel))
    return pgld_fail(h, PGLD_ERR_UNSUPPORTED, "pgld_hap_window_sums: tensor-core form needs "
                     "<= 2048 haplotypes and no separate validity plane");
  if (n_win == 0) return PGLD_OK;
  PGLD_REQUIRE(h, win_begin && win_end && sums && counts, "pgld_hap_window_sums: NULL buffer");
  PGLD_REQUIRE(h, panel->planes[0] != nullptr || panel->n_snp == 0,
               "pgld_hap_window_sums: NULL planes");
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  PGLD_CHECK_CUDA(h, cudaMemsetAsync(sums, 0, (size_t)n_win * pgld::win::kCols * 8, st));
  PGLD_CHECK_CUDA(h, cudaMemsetAsync(counts, 0, (size_t)n_win * pgld::win::kCnts * 8, st));
  if (form == PGLD_FORM_TC) {
    int rc = pgld_tc_windows(h, panel, snp_idx, n_idx, reinterpret_cast<const i64*>(win_begin),
                             reinterpret_cast<const i64*>(win_end), n_win, sums,
                             reinterpret_cast<unsigned long long*>(counts), st);
    if (rc) return rc;
    // the workspace holds the tile offsets and the operand: finish before reuse
    PGLD_CHECK_CUDA(h, cudaStreamSynchronize(st));
    return PGLD_OK;
  }
  return window_run(h, panel, snp_idx, n_idx, reinterpret_cast<const i64*>(win_begin),
                    reinterpret_cast<const i64*>(win_end), n_win, sums,
                    reinterpret_cast<unsigned long long*>(counts), -1, nullptr, nullptr, nullptr,
                    st);
}

extern "C" int pgld_hap_window_snp_sums(pgld_handle h, const pgld_hap_panel* panel,
                                        const int32_t* snp_idx, int64_t n_idx,
                                        const int64_t* win_begin, const int64_t* win_end,
                                        int32_t n_win, const int64_t* out_off, int32_t stat,
                                        double* row_sums, double* col_sums, int64_t n_out,
                                        void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_hap_window_snp_sums: NULL handle");
  PGLD_REQUIRE(h, panel != nullptr && panel->n_pops == 1,
               "pgld_hap_window_snp_sums: one population per call");
  PGLD_REQUIRE(h, panel->n_words[0] >= 1 && panel->n_snp >= 0, "pgld_hap_window_snp_sums: panel");
  PGLD_REQUIRE(h, n_win >= 0 && n_idx >= 0 && n_out >= 0, "pgld_hap_window_snp_sums: sizes");
  PGLD_REQUIRE(h, snp_idx != nullptr || n_idx == panel->n_snp,
               "pgld_hap_window_snp_sums: without an index list n_idx must be n_snp");
  PGLD_REQUIRE(h, stat >= 0 && stat < pgld::win::kCols, "pgld_hap_window_snp_sums: stat %d",
               (int)stat);
  if (n_win == 0) return PGLD_OK;
  PGLD_REQUIRE(h, win_begin && win_end && out_off && row_sums && col_sums,
               "pgld_hap_window_snp_sums: NULL buffer");
  PGLD_REQUIRE(h, panel->planes[0] != nullptr || panel->n_snp == 0,
               "pgld_hap_window_snp_sums: NULL planes");
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  PGLD_CHECK_CUDA(h, cudaMemsetAsync(row_sums, 0, (size_t)n_out * 8, st));
  PGLD_CHECK_CUDA(h, cudaMemsetAsync(col_sums, 0, (size_t)n_out * 8, st));
  return window_run(h, panel, snp_idx, n_idx, reinterpret_cast<const i64*>(win_begin),
                    reinterpret_cast<const i64*>(win_end), n_win, nullptr, nullptr, (int)stat,
                    reinterpret_cast<const i64*>(out_off), row_sums, col_sums, st);
}
