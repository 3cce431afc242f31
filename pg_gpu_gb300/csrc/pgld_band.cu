// Distance-band tile scheduler and the plain (AND + popcount) band kernels.
//
// The band {(i, j): i < j, pos[j] - pos[i] <= max_dist} is covered by
// 32 x 32 SNP tiles (bi, bj), bj >= bi.  Row block bi owns the tiles
// bi .. bj_hi(bi), where bj_hi is the block of the last j paired with the
// block's last SNP (positions are sorted, so that bound is monotone).  The
// work list is the prefix sum of those counts; a persistent grid walks it
// and recovers (bi, bj) from the item index by binary search, so no pair or
// tile list is ever materialised and nothing is copied back to the host.
#include <cuda_runtime.h>

#include <algorithm>

#include "pgld_internal.cuh"
#include "pgld_scan.cuh"
#include "pgld_band.cuh"

using pgld::i64;

namespace pgld {

// tiles of `tile` SNPs (rows) x `col_tile` SNPs (columns; a multiple of
// `tile`): row block b owns the column blocks from the one holding its first
// SNP to the one holding the last j paired with its last SNP
__global__ void band_items_kernel(const double* __restrict__ pos, i64 n_snp, double max_dist,
                                  i64 n_blocks, int tile, int col_tile, i64* __restrict__ items) {
  for (i64 b = (i64)blockIdx.x * blockDim.x + threadIdx.x; b < n_blocks;
       b += (i64)gridDim.x * blockDim.x) {
    i64 last = min(n_snp - 1, b * tile + tile - 1);
    double lim = pos[last] + max_dist;
    i64 lo = last, hi = n_snp;
    while (lo < hi) {
      i64 mid = (lo + hi) >> 1;
      if (pos[mid] <= lim) lo = mid + 1; else hi = mid;
    }
    i64 jhi = lo - 1;  // last j paired with `last` (>= last)
    const i64 bj_lo = (b * tile) / col_tile;
    i64 bj_hi = max(bj_lo, jhi / col_tile);
    items[b] = bj_hi - bj_lo + 1;
  }
}

int band_schedule(pgld_context* h, const double* pos, i64 n_snp, double max_dist, i64* items,
                  void* scratch, size_t scratch_bytes, cudaStream_t st, int tile, int col_tile) {
  i64 nb = (n_snp + tile - 1) / tile;
  if (col_tile <= 0) col_tile = tile;
  unsigned blocks = (unsigned)std::max<i64>(1, std::min<i64>((nb + 255) / 256, h->n_sm * 4));
  band_items_kernel<<<blocks, 256, 0, st>>>(pos, n_snp, max_dist, nb, tile, col_tile, items);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_items_kernel");
  return exclusive_scan_i64(h, items, nb, scratch, scratch_bytes, st);
}

// ---------------------------------------------------------------------------
// plain band kernel
// ---------------------------------------------------------------------------
constexpr int kKW = 32;     // words of a population staged per chunk
constexpr int kPad = 33;    // smem row pitch (bank-conflict free transpose)
constexpr int kThreads = 256;

struct __align__(16) TileSmem {
  uint32_t ci[kKW][kPad], zi[kKW][kPad], cj[kKW][kPad], zj[kKW][kPad];
  uint32_t vi[kKW][kPad], vj[kKW][kPad];
  double bins[kMaxBins + 1];
};

__device__ __forceinline__ i64 item_block(const i64* __restrict__ off, i64 nb, i64 k) {
  i64 lo = 0, hi = nb;  // largest b with off[b] <= k
  while (hi - lo > 1) {
    i64 mid = (lo + hi) >> 1;
    if (off[mid] <= k) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ int bin_of(const double* sb, int n_bins, double d) {
  // digitize(d, bins) - 1, right-open bins
  if (!(d >= sb[0]) || !(d < sb[n_bins])) return -1;
  int lo = 0, hi = n_bins;  // sb[lo] <= d < sb[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (sb[mid] <= d) lo = mid; else hi = mid;
  }
  return lo;
}

// stage a 32-SNP x 32-word chunk of one plane into smem, transposed to [word][snp]
__device__ __forceinline__ void stage(uint32_t (*dst)[kPad], const uint32_t* __restrict__ src,
                                      i64 s0, i64 n_snp, i64 stride, int w0, int W) {
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kTile / (kThreads / 32); ++q) {
    int sl = wid * (kTile / (kThreads / 32)) + q;
    i64 s = s0 + sl;
    int w = w0 + lane;
    uint32_t v = 0;
    if (s < n_snp && w < W) v = __ldg(src + s * stride + w);
    dst[lane][sl] = v;
  }
}

template <int P, int MODE>
__global__ void __launch_bounds__(kThreads) band_plain_kernel(BandArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TileSmem& sm = *reinterpret_cast<TileSmem*>(smem_raw);
  double* acc = reinterpret_cast<double*>(smem_raw + sizeof(TileSmem));
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(acc + (MODE == kModeBinned ? a.n_bins * a.n_stats : 0));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;

  if (MODE == kModeBinned) {
    for (int x = threadIdx.x; x < a.n_bins * a.n_stats; x += kThreads) acc[x] = 0.0;
    for (int x = threadIdx.x; x < a.n_bins; x += kThreads) cnt[x] = 0ull;
    for (int x = threadIdx.x; x <= a.n_bins; x += kThreads) sm.bins[x] = a.bins[x];
  }
  __syncthreads();
  i64 n_items = a.item_off[a.n_blocks];
  // a tile list longer than the upper triangle of tile blocks is corrupt
  if (n_items < 0 || n_items > a.n_blocks * (a.n_blocks + 1) / 2) {
    if (threadIdx.x == 0 && a.status) atomicCAS(a.status, 0, 2001);
    n_items = 0;
  }
  // binned mode over an anchor range: the row blocks holding anchors only
  const i64 n_anchor = MODE == kModeBinned ? anchors_of(a) : a.n_snp;
  if (n_items > 0 && n_anchor < a.n_snp) n_items = a.item_off[(n_anchor + kTile - 1) / kTile];

  for (i64 item = blockIdx.x; item < n_items; item += gridDim.x) {
    const i64 bi = item_block(a.item_off, a.n_blocks, item);
    const i64 bj = bi + (item - a.item_off[bi]);
    const i64 i0 = bi * kTile, j0 = bj * kTile;

    int c[P][4][4];
    int nv[P][4];
#pragma unroll
    for (int p = 0; p < P; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        c[p][q][0] = c[p][q][1] = c[p][q][2] = c[p][q][3] = 0;
        nv[p][q] = 0;
      }

#pragma unroll
    for (int p = 0; p < P; ++p) {
      const int W = a.W[p];
      const uint32_t* pl = a.planes[p];
      const uint32_t* vl = a.valid[p];
      for (int w0 = 0; w0 < W; w0 += kKW) {
        stage(sm.ci, pl, i0, a.n_snp, 2 * W, w0, W);
        stage(sm.zi, pl + W, i0, a.n_snp, 2 * W, w0, W);
        stage(sm.cj, pl, j0, a.n_snp, 2 * W, w0, W);
        stage(sm.zj, pl + W, j0, a.n_snp, 2 * W, w0, W);
        if (vl) {
          stage(sm.vi, vl, i0, a.n_snp, W, w0, W);
          stage(sm.vj, vl, j0, a.n_snp, W, w0, W);
        }
        __syncthreads();
        const int nw = min(kKW, W - w0);
        for (int w = 0; w < nw; ++w) {
          const uint32_t cj = sm.cj[w][lane], zj = sm.zj[w][lane];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int r = wid + 8 * q;
            const uint32_t ci = sm.ci[w][r], zi = sm.zi[w][r];
            c[p][q][0] += __popc(ci & cj);
            c[p][q][1] += __popc(ci & zj);
            c[p][q][2] += __popc(zi & cj);
            c[p][q][3] += __popc(zi & zj);
          }
        }
        if (vl) {
          for (int w = 0; w < nw; ++w) {
            const uint32_t vj = sm.vj[w][lane];
#pragma unroll
            for (int q = 0; q < 4; ++q) nv[p][q] += __popc(sm.vi[w][wid + 8 * q] & vj);
          }
        }
        __syncthreads();
      }
    }

    // ---- epilogue ----
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const i64 i = i0 + wid + 8 * q, j = j0 + lane;
      bool ok = (i < j) && (j < a.n_snp) && (i < n_anchor);
      double dpos = 0.0;
      if (ok) {
        dpos = a.pos[j] - a.pos[i];
        ok = dpos <= a.max_dist;
      }
      PopC pc[P];
#pragma unroll
      for (int p = 0; p < P; ++p) {
        i64 n = a.valid[p] ? (i64)nv[p][q]
                           : (i64)(c[p][q][0] + c[p][q][1] + c[p][q][2] + c[p][q][3]);
        pc[p] = make_pop(c[p][q][0], c[p][q][1], c[p][q][2], c[p][q][3], n);
      }
      if (MODE == kModePairs) {
        // rows come from the band offsets: write exactly the pairs they list
        if (i < j && j < a.n_snp) ok = (j - i - 1) < (a.pair_off[i + 1] - a.pair_off[i]);
        if (ok) {
          const i64 k = a.pair_off[i] + (j - i - 1);
          int4 cc = make_int4(c[0][q][0], c[0][q][1], c[0][q][2], c[0][q][3]);
          reinterpret_cast<int4*>(a.counts)[k] = cc;
          if (a.nvalid) a.nvalid[k] = (int32_t)pc[0].n;
          if (a.stats) {
            const PopC& p0 = pc[0];
            float r2;
            i64 rd = r_den(p0);
            r2 = rd > 0 ? ll2f(p0.x * p0.x) / ll2f(rd) : __int_as_float(0x7fc00000);
            ND v1 = dd_ii(p0), v2 = dz_iii(p0), v3 = pi2_iiii(p0);
            float4 o;
            o.x = r2;
            o.y = v1.den > 0 ? ll2f(v1.num) / ll2f(v1.den) : 0.f;
            o.z = v2.den > 0 ? ll2f(v2.num) / ll2f(v2.den) : 0.f;
            o.w = v3.den > 0 ? ll2f(v3.num) / ll2f(v3.den) : 0.f;
            reinterpret_cast<float4*>(a.stats)[k] = o;
          }
        }
      } else {
        int b = -1;
        if (ok) {
          double d = a.bcoord ? fabs(a.bcoord[j] - a.bcoord[i]) : dpos;
          b = bin_of(sm.bins, a.n_bins, d);
        }
        unsigned pending = __ballot_sync(0xffffffffu, b >= 0);
        while (pending) {
          const int leader = __ffs(pending) - 1;
          const int bb = __shfl_sync(0xffffffffu, b, leader);
          const bool mine = (b == bb);
          const unsigned grp = __ballot_sync(0xffffffffu, mine);
          int t = 0;
          for (int s = 0; s < a.n_stats; ++s) {
            float v = 0.f;
            for (; t < a.n_terms && a.terms[t].stat == s; ++t) {
              const pgld_term tm = a.terms[t];
              v += (float)tm.weight * term_value_f32(tm.kind, tm.pops, pc);
            }
            v = mine ? v : 0.f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) atomicAdd(&acc[bb * a.n_stats + s], (double)v);
          }
          if (lane == 0) atomicAdd(&cnt[bb], (unsigned long long)__popc(grp));
          pending &= ~grp;
        }
      }
    }
  }

  if (MODE == kModeBinned) {
    __syncthreads();
    for (int x = threadIdx.x; x < a.n_bins * a.n_stats; x += kThreads)
      if (acc[x] != 0.0) atomicAdd(a.sums + x, acc[x]);
    if (a.pair_counts)
      for (int x = threadIdx.x; x < a.n_bins; x += kThreads)
        if (cnt[x]) atomicAdd(reinterpret_cast<unsigned long long*>(a.pair_counts) + x, cnt[x]);
  }
}

size_t band_plain_smem(int mode, int n_bins, int n_stats) {
  size_t s = sizeof(TileSmem);
  if (mode == kModeBinned) s += (size_t)n_bins * n_stats * 8 + (size_t)n_bins * 8;
  return s;
}

template <int P, int MODE>
static int launch_p(pgld_context* h, const BandArgs& a, cudaStream_t st) {
  size_t smem = band_plain_smem(MODE, a.n_bins, a.n_stats);
  auto kern = band_plain_kernel<P, MODE>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_plain smem attribute");
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_plain occupancy");
  per_sm = std::max(1, per_sm);
  unsigned grid = (unsigned)(h->n_sm * per_sm);
  pgld_time_begin(h, st);
  kern<<<grid, kThreads, smem, st>>>(a);
  pgld_time_end(h, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_plain_kernel");
  return PGLD_OK;
}

int launch_band_plain(pgld_context* h, const BandArgs& a, int mode, cudaStream_t st) {
  if (band_fast_applies(a, mode)) return launch_band_fast(h, a, mode, st);
  if (mode == kModePairs) return launch_p<1, kModePairs>(h, a, st);
  switch (a.n_pops) {
    case 1: return launch_p<1, kModeBinned>(h, a, st);
    case 2: return launch_p<2, kModeBinned>(h, a, st);
    case 3: return launch_p<3, kModeBinned>(h, a, st);
    default: return launch_p<4, kModeBinned>(h, a, st);
  }
}

}  // namespace pgld

// ---------------------------------------------------------------------------
// entry points
// ---------------------------------------------------------------------------
static int check_panel(pgld_context* h, const pgld_hap_panel* panel, const char* fn) {
  PGLD_REQUIRE(h, panel != nullptr, "%s: NULL panel", fn);
  PGLD_REQUIRE(h, panel->n_pops >= 1 && panel->n_pops <= PGLD_MAX_POPS, "%s: n_pops %d", fn,
               panel->n_pops);
  PGLD_REQUIRE(h, panel->n_snp >= 0, "%s: n_snp < 0", fn);
  for (int p = 0; p < panel->n_pops; ++p) {
    PGLD_REQUIRE(h, panel->n_words[p] >= 1, "%s: population %d has no haplotypes", fn, p);
    PGLD_REQUIRE(h, panel->planes[p] != nullptr || panel->n_snp == 0, "%s: planes[%d] NULL", fn, p);
  }
  return PGLD_OK;
}

static void fill_panel(pgld::BandArgs& a, const pgld_hap_panel* panel) {
  a.n_pops = panel->n_pops;
  for (int p = 0; p < PGLD_MAX_POPS; ++p) {
    a.W[p] = p < panel->n_pops ? panel->n_words[p] : 0;
    a.planes[p] = p < panel->n_pops ? panel->planes[p] : nullptr;
    a.valid[p] = p < panel->n_pops ? panel->valid[p] : nullptr;
  }
  a.n_snp = panel->n_snp;
  a.nmax = 0;
  for (int p = 0; p < panel->n_pops; ++p) a.nmax = std::max(a.nmax, 32 * panel->n_words[p]);
}

int pgld_tc_supported(pgld_context* h, const pgld_hap_panel* panel);
int pgld_tc_binned(pgld_context* h, const pgld_hap_panel* panel, pgld::BandArgs& a,
                   cudaStream_t st);
int pgld_tc_pairs(pgld_context* h, const pgld_hap_panel* panel, pgld::BandArgs& a,
                  cudaStream_t st);

extern "C" int pgld_hap_band_pairs(pgld_handle h, const pgld_hap_panel* panel, const double* pos,
                                   double max_dist, int32_t* counts, int32_t* n_valid,
                                   float* stats, int64_t n_pairs, int32_t form, void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_hap_band_pairs: NULL handle");
  int rc = check_panel(h, panel, "pgld_hap_band_pairs");
  if (rc) return rc;
  PGLD_REQUIRE(h, panel->n_pops == 1, "pgld_hap_band_pairs: one population per call");
  PGLD_REQUIRE(h, form == PGLD_FORM_PLAIN || form == PGLD_FORM_TC, "pgld_hap_band_pairs: form");
  if (form == PGLD_FORM_TC && !pgld_tc_supported(h, panel))
    return pgld_fail(h, PGLD_ERR_UNSUPPORTED, "pgld_hap_band_pairs: tensor-core form needs "
                     "<= 2048 haplotypes and no separate validity plane");
  PGLD_REQUIRE(h, max_dist >= 0, "pgld_hap_band_pairs: negative max_dist");
  PGLD_REQUIRE(h, n_pairs >= 0, "pgld_hap_band_pairs: n_pairs < 0");
  const i64 n = panel->n_snp;
  if (n < 2) {
    PGLD_REQUIRE(h, n_pairs == 0, "pgld_hap_band_pairs: %lld pairs for %lld SNPs",
                 (long long)n_pairs, (long long)n);
    return PGLD_OK;
  }
  PGLD_REQUIRE(h, pos && counts, "pgld_hap_band_pairs: NULL buffer");
  PGLD_REQUIRE(h, ((uintptr_t)counts & 15) == 0 && (!stats || ((uintptr_t)stats & 15) == 0),
               "pgld_hap_band_pairs: counts/stats must be 16-byte aligned");
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  const i64 nb = (n + pgld::kTile - 1) / pgld::kTile;
  size_t sb1 = pgld::scan_scratch_bytes(n), sb2 = pgld::scan_scratch_bytes(nb);
  size_t off_bytes = (size_t)(n + 1) * 8, it_bytes = (size_t)(nb + 1) * 8;
  void* ws = nullptr;
  rc = pgld_workspace(h, off_bytes + it_bytes + sb1 + sb2 + 512, &ws);
  if (rc) return rc;
  char* w = (char*)ws;
  i64* off = (i64*)w;
  i64* items = (i64*)(w + ((off_bytes + 255) & ~size_t(255)));
  char* scratch = (char*)items + ((it_bytes + 255) & ~size_t(255));
  rc = pgld_band_offsets(h, pos, n, max_dist, off, scratch, std::max(sb1, sb2), st);
  if (rc) return rc;
  i64 tot = 0;
  PGLD_CHECK_CUDA(h, cudaMemcpyAsync(&tot, off + n, 8, cudaMemcpyDeviceToHost, st));
  PGLD_CHECK_CUDA(h, cudaStreamSynchronize(st));
  if (tot != n_pairs)
    return pgld_fail(h, PGLD_ERR_INVALID_ARG, "pgld_hap_band_pairs: n_pairs %lld != %lld in band",
                     (long long)n_pairs, (long long)tot);
  rc = pgld::band_schedule(h, pos, n, max_dist, items, scratch, std::max(sb1, sb2), st);
  if (rc) return rc;
  pgld::BandArgs a{};
  a.status = h->dev_status;
  fill_panel(a, panel);
  a.pos = pos;
  a.max_dist = max_dist;
  a.item_off = items;
  a.n_blocks = nb;
  a.pair_off = off;
  a.counts = counts;
  a.nvalid = n_valid;
  a.stats = stats;
  if (form == PGLD_FORM_TC) return pgld_tc_pairs(h, panel, a, st);
  return pgld::launch_band_plain(h, a, pgld::kModePairs, st);
}

namespace pgld {
// one past the last SNP within max_dist of SNP last (positions sorted): the
// halo of an anchor range ending at last + 1
__global__ void halo_end_kernel(const double* __restrict__ pos, i64 n, i64 last, double max_dist,
                                i64* __restrict__ out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const double lim = pos[last] + max_dist;
  i64 lo = last + 1, hi = n;
  while (lo < hi) {
    const i64 mid = (lo + hi) >> 1;
    if (pos[mid] <= lim) lo = mid + 1; else hi = mid;
  }
  *out = lo;
}
}  // namespace pgld

// binned sums over the pairs (i, j) whose first SNP i lies in [a0, a1)
static int binned_sums_range(pgld_context* h, const pgld_hap_panel* panel, const double* pos,
                             double max_dist, const double* bin_coord, const double* bins,
                             int32_t n_bins, i64 a0, i64 a1, double* sums, int64_t* pair_counts,
                             int32_t form, void* stream, const char* fn) {
  PGLD_REQUIRE(h, h != nullptr, "%s: NULL handle", fn);
  int rc = check_panel(h, panel, fn);
  if (rc) return rc;
  PGLD_REQUIRE(h, n_bins >= 1 && n_bins <= pgld::kMaxBins, "%s: n_bins %d not in [1, %d]", fn,
               n_bins, pgld::kMaxBins);
  PGLD_REQUIRE(h, bins && sums, "%s: NULL bins/sums", fn);
  PGLD_REQUIRE(h, max_dist >= 0, "%s: negative max_dist", fn);
  PGLD_REQUIRE(h, form == PGLD_FORM_PLAIN || form == PGLD_FORM_TC, "%s: form", fn);
  PGLD_REQUIRE(h, 0 <= a0 && a0 <= a1 && a1 <= panel->n_snp,
               "%s: anchor range [%lld, %lld) outside [0, %lld)", fn, (long long)a0,
               (long long)a1, (long long)panel->n_snp);
  if (form == PGLD_FORM_TC && !pgld_tc_supported(h, panel))
    return pgld_fail(h, PGLD_ERR_UNSUPPORTED, "%s: tensor-core form needs "
                     "1 or 2 populations and no separate validity plane", fn);
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  const int P = panel->n_pops;
  const int S = h->spec_n_stats[P];
  PGLD_CHECK_CUDA(h, cudaMemsetAsync(sums, 0, (size_t)n_bins * S * 8, st));
  if (pair_counts) PGLD_CHECK_CUDA(h, cudaMemsetAsync(pair_counts, 0, (size_t)n_bins * 8, st));
  if (panel->n_snp < 2 || a1 <= a0) return PGLD_OK;
  PGLD_REQUIRE(h, pos != nullptr, "%s: NULL pos", fn);
  // the SNP slice [a0, halo): the anchors and every partner within max_dist
  i64 halo = panel->n_snp;
  if (a1 < panel->n_snp) {
    i64* dev_halo = reinterpret_cast<i64*>(h->dev_status) + 1;
    pgld::halo_end_kernel<<<1, 32, 0, st>>>(pos, panel->n_snp, a1 - 1, max_dist, dev_halo);
    PGLD_CHECK_CUDA(h, cudaGetLastError());
    PGLD_CHECK_CUDA(h, cudaMemcpyAsync(&halo, dev_halo, 8, cudaMemcpyDeviceToHost, st));
    PGLD_CHECK_CUDA(h, cudaStreamSynchronize(st));
  }
  pgld_hap_panel sub = *panel;
  for (int p = 0; p < P; ++p) {
    sub.planes[p] = panel->planes[p] + a0 * 2 * panel->n_words[p];
    if (panel->valid[p]) sub.valid[p] = panel->valid[p] + a0 * panel->n_words[p];
  }
  sub.n_snp = halo - a0;
  pos += a0;
  if (bin_coord) bin_coord += a0;
  const i64 n = sub.n_snp;
  if (n < 2) return PGLD_OK;
  pgld::BandArgs a{};
  a.status = h->dev_status;
  fill_panel(a, &sub);
  a.n_anchor = a1 - a0;
  a.pos = pos;
  a.max_dist = max_dist;
  a.bcoord = bin_coord;
  a.bins = bins;
  a.n_bins = n_bins;
  a.sums = sums;
  a.pair_counts = pair_counts;
  a.terms = h->spec_terms[P];
  a.n_terms = h->spec_n_terms[P];
  a.n_stats = S;
  // the tensor-core form schedules its own 64-SNP tiles
  if (form == PGLD_FORM_TC) return pgld_tc_binned(h, &sub, a, st);
  const i64 nb = (n + pgld::kTile - 1) / pgld::kTile;
  size_t sb = pgld::scan_scratch_bytes(nb);
  void* ws = nullptr;
  rc = pgld_workspace(h, (size_t)(nb + 1) * 8 + sb + 512, &ws);
  if (rc) return rc;
  i64* items = (i64*)ws;
  char* scratch = (char*)ws + ((((size_t)(nb + 1) * 8) + 255) & ~size_t(255));
  rc = pgld::band_schedule(h, pos, n, max_dist, items, scratch, sb, st);
  if (rc) return rc;
  a.item_off = items;
  a.n_blocks = nb;
  return pgld::launch_band_plain(h, a, pgld::kModeBinned, st);
}

extern "C" int pgld_hap_binned_sums(pgld_handle h, const pgld_hap_panel* panel, const double* pos,
                                    double max_dist, const double* bin_coord, const double* bins,
                                    int32_t n_bins, double* sums, int64_t* pair_counts,
                                    int32_t form, void* stream) {
  const i64 n = panel ? panel->n_snp : 0;
  return binned_sums_range(h, panel, pos, max_dist, bin_coord, bins, n_bins, 0, n < 0 ? 0 : n, sums,
                           pair_counts, form, stream, "pgld_hap_binned_sums");
}

extern "C" int pgld_hap_binned_sums_range(pgld_handle h, const pgld_hap_panel* panel,
                                          const double* pos, double max_dist,
                                          const double* bin_coord, const double* bins,
                                          int32_t n_bins, int64_t anchor_begin, int64_t anchor_end,
                                          double* sums, int64_t* pair_counts, int32_t form,
                                          void* stream) {
  return binned_sums_range(h, panel, pos, max_dist, bin_coord, bins, n_bins, anchor_begin,
                           anchor_end, sums, pair_counts, form, stream,
                           "pgld_hap_binned_sums_range");
}
