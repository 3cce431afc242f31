// tcgen05 tensor-core form of the binned band kernel (sm_103a).
//
// The joint counts of a SNP pair are dot products of 0/1 vectors over the
// haplotypes: with A = the carrier / reference rows of 64 SNPs i and B the
// same for 64 SNPs j, D = A B^T holds n11, n10, n01, n00 of all 4096 pairs of
// the tile.  Operand rows are grouped by 8 SNPs (row 16g + k: carrier plane
// of SNP 8g + k, row 16g + 8 + k: its reference plane).  Operands are E4M3
// bytes (0x38 = 1.0, 0x00 = 0) in K-major rows padded to 128 bytes; products
// are exact and the float32 accumulators hold integers below 2^24, so the
// counts are exact.  This kernel serves one population (binned, per-pair and
// window modes) and two populations with one accumulator each (the 64 x 64
// layout); pgld_tc_wide.cu holds the combined two-population layout.
//
// One CTA per SM (it owns all 512 TMEM columns):
//   warp 0      TMA producer: 128-row x 128-byte A and B boxes (SWIZZLE_128B)
//               into a ring of smem stages, one K chunk of one population each
//   warp 1      allocates TMEM; one lane issues tcgen05.mma M=128 N=128 K=32
//               (kind::f8f6f4) into accumulator stage t%2 (population p at
//               columns 256*(t%2) + 128*p), commits stages and tiles
//   warps 4-11  epilogue: 16x256b tcgen05.ld of the grouped rows gives each
//               lane all four counts of two pairs as the float2 operands of
//               the packed float32 statistics (pgld_epilogue2.cuh), bin sums
// Every mbarrier wait is bounded; on expiry the kernel records an error code
// in the status word, drains its own copies and MMAs, frees TMEM and returns.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

#include "pgld_band.cuh"
#include "pgld_epilogue.cuh"
#include "pgld_epilogue2.cuh"
#include "pgld_internal.cuh"
#include "pgld_scan.cuh"
#include "pgld_tc_common.cuh"
#include "pgld_tcgen05.cuh"
#include "pgld_window.cuh"

namespace pgld {
namespace tc {

constexpr int kTileSnp = 64;
constexpr int kEpiWarps = 8;
// pairs mode: per epilogue warp two staging buffers of the counts and the
// float32 statistics of one step (8 rows i x 16 columns j, rows padded to 17
// entries of 16 bytes), written out by bulk copies of each row's band range
constexpr int kStgRow = 17 * 16;
constexpr int kStgArr = 8 * kStgRow;
constexpr int kStgBuf = 2 * kStgArr;
constexpr int kStgWarp = 2 * kStgBuf;
constexpr int kEpiThreads = kEpiWarps * 32;
constexpr int kThreads = (4 + kEpiWarps) * 32;
constexpr uint32_t kTmemCols = 512;
#ifndef PGLD_TC_MAXNREG
#define PGLD_TC_MAXNREG 0
#endif


struct Params {
  int n_pops;
  int kchunks[2];
  long long n_snp;
  long long n_anchor;  // binned mode: pairs whose first SNP lies below n_anchor
  const double* pos;
  double max_dist;
  const double* bcoord;
  const double* bins;
  int n_bins;
  const long long* item_off;
  long long n_blocks;
  double* sums;
  int64_t* pair_counts;
  int32_t* status;
  int stages;
  int nmax;  // largest per-population sample size (reciprocal table length - 1)
  long long wait_cycles;  // limit of every bounded mbarrier wait (SM clock cycles)
  int no_copies;          // test hook: the TMA producer issues nothing
  const int* ipos;     // integer positions (valid when *ipos_bad == 0)
  const int* ipos_bad;
  // per-pair outputs (pairs mode, one population)
  const long long* pair_off;  // [n_snp + 1] first output row of each anchor SNP
  int32_t* counts;            // [n_pairs][4]
  int32_t* nvalid;            // [n_pairs] or NULL
  float* stats;               // [n_pairs][4] r^2, DD, Dz, pi2, or NULL
  // windows mode (one population): operand rows are list positions
  const long long* win_begin;  // [n_win] list ranges
  const long long* win_end;
  int n_win;
  const long long* tile_off;   // [n_win + 1] prefix of 64-SNP tiles per window
  const int32_t* idx;          // list position -> SNP (NULL: identity)
  const float4* site;          // per-SNP (dac, nv, 1 / nv, 1 / (dac (nv - dac))) of the naive r^2
  long long n_panel;           // SNPs of the panel (bound of idx values)
  double* wsums;               // [n_win][6]
  unsigned long long* wcnt;    // [n_win][3]
};

// the tile of a work item: first list positions of its rows i0 and columns
// j0, the end of its range, and (windows mode) its window
struct TileRef {
  long long i0, j0, end, bi, bj;
  long long begin;  // first list position of the window (windows mode)
  int w;
};

// row_hint: the row block (windows mode: the window) of this thread's previous
// item (its items ascend), from which the search steps forward -- a load or
// two per tile instead of a binary search -- falling back to a binary search
// for long jumps
template <int MODE>
__device__ __forceinline__ TileRef decode_item(const Params& a, long long item,
                                               long long& row_hint) {
  TileRef r;
  if constexpr (MODE == kModeWindows) {
    // the window: forward from the previous item's window, like the rows below
    int lo = (int)row_hint;
    int steps = 0;
    while (lo + 1 < a.n_win && a.tile_off[lo + 1] <= item && steps < 4) {
      ++lo;
      ++steps;
    }
    if (steps == 4) {
      int hi = a.n_win;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (a.tile_off[mid] <= item) lo = mid; else hi = mid;
      }
    }
    row_hint = lo;
    // tiles start at the window's first list position rounded down to a
    // multiple of 8 (the operand rows are grouped by 8 positions); pairs
    // before the window are masked
    const long long base = a.win_begin[lo] & ~7ll, m = a.win_end[lo] - base;
    const long long T = a.win_end[lo] > a.win_begin[lo] ? (m + kTileSnp - 1) / kTileSnp : 0;
    const long long t = item - a.tile_off[lo];
    long long rlo = 0, rhi = T;  // row bi starts at bi*T - bi(bi-1)/2
    while (rhi - rlo > 1) {
      const long long mid = (rlo + rhi) >> 1;
      if (mid * T - mid * (mid - 1) / 2 <= t) rlo = mid; else rhi = mid;
    }
    r.bi = rlo;
    r.bj = rlo + (t - (rlo * T - rlo * (rlo - 1) / 2));
    r.i0 = base + r.bi * kTileSnp;
    r.j0 = base + r.bj * kTileSnp;
    r.end = base + m;
    r.begin = a.win_begin[lo];
    r.w = lo;
  } else {
    long long lo = row_hint;
    int steps = 0;
    while (lo + 1 < a.n_blocks && a.item_off[lo + 1] <= item && steps < 4) {
      ++lo;
      ++steps;
    }
    if (steps == 4) {
      long long hi = a.n_blocks;
      while (hi - lo > 1) {
        const long long mid = (lo + hi) >> 1;
        if (a.item_off[mid] <= item) lo = mid; else hi = mid;
      }
    }
    row_hint = lo;
    r.bi = lo;
    r.bj = lo + (item - a.item_off[lo]);
    r.i0 = r.bi * kTileSnp;
    r.j0 = r.bj * kTileSnp;
    r.end = a.n_snp;
    r.begin = 0;
    r.w = 0;
  }
  return r;
}

// MODE kModeBinned: distance-binned moments sums of P populations;
// kModePairs: per-pair counts / n / (r^2, DD, Dz, pi2) of one population
template <int P, int MODE>
__global__ void __launch_bounds__(kThreads, 1)
    band_tc_kernel(const __grid_constant__ CUtensorMap map0, const __grid_constant__ CUtensorMap map1,
                   Params a) {
  constexpr int S = (P == 1) ? 3 : 15;
  extern __shared__ unsigned char smem_dyn[];
  // 1024-byte aligned base for the swizzled stages
  unsigned char* base =
      smem_dyn + ((1024 - (smem_u32(smem_dyn) & 1023)) & 1023);
  const int stages = a.stages;
  unsigned char* ring = base;
  Ctrl* ctrl = reinterpret_cast<Ctrl*>(ring + (size_t)stages * kStageBytes);
  double* sbins = reinterpret_cast<double*>(ctrl + 1);
  int* thr = reinterpret_cast<int*>(sbins + (kMaxBins + 1));
  // per-warp bin sums [kEpiWarps][n_bins][S] (8-byte aligned: thr holds an even count)
  Slot* kacc = reinterpret_cast<Slot*>(thr + (kMaxBins + 2));
  unsigned long long* kcnt =
      reinterpret_cast<unsigned long long*>(kacc + kEpiWarps * a.n_bins * S);  // [kEpiWarps][n_bins]
  // reciprocal tables by n, 4 x (nmax + 1) floats: four arrays (1/n,
  // 1/(n(n-1)), 1/(n(n-1)(n-2)), 1/(n(n-1)(n-2)(n-3))) for the per-pair and
  // window modes, one interleaved float4 array for the binned mode (one load
  // per population and pair)
  unsigned char* tables_u8 = reinterpret_cast<unsigned char*>(kcnt + kEpiWarps * a.n_bins);
  tables_u8 += (16 - (smem_u32(tables_u8) & 15)) & 15;  // 16-byte aligned for float4 loads
  float* tables = reinterpret_cast<float*>(tables_u8);
  fast::Recip T;
  T.inv = tables;
  T.r2 = tables + (a.nmax + 1);
  T.r3 = tables + 2 * (a.nmax + 1);
  T.r4 = tables + 3 * (a.nmax + 1);
  const float4* T4 = reinterpret_cast<const float4*>(tables);
  // pairs mode: the epilogue warps' staging buffers, after the tables
  unsigned char* stg = reinterpret_cast<unsigned char*>(tables + 4 * (a.nmax + 1));
  stg += (16 - (smem_u32(stg) & 15)) & 15;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_bins = a.n_bins;
  volatile int* abort_flag = &ctrl->abort_flag;

  if (threadIdx.x == 0) {
    for (int s = 0; s < stages; ++s) {
      mbar_init(&ctrl->full[s], 1);
      mbar_init(&ctrl->empty[s], 1);
    }
    for (int s = 0; s < 2; ++s) {
      mbar_init(&ctrl->tfull[s], 1);
      mbar_init(&ctrl->tempty[s], kEpiWarps);
    }
    mbar_init(&ctrl->drain, 1);
    ctrl->abort_flag = 0;
    ctrl->produced = 0;
    ctrl->consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&ctrl->tmem_base)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (warp >= 4) {
    const int t = threadIdx.x - 128;
    for (int x = t; x < kEpiWarps * n_bins * S; x += kEpiThreads) kacc[x] = slot_zero();
    for (int x = t; x < kEpiWarps * n_bins; x += kEpiThreads) kcnt[x] = 0ull;
    for (int x = t; x <= a.nmax; x += kEpiThreads)
      if constexpr (MODE == kModeBinned)
        fast2::recip_entry4(x, reinterpret_cast<float4*>(tables) + x);
      else
        fast::recip_entry(x, tables + x, tables + (a.nmax + 1) + x, tables + 2 * (a.nmax + 1) + x,
                          tables + 3 * (a.nmax + 1) + x);
    for (int x = t; MODE == kModeBinned && x <= n_bins; x += kEpiThreads) {
      const double b = a.bins[x];
      sbins[x] = b;
      const double cb = ceil(b);
      thr[x] = cb > 2147483647.0 ? 2147483647 : (cb < -2147483647.0 ? -2147483647 : (int)cb);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = ctrl->tmem_base;

  long long n_items = MODE == kModeWindows ? a.tile_off[a.n_win] : a.item_off[a.n_blocks];
  if (n_items < 0 || (MODE != kModeWindows && n_items > a.n_blocks * (a.n_blocks + 1) / 2)) {
    if (threadIdx.x == 0) set_abort(ctrl, a.status, 3001);
    n_items = 0;
  }
  // binned mode over an anchor range: the row blocks holding anchors only
  if (MODE == kModeBinned && n_items > 0 && a.n_anchor < a.n_snp)
    n_items = a.item_off[(a.n_anchor + kTileSnp - 1) / kTileSnp];

  // Registers move from the producer / MMA warpgroup (warps 0-3) to the two
  // epilogue warpgroups: 128 x 56 + 256 x 224 = 384 x 168, the launch's total
  // (the host launches this kernel only when it was built with 168 registers).
  if (warp < 4) {
#if PGLD_TC_MAXNREG
  asm volatile("setmaxnreg.dec.sync.aligned.u32 56;" ::: "memory");
#endif
  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int issued = 0;
      long long row_hint = 0;
      // (with no_copies the MMA warp's wait for the first stage expires)
      const long long n_copy_items = a.no_copies ? 0 : n_items;
      for (long long item = blockIdx.x; item < n_copy_items && !*abort_flag; item += gridDim.x) {
        const TileRef tr = decode_item<MODE>(a, item, row_hint);
        const int yi = (int)(2 * tr.i0), yj = (int)(2 * tr.j0);
        for (int p = 0; p < P && !*abort_flag; ++p) {
          const CUtensorMap* map = p == 0 ? &map0 : &map1;
          for (int kc = 0; kc < a.kchunks[p]; ++kc) {
            if (!mbar_wait_role(&ctrl->empty[stage], phase ^ 1, abort_flag, a.wait_cycles)) {
              set_abort(ctrl, a.status, 3002);
              break;
            }
            mbar_expect_tx(&ctrl->full[stage], kStageBytes);
            unsigned char* sa = ring + (size_t)stage * kStageBytes;
            tma_load_2d(sa, map, &ctrl->full[stage], kc * kKChunk, yi);
            tma_load_2d(sa + kBoxBytes, map, &ctrl->full[stage], kc * kKChunk, yj);
            ++issued;
            if (++stage == stages) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
      }
      if (*abort_flag) {
        // drain: every issued copy lands before the CTA may exit
        const int consumed = *(volatile int*)&ctrl->consumed;
        int st2 = consumed % stages;
        uint32_t ph2 = (uint32_t)((consumed / stages) & 1);
        for (int k = consumed; k < issued; ++k) {
          mbar_wait_drain(&ctrl->full[st2], ph2);
          if (++st2 == stages) {
            st2 = 0;
            ph2 ^= 1;
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int t = 0;
      int consumed = 0;
      bool any = false;
      for (long long item = blockIdx.x; item < n_items && !*abort_flag; item += gridDim.x, ++t) {
        const int acc = t & 1;
        const uint32_t aph = (uint32_t)((t >> 1) & 1);
        if (!mbar_wait_role(&ctrl->tempty[acc], aph ^ 1, abort_flag, a.wait_cycles)) {
          set_abort(ctrl, a.status, 3003);
          break;
        }
        tc_fence_after();
        bool ok = true;
        for (int p = 0; p < P && ok; ++p) {
          const uint32_t d = tmem_base + (uint32_t)(acc * 256 + p * 128);
          for (int kc = 0; kc < a.kchunks[p]; ++kc) {
            if (!mbar_wait_role(&ctrl->full[stage], phase, abort_flag, a.wait_cycles)) {
              set_abort(ctrl, a.status, 3004);
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sa = smem_u32(ring + (size_t)stage * kStageBytes);
            const uint64_t da = smem_desc(sa), db = smem_desc(sa + kBoxBytes);
#pragma unroll
            for (int k = 0; k < kKChunk / 32; ++k)
              mma_f8(d, da + (uint64_t)(k * 2), db + (uint64_t)(k * 2), (kc | k) != 0);
            mma_commit(&ctrl->empty[stage]);
            any = true;
            *(volatile int*)&ctrl->consumed = ++consumed;
            if (++stage == stages) {
              stage = 0;
              phase ^= 1;
            }
          }
        }
        if (!ok) break;
        mma_commit(&ctrl->tfull[acc]);
      }
      if (*abort_flag && any) {
        // drain: every issued MMA completes before TMEM is freed
        mma_commit(&ctrl->drain);
        mbar_wait_drain(&ctrl->drain, 0);
      }
    }
  }
  } else {
#if PGLD_TC_MAXNREG
    asm volatile("setmaxnreg.inc.sync.aligned.u32 224;" ::: "memory");
#endif
    // ---------------- epilogue ----------------
    // Warp e reads TMEM lane quarter (warp & 3) and column half (e >> 2): the
    // 16 x 32 sub-tile i in i0 + 16*quarter + [0,16), j in j0 + 32*half + [0,32).
    const int e = warp - 4;
    const int quarter = warp & 3;
    const int half = e >> 2;
    const double maxd = a.max_dist;
    const int maxd_int = maxd >= 2147483647.0 ? 2147483647 : (int)floor(maxd);
    const bool use_int = MODE != kModeWindows && (a.bcoord == nullptr) && (*a.ipos_bad == 0);
    Slot* my_acc = kacc + (size_t)e * n_bins * S;
    unsigned long long* my_cnt = kcnt + (size_t)e * n_bins;
    int t = 0;
    long long row_hint = 0;
    int stg_step = 0;  // pairs mode: the warp's steps so far (staging buffer stg_step % 2)
    for (long long item = blockIdx.x; item < n_items; item += gridDim.x, ++t) {
      const int acc = t & 1;
      const uint32_t aph = (uint32_t)((t >> 1) & 1);
      const TileRef tr = decode_item<MODE>(a, item, row_hint);
      const long long bi = tr.bi, bj = tr.bj;
      const long long i0 = tr.i0, j0 = tr.j0;
      const long long si0 = i0 + 16 * quarter, sj0 = j0 + 32 * half;

      // classify the warp's sub-tile: 0 one bin, 1 two adjacent bins, 2 general
      int mode = 2, b0 = -1, thr_mid = 0;
      if (MODE == kModeBinned && use_int && bj > bi && sj0 + 31 < a.n_snp &&
          si0 + 15 < a.n_anchor) {
        const int dmin = a.ipos[sj0] - a.ipos[si0 + 15];
        const int dmax = a.ipos[sj0 + 31] - a.ipos[si0];
        if (dmax <= maxd_int) {
          // (dmin, dmax are the same in every lane: one vote per lookup)
          const int blo = bin_of_int_warp(thr, n_bins, dmin, lane);
          const int bhi = bin_of_int_warp(thr, n_bins, dmax, lane);
          if (blo >= 0 && bhi == blo) {
            mode = 0;
            b0 = blo;
          } else if (blo >= 0 && bhi == blo + 1) {
            mode = 1;
            b0 = blo;
            thr_mid = thr[bhi];
          }
        }
      }

      // windows mode: the naive-r^2 site terms of the thread's SNPs, loaded
      // before the accumulator wait so that their latency overlaps it
      float4 wfi[2], wfj[8];
      if constexpr (MODE == kModeWindows) {
        const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
        auto site_at = [&](long long pos) {
          if (pos < tr.begin || pos >= tr.end) return zero4;
          const long long sp = a.idx ? (long long)a.idx[pos] : pos;
          return (sp >= 0 && sp < a.n_panel) ? a.site[sp] : zero4;
        };
        const long long ib = i0 + 16 * quarter + (lane >> 2);
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) wfi[hh] = site_at(ib + 8 * hh);
#pragma unroll
        for (int gg = 0; gg < 4; ++gg)
#pragma unroll
          for (int y = 0; y < 2; ++y)
            wfj[2 * gg + y] = site_at(j0 + 32 * half + 8 * gg + 2 * (lane & 3) + y);
      }

      // binned mode with integer positions: the positions of the thread's
      // SNPs (rows ib, ib + 8; columns j0 + 32 half + 8 g + 2 (lane % 4) + y),
      // loaded before the accumulator wait for the sub-tiles that bin per pair
      int bp_i0 = 0, bp_i1 = 0, bp_j[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) bp_j[q] = 0;
      if (MODE == kModeBinned && use_int && mode != 0) {
        const long long ibp = i0 + 16 * quarter + (lane >> 2);
        bp_i0 = ibp < a.n_snp ? a.ipos[ibp] : 0;
        bp_i1 = ibp + 8 < a.n_snp ? a.ipos[ibp + 8] : 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const long long jq = j0 + 32 * half + 8 * (q >> 1) + 2 * (lane & 3) + (q & 1);
          bp_j[q] = jq < a.n_snp ? a.ipos[jq] : 0;
        }
      }

      // pairs mode: the band offsets of the thread's two rows, loaded before
      // the accumulator wait
      long long pf_off0 = 0, pf_np0 = 0, pf_off1 = 0, pf_np1 = 0;
      if constexpr (MODE == kModePairs) {
        const long long ibp = i0 + 16 * quarter + (lane >> 2);
        if (ibp < a.n_snp) {
          pf_off0 = a.pair_off[ibp];
          pf_np0 = a.pair_off[ibp + 1] - pf_off0;
        }
        if (ibp + 8 < a.n_snp) {
          pf_off1 = a.pair_off[ibp + 8];
          pf_np1 = a.pair_off[ibp + 9] - pf_off1;
        }
      }

      bool ready = true;
      if (lane == 0) ready = mbar_wait(&ctrl->tfull[acc], aph, abort_flag, a.wait_cycles);
      ready = __shfl_sync(0xffffffffu, ready ? 1 : 0, 0) != 0;
      if (!ready) {
        if (lane == 0) set_abort(ctrl, a.status, 3005);
        break;
      }
      tc_fence_after();

      if constexpr (MODE == kModeWindows) {
        // per-window sums: every pair of list positions begin <= a < b < end
        // of the item's window (the statistics of pgld_hap_window_sums).  The
        // operand rows are grouped by 8 list positions, so a 16x256b TMEM load
        // gives thread t all four counts of the pairs (a, b) and (a, b + 1),
        // a = i0 + 16 quarter + 8 hh + t / 4, b = j0 + 32 half + 8 g + 2 (t % 4)
        float2 ws2[6];
#pragma unroll
        for (int s2 = 0; s2 < 6; ++s2) ws2[s2] = make_float2(0.f, 0.f);
        int np = 0, nr2 = 0, nfour = 0;
        const long long ib = i0 + 16 * quarter + (lane >> 2);
        const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int hh = c & 1, gp = c >> 1;
          uint32_t r[16];
          tmem_ld16x256_x4(tmem_base + ((uint32_t)(quarter * 32 + hh * 16) << 16) +
                               (uint32_t)(acc * 256 + half * 64 + gp * 32),
                           r);
          tmem_wait_ld();
          if (c == 3) {
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&ctrl->tempty[acc]);
          }
          const long long is = ib + 8 * hh;
          const bool iok = is >= tr.begin && is < tr.end;
          const float4 fi = wfi[hh];
          auto u2 = [](uint32_t x, uint32_t y) {
            return make_float2(__uint_as_float(x), __uint_as_float(y));
          };
#pragma unroll
          for (int g = 0; g < 2; ++g) {
            const int o = 8 * g;
            const long long j = j0 + 32 * half + 8 * (2 * gp + g) + 2 * (lane & 3);
            const bool l0 = iok && is < j && j < tr.end;
            const bool l1 = iok && is < j + 1 && j + 1 < tr.end;
            if (!(l0 || l1)) continue;
            const fast2::Pop p = fast2::make(u2(r[o], r[o + 1]), u2(r[o + 4], r[o + 5]),
                                             u2(r[o + 2], r[o + 3]), u2(r[o + 6], r[o + 7]));
            const int gg = 2 * gp + g;
            win::window_pair2(p, u2(r[o], r[o + 1]),
                              [&](int n) { return make_float2(T.inv[n], T.r4[n]); }, fi,
                              l0 ? wfj[2 * gg] : zero4,
                              l1 ? wfj[2 * gg + 1] : zero4, l0, l1, ws2, np, nr2, nfour);
          }
        }
        float ws[6];
#pragma unroll
        for (int s2 = 0; s2 < 6; ++s2) ws[s2] = ws2[s2].x + ws2[s2].y;
#pragma unroll
        for (int s2 = 0; s2 < 6; ++s2) {
          const float v = warp_sum(ws[s2]);
          if (lane == 0 && v != 0.f) atomicAdd(a.wsums + (long long)tr.w * 6 + s2, (double)v);
        }
        const int tp = __reduce_add_sync(0xffffffffu, np);
        const int tr2 = __reduce_add_sync(0xffffffffu, nr2);
        const int tf = __reduce_add_sync(0xffffffffu, nfour);
        if (lane == 0) {
          if (tp) atomicAdd(a.wcnt + (long long)tr.w * 3 + 0, (unsigned long long)tp);
          if (tr2) atomicAdd(a.wcnt + (long long)tr.w * 3 + 1, (unsigned long long)tr2);
          if (tf) atomicAdd(a.wcnt + (long long)tr.w * 3 + 2, (unsigned long long)tf);
        }
        continue;
      }

      if constexpr (MODE == kModePairs) {
        // per-pair outputs.  The operand rows are grouped by 8 SNPs (as in the
        // binned mode), so a 16x256b TMEM load gives thread t all four counts
        // of the pairs (i, j) and (i, j + 1), i = i0 + 16 quarter + 8 hh + t/4,
        // j = j0 + 32 half + 8 g + 2 (t % 4); rows k = pair_off[i] + (j - i - 1)
        // in the reference's order.  A step's counts and statistics (8 rows i
        // x 16 columns j) go through a shared-memory staging buffer: the lane
        // of each row then writes the row's band range with one bulk copy per
        // array (contiguous output rows, whole sectors); n goes out directly.
        const long long ib = i0 + 16 * quarter + (lane >> 2);
        const long long off0 = pf_off0, np0 = pf_np0, off1 = pf_off1, np1 = pf_np1;
        unsigned char* wst = stg + (size_t)e * kStgWarp;
#pragma unroll 1
        for (int c = 0; c < 4; ++c) {
          const int hh = c & 1, gp = c >> 1;
          uint32_t r[16];
          tmem_ld16x256_x4(tmem_base + ((uint32_t)(quarter * 32 + hh * 16) << 16) +
                               (uint32_t)(acc * 256 + half * 64 + gp * 32),
                           r);
          tmem_wait_ld();
          if (c == 3) {
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&ctrl->tempty[acc]);
          }
          const long long is = ib + 8 * hh;
          const long long offh = hh ? off1 : off0, nph = hh ? np1 : np0;
          // this step's buffer is free once the copies issued from it two
          // steps ago have read it (one bulk group per row lane and step)
          unsigned char* buf = wst + (size_t)(stg_step & 1) * kStgBuf;
          bulk_wait_read<1>();
          __syncwarp();
          int4* cst = reinterpret_cast<int4*>(buf) + (lane >> 2) * 17;
          float4* sst = reinterpret_cast<float4*>(buf + kStgArr) + (lane >> 2) * 17;
          auto u2 = [](uint32_t x, uint32_t y) {
            return make_float2(__uint_as_float(x), __uint_as_float(y));
          };
#pragma unroll
          for (int g = 0; g < 2; ++g) {
            // the pairs (is, j) and (is, j + 1), two lanes of the packed epilogue
            const int o = 8 * g;
            const int jj = 8 * g + 2 * (lane & 3);  // column in the step's 16
            const long long j = j0 + 32 * half + 16 * gp + jj;
            // a pair is written exactly when the band offsets list it
            const bool ok0 = is < j && j < a.n_snp && (j - is - 1) < nph;
            const bool ok1 = is < j + 1 && j + 1 < a.n_snp && (j - is) < nph;
            if (!ok0 && !ok1) continue;
            const fast2::Pop p = fast2::make(u2(r[o], r[o + 1]), u2(r[o + 4], r[o + 5]),
                                             u2(r[o + 2], r[o + 3]), u2(r[o + 6], r[o + 7]));
            const long long k = offh + (j - is - 1);  // row of (is, j); (is, j + 1) follows
            float4 st[2];
            if (a.stats) fast2::pair_outputs(p, make_float2(T.r4[p.n0], T.r4[p.n1]), st);
#pragma unroll
            for (int y = 0; y < 2; ++y) {
              const int q = o + y;
              cst[jj + y] = make_int4(fast::f2i_small(__uint_as_float(r[q])),
                                      fast::f2i_small(__uint_as_float(r[q + 4])),
                                      fast::f2i_small(__uint_as_float(r[q + 2])),
                                      fast::f2i_small(__uint_as_float(r[q + 6])));
              if (a.stats) sst[jj + y] = st[y];
              if (a.nvalid) st_cs_if(y ? ok1 : ok0, a.nvalid + (k + y), y ? p.n1 : p.n0);
            }
          }
          fence_proxy_async_smem();
          __syncwarp();
          if ((lane & 3) == 0) {
            // the row's pairs in this step: columns jlo..jhi (j <= is + nph)
            const long long jb = j0 + 32 * half + 16 * gp;
            const long long jlo = jb > is + 1 ? jb : is + 1;
            long long jhi = jb + 15 < a.n_snp - 1 ? jb + 15 : a.n_snp - 1;
            if (is + nph < jhi) jhi = is + nph;
            if (jlo <= jhi) {
              const long long k0 = offh + (jlo - is - 1);
              const uint32_t bytes = (uint32_t)(jhi - jlo + 1) * 16u;
              const int q0 = (int)(jlo - jb);
              bulk_store(reinterpret_cast<int4*>(a.counts) + k0, cst + q0, bytes);
              if (a.stats) bulk_store(reinterpret_cast<float4*>(a.stats) + k0, sst + q0, bytes);
            }
            bulk_commit();
          }
          ++stg_step;
        }
        continue;
      }

      // the warp's sub-tile (16 SNPs i x 32 SNPs j) in 8 steps of 8 x 8 SNPs,
      // two pairs per lane.  The binned operand rows are grouped by 8 SNPs
      // (row 16g + k: SNP 8g + k plane 0; row 16g + 8 + k: plane 1), so a
      // 16x256b TMEM load gives thread t both planes of SNP i = t / 4 of its
      // 8-SNP row group against SNPs j = 2 (t % 4) and 2 (t % 4) + 1 of an
      // 8-SNP column group: (n11, n11, n01, n01) from the columns of plane 0
      // and (n10, n10, n00, n00) from those of plane 1 -- each count already
      // the float2 (.x: j even, .y: j odd) of the packed epilogue.
      // body(hh, g, p0, p1): row half hh (SNPs 8 hh + t / 4), column group g
      auto steps = [&](auto&& body) {
#pragma unroll 1
        for (int c = 0; c < 4; ++c) {
          const int hh = c & 1, gp = c >> 1;
          uint32_t r[P][16];
          const uint32_t taddr = tmem_base + ((uint32_t)(quarter * 32 + hh * 16) << 16) +
                                 (uint32_t)(acc * 256 + half * 64 + gp * 32);
#pragma unroll
          for (int p = 0; p < P; ++p) tmem_ld16x256_x4(taddr + p * 128, r[p]);
          tmem_wait_ld();
          if (c == 3) {
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&ctrl->tempty[acc]);
          }
          auto u2 = [](uint32_t x, uint32_t y) { return make_float2(__uint_as_float(x), __uint_as_float(y)); };
#pragma unroll
          for (int g = 0; g < 2; ++g) {
            const int o = 8 * g;
            const fast2::Pop p0 = fast2::make(u2(r[0][o], r[0][o + 1]), u2(r[0][o + 4], r[0][o + 5]),
                                              u2(r[0][o + 2], r[0][o + 3]), u2(r[0][o + 6], r[0][o + 7]));
            const fast2::Pop p1 =
                fast2::make(u2(r[P - 1][o], r[P - 1][o + 1]), u2(r[P - 1][o + 4], r[P - 1][o + 5]),
                            u2(r[P - 1][o + 2], r[P - 1][o + 3]), u2(r[P - 1][o + 6], r[P - 1][o + 7]));
            body(hh, 2 * gp + g, p0, p1);
          }
        }
      };
      // the lane's SNP i of row half hh and first SNP j of column group g
      const long long ib = i0 + 16 * quarter + (lane >> 2);
      const int ipos_b0 = bp_i0;
      const int ipos_b1 = bp_i1;
      auto jx_of = [&](int g) { return j0 + 32 * half + 8 * g + 2 * (lane & 3); };
      // the prefetched position of column j = jx_of(g) + y (g runtime: selects)
      auto jpos = [&](int g, int y) {
        const int a0 = y ? bp_j[1] : bp_j[0], a1 = y ? bp_j[3] : bp_j[2];
        const int a2 = y ? bp_j[5] : bp_j[4], a3 = y ? bp_j[7] : bp_j[6];
        return g == 0 ? a0 : g == 1 ? a1 : g == 2 ? a2 : a3;
      };
      auto stats_of = [&](const fast2::Pop& p0, const fast2::Pop& p1, float2 (&st)[S]) {
        if constexpr (P == 1) fast2::stats1(p0, T4, st);
        else fast2::stats2_raw(p0, p1, T4, st);
      };

      if (mode == 0) {
        // one bin: packed sums, each statistic's reciprocal factor fused into
        // its running sum
        float2 acc2[S];
#pragma unroll
        for (int s = 0; s < S; ++s) acc2[s] = make_float2(0.f, 0.f);
        steps([&](int, int, const fast2::Pop& p0, const fast2::Pop& p1) {
          auto sink = [&](int k, float2 num, float2 sc) { acc2[k] = fast2::vfma(num, sc, acc2[k]); };
          if constexpr (P == 1) fast2::stats1_to(p0, T4, sink);
          else fast2::stats2_to(p0, p1, T4, sink);
        });
        float v[S];
#pragma unroll
        for (int s = 0; s < S; ++s) v[s] = acc2[s].x + acc2[s].y;
        warp_totals_add<S>(v, lane, my_acc + b0 * S);
        if (lane == 31) my_cnt[b0] += 512ull;
      } else if (mode == 1) {
        // two adjacent bins split at thr_mid: weighted sums of both
        float acc_lo[S], acc_hi[S];
#pragma unroll
        for (int s = 0; s < S; ++s) acc_lo[s] = acc_hi[s] = 0.f;
        int n_hi = 0;
        steps([&](int hh, int g, const fast2::Pop& p0, const fast2::Pop& p1) {
          const int ipi = hh ? ipos_b1 : ipos_b0;
          const bool up0 = (jpos(g, 0) - ipi) >= thr_mid;
          const bool up1 = (jpos(g, 1) - ipi) >= thr_mid;
          const float2 fu = make_float2(up0 ? 1.f : 0.f, up1 ? 1.f : 0.f);
          const float2 fl = make_float2(up0 ? 0.f : 1.f, up1 ? 0.f : 1.f);
          n_hi += (up0 ? 1 : 0) + (up1 ? 1 : 0);
          auto sink = [&](int k, float2 num, float2 sc) {
            const float2 st = fast2::vmul(num, sc);
            acc_hi[k] = fmaf(fu.x, st.x, fmaf(fu.y, st.y, acc_hi[k]));
            acc_lo[k] = fmaf(fl.x, st.x, fmaf(fl.y, st.y, acc_lo[k]));
          };
          if constexpr (P == 1) fast2::stats1_to(p0, T4, sink);
          else fast2::stats2_to(p0, p1, T4, sink);
        });
        warp_totals_add<S>(acc_lo, lane, my_acc + b0 * S);
        warp_totals_add<S>(acc_hi, lane, my_acc + (b0 + 1) * S);
        const int hi_total = __reduce_add_sync(0xffffffffu, n_hi);
        if (lane == 31) {
          my_cnt[b0] += (unsigned long long)(512 - hi_total);
          my_cnt[b0 + 1] += (unsigned long long)hi_total;
        }
      } else {
        // general (diagonal and band-edge tiles, short distances): the bins
        // of the lane's two pairs per step (-1: none).  A step whose pairs
        // fall in at most two adjacent bins goes to running sums of bins
        // (key, key + 1), added to the warp's slots when the key changes; a
        // step without any pair in a bin is skipped; other steps take one warp
        // reduction per bin.
        float acc_lo[S], acc_hi[S];
#pragma unroll
        for (int s = 0; s < S; ++s) acc_lo[s] = acc_hi[s] = 0.f;
        int key = -1, n_lo = 0, n_hi = 0;
        auto flush = [&]() {
          if (key < 0) return;
          warp_totals_add<S>(acc_lo, lane, my_acc + key * S);
          const int tl = __reduce_add_sync(0xffffffffu, n_lo);
          const int th = __reduce_add_sync(0xffffffffu, n_hi);
          if (th) warp_totals_add<S>(acc_hi, lane, my_acc + (key + 1) * S);
          if (lane == 31) {
            my_cnt[key] += (unsigned long long)tl;
            if (th) my_cnt[key + 1] += (unsigned long long)th;
          }
#pragma unroll
          for (int s = 0; s < S; ++s) acc_lo[s] = acc_hi[s] = 0.f;
          n_lo = n_hi = 0;
          key = -1;
        };
        auto bin_of = [&](long long is, int ipi, long long j, int jp) -> int {
          if (!(is < j && j < a.n_snp && is < a.n_anchor)) return -1;
          if (use_int) {
            const int d = jp - ipi;
            return d <= maxd_int ? bin_of_int(thr, n_bins, d) : -1;
          }
          const double dp = a.pos[j] - a.pos[is];
          if (!(dp <= maxd)) return -1;
          const double d = a.bcoord ? fabs(a.bcoord[j] - a.bcoord[is]) : dp;
          return bin_of_f64(sbins, n_bins, d);
        };
        steps([&](int hh, int g, const fast2::Pop& p0, const fast2::Pop& p1) {
          const long long jx = jx_of(g);
          const long long is = ib + 8 * hh;
          const int ipi = hh ? ipos_b1 : ipos_b0;
          const int bx = bin_of(is, ipi, jx, jpos(g, 0)), by = bin_of(is, ipi, jx + 1, jpos(g, 1));
          const int lo = min(bx < 0 ? 0x7fffffff : bx, by < 0 ? 0x7fffffff : by);
          const int mn = __reduce_min_sync(0xffffffffu, lo);
          const int mx = __reduce_max_sync(0xffffffffu, max(bx, by));
          if (mx < 0) return;
          if (mx - mn <= 1) {
            if (mn != key) {
              flush();
              key = mn;
            }
            const float2 fl = make_float2(bx == key ? 1.f : 0.f, by == key ? 1.f : 0.f);
            const float2 fu = make_float2(bx == key + 1 ? 1.f : 0.f, by == key + 1 ? 1.f : 0.f);
            n_lo += (bx == key ? 1 : 0) + (by == key ? 1 : 0);
            n_hi += (bx == key + 1 ? 1 : 0) + (by == key + 1 ? 1 : 0);
            auto sink = [&](int k, float2 num, float2 sc) {
              const float2 st = fast2::vmul(num, sc);
              acc_hi[k] = fmaf(fu.x, st.x, fmaf(fu.y, st.y, acc_hi[k]));
              acc_lo[k] = fmaf(fl.x, st.x, fmaf(fl.y, st.y, acc_lo[k]));
            };
            if constexpr (P == 1) fast2::stats1_to(p0, T4, sink);
            else fast2::stats2_to(p0, p1, T4, sink);
            return;
          }
          flush();  // (the running sums are zero while the step's values live)
          float2 st[S];
          stats_of(p0, p1, st);
#pragma unroll 1
          for (int h = 0; h < 2; ++h) {
            const int b = h ? by : bx;
            unsigned pending = __ballot_sync(0xffffffffu, b >= 0);
            while (pending) {
              const int bb = __shfl_sync(0xffffffffu, b, __ffs(pending) - 1);
              const bool mine = (b == bb);
              const unsigned grp = __ballot_sync(0xffffffffu, mine);
              float v[S];
#pragma unroll
              for (int s = 0; s < S; ++s) v[s] = mine ? (h ? st[s].y : st[s].x) : 0.f;
              warp_totals_add<S>(v, lane, my_acc + bb * S);
              if (lane == 31) my_cnt[bb] += (unsigned long long)__popc(grp);
              pending &= ~grp;
            }
          }
        });
        flush();
      }
    }
    // pairs mode: every bulk copy of the warp has completed (its staging
    // buffers stay valid until then)
    if constexpr (MODE == kModePairs) bulk_wait_all();
  }

  // ---------------- teardown ----------------
  tc_fence_before();
  __syncthreads();
  if (warp >= 4 && !ctrl->abort_flag) {
    const int t = threadIdx.x - 128;
    for (int x = t; x < n_bins * S; x += kEpiThreads) {
      double v = 0.0;
#pragma unroll
      for (int w = 0; w < kEpiWarps; ++w) v += slot_value(kacc[w * n_bins * S + x]);
      if constexpr (P == 2) v *= fast2::post2(x % S);
      if (v != 0.0) atomicAdd(a.sums + x, v);
    }
    if (a.pair_counts)
      for (int x = t; x < n_bins; x += kEpiThreads) {
        unsigned long long v = 0;
#pragma unroll
        for (int w = 0; w < kEpiWarps; ++w) v += kcnt[w * n_bins + x];
        if (v) atomicAdd(reinterpret_cast<unsigned long long*>(a.pair_counts) + x, v);
      }
  }
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// integer copy of the positions for exact integer distances; *bad = 1 when a
// position is not an integer or lies outside (-2^30, 2^30)
__global__ void pos_to_int_kernel(const double* __restrict__ pos, long long n, int* __restrict__ ipos,
                                  int* __restrict__ bad) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const double v = pos[k];
    const bool ok = (v == rint(v)) && fabs(v) < 1073741824.0;
    ipos[k] = ok ? (int)v : 0;
    if (!ok) atomicOr(bad, 1);
  }
}

// ---------------------------------------------------------------------------
// operand packing: bit planes -> E4M3 rows (2 per SNP), K padded to 128
// ---------------------------------------------------------------------------
// Row order: interleaved (row 2r + plane: SNP r) or, with grouped, by groups of
// 8 SNPs (row 16g + 8 plane + k: SNP 8g + k; n_rows rounded up to 8, rows of
// SNPs past n_rows zero).  A block writes 8 operand rows, a warp one row in
// 16-byte chunks (16 haplotypes: one nibble-to-bytes lookup per 4).
__global__ void __launch_bounds__(256) pack_tc_kernel(const uint32_t* __restrict__ planes, int W,
                                                      long long n_snp, long long n_rows,
                                                      const int32_t* __restrict__ idx, int k_pad,
                                                      int grouped, uint32_t* __restrict__ out,
                                                      int32_t* __restrict__ status) {
  const long long rows_out = 2 * (grouped ? (n_rows + 7) / 8 * 8 : n_rows);
  const long long rowi = (long long)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (rowi >= rows_out) return;
  const int chunks = k_pad / 16;
  uint4* dst = reinterpret_cast<uint4*>(out) + rowi * chunks;
  long long r;
  int plane;
  if (grouped) {
    r = (rowi >> 4) * 8 + (rowi & 7);
    plane = (int)((rowi >> 3) & 1);
  } else {
    r = rowi >> 1;
    plane = (int)(rowi & 1);
  }
  long long s = -1;
  if (r < n_rows) {
    s = idx ? (long long)idx[r] : r;
    if (s < 0 || s >= n_snp) {
      if (status && lane == 0) atomicCAS(status, 0, 3102);
      s = -1;
    }
  }
  const uint32_t* src = planes + (s < 0 ? 0 : s) * 2 * W + plane * W;
  for (int c = lane; c < chunks; c += 32) {
    const int h0 = 16 * c;
    const int w = h0 >> 5;
    const uint32_t bits = (s >= 0 && w < W) ? (__ldg(src + w) >> (h0 & 31)) & 0xFFFFu : 0u;
    uint32_t v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t nib = (bits >> (4 * q)) & 0xFu;
      // byte b of v[q] = E4M3 1.0 where bit b of the nibble is set
      v[q] = (nib & 1u ? kOne : 0u) | (nib & 2u ? kOne << 8 : 0u) | (nib & 4u ? kOne << 16 : 0u) |
             (nib & 8u ? kOne << 24 : 0u);
    }
    dst[c] = make_uint4(v[0], v[1], v[2], v[3]);
  }
}

}  // namespace tc
}  // namespace pgld

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
using pgld::tchost::get_encode;
using pgld::tchost::make_map;

// The register split of the band kernel (setmaxnreg) needs the launch's
// total: 384 threads x 168 registers.  A build that allocated fewer would
// make the epilogue warps' increase wait forever, so it is never launched.
static int check_launch_regs(pgld_context* h, const void* kern) {
#if PGLD_TC_MAXNREG
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, kern);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_tc attributes");
  if (fa.numRegs != 168)
    return pgld_fail(h, PGLD_ERR_UNSUPPORTED,
                     "band_tc_kernel built with %d registers per thread; its register split "
                     "needs 168", fa.numRegs);
#else
  (void)h;
  (void)kern;
#endif
  return PGLD_OK;
}

int pgld_tc_supported(pgld_context* h, const pgld_hap_panel* panel) {
  if (panel->n_pops < 1 || panel->n_pops > 2) return 0;
  for (int p = 0; p < panel->n_pops; ++p) {
    if (panel->valid[p] != nullptr) return 0;
    if (panel->n_words[p] > 64) return 0;  // <= 2048 haplotypes per population
  }
  return 1;
}

// the tensor-core band kernel in binned (mode kModeBinned) or per-pair
// (kModePairs, one population) mode; a carries the band, bins or outputs
static int tc_launch(pgld_context* h, const pgld_hap_panel* panel, pgld::BandArgs& a, int mode,
                     cudaStream_t st) {
  using namespace pgld::tc;
  int rc = get_encode(h);
  if (rc) return rc;
  const long long n = panel->n_snp;
  const int P = panel->n_pops;
  const int S = P == 1 ? 3 : 15;
  if (mode == pgld::kModePairs && P != 1)
    return pgld_fail(h, PGLD_ERR_INVALID_ARG, "tensor-core pairs form: one population");
  const long long nb = (n + kTileSnp - 1) / kTileSnp;
  if (2 * (nb * kTileSnp) > 2147483647LL)
    return pgld_fail(h, PGLD_ERR_TOO_LARGE, "tensor-core form: too many SNPs");
  // the operand rows are grouped by 8 SNPs (see pack_tc_kernel)
  const int grouped = 1;
  const long long n_op = grouped ? (n + 7) / 8 * 8 : n;
  int k_pad[2] = {0, 0};
  size_t op_bytes[2] = {0, 0};
  for (int p = 0; p < P; ++p) {
    k_pad[p] = ((panel->n_words[p] * 32 + kKChunk - 1) / kKChunk) * kKChunk;
    op_bytes[p] = (size_t)2 * n_op * k_pad[p];
  }
  // the scan scratch serves both the tile list and (pairs mode) the per-SNP
  // pair offsets; the offsets live in this call's own workspace layout, since
  // pgld_workspace may move the workspace (a caller's copy would be stale)
  const size_t sb = pgld::scan_scratch_bytes(std::max<long long>(nb, n));
  auto al = [](size_t x) { return (x + 1023) & ~size_t(1023); };
  const size_t off_items = 0, off_scan = al((nb + 1) * 8), off_op0 = off_scan + al(sb),
               off_op1 = off_op0 + al(op_bytes[0]), off_ipos = off_op1 + al(op_bytes[1]),
               off_bad = off_ipos + al((size_t)n * 4), off_poff = off_bad + 1024,
               total = off_poff + (mode == pgld::kModePairs ? al((size_t)(n + 1) * 8) : 0);
  void* ws = nullptr;
  rc = pgld_workspace(h, total, &ws);
  if (rc) return rc;
  char* w = (char*)ws;
  long long* poff = mode == pgld::kModePairs ? (long long*)(w + off_poff) : nullptr;
  if (poff) {
    rc = pgld_band_offsets(h, a.pos, n, a.max_dist, poff, w + off_scan, sb, st);
    if (rc) return rc;
  }
  long long* items = (long long*)(w + off_items);
  unsigned char* ops[2] = {(unsigned char*)(w + off_op0), (unsigned char*)(w + off_op1)};

  // operands
  for (int p = 0; p < P; ++p) {
    const unsigned blocks = (unsigned)((2 * n_op + 7) / 8);
    pack_tc_kernel<<<std::max(1u, blocks), 256, 0, st>>>(panel->planes[p], panel->n_words[p], n,
                                                          n, nullptr, k_pad[p], grouped,
                                                          (uint32_t*)ops[p], h->dev_status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "pack_tc_kernel");
  }
  // 64-SNP tile work list
  rc = pgld::band_schedule(h, a.pos, n, a.max_dist, items, w + off_scan, sb, st, kTileSnp);
  if (rc) return rc;
  int* ipos = (int*)(w + off_ipos);
  int* ipos_bad = (int*)(w + off_bad);
  {
    cudaError_t e = cudaMemsetAsync(ipos_bad, 0, 4, st);
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "memset");
    unsigned blocks = (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, h->n_sm * 8));
    pos_to_int_kernel<<<blocks, 256, 0, st>>>(a.pos, n, ipos, ipos_bad);
    e = cudaGetLastError();
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "pos_to_int_kernel");
  }
  CUtensorMap maps[2];
  for (int p = 0; p < P; ++p) {
    rc = make_map(h, &maps[p], ops[p], 2 * n_op, k_pad[p]);
    if (rc) return rc;
  }
  if (P == 1) maps[1] = maps[0];

  Params prm{};
  prm.n_pops = P;
  for (int p = 0; p < P; ++p) prm.kchunks[p] = k_pad[p] / kKChunk;
  prm.n_snp = n;
  prm.n_anchor = pgld::anchors_of(a);
  prm.pos = a.pos;
  prm.max_dist = a.max_dist;
  prm.bcoord = a.bcoord;
  prm.bins = a.bins;
  prm.n_bins = a.n_bins;
  prm.item_off = items;
  prm.n_blocks = nb;
  prm.sums = a.sums;
  prm.pair_counts = a.pair_counts;
  prm.status = h->dev_status;
  prm.ipos = ipos;
  prm.ipos_bad = ipos_bad;
  prm.pair_off = poff;
  prm.counts = a.counts;
  prm.nvalid = a.nvalid;
  prm.stats = a.stats;
  prm.nmax = 0;
  for (int p = 0; p < P; ++p) prm.nmax = std::max(prm.nmax, 32 * panel->n_words[p]);
  prm.wait_cycles = kWaitCycles;
  if (h->test_fault == PGLD_TEST_FAULT_NO_COPIES) {
    // one-shot test hook: no operand copies, the bounded waits expire after
    // ~10 ms and the launch reports it in the device status word
    prm.no_copies = 1;
    prm.wait_cycles = 20000000ll;
    h->test_fault = 0;
  }

  const size_t fixed = sizeof(Ctrl) + (pgld::kMaxBins + 1) * 8 + (pgld::kMaxBins + 2) * 4 +
                       (size_t)kEpiWarps * a.n_bins * (S + 1) * 8 +
                       (size_t)4 * (prm.nmax + 1) * sizeof(float) + 1024 +
                       (mode == pgld::kModePairs ? (size_t)kEpiWarps * kStgWarp + 16 : 0);
  int max_smem = 0;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  int stages = (int)std::min<long long>(8, ((long long)max_smem - (long long)fixed) / kStageBytes);
  if (h->tc_stages_cap > 0) stages = std::min(stages, h->tc_stages_cap);
  if (stages < 2) return pgld_fail(h, PGLD_ERR_TOO_LARGE, "tensor-core form: shared memory");
  prm.stages = stages;
  const size_t smem = (size_t)stages * kStageBytes + fixed;
  auto kern = mode == pgld::kModePairs
                  ? band_tc_kernel<1, pgld::kModePairs>
                  : (P == 1 ? band_tc_kernel<1, pgld::kModeBinned> : band_tc_kernel<2, pgld::kModeBinned>);
  if (mode == pgld::kModeWindows) kern = band_tc_kernel<1, pgld::kModeWindows>;
  rc = check_launch_regs(h, (const void*)kern);
  if (rc) return rc;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_tc smem attribute");
  pgld_time_begin(h, st);
  kern<<<(unsigned)h->n_sm, kThreads, smem, st>>>(maps[0], maps[1], prm);
  pgld_time_end(h, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_tc_kernel");
  return PGLD_OK;
}

int pgld_tc_wide_supported(const pgld_hap_panel* panel);
int pgld_tc_wide_binned(pgld_context* h, const pgld_hap_panel* panel, pgld::BandArgs& a,
                        cudaStream_t st);

int pgld_tc_binned(pgld_context* h, const pgld_hap_panel* panel, pgld::BandArgs& a,
                   cudaStream_t st) {
  if (h->tc_layout != 1 && pgld_tc_wide_supported(panel))
    return pgld_tc_wide_binned(h, panel, a, st);
  return tc_launch(h, panel, a, pgld::kModeBinned, st);
}

int pgld_tc_wide_pairs(pgld_context* h, const pgld_hap_panel* panel, pgld::BandArgs& a,
                       cudaStream_t st);
int pgld_tc_wide_windows(pgld_context* h, const pgld_hap_panel* panel, const int32_t* idx,
                         long long n_idx, const long long* wb, const long long* we, int n_win,
                         double* sums, unsigned long long* counts, cudaStream_t st);

// per-pair outputs: 64 x 64 tiles unless the 64 x 128 layout (pgld_tc_wide.cu)
// is configured (the output stores bound this form; at 2,000 haplotypes the
// square tiles measured faster)
int pgld_tc_pairs(pgld_context* h, const pgld_hap_panel* panel, pgld::BandArgs& a,
                  cudaStream_t st) {
  if (h->tc_layout == 2) return pgld_tc_wide_pairs(h, panel, a, st);
  return tc_launch(h, panel, a, pgld::kModePairs, st);
}

// the E4M3 operand rows of a population's bit planes over an index list
// (pack_tc_kernel, rows grouped by 8 positions)
int pgld_tc_pack_rows(pgld_context* h, const uint32_t* planes, int W, long long n_snp,
                      long long n_rows, const int32_t* idx, int k_pad, unsigned char* out,
                      cudaStream_t st) {
  const long long rows_out = 2 * ((n_rows + 7) / 8 * 8);
  const unsigned blocks = (unsigned)std::max<long long>(1, (rows_out + 7) / 8);
  pgld::tc::pack_tc_kernel<<<blocks, 256, 0, st>>>(planes, W, n_snp, n_rows, idx, k_pad, 1,
                                                   (uint32_t*)out, h->dev_status);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "pack_tc_kernel");
  return PGLD_OK;
}

namespace pgld {
namespace tc {
// 64-SNP tiles per window (upper triangle); bad ranges get none and set the status
__global__ void tc_window_tiles_kernel(const long long* __restrict__ wb,
                                       const long long* __restrict__ we, int n_win, long long n_idx,
                                       long long* __restrict__ tiles, int32_t* __restrict__ status) {
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < n_win; w += gridDim.x * blockDim.x) {
    const long long lo = wb[w], hi = we[w];
    long long T = 0;
    if (lo < 0 || hi < lo || hi > n_idx)
      atomicCAS(status, 0, 3100);
    else if (hi > lo)
      T = (hi - (lo & ~7ll) + kTileSnp - 1) / kTileSnp;  // origin rounded down to 8
    tiles[w] = T * (T + 1) / 2;
  }
}
}  // namespace tc
}  // namespace pgld

int pgld_site_freqs(pgld_context* h, const uint32_t* planes, const uint32_t* valid, int W,
                    long long n_snp, float4* site, cudaStream_t st);

// Per-window sums on the tensor cores (one population, <= 2048 haplotypes, no
// validity plane): the operand is built over the index list so that each
// window is a contiguous range of operand rows.
int pgld_tc_windows(pgld_context* h, const pgld_hap_panel* panel, const int32_t* idx,
                    long long n_idx, const long long* wb, const long long* we, int n_win,
                    double* sums, unsigned long long* counts, cudaStream_t st) {
  using namespace pgld::tc;
  // 64 x 128 tiles (pgld_tc_wide.cu) unless the square layout is configured
  if (h->tc_layout != 1)
    return pgld_tc_wide_windows(h, panel, idx, n_idx, wb, we, n_win, sums, counts, st);
  int rc = get_encode(h);
  if (rc) return rc;
  const long long n = panel->n_snp;
  const int W = panel->n_words[0];
  if (2 * n_idx > 2147483647LL - 256)
    return pgld_fail(h, PGLD_ERR_TOO_LARGE, "tensor-core windows: too many SNPs");
  const int k_pad = ((W * 32 + kKChunk - 1) / kKChunk) * kKChunk;
  // operand rows grouped by 8 list positions (see pack_tc_kernel)
  const long long n_op = (std::max<long long>(n_idx, 1) + 7) / 8 * 8;
  const size_t op_bytes = (size_t)2 * n_op * k_pad;
  const size_t sb = pgld::scan_scratch_bytes(n_win);
  auto al = [](size_t x) { return (x + 1023) & ~size_t(1023); };
  const size_t off_tiles = 0, off_scan = al((size_t)(n_win + 1) * 8), off_op = off_scan + al(sb),
               off_site = off_op + al(op_bytes),
               total = off_site + al((size_t)std::max<long long>(n, 1) * 16);
  void* ws = nullptr;
  rc = pgld_workspace(h, total, &ws);
  if (rc) return rc;
  char* w = (char*)ws;
  long long* tiles = (long long*)(w + off_tiles);
  unsigned char* op = (unsigned char*)(w + off_op);
  float4* site = (float4*)(w + off_site);
  {
    const unsigned gb = (unsigned)std::max<long long>(1, std::min<long long>((n_win + 255) / 256, h->n_sm * 4LL));
    tc_window_tiles_kernel<<<gb, 256, 0, st>>>(wb, we, n_win, n_idx, tiles, h->dev_status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "tc_window_tiles_kernel");
  }
  rc = pgld::exclusive_scan_i64(h, tiles, n_win, w + off_scan, sb, st);
  if (rc) return rc;
  if (n > 0) {
    rc = pgld_site_freqs(h, panel->planes[0], nullptr, W, n, site, st);
    if (rc) return rc;
  }
  if (n_idx > 0) {
    const unsigned blocks = (unsigned)((2 * n_op + 7) / 8);
    pack_tc_kernel<<<blocks, 256, 0, st>>>(panel->planes[0], W, n, n_idx, idx, k_pad, 1, (uint32_t*)op,
                                           h->dev_status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "pack_tc_kernel");
  }
  CUtensorMap map;
  rc = make_map(h, &map, op, 2 * n_op, k_pad);
  if (rc) return rc;
  Params prm{};
  prm.n_pops = 1;
  prm.kchunks[0] = k_pad / kKChunk;
  prm.n_snp = n_idx;
  prm.n_bins = 0;
  prm.status = h->dev_status;
  prm.nmax = 32 * W;
  prm.wait_cycles = kWaitCycles;
  prm.win_begin = wb;
  prm.win_end = we;
  prm.n_win = n_win;
  prm.tile_off = tiles;
  prm.idx = idx;
  prm.n_panel = n;
  prm.site = site;
  prm.wsums = sums;
  prm.wcnt = counts;
  prm.ipos = nullptr;  // positions play no part in windows mode
  prm.ipos_bad = nullptr;
  const size_t fixed = sizeof(Ctrl) + (pgld::kMaxBins + 1) * 8 + (pgld::kMaxBins + 2) * 4 +
                       (size_t)4 * (prm.nmax + 1) * sizeof(float) + 1024;
  int max_smem = 0;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  int stages = (int)std::min<long long>(8, ((long long)max_smem - (long long)fixed) / kStageBytes);
  if (h->tc_stages_cap > 0) stages = std::min(stages, h->tc_stages_cap);
  if (stages < 2) return pgld_fail(h, PGLD_ERR_TOO_LARGE, "tensor-core windows: shared memory");
  prm.stages = stages;
  const size_t smem = (size_t)stages * kStageBytes + fixed;
  auto kern = band_tc_kernel<1, pgld::kModeWindows>;
  rc = check_launch_regs(h, (const void*)kern);
  if (rc) return rc;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "tc windows smem attribute");
  pgld_time_begin(h, st);
  kern<<<(unsigned)h->n_sm, kThreads, smem, st>>>(map, map, prm);
  pgld_time_end(h, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_tc_kernel (windows)");
  return PGLD_OK;
}
