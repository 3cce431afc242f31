// Tensor-core binned sums of two populations in one contraction (sm_103a).
//
// Both populations share one E4M3 operand row per SNP plane: its first K0
// bytes hold population 0's haplotypes as 1.0 (0x38), the next K1 bytes
// population 1's as 64.0 (0x68).  The dot product of two such rows is
// v = c0 + 4096 c1, c_p the joint count of population p; with at most 2,047
// haplotypes per population v < 2^23 is an exact float32 integer and
//   c1 = round-to-nearest(v / 4096)  (c0 / 4096 < 0.5),  c0 = v - 4096 c1.
// One accumulator therefore holds both populations' counts, and a tile of
// 64 SNPs i x 128 SNPs j -- an M = 128 (64 SNPs x carrier / reference
// plane) by N = 256 (128 SNPs x 2 planes) MMA -- takes 256 TMEM columns,
// so two accumulator buffers fit in the 512 columns.  Against the 64 x 64
// two-accumulator form this moves 96 instead of 128 operand bytes through
// shared memory per pair, and each 48 KB pipeline stage carries twice the
// tensor work (four M128 N256 K32 MMAs), which keeps the tensor pipe fed
// across the latency of the stage hand-offs.
//
// The same kernel serves one population in two more modes (a population's
// counts straight from the accumulator, no split): per-pair outputs over the
// distance band (counts, n, r^2, DD, Dz, pi2 in the reference's pair order)
// and per-window sums over the 64 x 128 tiles of every window's upper
// triangle (r^2, sigma_D^2, DD, Dz, pi2, naive r^2), all windows in one launch.
//
// Roles (one CTA per SM, 512 threads):
//   warp 0      TMA producer: A box 128 rows x 128 B, B box 256 rows x 128 B
//               (SWIZZLE_128B) per K chunk into a ring of 48 KB stages
//   warp 1      allocates TMEM; one lane issues tcgen05.mma M128 N256 K32
//               (kind::f8f6f4) into accumulator buffer t % 2
//   warps 4..   epilogue (8 or 12 warps): warp e owns TMEM lane quarter
//               e % 4 (16 SNPs i); the quarter's warps take its 32-SNP column
//               chunks of the CTA's tiles in order, each the next one when
//               it is free (16 x 32 sub-tiles);
//               decode, float32 statistics, float64 bin slots
// Every mbarrier wait is bounded; on expiry the kernel records an error code
// in the status word, drains its own copies and MMAs, frees TMEM and returns.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <type_traits>

#include "pgld_band.cuh"
#include "pgld_epilogue.cuh"
#include "pgld_epilogue2.cuh"
#include "pgld_internal.cuh"
#include "pgld_scan.cuh"
#include "pgld_tc_common.cuh"
#include "pgld_tcgen05.cuh"
#include "pgld_window.cuh"

#ifndef PGLD_TCW_MAXNREG
#define PGLD_TCW_MAXNREG 1
#endif
#ifndef PGLD_TCW_CUNROLL
#define PGLD_TCW_CUNROLL 1
#endif
// producer / MMA waits: 1 try_wait suspending up to PGLD_TCW_SUSPEND ns per
// probe (no issue slots taken while waiting), 0 probes with ~32 ns naps
#ifndef PGLD_TCW_PWAIT
#define PGLD_TCW_PWAIT 1
#endif
#ifndef PGLD_TCW_NAP_LONG
#define PGLD_TCW_NAP_LONG 0
#endif
#ifndef PGLD_TCW_SUSPEND
#define PGLD_TCW_SUSPEND 20000
#endif
#ifndef PGLD_TCW_SSINK
#define PGLD_TCW_SSINK 0
#endif
#ifndef PGLD_TCW_DYN
#define PGLD_TCW_DYN 1
#endif
#ifndef PGLD_TCW_EPI
#define PGLD_TCW_EPI 12
#endif

namespace pgld {
namespace tcw {

using namespace pgld::tc;

constexpr int kRowSnp = 64;    // SNPs i per tile (A: 128 operand rows)
constexpr int kColSnp = 128;   // SNPs j per tile (B: 256 operand rows)
constexpr int kBoxA = 128 * kKChunk;           // 16 KB
constexpr int kBoxB = 256 * kKChunk;           // 32 KB
constexpr int kStage = kBoxA + kBoxB;          // 48 KB
constexpr int kEpiWarps = PGLD_TCW_EPI;   // 8 or 12 epilogue warps (2 or 3 per sub-partition)
static_assert(kEpiWarps == 8 || kEpiWarps == 12, "8 or 12 epilogue warps");
constexpr int kUnitsPerTile = 16;          // 4 lane quarters x 4 column chunks of 32 SNPs
// registers per thread at launch, and the split between the producer / MMA
// warpgroup and the epilogue warpgroups: 128 lo + 32 kEpiWarps hi <= kThreads x launch
constexpr int kRegLaunch = kEpiWarps == 8 ? 168 : 128;
constexpr int kRegLo = kEpiWarps == 8 ? 56 : 32;
constexpr int kRegHi = kEpiWarps == 8 ? 224 : 160;
constexpr int kEpiThreads = kEpiWarps * 32;
constexpr int kThreads = (4 + kEpiWarps) * 32;
static_assert(128 * kRegLo + 32 * kEpiWarps * kRegHi <= kThreads * kRegLaunch,
              "register split above the launch's total");
constexpr int kSlotSets = 4;   // bin slot sets, each shared by two epilogue warps
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kOne64 = 0x68;  // E4M3 64.0
// instruction descriptor: D f32, A/B E4M3, both K-major, N = 256, M = 128
constexpr uint32_t kIdescW = (1u << 4) | ((256u >> 3) << 17) | ((128u >> 4) << 24);
constexpr int kS = 15;         // statistics of two populations
constexpr int kCUnroll = PGLD_TCW_CUNROLL;

struct Params {
  int kchunks;                 // K chunks of 128 bytes (both populations)
  long long n_snp;
  long long n_anchor;          // pairs whose first SNP lies below n_anchor
  const double* pos;
  double max_dist;
  const double* bcoord;
  const double* bins;
  int n_bins;
  const long long* item_off;   // [n_rb + 1] tiles of each 64-SNP row block
  long long n_rb, n_cb;        // 64-SNP row blocks, 128-SNP column blocks
  double* sums;
  int64_t* pair_counts;
  int32_t* status;
  int stages;
  int nmax;
  const int* ipos;
  const int* ipos_bad;
  long long wait_cycles;
  int no_copies;               // test hook: the TMA producer issues nothing
  // per-pair outputs (pairs mode)
  const long long* pair_off;   // [n_snp + 1] first output row of each SNP's pairs
  int32_t* counts;             // [n_pairs][4]
  int32_t* nvalid;             // [n_pairs] or NULL
  float* stats;                // [n_pairs][4] r^2, DD, Dz, pi2, or NULL
  // windows mode: operand rows are list positions; window w covers list
  // positions [win_begin[w], win_end[w]), its tiles start at win_begin & ~7
  const long long* win_begin;
  const long long* win_end;
  int n_win;
  const long long* tile_off;   // [n_win + 1] prefix of the windows' tile counts
  const int32_t* idx;          // list position -> SNP (NULL: identity)
  const float4* site;          // per-SNP (dac, nv, 1 / nv, 1 / (dac (nv - dac))) of the naive r^2
  long long n_panel;           // SNPs of the panel (bound of idx values)
  double* wsums;               // [n_win][6]
  unsigned long long* wcnt;    // [n_win][3]
};

// windows mode: row block b of a window of C column blocks holds the column
// blocks b / 2 .. C - 1; the tiles before row block b
__host__ __device__ __forceinline__ long long wtiles_before(long long b, long long C) {
  const long long k = b >> 1;
  return b * C - ((b & 1) ? k * k : k * (k - 1));
}

// a work item's tile: first list positions of its rows i0 and columns j0,
// and (windows mode) its window [begin, end) and index
struct WideTile {
  long long i0, j0, begin, end;
  int w;
};

// windows mode: the tile of an item, the window found by stepping forward
// from the previous item's window (hint), then the row block from the root of
// the window's tile count
__device__ __forceinline__ WideTile window_tile(const Params& a, long long item, long long& hint) {
  int lo = (int)hint;
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
  hint = lo;
  const long long base = a.win_begin[lo] & ~7ll, m = a.win_end[lo] - base;
  const long long R = (m + kRowSnp - 1) / kRowSnp, C = (m + kColSnp - 1) / kColSnp;
  const long long t = item - a.tile_off[lo];
  // the row block: the largest b < R with wtiles_before(b, C) <= t.  For even
  // b, wtiles_before = b C - b^2 / 4 + b / 2, whose root in b, (2C + 1) -
  // sqrt((2C + 1)^2 - 4 t), starts the search; the steps below make it exact
  // (wtiles_before rises by C - floor(b / 2) >= 1 per row block)
  const long long c2 = 2 * C + 1;
  const float disc = (float)(c2 * c2 - 4 * t);
  long long rlo = (long long)((float)c2 - sqrtf(disc > 0.f ? disc : 0.f));
  rlo = rlo < 0 ? 0 : (rlo > R - 1 ? R - 1 : rlo);
  while (rlo > 0 && wtiles_before(rlo, C) > t) --rlo;
  while (rlo + 1 < R && wtiles_before(rlo + 1, C) <= t) ++rlo;
  WideTile r;
  r.i0 = base + rlo * kRowSnp;
  r.j0 = base + ((rlo >> 1) + (t - wtiles_before(rlo, C))) * kColSnp;
  r.begin = a.win_begin[lo];
  r.end = a.win_end[lo];
  r.w = lo;
  return r;
}

__device__ __forceinline__ void mma_w(uint32_t d, uint64_t a, uint64_t b, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}" ::"r"(d),
      "l"(a), "l"(b), "r"(kIdescW), "r"(accum)
      : "memory");
}

// row block of a work item, stepping forward from the previous one
__device__ __forceinline__ long long row_of(const Params& a, long long item, long long& hint) {
  long long lo = hint;
  int steps = 0;
  while (lo + 1 < a.n_rb && a.item_off[lo + 1] <= item && steps < 4) {
    ++lo;
    ++steps;
  }
  if (steps == 4) {
    long long hi = a.n_rb;
    while (hi - lo > 1) {
      const long long mid = (lo + hi) >> 1;
      if (a.item_off[mid] <= item) lo = mid; else hi = mid;
    }
  }
  hint = lo;
  return lo;
}

// the decoded counts of one population, two pairs (.x, .y)
struct Counts2 {
  float2 c1, c2, c3, c4;
};

// v = c0 + 4096 c1 (exact) -> (c0, c1)
__device__ __forceinline__ void split2(float2 v, float2& lo, float2& hi) {
  const float2 u = fast2::vfma(v, fast2::vs(1.0f / 4096.0f), fast2::vs(12582912.0f));
  hi = fast2::vsub(u, fast2::vs(12582912.0f));
  lo = fast2::vfma(hi, fast2::vs(-4096.0f), v);
}

// the producer's and MMA issuer's waits.  try_wait suspends the thread until
// the phase completes or a hardware time limit passes; waits that usually
// outlast that limit (kNapNs > 0: a free accumulator buffer, a free stage)
// nap between probes, so that the waiting thread takes few issue slots from
// the epilogue warps of its sub-partition
template <int kNapNs>
__device__ __forceinline__ bool role_wait(uint64_t* b, uint32_t parity, volatile int* abort_flag,
                                          long long limit) {
#if PGLD_TCW_PWAIT == 1
  const long long t0 = clock64();
  for (long long k = 0; k < kSpinLimit; ++k) {
    if (mbar_try_for(b, parity, PGLD_TCW_SUSPEND)) return true;
    if (kNapNs > 0) __nanosleep(kNapNs);
    if ((k & 7) == 7 && (*abort_flag || clock64() - t0 > limit)) return false;
  }
  return false;
#else
  return mbar_wait_nap(b, parity, abort_flag, limit);
#endif
}

// MODE kModeBinned: distance-binned sums of two populations (combined
// operand); kModePairs: per-pair outputs of one population; kModeWindows:
// per-window sums of one population
template <int MODE>
__global__ void __launch_bounds__(kThreads, 1)
    band_wide_kernel(const __grid_constant__ CUtensorMap map_a,
                     const __grid_constant__ CUtensorMap map_b, Params a) {
  extern __shared__ unsigned char smem_dyn[];
  unsigned char* base = smem_dyn + ((1024 - (smem_u32(smem_dyn) & 1023)) & 1023);
  const int stages = a.stages;
  unsigned char* ring = base;
  Ctrl* ctrl = reinterpret_cast<Ctrl*>(ring + (size_t)stages * kStage);
  double* sbins = reinterpret_cast<double*>(ctrl + 1);
  int* thr = reinterpret_cast<int*>(sbins + (kMaxBins + 1));
  double* kacc = reinterpret_cast<double*>(thr + (kMaxBins + 2));  // [kSlotSets][n_bins][kS]
  unsigned long long* kcnt =
      reinterpret_cast<unsigned long long*>(kacc + kSlotSets * a.n_bins * kS);  // [sets][n_bins]
  unsigned char* tables_u8 = reinterpret_cast<unsigned char*>(kcnt + kSlotSets * a.n_bins);
  tables_u8 += (16 - (smem_u32(tables_u8) & 15)) & 15;
  float* tables = reinterpret_cast<float*>(tables_u8);
  const float4* T4 = reinterpret_cast<const float4*>(tables);

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
      mbar_init(&ctrl->tempty[s], kUnitsPerTile);
    }
    mbar_init(&ctrl->drain, 1);
    ctrl->abort_flag = 0;
    ctrl->produced = 0;
    ctrl->consumed = 0;
    for (int q = 0; q < 4; ++q) ctrl->unit_next[q] = 0u;
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
    for (int x = t; x < kSlotSets * n_bins * kS; x += kEpiThreads) kacc[x] = 0.0;
    for (int x = t; x < kSlotSets * n_bins; x += kEpiThreads) kcnt[x] = 0ull;
    for (int x = t; x <= a.nmax; x += kEpiThreads)
      fast2::recip_entry4(x, reinterpret_cast<float4*>(tables) + x);
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

  long long n_items = MODE == kModeWindows ? a.tile_off[a.n_win] : a.item_off[a.n_rb];
  if (n_items < 0 || (MODE != kModeWindows && n_items > a.n_rb * a.n_cb)) {
    if (threadIdx.x == 0) set_abort(ctrl, a.status, 3001);
    n_items = 0;
  }
  if (MODE == kModeBinned && n_items > 0 && a.n_anchor < a.n_snp)
    n_items = a.item_off[(a.n_anchor + kRowSnp - 1) / kRowSnp];

  // Registers move from the producer / MMA warpgroup (warps 0-3) to the two
  // epilogue warpgroups: 128 x 56 + 256 x 224 = 384 x 168, the launch's total
  // (the host launches this kernel only when it was built with 168 registers).
  if (warp < 4) {
#if PGLD_TCW_MAXNREG
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kRegLo) : "memory");
#endif
    if (warp == 0 && lane == 0) {
      // ---------------- TMA producer ----------------
      int stage = 0;
      uint32_t phase = 0;
      int issued = 0;
      long long hint = 0;
      const long long n_copy_items = a.no_copies ? 0 : n_items;
      for (long long item = blockIdx.x; item < n_copy_items && !*abort_flag; item += gridDim.x) {
        int yi, yj;
        if constexpr (MODE == kModeWindows) {
          const WideTile tw = window_tile(a, item, hint);
          yi = (int)(2 * tw.i0);
          yj = (int)(2 * tw.j0);
        } else {
          const long long bi = row_of(a, item, hint);
          const long long bj = (bi * kRowSnp) / kColSnp + (item - a.item_off[bi]);
          yi = (int)(2 * bi * kRowSnp);
          yj = (int)(2 * bj * kColSnp);
        }
        for (int kc = 0; kc < a.kchunks; ++kc) {
          if (!role_wait<PGLD_TCW_NAP_LONG>(&ctrl->empty[stage], phase ^ 1, abort_flag, a.wait_cycles)) {
            set_abort(ctrl, a.status, 3002);
            break;
          }
          mbar_expect_tx(&ctrl->full[stage], kStage);
          unsigned char* sa = ring + (size_t)stage * kStage;
          tma_load_2d(sa, &map_a, &ctrl->full[stage], kc * kKChunk, yi);
          tma_load_2d(sa + kBoxA, &map_b, &ctrl->full[stage], kc * kKChunk, yj);
          ++issued;
          if (++stage == stages) {
            stage = 0;
            phase ^= 1;
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
    } else if (warp == 1 && lane == 0) {
      // ---------------- MMA issuer ----------------
      int stage = 0;
      uint32_t phase = 0;
      int t = 0;
      int consumed = 0;
      bool any = false;
      for (long long item = blockIdx.x; item < n_items && !*abort_flag; item += gridDim.x, ++t) {
        const int acc = t & 1;
        const uint32_t aph = (uint32_t)((t >> 1) & 1);
        if (!role_wait<PGLD_TCW_NAP_LONG>(&ctrl->tempty[acc], aph ^ 1, abort_flag, a.wait_cycles)) {
          set_abort(ctrl, a.status, 3003);
          break;
        }
        tc_fence_after();
        bool ok = true;
        const uint32_t d = tmem_base + (uint32_t)(acc * 256);
        for (int kc = 0; kc < a.kchunks; ++kc) {
          if (!role_wait<0>(&ctrl->full[stage], phase, abort_flag, a.wait_cycles)) {
            set_abort(ctrl, a.status, 3004);
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t sa = smem_u32(ring + (size_t)stage * kStage);
          const uint64_t da = smem_desc(sa), db = smem_desc(sa + kBoxA);
#pragma unroll
          for (int k = 0; k < kKChunk / 32; ++k)
            mma_w(d, da + (uint64_t)(k * 2), db + (uint64_t)(k * 2), (kc | k) != 0);
          mma_commit(&ctrl->empty[stage]);
          any = true;
          *(volatile int*)&ctrl->consumed = ++consumed;
          if (++stage == stages) {
            stage = 0;
            phase ^= 1;
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
  } else {
#if PGLD_TCW_MAXNREG
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kRegHi) : "memory");
#endif
    // ---------------- epilogue ----------------
    const int e = warp - 4;
    const int quarter = warp & 3;
    // the warps of a lane quarter take its 32-SNP column chunks ("units") of
    // the CTA's tiles, unit U = 4 t + u (tile t, chunk u), in order: each
    // takes the quarter's next unit when it is free (a shared counter), or,
    // without PGLD_TCW_DYN, unit U goes to the quarter's warp U mod (kEpiWarps / 4)
    constexpr int kPerQuarter = kEpiWarps / 4;
    const int k_in_q = e >> 2;
    const double maxd = a.max_dist;
    const int maxd_int = maxd >= 2147483647.0 ? 2147483647 : (int)floor(maxd);
    // the largest distance in a bin (below INT_MAX, so top + 1 does not wrap)
    const int top = MODE != kModeBinned ? 0 : thr[n_bins] > maxd_int ? maxd_int : thr[n_bins] - 1;
    const bool use_int = MODE == kModeBinned && (a.bcoord == nullptr) && (*a.ipos_bad == 0);
    double* my_acc = kacc + (size_t)(e & (kSlotSets - 1)) * n_bins * kS;
    unsigned long long* my_cnt = kcnt + (size_t)(e & (kSlotSets - 1)) * n_bins;
    auto slot_add = [&](int bin, int k, float v) { atomicAdd(my_acc + bin * kS + k, (double)v); };
    auto cnt_add = [&](int bin, unsigned long long v) { atomicAdd(my_cnt + bin, v); };
    long long hint = 0;
    bool aborted = false;
    auto u2 = [](uint32_t x, uint32_t y) {
      return make_float2(__uint_as_float(x), __uint_as_float(y));
    };
    // windows mode: the warp's running sums (per lane, compensated) and
    // counts of its current window, added to the window's totals by win_emit
    int cur_w = -1;
    float run[6], comp[6];
    int run_np = 0, run_r2 = 0, run_four = 0, run_units = 0;
#pragma unroll
    for (int s2 = 0; s2 < 6; ++s2) run[s2] = comp[s2] = 0.f;
    auto win_emit = [&]() {
      if (cur_w >= 0) {
#pragma unroll
        for (int s2 = 0; s2 < 6; ++s2) {
          double v = (double)run[s2] + (double)comp[s2];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          if (lane == 0 && v != 0.0) atomicAdd(a.wsums + (long long)cur_w * 6 + s2, v);
        }
        const int tp = __reduce_add_sync(0xffffffffu, run_np);
        const int tr2 = __reduce_add_sync(0xffffffffu, run_r2);
        const int tf = __reduce_add_sync(0xffffffffu, run_four);
        if (lane == 0) {
          if (tp) atomicAdd(a.wcnt + (long long)cur_w * 3 + 0, (unsigned long long)tp);
          if (tr2) atomicAdd(a.wcnt + (long long)cur_w * 3 + 1, (unsigned long long)tr2);
          if (tf) atomicAdd(a.wcnt + (long long)cur_w * 3 + 2, (unsigned long long)tf);
        }
      }
#pragma unroll
      for (int s2 = 0; s2 < 6; ++s2) run[s2] = comp[s2] = 0.f;
      run_np = run_r2 = run_four = run_units = 0;
    };
#pragma unroll 1
    for (long long Us = k_in_q;; Us += kPerQuarter) {
#if PGLD_TCW_DYN
      // the quarter's next unit, whichever of its warps is free first
      uint32_t un = 0;
      if (lane == 0) un = atomicAdd(&ctrl->unit_next[quarter], 1u);
      const long long U = (long long)__shfl_sync(0xffffffffu, un, 0);
#else
      const long long U = Us;
#endif
      const long long t = U >> 2;
      const int u = (int)(U & 3);
      const long long item = blockIdx.x + t * gridDim.x;
      if (item >= n_items) break;
      const int acc = (int)(t & 1);
      const uint32_t aph = (uint32_t)((t >> 1) & 1);
      long long i0, j0;
      WideTile tw{};
      if constexpr (MODE == kModeWindows) {
        tw = window_tile(a, item, hint);
        i0 = tw.i0;
        j0 = tw.j0;
      } else {
        const long long bi = row_of(a, item, hint);
        const long long bj = (bi * kRowSnp) / kColSnp + (item - a.item_off[bi]);
        i0 = bi * kRowSnp;
        j0 = bj * kColSnp;
      }
      const long long si0 = i0 + 16 * quarter;
      const long long ib = si0 + (lane >> 2);  // the lane's SNP i of row half 0 (half 1: + 8)
      // the unit's 16 x 32 sub-tile: i in si0 + [0, 16), j in sj0 + [0, 32)
      const long long sj0 = j0 + 32 * u;
      const uint32_t colb = (uint32_t)(acc * 256 + u * 64);
      auto release = [&]() {
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&ctrl->tempty[acc]);
      };
      auto wait_tile = [&]() {
        // every lane waits (no divergent branch around the wait)
        const bool ready =
            __all_sync(0xffffffffu, mbar_wait(&ctrl->tfull[acc], aph, abort_flag, a.wait_cycles));
        if (!ready && lane == 0) set_abort(ctrl, a.status, 3005);
        tc_fence_after();
        return ready;
      };

      if constexpr (MODE == kModePairs) {
        // per-pair outputs.  A 16x256b TMEM load gives thread t all four
        // counts of the pairs (i, j) and (i, j + 1), i = si0 + 8 hh + t / 4,
        // j = sj0 + 8 g + 2 (t % 4); output rows k = pair_off[i] + (j - i - 1)
        // in the reference's order, two consecutive rows per thread.  The band
        // offsets of the lane's rows are loaded before the accumulator wait.
        long long off0 = 0, np0 = 0, off1 = 0, np1 = 0;
        if (ib < a.n_snp) {
          off0 = a.pair_off[ib];
          np0 = a.pair_off[ib + 1] - off0;
        }
        if (ib + 8 < a.n_snp) {
          off1 = a.pair_off[ib + 8];
          np1 = a.pair_off[ib + 9] - off1;
        }
        // no pair of the unit in the band: below the diagonal, past the last
        // SNP, or past the band of each of its rows
        const bool past = __all_sync(0xffffffffu, sj0 - ib - 1 >= np0 && sj0 - ib - 9 >= np1);
        const bool none = past || sj0 + 31 <= si0 || si0 >= a.n_snp || sj0 >= a.n_snp;
        if (!wait_tile()) {
          aborted = true;
          break;
        }
        if (none) {
          release();
          continue;
        }
#pragma unroll 1
        for (int c = 0; c < 4; ++c) {
          const int hh = c & 1, gp = c >> 1;
          uint32_t r[16];
          tmem_ld16x256_x4(tmem_base + ((uint32_t)(quarter * 32 + hh * 16) << 16) + colb +
                               (uint32_t)(gp * 32),
                           r);
          tmem_wait_ld();
          if (c == 3) release();
          const long long is = ib + 8 * hh;
          const long long offh = hh ? off1 : off0, nph = hh ? np1 : np0;
#pragma unroll
          for (int g = 0; g < 2; ++g) {
            const int o = 8 * g;
            const long long j = sj0 + 8 * (2 * gp + g) + 2 * (lane & 3);
            // a pair's row comes from the band offsets themselves, so a pair
            // is written exactly when the offsets list it
            const bool ok0 = is < j && j < a.n_snp && (j - is - 1) < nph;
            const bool ok1 = is < j + 1 && j + 1 < a.n_snp && (j - is) < nph;
            if (!ok0 && !ok1) continue;
            const fast2::Pop p = fast2::make(u2(r[o], r[o + 1]), u2(r[o + 4], r[o + 5]),
                                             u2(r[o + 2], r[o + 3]), u2(r[o + 6], r[o + 7]));
            const long long k = offh + (j - is - 1);  // row of (is, j); (is, j + 1) follows
            float4 st[2];
            if (a.stats) fast2::pair_outputs(p, make_float2(T4[p.n0].w, T4[p.n1].w), st);
#pragma unroll
            for (int y = 0; y < 2; ++y) {
              const bool oky = y ? ok1 : ok0;
              const int q = o + y;
              st_cs_if(oky, reinterpret_cast<int4*>(a.counts) + (k + y),
                       make_int4(fast::f2i_small(__uint_as_float(r[q])),
                                 fast::f2i_small(__uint_as_float(r[q + 4])),
                                 fast::f2i_small(__uint_as_float(r[q + 2])),
                                 fast::f2i_small(__uint_as_float(r[q + 6]))));
              if (a.nvalid) st_cs_if(oky, a.nvalid + (k + y), y ? p.n1 : p.n0);
              if (a.stats) st_cs_if(oky, reinterpret_cast<float4*>(a.stats) + (k + y), st[y]);
            }
          }
        }
        continue;
      }

      if constexpr (MODE == kModeWindows) {
        // per-window sums: every pair of list positions begin <= i < j < end
        // of the tile's window; the unit's sums go to the warp's running sums
        // of its current window (flushed when the window changes)
        const long long wb_ = tw.begin, we_ = tw.end;
        const long long il = si0 > wb_ ? si0 : wb_, ih = si0 + 15 < we_ - 1 ? si0 + 15 : we_ - 1;
        const long long jl = sj0 > wb_ ? sj0 : wb_, jh = sj0 + 31 < we_ - 1 ? sj0 + 31 : we_ - 1;
        const bool none = il > ih || jl > jh || il >= jh;
        // every pair of the unit in the window
        const bool full = si0 >= wb_ && si0 + 15 < sj0 && sj0 + 31 < we_;
        // the naive-r^2 site terms of the lane's SNPs, loaded before the wait
        const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
        float4 wfi[2], wfj[8];
        auto site_at = [&](long long pos) {
          if (pos < wb_ || pos >= we_) return zero4;
          const long long sp = a.idx ? (long long)a.idx[pos] : pos;
          return (sp >= 0 && sp < a.n_panel) ? a.site[sp] : zero4;
        };
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) wfi[hh] = none ? zero4 : site_at(ib + 8 * hh);
#pragma unroll
        for (int q = 0; q < 8; ++q)
          wfj[q] = none ? zero4 : site_at(sj0 + 8 * (q >> 1) + 2 * (lane & 3) + (q & 1));
        if (!wait_tile()) {
          aborted = true;
          break;
        }
        if (none) {
          release();
          continue;
        }
        if (tw.w != cur_w) {
          win_emit();
          cur_w = tw.w;
        }
        float2 ws2[6];
#pragma unroll
        for (int s2 = 0; s2 < 6; ++s2) ws2[s2] = make_float2(0.f, 0.f);
        int np = 0, nr2 = 0, nfour = 0;
        auto tab = [&](int n) {
          const float4 e4 = T4[n];
          return make_float2(e4.x, e4.w);
        };
        auto body = [&](auto full_c) {
          constexpr bool F = decltype(full_c)::value;
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int hh = c & 1, gp = c >> 1;
            uint32_t r[16];
            tmem_ld16x256_x4(tmem_base + ((uint32_t)(quarter * 32 + hh * 16) << 16) + colb +
                                 (uint32_t)(gp * 32),
                             r);
            tmem_wait_ld();
            if (c == 3) release();
            const long long is = ib + 8 * hh;
            const bool iok = F || (is >= wb_ && is < we_);
            const float4 fi = wfi[hh];
            // the shorter form's n is the row SNP's nv: its r4 and n >= 4 once
            const int nvi = fast::f2i_small(fi.y);
            const float r4i = T4[nvi].w;
            const bool four_i = nvi >= 4;
#pragma unroll
            for (int g = 0; g < 2; ++g) {
              const int o = 8 * g;
              const int gg = 2 * gp + g;
              const long long j = sj0 + 8 * gg + 2 * (lane & 3);
              const bool l0 = F || (iok && is < j && j < we_);
              const bool l1 = F || (iok && is < j + 1 && j + 1 < we_);
              // a step without a live pair in any lane is skipped by the whole
              // warp (the vote below needs every lane)
              if (!F && !__any_sync(0xffffffffu, l0 || l1)) continue;
              const fast2::Pop p = fast2::make(u2(r[o], r[o + 1]), u2(r[o + 4], r[o + 5]),
                                               u2(r[o + 2], r[o + 3]), u2(r[o + 6], r[o + 7]));
              const float4 sj0 = l0 ? wfj[2 * gg] : zero4, sj1 = l1 ? wfj[2 * gg + 1] : zero4;
              // both SNPs of each live pair with the same valid haplotypes
              // (n = nv_i = nv_j), for every lane: the shorter form
              const bool same = (!l0 || (p.ns.x == fi.y && p.ns.x == sj0.y)) &&
                                (!l1 || (p.ns.y == fi.y && p.ns.y == sj1.y));
              if (__all_sync(0xffffffffu, same))
                win::window_pair2_same(p, four_i, r4i, fi, sj0, sj1, l0, l1, ws2, np, nr2, nfour);
              else
                win::window_pair2(p, u2(r[o], r[o + 1]), tab, fi, sj0, sj1, l0, l1, ws2, np, nr2,
                                  nfour);
            }
          }
        };
        if (full) body(std::true_type{});
        else body(std::false_type{});
        // compensated (Neumaier) running sums of the lane's unit totals
#pragma unroll
        for (int s2 = 0; s2 < 6; ++s2) {
          const float v = __fadd_rn(ws2[s2].x, ws2[s2].y);
          const float sum = __fadd_rn(run[s2], v);
          const float err = fabsf(run[s2]) >= fabsf(v) ? __fadd_rn(__fsub_rn(run[s2], sum), v)
                                                       : __fadd_rn(__fsub_rn(v, sum), run[s2]);
          comp[s2] = __fadd_rn(comp[s2], err);
          run[s2] = sum;
        }
        run_np += np;
        run_r2 += nr2;
        run_four += nfour;
        // bounded lane counts and compensated sums: flush every 4,096 units
        if (++run_units == 4096) win_emit();
        continue;
      }

      bool waited = false;
      {
        // classify: 0 one bin; 1 bin b0 below distance thr_mid, bin b0 + 1
        // from thr_mid below thr_hi, nothing from thr_hi; 2 general; 3 no
        // pair in a bin (the unit only releases its share of the buffer)
        int mode = 2, b0 = -1, thr_mid = 0, thr_hi = 0;
        if (use_int) {
          if (sj0 + 31 <= si0 || si0 >= a.n_anchor || sj0 >= a.n_snp) {
            mode = 3;
          } else if (sj0 >= si0 + 16 && sj0 + 31 < a.n_snp && si0 + 15 < a.n_anchor) {
            const int dmin = a.ipos[sj0] - a.ipos[si0 + 15];
            const int dmax = a.ipos[sj0 + 31] - a.ipos[si0];
            if (dmax < thr[0] || dmin > top) {
              mode = 3;
            } else {
              // (dmin, dmax are the same in every lane: one vote per lookup)
              const int blo = bin_of_int_warp(thr, n_bins, dmin, lane);
              const int bhi = bin_of_int_warp(thr, n_bins, min(dmax, top), lane);
              if (blo >= 0 && bhi == blo && dmax <= top) {
                mode = 0;
                b0 = blo;
              } else if (blo >= 0 && bhi >= blo && bhi <= blo + 1) {
                mode = 1;
                b0 = blo;
                thr_mid = min(thr[blo + 1], top + 1);
                thr_hi = max(thr_mid, blo + 2 <= n_bins ? min(thr[blo + 2], top + 1) : top + 1);
              }
            }
          }
        }
        // positions of the lane's SNPs for the sub-tiles that bin per pair
        // (rows ib, ib + 8; columns sj0 + 8 g + 2 (lane % 4) + y)
        int bp_i0 = 0, bp_i1 = 0, bp_j[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) bp_j[q] = 0;
        if (use_int && (mode == 1 || mode == 2)) {
          bp_i0 = ib < a.n_snp ? a.ipos[ib] : 0;
          bp_i1 = ib + 8 < a.n_snp ? a.ipos[ib + 8] : 0;
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const long long jq = sj0 + 8 * (q >> 1) + 2 * (lane & 3) + (q & 1);
            bp_j[q] = jq < a.n_snp ? a.ipos[jq] : 0;
          }
        }
        if (!waited) {
          // every lane waits (no divergent branch around the wait)
          const bool ready =
              __all_sync(0xffffffffu, mbar_wait(&ctrl->tfull[acc], aph, abort_flag, a.wait_cycles));
          if (!ready) {
            if (lane == 0) set_abort(ctrl, a.status, 3005);
            aborted = true;
          }
          tc_fence_after();
          waited = true;
        }
        if (aborted) break;
        if (mode == 3) {
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&ctrl->tempty[acc]);
          continue;
        }

        // four steps (row half hh, column pair gp) of 8 x 16 SNPs: one
        // 16x256b TMEM load gives thread t both planes of SNP i = t / 4 of
        // its 8-SNP row group against SNPs 2 (t % 4), 2 (t % 4) + 1 of two
        // 8-SNP column groups, each value both populations' count
        auto steps = [&](auto&& body) {
#pragma unroll kCUnroll
          for (int c = 0; c < 4; ++c) {
            const int hh = c & 1, gp = c >> 1;
            uint32_t r[16];
            tmem_ld16x256_x4(tmem_base + ((uint32_t)(quarter * 32 + hh * 16) << 16) + colb +
                                 (uint32_t)(gp * 32),
                             r);
            tmem_wait_ld();
            if (c == 3) {
              // the unit's last TMEM load: release its share of the buffer
              tc_fence_before();
              __syncwarp();
              if (lane == 0) mbar_arrive(&ctrl->tempty[acc]);
            }
            auto u2 = [](uint32_t x, uint32_t y) {
              return make_float2(__uint_as_float(x), __uint_as_float(y));
            };
#pragma unroll
            for (int g = 0; g < 2; ++g) {
              const int o = 8 * g;
              float2 n11[2], n10[2], n01[2], n00[2];
              split2(u2(r[o], r[o + 1]), n11[0], n11[1]);
              split2(u2(r[o + 4], r[o + 5]), n10[0], n10[1]);
              split2(u2(r[o + 2], r[o + 3]), n01[0], n01[1]);
              split2(u2(r[o + 6], r[o + 7]), n00[0], n00[1]);
              const fast2::Pop p0 = fast2::make(n11[0], n10[0], n01[0], n00[0]);
              const fast2::Pop p1 = fast2::make(n11[1], n10[1], n01[1], n00[1]);
              body(hh, 2 * gp + g, p0, p1);
            }
          }
        };
        auto jx_of = [&](int g) { return sj0 + 8 * g + 2 * (lane & 3); };
        auto jpos = [&](int g, int y) {
          const int a0 = y ? bp_j[1] : bp_j[0], a1 = y ? bp_j[3] : bp_j[2];
          const int a2 = y ? bp_j[5] : bp_j[4], a3 = y ? bp_j[7] : bp_j[6];
          return g == 0 ? a0 : g == 1 ? a1 : g == 2 ? a2 : a3;
        };

        if (mode == 0) {
          // one bin: packed sums, each statistic's reciprocal factor fused
          float2 acc2[kS];
#pragma unroll
          for (int s = 0; s < kS; ++s) acc2[s] = make_float2(0.f, 0.f);
          steps([&](int, int, const fast2::Pop& p0, const fast2::Pop& p1) {
#if PGLD_TCW_SSINK
            fast2::stats2_to(p0, p1, T4,
                             [&](int k, float2 num, float2 sc) { acc2[k] = fast2::vfma_s(num, sc, acc2[k]); });
#else
            fast2::stats2_to(p0, p1, T4,
                             [&](int k, float2 num, float2 sc) { acc2[k] = fast2::vfma(num, sc, acc2[k]); });
#endif
          });
          float v[kS];
#pragma unroll
          for (int s = 0; s < kS; ++s) v[s] = acc2[s].x + acc2[s].y;
          const float tot = warp_totals<kS>(v, lane);
          constexpr int sh_t = totals_shift<kS>();
          const int k = lane >> sh_t;
          if ((lane & ((1 << sh_t) - 1)) == 0 && k < kS) slot_add(b0, k, tot);
          if (lane == 31) cnt_add(b0, 512ull);
        } else if (mode == 1) {
          // bins b0 (d < thr_mid) and b0 + 1 (thr_mid <= d < thr_hi)
          float acc_lo[kS], acc_hi[kS];
          int n_lo = 0, n_hi = 0;
#pragma unroll
          for (int s = 0; s < kS; ++s) acc_lo[s] = acc_hi[s] = 0.f;
          steps([&](int hh, int g, const fast2::Pop& p0, const fast2::Pop& p1) {
            const int ipi = hh ? bp_i1 : bp_i0;
            const int d0 = jpos(g, 0) - ipi, d1 = jpos(g, 1) - ipi;
            const bool lo0 = d0 < thr_mid, lo1 = d1 < thr_mid;
            const bool hi0 = !lo0 && d0 < thr_hi, hi1 = !lo1 && d1 < thr_hi;
            const float2 fu = make_float2(hi0 ? 1.f : 0.f, hi1 ? 1.f : 0.f);
            const float2 fl = make_float2(lo0 ? 1.f : 0.f, lo1 ? 1.f : 0.f);
            n_lo += (lo0 ? 1 : 0) + (lo1 ? 1 : 0);
            n_hi += (hi0 ? 1 : 0) + (hi1 ? 1 : 0);
            fast2::stats2_to(p0, p1, T4, [&](int kk, float2 num, float2 sc) {
              const float2 st = fast2::vmul(num, sc);
              acc_hi[kk] = fmaf(fu.x, st.x, fmaf(fu.y, st.y, acc_hi[kk]));
              acc_lo[kk] = fmaf(fl.x, st.x, fmaf(fl.y, st.y, acc_lo[kk]));
            });
          });
          constexpr int sh_t = totals_shift<kS>();
          const int k = lane >> sh_t;
          const bool leader = (lane & ((1 << sh_t) - 1)) == 0 && k < kS;
          const int lo_total = __reduce_add_sync(0xffffffffu, n_lo);
          const int hi_total = __reduce_add_sync(0xffffffffu, n_hi);
          if (lo_total) {
            const float tlo = warp_totals<kS>(acc_lo, lane);
            if (leader) slot_add(b0, k, tlo);
          }
          if (hi_total) {
            const float thi = warp_totals<kS>(acc_hi, lane);
            if (leader) slot_add(b0 + 1, k, thi);
          }
          if (lane == 31) {
            if (lo_total) cnt_add(b0, (unsigned long long)lo_total);
            if (hi_total) cnt_add(b0 + 1, (unsigned long long)hi_total);
          }
        } else {
          // general (diagonal and band-edge sub-tiles, short distances,
          // non-integer positions): per step, the bins of the lane's two
          // pairs; steps over at most two adjacent bins go to running sums
          // of bins (key, key + 1), the others take one warp total per bin
          float acc_lo[kS], acc_hi[kS];
#pragma unroll
          for (int s = 0; s < kS; ++s) acc_lo[s] = acc_hi[s] = 0.f;
          int key = -1, n_lo = 0, n_hi = 0;
          constexpr int sh_t = totals_shift<kS>();
          const int kl = lane >> sh_t;
          const bool leader = (lane & ((1 << sh_t) - 1)) == 0 && kl < kS;
          auto flush = [&]() {
            if (key < 0) return;
            const float tlo = warp_totals<kS>(acc_lo, lane);
            if (leader) slot_add(key, kl, tlo);
            const int tl = __reduce_add_sync(0xffffffffu, n_lo);
            const int th = __reduce_add_sync(0xffffffffu, n_hi);
            if (th) {
              const float thi = warp_totals<kS>(acc_hi, lane);
              if (leader) slot_add(key + 1, kl, thi);
            }
            if (lane == 31) {
              cnt_add(key, (unsigned long long)tl);
              if (th) cnt_add(key + 1, (unsigned long long)th);
            }
#pragma unroll
            for (int s = 0; s < kS; ++s) acc_lo[s] = acc_hi[s] = 0.f;
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
            const int ipi = hh ? bp_i1 : bp_i0;
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
              fast2::stats2_to(p0, p1, T4, [&](int kk, float2 num, float2 sc) {
                const float2 st = fast2::vmul(num, sc);
                acc_hi[kk] = fmaf(fu.x, st.x, fmaf(fu.y, st.y, acc_hi[kk]));
                acc_lo[kk] = fmaf(fl.x, st.x, fmaf(fl.y, st.y, acc_lo[kk]));
              });
              return;
            }
            flush();
            float2 st[kS];
            fast2::stats2_raw(p0, p1, T4, st);
            // one warp total per distinct bin of the step's 64 pairs (both
            // pairs of a lane at once), lowest bin first
            int rx = bx, ry = by;
#pragma unroll 1
            for (;;) {
              const int lo2 = min(rx < 0 ? 0x7fffffff : rx, ry < 0 ? 0x7fffffff : ry);
              const int bb = __reduce_min_sync(0xffffffffu, lo2);
              if (bb == 0x7fffffff) break;
              const bool mx = rx == bb, my = ry == bb;
              float v[kS];
#pragma unroll
              for (int s = 0; s < kS; ++s) v[s] = (mx ? st[s].x : 0.f) + (my ? st[s].y : 0.f);
              const float tot = warp_totals<kS>(v, lane);
              if (leader) slot_add(bb, kl, tot);
              const int nb = __reduce_add_sync(0xffffffffu, (mx ? 1 : 0) + (my ? 1 : 0));
              if (lane == 31) cnt_add(bb, (unsigned long long)nb);
              if (mx) rx = -1;
              if (my) ry = -1;
            }
          });
          flush();
        }
      }
      if (!waited) break;  // the accumulator wait ran out (recorded above)
    }
    if constexpr (MODE == kModeWindows)
      if (!aborted) win_emit();
  }

  // ---------------- teardown ----------------
  tc_fence_before();
  __syncthreads();
  if (warp >= 4 && !ctrl->abort_flag) {
    const int t = threadIdx.x - 128;
    for (int x = t; x < n_bins * kS; x += kEpiThreads) {
      double v = 0.0;
#pragma unroll
      for (int w = 0; w < kSlotSets; ++w) v += kacc[w * n_bins * kS + x];
      v *= fast2::post2(x % kS);
      if (v != 0.0) atomicAdd(a.sums + x, v);
    }
    if (a.pair_counts)
      for (int x = t; x < n_bins; x += kEpiThreads) {
        unsigned long long v = 0;
#pragma unroll
        for (int w = 0; w < kSlotSets; ++w) v += kcnt[w * n_bins + x];
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

// Both populations' bit planes -> one E4M3 operand (rows grouped by 8 SNPs:
// row 16g + 8 plane + k is plane `plane` of SNP 8g + k; SNPs past n_snp are
// zero rows).  Bytes [0, k0) of a row: population 0 (1.0), [k0, k0 + k1):
// population 1 (64.0).  A block writes 8 rows, a warp one row in 16-byte
// chunks.
__global__ void __launch_bounds__(256) pack_wide_kernel(const uint32_t* __restrict__ pl0, int W0,
                                                        const uint32_t* __restrict__ pl1, int W1,
                                                        long long n_snp, long long rows_out, int k0,
                                                        int k1, uint32_t* __restrict__ out) {
  const long long rowi = (long long)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (rowi >= rows_out) return;
  const int chunks0 = k0 / 16, chunks = (k0 + k1) / 16;
  uint4* dst = reinterpret_cast<uint4*>(out) + rowi * chunks;
  const long long r = (rowi >> 4) * 8 + (rowi & 7);
  const int plane = (int)((rowi >> 3) & 1);
  const bool live = r < n_snp;
  const uint32_t* src0 = pl0 + (live ? r : 0) * 2 * W0 + plane * W0;
  const uint32_t* src1 = pl1 + (live ? r : 0) * 2 * W1 + plane * W1;
  for (int c = lane; c < chunks; c += 32) {
    const bool p1 = c >= chunks0;
    const int h0 = 16 * (p1 ? c - chunks0 : c);
    const int w = h0 >> 5;
    const uint32_t one = p1 ? kOne64 : kOne;
    uint32_t bits = 0u;
    if (live) {
      if (!p1 && w < W0) bits = (__ldg(src0 + w) >> (h0 & 31)) & 0xFFFFu;
      if (p1 && w < W1) bits = (__ldg(src1 + w) >> (h0 & 31)) & 0xFFFFu;
    }
    uint32_t v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t nib = (bits >> (4 * q)) & 0xFu;
      v[q] = (nib & 1u ? one : 0u) | (nib & 2u ? one << 8 : 0u) | (nib & 4u ? one << 16 : 0u) |
             (nib & 8u ? one << 24 : 0u);
    }
    dst[c] = make_uint4(v[0], v[1], v[2], v[3]);
  }
}

__global__ void pos_to_int_kernel_w(const double* __restrict__ pos, long long n, int* __restrict__ ipos,
                                    int* __restrict__ bad) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const double v = pos[k];
    const bool ok = (v == rint(v)) && fabs(v) < 1073741824.0;
    ipos[k] = ok ? (int)v : 0;
    if (!ok) atomicOr(bad, 1);
  }
}

// 64 x 128 tiles of each window's upper triangle (list positions from
// win_begin & ~7); bad ranges get none and set the status
__global__ void wide_window_tiles_kernel(const long long* __restrict__ wb,
                                         const long long* __restrict__ we, int n_win,
                                         long long n_idx, long long* __restrict__ tiles,
                                         int32_t* __restrict__ status) {
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < n_win; w += gridDim.x * blockDim.x) {
    const long long lo = wb[w], hi = we[w];
    long long T = 0;
    if (lo < 0 || hi < lo || hi > n_idx) {
      atomicCAS(status, 0, 3100);
    } else if (hi > lo) {
      const long long m = hi - (lo & ~7ll);
      T = wtiles_before((m + kRowSnp - 1) / kRowSnp, (m + kColSnp - 1) / kColSnp);
    }
    tiles[w] = T;
  }
}

}  // namespace tcw
}  // namespace pgld

using pgld::tchost::get_encode;
using pgld::tchost::make_map;

// The combined-population form applies to two populations of at most 2,016
// haplotypes each (63 words: c0 / 4096 < 0.5) without a validity plane.
int pgld_tc_wide_supported(const pgld_hap_panel* panel) {
  if (panel->n_pops != 2) return 0;
  for (int p = 0; p < 2; ++p)
    if (panel->valid[p] != nullptr || panel->n_words[p] > 63) return 0;
  return 1;
}

int pgld_tc_wide_binned(pgld_context* h, const pgld_hap_panel* panel, pgld::BandArgs& a,
                        cudaStream_t st) {
  using namespace pgld::tcw;
  int rc = get_encode(h);
  if (rc) return rc;
  const long long n = panel->n_snp;
  const long long n_rb = (n + kRowSnp - 1) / kRowSnp;
  const long long n_cb = (n + kColSnp - 1) / kColSnp;
  // operand rows: SNPs rounded up to whole 128-SNP column blocks (B boxes
  // stay inside the matrix), two planes each, grouped by 8 SNPs
  const long long n_op = n_cb * kColSnp;
  if (2 * n_op > 2147483647LL) return pgld_fail(h, PGLD_ERR_TOO_LARGE, "tensor-core form: too many SNPs");
  const int k0 = ((panel->n_words[0] * 32 + pgld::tc::kKChunk - 1) / pgld::tc::kKChunk) * pgld::tc::kKChunk;
  const int k1 = ((panel->n_words[1] * 32 + pgld::tc::kKChunk - 1) / pgld::tc::kKChunk) * pgld::tc::kKChunk;
  const size_t op_bytes = (size_t)2 * n_op * (k0 + k1);
  const size_t sb = pgld::scan_scratch_bytes(n_rb);
  auto al = [](size_t x) { return (x + 1023) & ~size_t(1023); };
  const size_t off_items = 0, off_scan = al((n_rb + 1) * 8), off_op = off_scan + al(sb),
               off_ipos = off_op + al(op_bytes), off_bad = off_ipos + al((size_t)n * 4),
               total = off_bad + 1024;
  void* ws = nullptr;
  rc = pgld_workspace(h, total, &ws);
  if (rc) return rc;
  char* w = (char*)ws;
  long long* items = (long long*)(w + off_items);
  unsigned char* op = (unsigned char*)(w + off_op);
  {
    const unsigned blocks = (unsigned)((2 * n_op + 7) / 8);
    pack_wide_kernel<<<blocks, 256, 0, st>>>(panel->planes[0], panel->n_words[0], panel->planes[1],
                                             panel->n_words[1], n, 2 * n_op, k0, k1, (uint32_t*)op);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "pack_wide_kernel");
  }
  rc = pgld::band_schedule(h, a.pos, n, a.max_dist, items, w + off_scan, sb, st, kRowSnp, kColSnp);
  if (rc) return rc;
  int* ipos = (int*)(w + off_ipos);
  int* ipos_bad = (int*)(w + off_bad);
  {
    cudaError_t e = cudaMemsetAsync(ipos_bad, 0, 4, st);
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "memset");
    unsigned blocks = (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, h->n_sm * 8));
    pos_to_int_kernel_w<<<blocks, 256, 0, st>>>(a.pos, n, ipos, ipos_bad);
    e = cudaGetLastError();
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "pos_to_int_kernel");
  }
  CUtensorMap map_a, map_b;
  rc = make_map(h, &map_a, op, 2 * n_op, k0 + k1, 128);
  if (rc) return rc;
  rc = make_map(h, &map_b, op, 2 * n_op, k0 + k1, 256);
  if (rc) return rc;

  Params prm{};
  prm.kchunks = (k0 + k1) / pgld::tc::kKChunk;
  prm.n_snp = n;
  prm.n_anchor = pgld::anchors_of(a);
  prm.pos = a.pos;
  prm.max_dist = a.max_dist;
  prm.bcoord = a.bcoord;
  prm.bins = a.bins;
  prm.n_bins = a.n_bins;
  prm.item_off = items;
  prm.n_rb = n_rb;
  prm.n_cb = n_cb;
  prm.sums = a.sums;
  prm.pair_counts = a.pair_counts;
  prm.status = h->dev_status;
  prm.nmax = 32 * std::max(panel->n_words[0], panel->n_words[1]);
  prm.ipos = ipos;
  prm.ipos_bad = ipos_bad;
  prm.wait_cycles = pgld::tc::kWaitCycles;
  if (h->test_fault == PGLD_TEST_FAULT_NO_COPIES) {
    prm.no_copies = 1;
    prm.wait_cycles = 20000000ll;
    h->test_fault = 0;
  }
  const size_t fixed = sizeof(pgld::tc::Ctrl) + (pgld::kMaxBins + 1) * 8 + (pgld::kMaxBins + 2) * 4 +
                       (size_t)kSlotSets * a.n_bins * (kS + 1) * 8 +
                       (size_t)4 * (prm.nmax + 1) * sizeof(float) + 16 + 1024;
  int max_smem = 0;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  int stages = (int)std::min<long long>(8, ((long long)max_smem - (long long)fixed) / kStage);
  if (h->tc_stages_cap > 0) stages = std::min(stages, h->tc_stages_cap);
  if (stages < 2) return pgld_fail(h, PGLD_ERR_TOO_LARGE, "tensor-core form: shared memory");
  prm.stages = stages;
  const size_t smem = (size_t)stages * kStage + fixed;
  auto kern = band_wide_kernel<pgld::kModeBinned>;
#if PGLD_TCW_MAXNREG
  {
    // the register split needs the launch's total (384 x 168): a build that
    // allocated fewer would make the epilogue's increase wait forever
    cudaFuncAttributes fa;
    cudaError_t e0 = cudaFuncGetAttributes(&fa, (const void*)kern);
    if (e0 != cudaSuccess) return pgld_cuda_fail(h, e0, "band_wide attributes");
    if (fa.numRegs != kRegLaunch)
      return pgld_fail(h, PGLD_ERR_UNSUPPORTED, "band_wide_kernel built with %d registers; its "
                       "register split needs %d", fa.numRegs, kRegLaunch);
  }
#endif
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_wide smem attribute");
  pgld_time_begin(h, st);
  kern<<<(unsigned)h->n_sm, kThreads, smem, st>>>(map_a, map_b, prm);
  pgld_time_end(h, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_wide_kernel");
  return PGLD_OK;
}

// ---------------------------------------------------------------------------
// one population: per-pair outputs and per-window sums on 64 x 128 tiles
// ---------------------------------------------------------------------------
int pgld_tc_pack_rows(pgld_context* h, const uint32_t* planes, int W, long long n_snp,
                      long long n_rows, const int32_t* idx, int k_pad, unsigned char* out,
                      cudaStream_t st);
int pgld_site_freqs(pgld_context* h, const uint32_t* planes, const uint32_t* valid, int W,
                    long long n_snp, float4* site, cudaStream_t st);

// shared memory, stages and the register check of a one-population launch
template <int MODE>
static int wide_one_pop_launch(pgld_context* h, pgld::tcw::Params& prm, const CUtensorMap& map_a,
                               const CUtensorMap& map_b, cudaStream_t st, const char* what) {
  using namespace pgld::tcw;
  if (h->test_fault == PGLD_TEST_FAULT_NO_COPIES) {
    prm.no_copies = 1;
    prm.wait_cycles = 20000000ll;
    h->test_fault = 0;
  }
  const size_t fixed = sizeof(pgld::tc::Ctrl) + (pgld::kMaxBins + 1) * 8 + (pgld::kMaxBins + 2) * 4 +
                       (size_t)4 * (prm.nmax + 1) * sizeof(float) + 16 + 1024;
  int max_smem = 0;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  int stages = (int)std::min<long long>(8, ((long long)max_smem - (long long)fixed) / kStage);
  if (h->tc_stages_cap > 0) stages = std::min(stages, h->tc_stages_cap);
  if (stages < 2) return pgld_fail(h, PGLD_ERR_TOO_LARGE, "%s: shared memory", what);
  prm.stages = stages;
  const size_t smem = (size_t)stages * kStage + fixed;
  auto kern = band_wide_kernel<MODE>;
#if PGLD_TCW_MAXNREG
  {
    cudaFuncAttributes fa;
    cudaError_t e0 = cudaFuncGetAttributes(&fa, (const void*)kern);
    if (e0 != cudaSuccess) return pgld_cuda_fail(h, e0, "band_wide attributes");
    if (fa.numRegs != kRegLaunch)
      return pgld_fail(h, PGLD_ERR_UNSUPPORTED, "band_wide_kernel built with %d registers; its "
                       "register split needs %d", fa.numRegs, kRegLaunch);
  }
#endif
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "band_wide smem attribute");
  pgld_time_begin(h, st);
  kern<<<(unsigned)h->n_sm, kThreads, smem, st>>>(map_a, map_b, prm);
  pgld_time_end(h, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, what);
  return PGLD_OK;
}

// Per-pair outputs of one population (<= 2,048 haplotypes, no validity
// plane) over the distance band: a's pair_off / counts / nvalid / stats as
// for the square form; the band offsets are rebuilt in this call's workspace.
int pgld_tc_wide_pairs(pgld_context* h, const pgld_hap_panel* panel, pgld::BandArgs& a,
                       cudaStream_t st) {
  using namespace pgld::tcw;
  int rc = get_encode(h);
  if (rc) return rc;
  const long long n = panel->n_snp;
  const int W = panel->n_words[0];
  const long long n_rb = (n + kRowSnp - 1) / kRowSnp;
  const long long n_cb = (n + kColSnp - 1) / kColSnp;
  const long long n_op = n_cb * kColSnp;
  if (2 * n_op > 2147483647LL) return pgld_fail(h, PGLD_ERR_TOO_LARGE, "tensor-core form: too many SNPs");
  const int k0 = ((W * 32 + pgld::tc::kKChunk - 1) / pgld::tc::kKChunk) * pgld::tc::kKChunk;
  const size_t op_bytes = (size_t)2 * n_op * k0;
  const size_t sb = pgld::scan_scratch_bytes(std::max<long long>(n_rb, n));
  auto al = [](size_t x) { return (x + 1023) & ~size_t(1023); };
  const size_t off_items = 0, off_scan = al((n_rb + 1) * 8), off_op = off_scan + al(sb),
               off_poff = off_op + al(op_bytes), total = off_poff + al((size_t)(n + 1) * 8);
  void* ws = nullptr;
  rc = pgld_workspace(h, total, &ws);
  if (rc) return rc;
  char* w = (char*)ws;
  long long* items = (long long*)(w + off_items);
  unsigned char* op = (unsigned char*)(w + off_op);
  long long* poff = (long long*)(w + off_poff);
  rc = pgld_band_offsets(h, a.pos, n, a.max_dist, poff, w + off_scan, sb, st);
  if (rc) return rc;
  {
    const unsigned blocks = (unsigned)((2 * n_op + 7) / 8);
    pack_wide_kernel<<<blocks, 256, 0, st>>>(panel->planes[0], W, panel->planes[0], 0, n, 2 * n_op,
                                             k0, 0, (uint32_t*)op);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "pack_wide_kernel");
  }
  rc = pgld::band_schedule(h, a.pos, n, a.max_dist, items, w + off_scan, sb, st, kRowSnp, kColSnp);
  if (rc) return rc;
  CUtensorMap map_a, map_b;
  rc = make_map(h, &map_a, op, 2 * n_op, k0, 128);
  if (rc) return rc;
  rc = make_map(h, &map_b, op, 2 * n_op, k0, 256);
  if (rc) return rc;
  Params prm{};
  prm.kchunks = k0 / pgld::tc::kKChunk;
  prm.n_snp = n;
  prm.n_anchor = n;
  prm.pos = a.pos;
  prm.max_dist = a.max_dist;
  prm.item_off = items;
  prm.n_rb = n_rb;
  prm.n_cb = n_cb;
  prm.status = h->dev_status;
  prm.nmax = 32 * W;
  prm.wait_cycles = pgld::tc::kWaitCycles;
  prm.pair_off = poff;
  prm.counts = a.counts;
  prm.nvalid = a.nvalid;
  prm.stats = a.stats;
  return wide_one_pop_launch<pgld::kModePairs>(h, prm, map_a, map_b, st, "band_wide_kernel (pairs)");
}

// Per-window sums of one population (<= 2,048 haplotypes, no validity plane):
// the operand is built over the index list, so a window is a contiguous range
// of operand rows; one launch over the tiles of every window.
int pgld_tc_wide_windows(pgld_context* h, const pgld_hap_panel* panel, const int32_t* idx,
                         long long n_idx, const long long* wb, const long long* we, int n_win,
                         double* sums, unsigned long long* counts, cudaStream_t st) {
  using namespace pgld::tcw;
  int rc = get_encode(h);
  if (rc) return rc;
  const long long n = panel->n_snp;
  const int W = panel->n_words[0];
  const int k_pad = ((W * 32 + pgld::tc::kKChunk - 1) / pgld::tc::kKChunk) * pgld::tc::kKChunk;
  // operand rows: list positions grouped by 8, then zero rows for the column
  // blocks that reach past the last position (a tile's columns start at most
  // 127 positions before its window's end)
  const long long n_pk = (std::max<long long>(n_idx, 1) + 7) / 8 * 8;
  const long long n_op = n_pk + kColSnp;
  if (2 * n_op > 2147483647LL - 256)
    return pgld_fail(h, PGLD_ERR_TOO_LARGE, "tensor-core windows: too many SNPs");
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
    wide_window_tiles_kernel<<<gb, 256, 0, st>>>(wb, we, n_win, n_idx, tiles, h->dev_status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "wide_window_tiles_kernel");
  }
  rc = pgld::exclusive_scan_i64(h, tiles, n_win, w + off_scan, sb, st);
  if (rc) return rc;
  if (n > 0) {
    rc = pgld_site_freqs(h, panel->planes[0], nullptr, W, n, site, st);
    if (rc) return rc;
  }
  if (n_idx > 0) {
    rc = pgld_tc_pack_rows(h, panel->planes[0], W, n, n_idx, idx, k_pad, op, st);
    if (rc) return rc;
  }
  {
    const size_t packed = n_idx > 0 ? (size_t)2 * n_pk * k_pad : 0;
    cudaError_t e = cudaMemsetAsync(op + packed, 0, op_bytes - packed, st);
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "memset");
  }
  CUtensorMap map_a, map_b;
  rc = make_map(h, &map_a, op, 2 * n_op, k_pad, 128);
  if (rc) return rc;
  rc = make_map(h, &map_b, op, 2 * n_op, k_pad, 256);
  if (rc) return rc;
  Params prm{};
  prm.kchunks = k_pad / pgld::tc::kKChunk;
  prm.n_snp = n_idx;
  prm.n_anchor = n_idx;
  prm.status = h->dev_status;
  prm.nmax = 32 * W;
  prm.wait_cycles = pgld::tc::kWaitCycles;
  prm.win_begin = wb;
  prm.win_end = we;
  prm.n_win = n_win;
  prm.tile_off = tiles;
  prm.idx = idx;
  prm.site = site;
  prm.n_panel = n;
  prm.wsums = sums;
  prm.wcnt = counts;
  return wide_one_pop_launch<pgld::kModeWindows>(h, prm, map_a, map_b, st,
                                                 "band_wide_kernel (windows)");
}
