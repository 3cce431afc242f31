// tcgen05 tensor-core form of the genotype distance-band pairs (sm_103a).
//
// Everything a single-population pair needs -- the 9-way counts, the
// pairwise-valid n, Rogers-Huff r^2 and the moments DD, Dz, pi2 -- follows
// from the nine centred moments m[3 x + y] = sum c_i^x c_j^y over the
// individuals valid at both SNPs, c = dosage - 1 in {-1, 0, 1}
// (pgld_geno_mom.cuh).  Those are dot products over the individuals: with A =
// the planes (valid, c, c^2) of 32 SNPs i and B the same for 32 SNPs j,
// D = A B^T holds m[3 x + y] for all 1,024 pairs of the tile.  The operand
// rows are plane-major within a 32-SNP block (row = 96 * block + 32 * plane
// + SNP), so D[32 x + i][32 y + j] = m[3 x + y](i, j); the A tile's rows
// 96..127 (M = 128) are zero rows kept in shared memory.
// Operands are E4M3 bytes (0x38 = 1.0, 0xB8 = -1.0) in K-major rows padded to
// 128 bytes; the float32 accumulators hold integers of magnitude below 2^24,
// so the moments are exact.
//
// One CTA per SM:
//   warp 0      TMA producer (96-row x 128-byte boxes, SWIZZLE_128B; 28 KB
//               stages, so six are in flight)
//   warp 1      allocates 256 TMEM columns; one lane issues M=128 N=96 K=32
//               kind::f8f6f4 MMAs (the B rows of planes 0-2) into
//               accumulator stage t % 2
//   warps 4-11  epilogue: two groups of four warps on alternate tiles
//               (accumulator stage and moment buffer per group); in a group
//               the warps of TMEM lane quarters 0-2 (planes 0-2) copy the
//               3 x 3 moment blocks to shared memory, then all four turn
//               1,024 pairs into outputs (8 per thread)
// Every mbarrier wait is bounded; the warps of an epilogue group meet at
// their named barrier twice per tile and agree on aborting at the first.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "pgld_band.cuh"
#include "pgld_epilogue.cuh"
#include "pgld_geno_mom.cuh"
#include "pgld_internal.cuh"
#include "pgld_geno.cuh"
#include "pgld_scan.cuh"
#include "pgld_tc_common.cuh"
#include "pgld_tcgen05.cuh"

namespace pgld {
namespace gtc {

using namespace pgld::tc;

constexpr int kTileSnp = 32;          // SNPs per tile side (4 planes = 128 rows)
constexpr int kEpiWarps = 8;
constexpr int kThreads = (4 + kEpiWarps) * 32;
constexpr uint32_t kTmemCols = 256;   // two accumulator stages of 128 columns
constexpr int kBlkRows = 96;          // operand rows of a 32-SNP block (3 planes)
constexpr int kABytes = kBoxBytes;     // A: 96 loaded rows + 32 zero rows (M = 128)
constexpr int kBBytes = kBlkRows * kKChunk;  // B: 96 rows (N = 96)
constexpr int kGStageBytes = kABytes + kBBytes;  // 28 KB
constexpr int kCntPitch = 98;         // int16 pitch of the 96 x 96 moment block (49 words: odd)
// instruction descriptor: D f32, A/B E4M3, both K-major, N = 96, M = 128
constexpr uint32_t kIdescN96 = (1u << 4) | ((96u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mma_f8_n96(uint32_t dtmem, uint64_t a, uint64_t b,
                                           uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(kIdescN96), "r"(accum)
      : "memory");
}

struct Params {
  int kchunks;
  long long n_snp;
  const long long* item_off;
  long long n_blocks;
  const long long* pair_off;
  int32_t* counts;   // [n_pairs][9] or NULL
  int32_t* nvalid;   // [n_pairs] or NULL
  float* stats;      // [n_pairs][4] or NULL
  int stat_mask;
  int32_t* status;
  int stages;
};

constexpr int kChunkItems = 16;  // consecutive tiles a CTA takes per turn (resident form)

// control block: the stage / accumulator barriers, plus the resident form's
// B barriers and the per-stage tile flags the producer hands the MMA issuer
struct GCtrl : Ctrl {
  uint64_t bfull, bempty;
  int meta[8];  // first stage of a tile: bit 0 = first tile of a strip, bit 1 = last
};

// the t-th tile of this CTA: turns of `chunk` consecutive items, round robin
// over the CTAs (chunk 1: item blockIdx.x + t * gridDim.x)
__device__ __forceinline__ long long tile_item(int t, int chunk) {
  return ((long long)blockIdx.x + (long long)(t / chunk) * gridDim.x) * chunk + t % chunk;
}

// row block of an item, moving forward from lo (the items a thread visits
// ascend): a few steps, then a binary search
__device__ __forceinline__ long long advance_block(const long long* item_off, long long n_blocks,
                                                   long long lo, long long item) {
#pragma unroll 1
  for (int s = 0; s < 4; ++s) {
    if (lo + 1 >= n_blocks || item_off[lo + 1] > item) return lo;
    ++lo;
  }
  long long hi = n_blocks;
  while (hi - lo > 1) {
    const long long mid = (lo + hi) >> 1;
    if (item_off[mid] <= item) lo = mid; else hi = mid;
  }
  return lo;
}

// MASK: the statistic columns when fixed at compile time (-1: a.stat_mask).
// RES: the resident form -- the row block's 96 operand rows (every K chunk)
// stay in shared memory as the B operand (N = 96) for a strip of consecutive
// tiles of that row block, and only the column block streams (A, M = 128 with
// 32 zero rows); the accumulator is then transposed (lanes: planes of the
// SNPs j, columns: planes of the SNPs i).  Otherwise both blocks stream per
// K chunk (A = row block, B = column block).
template <int MASK, bool RES>
__global__ void __launch_bounds__(kThreads, 1)
    gtc_pairs_kernel(const __grid_constant__ CUtensorMap map, Params a) {
  extern __shared__ unsigned char smem_dyn[];
  unsigned char* base = smem_dyn + ((1024 - (smem_u32(smem_dyn) & 1023)) & 1023);
  const int stages = a.stages;
  constexpr int kStage = RES ? kABytes : kGStageBytes;
  const int chunk = RES ? kChunkItems : 1;
  unsigned char* ring = base;
  unsigned char* bres = ring + (size_t)stages * kStage;  // resident B (RES only)
  GCtrl* ctrl = reinterpret_cast<GCtrl*>(bres + (RES ? (size_t)a.kchunks * kBBytes : 0));
  int16_t* cnt = reinterpret_cast<int16_t*>(ctrl + 1);  // [2][96][kCntPitch]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile int* abort_flag = &ctrl->abort_flag;

  if (threadIdx.x == 0) {
    for (int s = 0; s < stages; ++s) {
      mbar_init(&ctrl->full[s], 1);
      mbar_init(&ctrl->empty[s], 1);
    }
    for (int s = 0; s < 2; ++s) {
      mbar_init(&ctrl->tfull[s], 1);
      mbar_init(&ctrl->tempty[s], kEpiWarps / 2);  // the four warps of epilogue group s
    }
    mbar_init(&ctrl->drain, 1);
    mbar_init(&ctrl->bfull, 1);
    mbar_init(&ctrl->bempty, 1);
    ctrl->abort_flag = 0;
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
  // rows 96..127 of every A stage (the last 4 KB: whole 1 KB swizzle atoms)
  // stay zero: TMA writes only the 96 operand rows
  for (int s = 0; s < stages; ++s) {
    uint4* z = reinterpret_cast<uint4*>(ring + (size_t)s * kStage + kBlkRows * kKChunk);
    for (int k = threadIdx.x; k < (kABytes - kBlkRows * kKChunk) / 16; k += blockDim.x)
      z[k] = make_uint4(0u, 0u, 0u, 0u);
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = ctrl->tmem_base;

  long long n_items = a.item_off[a.n_blocks];
  if (n_items < 0 || n_items > a.n_blocks * (a.n_blocks + 1) / 2) {
    if (threadIdx.x == 0) set_abort(ctrl, a.status, 4001);
    n_items = 0;
  }

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int issued = 0, strips = 0;
      long long item = tile_item(0, chunk);
      long long lo = item < n_items ? advance_block(a.item_off, a.n_blocks, 0, item) : 0;
      long long lo_prev = -1;
      for (int t = 0; item < n_items && !*abort_flag; ++t) {
        const long long jb = lo + (item - a.item_off[lo]);
        const long long next = tile_item(t + 1, chunk);
        const long long lo_next =
            next < n_items ? advance_block(a.item_off, a.n_blocks, lo, next) : -1;
        const bool first = lo != lo_prev, last = lo_next != lo;
        bool ok = true;
        if (RES && first) {
          // a new strip: its row block replaces the resident B once the MMAs
          // of the previous strip are done with it
          if (strips > 0 && !mbar_wait_role(&ctrl->bempty, (uint32_t)((strips - 1) & 1),
                                            abort_flag)) {
            set_abort(ctrl, a.status, 4006);
            break;
          }
          mbar_expect_tx(&ctrl->bfull, (uint32_t)(a.kchunks * kBBytes));
          for (int kc = 0; kc < a.kchunks; ++kc)
            tma_load_2d(bres + (size_t)kc * kBBytes, &map, &ctrl->bfull, kc * kKChunk,
                        (int)(lo * kBlkRows));
          ++strips;
        }
        for (int kc = 0; kc < a.kchunks; ++kc) {
          if (!mbar_wait_role(&ctrl->empty[stage], phase ^ 1, abort_flag)) {
            set_abort(ctrl, a.status, 4002);
            ok = false;
            break;
          }
          if (kc == 0) ctrl->meta[stage] = (first ? 1 : 0) | (last ? 2 : 0);
          unsigned char* sa = ring + (size_t)stage * kStage;
          if (RES) {
            mbar_expect_tx(&ctrl->full[stage], kBBytes);
            tma_load_2d(sa, &map, &ctrl->full[stage], kc * kKChunk, (int)(jb * kBlkRows));
          } else {
            mbar_expect_tx(&ctrl->full[stage], 2 * kBBytes);
            tma_load_2d(sa, &map, &ctrl->full[stage], kc * kKChunk, (int)(lo * kBlkRows));
            tma_load_2d(sa + kABytes, &map, &ctrl->full[stage], kc * kKChunk,
                        (int)(jb * kBlkRows));
          }
          ++issued;
          if (++stage == stages) {
            stage = 0;
            phase ^= 1;
          }
        }
        if (!ok) break;
        lo_prev = lo;
        lo = lo_next;
        item = next;
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
        if (RES && strips > 0) mbar_wait_drain(&ctrl->bfull, (uint32_t)((strips - 1) & 1));
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int consumed = 0, strips = 0;
      bool any = false;
      for (int t = 0; !*abort_flag; ++t) {
        if (tile_item(t, chunk) >= n_items) break;
        const int acc = t & 1;
        const uint32_t aph = (uint32_t)((t >> 1) & 1);
        if (!mbar_wait_role(&ctrl->tempty[acc], aph ^ 1, abort_flag)) {
          set_abort(ctrl, a.status, 4003);
          break;
        }
        tc_fence_after();
        bool ok = true, last = false;
        const uint32_t d = tmem_base + (uint32_t)(acc * 128);
        for (int kc = 0; kc < a.kchunks; ++kc) {
          if (!mbar_wait_role(&ctrl->full[stage], phase, abort_flag)) {
            set_abort(ctrl, a.status, 4004);
            ok = false;
            break;
          }
          if (kc == 0) {
            const int m = ctrl->meta[stage];
            last = (m & 2) != 0;
            if (RES && (m & 1)) {
              if (!mbar_wait_role(&ctrl->bfull, (uint32_t)(strips & 1), abort_flag)) {
                set_abort(ctrl, a.status, 4007);
                ok = false;
                break;
              }
              ++strips;
            }
          }
          tc_fence_after();
          const uint32_t sa = smem_u32(ring + (size_t)stage * kStage);
          const uint64_t da = smem_desc(sa);
          const uint64_t db =
              smem_desc(RES ? smem_u32(bres + (size_t)kc * kBBytes) : sa + kABytes);
#pragma unroll
          for (int k = 0; k < kKChunk / 32; ++k)
            mma_f8_n96(d, da + (uint64_t)(k * 2), db + (uint64_t)(k * 2), (kc | k) != 0);
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
        if (RES && last) mma_commit(&ctrl->bempty);  // the strip's MMAs are all issued
      }
      if (*abort_flag && any) {
        mma_commit(&ctrl->drain);
        mbar_wait_drain(&ctrl->drain, 0);
      }
    }
  } else if (warp >= 4) {
    // ---------------- epilogue ----------------
    // Two groups of four warps take alternate tiles (group g: tiles g, g + 2,
    // ... of this CTA, accumulator stage g, moment buffer g), so one group's
    // copy and the other's statistics overlap.  Within a group the warp of
    // TMEM lane quarter q < 3 copies plane q's 96 moment columns, and all four
    // warps turn the 1,024 pairs into outputs (8 per thread).
    const int e = warp - 4;
    const int grp = e >> 2;
    const int wq = warp & 3;  // TMEM lanes 32q..32q+31: plane q of the SNPs i (j if RES)
    const uint32_t lane_base = (uint32_t)(wq * 32) << 16;
    const uint32_t bar_id = 1u + (uint32_t)grp;
    int16_t* buf = cnt + grp * 96 * kCntPitch;
    int t = grp;
    long long item = tile_item(t, chunk);

    // tile location: items ascend, so the row block lo only moves forward;
    // nv holds item_off[lo + 1 + lane], loaded one tile ahead
    long long lo = 0;
    long long nv = 1 + lane <= a.n_blocks ? a.item_off[1 + lane] : LLONG_MAX;
    long long i0 = 0, j0 = 0, off_lo = 0;
    int off_n = 0;
    auto locate = [&](long long it) {
      unsigned bal = __ballot_sync(0xffffffffu, nv <= it);
      lo += __popc(bal);
      if (bal == 0xffffffffu) {
        const long long idx = lo + 1 + lane;
        bal = __ballot_sync(0xffffffffu, idx <= a.n_blocks && a.item_off[idx] <= it);
        lo += __popc(bal);
        if (bal == 0xffffffffu) {
          long long l2 = lo, h2 = a.n_blocks;
          while (h2 - l2 > 1) {
            const long long mid = (l2 + h2) >> 1;
            if (a.item_off[mid] <= it) l2 = mid; else h2 = mid;
          }
          lo = l2;
        }
      }
      i0 = lo * kTileSnp;
      j0 = (lo + (it - a.item_off[lo])) * kTileSnp;
      // band offsets of the tile's 32 rows: lane l holds row i0 + l
      const long long ri = i0 + lane < a.n_snp ? i0 + lane : a.n_snp;
      off_lo = a.pair_off[ri];
      off_n = (int)((ri < a.n_snp ? a.pair_off[ri + 1] : off_lo) - off_lo);
    };
    if (item < n_items) locate(item);

    for (int u = 0; item < n_items; ++u) {
      bool ready = true;
      if (lane == 0) ready = mbar_wait(&ctrl->tfull[grp], (uint32_t)(u & 1), abort_flag);
      ready = __shfl_sync(0xffffffffu, ready ? 1 : 0, 0) != 0;
      if (!ready && lane == 0) set_abort(ctrl, a.status, 4005);
      // the group meets before overwriting its buffer (every warp is done
      // reading the previous tile) and takes one decision on aborting: the
      // barrier ORs every thread's view (its own wait failed, or the control
      // block's flag is set), so no warp is left waiting
      uint32_t any_abort = 0;
      const uint32_t mine = (ready ? 0u : 1u) | (uint32_t)(*abort_flag != 0);
      asm volatile(
          "{\n .reg .pred pin, pout;\n setp.ne.u32 pin, %1, 0;\n"
          " bar.red.or.pred pout, %2, 128, pin;\n selp.u32 %0, 1, 0, pout;\n}"
          : "=r"(any_abort)
          : "r"(mine), "r"(bar_id)
          : "memory");
      if (any_abort) break;
      tc_fence_after();
      if (wq < 3) {
        int16_t* row = buf + (wq * 32 + lane) * kCntPitch;
#pragma unroll 1
        for (int h = 0; h < 2; ++h) {
          uint32_t r[3][16];
#pragma unroll
          for (int c = 0; c < 3; ++c)
            tmem_ld16(tmem_base + lane_base + (uint32_t)(grp * 128 + 48 * h + 16 * c), r[c]);
          tmem_wait_ld();
#pragma unroll
          for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int v = 0; v < 16; ++v)
              row[48 * h + 16 * c + v] = (int16_t)fast::f2i_small(__uint_as_float(r[c][v]));
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&ctrl->tempty[grp]);
      asm volatile("bar.sync %0, 128;" ::"r"(bar_id) : "memory");

      const bool want_nv = a.nvalid != nullptr;
      // this tile's location; the next tile's offsets load during the pairs
      const long long ti0 = i0, tj0 = j0, toff = off_lo;
      const int tn = off_n;
      t += 2;
      const long long next = tile_item(t, chunk);
      if (next < n_items) nv = lo + 1 + lane <= a.n_blocks ? a.item_off[lo + 1 + lane] : LLONG_MAX;

      // eight pairs per thread; every value is computed and only the stores
      // depend on the pair lying in the band.  The outputs go out as
      // streaming global stores (st.global.cs): they are not re-read, and
      // being global-space they cannot alias the shared-memory moments, so
      // the loads of later pairs may move ahead of earlier pairs' stores.
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int il = wq + 4 * k, jl = lane;
        const long long row_off = __shfl_sync(0xffffffffu, toff, il);
        const int row_n = __shfl_sync(0xffffffffu, tn, il);
        const int d = (int)(tj0 - ti0) + jl - il - 1;  // j - i - 1
        // d < row_n keeps j inside the band and below n_snp
        const bool ok = d >= 0 && d < row_n;
        gmom::Mom mo;
#pragma unroll
        for (int x = 0; x < 3; ++x)
#pragma unroll
          for (int y = 0; y < 3; ++y)
            mo.m[3 * x + y] = RES ? buf[(y * 32 + jl) * kCntPitch + x * 32 + il]
                                  : buf[(x * 32 + il) * kCntPitch + y * 32 + jl];
        const long long kk = row_off + d;
        if (a.counts) {
          int c9[9];
          gmom::to_counts(mo, c9);
          if (ok) {
            int32_t* o = a.counts + kk * 9;
#pragma unroll
            for (int x = 0; x < 9; ++x) __stcs(o + x, c9[x]);
          }
        }
        st_cs_if(ok && want_nv, a.nvalid + kk, mo.m[0]);
        if (a.stats) {
          const float4 o = gmom::stats_f32<MASK>(mo, a.stat_mask);
          st_cs_if(ok, reinterpret_cast<float4*>(a.stats) + kk, o);
        }
      }
      item = next;
      if (item < n_items) locate(item);
    }
  }

  // ---------------- teardown ----------------
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(kTmemCols)
                 : "memory");
  }
}

// operand rows: row 96 * (s / 32) + 32 * plane + s % 32 holds, per
// individual, plane 0: 1 if the dosage at SNP s is known, plane 1: c = dosage
// - 1 (+1, 0, -1; 0 if missing), plane 2: c^2.  A block
// writes 8 rows, a warp one row in 16-byte chunks (16 individuals, one
// nibble-to-bytes step per 4).
__device__ __forceinline__ uint32_t e4m3_nibble(uint32_t mag, uint32_t neg) {
  // byte q = (bit q of mag ? 1.0 : 0) with the sign bit from neg
  uint32_t v = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q)
    v |= ((mag >> q & 1u) ? kOne : 0u) << (8 * q) | ((neg >> q & 1u) ? 0x80u : 0u) << (8 * q);
  return v;
}

__global__ void __launch_bounds__(256) pack_gtc_kernel(const uint32_t* __restrict__ planes, int W,
                                                       long long n_snp, long long n_blocks,
                                                       int k_pad, uint32_t* __restrict__ out) {
  const long long row = (long long)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n_blocks * kBlkRows) return;
  const int chunks = k_pad / 16;
  uint4* dst = reinterpret_cast<uint4*>(out) + row * chunks;
  const long long blk = row / kBlkRows;
  const int within = (int)(row - blk * kBlkRows);
  const int plane = within >> 5;
  const long long s = blk * kTileSnp + (within & 31);
  const uint32_t* ps = planes + (s < n_snp ? s : 0) * 3 * W;
  for (int c = lane; c < chunks; c += 32) {
    const int h0 = 16 * c;
    const int w = h0 >> 5;
    uint32_t mag = 0, neg = 0;
    if (s < n_snp && w < W) {
      const uint32_t g0 = __ldg(ps + w), g2 = __ldg(ps + 2 * W + w);
      const uint32_t word = plane == 0 ? (g0 | __ldg(ps + W + w) | g2) : (g0 | g2);
      mag = (word >> (h0 & 31)) & 0xFFFFu;
      if (plane == 1) neg = (g0 >> (h0 & 31)) & 0xFFFFu;
    }
    uint32_t v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = e4m3_nibble(mag >> (4 * q), neg >> (4 * q));
    dst[c] = make_uint4(v[0], v[1], v[2], v[3]);
  }
}

// ---------------------------------------------------------------------------
// Distance-binned sums of the genotype statistics of 1-4 populations.  The
// tile of 32 x 32 SNPs takes one M = 128, N = 96 MMA chain per population
// (the operand rows of population p start at row p * n_blocks * 96), each
// into its own 96 TMEM columns of the tile's accumulator stage.  One
// population: DD, Dz and pi2 in float32 straight from the moments
// (gmom::stats_f32).  Several: the epilogue turns each population's moments
// into 9-way counts and evaluates the term table of the statistics (the
// exact 64-bit integer forms of the popcount kernel, pgld_geno.cuh) per pair,
// which costs far more than the counting (the form is then as fast as the
// popcount one).  Sums per distance bin in float64 slots of the CTA.  G epilogue groups take alternate tiles: G = 2 for at most two
// populations (two accumulator stages of 256 columns), G = 1 for three or
// four (one stage of 384 columns).
// ---------------------------------------------------------------------------
struct BParams {
  int kchunks;
  long long n_snp;
  const long long* item_off;
  long long n_blocks;
  int n_pops;
  int pop_rows;             // operand rows per population (n_blocks * 96)
  const double* pos;
  const double* bcoord;     // distances for binning (NULL: positions)
  double max_dist;
  const double* bins;
  int n_bins;
  const pgld_term* terms;
  int n_terms, n_stats;
  double* sums;             // [n_bins][n_stats]
  unsigned long long* pair_counts;
  int32_t* status;
  int stages;
};

template <int G>
__global__ void __launch_bounds__(kThreads, 1)
    gtc_binned_kernel(const __grid_constant__ CUtensorMap map, BParams a) {
  constexpr int kGW = kEpiWarps / G;   // warps per epilogue group
  constexpr int kPMax = G == 2 ? 2 : 4;
  constexpr uint32_t kStageCols = G == 2 ? 256u : 0u;
  extern __shared__ unsigned char smem_dyn[];
  unsigned char* base = smem_dyn + ((1024 - (smem_u32(smem_dyn) & 1023)) & 1023);
  const int stages = a.stages;
  unsigned char* ring = base;
  GCtrl* ctrl = reinterpret_cast<GCtrl*>(ring + (size_t)stages * kGStageBytes);
  int16_t* cnt = reinterpret_cast<int16_t*>(ctrl + 1);  // [G][kPMax][96][kCntPitch]
  double* sbins = reinterpret_cast<double*>(cnt + (size_t)G * kPMax * 96 * kCntPitch);
  double* acc = sbins + (kMaxBins + 1);                 // [n_bins][n_stats]
  unsigned long long* bcnt =
      reinterpret_cast<unsigned long long*>(acc + (size_t)a.n_bins * a.n_stats);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile int* abort_flag = &ctrl->abort_flag;
  const int P = a.n_pops;

  if (threadIdx.x == 0) {
    for (int s = 0; s < stages; ++s) {
      mbar_init(&ctrl->full[s], 1);
      mbar_init(&ctrl->empty[s], 1);
    }
    for (int s = 0; s < G; ++s) {
      mbar_init(&ctrl->tfull[s], 1);
      mbar_init(&ctrl->tempty[s], kGW);
    }
    mbar_init(&ctrl->drain, 1);
    ctrl->abort_flag = 0;
    ctrl->consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&ctrl->tmem_base)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  for (int s = 0; s < stages; ++s) {
    uint4* z = reinterpret_cast<uint4*>(ring + (size_t)s * kGStageBytes + kBlkRows * kKChunk);
    for (int k = threadIdx.x; k < (kABytes - kBlkRows * kKChunk) / 16; k += blockDim.x)
      z[k] = make_uint4(0u, 0u, 0u, 0u);
  }
  for (int x = threadIdx.x; x < a.n_bins * a.n_stats; x += blockDim.x) acc[x] = 0.0;
  for (int x = threadIdx.x; x < a.n_bins; x += blockDim.x) bcnt[x] = 0ull;
  for (int x = threadIdx.x; x <= a.n_bins; x += blockDim.x) sbins[x] = a.bins[x];
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = ctrl->tmem_base;

  long long n_items = a.item_off[a.n_blocks];
  if (n_items < 0 || n_items > a.n_blocks * (a.n_blocks + 1) / 2) {
    if (threadIdx.x == 0) set_abort(ctrl, a.status, 4101);
    n_items = 0;
  }

  if (warp == 0) {
    // ---------------- TMA producer: per tile, every population's K chunks ----------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int issued = 0;
      long long lo = 0;
      bool ok = true;
      for (long long item = blockIdx.x; item < n_items && ok && !*abort_flag; item += gridDim.x) {
        lo = advance_block(a.item_off, a.n_blocks, lo, item);
        const long long jb = lo + (item - a.item_off[lo]);
        for (int p = 0; p < P && ok; ++p)
          for (int kc = 0; kc < a.kchunks; ++kc) {
            if (!mbar_wait_role(&ctrl->empty[stage], phase ^ 1, abort_flag)) {
              set_abort(ctrl, a.status, 4102);
              ok = false;
              break;
            }
            unsigned char* sa = ring + (size_t)stage * kGStageBytes;
            mbar_expect_tx(&ctrl->full[stage], 2 * kBBytes);
            tma_load_2d(sa, &map, &ctrl->full[stage], kc * kKChunk,
                        p * a.pop_rows + (int)(lo * kBlkRows));
            tma_load_2d(sa + kABytes, &map, &ctrl->full[stage], kc * kKChunk,
                        p * a.pop_rows + (int)(jb * kBlkRows));
            ++issued;
            if (++stage == stages) {
              stage = 0;
              phase ^= 1;
            }
          }
      }
      if (*abort_flag) {
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
      int consumed = 0;
      bool any = false, ok = true;
      for (int t = 0; ok && !*abort_flag; ++t) {
        if ((long long)blockIdx.x + (long long)t * gridDim.x >= n_items) break;
        const int sg = t % G;
        const uint32_t tph = (uint32_t)((t / G) & 1);
        if (!mbar_wait_role(&ctrl->tempty[sg], tph ^ 1, abort_flag)) {
          set_abort(ctrl, a.status, 4103);
          break;
        }
        tc_fence_after();
        for (int p = 0; p < P && ok; ++p) {
          const uint32_t d = tmem_base + (uint32_t)sg * kStageCols + (uint32_t)(p * 96);
          for (int kc = 0; kc < a.kchunks; ++kc) {
            if (!mbar_wait_role(&ctrl->full[stage], phase, abort_flag)) {
              set_abort(ctrl, a.status, 4104);
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sa = smem_u32(ring + (size_t)stage * kGStageBytes);
            const uint64_t da = smem_desc(sa), db = smem_desc(sa + kABytes);
#pragma unroll
            for (int k = 0; k < kKChunk / 32; ++k)
              mma_f8_n96(d, da + (uint64_t)(k * 2), db + (uint64_t)(k * 2), (kc | k) != 0);
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
        mma_commit(&ctrl->tfull[sg]);
      }
      if (*abort_flag && any) {
        mma_commit(&ctrl->drain);
        mbar_wait_drain(&ctrl->drain, 0);
      }
    }
  } else if (warp >= 4) {
    // ---------------- epilogue ----------------
    const int e = warp - 4;
    const int grp = e / kGW;
    const int gi = e % kGW;                // warp within the group
    const int wq = warp & 3;               // TMEM lane quarter: plane wq of the SNPs i
    const uint32_t lane_base = (uint32_t)(wq * 32) << 16;
    const uint32_t bar_id = 1u + (uint32_t)grp;
    int16_t* gbuf = cnt + (size_t)grp * kPMax * 96 * kCntPitch;
    long long lo = 0;
    for (int t = grp, u = 0;; t += G, ++u) {
      const long long item = (long long)blockIdx.x + (long long)t * gridDim.x;
      if (item >= n_items) break;
      bool ready = true;
      if (lane == 0) ready = mbar_wait(&ctrl->tfull[grp], (uint32_t)(u & 1), abort_flag);
      ready = __shfl_sync(0xffffffffu, ready ? 1 : 0, 0) != 0;
      if (!ready && lane == 0) set_abort(ctrl, a.status, 4105);
      // the group meets before overwriting its moment buffers and takes one
      // decision on aborting (bar.red.or over every thread's view)
      uint32_t any_abort = 0;
      const uint32_t mine = (ready ? 0u : 1u) | (uint32_t)(*abort_flag != 0);
      asm volatile(
          "{\n .reg .pred pin, pout;\n setp.ne.u32 pin, %1, 0;\n"
          " bar.red.or.pred pout, %2, %3, pin;\n selp.u32 %0, 1, 0, pout;\n}"
          : "=r"(any_abort)
          : "r"(mine), "r"(bar_id), "r"(kGW * 32)
          : "memory");
      if (any_abort) break;
      tc_fence_after();
      // copy: the warps of lane quarters 0-2 copy plane wq's moments of the
      // populations they own (with two warps per quarter, alternate ones)
      if (wq < 3) {
        const int half = gi >> 2;   // 0 with four warps per group
        for (int p = half; p < P; p += kGW / 4) {
          int16_t* row = gbuf + ((size_t)p * 96 + wq * 32 + lane) * kCntPitch;
#pragma unroll 1
          for (int h = 0; h < 2; ++h) {
            uint32_t r[3][16];
#pragma unroll
            for (int c = 0; c < 3; ++c)
              tmem_ld16(tmem_base + lane_base +
                            ((uint32_t)grp * kStageCols + (uint32_t)(p * 96 + 48 * h + 16 * c)),
                        r[c]);
            tmem_wait_ld();
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
              for (int v = 0; v < 16; ++v)
                row[48 * h + 16 * c + v] = (int16_t)fast::f2i_small(__uint_as_float(r[c][v]));
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&ctrl->tempty[grp]);
      asm volatile("bar.sync %0, %1;" ::"r"(bar_id), "r"(kGW * 32) : "memory");

      lo = advance_block(a.item_off, a.n_blocks, lo, item);
      const long long i0 = lo * kTileSnp, j0 = (lo + (item - a.item_off[lo])) * kTileSnp;
      const long long j = j0 + lane;
      const bool j_ok = j < a.n_snp;
      const double pj = j_ok ? a.pos[j] : 0.0;
      const double cj = (j_ok && a.bcoord) ? a.bcoord[j] : 0.0;
#pragma unroll 1
      for (int k = 0; k < 32 / kGW; ++k) {
        const int il = gi + kGW * k;
        const long long i = i0 + il;
        bool ok = i < j && j_ok;
        double dpos = 0.0;
        if (ok) {
          dpos = pj - a.pos[i];
          ok = dpos <= a.max_dist;
        }
        int b = -1;
        if (ok) {
          const double d = a.bcoord ? fabs(cj - a.bcoord[i]) : dpos;
          b = bin_of_f64(sbins, a.n_bins, d);
        }
        unsigned pending = __ballot_sync(0xffffffffu, b >= 0);
        if (!pending) continue;
        if (P == 1) {
          // one population: DD, Dz, pi2 in float32 from the moments
          // (gmom::stats_f32, within 1e-6 relative of each exact value)
          gmom::Mom mo;
#pragma unroll
          for (int x = 0; x < 3; ++x)
#pragma unroll
            for (int y = 0; y < 3; ++y)
              mo.m[3 * x + y] = gbuf[(x * 32 + il) * kCntPitch + y * 32 + lane];
          const float4 o4 = gmom::stats_f32<14>(mo, 14);
          while (pending) {
            const int bb = __shfl_sync(0xffffffffu, b, __ffs(pending) - 1);
            const bool mine = (b == bb);
            const unsigned grpm = __ballot_sync(0xffffffffu, mine);
            float v[3] = {mine ? o4.y : 0.f, mine ? o4.z : 0.f, mine ? o4.w : 0.f};
#pragma unroll
            for (int q = 0; q < 3; ++q) {
#pragma unroll
              for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
            }
            if (lane == 0) {
#pragma unroll
              for (int q = 0; q < 3; ++q) atomicAdd(&acc[bb * 3 + q], (double)v[q]);
              atomicAdd(&bcnt[bb], (unsigned long long)__popc(grpm));
            }
            pending &= ~grpm;
          }
          continue;
        }
        int cc[kPMax][9];
        geno::GPop gp[kPMax];
        const int* cp[kPMax];
#pragma unroll
        for (int p = 0; p < kPMax; ++p) {
          if (p < P) {
            gmom::Mom mo;
            const int16_t* bp = gbuf + (size_t)p * 96 * kCntPitch;
#pragma unroll
            for (int x = 0; x < 3; ++x)
#pragma unroll
              for (int y = 0; y < 3; ++y) mo.m[3 * x + y] = bp[(x * 32 + il) * kCntPitch + y * 32 + lane];
            gmom::to_counts(mo, cc[p]);
            gp[p] = geno::make_gpop(cc[p], -1);
          }
          cp[p] = cc[p];
        }
        while (pending) {
          const int bb = __shfl_sync(0xffffffffu, b, __ffs(pending) - 1);
          const bool mine = (b == bb);
          const unsigned grpm = __ballot_sync(0xffffffffu, mine);
          int tt = 0;
          for (int s = 0; s < a.n_stats; ++s) {
            float v = 0.f;
            for (; tt < a.n_terms && a.terms[tt].stat == s; ++tt) {
              const pgld_term tm = a.terms[tt];
              if (mine) v += (float)tm.weight * geno::term_value<float>(tm, gp, cp);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) atomicAdd(&acc[bb * a.n_stats + s], (double)v);
          }
          if (lane == 0) atomicAdd(&bcnt[bb], (unsigned long long)__popc(grpm));
          pending &= ~grpm;
        }
      }
    }
  }

  // ---------------- teardown ----------------
  tc_fence_before();
  __syncthreads();
  if (!*abort_flag) {
    for (int x = threadIdx.x; x < a.n_bins * a.n_stats; x += blockDim.x)
      if (acc[x] != 0.0) atomicAdd(a.sums + x, acc[x]);
    if (a.pair_counts)
      for (int x = threadIdx.x; x < a.n_bins; x += blockDim.x)
        if (bcnt[x]) atomicAdd(a.pair_counts + x, bcnt[x]);
  }
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(512)
                 : "memory");
  }
}

}  // namespace gtc
}  // namespace pgld

// Genotype band pairs on the tensor cores: one population, dosages 0/1/2
// (missing allowed), no values above 2.  a carries the band and outputs.
int pgld_geno_tc_pairs(pgld_context* h, const pgld_geno_panel* panel, const double* pos,
                       double max_dist, int32_t* counts, int32_t* n_valid, float* stats,
                       int32_t stat_mask, cudaStream_t st) {
  using namespace pgld::gtc;
  int rc = pgld::tchost::get_encode(h);
  if (rc) return rc;
  const long long n = panel->n_snp;
  const int W = panel->n_words[0];
  const long long nb = (n + kTileSnp - 1) / kTileSnp;
  if (nb * kBlkRows > 2147483647LL)
    return pgld_fail(h, PGLD_ERR_TOO_LARGE, "genotype tensor-core form: too many SNPs");
  const int k_pad = ((W * 32 + kKChunk - 1) / kKChunk) * kKChunk;
  const size_t op_bytes = (size_t)nb * kBlkRows * k_pad;
  const size_t sb = pgld::scan_scratch_bytes(std::max<long long>(nb, n));
  auto al = [](size_t x) { return (x + 1023) & ~size_t(1023); };
  const size_t off_items = 0, off_scan = al((nb + 1) * 8), off_op = off_scan + al(sb),
               off_poff = off_op + al(op_bytes), total = off_poff + al((size_t)(n + 1) * 8);
  void* ws = nullptr;
  rc = pgld_workspace(h, total, &ws);
  if (rc) return rc;
  char* w = (char*)ws;
  long long* items = (long long*)(w + off_items);
  long long* poff = (long long*)(w + off_poff);
  unsigned char* op = (unsigned char*)(w + off_op);
  rc = pgld_band_offsets(h, pos, n, max_dist, poff, w + off_scan, sb, st);
  if (rc) return rc;
  {
    const unsigned blocks = (unsigned)std::max<long long>(1, (nb * kBlkRows + 7) / 8);
    pack_gtc_kernel<<<blocks, 256, 0, st>>>(panel->planes[0], W, n, nb, k_pad, (uint32_t*)op);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "pack_gtc_kernel");
  }
  rc = pgld::band_schedule(h, pos, n, max_dist, items, w + off_scan, sb, st, kTileSnp);
  if (rc) return rc;
  CUtensorMap map;
  rc = pgld::tchost::make_map(h, &map, op, nb * kBlkRows, k_pad, kBlkRows);
  if (rc) return rc;
  Params prm{};
  prm.kchunks = k_pad / kKChunk;
  prm.n_snp = n;
  prm.item_off = items;
  prm.n_blocks = nb;
  prm.pair_off = poff;
  prm.counts = counts;
  prm.nvalid = n_valid;
  prm.stats = stats;
  prm.stat_mask = stat_mask;
  prm.status = h->dev_status;
  const size_t fixed = sizeof(GCtrl) + (size_t)2 * 96 * kCntPitch * 2 + 1024;
  int max_smem = 0;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  // the resident form when the row block (every K chunk) fits beside at
  // least four 16 KB A stages: up to 1,280 individuals
  const long long res_bytes = (long long)prm.kchunks * kBBytes;
  const long long res_stages =
      std::min<long long>(8, ((long long)max_smem - (long long)fixed - res_bytes) / kABytes);
  const bool res = res_stages >= 4;
  const int stages = res ? (int)res_stages
                         : (int)std::min<long long>(
                               8, ((long long)max_smem - (long long)fixed) / kGStageBytes);
  if (stages < 2) return pgld_fail(h, PGLD_ERR_TOO_LARGE, "genotype tensor-core form: shared memory");
  prm.stages = stages;
  const size_t smem =
      res ? (size_t)stages * kABytes + (size_t)res_bytes + fixed : (size_t)stages * kGStageBytes + fixed;
  // the two column sets of the band workloads get their own instantiation
  void (*kern)(CUtensorMap, Params);
  if (res)
    kern = !stats ? gtc_pairs_kernel<0, true>
           : stat_mask == 3 ? gtc_pairs_kernel<3, true>
           : stat_mask == 15 ? gtc_pairs_kernel<15, true>
                             : gtc_pairs_kernel<-1, true>;
  else
    kern = !stats ? gtc_pairs_kernel<0, false>
           : stat_mask == 3 ? gtc_pairs_kernel<3, false>
           : stat_mask == 15 ? gtc_pairs_kernel<15, false>
                             : gtc_pairs_kernel<-1, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "gtc smem attribute");
  pgld_time_begin(h, st);
  kern<<<(unsigned)h->n_sm, kThreads, smem, st>>>(map, prm);
  pgld_time_end(h, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "gtc_pairs_kernel");
  return PGLD_OK;
}

// Genotype distance-binned sums on the tensor cores: 1-4 populations of
// dosages 0/1/2 (missing allowed, no values above 2), at most kMaxGenoN
// individuals each; ba carries the bins, term table and outputs (sums and
// pair counts already zeroed).
int pgld_geno_tc_binned(pgld_context* h, const pgld_geno_panel* panel, const pgld::BandArgs& ba,
                        cudaStream_t st) {
  using namespace pgld::gtc;
  int rc = pgld::tchost::get_encode(h);
  if (rc) return rc;
  const int P = panel->n_pops;
  const long long n = panel->n_snp;
  const long long nb = (n + kTileSnp - 1) / kTileSnp;
  int W = 0;
  for (int p = 0; p < P; ++p) W = std::max(W, panel->n_words[p]);
  if ((long long)P * nb * kBlkRows > 2147483647LL)
    return pgld_fail(h, PGLD_ERR_TOO_LARGE, "genotype tensor-core binned form: too many SNPs");
  const int k_pad = ((W * 32 + kKChunk - 1) / kKChunk) * kKChunk;
  const size_t op_pop = (size_t)nb * kBlkRows * k_pad;
  const size_t sb = pgld::scan_scratch_bytes(nb);
  auto al = [](size_t x) { return (x + 1023) & ~size_t(1023); };
  const size_t off_items = 0, off_scan = al((nb + 1) * 8), off_op = off_scan + al(sb),
               total = off_op + al(op_pop * P);
  void* ws = nullptr;
  rc = pgld_workspace(h, total, &ws);
  if (rc) return rc;
  char* w = (char*)ws;
  long long* items = (long long*)(w + off_items);
  unsigned char* op = (unsigned char*)(w + off_op);
  for (int p = 0; p < P; ++p) {
    const unsigned blocks = (unsigned)std::max<long long>(1, (nb * kBlkRows + 7) / 8);
    pack_gtc_kernel<<<blocks, 256, 0, st>>>(panel->planes[p], panel->n_words[p], n, nb, k_pad,
                                            (uint32_t*)(op + op_pop * p));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "pack_gtc_kernel");
  }
  rc = pgld::band_schedule(h, ba.pos, n, ba.max_dist, items, w + off_scan, sb, st, kTileSnp);
  if (rc) return rc;
  CUtensorMap map;
  rc = pgld::tchost::make_map(h, &map, op, (long long)P * nb * kBlkRows, k_pad, kBlkRows);
  if (rc) return rc;
  BParams prm{};
  prm.kchunks = k_pad / kKChunk;
  prm.n_snp = n;
  prm.item_off = items;
  prm.n_blocks = nb;
  prm.n_pops = P;
  prm.pop_rows = (int)(nb * kBlkRows);
  prm.pos = ba.pos;
  prm.bcoord = ba.bcoord;
  prm.max_dist = ba.max_dist;
  prm.bins = ba.bins;
  prm.n_bins = ba.n_bins;
  prm.terms = ba.terms;
  prm.n_terms = ba.n_terms;
  prm.n_stats = ba.n_stats;
  prm.sums = ba.sums;
  prm.pair_counts = reinterpret_cast<unsigned long long*>(ba.pair_counts);
  prm.status = h->dev_status;
  const int G = P <= 2 ? 2 : 1;
  const int pmax = G == 2 ? 2 : 4;
  const size_t fixed = sizeof(GCtrl) + (size_t)G * pmax * 96 * kCntPitch * 2 +
                       (size_t)(pgld::kMaxBins + 1) * 8 + (size_t)ba.n_bins * ba.n_stats * 8 +
                       (size_t)ba.n_bins * 8 + 1024;
  int max_smem = 0;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  const int stages =
      (int)std::min<long long>(8, ((long long)max_smem - (long long)fixed) / kGStageBytes);
  if (stages < 2)
    return pgld_fail(h, PGLD_ERR_TOO_LARGE, "genotype tensor-core binned form: shared memory");
  prm.stages = stages;
  const size_t smem = (size_t)stages * kGStageBytes + fixed;
  void (*kern)(CUtensorMap, BParams) = G == 2 ? gtc_binned_kernel<2> : gtc_binned_kernel<1>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "gtc binned smem attribute");
  pgld_time_begin(h, st);
  kern<<<(unsigned)h->n_sm, kThreads, smem, st>>>(map, prm);
  pgld_time_end(h, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "gtc_binned_kernel");
  return PGLD_OK;
}
