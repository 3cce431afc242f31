// tcgen05 tensor-core form of the genotype distance-band pairs (sm_103a).
//
// The 9-way counts of a SNP pair are dot products of 0/1 indicator vectors
// over the individuals: with A = the planes (g == 0, g == 1, g == 2, g >= 0)
// of 32 SNPs i and B the same for 32 SNPs j, D = A B^T holds n_ab for every
// a, b of all 1,024 pairs of the tile.  The operand rows are plane-major
// within a 32-SNP block (row = 128 * block + 32 * plane + SNP), so D[32 a +
// i][32 b + j] = n_ab(i, j).  Operands are E4M3 bytes (0x38 = 1.0) in
// K-major rows padded to 128 bytes; the float32 accumulators hold integers
// below 2^24, so the counts are exact.
//
// One CTA per SM:
//   warp 0      TMA producer (128-row x 128-byte boxes, SWIZZLE_128B)
//   warp 1      allocates 256 TMEM columns; one lane issues M=128 N=128 K=32
//               kind::f8f6f4 MMAs into accumulator stage t % 2
//   warps 4-11  epilogue: the warps of TMEM lane quarters 0-2 (planes 0-2)
//               copy the 3 x 3 count blocks to shared memory, then all eight
//               warps turn 1,024 pairs into outputs (4 per thread)
// Every mbarrier wait is bounded; the epilogue warps meet at one named
// barrier per tile and agree on aborting after it.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "pgld_band.cuh"
#include "pgld_epilogue.cuh"
#include "pgld_geno.cuh"
#include "pgld_internal.cuh"
#include "pgld_scan.cuh"
#include "pgld_tcgen05.cuh"

namespace pgld {
namespace gtc {

using namespace pgld::tc;

constexpr int kTileSnp = 32;          // SNPs per tile side (4 planes = 128 rows)
constexpr int kEpiWarps = 8;
constexpr int kEpiThreads = kEpiWarps * 32;
constexpr int kThreads = (4 + kEpiWarps) * 32;
constexpr uint32_t kTmemCols = 256;   // two accumulator stages of 128 columns
constexpr int kCntPitch = 97;         // int pitch of the 96 x 96 count block

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

template <int DUMMY>
__global__ void __launch_bounds__(kThreads, 1)
    gtc_pairs_kernel(const __grid_constant__ CUtensorMap map, Params a) {
  extern __shared__ unsigned char smem_dyn[];
  unsigned char* base = smem_dyn + ((1024 - (smem_u32(smem_dyn) & 1023)) & 1023);
  const int stages = a.stages;
  unsigned char* ring = base;
  Ctrl* ctrl = reinterpret_cast<Ctrl*>(ring + (size_t)stages * kStageBytes);
  int* cnt = reinterpret_cast<int*>(ctrl + 1);  // [2][96][kCntPitch]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
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
      int issued = 0;
      for (long long item = blockIdx.x; item < n_items && !*abort_flag; item += gridDim.x) {
        long long lo = 0, hi = a.n_blocks;
        while (hi - lo > 1) {
          const long long mid = (lo + hi) >> 1;
          if (a.item_off[mid] <= item) lo = mid; else hi = mid;
        }
        const int yi = (int)(lo * kRows), yj = (int)((lo + (item - a.item_off[lo])) * kRows);
        for (int kc = 0; kc < a.kchunks; ++kc) {
          if (!mbar_wait(&ctrl->empty[stage], phase ^ 1, abort_flag)) {
            set_abort(ctrl, a.status, 4002);
            break;
          }
          mbar_expect_tx(&ctrl->full[stage], kStageBytes);
          unsigned char* sa = ring + (size_t)stage * kStageBytes;
          tma_load_2d(sa, &map, &ctrl->full[stage], kc * kKChunk, yi);
          tma_load_2d(sa + kBoxBytes, &map, &ctrl->full[stage], kc * kKChunk, yj);
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
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int t = 0, consumed = 0;
      bool any = false;
      for (long long item = blockIdx.x; item < n_items && !*abort_flag; item += gridDim.x, ++t) {
        const int acc = t & 1;
        const uint32_t aph = (uint32_t)((t >> 1) & 1);
        if (!mbar_wait(&ctrl->tempty[acc], aph ^ 1, abort_flag)) {
          set_abort(ctrl, a.status, 4003);
          break;
        }
        tc_fence_after();
        bool ok = true;
        const uint32_t d = tmem_base + (uint32_t)(acc * 128);
        for (int kc = 0; kc < a.kchunks; ++kc) {
          if (!mbar_wait(&ctrl->full[stage], phase, abort_flag)) {
            set_abort(ctrl, a.status, 4004);
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
        if (!ok) break;
        mma_commit(&ctrl->tfull[acc]);
      }
      if (*abort_flag && any) {
        mma_commit(&ctrl->drain);
        mbar_wait_drain(&ctrl->drain, 0);
      }
    }
  } else if (warp >= 4) {
    // ---------------- epilogue ----------------
    const int e = warp - 4;
    const int quarter = warp & 3;  // TMEM lanes 32q..32q+31 = plane q of the 32 SNPs i
    const int half = e >> 2;       // columns 64h..64h+63 = planes 2h, 2h+1 of the SNPs j
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    const int t_epi = threadIdx.x - 128;
    int t = 0;
    for (long long item = blockIdx.x; item < n_items; item += gridDim.x, ++t) {
      const int acc = t & 1;
      const uint32_t aph = (uint32_t)((t >> 1) & 1);
      int* buf = cnt + acc * 96 * kCntPitch;
      bool ready = true;
      if (lane == 0) ready = mbar_wait(&ctrl->tfull[acc], aph, abort_flag);
      ready = __shfl_sync(0xffffffffu, ready ? 1 : 0, 0) != 0;
      if (!ready && lane == 0) set_abort(ctrl, a.status, 4005);
      const uint32_t local_abort = ready ? 0u : 1u;
      if (ready) {
        tc_fence_after();
        if (quarter < 3) {
#pragma unroll 1
          for (int c = 0; c < 4; ++c) {
            const int col0 = half * 64 + c * 16;
            if (col0 >= 96) break;  // plane 3 of the SNPs j is not needed
            uint32_t r[16];
            tmem_ld16(tmem_base + lane_base + (uint32_t)(acc * 128 + col0), r);
            tmem_wait_ld();
            int* row = buf + (quarter * 32 + lane) * kCntPitch + col0;
#pragma unroll
            for (int v = 0; v < 16; ++v) row[v] = fast::f2i_small(__uint_as_float(r[v]));
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&ctrl->tempty[acc]);
      }
      // all epilogue warps meet once per tile and take one decision on
      // aborting: the barrier ORs every thread's view (its own wait failed,
      // or the control block's flag is set), so no warp is left waiting
      uint32_t any_abort = 0;
      const uint32_t mine = local_abort | (uint32_t)(*abort_flag != 0);
      asm volatile(
          "{\n .reg .pred pin, pout;\n setp.ne.u32 pin, %1, 0;\n"
          " bar.red.or.pred pout, 1, %2, pin;\n selp.u32 %0, 1, 0, pout;\n}"
          : "=r"(any_abort)
          : "r"(mine), "r"(kEpiThreads)
          : "memory");
      if (any_abort) break;

      long long lo = 0, hi = a.n_blocks;
      while (hi - lo > 1) {
        const long long mid = (lo + hi) >> 1;
        if (a.item_off[mid] <= item) lo = mid; else hi = mid;
      }
      const long long i0 = lo * kTileSnp, j0 = (lo + (item - a.item_off[lo])) * kTileSnp;
#pragma unroll 1
      for (int k = 0; k < 4; ++k) {
        const int il = (t_epi >> 5) + 8 * k, jl = lane;
        const long long i = i0 + il, j = j0 + jl;
        bool ok = (i < j) && (j < a.n_snp);
        if (ok) ok = (j - i - 1) < (a.pair_off[i + 1] - a.pair_off[i]);
        if (!ok) continue;
        int c9[9];
#pragma unroll
        for (int x = 0; x < 3; ++x)
#pragma unroll
          for (int y = 0; y < 3; ++y) c9[3 * x + y] = buf[(x * 32 + il) * kCntPitch + y * 32 + jl];
        const long long kk = a.pair_off[i] + (j - i - 1);
        const geno::GPop P = geno::make_gpop(c9, -1);
        if (a.counts) {
          int32_t* o = a.counts + kk * 9;
#pragma unroll
          for (int x = 0; x < 9; ++x) o[x] = c9[x];
        }
        if (a.nvalid) a.nvalid[kk] = (int32_t)P.ns;
        if (a.stats) {
          float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
          if (a.stat_mask & 1) o.x = geno::rh2_f32(c9);
          if (a.stat_mask & 2) o.y = geno::gv_f32(geno::dd_single(P));
          if (a.stat_mask & 4) o.z = geno::gv_f32(geno::dz_single(P));
          if (a.stat_mask & 8) o.w = geno::gv_f32(geno::pi2_single(P));
          reinterpret_cast<float4*>(a.stats)[kk] = o;
        }
      }
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

// operand rows: row 128 * (s / 32) + 32 * plane + s % 32 holds, for plane 0..2,
// the individuals with dosage == plane at SNP s, and for plane 3 the valid
// ones.  A block writes 8 rows, a warp one row in 16-byte chunks (16
// individuals, one nibble-to-bytes step per 4).
__global__ void __launch_bounds__(256) pack_gtc_kernel(const uint32_t* __restrict__ planes, int W,
                                                       long long n_snp, long long n_blocks,
                                                       int k_pad, uint32_t* __restrict__ out) {
  const long long row = (long long)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n_blocks * kRows) return;
  const int chunks = k_pad / 16;
  uint4* dst = reinterpret_cast<uint4*>(out) + row * chunks;
  const long long blk = row >> 7;
  const int within = (int)(row & 127);
  const int plane = within >> 5;
  const long long s = blk * kTileSnp + (within & 31);
  const uint32_t* ps = planes + (s < n_snp ? s : 0) * 3 * W;
  for (int c = lane; c < chunks; c += 32) {
    const int h0 = 16 * c;
    const int w = h0 >> 5;
    uint32_t bits = 0;
    if (s < n_snp && w < W) {
      const uint32_t word = plane < 3 ? __ldg(ps + plane * W + w)
                                      : (__ldg(ps + w) | __ldg(ps + W + w) | __ldg(ps + 2 * W + w));
      bits = (word >> (h0 & 31)) & 0xFFFFu;
    }
    uint32_t v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t nib = (bits >> (4 * q)) & 0xFu;
      v[q] = (nib & 1u ? kOne : 0u) | (nib & 2u ? kOne << 8 : 0u) | (nib & 4u ? kOne << 16 : 0u) |
             (nib & 8u ? kOne << 24 : 0u);
    }
    dst[c] = make_uint4(v[0], v[1], v[2], v[3]);
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
  if (nb * kRows > 2147483647LL)
    return pgld_fail(h, PGLD_ERR_TOO_LARGE, "genotype tensor-core form: too many SNPs");
  const int k_pad = ((W * 32 + kKChunk - 1) / kKChunk) * kKChunk;
  const size_t op_bytes = (size_t)nb * kRows * k_pad;
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
    const unsigned blocks = (unsigned)std::max<long long>(1, (nb * kRows + 7) / 8);
    pack_gtc_kernel<<<blocks, 256, 0, st>>>(panel->planes[0], W, n, nb, k_pad, (uint32_t*)op);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return pgld_cuda_fail(h, e, "pack_gtc_kernel");
  }
  rc = pgld::band_schedule(h, pos, n, max_dist, items, w + off_scan, sb, st, kTileSnp);
  if (rc) return rc;
  CUtensorMap map;
  rc = pgld::tchost::make_map(h, &map, op, nb * kRows, k_pad);
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
  const size_t fixed = sizeof(pgld::tc::Ctrl) + (size_t)2 * 96 * kCntPitch * 4 + 1024;
  int max_smem = 0;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  const int stages =
      (int)std::min<long long>(8, ((long long)max_smem - (long long)fixed) / kStageBytes);
  if (stages < 2) return pgld_fail(h, PGLD_ERR_TOO_LARGE, "genotype tensor-core form: shared memory");
  prm.stages = stages;
  const size_t smem = (size_t)stages * kStageBytes + fixed;
  auto kern = gtc_pairs_kernel<0>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "gtc smem attribute");
  kern<<<(unsigned)h->n_sm, kThreads, smem, st>>>(map, prm);
  e = cudaGetLastError();
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "gtc_pairs_kernel");
  return PGLD_OK;
}
