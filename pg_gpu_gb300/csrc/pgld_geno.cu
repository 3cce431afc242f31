// Genotype (unphased diploid dosage) path: dosage bit planes, 9-way pair
// counts, the moments genotype statistics, and the distance-band kernels.
//
// A population's dosages at one SNP are three bit planes (g == 0, 1, 2) of
// W = ceil(N / 32) words.  The 9-way count n_ab of a pair (i, j) is
// popc(plane_a(i) & plane_b(j)) summed over the words, so a pair costs
// 9 AND + POPC per word instead of the reference's one-thread-per-pair loop
// over individuals with uncoalesced byte loads (ld_pipeline.py:183-217).
#include <cuda_runtime.h>

#include <algorithm>

#include "pgld_band.cuh"
#include "pgld_geno.cuh"
#include "pgld_internal.cuh"
#include "pgld_scan.cuh"

using pgld::i64;

namespace pgld {
namespace geno {

// ---------------------------------------------------------------------------
// packing: grid (ceil(n_snp/256), W), thread = one SNP x one 32-individual word
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) pack_geno_kernel(const int8_t* __restrict__ geno, i64 ld,
                                                        i64 n_snp, const int32_t* __restrict__ rows,
                                                        int n_rows, int W,
                                                        uint32_t* __restrict__ planes,
                                                        uint32_t* __restrict__ valid,
                                                        uint32_t* __restrict__ ext,
                                                        int32_t* __restrict__ flags) {
  const i64 s = (i64)blockIdx.x * 256 + threadIdx.x;
  const int w = blockIdx.y;
  uint32_t p0 = 0, p1 = 0, p2 = 0, vw = 0;
  uint32_t x[6] = {0, 0, 0, 0, 0, 0};
  bool miss = false, other = false;
  if (s < n_snp) {
    for (int r = 0; r < 32; ++r) {
      const int row = w * 32 + r;
      if (row >= n_rows) break;
      const i64 gr = rows ? (i64)__ldg(rows + row) : (i64)row;
      const int v = __ldg(geno + gr * ld + s);
      p0 |= (uint32_t)(v == 0) << r;
      p1 |= (uint32_t)(v == 1) << r;
      p2 |= (uint32_t)(v == 2) << r;
      vw |= (uint32_t)(v >= 0) << r;
#pragma unroll
      for (int e = 0; e < 6; ++e) x[e] |= (uint32_t)(v == 3 + e) << r;
      miss |= v < 0;
      other |= v > 2;
    }
    uint32_t* o = planes + s * 3 * W;
    o[w] = p0;
    o[W + w] = p1;
    o[2 * W + w] = p2;
    if (valid) valid[s * W + w] = vw;
    if (ext)
#pragma unroll
      for (int e = 0; e < 6; ++e) ext[s * 6 * W + e * W + w] = x[e];
  }
  const unsigned any_miss = __ballot_sync(0xffffffffu, miss);
  const unsigned any_other = __ballot_sync(0xffffffffu, other);
  if ((threadIdx.x & 31) == 0) {
    if (any_miss) atomicOr(flags, 1);
    if (any_other) atomicOr(flags + 1, 1);
  }
}

// ---------------------------------------------------------------------------
// counts of listed pairs: a group of G lanes per pair, words strided by G
// ---------------------------------------------------------------------------
template <int G>
__global__ void __launch_bounds__(256) geno_counts_pairs_kernel(
    const uint32_t* __restrict__ planes, const uint32_t* __restrict__ valid,
    const uint32_t* __restrict__ ext, int W, i64 n_snp, const int32_t* __restrict__ idx_i,
    const int32_t* __restrict__ idx_j, i64 n_pairs, int32_t* __restrict__ counts, i64 counts_ld,
    int32_t* __restrict__ n_valid, int32_t* __restrict__ status) {
  const i64 g = ((i64)blockIdx.x * 256 + threadIdx.x) / G;
  const int lane = threadIdx.x % G;
  const i64 ngroups = (i64)gridDim.x * 256 / G;
  const i64 span = n_pairs + (ngroups - (n_pairs % ngroups)) % ngroups;
  for (i64 k = g; k < span; k += ngroups) {
    bool live = k < n_pairs;
    i64 i = 0, j = 0;
    if (live) {
      i = idx_i[k];
      j = idx_j[k];
      if (i < 0 || j < 0 || i >= n_snp || j >= n_snp) {
        if (lane == 0) atomicCAS(status, 0, 1101);
        live = false;
      }
    }
    int c[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) c[q] = 0;
    int nv = 0;
    if (live) {
      const uint32_t* pi = planes + i * 3 * W;
      const uint32_t* pj = planes + j * 3 * W;
      for (int w = lane; w < W; w += G) {
        uint32_t a[3], b[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          a[q] = __ldg(pi + q * W + w);
          b[q] = __ldg(pj + q * W + w);
        }
#pragma unroll
        for (int x = 0; x < 3; ++x)
#pragma unroll
          for (int y = 0; y < 3; ++y) c[3 * x + y] += __popc(a[x] & b[y]);
        if (ext) {
          // class 3 g_i + g_j of the values 3..8 at the second SNP
          const uint32_t* ej = ext + j * 6 * W + w;
#pragma unroll
          for (int e = 0; e < 6; ++e) {
            const uint32_t xe = __ldg(ej + e * W);
            c[3 + e] += __popc(a[0] & xe);
            if (e < 3) c[6 + e] += __popc(a[1] & xe);
          }
        }
        if (valid) nv += __popc(__ldg(valid + i * W + w) & __ldg(valid + j * W + w));
      }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
#pragma unroll
      for (int q = 0; q < 9; ++q) c[q] += __shfl_xor_sync(0xffffffffu, c[q], o, G);
      nv += __shfl_xor_sync(0xffffffffu, nv, o, G);
    }
    if (live && lane == 0) {
      int32_t* out = counts + k * counts_ld;
      int tot = 0;
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        out[q] = c[q];
        tot += c[q];
      }
      if (n_valid) n_valid[k] = valid ? nv : tot;
    }
  }
}

struct GStatsArgs {
  const int32_t* counts[PGLD_MAX_POPS];
  i64 counts_ld[PGLD_MAX_POPS];
  const int32_t* nvalid[PGLD_MAX_POPS];
  i64 nvalid_ld[PGLD_MAX_POPS];
  int n_pops;
};

template <typename T>
__global__ void __launch_bounds__(256) geno_stats_kernel(GStatsArgs a, i64 n_pairs,
                                                         const pgld_term* __restrict__ terms,
                                                         int n_terms, T* __restrict__ out,
                                                         i64 out_ld) {
  for (i64 k = (i64)blockIdx.x * 256 + threadIdx.x; k < n_pairs; k += (i64)gridDim.x * 256) {
    int c[PGLD_MAX_POPS][9];
    GPop P[PGLD_MAX_POPS];
    const int* cp[PGLD_MAX_POPS];
    for (int p = 0; p < a.n_pops; ++p) {
      const int32_t* src = a.counts[p] + k * a.counts_ld[p];
#pragma unroll
      for (int q = 0; q < 9; ++q) c[p][q] = src[q];
      const i64 nv = a.nvalid[p] ? (i64)a.nvalid[p][k * a.nvalid_ld[p]] : -1;
      P[p] = make_gpop(c[p], nv);
      cp[p] = c[p];
    }
    T* o = out + k * out_ld;
    int cur = -1, in_stat = 0;
    T acc = 0;
    for (int t = 0; t < n_terms; ++t) {
      const pgld_term tm = terms[t];
      if (tm.stat != cur) {
        if (cur >= 0) o[cur] = acc;
        cur = tm.stat;
        acc = 0;
        in_stat = 0;
      }
      const T v = term_value<T>(tm, P, cp);
      const bool last = (t + 1 == n_terms) || (terms[t + 1].stat != cur);
      acc = (in_stat == 0 && last && tm.weight == 1.0) ? v : acc + (T)tm.weight * v;
      ++in_stat;
    }
    if (cur >= 0) o[cur] = acc;
  }
}

// ---------------------------------------------------------------------------
// distance-band kernel: 32 x 32 SNP tiles of the band work list
// ---------------------------------------------------------------------------
constexpr int kT = 32;       // SNPs per tile side (the work list's tile)
constexpr int kKW = 32;      // words of a plane staged per chunk
constexpr int kPad = 33;
constexpr int kThreads = 256;

struct __align__(16) GTileSmem {
  uint32_t pi[3][kKW][kPad], pj[3][kKW][kPad];
  uint32_t vi[kKW][kPad], vj[kKW][kPad];
  double bins[kMaxBins + 1];
};

__device__ __forceinline__ void stage_plane(uint32_t (*dst)[kPad], const uint32_t* __restrict__ src,
                                            i64 s0, i64 n_snp, i64 stride, int w0, int W) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kT / (kThreads / 32); ++q) {
    const int sl = wid * (kT / (kThreads / 32)) + q;
    const i64 s = s0 + sl;
    const int w = w0 + lane;
    uint32_t v = 0;
    if (s < n_snp && w < W) v = __ldg(src + s * stride + w);
    dst[lane][sl] = v;
  }
}

__device__ __forceinline__ i64 find_block(const i64* __restrict__ off, i64 nb, i64 k) {
  i64 lo = 0, hi = nb;
  while (hi - lo > 1) {
    const i64 mid = (lo + hi) >> 1;
    if (off[mid] <= k) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ int bin_index(const double* sb, int n_bins, double d) {
  if (!(d >= sb[0]) || !(d < sb[n_bins])) return -1;
  int lo = 0, hi = n_bins;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (sb[mid] <= d) lo = mid; else hi = mid;
  }
  return lo;
}

// MODE kModePairs: one population, per-pair outputs; kModeBinned: sums of the
// term table into distance bins.  PMAX bounds the population count.
template <int MODE, int PMAX>
__global__ void __launch_bounds__(kThreads) geno_band_kernel(BandArgs a) {
  const int n_pops = PMAX == 1 ? 1 : a.n_pops;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  GTileSmem& sm = *reinterpret_cast<GTileSmem*>(smem_raw);
  // per-tile counts [pop][class][row][col] and valid n [pop][row][col]
  int* tcnt = reinterpret_cast<int*>(smem_raw + sizeof(GTileSmem));
  int* tnv = tcnt + n_pops * 9 * kT * kPad;
  double* acc = reinterpret_cast<double*>(tnv + ((n_pops * kT * kPad + 1) & ~1));
  unsigned long long* bcnt =
      reinterpret_cast<unsigned long long*>(acc + (MODE == kModeBinned ? a.n_bins * a.n_stats : 0));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;

  if (MODE == kModeBinned) {
    for (int x = threadIdx.x; x < a.n_bins * a.n_stats; x += kThreads) acc[x] = 0.0;
    for (int x = threadIdx.x; x < a.n_bins; x += kThreads) bcnt[x] = 0ull;
    for (int x = threadIdx.x; x <= a.n_bins; x += kThreads) sm.bins[x] = a.bins[x];
  }
  __syncthreads();
  i64 n_items = a.item_off[a.n_blocks];
  if (n_items < 0 || n_items > a.n_blocks * (a.n_blocks + 1) / 2) {
    if (threadIdx.x == 0 && a.status) atomicCAS(a.status, 0, 2101);
    n_items = 0;
  }

  for (i64 item = blockIdx.x; item < n_items; item += gridDim.x) {
    const i64 bi = find_block(a.item_off, a.n_blocks, item);
    const i64 bj = bi + (item - a.item_off[bi]);
    const i64 i0 = bi * kT, j0 = bj * kT;

    for (int p = 0; p < n_pops; ++p) {
      const int W = a.W[p];
      const uint32_t* pl = a.planes[p];
      const uint32_t* vl = a.valid[p];
      int c[4][9];
      int nv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        nv[q] = 0;
#pragma unroll
        for (int x = 0; x < 9; ++x) c[q][x] = 0;
      }
      for (int w0 = 0; w0 < W; w0 += kKW) {
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          stage_plane(sm.pi[x], pl + x * W, i0, a.n_snp, 3 * W, w0, W);
          stage_plane(sm.pj[x], pl + x * W, j0, a.n_snp, 3 * W, w0, W);
        }
        if (vl) {
          stage_plane(sm.vi, vl, i0, a.n_snp, W, w0, W);
          stage_plane(sm.vj, vl, j0, a.n_snp, W, w0, W);
        }
        __syncthreads();
        const int nw = min(kKW, W - w0);
        for (int w = 0; w < nw; ++w) {
          const uint32_t b0 = sm.pj[0][w][lane], b1 = sm.pj[1][w][lane], b2 = sm.pj[2][w][lane];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int r = wid + 8 * q;
            const uint32_t a0 = sm.pi[0][w][r], a1 = sm.pi[1][w][r], a2 = sm.pi[2][w][r];
            c[q][0] += __popc(a0 & b0);
            c[q][1] += __popc(a0 & b1);
            c[q][2] += __popc(a0 & b2);
            c[q][3] += __popc(a1 & b0);
            c[q][4] += __popc(a1 & b1);
            c[q][5] += __popc(a1 & b2);
            c[q][6] += __popc(a2 & b0);
            c[q][7] += __popc(a2 & b1);
            c[q][8] += __popc(a2 & b2);
          }
        }
        if (vl)
          for (int w = 0; w < nw; ++w) {
            const uint32_t vj = sm.vj[w][lane];
#pragma unroll
            for (int q = 0; q < 4; ++q) nv[q] += __popc(sm.vi[w][wid + 8 * q] & vj);
          }
        __syncthreads();
      }
      if (a.gext[p]) {
        // values 3..8 at the second SNP fold into the classes 3 g_i + g_j
        // (values 0 and 1 at the first SNP); two passes of three planes
        const uint32_t* xl = a.gext[p];
        for (int half = 0; half < 2; ++half)
          for (int w0 = 0; w0 < W; w0 += kKW) {
            stage_plane(sm.pi[0], pl, i0, a.n_snp, 3 * W, w0, W);
            stage_plane(sm.pi[1], pl + W, i0, a.n_snp, 3 * W, w0, W);
#pragma unroll
            for (int x = 0; x < 3; ++x)
              stage_plane(sm.pj[x], xl + (3 * half + x) * W, j0, a.n_snp, 6 * W, w0, W);
            __syncthreads();
            const int nw = min(kKW, W - w0);
            for (int w = 0; w < nw; ++w)
#pragma unroll
              for (int x = 0; x < 3; ++x) {
                const uint32_t b = sm.pj[x][w][lane];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                  const int r = wid + 8 * q;
                  c[q][3 + 3 * half + x] += __popc(sm.pi[0][w][r] & b);
                  if (half == 0) c[q][6 + x] += __popc(sm.pi[1][w][r] & b);
                }
              }
            __syncthreads();
          }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = wid + 8 * q;
        int tot = 0;
#pragma unroll
        for (int x = 0; x < 9; ++x) {
          tcnt[((p * 9 + x) * kT + r) * kPad + lane] = c[q][x];
          tot += c[q][x];
        }
        tnv[(p * kT + r) * kPad + lane] = vl ? nv[q] : tot;
      }
    }
    __syncwarp();

    // ---- epilogue: thread (wid, lane) owns the pairs (wid + 8q, lane) ----
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
      const int r = wid + 8 * q;
      const i64 i = i0 + r, j = j0 + lane;
      bool ok = (i < j) && (j < a.n_snp);
      double dpos = 0.0;
      if (ok) {
        dpos = a.pos[j] - a.pos[i];
        ok = dpos <= a.max_dist;
      }
      int cc[PMAX][9];
      GPop P[PMAX];
      const int* cp[PMAX];
      for (int p = 0; p < n_pops; ++p) {
#pragma unroll
        for (int x = 0; x < 9; ++x) cc[p][x] = tcnt[((p * 9 + x) * kT + r) * kPad + lane];
        const int n = tnv[(p * kT + r) * kPad + lane];
        P[p] = make_gpop(cc[p], a.valid[p] ? (i64)n : -1);
        cp[p] = cc[p];
      }
      if (MODE == kModePairs) {
        // rows come from the band offsets: write exactly the pairs they list
        if (i < j && j < a.n_snp) ok = (j - i - 1) < (a.pair_off[i + 1] - a.pair_off[i]);
        if (ok) {
          const i64 k = a.pair_off[i] + (j - i - 1);
          if (a.counts) {
            int32_t* o = a.counts + k * 9;
#pragma unroll
            for (int x = 0; x < 9; ++x) o[x] = cc[0][x];
          }
          if (a.nvalid) a.nvalid[k] = (int32_t)P[0].n;
          if (a.stats) {
            // only the requested columns are evaluated; the others are 0
            reinterpret_cast<float4*>(a.stats)[k] =
                gmom::stats_f32<-1>(gmom::from_counts(cc[0]), a.stat_mask);
          }
        }
      } else {
        int b = -1;
        if (ok) {
          const double d = a.bcoord ? fabs(a.bcoord[j] - a.bcoord[i]) : dpos;
          b = bin_index(sm.bins, a.n_bins, d);
        }
        unsigned pending = __ballot_sync(0xffffffffu, b >= 0);
        while (pending) {
          const int bb = __shfl_sync(0xffffffffu, b, __ffs(pending) - 1);
          const bool mine = (b == bb);
          const unsigned grp = __ballot_sync(0xffffffffu, mine);
          int t = 0;
          for (int s = 0; s < a.n_stats; ++s) {
            float v = 0.f;
            for (; t < a.n_terms && a.terms[t].stat == s; ++t) {
              const pgld_term tm = a.terms[t];
              if (mine) v += (float)tm.weight * term_value<float>(tm, P, cp);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) atomicAdd(&acc[bb * a.n_stats + s], (double)v);
          }
          if (lane == 0) atomicAdd(&bcnt[bb], (unsigned long long)__popc(grp));
          pending &= ~grp;
        }
      }
    }
    __syncthreads();
  }

  if (MODE == kModeBinned) {
    __syncthreads();
    for (int x = threadIdx.x; x < a.n_bins * a.n_stats; x += kThreads)
      if (acc[x] != 0.0) atomicAdd(a.sums + x, acc[x]);
    if (a.pair_counts)
      for (int x = threadIdx.x; x < a.n_bins; x += kThreads)
        if (bcnt[x]) atomicAdd(reinterpret_cast<unsigned long long*>(a.pair_counts) + x, bcnt[x]);
  }
}

size_t geno_band_smem(int mode, int n_pops, int n_bins, int n_stats) {
  size_t s = sizeof(GTileSmem);
  s += (size_t)n_pops * 9 * kT * kPad * 4;
  s += (size_t)((n_pops * kT * kPad + 1) & ~1) * 4;
  if (mode == kModeBinned) s += (size_t)n_bins * n_stats * 8 + (size_t)n_bins * 8;
  return s;
}

template <int MODE, int PMAX>
int launch_geno_band(pgld_context* h, const BandArgs& a, cudaStream_t st) {
  const size_t smem = geno_band_smem(MODE, PMAX == 1 ? 1 : a.n_pops, a.n_bins, a.n_stats);
  auto kern = geno_band_kernel<MODE, PMAX>;
  cudaError_t e =
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "geno_band smem attribute");
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "geno_band occupancy");
  per_sm = std::max(1, per_sm);
  pgld_time_begin(h, st);
  kern<<<(unsigned)(h->n_sm * per_sm), kThreads, smem, st>>>(a);
  pgld_time_end(h, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return pgld_cuda_fail(h, e, "geno_band_kernel");
  return PGLD_OK;
}

}  // namespace geno
}  // namespace pgld

// ---------------------------------------------------------------------------
// entry points
// ---------------------------------------------------------------------------
extern "C" int pgld_pack_genotypes(pgld_handle h, const int8_t* geno, int64_t ld, int64_t n_snp,
                                   const int32_t* rows, int32_t n_rows, uint32_t* planes,
                                   uint32_t* valid, uint32_t* ext, int32_t* flags, void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_pack_genotypes: NULL handle");
  PGLD_REQUIRE(h, n_snp >= 0 && n_rows >= 0, "pgld_pack_genotypes: negative size");
  PGLD_REQUIRE(h, planes && flags && (geno || n_snp == 0 || n_rows == 0),
               "pgld_pack_genotypes: NULL buffer");
  PGLD_REQUIRE(h, ld >= n_snp, "pgld_pack_genotypes: row stride %lld < n_snp %lld",
               (long long)ld, (long long)n_snp);
  PGLD_REQUIRE(h, n_rows <= pgld::geno::kMaxGenoN,
               "pgld_pack_genotypes: %d individuals exceed %d per population", n_rows,
               pgld::geno::kMaxGenoN);
  const int W = (n_rows + 31) / 32;
  if (n_snp == 0 || W == 0) return PGLD_OK;
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  dim3 grid((unsigned)((n_snp + 255) / 256), (unsigned)W);
  pgld::geno::pack_geno_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(geno, ld, n_snp, rows,
                                                                       n_rows, W, planes, valid,
                                                                       ext, flags);
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  return PGLD_OK;
}

extern "C" int pgld_geno_counts_pairs(pgld_handle h, const uint32_t* planes, const uint32_t* valid,
                                      const uint32_t* ext, int32_t n_words, int64_t n_snp,
                                      const int32_t* idx_i,
                                      const int32_t* idx_j, int64_t n_pairs, int32_t* counts,
                                      int64_t counts_ld, int32_t* n_valid, void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_geno_counts_pairs: NULL handle");
  PGLD_REQUIRE(h, n_pairs >= 0 && n_words >= 0 && n_snp >= 0,
               "pgld_geno_counts_pairs: negative size");
  if (n_pairs == 0) return PGLD_OK;
  PGLD_REQUIRE(h, planes && idx_i && idx_j && counts, "pgld_geno_counts_pairs: NULL buffer");
  PGLD_REQUIRE(h, counts_ld >= 9, "pgld_geno_counts_pairs: counts_ld < 9");
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  int G = 1;
  while (G < n_words && G < 32) G <<= 1;
  const i64 blocks = std::min<i64>(std::max<i64>((n_pairs * G + 255) / 256, 1), (i64)h->n_sm * 16);
#define PGLD_LAUNCH_GC(GG)                                                                  \
  pgld::geno::geno_counts_pairs_kernel<GG><<<(unsigned)blocks, 256, 0, st>>>(              \
      planes, valid, ext, n_words, n_snp, idx_i, idx_j, n_pairs, counts, counts_ld, n_valid, \
      h->dev_status)
  switch (G) {
    case 1: PGLD_LAUNCH_GC(1); break;
    case 2: PGLD_LAUNCH_GC(2); break;
    case 4: PGLD_LAUNCH_GC(4); break;
    case 8: PGLD_LAUNCH_GC(8); break;
    case 16: PGLD_LAUNCH_GC(16); break;
    default: PGLD_LAUNCH_GC(32); break;
  }
#undef PGLD_LAUNCH_GC
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  return PGLD_OK;
}

extern "C" int pgld_geno_stat_terms(int32_t n_pops, pgld_term* out, int32_t capacity,
                                    int32_t* n_terms_out, int32_t* n_stats_out) {
  if (n_pops < 1 || n_pops > PGLD_MAX_POPS)
    return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_geno_stat_terms: n_pops %d", n_pops);
  std::vector<pgld_term> t;
  pgld_build_spec_terms(n_pops, t, true);
  if (n_terms_out) *n_terms_out = (int32_t)t.size();
  if (n_stats_out) *n_stats_out = pgld_n_stats(n_pops);
  if (out) {
    if (capacity < (int32_t)t.size())
      return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_geno_stat_terms: capacity %d < %d",
                       capacity, (int)t.size());
    std::copy(t.begin(), t.end(), out);
  }
  return PGLD_OK;
}

extern "C" int pgld_geno_stats(pgld_handle h, const pgld_pair_counts* counts, int64_t n_pairs,
                               const pgld_term* terms, int32_t n_terms, int32_t n_stats, void* out,
                               int32_t out_dtype, int64_t out_ld, void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_geno_stats: NULL handle");
  PGLD_REQUIRE(h, counts && terms && n_terms > 0, "pgld_geno_stats: NULL argument");
  PGLD_REQUIRE(h, counts->n_pops >= 1 && counts->n_pops <= PGLD_MAX_POPS,
               "pgld_geno_stats: n_pops %d", counts->n_pops);
  PGLD_REQUIRE(h, n_pairs >= 0 && n_stats >= 1 && out_ld >= n_stats, "pgld_geno_stats: bad sizes");
  PGLD_REQUIRE(h, out_dtype == PGLD_F64 || out_dtype == PGLD_F32, "pgld_geno_stats: out_dtype");
  if (n_pairs == 0) return PGLD_OK;
  PGLD_REQUIRE(h, out != nullptr, "pgld_geno_stats: NULL out");
  pgld::geno::GStatsArgs a{};
  a.n_pops = counts->n_pops;
  for (int p = 0; p < a.n_pops; ++p) {
    PGLD_REQUIRE(h, counts->counts[p] && counts->counts_ld[p] >= 9,
                 "pgld_geno_stats: counts of population %d", p);
    a.counts[p] = counts->counts[p];
    a.counts_ld[p] = counts->counts_ld[p];
    a.nvalid[p] = counts->n_valid[p];
    a.nvalid_ld[p] = counts->nvalid_ld[p];
  }
  int prev = -1;
  for (int t = 0; t < n_terms; ++t) {
    const pgld_term& x = terms[t];
    PGLD_REQUIRE(h, x.stat >= 0 && x.stat < n_stats && x.stat >= prev,
                 "pgld_geno_stats: term %d stat column %d (columns must be non-decreasing)", t,
                 x.stat);
    prev = x.stat;
    PGLD_REQUIRE(h, x.kind >= PGLD_G_DD_II && x.kind <= PGLD_G_RH_R2,
                 "pgld_geno_stats: term %d kind %d is not a genotype kind", t, x.kind);
    for (int q = 0; q < 4; ++q)
      PGLD_REQUIRE(h, x.pops[q] >= 0 && x.pops[q] < a.n_pops,
                   "pgld_geno_stats: term %d population %d", t, x.pops[q]);
  }
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  void* ws = nullptr;
  int rc = pgld_workspace(h, n_terms * sizeof(pgld_term), &ws);
  if (rc) return rc;
  PGLD_CHECK_CUDA(h, cudaMemcpyAsync(ws, terms, n_terms * sizeof(pgld_term),
                                     cudaMemcpyHostToDevice, st));
  const i64 blocks = std::min<i64>((n_pairs + 255) / 256, (i64)h->n_sm * 8);
  if (out_dtype == PGLD_F64)
    pgld::geno::geno_stats_kernel<double><<<(unsigned)blocks, 256, 0, st>>>(
        a, n_pairs, (const pgld_term*)ws, n_terms, (double*)out, out_ld);
  else
    pgld::geno::geno_stats_kernel<float><<<(unsigned)blocks, 256, 0, st>>>(
        a, n_pairs, (const pgld_term*)ws, n_terms, (float*)out, out_ld);
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  // the term table lives in the workspace: keep it alive until the kernel ran
  PGLD_CHECK_CUDA(h, cudaStreamSynchronize(st));
  return PGLD_OK;
}

static int check_geno_panel(pgld_context* h, const pgld_geno_panel* panel, const char* fn) {
  PGLD_REQUIRE(h, panel != nullptr, "%s: NULL panel", fn);
  PGLD_REQUIRE(h, panel->n_pops >= 1 && panel->n_pops <= PGLD_MAX_POPS, "%s: n_pops %d", fn,
               panel->n_pops);
  PGLD_REQUIRE(h, panel->n_snp >= 0, "%s: n_snp < 0", fn);
  for (int p = 0; p < panel->n_pops; ++p) {
    PGLD_REQUIRE(h, panel->n_words[p] >= 1 && panel->n_words[p] * 32 <= pgld::geno::kMaxGenoN + 31,
                 "%s: population %d has %d words", fn, p, panel->n_words[p]);
    PGLD_REQUIRE(h, panel->planes[p] != nullptr || panel->n_snp == 0, "%s: planes[%d] NULL", fn, p);
  }
  return PGLD_OK;
}

static void fill_geno_panel(pgld::BandArgs& a, const pgld_geno_panel* panel) {
  a.n_pops = panel->n_pops;
  for (int p = 0; p < PGLD_MAX_POPS; ++p) {
    a.W[p] = p < panel->n_pops ? panel->n_words[p] : 0;
    a.planes[p] = p < panel->n_pops ? panel->planes[p] : nullptr;
    a.valid[p] = p < panel->n_pops ? panel->valid[p] : nullptr;
    a.gext[p] = p < panel->n_pops ? panel->ext[p] : nullptr;
  }
  a.n_snp = panel->n_snp;
}

int pgld_geno_tc_pairs(pgld_context* h, const pgld_geno_panel* panel, const double* pos,
                       double max_dist, int32_t* counts, int32_t* n_valid, float* stats,
                       int32_t stat_mask, cudaStream_t st);

extern "C" int pgld_geno_band_pairs(pgld_handle h, const pgld_geno_panel* panel, const double* pos,
                                    double max_dist, int32_t* counts, int32_t* n_valid,
                                    float* stats, int32_t stat_mask, int64_t n_pairs,
                                    int32_t form, void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_geno_band_pairs: NULL handle");
  int rc = check_geno_panel(h, panel, "pgld_geno_band_pairs");
  if (rc) return rc;
  PGLD_REQUIRE(h, panel->n_pops == 1, "pgld_geno_band_pairs: one population per call");
  PGLD_REQUIRE(h, max_dist >= 0, "pgld_geno_band_pairs: negative max_dist");
  PGLD_REQUIRE(h, n_pairs >= 0, "pgld_geno_band_pairs: n_pairs < 0");
  const i64 n = panel->n_snp;
  if (n < 2) {
    PGLD_REQUIRE(h, n_pairs == 0, "pgld_geno_band_pairs: %lld pairs for %lld SNPs",
                 (long long)n_pairs, (long long)n);
    return PGLD_OK;
  }
  PGLD_REQUIRE(h, pos != nullptr, "pgld_geno_band_pairs: NULL pos");
  PGLD_REQUIRE(h, !stats || ((uintptr_t)stats & 15) == 0,
               "pgld_geno_band_pairs: stats must be 16-byte aligned");
  PGLD_REQUIRE(h, (stat_mask & ~15) == 0, "pgld_geno_band_pairs: stat_mask %d", stat_mask);
  PGLD_REQUIRE(h, form == PGLD_FORM_PLAIN || form == PGLD_FORM_TC, "pgld_geno_band_pairs: form");
  if (form == PGLD_FORM_TC && (panel->ext[0] != nullptr || panel->valid[0] != nullptr))
    return pgld_fail(h, PGLD_ERR_UNSUPPORTED, "pgld_geno_band_pairs: the tensor-core form "
                     "takes dosages 0/1/2 only (missing allowed)");
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  const i64 nb = (n + pgld::geno::kT - 1) / pgld::geno::kT;
  const size_t sb1 = pgld::scan_scratch_bytes(n), sb2 = pgld::scan_scratch_bytes(nb);
  const size_t off_bytes = (size_t)(n + 1) * 8, it_bytes = (size_t)(nb + 1) * 8;
  void* ws = nullptr;
  rc = pgld_workspace(h, off_bytes + it_bytes + std::max(sb1, sb2) + 768, &ws);
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
    return pgld_fail(h, PGLD_ERR_INVALID_ARG, "pgld_geno_band_pairs: n_pairs %lld != %lld in band",
                     (long long)n_pairs, (long long)tot);
  if (tot == 0) return PGLD_OK;
  if (form == PGLD_FORM_TC)
    return pgld_geno_tc_pairs(h, panel, pos, max_dist, counts, n_valid, stats, stat_mask, st);
  rc = pgld::band_schedule(h, pos, n, max_dist, items, scratch, std::max(sb1, sb2), st,
                           pgld::geno::kT);
  if (rc) return rc;
  pgld::BandArgs a{};
  a.status = h->dev_status;
  fill_geno_panel(a, panel);
  a.pos = pos;
  a.max_dist = max_dist;
  a.item_off = items;
  a.n_blocks = nb;
  a.pair_off = off;
  a.counts = counts;
  a.nvalid = n_valid;
  a.stats = stats;
  a.stat_mask = stat_mask;
  return pgld::geno::launch_geno_band<pgld::kModePairs, 1>(h, a, st);
}

int pgld_geno_tc_binned(pgld_context* h, const pgld_geno_panel* panel, const pgld::BandArgs& ba,
                        cudaStream_t st);

extern "C" int pgld_geno_binned_sums(pgld_handle h, const pgld_geno_panel* panel,
                                     const double* pos, double max_dist, const double* bin_coord,
                                     const double* bins, int32_t n_bins, double* sums,
                                     int64_t* pair_counts, void* stream) {
  return pgld_geno_binned_sums_form(h, panel, pos, max_dist, bin_coord, bins, n_bins, sums,
                                    pair_counts, PGLD_FORM_PLAIN, stream);
}

extern "C" int pgld_geno_binned_sums_form(pgld_handle h, const pgld_geno_panel* panel,
                                          const double* pos, double max_dist,
                                          const double* bin_coord, const double* bins,
                                          int32_t n_bins, double* sums, int64_t* pair_counts,
                                          int32_t form, void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_geno_binned_sums: NULL handle");
  PGLD_REQUIRE(h, form == PGLD_FORM_PLAIN || form == PGLD_FORM_TC,
               "pgld_geno_binned_sums: unknown form %d", form);
  int rc = check_geno_panel(h, panel, "pgld_geno_binned_sums");
  if (rc) return rc;
  PGLD_REQUIRE(h, n_bins >= 1 && n_bins <= pgld::kMaxBins,
               "pgld_geno_binned_sums: n_bins %d not in [1, %d]", n_bins, pgld::kMaxBins);
  PGLD_REQUIRE(h, bins && sums, "pgld_geno_binned_sums: NULL bins/sums");
  PGLD_REQUIRE(h, max_dist >= 0, "pgld_geno_binned_sums: negative max_dist");
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  const int P = panel->n_pops;
  const int S = h->spec_n_stats[P];
  PGLD_CHECK_CUDA(h, cudaMemsetAsync(sums, 0, (size_t)n_bins * S * 8, st));
  if (pair_counts) PGLD_CHECK_CUDA(h, cudaMemsetAsync(pair_counts, 0, (size_t)n_bins * 8, st));
  const i64 n = panel->n_snp;
  if (n < 2) return PGLD_OK;
  PGLD_REQUIRE(h, pos != nullptr, "pgld_geno_binned_sums: NULL pos");
  const i64 nb = (n + pgld::geno::kT - 1) / pgld::geno::kT;
  const size_t sb = pgld::scan_scratch_bytes(nb);
  void* ws = nullptr;
  rc = pgld_workspace(h, (size_t)(nb + 1) * 8 + sb + 512, &ws);
  if (rc) return rc;
  i64* items = (i64*)ws;
  char* scratch = (char*)ws + ((((size_t)(nb + 1) * 8) + 255) & ~size_t(255));
  rc = pgld::band_schedule(h, pos, n, max_dist, items, scratch, sb, st, pgld::geno::kT);
  if (rc) return rc;
  pgld::BandArgs a{};
  a.status = h->dev_status;
  fill_geno_panel(a, panel);
  a.pos = pos;
  a.max_dist = max_dist;
  a.bcoord = bin_coord;
  a.bins = bins;
  a.n_bins = n_bins;
  a.item_off = items;
  a.n_blocks = nb;
  a.sums = sums;
  a.pair_counts = pair_counts;
  a.terms = h->gspec_terms[P];
  a.n_terms = h->gspec_n_terms[P];
  a.n_stats = S;
  if (form == PGLD_FORM_TC) {
    for (int p = 0; p < P; ++p)
      PGLD_REQUIRE(h, panel->ext[p] == nullptr,
                   "pgld_geno_binned_sums: the tensor-core form takes dosages 0..2 only");
    return pgld_geno_tc_binned(h, panel, a, st);
  }
  if (P == 1) return pgld::geno::launch_geno_band<pgld::kModeBinned, 1>(h, a, st);
  return pgld::geno::launch_geno_band<pgld::kModeBinned, PGLD_MAX_POPS>(h, a, st);
}
