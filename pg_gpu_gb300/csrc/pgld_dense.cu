// Dense all-pairs LD of one population (the M x M outputs of
// HaplotypeMatrix.pairwise_LD_v / pairwise_r2, haplotype_matrix.py:1092-1170)
// and the distance-binned r^2 percentiles of windowed_r_squared
// (haplotype_matrix.py:1235-1317) without moving the pair values to the host:
// the valid pairs' r^2 are grouped by distance bin on the device and each
// requested order statistic is found by an 8-bit radix select (one CTA per
// order statistic, eight passes over its bin's values).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "pgld_band.cuh"
#include "pgld_internal.cuh"

using pgld::i64;

namespace pgld {
namespace dense {

constexpr int kT = 32;         // SNPs per tile side
constexpr int kThreads = 256;  // warp w: rows w + 8 q of the tile, lane: column
constexpr int kKW = 32;        // words of a plane staged per chunk
constexpr int kPad = 33;

struct __align__(16) Smem {
  uint32_t ci[kKW][kPad], vi[kKW][kPad], cj[kKW][kPad], vj[kKW][kPad];
  double tr[kT][kT + 1];   // mirrored tile
  double bins[kMaxBins + 1];
  int bin_cnt[kMaxBins];
  long long bin_base[kMaxBins];
};

// upper-triangle tile t -> (bi, bj), bj >= bi, of nb blocks (row bi owns
// tiles bi .. nb - 1, starting at bi nb - bi (bi - 1) / 2)
__device__ __forceinline__ void tri_decode(i64 t, i64 nb, i64& bi, i64& bj) {
  // largest bi with start(bi) <= t, from the quadratic, then corrected
  const double b = (double)(2 * nb + 1);
  i64 r = (i64)floor((b - sqrt(b * b - 8.0 * (double)t)) / 2.0);
  r = max((i64)0, min(r, nb - 1));
  auto start = [&](i64 x) { return x * nb - x * (x - 1) / 2; };
  while (r > 0 && start(r) > t) --r;
  while (r + 1 < nb && start(r + 1) <= t) ++r;
  bi = r;
  bj = r + (t - start(r));
}

// stage carrier and valid (carrier | reference) words of 32 SNPs, transposed
__device__ __forceinline__ void stage(uint32_t (*c)[kPad], uint32_t (*v)[kPad],
                                      const uint32_t* __restrict__ planes, int W, i64 s0, i64 n,
                                      int w0) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kT / 8; ++q) {
    const int sl = wid * (kT / 8) + q;
    const i64 s = s0 + sl;
    const int w = w0 + lane;
    uint32_t cc = 0, zz = 0;
    if (s < n && w < W) {
      cc = __ldg(planes + s * 2 * W + w);
      zz = __ldg(planes + s * 2 * W + W + w);
    }
    c[lane][sl] = cc;
    v[lane][sl] = cc | zz;
  }
}

// joint counts of the tile's pairs (i0 + wid + 8 q, j0 + lane): C_i.C_j
// (n11), C_i.V_j (pA), V_i.C_j (pB) and V_i.V_j (the pairwise-valid n)
__device__ __forceinline__ void tile_counts(Smem& sm, const uint32_t* planes, int W, i64 n, i64 i0,
                                            i64 j0, int (&cc)[4], int (&cv)[4], int (&vc)[4],
                                            int (&vv)[4]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 4; ++q) cc[q] = cv[q] = vc[q] = vv[q] = 0;
  for (int w0 = 0; w0 < W; w0 += kKW) {
    __syncthreads();
    stage(sm.ci, sm.vi, planes, W, i0, n, w0);
    stage(sm.cj, sm.vj, planes, W, j0, n, w0);
    __syncthreads();
    const int nw = min(kKW, W - w0);
    for (int w = 0; w < nw; ++w) {
      const uint32_t cj = sm.cj[w][lane], vj = sm.vj[w][lane];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = wid + 8 * q;
        const uint32_t ci = sm.ci[w][r], vi = sm.vi[w][r];
        cc[q] += __popc(ci & cj);
        cv[q] += __popc(ci & vj);
        vc[q] += __popc(vi & cj);
        vv[q] += __popc(vi & vj);
      }
    }
  }
}

__global__ void site_freq_kernel(const uint32_t* __restrict__ planes, int W, i64 n,
                                 double* __restrict__ p) {
  for (i64 s = (i64)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (i64)gridDim.x * blockDim.x) {
    int car = 0, val = 0;
    for (int w = 0; w < W; ++w) {
      const uint32_t c = planes[s * 2 * W + w], z = planes[s * 2 * W + W + w];
      car += __popc(c);
      val += __popc(c | z);
    }
    // p = sum / n_valid where n_valid > 0 (haplotype_matrix.py:1122)
    p[s] = val > 0 ? __ddiv_rn((double)car, (double)val) : 0.0;
  }
}

// D = pAB - p_i p_j and r^2 = D^2 / (p_i (1 - p_i) p_j (1 - p_j)) of every
// pair, rounded operation by operation as the reference's float64 matrix
// expressions (haplotype_matrix.py:1125-1128, 1165-1169), zero diagonal
__global__ void __launch_bounds__(kThreads) pairwise_ld_kernel(const uint32_t* __restrict__ planes,
                                                               int W, i64 n,
                                                               const double* __restrict__ p,
                                                               double* __restrict__ D_out,
                                                               double* __restrict__ r2_out, i64 ld) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const i64 nb = (n + kT - 1) / kT;
  const i64 n_tiles = nb * (nb + 1) / 2;
  for (i64 t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    i64 bi, bj;
    tri_decode(t, nb, bi, bj);
    const i64 i0 = bi * kT, j0 = bj * kT;
    int n11[4], cv[4], vc[4], nv[4];
    tile_counts(sm, planes, W, n, i0, j0, n11, cv, vc, nv);
    for (int out = 0; out < 2; ++out) {
      double* M = out == 0 ? D_out : r2_out;
      if (!M) continue;
      double val[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const i64 i = i0 + wid + 8 * q, j = j0 + lane;
        double v = 0.0;
        if (i < n && j < n && i != j) {
          const double pi = p[i], pj = p[j];
          const double pab = nv[q] > 0 ? __ddiv_rn((double)n11[q], (double)nv[q]) : 0.0;
          const double d = __dsub_rn(pab, __dmul_rn(pi, pj));
          if (out == 0) {
            v = d;
          } else {
            const double den = __dmul_rn(__dmul_rn(pi, __dsub_rn(1.0, pi)),
                                         __dmul_rn(pj, __dsub_rn(1.0, pj)));
            v = den > 0.0 ? __ddiv_rn(__dmul_rn(d, d), den) : 0.0;
          }
        }
        val[q] = v;
        if (i < n && j < n) M[i * ld + j] = v;
      }
      if (bj != bi) {
        // the mirrored block (j, i), written row by row through shared memory
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 4; ++q) sm.tr[lane][wid + 8 * q] = val[q];
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const i64 j = j0 + wid + 8 * q, i = i0 + lane;
          if (i < n && j < n) M[j * ld + i] = sm.tr[wid + 8 * q][lane];
        }
      }
    }
  }
}

__device__ __forceinline__ int bin_index(const double* sb, int n_bins, double d) {
  // digitize(d, bins) - 1 with right-open bins; -1 outside [bins[0], bins[n_bins])
  if (!(d >= sb[0]) || !(d < sb[n_bins])) return -1;
  int lo = 0, hi = n_bins;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (sb[mid] <= d) lo = mid; else hi = mid;
  }
  return lo;
}

// every pair i < j: its value (r^2 from the joint counts, or values[k] of the
// condensed upper triangle), NaN skipped, binned by pos[j] - pos[i].
// counts mode (out == NULL): bin_counts[b] += pairs; fill mode: the values
// are written grouped by bin at cursor[b] (advanced atomically per tile).
__global__ void __launch_bounds__(kThreads) pairs_by_bin_kernel(
    const uint32_t* __restrict__ planes, int W, const double* __restrict__ values, i64 n,
    const double* __restrict__ pos, const double* __restrict__ bins, int n_bins,
    unsigned long long* __restrict__ bin_counts, unsigned long long* __restrict__ cursor,
    const unsigned long long* __restrict__ bin_end, double* __restrict__ out,
    int32_t* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int x = threadIdx.x; x <= n_bins; x += kThreads) sm.bins[x] = bins[x];
  const i64 nb = (n + kT - 1) / kT;
  const i64 n_tiles = nb * (nb + 1) / 2;
  for (i64 t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    i64 bi, bj;
    tri_decode(t, nb, bi, bj);
    const i64 i0 = bi * kT, j0 = bj * kT;
    int n11[4] = {0, 0, 0, 0}, cv[4] = {0, 0, 0, 0}, vc[4] = {0, 0, 0, 0}, nv[4] = {0, 0, 0, 0};
    if (!values) {
      tile_counts(sm, planes, W, n, i0, j0, n11, cv, vc, nv);
    } else {
      __syncthreads();
    }
    for (int x = threadIdx.x; x < n_bins; x += kThreads) sm.bin_cnt[x] = 0;
    __syncthreads();
    int bin[4], slot[4];
    double val[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const i64 i = i0 + wid + 8 * q, j = j0 + lane;
      bin[q] = -1;
      val[q] = 0.0;
      if (i < j && j < n) {
        double v;
        if (values) {
          v = values[i * (2 * n - i - 1) / 2 + (j - i - 1)];
        } else {
          // r^2 of ld_statistics.r_squared (haplotype_kernels.py:32-42):
          // (n11 n00 - n10 n01)^2 over pA (n - pA) pB (n - pB) of the pair's
          // valid haplotypes as exact integers, divided once; NaN where the
          // denominator is 0
          const long long a = n11[q], pa = cv[q], pb = vc[q], nn = nv[q];
          const long long b = pa - a, c = pb - a, d = nn - pa - pb + a;
          const long long x = a * d - b * c;
          const long long den = pa * (nn - pa) * pb * (nn - pb);
          v = den > 0 ? __ddiv_rn((double)(x * x), (double)den)
                      : __longlong_as_double(0x7ff8000000000000LL);
        }
        val[q] = v;
        if (v == v) bin[q] = bin_index(sm.bins, n_bins, pos[j] - pos[i]);
      }
      slot[q] = bin[q] >= 0 ? atomicAdd(&sm.bin_cnt[bin[q]], 1) : 0;
    }
    __syncthreads();
    for (int x = threadIdx.x; x < n_bins; x += kThreads) {
      const int c = sm.bin_cnt[x];
      if (!out) {
        if (c) atomicAdd(bin_counts + x, (unsigned long long)c);
      } else {
        sm.bin_base[x] = c ? (long long)atomicAdd(cursor + x, (unsigned long long)c) : 0;
      }
    }
    __syncthreads();
    if (out) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (bin[q] < 0) continue;
        const unsigned long long k = (unsigned long long)sm.bin_base[bin[q]] + (unsigned)slot[q];
        // the bin's range comes from a counting pass over the same inputs;
        // a pair beyond it (inputs changed in between) is dropped and flagged
        if (k < bin_end[bin[q]]) out[k] = val[q];
        else if (status) atomicCAS(status, 0, 4001);
      }
    }
    __syncthreads();
  }
}

// the rank-th smallest (0-based) value of each target's segment; values are
// non-negative doubles, whose bit patterns order like the values: eight
// passes over the segment, each fixing the next 8 bits of the answer from a
// histogram of the values that share the bits fixed so far
__global__ void __launch_bounds__(256) segment_kth_kernel(const double* __restrict__ values,
                                                          const long long* __restrict__ seg_off,
                                                          const long long* __restrict__ tseg,
                                                          const long long* __restrict__ trank,
                                                          double* __restrict__ out) {
  __shared__ unsigned hist[8][256];
  __shared__ unsigned long long prefix;
  __shared__ long long rem;
  const int t = blockIdx.x;
  const long long seg = tseg[t];
  const long long lo = seg_off[seg], hi = seg_off[seg + 1];
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    prefix = 0ull;
    rem = trank[t];
  }
  for (int pass = 0; pass < 8; ++pass) {
    const int shift = 56 - 8 * pass;
    for (int x = threadIdx.x; x < 8 * 256; x += blockDim.x) (&hist[0][0])[x] = 0u;
    __syncthreads();
    const unsigned long long want = pass == 0 ? 0ull : (prefix >> (shift + 8));
    for (long long k = lo + threadIdx.x; k < hi; k += blockDim.x) {
      const unsigned long long key = (unsigned long long)__double_as_longlong(values[k]);
      if (pass == 0 || (key >> (shift + 8)) == want)
        atomicAdd(&hist[warp][(unsigned)(key >> shift) & 255u], 1u);
    }
    __syncthreads();
    {
      unsigned v = 0;
#pragma unroll
      for (int w = 0; w < 8; ++w) v += hist[w][threadIdx.x];
      __syncthreads();
      hist[0][threadIdx.x] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      long long r = rem;
      int d = 255;
      for (int x = 0; x < 256; ++x) {
        if (r < (long long)hist[0][x]) {
          d = x;
          break;
        }
        r -= hist[0][x];
      }
      rem = r;
      prefix |= (unsigned long long)d << shift;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[t] = __longlong_as_double((long long)prefix);
}

}  // namespace dense
}  // namespace pgld

// ---------------------------------------------------------------------------
// entry points
// ---------------------------------------------------------------------------
static int dense_grid(pgld_context* h, const void* kern, size_t smem, i64 n_tiles) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, pgld::dense::kThreads, smem);
  per_sm = std::max(1, per_sm);
  return (int)std::max<i64>(1, std::min<i64>(n_tiles, (i64)h->n_sm * per_sm));
}

extern "C" int pgld_hap_pairwise_ld(pgld_handle h, const uint32_t* planes, int32_t n_words,
                                    int64_t n_snp, double* D_out, double* r2_out, int64_t ld,
                                    void* stream) {
  using namespace pgld::dense;
  PGLD_REQUIRE(h, h != nullptr, "pgld_hap_pairwise_ld: NULL handle");
  PGLD_REQUIRE(h, n_words >= 1 && n_snp >= 0 && ld >= n_snp, "pgld_hap_pairwise_ld: sizes");
  PGLD_REQUIRE(h, D_out || r2_out, "pgld_hap_pairwise_ld: no output");
  if (n_snp == 0) return PGLD_OK;
  PGLD_REQUIRE(h, planes != nullptr, "pgld_hap_pairwise_ld: NULL planes");
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  void* ws = nullptr;
  int rc = pgld_workspace(h, (size_t)n_snp * 8, &ws);
  if (rc) return rc;
  double* p = (double*)ws;
  const unsigned sb = (unsigned)std::max<i64>(1, std::min<i64>((n_snp + 255) / 256, h->n_sm * 8LL));
  site_freq_kernel<<<sb, 256, 0, st>>>(planes, n_words, n_snp, p);
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  const i64 nb = (n_snp + kT - 1) / kT;
  const size_t smem = sizeof(Smem);
  auto kern = pairwise_ld_kernel;
  PGLD_CHECK_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = dense_grid(h, (const void*)kern, smem, nb * (nb + 1) / 2);
  pgld_time_begin(h, st);
  kern<<<grid, kThreads, smem, st>>>(planes, n_words, n_snp, p, D_out, r2_out, ld);
  pgld_time_end(h, st);
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  return PGLD_OK;
}

extern "C" int pgld_pairs_by_bin(pgld_handle h, const uint32_t* planes, int32_t n_words,
                                 const double* pair_values, int64_t n_snp, const double* pos,
                                 const double* bins, int32_t n_bins, int64_t* bin_counts,
                                 double* values_out, void* stream) {
  using namespace pgld::dense;
  PGLD_REQUIRE(h, h != nullptr, "pgld_pairs_by_bin: NULL handle");
  PGLD_REQUIRE(h, n_bins >= 1 && n_bins <= pgld::kMaxBins, "pgld_pairs_by_bin: n_bins %d", n_bins);
  PGLD_REQUIRE(h, bins && bin_counts && n_snp >= 0, "pgld_pairs_by_bin: arguments");
  PGLD_REQUIRE(h, pair_values || (planes && n_words >= 1) || n_snp < 2,
               "pgld_pairs_by_bin: needs planes or pair values");
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  if (!values_out)
    for (int b = 0; b < n_bins; ++b) bin_counts[b] = 0;
  if (n_snp < 2) return PGLD_OK;
  PGLD_REQUIRE(h, pos != nullptr, "pgld_pairs_by_bin: NULL pos");
  // workspace: counters [n_bins], cursors [n_bins], bin ends [n_bins]
  void* ws = nullptr;
  int rc = pgld_workspace(h, (size_t)3 * n_bins * 8, &ws);
  if (rc) return rc;
  unsigned long long* cnt = (unsigned long long*)ws;
  unsigned long long* cur = cnt + n_bins;
  unsigned long long* end = cur + n_bins;
  std::vector<unsigned long long> host(2 * n_bins);
  if (values_out) {
    unsigned long long acc = 0;
    for (int b = 0; b < n_bins; ++b) {
      PGLD_REQUIRE(h, bin_counts[b] >= 0, "pgld_pairs_by_bin: negative count");
      host[b] = acc;
      acc += (unsigned long long)bin_counts[b];
      host[n_bins + b] = acc;
    }
    PGLD_CHECK_CUDA(h, cudaMemcpyAsync(cur, host.data(), (size_t)2 * n_bins * 8,
                                       cudaMemcpyHostToDevice, st));
    PGLD_CHECK_CUDA(h, cudaStreamSynchronize(st));  // host staging buffer is freed below
  } else {
    PGLD_CHECK_CUDA(h, cudaMemsetAsync(cnt, 0, (size_t)n_bins * 8, st));
  }
  const i64 nb = (n_snp + kT - 1) / kT;
  const size_t smem = sizeof(Smem);
  auto kern = pairs_by_bin_kernel;
  PGLD_CHECK_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = dense_grid(h, (const void*)kern, smem, nb * (nb + 1) / 2);
  pgld_time_begin(h, st);
  kern<<<grid, kThreads, smem, st>>>(planes, n_words, pair_values, n_snp, pos, bins, n_bins, cnt,
                                     cur, end, values_out, h->dev_status);
  pgld_time_end(h, st);
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  if (!values_out) {
    PGLD_CHECK_CUDA(h, cudaMemcpyAsync(host.data(), cnt, (size_t)n_bins * 8, cudaMemcpyDeviceToHost, st));
    PGLD_CHECK_CUDA(h, cudaStreamSynchronize(st));
    for (int b = 0; b < n_bins; ++b) bin_counts[b] = (int64_t)host[b];
  }
  return PGLD_OK;
}

extern "C" int pgld_segment_kth(pgld_handle h, const double* values, const int64_t* seg_offsets,
                                int32_t n_seg, const int64_t* targets, int32_t n_targets,
                                double* out, void* stream) {
  using namespace pgld::dense;
  PGLD_REQUIRE(h, h != nullptr, "pgld_segment_kth: NULL handle");
  PGLD_REQUIRE(h, n_seg >= 1 && n_targets >= 0 && seg_offsets && (n_targets == 0 || (targets && out)),
               "pgld_segment_kth: arguments");
  if (n_targets == 0) return PGLD_OK;
  PGLD_REQUIRE(h, values != nullptr, "pgld_segment_kth: NULL values");
  for (int s = 0; s < n_seg; ++s)
    PGLD_REQUIRE(h, seg_offsets[s] >= 0 && seg_offsets[s + 1] >= seg_offsets[s] &&
                        seg_offsets[s + 1] - seg_offsets[s] < (1ll << 32),
                 "pgld_segment_kth: segment %d offsets", s);
  for (int t = 0; t < n_targets; ++t) {
    const int64_t sg = targets[2 * t], rk = targets[2 * t + 1];
    PGLD_REQUIRE(h, sg >= 0 && sg < n_seg && rk >= 0 && rk < seg_offsets[sg + 1] - seg_offsets[sg],
                 "pgld_segment_kth: target %d (segment %lld, rank %lld) out of range", t,
                 (long long)sg, (long long)rk);
  }
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  const size_t off_b = (size_t)(n_seg + 1) * 8, tb = (size_t)n_targets * 8;
  void* ws = nullptr;
  int rc = pgld_workspace(h, off_b + 3 * tb + 256, &ws);
  if (rc) return rc;
  long long* d_off = (long long*)ws;
  long long* d_ts = d_off + (n_seg + 1);
  long long* d_tr = d_ts + n_targets;
  double* d_out = (double*)(d_tr + n_targets);
  std::vector<long long> ts(n_targets), tr(n_targets);
  for (int t = 0; t < n_targets; ++t) {
    ts[t] = targets[2 * t];
    tr[t] = targets[2 * t + 1];
  }
  PGLD_CHECK_CUDA(h, cudaMemcpyAsync(d_off, seg_offsets, off_b, cudaMemcpyHostToDevice, st));
  PGLD_CHECK_CUDA(h, cudaMemcpyAsync(d_ts, ts.data(), tb, cudaMemcpyHostToDevice, st));
  PGLD_CHECK_CUDA(h, cudaMemcpyAsync(d_tr, tr.data(), tb, cudaMemcpyHostToDevice, st));
  segment_kth_kernel<<<n_targets, 256, 0, st>>>(values, d_off, d_ts, d_tr, d_out);
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  PGLD_CHECK_CUDA(h, cudaMemcpyAsync(out, d_out, tb, cudaMemcpyDeviceToHost, st));
  PGLD_CHECK_CUDA(h, cudaStreamSynchronize(st));
  return PGLD_OK;
}
