// libpgld: handle, argument checks, bit-plane packing, pair-list counting,
// statistic finalisation and distance-band pair enumeration.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "pgld_internal.cuh"
#include "pgld_scan.cuh"
#include "pgld_band.cuh"

using pgld::i64;

static thread_local std::string g_last_error;

int pgld_fail(pgld_context* h, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  if (h) h->err = buf;
  return code;
}

int pgld_cuda_fail(pgld_context* h, cudaError_t e, const char* what) {
  return pgld_fail(h, PGLD_ERR_CUDA, "CUDA error %s (%d) in %s", cudaGetErrorString(e), (int)e,
                   what);
}

int pgld_workspace(pgld_context* h, size_t bytes, void** out) {
  bytes = (bytes + 255) & ~size_t(255);
  if (bytes > h->ws_bytes) {
    if (h->ws) {
      PGLD_CHECK_CUDA(h, cudaDeviceSynchronize());
      PGLD_CHECK_CUDA(h, cudaFree(h->ws));
      h->ws = nullptr;
      h->ws_bytes = 0;
    }
    size_t want = std::max(bytes, size_t(1) << 20);
    cudaError_t e = cudaMalloc(&h->ws, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return pgld_fail(h, PGLD_ERR_NO_MEMORY, "workspace of %zu bytes: %s", want,
                       cudaGetErrorString(e));
    }
    h->ws_bytes = want;
  }
  *out = h->ws;
  return PGLD_OK;
}

// at most this many timed launches are kept between two reads
constexpr int kMaxTimedLaunches = 4096;

void pgld_time_begin(pgld_context* h, cudaStream_t st) {
  if (!h || !h->timing) return;
  if (h->tev_used + 2 > 2 * kMaxTimedLaunches) {
    h->tev_overflow = true;
    return;
  }
  while ((int)h->tev.size() < h->tev_used + 2) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      h->tev_overflow = true;
      return;
    }
    h->tev.push_back(e);
  }
  cudaEventRecord(h->tev[h->tev_used], st);
}

void pgld_time_end(pgld_context* h, cudaStream_t st) {
  if (!h || !h->timing || h->tev_overflow || h->tev_used + 2 > (int)h->tev.size()) return;
  cudaEventRecord(h->tev[h->tev_used + 1], st);
  h->tev_used += 2;
}

extern "C" int pgld_set_test_fault(pgld_handle h, int32_t kind) {
  if (!h) return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_set_test_fault: NULL handle");
  if (kind != 0 && kind != PGLD_TEST_FAULT_NO_COPIES)
    return pgld_fail(h, PGLD_ERR_INVALID_ARG, "pgld_set_test_fault: kind %d", kind);
  h->test_fault = kind;
  return PGLD_OK;
}

extern "C" int pgld_set_tc_config(pgld_handle h, int32_t layout, int32_t max_stages) {
  if (!h) return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_set_tc_config: NULL handle");
  if (layout < 0 || layout > 2 || max_stages < 0)
    return pgld_fail(h, PGLD_ERR_INVALID_ARG, "pgld_set_tc_config: layout %d, max_stages %d", layout,
                     max_stages);
  h->tc_layout = layout;
  h->tc_stages_cap = max_stages;
  return PGLD_OK;
}

extern "C" int pgld_set_kernel_timing(pgld_handle h, int32_t on) {
  if (!h) return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_set_kernel_timing: NULL handle");
  h->timing = on != 0;
  h->tev_used = 0;
  h->tev_overflow = false;
  return PGLD_OK;
}

extern "C" int pgld_kernel_times(pgld_handle h, float* ms_out, int32_t capacity, int32_t* n_out) {
  if (!h || !n_out || capacity < 0 || (capacity > 0 && !ms_out))
    return pgld_fail(h, PGLD_ERR_INVALID_ARG, "pgld_kernel_times: bad arguments");
  const int n = h->tev_used / 2;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(h->device);
  int rc = PGLD_OK;
  for (int k = 0; k < n && k < capacity; ++k) {
    cudaError_t e = cudaEventSynchronize(h->tev[2 * k + 1]);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, h->tev[2 * k], h->tev[2 * k + 1]);
    if (e != cudaSuccess) {
      rc = pgld_cuda_fail(h, e, "pgld_kernel_times");
      break;
    }
    ms_out[k] = ms;
  }
  cudaSetDevice(prev);
  *n_out = n;
  if (rc == PGLD_OK && h->tev_overflow)
    rc = pgld_fail(h, PGLD_ERR_TOO_LARGE, "pgld_kernel_times: more than %d launches since the last read",
                   kMaxTimedLaunches);
  h->tev_used = 0;
  h->tev_overflow = false;
  return rc;
}

// ---------------------------------------------------------------------------
// moments statistic table (ld_pipeline.py:357-457) as case terms
// ---------------------------------------------------------------------------
int pgld_n_stats(int P) {
  static const int n[5] = {0, 3, 15, 45, 105};
  return (P >= 1 && P <= 4) ? n[P] : 0;
}

// genotype kinds are the haplotype kinds shifted by this offset, except the
// two triple forms of pi2 (genotype_kernels.py:744-746)
constexpr int kGenoShift = PGLD_G_DD_II - PGLD_DD_II;

static void add_dd(std::vector<pgld_term>& t, int stat, double w, int a, int b) {
  pgld_term x{};
  x.stat = stat;
  x.weight = w;
  if (a == b) {
    x.kind = PGLD_DD_II;
    x.pops[0] = a;
  } else {
    x.kind = PGLD_DD_IJ;
    x.pops[0] = a;
    x.pops[1] = b;
  }
  t.push_back(x);
}

static void add_dz(std::vector<pgld_term>& t, int stat, double w, int i, int j, int k) {
  pgld_term x{};
  x.stat = stat;
  x.weight = w;
  if (i == j && j == k) {
    x.kind = PGLD_DZ_III;
    x.pops[0] = i;
  } else if (i == j) {
    x.kind = PGLD_DZ_IIJ;
    x.pops[0] = i;
    x.pops[1] = k;
  } else if (i == k) {
    x.kind = PGLD_DZ_IJI;
    x.pops[0] = i;
    x.pops[1] = j;
  } else if (j == k) {
    x.kind = PGLD_DZ_IJJ;
    x.pops[0] = i;
    x.pops[1] = j;
  } else {
    x.kind = PGLD_DZ_IJK;
    x.pops[0] = i;
    x.pops[1] = j;
    x.pops[2] = k;
  }
  t.push_back(x);
}

// case selection of haplotype_kernels.compute_all_pi2_hap (haplotype_kernels.py:463-486)
static void add_pi2(std::vector<pgld_term>& t, int stat, double w, int i, int j, int k, int l,
                    bool geno) {
  pgld_term x{};
  x.stat = stat;
  x.weight = w;
  int pp[4] = {i, j, k, l};
  std::map<int, int> cnt;
  for (int q : pp) cnt[q]++;
  int nu = (int)cnt.size(), mc = 0;
  for (auto& kv : cnt) mc = std::max(mc, kv.second);
  if (nu == 1) {
    x.kind = PGLD_PI2_IIII;
    x.pops[0] = i;
  } else if (mc == 3) {
    x.kind = PGLD_PI2_TRIPLE;
    for (auto& kv : cnt) {
      if (kv.second == 3) x.pops[0] = kv.first;
      if (kv.second == 1) x.pops[1] = kv.first;
    }
    if (geno) {
      x.kind = (i == x.pops[0] && j == x.pops[0]) ? PGLD_G_PI2_IIIJ : PGLD_G_PI2_IJII;
      t.push_back(x);
      return;
    }
  } else if (i == j && k == l) {
    x.kind = PGLD_PI2_IIKK;
    x.pops[0] = i;
    x.pops[1] = k;
  } else if (i == j) {
    x.kind = PGLD_PI2_IIKL;
    x.pops[0] = i;
    x.pops[1] = k;
    x.pops[2] = l;
  } else if (k == l) {
    x.kind = PGLD_PI2_IJKK;
    x.pops[0] = i;
    x.pops[1] = j;
    x.pops[2] = k;
  } else if ((i == k && j == l) || (i == l && j == k)) {
    x.kind = PGLD_PI2_IJIJ;
    x.pops[0] = i;
    x.pops[1] = j;
  } else if (nu == 3) {
    x.kind = PGLD_PI2_SHARED;
    int s, a, b;
    if (i == k) { s = i; a = j; b = l; }
    else if (i == l) { s = i; a = j; b = k; }
    else if (j == k) { s = j; a = i; b = l; }
    else { s = j; a = i; b = k; }
    x.pops[0] = s;
    x.pops[1] = a;
    x.pops[2] = b;
  } else {
    x.kind = PGLD_PI2_ALLDIFF;
    for (int q = 0; q < 4; ++q) x.pops[q] = pp[q];
  }
  if (geno) {
    static const int map[] = {0, 0, 0, 0, 0, 0, 0, PGLD_G_PI2_IIII, 0, PGLD_G_PI2_IIKK, 0,
                              PGLD_G_PI2_IIKL, PGLD_G_PI2_IJKK, PGLD_G_PI2_IJIJ,
                              PGLD_G_PI2_SHARED, PGLD_G_PI2_ALLDIFF};
    x.kind = map[x.kind];
  }
  t.push_back(x);
}

void pgld_build_spec_terms(int P, std::vector<pgld_term>& t, bool geno) {
  t.clear();
  int s = 0;
  for (int i = 0; i < P; ++i)
    for (int j = i; j < P; ++j) add_dd(t, s++, 1.0, i, j);
  for (int i = 0; i < P; ++i)
    for (int j = 0; j < P; ++j)
      for (int k = j; k < P; ++k) {
        if (j == k) {
          add_dz(t, s, 1.0, i, j, k);
        } else {
          add_dz(t, s, 0.5, i, j, k);
          add_dz(t, s, 0.5, i, k, j);
        }
        ++s;
      }
  for (int i = 0; i < P; ++i)
    for (int j = i; j < P; ++j)
      for (int k = i; k < P; ++k)
        for (int l = k; l < P; ++l) {
          if (k == i && i == l && j != i) continue;
          if (i == k && l < j) continue;
          if (i == j) {
            if (k == l) {
              if (i == k) {
                add_pi2(t, s, 1.0, i, j, k, l, geno);
              } else {
                add_pi2(t, s, 0.5, i, j, k, l, geno);
                add_pi2(t, s, 0.5, k, l, i, j, geno);
              }
            } else {
              add_pi2(t, s, 0.25, i, j, k, l, geno);
              add_pi2(t, s, 0.25, i, j, l, k, geno);
              add_pi2(t, s, 0.25, k, l, i, j, geno);
              add_pi2(t, s, 0.25, l, k, i, j, geno);
            }
          } else if (k == l) {
            add_pi2(t, s, 0.25, i, j, k, l, geno);
            add_pi2(t, s, 0.25, j, i, k, l, geno);
            add_pi2(t, s, 0.25, k, l, i, j, geno);
            add_pi2(t, s, 0.25, k, l, j, i, geno);
          } else {
            const int o[8][4] = {{i, j, k, l}, {i, j, l, k}, {j, i, k, l}, {j, i, l, k},
                                 {k, l, i, j}, {l, k, i, j}, {k, l, j, i}, {l, k, j, i}};
            for (auto& q : o) add_pi2(t, s, 0.125, q[0], q[1], q[2], q[3], geno);
          }
          ++s;
        }
  if (geno)
    for (auto& x : t)
      if (x.kind <= PGLD_DZ_IJK) x.kind += kGenoShift;
}

extern "C" int pgld_stat_terms(int32_t n_pops, pgld_term* out, int32_t capacity,
                               int32_t* n_terms_out, int32_t* n_stats_out) {
  if (n_pops < 1 || n_pops > PGLD_MAX_POPS)
    return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_stat_terms: n_pops %d", n_pops);
  std::vector<pgld_term> t;
  pgld_build_spec_terms(n_pops, t);
  if (n_terms_out) *n_terms_out = (int32_t)t.size();
  if (n_stats_out) *n_stats_out = pgld_n_stats(n_pops);
  if (out) {
    if (capacity < (int32_t)t.size())
      return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_stat_terms: capacity %d < %d",
                       capacity, (int)t.size());
    std::copy(t.begin(), t.end(), out);
  }
  return PGLD_OK;
}

// ---------------------------------------------------------------------------
// handle
// ---------------------------------------------------------------------------
extern "C" int pgld_version(void) { return 10000; }

extern "C" int pgld_create(int device, pgld_handle* out) {
  if (!out) return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_create: out is NULL");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return pgld_fail(nullptr, PGLD_ERR_CUDA, "pgld_create: no CUDA device (%s)",
                     cudaGetErrorString(e));
  }
  if (device < 0 || device >= n)
    return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_create: device %d of %d", device, n);
  pgld_context* h = new pgld_context();
  h->device = device;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(device);
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, device);
  h->n_sm = prop.multiProcessorCount;
  if (prop.major < 10) {
    delete h;
    cudaSetDevice(prev);
    return pgld_fail(nullptr, PGLD_ERR_UNSUPPORTED,
                     "pgld_create: device %d is sm_%d%d; this build targets sm_103a", device,
                     prop.major, prop.minor);
  }
  if (cudaMalloc(&h->dev_status, 64) != cudaSuccess || cudaMemset(h->dev_status, 0, 64) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    cudaSetDevice(prev);
    return pgld_fail(nullptr, PGLD_ERR_NO_MEMORY, "pgld_create: status word");
  }
  for (int P = 1; P <= PGLD_MAX_POPS; ++P) {
    std::vector<pgld_term> t;
    pgld_build_spec_terms(P, t);
    if (cudaMalloc(&h->spec_terms[P], t.size() * sizeof(pgld_term)) != cudaSuccess ||
        cudaMemcpy(h->spec_terms[P], t.data(), t.size() * sizeof(pgld_term),
                   cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      pgld_destroy(h);
      cudaSetDevice(prev);
      return pgld_fail(nullptr, PGLD_ERR_NO_MEMORY, "pgld_create: term tables");
    }
    h->spec_n_terms[P] = (int)t.size();
    h->spec_n_stats[P] = pgld_n_stats(P);
    pgld_build_spec_terms(P, t, true);
    if (cudaMalloc(&h->gspec_terms[P], t.size() * sizeof(pgld_term)) != cudaSuccess ||
        cudaMemcpy(h->gspec_terms[P], t.data(), t.size() * sizeof(pgld_term),
                   cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      pgld_destroy(h);
      cudaSetDevice(prev);
      return pgld_fail(nullptr, PGLD_ERR_NO_MEMORY, "pgld_create: genotype term tables");
    }
    h->gspec_n_terms[P] = (int)t.size();
  }
  cudaSetDevice(prev);
  *out = h;
  return PGLD_OK;
}

extern "C" int pgld_destroy(pgld_handle h) {
  if (!h) return PGLD_OK;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(h->device);
  cudaDeviceSynchronize();
  if (h->ws) cudaFree(h->ws);
  if (h->dev_status) cudaFree(h->dev_status);
  for (cudaEvent_t e : h->tev) cudaEventDestroy(e);
  for (int P = 0; P <= PGLD_MAX_POPS; ++P)
    if (h->spec_terms[P]) cudaFree(h->spec_terms[P]);
  for (int P = 0; P <= PGLD_MAX_POPS; ++P)
    if (h->gspec_terms[P]) cudaFree(h->gspec_terms[P]);
  cudaSetDevice(prev);
  delete h;
  return PGLD_OK;
}

extern "C" const char* pgld_last_error(pgld_handle h) {
  if (h && !h->err.empty()) return h->err.c_str();
  return g_last_error.c_str();
}

extern "C" int pgld_device_status(pgld_handle h, int32_t* code_out, void* stream) {
  if (!h || !code_out) return pgld_fail(h, PGLD_ERR_INVALID_ARG, "pgld_device_status: NULL");
  cudaStream_t st = (cudaStream_t)stream;
  int32_t v = 0;
  PGLD_CHECK_CUDA(h, cudaMemcpyAsync(&v, h->dev_status, 4, cudaMemcpyDeviceToHost, st));
  PGLD_CHECK_CUDA(h, cudaStreamSynchronize(st));
  PGLD_CHECK_CUDA(h, cudaMemsetAsync(h->dev_status, 0, 4, st));
  *code_out = v;
  return PGLD_OK;
}

// ---------------------------------------------------------------------------
// bit-plane packing
// ---------------------------------------------------------------------------
// block = one 32-haplotype word w x 512 SNPs.  The 32 rows x 512 bytes are
// staged in shared memory with coalesced 16-byte (VEC) or 1-byte loads -- the
// matrix may be pinned host memory read over the C2C link -- and each warp then
// turns 64 SNPs into words: lane r holds row r's byte and one ballot per plane
// gives the 32-bit word of a SNP.
constexpr int kPackSnps = 512;
constexpr int kPackPitch = kPackSnps + 4;  // row pitch: lanes of a column hit distinct banks
template <bool VEC>
__global__ void __launch_bounds__(256) pack_hap_kernel(const int8_t* __restrict__ hap, i64 ld,
                                                       i64 n_snp, const int32_t* __restrict__ rows,
                                                       int n_rows, int W, uint32_t* __restrict__ planes,
                                                       uint32_t* __restrict__ valid,
                                                       int32_t* __restrict__ flags) {
  __shared__ __align__(16) int8_t tile[32 * kPackPitch];
  const int w = blockIdx.y;
  const i64 s0 = (i64)blockIdx.x * kPackSnps;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // load: warp k stages rows 4k .. 4k+3 of the word
  for (int rr = 0; rr < 4; ++rr) {
    const int r = warp * 4 + rr;
    const int row = w * 32 + r;
    int8_t* dst = tile + r * kPackPitch;
    if (row >= n_rows) continue;
    const i64 hr = rows ? (i64)__ldg(rows + row) : (i64)row;
    const int8_t* src = hap + hr * ld + s0;
    if (VEC && s0 + kPackSnps <= n_snp) {
      const int4 v = __ldg(reinterpret_cast<const int4*>(src) + lane);
      // kPackPitch is not a multiple of 16: store as four words
      int* d4 = reinterpret_cast<int*>(dst + 16 * lane);
      d4[0] = v.x; d4[1] = v.y; d4[2] = v.z; d4[3] = v.w;
    } else {
      for (int k = lane; k < kPackSnps; k += 32)
        dst[k] = (s0 + k < n_snp) ? __ldg(src + k) : (int8_t)0;
    }
  }
  __syncthreads();
  // rows of the word that exist (the staged bytes of the others are not read
  // into any word); bytes past n_snp are staged as 0
  const int n_live = n_rows - w * 32;
  const uint32_t live = n_live >= 32 ? 0xffffffffu : ((1u << n_live) - 1u);
  const int8_t* mine = tile + lane * kPackPitch;
  uint32_t any_miss = 0, any_other = 0;
  for (int c = warp * 64; c < warp * 64 + 64; c += 32) {
    // 32 SNPs: lane k keeps the words of SNP c + k and stores them
    uint32_t mc = 0, mz = 0, mv = 0;
#pragma unroll 8
    for (int k = 0; k < 32; ++k) {
      const int v = (int)mine[c + k];
      const uint32_t cw = __ballot_sync(0xffffffffu, v == 1) & live;
      const uint32_t zw = __ballot_sync(0xffffffffu, v == 0) & live;
      const uint32_t vw = __ballot_sync(0xffffffffu, v >= 0) & live;
      any_miss |= __ballot_sync(0xffffffffu, v == -1);
      any_other |= __ballot_sync(0xffffffffu, (unsigned)(v + 1) > 2u);
      if (lane == k) {
        mc = cw;
        mz = zw;
        mv = vw;
      }
    }
    const i64 s = s0 + c + lane;
    if (s < n_snp) {
      planes[s * 2 * W + w] = mc;
      planes[s * 2 * W + W + w] = mz;
      if (valid) valid[s * W + w] = mv;
    }
  }
  if (lane == 0) {
    if (any_miss & live) atomicOr(flags, 1);
    if (any_other & live) atomicOr(flags + 1, 1);
  }
}

extern "C" int pgld_pack_haplotypes(pgld_handle h, const int8_t* hap, int64_t ld, int64_t n_snp,
                                    const int32_t* rows, int32_t n_rows, uint32_t* planes,
                                    uint32_t* valid, int32_t* flags, void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_pack_haplotypes: NULL handle");
  PGLD_REQUIRE(h, n_snp >= 0 && n_rows >= 0, "pgld_pack_haplotypes: negative size");
  PGLD_REQUIRE(h, planes && flags && (hap || n_snp == 0 || n_rows == 0),
               "pgld_pack_haplotypes: NULL buffer");
  PGLD_REQUIRE(h, ld >= n_snp, "pgld_pack_haplotypes: row stride %lld < n_snp %lld",
               (long long)ld, (long long)n_snp);
  int W = (n_rows + 31) / 32;
  if (n_snp == 0 || W == 0) return PGLD_OK;
  PGLD_REQUIRE(h, W <= 65535, "pgld_pack_haplotypes: too many rows");
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  dim3 grid((unsigned)((n_snp + kPackSnps - 1) / kPackSnps), (unsigned)W);
  const bool vec = ((uintptr_t)hap % 16 == 0) && (ld % 16 == 0);
  if (vec)
    pack_hap_kernel<true><<<grid, 256, 0, (cudaStream_t)stream>>>(hap, ld, n_snp, rows, n_rows, W,
                                                                  planes, valid, flags);
  else
    pack_hap_kernel<false><<<grid, 256, 0, (cudaStream_t)stream>>>(hap, ld, n_snp, rows, n_rows, W,
                                                                   planes, valid, flags);
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  return PGLD_OK;
}

// ---------------------------------------------------------------------------
// counts of listed pairs: a group of G lanes per pair, words strided by G
// ---------------------------------------------------------------------------
template <int G>
__global__ void __launch_bounds__(256) counts_pairs_kernel(
    const uint32_t* __restrict__ planes, const uint32_t* __restrict__ valid, int W, i64 n_snp,
    const int32_t* __restrict__ idx_i, const int32_t* __restrict__ idx_j, i64 n_pairs,
    i64 tri_m, int32_t* __restrict__ counts, i64 counts_ld, int32_t* __restrict__ n_valid,
    int32_t* __restrict__ status) {
  i64 g = ((i64)blockIdx.x * 256 + threadIdx.x) / G;
  int lane = threadIdx.x % G;
  i64 ngroups = (i64)gridDim.x * 256 / G;
  for (i64 k = g; k < n_pairs + (ngroups - (n_pairs % ngroups)) % ngroups; k += ngroups) {
    bool live = k < n_pairs;
    i64 i = 0, j = 0;
    if (live) {
      if (tri_m > 0) {
        // row-major upper triangle of an m x m matrix: row i starts at i*m - i(i+1)/2
        i64 lo = 0, hi = tri_m - 1;
        while (hi - lo > 1) {
          i64 mid = (lo + hi) >> 1;
          i64 st = mid * tri_m - mid * (mid + 1) / 2;
          if (st <= k) lo = mid; else hi = mid;
        }
        i = lo;
        j = k - (i * tri_m - i * (i + 1) / 2) + i + 1;
      } else {
        i = idx_i[k];
        j = idx_j[k];
      }
      if (i < 0 || j < 0 || i >= n_snp || j >= n_snp) {
        if (lane == 0) atomicCAS(status, 0, 1001);
        live = false;
      }
    }
    int n11 = 0, n10 = 0, n01 = 0, n00 = 0, nv = 0;
    if (live) {
      const uint32_t* pi = planes + i * 2 * W;
      const uint32_t* pj = planes + j * 2 * W;
      for (int w = lane; w < W; w += G) {
        uint32_t ci = __ldg(pi + w), zi = __ldg(pi + W + w);
        uint32_t cj = __ldg(pj + w), zj = __ldg(pj + W + w);
        n11 += __popc(ci & cj);
        n10 += __popc(ci & zj);
        n01 += __popc(zi & cj);
        n00 += __popc(zi & zj);
        if (valid) nv += __popc(__ldg(valid + i * W + w) & __ldg(valid + j * W + w));
      }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      n11 += __shfl_xor_sync(0xffffffffu, n11, o, G);
      n10 += __shfl_xor_sync(0xffffffffu, n10, o, G);
      n01 += __shfl_xor_sync(0xffffffffu, n01, o, G);
      n00 += __shfl_xor_sync(0xffffffffu, n00, o, G);
      nv += __shfl_xor_sync(0xffffffffu, nv, o, G);
    }
    if (live && lane == 0) {
      int32_t* c = counts + k * counts_ld;
      c[0] = n11; c[1] = n10; c[2] = n01; c[3] = n00;
      if (n_valid) n_valid[k] = valid ? nv : (n11 + n10 + n01 + n00);
    }
  }
}

static int launch_counts_pairs(pgld_context* h, const uint32_t* planes, const uint32_t* valid,
                               int W, i64 n_snp, const int32_t* ii, const int32_t* jj, i64 n,
                               i64 tri_m, int32_t* counts, i64 ld, int32_t* nv, cudaStream_t st) {
  int G = 1;
  while (G < W && G < 32) G <<= 1;
  i64 groups_needed = n;
  i64 blocks = (groups_needed * G + 255) / 256;
  blocks = std::min<i64>(std::max<i64>(blocks, 1), (i64)h->n_sm * 16);
#define PGLD_LAUNCH_CP(GG)                                                                     \
  counts_pairs_kernel<GG><<<(unsigned)blocks, 256, 0, st>>>(planes, valid, W, n_snp, ii, jj, n, \
                                                             tri_m, counts, ld, nv, h->dev_status)
  switch (G) {
    case 1: PGLD_LAUNCH_CP(1); break;
    case 2: PGLD_LAUNCH_CP(2); break;
    case 4: PGLD_LAUNCH_CP(4); break;
    case 8: PGLD_LAUNCH_CP(8); break;
    case 16: PGLD_LAUNCH_CP(16); break;
    default: PGLD_LAUNCH_CP(32); break;
  }
#undef PGLD_LAUNCH_CP
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  return PGLD_OK;
}

extern "C" int pgld_hap_counts_pairs(pgld_handle h, const uint32_t* planes, const uint32_t* valid,
                                     int32_t n_words, int64_t n_snp, const int32_t* idx_i,
                                     const int32_t* idx_j, int64_t n_pairs, int32_t* counts,
                                     int64_t counts_ld, int32_t* n_valid, void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_hap_counts_pairs: NULL handle");
  PGLD_REQUIRE(h, n_pairs >= 0 && n_words >= 0 && n_snp >= 0,
               "pgld_hap_counts_pairs: negative size");
  if (n_pairs == 0) return PGLD_OK;
  PGLD_REQUIRE(h, planes && idx_i && idx_j && counts, "pgld_hap_counts_pairs: NULL buffer");
  PGLD_REQUIRE(h, counts_ld >= 4, "pgld_hap_counts_pairs: counts_ld < 4");
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  return launch_counts_pairs(h, planes, valid, n_words, n_snp, idx_i, idx_j, n_pairs, 0, counts,
                             counts_ld, n_valid, (cudaStream_t)stream);
}

extern "C" int pgld_hap_tally(pgld_handle h, const uint32_t* planes, const uint32_t* valid,
                              int32_t n_words, int64_t n_snp, int32_t* counts, int32_t* n_valid,
                              void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_hap_tally: NULL handle");
  PGLD_REQUIRE(h, n_snp >= 0 && n_words >= 0, "pgld_hap_tally: negative size");
  i64 n_pairs = n_snp * (n_snp - 1) / 2;
  if (n_pairs <= 0) return PGLD_OK;
  PGLD_REQUIRE(h, planes && counts, "pgld_hap_tally: NULL buffer");
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  return launch_counts_pairs(h, planes, valid, n_words, n_snp, nullptr, nullptr, n_pairs, n_snp,
                             counts, 4, n_valid, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// statistic columns from per-pair counts
// ---------------------------------------------------------------------------
struct StatsArgs {
  const int32_t* counts[PGLD_MAX_POPS];
  i64 counts_ld[PGLD_MAX_POPS];
  const int32_t* nvalid[PGLD_MAX_POPS];
  i64 nvalid_ld[PGLD_MAX_POPS];
  int n_pops;
};

template <typename T>
__global__ void __launch_bounds__(256) stats_kernel(StatsArgs a, i64 n_pairs,
                                                    const pgld_term* __restrict__ terms,
                                                    int n_terms, T* __restrict__ out, i64 out_ld) {
  for (i64 k = (i64)blockIdx.x * 256 + threadIdx.x; k < n_pairs; k += (i64)gridDim.x * 256) {
    pgld::PopC P[PGLD_MAX_POPS];
    for (int p = 0; p < a.n_pops; ++p) {
      const int32_t* c = a.counts[p] + k * a.counts_ld[p];
      i64 c1 = c[0], c2 = c[1], c3 = c[2], c4 = c[3];
      i64 n = a.nvalid[p] ? (i64)a.nvalid[p][k * a.nvalid_ld[p]] : c1 + c2 + c3 + c4;
      P[p] = pgld::make_pop(c1, c2, c3, c4, n);
    }
    T* o = out + k * out_ld;
    int cur = -1;
    T acc = 0;
    int nt_in_stat = 0;
    for (int t = 0; t < n_terms; ++t) {
      pgld_term tm = terms[t];
      if (tm.stat != cur) {
        if (cur >= 0) o[cur] = acc;
        cur = tm.stat;
        acc = 0;
        nt_in_stat = 0;
      }
      T v;
      if (sizeof(T) == 8)
        v = (T)pgld::term_value_f64(tm.kind, tm.pops, P);
      else
        v = (T)pgld::term_value_f32(tm.kind, tm.pops, P);
      // single weight-1 term: the value itself (NaN passes through); else sum of weighted terms
      bool last_of_stat = (t + 1 == n_terms) || (terms[t + 1].stat != cur);
      if (nt_in_stat == 0 && last_of_stat && tm.weight == 1.0)
        acc = v;
      else
        acc = acc + (T)tm.weight * v;
      ++nt_in_stat;
    }
    if (cur >= 0) o[cur] = acc;
  }
}

extern "C" int pgld_hap_stats(pgld_handle h, const pgld_pair_counts* counts, int64_t n_pairs,
                              const pgld_term* terms, int32_t n_terms, int32_t n_stats, void* out,
                              int32_t out_dtype, int64_t out_ld, void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_hap_stats: NULL handle");
  PGLD_REQUIRE(h, counts && terms && n_terms > 0, "pgld_hap_stats: NULL argument");
  PGLD_REQUIRE(h, counts->n_pops >= 1 && counts->n_pops <= PGLD_MAX_POPS,
               "pgld_hap_stats: n_pops %d", counts->n_pops);
  PGLD_REQUIRE(h, n_pairs >= 0 && n_stats >= 1 && out_ld >= n_stats,
               "pgld_hap_stats: bad sizes");
  PGLD_REQUIRE(h, out_dtype == PGLD_F64 || out_dtype == PGLD_F32, "pgld_hap_stats: out_dtype");
  if (n_pairs == 0) return PGLD_OK;
  PGLD_REQUIRE(h, out != nullptr, "pgld_hap_stats: NULL out");
  StatsArgs a{};
  a.n_pops = counts->n_pops;
  for (int p = 0; p < a.n_pops; ++p) {
    PGLD_REQUIRE(h, counts->counts[p] && counts->counts_ld[p] >= 4,
                 "pgld_hap_stats: counts of population %d", p);
    a.counts[p] = counts->counts[p];
    a.counts_ld[p] = counts->counts_ld[p];
    a.nvalid[p] = counts->n_valid[p];
    a.nvalid_ld[p] = counts->nvalid_ld[p];
  }
  int prev = -1;
  for (int t = 0; t < n_terms; ++t) {
    const pgld_term& x = terms[t];
    PGLD_REQUIRE(h, x.stat >= 0 && x.stat < n_stats && x.stat >= prev,
                 "pgld_hap_stats: term %d stat column %d (columns must be non-decreasing)", t,
                 x.stat);
    prev = x.stat;
    PGLD_REQUIRE(h, x.kind >= 0 && x.kind <= PGLD_DPRIME, "pgld_hap_stats: term %d kind", t);
    for (int q = 0; q < 4; ++q)
      PGLD_REQUIRE(h, x.pops[q] >= 0 && x.pops[q] < a.n_pops,
                   "pgld_hap_stats: term %d population %d", t, x.pops[q]);
  }
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  void* ws = nullptr;
  int rc = pgld_workspace(h, n_terms * sizeof(pgld_term), &ws);
  if (rc) return rc;
  PGLD_CHECK_CUDA(h, cudaMemcpyAsync(ws, terms, n_terms * sizeof(pgld_term),
                                     cudaMemcpyHostToDevice, st));
  i64 blocks = std::min<i64>((n_pairs + 255) / 256, (i64)h->n_sm * 8);
  if (out_dtype == PGLD_F64)
    stats_kernel<double><<<(unsigned)blocks, 256, 0, st>>>(a, n_pairs, (const pgld_term*)ws,
                                                           n_terms, (double*)out, out_ld);
  else
    stats_kernel<float><<<(unsigned)blocks, 256, 0, st>>>(a, n_pairs, (const pgld_term*)ws,
                                                          n_terms, (float*)out, out_ld);
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  // the term table lives in the workspace: keep it alive until the kernel ran
  PGLD_CHECK_CUDA(h, cudaStreamSynchronize(st));
  return PGLD_OK;
}

// ---------------------------------------------------------------------------
// distance band: jmax, pair offsets, pair lists
// ---------------------------------------------------------------------------
__global__ void jmax_kernel(const double* __restrict__ pos, i64 n, double max_dist,
                            i64* __restrict__ per) {
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
    double lim = pos[i] + max_dist;
    i64 lo = i, hi = n;  // first index with pos > lim, searching (i, n]
    while (lo < hi) {
      i64 mid = (lo + hi) >> 1;
      if (pos[mid] <= lim) lo = mid + 1; else hi = mid;
    }
    i64 c = lo - i - 1;
    per[i] = c > 0 ? c : 0;
  }
}

int pgld_band_offsets(pgld_context* h, const double* pos, i64 n_snp, double max_dist, i64* off,
                      void* scratch, size_t scratch_bytes, cudaStream_t st) {
  // off[0..n] = exclusive prefix sum of the per-SNP pair counts
  unsigned blocks = (unsigned)std::min<i64>((n_snp + 255) / 256, (i64)h->n_sm * 8);
  jmax_kernel<<<std::max(1u, blocks), 256, 0, st>>>(pos, n_snp, max_dist, off);
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  return pgld::exclusive_scan_i64(h, off, n_snp, scratch, scratch_bytes, st);
}

extern "C" int pgld_count_pairs_within(pgld_handle h, const double* pos, int64_t n_snp,
                                       double max_dist, int64_t* n_pairs_out, int64_t* offsets,
                                       void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_count_pairs_within: NULL handle");
  PGLD_REQUIRE(h, n_pairs_out != nullptr && n_snp >= 0, "pgld_count_pairs_within: bad argument");
  PGLD_REQUIRE(h, max_dist >= 0, "pgld_count_pairs_within: negative max_dist");
  *n_pairs_out = 0;
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  if (n_snp < 2) {
    if (offsets) PGLD_CHECK_CUDA(h, cudaMemsetAsync(offsets, 0, (n_snp + 1) * 8, st));
    return PGLD_OK;
  }
  PGLD_REQUIRE(h, pos != nullptr, "pgld_count_pairs_within: NULL pos");
  size_t sbytes = pgld::scan_scratch_bytes(n_snp);
  void* ws = nullptr;
  int rc = pgld_workspace(h, (n_snp + 1) * 8 + sbytes, &ws);
  if (rc) return rc;
  i64* off = offsets ? (i64*)offsets : (i64*)ws;
  rc = pgld_band_offsets(h, pos, n_snp, max_dist, off, (char*)ws + (n_snp + 1) * 8, sbytes, st);
  if (rc) return rc;
  i64 tot = 0;
  PGLD_CHECK_CUDA(h, cudaMemcpyAsync(&tot, off + n_snp, 8, cudaMemcpyDeviceToHost, st));
  PGLD_CHECK_CUDA(h, cudaStreamSynchronize(st));
  *n_pairs_out = tot;
  return PGLD_OK;
}

// one warp per anchor SNP i in [i_begin, i_end) writes its row of pairs
__global__ void pairs_rows_kernel(const i64* __restrict__ off, i64 i_begin, i64 i_end,
                                  int32_t* __restrict__ ii, int32_t* __restrict__ jj) {
  int lane = threadIdx.x & 31;
  i64 warp = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  i64 nw = ((i64)gridDim.x * blockDim.x) >> 5;
  const i64 base = off[i_begin];
  for (i64 i = i_begin + warp; i < i_end; i += nw) {
    i64 a = off[i], b = off[i + 1];
    for (i64 k = a + lane; k < b; k += 32) {
      ii[k - base] = (int32_t)i;
      jj[k - base] = (int32_t)(i + 1 + (k - a));
    }
  }
}

extern "C" int pgld_pairs_within(pgld_handle h, const double* pos, int64_t n_snp, double max_dist,
                                 int64_t i_begin, int64_t i_end, int32_t* idx_i, int32_t* idx_j,
                                 int64_t n_pairs, void* stream) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_pairs_within: NULL handle");
  PGLD_REQUIRE(h, n_snp >= 0 && n_pairs >= 0, "pgld_pairs_within: negative size");
  PGLD_REQUIRE(h, 0 <= i_begin && i_begin <= i_end && i_end <= n_snp,
               "pgld_pairs_within: anchor range [%lld, %lld) outside [0, %lld)",
               (long long)i_begin, (long long)i_end, (long long)n_snp);
  PGLD_REQUIRE(h, max_dist >= 0, "pgld_pairs_within: negative max_dist");
  if (n_snp < 2 || i_begin == i_end) {
    PGLD_REQUIRE(h, n_pairs == 0, "pgld_pairs_within: capacity %lld for an empty range",
                 (long long)n_pairs);
    return PGLD_OK;
  }
  PGLD_REQUIRE(h, pos != nullptr, "pgld_pairs_within: NULL pos");
  PGLD_REQUIRE(h, n_snp < (int64_t(1) << 31), "pgld_pairs_within: n_snp exceeds int32 indices");
  PGLD_CHECK_CUDA(h, cudaSetDevice(h->device));
  cudaStream_t st = (cudaStream_t)stream;
  size_t sbytes = pgld::scan_scratch_bytes(n_snp);
  void* ws = nullptr;
  int rc = pgld_workspace(h, (n_snp + 1) * 8 + sbytes, &ws);
  if (rc) return rc;
  i64* off = (i64*)ws;
  rc = pgld_band_offsets(h, pos, n_snp, max_dist, off, (char*)ws + (n_snp + 1) * 8, sbytes, st);
  if (rc) return rc;
  i64 lo = 0, hi = 0;
  PGLD_CHECK_CUDA(h, cudaMemcpyAsync(&lo, off + i_begin, 8, cudaMemcpyDeviceToHost, st));
  PGLD_CHECK_CUDA(h, cudaMemcpyAsync(&hi, off + i_end, 8, cudaMemcpyDeviceToHost, st));
  PGLD_CHECK_CUDA(h, cudaStreamSynchronize(st));
  if (hi - lo != n_pairs)
    return pgld_fail(h, PGLD_ERR_INVALID_ARG, "pgld_pairs_within: capacity %lld != %lld pairs",
                     (long long)n_pairs, (long long)(hi - lo));
  if (n_pairs == 0) return PGLD_OK;
  PGLD_REQUIRE(h, idx_i && idx_j, "pgld_pairs_within: NULL output");
  unsigned blocks =
      (unsigned)std::max<i64>(1, std::min<i64>(((i_end - i_begin) * 32 + 255) / 256, (i64)h->n_sm * 16));
  pairs_rows_kernel<<<blocks, 256, 0, st>>>(off, i_begin, i_end, idx_i, idx_j);
  PGLD_CHECK_CUDA(h, cudaGetLastError());
  // the offsets live in the workspace: finish before the next call reuses it
  PGLD_CHECK_CUDA(h, cudaStreamSynchronize(st));
  return PGLD_OK;
}

// ---------------------------------------------------------------------------
// locate_unlinked pruning (host): sliding windows of `size` variants advanced
// by `step`; within a window, for active variants i < j in order, j is
// dropped when r2[pair (i, j)] > threshold.  r2 holds the band pairs j - i <
// size in row order (row i at pair_off[i], j = i + 1 + k), as the band pair
// list of positions 0..n_snp-1 within size - 1.  Follows
// HaplotypeMatrix.locate_unlinked (haplotype_matrix.py:1172-1233), whose
// pruning also runs on the host.
// ---------------------------------------------------------------------------
extern "C" int pgld_prune_unlinked(pgld_handle h, const double* r2, const int64_t* pair_off,
                                   int64_t n_snp, int32_t size, int32_t step, double threshold,
                                   uint8_t* loc) {
  PGLD_REQUIRE(h, h != nullptr, "pgld_prune_unlinked: NULL handle");
  PGLD_REQUIRE(h, size >= 1 && step >= 1, "pgld_prune_unlinked: size %d, step %d", (int)size,
               (int)step);
  PGLD_REQUIRE(h, n_snp >= 0, "pgld_prune_unlinked: n_snp < 0");
  if (n_snp == 0) return PGLD_OK;
  PGLD_REQUIRE(h, pair_off && loc && (r2 || pair_off[n_snp] == 0),
               "pgld_prune_unlinked: NULL buffer");
  for (int64_t s = 0; s < n_snp; ++s) loc[s] = 1;
  std::vector<int64_t> act;
  act.reserve((size_t)size);
  for (int64_t ws = 0; ws < n_snp; ws += step) {
    const int64_t we = std::min<int64_t>(ws + size, n_snp);
    act.clear();
    for (int64_t s = ws; s < we; ++s)
      if (loc[s]) act.push_back(s);
    if (act.size() <= 1) continue;
    for (size_t a = 0; a < act.size(); ++a) {
      const int64_t i = act[a];
      if (!loc[i]) continue;
      const int64_t row = pair_off[i], row_n = pair_off[i + 1] - row;
      for (size_t b = a + 1; b < act.size(); ++b) {
        const int64_t j = act[b];
        if (!loc[j]) continue;
        PGLD_REQUIRE(h, j - i - 1 < row_n, "pgld_prune_unlinked: pair (%lld, %lld) not in the band",
                     (long long)i, (long long)j);
        if (r2[row + (j - i - 1)] > threshold) loc[j] = 0;
      }
    }
  }
  return PGLD_OK;
}
