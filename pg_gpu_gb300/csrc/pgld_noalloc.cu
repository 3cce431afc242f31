// Distance-binned sums for callers that cannot allocate device memory.
//
// Same kernels as pgld_hap_binned_sums (plain form), but the tile work list
// and the prefix-sum partials live in one file-scope static device array
// instead of a handle's cudaMalloc'd workspace, and no handle is needed.
// Every GPU that loads the library holds that array (kNoAllocScratchBytes)
// until the process exits.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "pgld_band.cuh"
#include "pgld_internal.cuh"
#include "pgld_scan.cuh"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;  // 4 MiB
constexpr int kNoAllocMaxTerms = 512;                     // 354 terms for 4 populations
constexpr int kMaxDevices = 64;

// Scratch shared by every call on a device: tile work-list offsets followed by
// the scan partials.  Each call rewrites what it reads; calls that overlap on
// the GPU (other streams, other host threads) race on it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
// Constant moments term tables (1..4 populations) and a device status word.
static __device__ __align__(256) pgld_term g_noalloc_terms[PGLD_MAX_POPS][kNoAllocMaxTerms];
static __device__ __align__(256) int32_t g_noalloc_status[64];

struct DeviceSetup {
  bool ready = false;
  int n_sm = 0;
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
  pgld_term* terms = nullptr;        // device address of g_noalloc_terms
  int32_t* status = nullptr;         // device address of g_noalloc_status
  int n_terms[PGLD_MAX_POPS + 1] = {0};
};

std::mutex g_setup_mutex;
DeviceSetup g_setup[kMaxDevices];

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

size_t noalloc_bytes(long long n_blocks) {
  return align256((size_t)(n_blocks + 1) * 8) + pgld::scan_scratch_bytes(n_blocks);
}

// Once per device, with that device current: resolve the symbols' device
// addresses (host code cannot use the arrays' names as device pointers) and
// fill the term tables.  Allocates nothing.
int setup_device(int device, DeviceSetup** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  DeviceSetup& s = g_setup[device];
  if (s.ready) {
    *out = &s;
    return PGLD_OK;
  }
  int prev = 0;
  cudaError_t e = cudaGetDevice(&prev);
  if (e != cudaSuccess) return pgld_cuda_fail(nullptr, e, "cudaGetDevice");
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return pgld_cuda_fail(nullptr, e, "cudaSetDevice");
  int rc = PGLD_OK;
  do {
    e = cudaGetSymbolAddress((void**)&s.scratch, g_noalloc_scratch);
    if (e != cudaSuccess) { rc = pgld_cuda_fail(nullptr, e, "cudaGetSymbolAddress(scratch)"); break; }
    e = cudaGetSymbolAddress((void**)&s.terms, g_noalloc_terms);
    if (e != cudaSuccess) { rc = pgld_cuda_fail(nullptr, e, "cudaGetSymbolAddress(terms)"); break; }
    e = cudaGetSymbolAddress((void**)&s.status, g_noalloc_status);
    if (e != cudaSuccess) { rc = pgld_cuda_fail(nullptr, e, "cudaGetSymbolAddress(status)"); break; }
    e = cudaDeviceGetAttribute(&s.n_sm, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) { rc = pgld_cuda_fail(nullptr, e, "cudaDeviceGetAttribute"); break; }
    for (int P = 1; P <= PGLD_MAX_POPS; ++P) {
      std::vector<pgld_term> t;
      pgld_build_spec_terms(P, t);
      if ((int)t.size() > kNoAllocMaxTerms) {
        rc = pgld_fail(nullptr, PGLD_ERR_TOO_LARGE, "term table of %d populations", P);
        break;
      }
      e = cudaMemcpyToSymbol(g_noalloc_terms, t.data(), t.size() * sizeof(pgld_term),
                             (size_t)(P - 1) * kNoAllocMaxTerms * sizeof(pgld_term),
                             cudaMemcpyHostToDevice);
      if (e != cudaSuccess) { rc = pgld_cuda_fail(nullptr, e, "cudaMemcpyToSymbol(terms)"); break; }
      s.n_terms[P] = (int)t.size();
    }
  } while (0);
  cudaSetDevice(prev);
  if (rc != PGLD_OK) return rc;
  s.ready = true;
  *out = &s;
  return PGLD_OK;
}

}  // namespace

extern "C" int pgld_hap_binned_sums_noalloc(int device, const pgld_hap_panel* panel,
                                            const double* pos, double max_dist,
                                            const double* bin_coord, const double* bins,
                                            int32_t n_bins, double* sums, int64_t* pair_counts,
                                            void* stream) {
  int n_dev = 0;
  cudaError_t e = cudaGetDeviceCount(&n_dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return pgld_cuda_fail(nullptr, e, "pgld_hap_binned_sums_noalloc: cudaGetDeviceCount");
  }
  if (device < 0 || device >= n_dev || device >= kMaxDevices)
    return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_hap_binned_sums_noalloc: device %d",
                     device);
  if (!panel || panel->n_pops < 1 || panel->n_pops > PGLD_MAX_POPS || panel->n_snp < 0)
    return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_hap_binned_sums_noalloc: bad panel");
  for (int p = 0; p < panel->n_pops; ++p)
    if (panel->n_words[p] < 1 || (!panel->planes[p] && panel->n_snp > 0))
      return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG,
                       "pgld_hap_binned_sums_noalloc: population %d planes", p);
  if (n_bins < 1 || n_bins > pgld::kMaxBins || !bins || !sums)
    return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG,
                     "pgld_hap_binned_sums_noalloc: n_bins %d not in [1, %d] or NULL buffer",
                     n_bins, pgld::kMaxBins);
  if (!(max_dist >= 0))
    return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_hap_binned_sums_noalloc: max_dist");
  const long long n = panel->n_snp;
  const long long nb = (n + pgld::kTile - 1) / pgld::kTile;
  if (noalloc_bytes(nb) > kNoAllocScratchBytes) {
    long long max_snp = 0;
    for (long long b = (long long)(kNoAllocScratchBytes / 8); b > 0; --b)
      if (noalloc_bytes(b) <= kNoAllocScratchBytes) { max_snp = b * pgld::kTile; break; }
    return pgld_fail(nullptr, PGLD_ERR_TOO_LARGE,
                     "pgld_hap_binned_sums_noalloc: %lld SNPs need %zu bytes of scratch; the "
                     "static scratch holds %zu bytes (at most %lld SNPs per call)",
                     n, noalloc_bytes(nb), kNoAllocScratchBytes, max_snp);
  }
  DeviceSetup* s = nullptr;
  int rc = setup_device(device, &s);
  if (rc) return rc;
  int prev = 0;
  cudaGetDevice(&prev);
  if (prev != device && (e = cudaSetDevice(device)) != cudaSuccess)
    return pgld_cuda_fail(nullptr, e, "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  const int P = panel->n_pops;
  const int S = pgld_n_stats(P);
  // a stack context: no workspace, no term buffers of its own
  pgld_context ctx;
  ctx.device = device;
  ctx.n_sm = s->n_sm;
  ctx.dev_status = s->status;
  do {
    if ((e = cudaMemsetAsync(sums, 0, (size_t)n_bins * S * 8, st)) != cudaSuccess) break;
    if (pair_counts && (e = cudaMemsetAsync(pair_counts, 0, (size_t)n_bins * 8, st)) != cudaSuccess)
      break;
    if ((e = cudaMemsetAsync(s->status, 0, 4, st)) != cudaSuccess) break;
  } while (0);
  if (e != cudaSuccess) {
    rc = pgld_cuda_fail(nullptr, e, "pgld_hap_binned_sums_noalloc: memset");
  } else if (n >= 2) {
    if (!pos) {
      rc = pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_hap_binned_sums_noalloc: NULL pos");
    } else {
      long long* items = (long long*)s->scratch;
      unsigned char* scan = s->scratch + align256((size_t)(nb + 1) * 8);
      rc = pgld::band_schedule(&ctx, pos, n, max_dist, items, scan,
                               kNoAllocScratchBytes - align256((size_t)(nb + 1) * 8), st);
      if (rc == PGLD_OK) {
        pgld::BandArgs a{};
        a.status = s->status;
        a.n_pops = P;
        for (int p = 0; p < PGLD_MAX_POPS; ++p) {
          a.W[p] = p < P ? panel->n_words[p] : 0;
          a.planes[p] = p < P ? panel->planes[p] : nullptr;
          a.valid[p] = p < P ? panel->valid[p] : nullptr;
        }
        a.n_snp = n;
        a.nmax = 0;
        for (int p = 0; p < P; ++p) a.nmax = std::max(a.nmax, 32 * panel->n_words[p]);
        a.pos = pos;
        a.max_dist = max_dist;
        a.bcoord = bin_coord;
        a.bins = bins;
        a.n_bins = n_bins;
        a.item_off = items;
        a.n_blocks = nb;
        a.sums = sums;
        a.pair_counts = pair_counts;
        a.terms = s->terms + (size_t)(P - 1) * kNoAllocMaxTerms;
        a.n_terms = s->n_terms[P];
        a.n_stats = S;
        rc = pgld::launch_band_plain(&ctx, a, pgld::kModeBinned, st);
      }
    }
  }
  if (prev != device) cudaSetDevice(prev);
  return rc;
}

extern "C" int pgld_noalloc_status(int device, int32_t* code_out) {
  if (!code_out)
    return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_noalloc_status: NULL code_out");
  int n_dev = 0;
  cudaError_t e = cudaGetDeviceCount(&n_dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return pgld_cuda_fail(nullptr, e, "pgld_noalloc_status: cudaGetDeviceCount");
  }
  if (device < 0 || device >= n_dev || device >= kMaxDevices)
    return pgld_fail(nullptr, PGLD_ERR_INVALID_ARG, "pgld_noalloc_status: device %d", device);
  *code_out = 0;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_setup[device].ready) return PGLD_OK;  // no call has run on the device
  }
  int prev = 0;
  cudaGetDevice(&prev);
  if (prev != device && (e = cudaSetDevice(device)) != cudaSuccess)
    return pgld_cuda_fail(nullptr, e, "cudaSetDevice");
  int32_t v = 0;
  const int32_t zero = 0;
  // symbol copies: no allocation; they wait for the device's earlier work
  e = cudaMemcpyFromSymbol(&v, g_noalloc_status, sizeof(v));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_noalloc_status, &zero, sizeof(zero));
  if (prev != device) cudaSetDevice(prev);
  if (e != cudaSuccess) return pgld_cuda_fail(nullptr, e, "pgld_noalloc_status");
  *code_out = v;
  return PGLD_OK;
}
