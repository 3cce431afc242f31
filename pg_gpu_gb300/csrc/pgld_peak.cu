// Throughput of the tensor-core contraction this library runs on (sm_103a):
// tcgen05.mma.cta_group::1.kind::f8f6f4 with E4M3 operands, M = 128, K = 32,
// N = 64 / 128 / 256, float32 accumulators in TMEM -- the instruction of the
// tensor-core band kernels -- issued back to back by one thread per SM from
// two operand tiles resident in shared memory.  The measured rate is the
// denominator of the tensor-pipe roofline of those kernels.
//
// Operand bytes are 0 or E4M3 1.0 at random (half of each), as in a
// haplotype operand, so the data toggle like real tiles.  The one wait (the
// final commit) is bounded; on expiry the kernel records an error code,
// frees TMEM and returns.
#include <cuda_runtime.h>

#include "pgld_internal.cuh"
#include "pgld_tcgen05.cuh"

namespace pgld {
namespace peak {

using namespace pgld::tc;

constexpr int kThreads = 128;
constexpr uint32_t kCols = 256;  // TMEM columns allocated (largest N)

__device__ __forceinline__ void mma_f8_idesc(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                             uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}

__global__ void __launch_bounds__(kThreads, 1)
    mma_rate_kernel(long long n_mma, int n_cols, int32_t* status) {
  extern __shared__ unsigned char smem_dyn[];
  __shared__ uint64_t done;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  unsigned char* base = smem_dyn + ((1024 - (smem_u32(smem_dyn) & 1023)) & 1023);
  unsigned char* a_tile = base;          // 128 rows x 128 bytes
  unsigned char* b_tile = base + 16384;  // n_cols rows x 128 bytes
  const int bytes = 16384 + n_cols * 128;
  for (int x = 4 * threadIdx.x; x < bytes; x += 4 * kThreads) {
    uint32_t hsh = ((uint32_t)x + 7919u * blockIdx.x) * 2654435761u;
    hsh ^= hsh >> 15;
    hsh *= 2246822519u;
    uint32_t v = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if ((hsh >> (7 + 5 * q)) & 1u) v |= kOne << (8 * q);
    *reinterpret_cast<uint32_t*>(base + x) = v;
  }
  // the tensor cores read shared memory through the async proxy
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (threadIdx.x == 0) {
    mbar_init(&done, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  if (threadIdx.x == 0) {
    // D f32, A/B E4M3 K-major, N = n_cols, M = 128
    const uint32_t idesc = (1u << 4) | ((uint32_t)(n_cols >> 3) << 17) | ((128u >> 4) << 24);
    const uint64_t da = smem_desc(smem_u32(a_tile)), db = smem_desc(smem_u32(b_tile));
    for (long long k = 0; k < n_mma; ++k) {
      const uint64_t kk = (uint64_t)(2 * (k & 3));  // the four 32-byte K steps of a 128-byte row
      mma_f8_idesc(tmem, da + kk, db + kk, idesc, k != 0 ? 1u : 0u);
    }
    mma_commit(&done);
    if (!mbar_wait(&done, 0, &abort_flag)) atomicCAS(status, 0, 3201);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols)
                 : "memory");
}

}  // namespace peak
}  // namespace pgld

extern "C" int pgld_tc_mma_rate(pgld_handle h, int32_t n_cols, int64_t mmas_per_sm,
                                int32_t launches, float* ms_out, double* flops_out,
                                void* stream) {
  if (!h || !ms_out || !flops_out)
    return pgld_fail(h, PGLD_ERR_INVALID_ARG, "pgld_tc_mma_rate: NULL argument");
  PGLD_REQUIRE(h, n_cols == 64 || n_cols == 128 || n_cols == 256,
               "pgld_tc_mma_rate: n_cols must be 64, 128 or 256");
  // a launch issues at most 2^24 MMAs per SM (well under a second)
  PGLD_REQUIRE(h, mmas_per_sm >= 1 && mmas_per_sm <= (1ll << 24),
               "pgld_tc_mma_rate: mmas_per_sm out of [1, 2^24]");
  PGLD_REQUIRE(h, launches >= 1 && launches <= 10000, "pgld_tc_mma_rate: launches out of [1, 10000]");
  cudaStream_t st = (cudaStream_t)stream;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(h->device);
  // operands take at most 49 KB; 120 KB keeps one CTA (one MMA issuer) per SM
  const size_t smem = 120 * 1024;
  auto kern = pgld::peak::mma_rate_kernel;
  int rc = PGLD_OK;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaEventRecord(e0, st);
  for (int l = 0; e == cudaSuccess && l < launches; ++l) {
    kern<<<(unsigned)h->n_sm, pgld::peak::kThreads, smem, st>>>(mmas_per_sm, n_cols, h->dev_status);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(e1, st);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e != cudaSuccess) rc = pgld_cuda_fail(h, e, "pgld_tc_mma_rate");
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc == PGLD_OK) {
    int32_t code = 0;
    e = cudaMemcpy(&code, h->dev_status, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = pgld_cuda_fail(h, e, "pgld_tc_mma_rate status");
    else if (code != 0) {
      cudaMemset(h->dev_status, 0, 4);
      rc = pgld_fail(h, PGLD_ERR_TIMEOUT, "pgld_tc_mma_rate: device status %d", code);
    }
  }
  cudaSetDevice(prev);
  if (rc != PGLD_OK) return rc;
  *ms_out = ms;
  *flops_out = 2.0 * 128.0 * n_cols * 32.0 * (double)mmas_per_sm * h->n_sm * launches;
  return PGLD_OK;
}
