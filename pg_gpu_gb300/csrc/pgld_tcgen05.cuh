// Shared tcgen05 / TMA / mbarrier plumbing of the tensor-core kernels
// (sm_103a): PTX wrappers, the control block with bounded waits, and the
// host-side TMA tensor-map encoding of K-major E4M3 operand matrices
// (128-row x 128-byte boxes, 128-byte swizzle).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <mutex>

#include "pgld_internal.cuh"

namespace pgld {
namespace tc {

constexpr int kRows = 128;          // rows of an MMA operand tile (M = N = 128)
constexpr int kKChunk = 128;        // bytes (= E4M3 elements) of K per stage
constexpr int kBoxBytes = kRows * kKChunk;  // 16 KB
constexpr int kStageBytes = 2 * kBoxBytes;  // A + B
constexpr uint32_t kOne = 0x38;     // E4M3 1.0
constexpr long long kSpinLimit = 1ll << 26;

// instruction descriptor: D f32, A/B E4M3, both K-major, N = 128, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (0u << 7) | (0u << 10) | ((128u >> 3) << 17) |
                            ((128u >> 4) << 24);

// ---------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
// try_wait that may suspend the thread for up to ns nanoseconds; the thread
// resumes as soon as the phase completes
__device__ __forceinline__ bool mbar_try_for(uint64_t* b, uint32_t parity, uint32_t ns) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity), "r"(ns)
      : "memory");
  return ok != 0;
}
// bounded wait: false once ~2 s of SM clock passed or another role aborted.
// Each poll may suspend the thread until the phase completes (or 20 us pass).
constexpr long long kWaitCycles = 4000000000ll;
constexpr uint32_t kSuspendNs = 20000;
// (limit: SM clock cycles before giving up; kWaitCycles unless a launch
// shortens it)
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* abort_flag,
                                          long long limit = kWaitCycles) {
  const long long t0 = clock64();
  for (long long k = 0; k < kSpinLimit; ++k) {
    if (mbar_try_for(b, parity, kSuspendNs)) return true;
    if (*abort_flag || clock64() - t0 > limit) return false;
  }
  return false;
}
// non-blocking probe of a phase
__device__ __forceinline__ bool mbar_test(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded polling wait for the single producer / MMA threads, whose stages
// are short: reacts to a completed phase within a few cycles (no suspension);
// false once `limit` cycles of SM clock passed or another role aborted
__device__ __forceinline__ bool mbar_wait_poll(uint64_t* b, uint32_t parity,
                                               volatile int* abort_flag,
                                               long long limit = kWaitCycles) {
  const long long t0 = clock64();
  for (long long k = 0; k < kSpinLimit; ++k) {
    if (mbar_test(b, parity)) return true;
    if ((k & 63) == 63 && (*abort_flag || clock64() - t0 > limit)) return false;
  }
  return false;
}
// bounded polling wait that naps ~32 ns between probes, so that a waiting
// producer / MMA thread leaves the issue slots of its sub-partition to the
// epilogue warps there; false once `limit` cycles passed or another role
// aborted
#ifndef PGLD_NAP_NS
#define PGLD_NAP_NS 32
#endif
__device__ __forceinline__ bool mbar_wait_nap(uint64_t* b, uint32_t parity,
                                              volatile int* abort_flag,
                                              long long limit = kWaitCycles) {
  const long long t0 = clock64();
  for (long long k = 0; k < kSpinLimit; ++k) {
    if (mbar_test(b, parity)) return true;
    __nanosleep(PGLD_NAP_NS);
    if ((k & 15) == 15 && (*abort_flag || clock64() - t0 > limit)) return false;
  }
  return false;
}
// the wait of a single producer / MMA-issuer thread: try_wait suspends the
// thread until the phase completes or a hardware time limit passes, so the
// waiting thread takes few issue slots from the epilogue warps of its
// sub-partition (PGLD_ROLE_WAIT 0: polling test_wait, mbar_wait_poll);
// false once `limit` cycles passed or another role aborted
#ifndef PGLD_ROLE_WAIT
#define PGLD_ROLE_WAIT 1
#endif
__device__ __forceinline__ bool mbar_wait_role(uint64_t* b, uint32_t parity,
                                               volatile int* abort_flag,
                                               long long limit = kWaitCycles) {
#if PGLD_ROLE_WAIT
  const long long t0 = clock64();
  for (long long k = 0; k < kSpinLimit; ++k) {
    if (mbar_try_for(b, parity, kSuspendNs)) return true;
    if ((k & 7) == 7 && (*abort_flag || clock64() - t0 > limit)) return false;
  }
  return false;
#else
  return mbar_wait_poll(b, parity, abort_flag, limit);
#endif
}
// drain wait: bounded by time only
__device__ __forceinline__ void mbar_wait_drain(uint64_t* b, uint32_t parity) {
  const long long t0 = clock64();
  for (long long k = 0; k < kSpinLimit; ++k) {
    if (mbar_try_for(b, parity, kSuspendNs)) return;
    if (clock64() - t0 > kWaitCycles) return;
  }
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x,
                                            int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%3, %4}], [%2];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  // K-major, 128-byte swizzle: SBO = 1024 B (8 rows x 128 B), LBO unused (1),
  // descriptor version 1 (bits 46-47), layout SWIZZLE_128B = 2 (bits 61-63)
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
__device__ __forceinline__ void mma_f8(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// 16 lanes x 4 x 256 bits: thread t gets lane (t / 4) and lane (8 + t / 4) of
// the 16, columns 2 (t % 4) and 2 (t % 4) + 1 of each 8-column repetition:
// r[4k .. 4k + 3] = (lane t/4, col 8k + 2(t%4)), (lane t/4, col + 1),
// (lane 8 + t/4, col 8k + 2(t%4)), (lane 8 + t/4, col + 1)
__device__ __forceinline__ void tmem_ld16x256_x4(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.16x256b.x4.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// bulk copy of `bytes` (a multiple of 16) from shared to global memory, both
// addresses 16-byte aligned, in the issuing thread's current bulk async-group
__device__ __forceinline__ void bulk_store(void* gdst, const void* ssrc, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst),
               "r"(smem_u32(ssrc)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// the thread's bulk groups but the newest N have read their shared memory
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
// every bulk group of the thread has completed
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}
// shared-memory writes of this thread visible to the async proxy (bulk copies)
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// streaming (evict-first) global stores of per-pair outputs under a
// predicate, without a branch around them; global-space stores cannot alias
// shared-memory loads, so later loads may be scheduled ahead of them
__device__ __forceinline__ void st_cs_if(bool p, int32_t* ptr, int v) {
  asm volatile(
      "{\n .reg .pred q;\n setp.ne.b32 q, %0, 0;\n @q st.global.cs.b32 [%1], %2;\n}" ::"r"(
          (int)p),
      "l"(ptr), "r"(v));
}
__device__ __forceinline__ void st_cs_if(bool p, float4* ptr, float4 v) {
  asm volatile(
      "{\n .reg .pred q;\n setp.ne.b32 q, %0, 0;\n"
      " @q st.global.cs.v4.f32 [%1], {%2, %3, %4, %5};\n}" ::"r"((int)p),
      "l"(ptr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w));
}
__device__ __forceinline__ void st_cs_if(bool p, int4* ptr, int4 v) {
  asm volatile(
      "{\n .reg .pred q;\n setp.ne.b32 q, %0, 0;\n"
      " @q st.global.cs.v4.b32 [%1], {%2, %3, %4, %5};\n}" ::"r"((int)p),
      "l"(ptr), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w));
}

struct Ctrl {
  uint64_t full[8], empty[8], tfull[2], tempty[2], drain;
  uint32_t tmem_base;
  int abort_flag;
  int produced, consumed;
  uint32_t unit_next[4];  // the next work unit of each lane quarter (dynamic epilogue order)
};

__device__ __forceinline__ void set_abort(Ctrl* c, int32_t* status, int code) {
  if (status) atomicCAS(status, 0, code);
  *(volatile int*)&c->abort_flag = 1;
}

}  // namespace tc
}  // namespace pgld

namespace pgld {
namespace tchost {

inline PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
  });
  return fn;
}

inline int get_encode(pgld_context* h) {
  if (!encode_fn())
    return pgld_fail(h, PGLD_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
  return PGLD_OK;
}

// rows x k_pad bytes, row-major, k_pad a multiple of 128; boxes of box_rows
// rows x 128 bytes
inline int make_map(pgld_context* h, CUtensorMap* map, const void* base, long long rows,
                    int k_pad, int box_rows = pgld::tc::kRows) {
  cuuint64_t dims[2] = {(cuuint64_t)k_pad, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)k_pad};
  cuuint32_t box[2] = {(cuuint32_t)pgld::tc::kKChunk, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims,
                           strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return pgld_fail(h, PGLD_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return PGLD_OK;
}

}  // namespace tchost
}  // namespace pgld
