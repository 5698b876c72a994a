// Device helpers shared by the sky-loop and td-amplitude kernels (sm_103a).
//
// Bulk copies global -> shared use the TMA engine (cp.async.bulk) completing
// on an mbarrier; every wait on an mbarrier or on a flag written by another
// CTA is bounded by the global nanosecond timer so that a kernel can never
// hang the GPU: on expiry it records PGW_ERR_TIMEOUT and returns.
#pragma once

#include <cstdint>

#include "../../include/pycwb_gb300.h"

namespace pgw {

// One second: the longest any kernel waits for a copy or for another CTA.
constexpr uint64_t kWaitLimitNs = 1000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (TMA) accesses to the same shared memory.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// 1-D TMA bulk copy; dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void tma_bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                             uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for phase `parity` of `bar` to complete; false after kWaitLimitNs.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > kWaitLimitNs) return false;
  }
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Spins (with back-off) until *flag != 0; false after kWaitLimitNs.
__device__ __forceinline__ bool wait_flag_bounded(const int* flag) {
  if (ld_acquire(flag)) return true;
  const uint64_t t0 = global_ns();
  unsigned ns = 32;
  while (!ld_acquire(flag)) {
    if (global_ns() - t0 > kWaitLimitNs) return false;
    __nanosleep(ns);
    if (ns < 1024) ns <<= 1;
  }
  return true;
}

__device__ __forceinline__ void flag_error(int* status, int code) {
  atomicOr(status, 1 << code);
}

__device__ __forceinline__ unsigned long long shfl_xor_u64(unsigned long long v, int o,
                                                          unsigned mask = 0xffffffffu) {
  unsigned lo = static_cast<unsigned>(v), hi = static_cast<unsigned>(v >> 32);
  lo = __shfl_xor_sync(mask, lo, o);
  hi = __shfl_xor_sync(mask, hi, o);
  return (static_cast<unsigned long long>(hi) << 32) | lo;
}

}  // namespace pgw
