// srs_cluster.cuh — shared-memory / distributed-shared-memory access and the
// per-step barrier of the persistent cluster kernels (inline PTX, sm_90+).
#pragma once
#include <cstdint>

namespace srs {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint32_t map_rank(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ float4 ld_dsmem_f4(uint32_t addr) {
  float4 v;
  asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(addr));
  return v;
}
__device__ __forceinline__ int32_t ld_dsmem_s32(uint32_t addr) {
  int32_t v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(addr));
  return v;
}
__device__ __forceinline__ float4 ld_smem_f4(uint32_t addr) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(addr));
  return v;
}
__device__ __forceinline__ void cluster_arrive_wait() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Bulk prefetch of a global range into L2 (address 16-byte aligned, size a
// multiple of 16 bytes).
__device__ __forceinline__ void l2_prefetch(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Bulk prefetch into L2 of [p, p + bytes) within an array that starts on a
// 16-byte boundary: the span is trimmed inward to 16-byte boundaries.
__device__ __forceinline__ void prefetch_span(const void* p, size_t bytes) {
  const uintptr_t b0 = ((uintptr_t)p + 15) & ~(uintptr_t)15;
  const uintptr_t b1 = ((uintptr_t)p + bytes) & ~(uintptr_t)15;
  if (b1 > b0) l2_prefetch((const void*)b0, (uint32_t)(b1 - b0));
}

// mbarrier and bulk asynchronous copies (global -> this CTA's shared memory).
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// dst and src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// Orders this CTA's generic-proxy shared-memory accesses before later
// asynchronous-proxy ones (bulk copies into the same buffers).
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Split cluster barrier: arrive (release) and wait (acquire) of one phase.
// With C == 1 the CTA barrier of the caller orders everything.
template <int C>
__device__ __forceinline__ void cl_arrive() {
  if constexpr (C > 1) asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
template <int C>
__device__ __forceinline__ void cl_wait() {
  if constexpr (C > 1) asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <int C>
__device__ __forceinline__ void step_barrier() {
  if constexpr (C == 1) {
    __syncthreads();
  } else {
    cluster_arrive_wait();
  }
}

}  // namespace srs
