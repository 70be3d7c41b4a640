// Tensor Memory Accelerator (TMA) helpers for sm_103a: mbarrier set-up, bounded waits
// and tiled bulk-tensor loads from global into shared memory (inline PTX).
//
// Every wait is bounded: after kWaitLimit unsuccessful try_wait probes the caller gets
// `false`, records kStatusTmaTimeout in the device status word and returns instead of
// hanging the GPU.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace convgpu {

constexpr unsigned kStatusTmaTimeout = 1u;
constexpr uint32_t kWaitLimit = 1u << 22;

// The device status word is followed by a second word, the dependency-wait limit: 0
// keeps each dependency wait's own probe limit; v > 0 limits every dependency wait (on a
// counter another CTA advances: plane dependencies of the L2-staged pass, the uneven work
// queue, the small-cube grid barriers) to v - 1 probes, so v = 1 makes them give up at
// once. It exists for tests of the failure path; waits for copies or MMAs in flight
// (mbarrier waits) never read it.
__device__ __forceinline__ uint32_t dep_wait_limit(const unsigned *status, uint32_t dflt) {
  if (!status) return dflt;
  const unsigned v = *reinterpret_cast<const volatile unsigned *>(status + 1);
  return v ? v - 1u : dflt;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// Makes the initialised barrier visible to the async (TMA) proxy.
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits for phase `parity` of the barrier, at most kWaitLimit probes.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  for (uint32_t i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Orders the async proxy's view of a 128-byte tensor map held in global memory after the
// generic writes that produced it (maps uploaded to device arrays).
__device__ __forceinline__ void tensormap_acquire(const CUtensorMap *map) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(map))
               : "memory");
}

// 2D tiled load of the box at (c0, c1) (c0 innermost).
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int c0, int c1, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}

// 3D tiled load of the box at coordinates (c0, c1, c2) (c0 innermost) into shared
// memory; completion is signalled on `bar` as transaction bytes.
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}

// Contiguous copy of `bytes` (a multiple of 16; both addresses 16-byte aligned) from global
// into shared memory; completion is signalled on `bar` as transaction bytes.
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(bar)
               : "memory");
}

}  // namespace convgpu
