// sbm_async.cuh -- inline-PTX helpers of the asynchronous copies shared by
// the TMA-staged kernels (sbm_tma.cu, sbm_net.cu): shared-memory addresses,
// mbarriers (init, expect_tx, bounded parity waits), 3-D tensor-map loads
// (cp.async.bulk.tensor) and per-thread 4-byte cp.async copies, plus the
// host-side builder of a 3-D tensor map over an FP32-layout buffer.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "sbm_internal.cuh"

namespace sbm {

__device__ __forceinline__ uint32_t saddr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* b, unsigned parity, unsigned tries) {
  for (unsigned n = 0; n < tries; ++n)
    if (mbar_try_wait(b, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(saddr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(saddr(bar))
      : "memory");
}

// Per-thread asynchronous 4-byte copy global -> shared (cp.async, cached in
// L1), its group commit and the wait for all of the thread's groups.
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(saddr(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// 3-D tensor map over an FP32-layout buffer (base = allocation start,
// 16-byte aligned: element (i, j, k) at coordinates (i + kOff32, j, k)) with
// boxes of bx x by x bz floats (sbm_tma.cu).
bool make_map_box(CUtensorMap* m, const float* base, const Geo& g32, int bx, int by, int bz);

}  // namespace sbm
