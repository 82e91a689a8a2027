// tma.cuh — tiled bulk-tensor loads (TMA) into shared memory with mbarrier
// completion, as inline PTX for sm_100-class GPUs, and the host-side tensor
// map encoder.  Only loads from this GPU's own global memory into the
// issuing CTA's shared memory; no cluster multicast.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gm {

// Error bits that kernels record in a device word instead of trapping
// (read with kernel_error_flags()).
constexpr unsigned int kErrTmaTimeout = 1u;  // an mbarrier wait for a TMA tile ran out of polls

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  // make the initialised barrier visible to the async (TMA) proxy
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// The calling thread arrives once and announces `bytes` of transactions.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits for phase `parity` of the barrier, giving up after `polls` tries
// (false).  Never spins without bound.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t polls) {
  for (uint32_t i = 0; i < polls; i++) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i >= 32) __nanosleep(64);
  }
  return false;
}

// 3-D tiled load of one box of `map` at element coordinates (c0, c1, c2)
// (c0 innermost) into shared memory at `dst` (128-byte aligned); completion
// is counted on `bar` in bytes.  Out-of-range elements are filled with zeros.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_prefetch_map(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Host: looks up the driver's tensor-map encoder (once per process; call
// before any stream capture).
void tma_init();
// Host: a 3-D tensor map over a dense x-fastest field of `elem_bytes`-byte
// unsigned integers with extents (nx, ny, nz), read in boxes of
// (bx, by, bz) elements.  Returns false when the driver refuses it (the
// caller then loads the tile without TMA).
bool encode_tensor_map_3d(CUtensorMap* map, const void* base, int elem_bytes, int nx, int ny, int nz, int bx, int by,
                          int bz);

}  // namespace gm
