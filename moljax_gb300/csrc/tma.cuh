// Tensor-memory-accelerator (TMA) tile loads into shared memory with an mbarrier
// (sm_90+ PTX, used on sm_103a): host-side tensor maps of 2D FP32 arrays and the
// device-side barrier / bulk-copy helpers.  Every wait is bounded: a wait that runs
// out records an error word and the caller skips the data instead of hanging.
#pragma once

#include <cuda.h>  // CUtensorMap and its enums (types only: the encoder comes from the runtime)

#include "common.cuh"

namespace mjx {

// 2D tensor map of FP32 data: rows of `inner` floats, `rows` rows, `row_bytes` apart
// (a multiple of 16), boxes of box_inner floats (box_inner * 4 a multiple of 16) by
// box_rows rows (<= 256).  base must be 16-byte aligned.
mjx_status make_tmap_2d_f32(CUtensorMap* map, const void* base, unsigned long long inner, unsigned long long rows,
                            unsigned long long row_bytes, unsigned box_inner, unsigned box_rows);

// 3D tensor map of FP32 data [nz][ny][nx] (rows nx floats, planes ny rows; nx * 4 a
// multiple of 16), boxes of box_x x box_y x 1 (box_x * 4 a multiple of 16, box sides <= 256).
mjx_status make_tmap_3d_f32(CUtensorMap* map, const void* base, unsigned long long nx, unsigned long long ny,
                            unsigned long long nz, unsigned box_x, unsigned box_y);

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  // make the initialisation visible to the async (TMA) proxy
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// one 2D box at element coordinates (x, y) of the map into shared memory dst
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// one 3D box at element coordinates (x, y, z) of the map into shared memory dst
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z),
        "r"(smem_u32(bar))
      : "memory");
}

// Waits for phase `parity` of the barrier to complete, at most max_tries polls
// (each poll may itself suspend for a hardware-defined time); false when it ran out.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int max_tries) {
  for (int i = 0; i < max_tries; ++i) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

}  // namespace mjx
