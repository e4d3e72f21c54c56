// One-warp 1024-point FP32 transform (sm_103a).
//
// A 1024-point row transform held by one warp: lane l keeps the 32 elements l + 32 j in
// registers.  Four-step split 1024 = 32 x 32: a 32-point DFT per lane over j, the twiddles
// w^(l k1) (w = exp(-2 pi i/1024), from the transposed part of the plan's row table), one transpose through a 32 x 33 shared
// tile of the warp (only __syncwarp, no block barrier), and a second 32-point DFT per lane;
// element k1 + 32 k2 of the result ends in register k2 of lane k1, which is again the
// layout "lane = index mod 32", so the inverse transform's output feeds the pointwise work
// and the forward transform without any reordering.  The two-for-one packing of two real
// rows pairs index k with 1024 - k, which lives in lane (32 - l) mod 32: one shuffle each.
#pragma once

#include "fft.cuh"

namespace mjx {

// cos / sin of 2 pi k / 32, k = 0..15
static __constant__ const float kW32C[16] = {1.0f, 0.98078528040323044913f, 0.92387953251128675613f,
                                             0.83146961230254523708f, 0.70710678118654752440f, 0.55557023301960222474f,
                                             0.38268343236508977173f, 0.19509032201612826785f, 0.0f,
                                             -0.19509032201612826785f, -0.38268343236508977173f, -0.55557023301960222474f,
                                             -0.70710678118654752440f, -0.83146961230254523708f, -0.92387953251128675613f,
                                             -0.98078528040323044913f};
static __constant__ const float kW32S[16] = {0.0f, 0.19509032201612826785f, 0.38268343236508977173f,
                                             0.55557023301960222474f, 0.70710678118654752440f, 0.83146961230254523708f,
                                             0.92387953251128675613f, 0.98078528040323044913f, 1.0f,
                                             0.98078528040323044913f, 0.92387953251128675613f, 0.83146961230254523708f,
                                             0.70710678118654752440f, 0.55557023301960222474f, 0.38268343236508977173f,
                                             0.19509032201612826785f};

// 32-point DFT in registers, natural order in and out: 16-point DFTs of the even and odd
// samples and one radix-2 step with w32^k
template <bool INV>
__device__ __forceinline__ void dft32(float2 (&a)[32]) {
  float2 e[16], o[16];
#pragma unroll
  for (int m = 0; m < 16; ++m) { e[m] = a[2 * m]; o[m] = a[2 * m + 1]; }
  dft16<INV>(e);
  dft16<INV>(o);
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const float c = kW32C[k], sn = INV ? kW32S[k] : -kW32S[k];
    const float2 t = mk<float2>(o[k].x * c - o[k].y * sn, o[k].x * sn + o[k].y * c);
    a[k] = cadd(e[k], t);
    a[k + 16] = csub(e[k], t);
  }
}

template <bool INV>
__device__ __forceinline__ void wfft1024(float2 (&z)[32], float2* tile, const float2* __restrict__ tw, int lane) {
  dft32<INV>(z);
  // w^(lane k1) from the transposed copy that FP32 plans of 1024-point rows append to
  // their twiddle table (tw[1024 + 32 k1 + lane] == tw[lane k1]): one contiguous run per k1
#pragma unroll
  for (int k1 = 1; k1 < 32; ++k1) {
    const float2 w = __ldg(&tw[1024 + 32 * k1 + lane]);
    z[k1] = INV ? cmulc(z[k1], w) : cmul(z[k1], w);
  }
#pragma unroll
  for (int k1 = 0; k1 < 32; ++k1) tile[k1 * 33 + lane] = z[k1];
  __syncwarp();
#pragma unroll
  for (int j2 = 0; j2 < 32; ++j2) z[j2] = tile[lane * 33 + j2];
  __syncwarp();
  dft32<INV>(z);
}

__device__ __forceinline__ float2 shfl2(float2 v, int src) {
  return mk<float2>(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

}  // namespace mjx
