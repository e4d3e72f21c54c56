// Mixed-precision (float-float spectral state) building blocks of the adaptive
// IMEX-Strang attempt, shared by the single-solve driver (csrc/imex_mixed.cu)
// and the batched engine (csrc/imex_batch.cu).  See csrc/imex_mixed.cu for the
// attempt's six passes.
#pragma once

#include "spectral.cuh"

namespace mjx {

// MC_MID_BOTH is MC_FULL_END and MC_HALF_MID of the same columns in one tile (ZA in the
// left half, ZB in the right half): the C2 pass then needs half the CTAs
enum { MC_SPLIT = 0, MC_FULL_END = 1, MC_HALF_MID = 2, MC_HALF_END = 3, MC_MID_BOTH = 4 };

__device__ __forceinline__ float2 fmk(float x, float y) { float2 r; r.x = x; r.y = y; return r; }

// ---- float-float arithmetic (error-free transformations: Knuth's two-sum,
// Dekker's fast two-sum, the FMA two-product).  The _rn intrinsics are never
// contracted into FMAs or reassociated, which the transformations rely on.
struct FF { float h, l; };

__device__ __forceinline__ FF ff_fast2sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  FF r; r.h = s; r.l = __fsub_rn(b, __fsub_rn(s, a));
  return r;
}
__device__ __forceinline__ float ff_2sum_err(float a, float b, float s) {  // s = fl(a + b)
  const float bb = __fsub_rn(s, a);
  return __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// x + d, d an FP32 number
__device__ __forceinline__ FF ff_add_f(FF x, float d) {
  const float s = __fadd_rn(x.h, d);
  return ff_fast2sum(s, __fadd_rn(ff_2sum_err(x.h, d, s), x.l));
}
// x + x * mu
__device__ __forceinline__ FF ff_mstep(FF x, float mu) {
  const float p = __fmul_rn(x.h, mu);
  const float pe = __fmaf_rn(x.l, mu, __fmaf_rn(x.h, mu, -p));  // x*mu - p
  const float s = __fadd_rn(x.h, p);
  return ff_fast2sum(s, __fadd_rn(ff_2sum_err(x.h, p, s), __fadd_rn(x.l, pe)));
}
// s * (x - y) rounded to FP32 (the hi difference is exact when x, y are close)
__device__ __forceinline__ float ff_diff_scaled(FF x, FF y, float s) {
  return __fmul_rn(__fadd_rn(__fsub_rn(x.h, y.h), __fsub_rn(x.l, y.l)), s);
}
// s * x rounded to FP32
__device__ __forceinline__ float ff_scaled(FF x, float s) { return __fmaf_rn(x.l, s, __fmul_rn(x.h, s)); }

__device__ __forceinline__ FF ff_re(float4 v) { FF r; r.h = v.x; r.l = v.z; return r; }
__device__ __forceinline__ FF ff_im(float4 v) { FF r; r.h = v.y; r.l = v.w; return r; }
__device__ __forceinline__ float4 ff_pack(FF re, FF im) { return make_float4(re.h, im.h, re.l, im.l); }

// mu = x/(1-x), x = hD * lam (FP32, |1-x| clamped at 1e-14 like the reference)
__device__ __forceinline__ float mu_of(float hD, float lam) {
  const float x = hD * lam;
  float den = 1.0f - x;
  if (fabsf(den) < 1e-14f) den = 1e-14f;
  return x / den;
}
__device__ __forceinline__ float4 ff_mstep_c(float4 X, float mu) {
  return ff_pack(ff_mstep(ff_re(X), mu), ff_mstep(ff_im(X), mu));
}
__device__ __forceinline__ float4 ff_add_c(float4 X, float2 d) {
  return ff_pack(ff_add_f(ff_re(X), d.x), ff_add_f(ff_im(X), d.y));
}

// Everything one column tile of a mixed attempt needs: the single-solve kernel
// fills it from MColArgs, the batched kernel (csrc/imex_batch.cu) from its
// instance table.
struct MColTile {
  int ny, log2ny, ncols, C, type, kx0;
  long long ldc, off;       // row stride; field offset shared by every buffer
  const float4* ys_cur;     // state Y^[cur]
  float4* ys_next;          // state Y^[1-cur]
  float4* pa;
  float4* pb;
  float2* za;
  float2* zb;
  const float* lamx;
  const float* lamy;
  const float2* tw;
  float hA, hB, nrm;        // dt/2 D, dt/4 D, 1/(nx ny)
};

// One tile: C adjacent kx columns of one job over all ny rows.  Threads per CTA
// = 2 C ny/16, so every thread combines exactly min(8, ny/2) elements.  The state
// operands are read in the combine loop rather than held across the forward
// transform: 64 registers, so four 256-thread CTAs share an SM and hide each
// other's load latency (the column passes are latency-bound at 1024^2, where the
// whole working set sits in L2).  Only ny = 4096 needs 512-thread CTAs.
// The caller synchronises the block before buf is reused for another tile.
// LOG2NY, CN, NTH > 0 fix the column length, the tile width and the thread count at compile
// time (the 1024-row passes of the benchmark size), so that the index arithmetic and the
// transforms' radix schedule fold into the code; 0 reads them at run time.
__host__ __device__ constexpr int mc_log2(int v) { return v <= 1 ? 0 : 1 + mc_log2(v >> 1); }

template <int LOG2NY = 0, int CN = 0, int NTH = 0>
__device__ __forceinline__ void mcol_tile(float2* buf, const MColTile& t, int tid, int nth_rt) {
  // the tile holds two outputs side by side (W = 2C) where a job writes two transforms
  // (C1 split, C3 end); the single-output jobs of C2 use a compact tile (W = C), whose
  // column transforms then walk shared memory with half the stride
  const int type = t.type;
  const int nth = NTH ? NTH : nth_rt;
  const int Cn = CN ? CN : t.C, W = (type == MC_FULL_END || type == MC_HALF_MID) ? Cn : 2 * Cn;
  const int kx0 = t.kx0;
  const int ny = LOG2NY ? (1 << LOG2NY) : t.ny;
  const int log2ny = LOG2NY ? LOG2NY : t.log2ny;
  const int total = ny * Cn;
  const int lc = CN ? mc_log2(CN) : __ffs(Cn) - 1;  // the tile width is a power of two
  const long long ldc = t.ldc;
  const float hA = t.hA, hB = t.hB, nrm = t.nrm;

  if (type != MC_SPLIT) {
    // load the FP32 increment tile(s) and transform them forward along y
    const int halves = type == MC_MID_BOTH ? 2 : 1;
    for (int hf = 0; hf < halves; ++hf) {
      const float2* zin = (type == MC_FULL_END || (type == MC_MID_BOTH && hf == 0)) ? t.za : t.zb;
      float2 v[8];
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const int e = tid + m * nth;
        const int ky = e >> lc, c = e & (Cn - 1), kx = kx0 + c;
        if (e < total) v[m] = kx < t.ncols ? zin[t.off + ky * ldc + kx] : fmk(0.f, 0.f);
      }
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const int e = tid + m * nth;
        const int ky = e >> lc, c = e & (Cn - 1);
        if (e < total) buf[sp(ky * W + hf * Cn + c)] = v[m];
      }
    }
    __syncthreads();
    if (LOG2NY) fft_smem_inl<float, false, true>(buf, ny, log2ny, type == MC_MID_BOTH ? W : Cn, 1, W, t.tw, tid);
    else fft_smem<float, false, true>(buf, ny, log2ny, type == MC_MID_BOTH ? W : Cn, 1, W, t.tw, tid);
  }

  // float-float combine, element by element
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const int e = tid + m * nth;
    if (e >= total) continue;
    const int ky = e >> lc, c = e & (Cn - 1), kx = kx0 + c;
    if (kx >= t.ncols) {
      buf[sp(ky * W + c)] = fmk(0.f, 0.f);
      if (W > Cn) buf[sp(ky * W + Cn + c)] = fmk(0.f, 0.f);
      continue;
    }
    const long long g = t.off + ky * ldc + kx;
    const float lam = t.lamx[kx] + t.lamy[ky];
    float4 Pm, Qm;
    if (type == MC_SPLIT) Pm = t.ys_cur[g];
    else if (type == MC_FULL_END || type == MC_MID_BOTH) Pm = t.pa[g];
    else Pm = t.pb[g];
    if (type == MC_HALF_END) Qm = t.pa[g];
    if (type == MC_MID_BOTH) Qm = t.pb[g];
    if (type == MC_MID_BOTH) {  // MC_FULL_END on the left half, MC_HALF_MID on the right
      const float2 d = buf[sp(ky * W + c)], d2 = buf[sp(ky * W + Cn + c)];
      t.pa[g] = ff_mstep_c(ff_add_c(Pm, d), mu_of(hA, lam));
      const float mu = mu_of(hB, lam);
      const float4 X = ff_mstep_c(ff_mstep_c(ff_add_c(Qm, d2), mu), mu);
      t.pb[g] = X;
      buf[sp(ky * W + Cn + c)] = fmk(ff_scaled(ff_re(X), nrm), ff_scaled(ff_im(X), nrm));
    } else if (type == MC_SPLIT) {
      const float4 PA = ff_mstep_c(Pm, mu_of(hA, lam)), PB = ff_mstep_c(Pm, mu_of(hB, lam));
      t.pa[g] = PA;
      t.pb[g] = PB;
      buf[sp(ky * W + c)] = fmk(ff_scaled(ff_re(PA), nrm), ff_scaled(ff_im(PA), nrm));
      buf[sp(ky * W + Cn + c)] = fmk(ff_scaled(ff_re(PB), nrm), ff_scaled(ff_im(PB), nrm));
    } else {
      const float2 d = buf[sp(ky * W + c)];
      if (type == MC_FULL_END) {
        t.pa[g] = ff_mstep_c(ff_add_c(Pm, d), mu_of(hA, lam));
      } else if (type == MC_HALF_MID) {
        const float mu = mu_of(hB, lam);
        const float4 X = ff_mstep_c(ff_mstep_c(ff_add_c(Pm, d), mu), mu);
        t.pb[g] = X;
        buf[sp(ky * W + c)] = fmk(ff_scaled(ff_re(X), nrm), ff_scaled(ff_im(X), nrm));
      } else {  // MC_HALF_END
        const float4 X = ff_mstep_c(ff_add_c(Pm, d), mu_of(hB, lam));
        t.ys_next[g] = X;
        const float4 Fa = Qm;
        buf[sp(ky * W + c)] = fmk(ff_diff_scaled(ff_re(X), ff_re(Fa), nrm),
                                  ff_diff_scaled(ff_im(X), ff_im(Fa), nrm));
        buf[sp(ky * W + Cn + c)] = fmk(ff_scaled(ff_re(X), nrm), ff_scaled(ff_im(X), nrm));
      }
    }
  }
  if (type == MC_FULL_END) return;
  __syncthreads();
  if (type == MC_MID_BOTH) {  // only the right (MC_HALF_MID) half goes back
    if (LOG2NY) fft_smem_inl<float, true, true>(buf, ny, log2ny, Cn, 1, W, t.tw, tid, Cn);
    else fft_smem<float, true, true>(buf, ny, log2ny, Cn, 1, W, t.tw, tid, Cn);
    for (int e = tid; e < ny * Cn; e += nth) {
      const int ky = e >> lc, c = e & (Cn - 1), kx = kx0 + c;
      if (kx < t.ncols) t.zb[t.off + ky * ldc + kx] = buf[sp(ky * W + Cn + c)];
    }
    return;
  }
  const int nseq = (type == MC_HALF_MID) ? Cn : W;
  if (LOG2NY) fft_smem_inl<float, true, true>(buf, ny, log2ny, nseq, 1, W, t.tw, tid);
  else fft_smem<float, true, true>(buf, ny, log2ny, nseq, 1, W, t.tw, tid);
  const int lns = __ffs(nseq) - 1;
  for (int e = tid; e < ny * nseq; e += nth) {
    const int ky = e >> lns, col = e & (nseq - 1);
    const int half = col >> lc, c = col & (Cn - 1), kx = kx0 + c;
    if (kx >= t.ncols) continue;
    const long long g = t.off + ky * ldc + kx;
    const float2 v = buf[sp(ky * W + col)];
    if (type == MC_HALF_MID) t.zb[g] = v;
    else if (half == 0) t.za[g] = v;
    else t.zb[g] = v;
  }
}

// Initial state: y ([nf][ny][nx], io_dtype) -> FP64 transform (plan64) -> the
// float-float half spectrum ys ([nf][ny][ldc] float4).  real64 is scratch of
// nf*ny*nx doubles (it may alias the PA buffer of a mixed workspace, not ys).
mjx_status mix_state_from_real(const void* plan64, const mjx_grid2d* g, int nf, int io_dtype, const void* y,
                               double* real64, float4* ys, cudaStream_t s);
// Final state: the float-float spectrum Y^[cur] (cur read on the device from st, or 0
// when st is null) -> FP64 inverse transform -> y_out (io_dtype).  spec64 holds
// nf*ny*ldc double2 and real64 nf*ny*nx doubles of scratch; neither may alias ys0/ys1.
mjx_status mix_real_from_state(const void* plan64, const mjx_grid2d* g, int nf, const DevState* st,
                               const float4* ys0, const float4* ys1, double2* spec64, double* real64,
                               int io_dtype, void* y_out, cudaStream_t s);

}  // namespace mjx
