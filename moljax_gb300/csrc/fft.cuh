// Shared-memory Stockham FFT for power-of-two lengths 2..4096 (sm_103a).
//
// A block transforms `nseq` sequences of length n that live in shared memory:
// element j of sequence s sits at buf[sp(s * ss + j * es)] (sp pads 1 per 16).  Each sequence gets
// tps = max(1, n/16) threads; every pass is one radix-16 butterfly per thread
// (the last pass uses radix 2/4/8 with 16/R butterflies per thread), held in
// registers, with one shared-memory exchange per pass (Stockham autosort, so
// the output is in natural order).  Twiddles come from a per-length table
// tw[j] = exp(-2 pi i j / n) computed on the host in FP64.
//
// COLMAJOR selects the thread mapping: false -> threads of one sequence are
// consecutive (rows, es == 1); true -> consecutive threads walk across
// sequences (columns, ss == 1, es == number of columns) so that a warp reads
// consecutive shared-memory words in both layouts.
#pragma once

#include "common.cuh"

namespace mjx {

// Shared-memory index with one pad element per 16, so that the stride-16
// writes of the first Stockham pass (and column tiles) spread over the banks.
__device__ __forceinline__ int sp(int e) { return e + (e >> 4); }
// number of padded elements needed to hold e logical elements
__host__ __device__ __forceinline__ int sp_size(int e) { return e + (e >> 4) + 1; }

// cos/sin(2 pi m / 16) for the in-register radix-16 kernel.
#define MJX_C1 0.92387953251128675613
#define MJX_S1 0.38268343236508977173
#define MJX_C2 0.70710678118654752440

// a * exp(-/+ i theta) given cos/sin of theta (forward uses the minus sign).
template <bool INV, typename C>
__device__ __forceinline__ C tw_const(C a, double cs, double sn) {
  typedef decltype(C::x) R;
  const R c = (R)cs, s = INV ? (R)sn : (R)(-sn);
  return mk<C>(a.x * c - a.y * s, a.x * s + a.y * c);
}
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename C> __device__ __forceinline__ C rot(C a) {
  return INV ? mk<C>(-a.y, a.x) : mk<C>(a.y, -a.x);
}

template <bool INV, typename C>
__device__ __forceinline__ void dft2(C& a, C& b) {
  C t = a; a = cadd(t, b); b = csub(t, b);
}

template <bool INV, typename C>
__device__ __forceinline__ void dft4(C& x0, C& x1, C& x2, C& x3) {
  C a = cadd(x0, x2), b = csub(x0, x2), c = cadd(x1, x3), d = rot<INV>(csub(x1, x3));
  x0 = cadd(a, c); x2 = csub(a, c); x1 = cadd(b, d); x3 = csub(b, d);
}

template <bool INV, typename C>
__device__ __forceinline__ void dft8(C* x) {
  C e0 = x[0], e1 = x[2], e2 = x[4], e3 = x[6];
  C o0 = x[1], o1 = x[3], o2 = x[5], o3 = x[7];
  dft4<INV>(e0, e1, e2, e3);
  dft4<INV>(o0, o1, o2, o3);
  o1 = tw_const<INV>(o1, MJX_C2, MJX_C2);
  o2 = rot<INV>(o2);
  o3 = tw_const<INV>(o3, -MJX_C2, MJX_C2);
  x[0] = cadd(e0, o0); x[4] = csub(e0, o0);
  x[1] = cadd(e1, o1); x[5] = csub(e1, o1);
  x[2] = cadd(e2, o2); x[6] = csub(e2, o2);
  x[3] = cadd(e3, o3); x[7] = csub(e3, o3);
}

template <bool INV, typename C>
__device__ __forceinline__ void dft16(C* x) {
  // r = 4 r1 + r2, q = q1 + 4 q2
#pragma unroll
  for (int r2 = 0; r2 < 4; ++r2) dft4<INV>(x[r2], x[4 + r2], x[8 + r2], x[12 + r2]);
  // after the inner transforms x[4*q1 + r2] holds A[r2][q1]; twiddle by w16^(r2 q1)
  x[5] = tw_const<INV>(x[5], MJX_C1, MJX_S1);    // r2=1,q1=1: m=1
  x[9] = tw_const<INV>(x[9], MJX_C2, MJX_C2);    // r2=1,q1=2: m=2
  x[13] = tw_const<INV>(x[13], MJX_S1, MJX_C1);  // r2=1,q1=3: m=3
  x[6] = tw_const<INV>(x[6], MJX_C2, MJX_C2);    // r2=2,q1=1: m=2
  x[10] = rot<INV>(x[10]);                       // r2=2,q1=2: m=4
  x[14] = tw_const<INV>(x[14], -MJX_C2, MJX_C2); // r2=2,q1=3: m=6
  x[7] = tw_const<INV>(x[7], MJX_S1, MJX_C1);    // r2=3,q1=1: m=3
  x[11] = tw_const<INV>(x[11], -MJX_C2, MJX_C2); // r2=3,q1=2: m=6
  x[15] = tw_const<INV>(x[15], -MJX_C1, -MJX_S1);// r2=3,q1=3: m=9
#pragma unroll
  for (int q1 = 0; q1 < 4; ++q1) dft4<INV>(x[4 * q1], x[4 * q1 + 1], x[4 * q1 + 2], x[4 * q1 + 3]);
  // now x[4*q1 + q2] holds X[q1 + 4 q2]; transpose the 4x4 index map in registers
  C t;
  t = x[1]; x[1] = x[4]; x[4] = t;
  t = x[2]; x[2] = x[8]; x[8] = t;
  t = x[3]; x[3] = x[12]; x[12] = t;
  t = x[6]; x[6] = x[9]; x[9] = t;
  t = x[7]; x[7] = x[13]; x[13] = t;
  t = x[11]; x[11] = x[14]; x[14] = t;
}

template <int R, bool INV, typename C>
__device__ __forceinline__ void dft_r(C* x) {
  if (R == 2) dft2<INV>(x[0], x[1]);
  else if (R == 4) dft4<INV>(x[0], x[1], x[2], x[3]);
  else if (R == 8) dft8<INV>(x);
  else dft16<INV>(x);
}

// Twiddle w^r (r = 1..R-1) for a butterfly whose base index is t (w^r = tw[r t]),
// rebuilt from at most six table reads: w^(4a+b) = w^(4a) * w^b.
template <typename T, int R, bool INV>
__device__ __forceinline__ void apply_twiddles(cx<T>* x, int t, const cx<T>* __restrict__ tw) {
  typedef cx<T> C;
  const C w1 = __ldg(&tw[t]);
  if constexpr (R == 2) { x[1] = INV ? cmulc(x[1], w1) : cmul(x[1], w1); return; }
  const C w2 = __ldg(&tw[2 * t]), w3 = __ldg(&tw[3 * t]);
  C wb[4];
  wb[1] = w1; wb[2] = w2; wb[3] = w3;
#pragma unroll
  for (int b = 1; b < 4; ++b) x[b] = INV ? cmulc(x[b], wb[b]) : cmul(x[b], wb[b]);
  if constexpr (R > 4) {
#pragma unroll
  for (int a4 = 1; a4 < R / 4; ++a4) {
    const C wa = __ldg(&tw[4 * a4 * t]);
    x[4 * a4] = INV ? cmulc(x[4 * a4], wa) : cmul(x[4 * a4], wa);
#pragma unroll
    for (int b = 1; b < 4; ++b) {
      const C w = cmul(wa, wb[b]);
      x[4 * a4 + b] = INV ? cmulc(x[4 * a4 + b], w) : cmul(x[4 * a4 + b], w);
    }
  }
  }
}

// a / b and a % b for a >= 0, b > 0: a shift and a mask when b is a power of two (every
// length, thread count and sequence count of the transforms here), a division otherwise
__device__ __forceinline__ int pdiv(int a, int b) { return (b & (b - 1)) == 0 ? a >> (__ffs(b) - 1) : a / b; }
__device__ __forceinline__ int pmod(int a, int b) { return (b & (b - 1)) == 0 ? a & (b - 1) : a % b; }

// One Stockham pass of radix R with current sub-length p (p*R divides n).
// Element j of this thread's sequence is buf[base + j * es]; ES1 fixes es = 1.
template <typename T, int R, bool INV, bool ES1>
__device__ __forceinline__ void stockham_pass(cx<T>* buf, int n, int p, int tps, int lt, int base,
                                              int es_rt, bool active,
                                              const cx<T>* __restrict__ tw) {
  typedef cx<T> C;
  const int es = ES1 ? 1 : es_rt;
  const int Tn = pdiv(n, R);                       // butterflies per sequence
  const int nb = (Tn >= tps) ? pdiv(Tn, tps) : 1;  // butterflies per thread (<= 16/R)
  constexpr int NBMAX = 16 / R;
  C x[16];
  if (active) {
#pragma unroll
    for (int m = 0; m < NBMAX; ++m) {
      if (m < nb) {
        const int i = lt + m * tps;
#pragma unroll
        for (int r = 0; r < R; ++r) x[m * R + r] = buf[sp(base + (i + r * Tn) * es)];
      }
    }
  }
  __syncthreads();
  if (active) {
    const int twstep = pdiv(n, p * R);
#pragma unroll
    for (int m = 0; m < NBMAX; ++m) {
      if (m < nb) {
        const int i = lt + m * tps;
        const int k = i & (p - 1);
        if (p > 1) apply_twiddles<T, R, INV>(&x[m * R], k * twstep, tw);
        dft_r<R, INV>(&x[m * R]);
        const int j = (i - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) buf[sp(base + (j + r * p) * es)] = x[m * R + r];
      }
    }
  }
  __syncthreads();
}

// In-place FFT of nseq sequences (see file comment), sequences s0 .. s0 + nseq - 1.
// All threads of the block must call it; threads with tid >= nseq*tps only join the
// barriers.  The caller must __syncthreads() after filling buf; on return buf is complete.
template <typename T, bool INV, bool COLMAJOR>
__device__ __forceinline__ void fft_smem_inl(cx<T>* buf, int n, int log2n, int nseq, int ss, int es,
                         const cx<T>* __restrict__ tw, int tid, int s0 = 0) {
  const int tps = n >= 16 ? pdiv(n, 16) : 1;
  const bool active = tid < nseq * tps;
  int lt, s;
  if (COLMAJOR) { s = pmod(tid, nseq); lt = pdiv(tid, nseq); }
  else { lt = pmod(tid, tps); s = pdiv(tid, tps); }
  const int base = (s + s0) * ss;
  // straight-line schedule: up to three radix-16 passes (n <= 4096), then radix 2/4/8
  int p = 1, rem = log2n;
#pragma unroll
  for (int k16 = 0; k16 < 3; ++k16) {
    if (rem >= 4) {
      stockham_pass<T, 16, INV, !COLMAJOR>(buf, n, p, tps, lt, base, es, active, tw);
      p <<= 4;
      rem -= 4;
    }
  }
  if (rem == 3) stockham_pass<T, 8, INV, !COLMAJOR>(buf, n, p, tps, lt, base, es, active, tw);
  else if (rem == 2) stockham_pass<T, 4, INV, !COLMAJOR>(buf, n, p, tps, lt, base, es, active, tw);
  else if (rem == 1) stockham_pass<T, 2, INV, !COLMAJOR>(buf, n, p, tps, lt, base, es, active, tw);
}


// fft_smem_inl is always inlined, so that a caller passing compile-time lengths gets the
// index arithmetic and the radix schedule folded; fft_smem leaves the choice to the compiler.
template <typename T, bool INV, bool COLMAJOR>
__device__ void fft_smem(cx<T>* buf, int n, int log2n, int nseq, int ss, int es, const cx<T>* __restrict__ tw,
                         int tid, int s0 = 0) {
  fft_smem_inl<T, INV, COLMAJOR>(buf, n, log2n, nseq, ss, es, tw, tid, s0);
}

// The same transform in radix-4 passes (a final radix-2 pass when log2 n is odd), n/4
// threads per sequence with one butterfly each: four times the threads of the radix-16
// schedule and about a third of the arithmetic per thread.  Used for short FP64 transforms,
// where each warp of the radix-16 schedule would keep only n/16 lanes busy and wait on
// GB300's narrow FP64 pipe.  Same layout, barriers and output order as fft_smem.
template <typename T, bool INV, bool COLMAJOR>
__device__ void fft_smem_r4(cx<T>* buf, int n, int log2n, int nseq, int ss, int es, const cx<T>* __restrict__ tw,
                            int tid, int s0 = 0) {
  const int tps = n >= 4 ? pdiv(n, 4) : 1;
  const bool active = tid < nseq * tps;
  int lt, s;
  if (COLMAJOR) { s = pmod(tid, nseq); lt = pdiv(tid, nseq); }
  else { lt = pmod(tid, tps); s = pdiv(tid, tps); }
  const int base = (s + s0) * ss;
  int p = 1;
  for (int rem = log2n; rem >= 2; rem -= 2) {
    stockham_pass<T, 4, INV, !COLMAJOR>(buf, n, p, tps, lt, base, es, active, tw);
    p <<= 2;
  }
  if (log2n & 1) stockham_pass<T, 2, INV, !COLMAJOR>(buf, n, p, tps, lt, base, es, active, tw);
}
}  // namespace mjx
