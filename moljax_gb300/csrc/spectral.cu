// Periodic 2D spectral passes: fused row r2c/c2r (+ pointwise work) and
// column forward-multiply-inverse kernels, plans, and the C ABI for the
// Helmholtz / CN / exponential multipliers and the FFT-CN stepper.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "spectral.cuh"
#include "tma.cuh"
#include "wfft.cuh"

namespace mjx {

static inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

int spec_ldc(int nx) { return ((nx / 2 + 1) + 3) & ~3; }

// Entries of the x twiddle table: FP32 plans of 1024-point rows append the same 1024 values
// transposed for the one-warp transform (entry 1024 + 32 k1 + l holds w^(l k1)), so that
// the 32 lanes of a warp read one contiguous 256-byte run per twiddle instead of 32 rows
// of the table.
static int twx_count(int nx, int elem) { return (nx == 1024 && elem == 4) ? 2048 : nx; }

size_t plan_bytes(int ny, int nx, int elem) {
  const size_t c = 2 * (size_t)elem;
  return align256(twx_count(nx, elem) * c) + align256(ny * c) + align256(spec_ldc(nx) * (size_t)elem) +
         align256(ny * (size_t)elem);
}

PlanView plan_view(const void* plan, int ny, int nx, int elem) {
  const size_t c = 2 * (size_t)elem;
  const char* p = (const char*)plan;
  PlanView v;
  v.twx = p; p += align256(twx_count(nx, elem) * c);
  v.twy = p; p += align256(ny * c);
  v.lamx = p; p += align256(spec_ldc(nx) * (size_t)elem);
  v.lamy = p;
  return v;
}

// Sequences (row pairs) per CTA: ~128 threads per CTA, so that the 1024-row passes
// launch enough CTAs to fill every SM (n = 1024: 2 sequences, n = 4096: one of 256 threads).
int row_nseq(int n, int nrows) {
  const int tps = n >= 16 ? n / 16 : 1;
  int ns = 128 / tps;
  if (ns < 1) ns = 1;
  if (ns > nrows) ns = nrows;
  return ns;
}

int row_ctas(int n, int nrows, int npairs) { return npairs * nrows / row_nseq(n, nrows); }

// ------------------------------------------------------------------ reactions
template <typename T, int RX>
__device__ __forceinline__ void react_heun(T& a, T& b, T h, T F, T k, T r) {
  if (RX == RX_GRAY_SCOTT) {
    // moljax/core/stepping.py:402-415 with operators.py:655-667
    const T uvv = a * b * b;
    const T fu = -uvv + F * ((T)1 - a);
    const T fv = uvv - (F + k) * b;
    const T ua = a + h * fu, va = b + h * fv;
    const T uvv2 = ua * va * va;
    const T gu = -uvv2 + F * ((T)1 - ua);
    const T gv = uvv2 - (F + k) * va;
    const T hh = (T)0.5 * h;
    a = a + hh * (fu + gu);
    b = b + hh * (fv + gv);
  } else if (RX == RX_FISHER) {
    const T fa = r * a * ((T)1 - a), fb = r * b * ((T)1 - b);
    const T ta = a + h * fa, tb = b + h * fb;
    const T hh = (T)0.5 * h;
    a = a + hh * (fa + r * ta * ((T)1 - ta));
    b = b + hh * (fb + r * tb * ((T)1 - tb));
  }
}

// Explicit Euler reaction step y + h N(y) (imex_euler_step, stepping.py:349-359).
template <typename T, int RX>
__device__ __forceinline__ void react_euler(T& a, T& b, T h, T F, T k, T r) {
  if (RX == RX_GRAY_SCOTT) {
    const T uvv = a * b * b;
    const T fu = -uvv + F * ((T)1 - a);
    const T fv = uvv - (F + k) * b;
    a = a + h * fu;
    b = b + h * fv;
  } else if (RX == RX_FISHER) {
    const T fa = r * a * ((T)1 - a), fb = r * b * ((T)1 - b);
    a = a + h * fa;
    b = b + h * fb;
  }
}

template <typename T> __device__ __forceinline__ bool finite_(T v) { return isfinite(v); }

// ------------------------------------------------------------------ row pass
template <typename T> struct Occ { static constexpr int row = sizeof(T) == 4 ? 4 : 2, col = sizeof(T) == 4 ? 2 : 1; };

// LOG2N > 0: the row length 2^LOG2N and one sequence per CTA are compile-time constants
// (FP32 rows of 2048 and 4096 points), so that the transform's index arithmetic and radix
// schedule fold into the code; LOG2N = 0 reads both from the arguments.
// R4: radix-4 transforms with n/4 threads per sequence (short FP64 rows, fft_smem_r4).
template <typename T, int RX, int LOG2N = 0, bool R4 = false>
__global__ void __launch_bounds__(256, Occ<T>::row) row_kernel(const __grid_constant__ RowArgs<T> a) {
  typedef cx<T> C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const DevState* st = a.st;
  if (st != nullptr && st->done) return;

  const int n = LOG2N ? (1 << LOG2N) : a.n, half = n >> 1;
  const int log2n = LOG2N ? LOG2N : a.log2n, nseq = LOG2N ? 1 : a.nseq;
  const int tps = R4 ? (n >= 4 ? n / 4 : 1) : (n >= 16 ? n / 16 : 1);
  const int tid = threadIdx.x;
  const int s_loc = tid / tps, lt = tid % tps;
  const int seq0 = blockIdx.x * nseq;
  const int q = seq0 / a.nrows;  // uniform within the CTA (nrows % nseq == 0)
  const RowPair pr = a.pr[q];
  const int flags = pr.flags;
  const long long y = (seq0 % a.nrows) + s_loc;
  const int cur = st != nullptr ? st->cur : 0;
  const T* rin = a.rin_sel < 0 ? a.rin[0] : a.rin[a.rin_sel == 0 ? cur : 1 - cur];
  T* rout = a.rout_sel < 0 ? a.rout[0] : a.rout[a.rout_sel == 0 ? cur : 1 - cur];
  const int zb = s_loc * n;  // this sequence's first logical smem element
#define Z(x) buf[sp(zb + (x))]

  // 1. load: spectrum rows (c2r) or real rows
  if (flags & ROW_LOAD_SPEC) {
    const C* A = a.spec + pr.sa + y * a.ldc;
    const C* B = a.spec + pr.sb + y * a.ldc;
    // every thread owns kk = lt + m*tps, m < 9 (n/2+1 <= 9*tps): issue all loads first
    C Ak[9], Bk[9];
#pragma unroll
    for (int m = 0; m < 9; ++m) {
      const int kk = lt + m * tps;
      if (kk <= half) { Ak[m] = A[kk]; Bk[m] = B[kk]; }
    }
#pragma unroll
    for (int m = 0; m < 9; ++m) {
      const int kk = lt + m * tps;
      if (kk <= half) {
        Z(kk) = mk<C>(Ak[m].x - Bk[m].y, Ak[m].y + Bk[m].x);                    // A_k + i B_k
        if (kk > 0 && kk < half) Z(n - kk) = mk<C>(Ak[m].x + Bk[m].y, Bk[m].x - Ak[m].y);  // conj(A_k) + i conj(B_k)
      }
    }
    __syncthreads();
    if (R4) fft_smem_r4<T, true, false>(buf, n, log2n, nseq, n, 1, a.tw, tid);
    else if (LOG2N) fft_smem_inl<T, true, false>(buf, n, log2n, nseq, n, 1, a.tw, tid);
    else fft_smem<T, true, false>(buf, n, log2n, nseq, n, 1, a.tw, tid);
  } else {
    const T* ra = rin + pr.ra + y * a.rstride;
    const T* rb = rin + pr.rb + y * a.rstride;
    T va[16], vb[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int x = lt + m * tps;
      if (x < n) { va[m] = ra[x]; vb[m] = rb[x]; }
    }
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int x = lt + m * tps;
      if (x < n) Z(x) = mk<C>(va[m], vb[m]);
    }
    __syncthreads();
  }

  // 2. pointwise work on the real rows (each thread owns x = lt + m*tps)
  const T sc = (flags & ROW_LOAD_SPEC) ? a.inv_scale : (T)1;
  T h = (T)0;
  if (flags & ROW_REACT) h = (T)((st != nullptr ? st->dtc : a.hfixed) * pr.hfac);
  T esum = (T)0;
  int bad = 0;
  T* oa = rout + pr.ra + y * a.rstride;
  T* ob = rout + pr.rb + y * a.rstride;
  const T* ea = a.eref + pr.ra + y * a.rstride;
  const T* eb = a.eref + pr.rb + y * a.rstride;
  // parameters converted once (the per-element double arithmetic would occupy the FP64 pipe)
  const T pF = (T)a.F, pK = (T)a.k, pR = (T)a.r, pFK = (T)(a.F + a.k);
  const T pAtol = (T)a.atol, pRtol = (T)a.rtol;
  T ra_[16], rb_[16];
  if (flags & ROW_ERRNORM) {
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int x = lt + m * tps;
      if (x < n) { ra_[m] = ea[x]; rb_[m] = eb[x]; }
    }
  }
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const int x = lt + m * tps;
    if (x >= n) continue;
    const C v = Z(x);
    T va = v.x * sc, vb = v.y * sc;
    if (flags & ROW_NONLIN) {
      // Gray-Scott reaction terms (operators.py:655-667); Fisher-KPP r u (1-u)
      if (RX == RX_GRAY_SCOTT) {
        const T uvv = va * vb * vb;
        const T nu = -uvv + pF * ((T)1 - va), nv = uvv - pFK * vb;
        va = nu; vb = nv;
      } else if (RX == RX_FISHER) {
        va = pR * va * ((T)1 - va); vb = pR * vb * ((T)1 - vb);
      } else {
        va = (T)0; vb = (T)0;
      }
    }
    if (flags & ROW_REACT) {
      if (flags & ROW_DELTA) react_delta<T, RX>(va, vb, h, pF, pK, pR);
      else if (flags & ROW_EULER) {
        react_euler<T, RX>(va, vb, h, pF, pK, pR);
        if (flags & ROW_EULER2) react_euler<T, RX>(va, vb, h, pF, pK, pR);
      }
      else react_heun<T, RX>(va, vb, h, pF, pK, pR);
    }
    if (flags & ROW_STORE_REAL) { oa[x] = va; ob[x] = vb; }
    if (flags & ROW_ERRNORM) {
      // moljax/core/state.py:335-339: (err / (atol + rtol |y_new|))^2
      const T da = (va - ra_[m]) / (pAtol + pRtol * fabs(va));
      const T db = (vb - rb_[m]) / (pAtol + pRtol * fabs(vb));
      esum += da * da + db * db;
      bad |= !(finite_(va) && finite_(vb));
    }
    if (flags & ROW_ERRPAIR) {
      const T da = va / (pAtol + pRtol * fabs(vb));
      esum += da * da;
      bad |= !(finite_(va) && finite_(vb));
    }
    Z(x) = mk<C>(va, vb);
  }

  // 3. r2c and split into the two half spectra
  if (flags & ROW_STORE_SPEC) {
    __syncthreads();
    if (R4) fft_smem_r4<T, false, false>(buf, n, log2n, nseq, n, 1, a.tw, tid);
    else if (LOG2N) fft_smem_inl<T, false, false>(buf, n, log2n, nseq, n, 1, a.tw, tid);
    else fft_smem<T, false, false>(buf, n, log2n, nseq, n, 1, a.tw, tid);
    C* A = a.spec + ((flags & ROW_SPEC_ALT) ? pr.oa : pr.sa) + y * a.ldc;
    C* B = a.spec + ((flags & ROW_SPEC_ALT) ? pr.ob : pr.sb) + y * a.ldc;
#pragma unroll
    for (int m = 0; m < 9; ++m) {
      const int kk = lt + m * tps;
      if (kk > half) continue;
      const C Zk = Z(kk), Zm = Z((n - kk) & (n - 1));
      A[kk] = mk<C>((T)0.5 * (Zk.x + Zm.x), (T)0.5 * (Zk.y - Zm.y));
      B[kk] = mk<C>((T)0.5 * (Zk.y + Zm.y), (T)0.5 * (Zm.x - Zk.x));
    }
  }

  // 4. block reduction of the error partials (FP64 across threads)
  if (flags & (ROW_ERRNORM | ROW_ERRPAIR)) {
    __shared__ double red[32];
    __shared__ int redbad[32];
    double v = (double)esum;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v += __shfl_xor_sync(0xffffffffu, v, o);
      bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    const int w = tid >> 5, nw = (blockDim.x + 31) >> 5;
    if ((tid & 31) == 0) { red[w] = v; redbad[w] = bad; }
    __syncthreads();
    if (tid == 0) {
      double s = 0.0, c = 0.0;  // Kahan
      int b2 = 0;
      for (int i = 0; i < nw; ++i) {
        const double yv = red[i] - c;
        const double tv = s + yv;
        c = (tv - s) - yv;
        s = tv;
        b2 |= redbad[i];
      }
      a.partial[blockIdx.x] = s;
      a.nonfinite[blockIdx.x] = b2;
    }
  }
#undef Z
}

// ------------------------------------------------------------------ column pass
template <typename T>
__device__ __forceinline__ T multiplier(int mul, T hD, T lam, int pw) {
  T m;
  if (mul == MUL_HELMHOLTZ) {
    T den = (T)1 - hD * lam;  // moljax/core/fft_solvers.py:281-285
    if (fabs(den) < (T)1e-14) den = (T)1e-14;
    m = (T)1 / den;
  } else if (mul == MUL_CN) {
    const T x = (T)0.5 * hD * lam;
    m = ((T)1 + x) / ((T)1 - x);
  } else if (mul == MUL_EXP) {
    m = exp(hD * lam);
  } else if (mul == MUL_LAP) {
    m = hD * lam;
  } else {
    m = (T)1;
  }
  return pw == 2 ? m * m : m;
}

template <typename T> struct ColThreads { static constexpr int v = sizeof(T) == 4 ? 1024 : 512; };

// R4: radix-4 column transforms with ny/4 threads per column (short FP64 columns).
template <typename T, bool R4 = false>
__global__ void __launch_bounds__(ColThreads<T>::v, 1) col_kernel(const __grid_constant__ ColArgs<T> a) {
  typedef cx<T> C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  if (a.st != nullptr && a.st->done) return;
  const ColJob jb = a.job[blockIdx.y];
  const int Cn = a.C, nout = jb.nout, W = Cn * nout;
  const int kx0 = blockIdx.x * Cn;
  const int ny = a.ny, tid = threadIdx.x, nth = blockDim.x;
  const int lc = __ffs(Cn) - 1;  // the tile width is a power of two (col_tile / tile halve from one)
  const long long ldc = a.ldc;
  const long long po = (long long)blockIdx.z * a.pstride;

  {
    C v[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int e = tid + m * nth;
      const int ky = e >> lc, c = e & (Cn - 1), kx = kx0 + c;
      const bool mir = a.oddy && ky >= (ny >> 1);
      const int kyl = mir ? ny - 1 - ky : ky;
      if (e < ny * Cn) {
        v[m] = kx < a.ncols ? a.spec[po + jb.sin + kyl * ldc + kx] : mk<C>((T)0, (T)0);
        if (mir) v[m] = mk<C>(-v[m].x, -v[m].y);
      }
    }
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int e = tid + m * nth;
      const int ky = e >> lc, c = e & (Cn - 1);
      if (e < ny * Cn) buf[sp(ky * W + c)] = v[m];
    }
  }
  __syncthreads();
  const int dirs = jb.dirs ? jb.dirs : 3;
  if (dirs & 1) {
    if (R4) fft_smem_r4<T, false, true>(buf, ny, a.log2ny, Cn, 1, W, a.tw, tid);
    else fft_smem<T, false, true>(buf, ny, a.log2ny, Cn, 1, W, a.tw, tid);
  }
  const T jscale = jb.scale != 0.0 ? (T)jb.scale : a.scale;

  const double h = a.st != nullptr ? a.st->dtc : a.hfixed;
  const T hD0 = (T)(h * jb.hfac[0] * jb.D), hD1 = (T)(h * jb.hfac[1] * jb.D);
  for (int e = tid; e < ny * Cn; e += nth) {
    const int ky = e >> lc, c = e & (Cn - 1), kx = kx0 + c;
    T lxy = (T)0;
    if (kx < a.ncols) lxy = a.ldc3 ? a.lamx[kx % a.ldc3] + a.lamy2[kx / a.ldc3] : a.lamx[kx];
    const T lam = lxy + a.lamy[ky];
    const C v = buf[sp(ky * W + c)];
    if (jb.mul == MUL_ADVDIFF || jb.mul == MUL_ADV_LAP || jb.mul == MUL_ADV_EXP || jb.mul == MUL_ADV_CN) {
      // z = h (D lam - i (vx kx + vy ky)), kx, ky = 2 pi fftfreq (the Nyquist index
      // negative); m = 1/(1 - z) with |1 - z| < 1e-14 -> 1e-14 (the solve of
      // FFTAdvectionDiffusionPreconditioner, moljax/core/preconditioners.py:297-420, and of
      // AdvectionDiffusionOperator, fft_operators.py:179-260), z itself (matvec) or exp(z)
      // (exp_matvec), or the Crank-Nicolson factor (1 + z/2)/(1 - z/2) of the 1D advective
      // FFT-CN (benchmarks/benchmark_solver_comparison.py:152-163).  The reference keeps
      // real(ifft(.)); on the half spectrum that is the
      // multiplier (m(k) + conj(m(-k)))/2, which equals m(k) except on the Nyquist lines,
      // where fftfreq breaks the oddness of the advection term.
      const int nxl = 2 * (a.ncols - 1);
      const int mx = kx < nxl / 2 ? kx : kx - nxl, my = ky < ny / 2 ? ky : ky - ny;
      const int nmx = mx == -nxl / 2 ? mx : -mx, nmy = my == -ny / 2 ? my : -my;
      const double hh = h * jb.hfac[0];
      const double zr = (double)hD0 * (double)lam;
      double mre = 0.0, mim = 0.0;
      for (int side = 0; side < 2; ++side) {
        const int qx = side ? nmx : mx, qy = side ? nmy : my;
        const double zi = -hh * (jb.vx * a.kxs * qx + jb.vy * a.kys * qy);
        double fr, fi;
        if (jb.mul == MUL_ADVDIFF) {
          double dr = 1.0 - zr, di = -zi;
          if (sqrt(dr * dr + di * di) < 1e-14) { dr = 1e-14; di = 0.0; }
          const double den = dr * dr + di * di;
          fr = dr / den;
          fi = -di / den;
        } else if (jb.mul == MUL_ADV_LAP) {
          fr = zr;
          fi = zi;
        } else if (jb.mul == MUL_ADV_CN) {
          const double nr = 1.0 + 0.5 * zr, ni = 0.5 * zi, dr = 1.0 - 0.5 * zr, di = -0.5 * zi;
          const double den = dr * dr + di * di;
          fr = (nr * dr + ni * di) / den;
          fi = (ni * dr - nr * di) / den;
        } else {
          double sn, cs;
          sincos(zi, &sn, &cs);
          const double ez = exp(zr);
          fr = ez * cs;
          fi = ez * sn;
        }
        mre += 0.5 * fr;
        mim += side ? -0.5 * fi : 0.5 * fi;  // conj(m(-k)) on the second side
      }
      const T mr = (T)mre, mi = (T)mim;
      buf[sp(ky * W + c)] = cscale(mk<C>(v.x * mr - v.y * mi, v.x * mi + v.y * mr), jscale);
      continue;
    }
    if (jb.mul == MUL_TABLE) {
      buf[sp(ky * W + c)] = cscale(v, jscale * a.mtab[(long long)ky * ldc + kx]);
      continue;
    }
    buf[sp(ky * W + c)] = cscale(v, jscale * multiplier<T>(jb.mul, hD0, lam, jb.pow[0]));
    if (nout > 1) buf[sp(ky * W + Cn + c)] = cscale(v, jscale * multiplier<T>(jb.mul, hD1, lam, jb.pow[1]));
  }
  __syncthreads();
  if (dirs & 2) {
    if (R4) fft_smem_r4<T, true, true>(buf, ny, a.log2ny, W, 1, W, a.tw, tid);
    else fft_smem<T, true, true>(buf, ny, a.log2ny, W, 1, W, a.tw, tid);
  }

  const int lw = __ffs(W) - 1;  // W = Cn or 2 Cn
  for (int e = tid; e < ny * W; e += nth) {
    const int ky = e >> lw, col = e & (W - 1);
    const int o = col >> lc, c = col & (Cn - 1), kx = kx0 + c;
    if (kx < a.ncols && !(a.oddy && ky >= (ny >> 1))) a.spec[po + jb.sout[o] + ky * ldc + kx] = buf[sp(ky * W + col)];
  }
}

// ------------------------------------------------------------------ warp row pass (n = 1024)
// The row pass of row_kernel (same flags, pair table, pointwise work and error partials) for
// FP32 rows of 1024 points, one warp per sequence.
template <int RX>
__global__ void __launch_bounds__(128) row_kernel_w32(const __grid_constant__ RowArgs<float> a) {
  typedef float2 C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const DevState* st = a.st;
  if (st != nullptr && st->done) return;
  const int lane = threadIdx.x & 31, s_loc = threadIdx.x >> 5;
  C* tile = reinterpret_cast<C*>(smem_raw) + s_loc * (32 * 33);
  const int seq0 = blockIdx.x * a.nseq;
  const int q = seq0 / a.nrows;  // uniform within the CTA (nrows % nseq == 0)
  const RowPair pr = a.pr[q];
  const int flags = pr.flags;
  const long long y = (seq0 % a.nrows) + s_loc;
  const int cur = st != nullptr ? st->cur : 0;
  const float* rin = a.rin_sel < 0 ? a.rin[0] : a.rin[a.rin_sel == 0 ? cur : 1 - cur];
  float* rout = a.rout_sel < 0 ? a.rout[0] : a.rout[a.rout_sel == 0 ? cur : 1 - cur];
  const int src = (32 - lane) & 31;  // the lane holding index 1024 - k of this lane's k
  C z[32];
  // 1. load: spectrum rows (c2r) or real rows, element lane + 32 j in z[j]
  if (flags & ROW_LOAD_SPEC) {
    const C* A = a.spec + pr.sa + y * a.ldc;
    const C* B = a.spec + pr.sb + y * a.ldc;
    C Ar[17], Br[17];
#pragma unroll
    for (int j = 0; j < 16; ++j) { Ar[j] = A[32 * j + lane]; Br[j] = B[32 * j + lane]; }
    Ar[16] = lane == 0 ? A[512] : mk<C>(0.f, 0.f);
    Br[16] = lane == 0 ? B[512] : mk<C>(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < 16; ++j) z[j] = mk<C>(Ar[j].x - Br[j].y, Ar[j].y + Br[j].x);  // A_k + i B_k
#pragma unroll
    for (int j = 16; j < 32; ++j) {  // k = 32 j + lane > 512 (and k = 512 on lane 0)
      C av = shfl2(Ar[31 - j], src), bv = shfl2(Br[31 - j], src);
      if (lane == 0) { av = Ar[32 - j]; bv = Br[32 - j]; }
      if (lane == 0 && j == 16) z[j] = mk<C>(av.x - bv.y, av.y + bv.x);
      else z[j] = mk<C>(av.x + bv.y, bv.x - av.y);  // conj(A_k') + i conj(B_k'), k' = 1024 - k
    }
    wfft1024<true>(z, tile, a.tw, lane);
  } else {
    const float* ra = rin + pr.ra + y * a.rstride;
    const float* rb = rin + pr.rb + y * a.rstride;
#pragma unroll
    for (int j = 0; j < 32; ++j) z[j] = mk<C>(ra[32 * j + lane], rb[32 * j + lane]);
  }

  // 2. pointwise work on element x = lane + 32 j (as row_kernel)
  const float sc = (flags & ROW_LOAD_SPEC) ? a.inv_scale : 1.0f;
  float h = 0.f;
  if (flags & ROW_REACT) h = (float)((st != nullptr ? st->dtc : a.hfixed) * pr.hfac);
  float esum = 0.f;
  int bad = 0;
  float* oa = rout + pr.ra + y * a.rstride;
  float* ob = rout + pr.rb + y * a.rstride;
  const float* ea = a.eref + pr.ra + y * a.rstride;
  const float* eb = a.eref + pr.rb + y * a.rstride;
  const float pF = (float)a.F, pK = (float)a.k, pR = (float)a.r, pFK = (float)(a.F + a.k);
  const float pAtol = (float)a.atol, pRtol = (float)a.rtol;
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    const int x = lane + 32 * j;
    float va = z[j].x * sc, vb = z[j].y * sc;
    if (flags & ROW_NONLIN) {
      if (RX == RX_GRAY_SCOTT) {
        const float uvv = va * vb * vb;
        const float nu = -uvv + pF * (1.f - va), nv = uvv - pFK * vb;
        va = nu; vb = nv;
      } else if (RX == RX_FISHER) {
        va = pR * va * (1.f - va); vb = pR * vb * (1.f - vb);
      } else {
        va = 0.f; vb = 0.f;
      }
    }
    if (flags & ROW_REACT) {
      if (flags & ROW_DELTA) react_delta<float, RX>(va, vb, h, pF, pK, pR);
      else if (flags & ROW_EULER) {
        react_euler<float, RX>(va, vb, h, pF, pK, pR);
        if (flags & ROW_EULER2) react_euler<float, RX>(va, vb, h, pF, pK, pR);
      }
      else react_heun<float, RX>(va, vb, h, pF, pK, pR);
    }
    if (flags & ROW_STORE_REAL) { oa[x] = va; ob[x] = vb; }
    if (flags & ROW_ERRNORM) {
      const float da = (va - ea[x]) / (pAtol + pRtol * fabsf(va));
      const float db = (vb - eb[x]) / (pAtol + pRtol * fabsf(vb));
      esum += da * da + db * db;
      bad |= !(finite_(va) && finite_(vb));
    }
    if (flags & ROW_ERRPAIR) {
      const float da = va / (pAtol + pRtol * fabsf(vb));
      esum += da * da;
      bad |= !(finite_(va) && finite_(vb));
    }
    z[j] = mk<C>(va, vb);
  }

  // 3. r2c and split into the two half spectra: X_k in z[k2] of lane k1, k = k1 + 32 k2
  if (flags & ROW_STORE_SPEC) {
    wfft1024<false>(z, tile, a.tw, lane);
    C* A = a.spec + ((flags & ROW_SPEC_ALT) ? pr.oa : pr.sa) + y * a.ldc;
    C* B = a.spec + ((flags & ROW_SPEC_ALT) ? pr.ob : pr.sb) + y * a.ldc;
#pragma unroll
    for (int k2 = 0; k2 <= 16; ++k2) {
      C Zm = shfl2(z[k2 <= 15 ? 31 - k2 : 15], src);  // X_{1024-k} (lanes > 0)
      if (lane == 0) Zm = z[(32 - k2) & 31];
      const int k = lane + 32 * k2;
      if (k2 == 16 && lane != 0) continue;
      const C Zk = z[k2];
      A[k] = mk<C>(0.5f * (Zk.x + Zm.x), 0.5f * (Zk.y - Zm.y));
      B[k] = mk<C>(0.5f * (Zk.y + Zm.y), 0.5f * (Zm.x - Zk.x));
    }
  }

  // 4. block reduction of the error partials (FP64 across warps)
  if (flags & (ROW_ERRNORM | ROW_ERRPAIR)) {
    __shared__ double red[4];
    __shared__ int redbad[4];
    double v = (double)esum;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v += __shfl_xor_sync(0xffffffffu, v, o);
      bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if (lane == 0) { red[s_loc] = v; redbad[s_loc] = bad; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double sum = 0.0, c = 0.0;  // Kahan
      int b2 = 0;
      for (int i = 0; i < a.nseq; ++i) {
        const double yv = red[i] - c;
        const double tv = sum + yv;
        c = (tv - sum) - yv;
        sum = tv;
        b2 |= redbad[i];
      }
      a.partial[blockIdx.x] = sum;
      a.nonfinite[blockIdx.x] = b2;
    }
  }
}

// ------------------------------------------------------------------ launchers
static size_t row_smem(int n, int nseq, int elem) { return (size_t)sp_size(nseq * n) * 2 * elem; }

template <typename T, int RX>
cudaError_t launch_row(const RowArgs<T>& a0, cudaStream_t s) {
  // Small grids: fewer row pairs per CTA until the pass covers every SM (the partial-sum
  // passes keep their CTA count, which sizes the controller's reduction).  FP64 transforms
  // are bound by the FP64 units, so a pass on a few SMs is a few times slower.
  RowArgs<T> a = a0;
  bool partials = false;
  for (int q = 0; q < a.npairs && q < MJX_MAXPAIR; ++q)
    partials |= (a.pr[q].flags & (ROW_ERRNORM | ROW_ERRPAIR)) != 0;
  if (!partials)
    while (a.nseq > 1 && a.npairs * a.nrows / a.nseq < 152) a.nseq >>= 1;
  const int tps = a.n >= 16 ? a.n / 16 : 1;
  const int grid = a.npairs * a.nrows / a.nseq;
  if constexpr (sizeof(T) == 4) {
    if (a.n == 1024 && a.nseq <= 4) {  // one warp per 1024-point row
      row_kernel_w32<RX><<<grid, 32 * a.nseq, (size_t)a.nseq * 32 * 33 * sizeof(float2), s>>>(a);
      return cudaGetLastError();
    }
  }
  if constexpr (sizeof(T) == 8) {
    // short FP64 rows on a small grid (no error partials, whose CTA count is fixed): radix-4
    // transforms, n/4 threads per sequence, at most 256 threads per CTA, every SM covered
    // where possible.  Only when the radix-16 pass would run fewer than four warps per SM:
    // with more rows the extra passes of radix 4 cost more than the threads gain.
    if (!partials && a.n >= 4 && a.n <= 256 && (long long)a.npairs * a.nrows * tps < 152LL * 128) {
      RowArgs<T> b = a;
      const int tps4 = a.n / 4;
      while (b.nseq > 1 && b.nseq * tps4 > 256) b.nseq >>= 1;
      while (b.nseq > 1 && b.npairs * b.nrows / b.nseq < 152) b.nseq >>= 1;
      const int grid4 = b.npairs * b.nrows / b.nseq;
      row_kernel<T, RX, 0, true><<<grid4, b.nseq * tps4, row_smem(b.n, b.nseq, sizeof(T)), s>>>(b);
      return cudaGetLastError();
    }
  }
  const size_t smem = row_smem(a.n, a.nseq, sizeof(T));
  if constexpr (sizeof(T) == 4) {
    if (a.n == 4096 && a.nseq == 1) {
      row_kernel<T, RX, 12><<<grid, tps, smem, s>>>(a);
      return cudaGetLastError();
    }
    if (a.n == 2048 && a.nseq == 1) {
      row_kernel<T, RX, 11><<<grid, tps, smem, s>>>(a);
      return cudaGetLastError();
    }
  }
  row_kernel<T, RX><<<grid, a.nseq * tps, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_col(const ColArgs<T>& a0, cudaStream_t s) {
  ColArgs<T> a = a0;
  int maxout = 1;
  for (int j = 0; j < a.njobs; ++j) maxout = a.job[j].nout > maxout ? a.job[j].nout : maxout;
  const int tps = a.ny >= 16 ? a.ny / 16 : 1;
  // small grids: narrower tiles until the pass covers every SM (as launch_row)
  const long long planes = a.nplanes > 1 ? a.nplanes : 1;
  while (a.C > 1 && (long long)((a.ncols + a.C - 1) / a.C) * a.njobs * planes < 152) a.C >>= 1;
  if constexpr (sizeof(T) == 8) {
    // short FP64 columns on a small grid (fewer than four warps per SM at radix 16): radix-4
    // transforms, ny/4 threads per column, narrower tiles to stay within the thread cap
    if (a.ny >= 4 && a.ny <= 256 && (long long)a.ncols * a.njobs * planes * tps < 152LL * 128) {
      ColArgs<T> b = a;
      const int tps4 = a.ny / 4;
      while (b.C > 1 && b.C * maxout * tps4 > ColThreads<T>::v) b.C >>= 1;
      dim3 g4((b.ncols + b.C - 1) / b.C, b.njobs, b.nplanes > 1 ? b.nplanes : 1);
      const size_t sm4 = (size_t)sp_size(b.ny * b.C * maxout) * sizeof(cx<T>);
      col_kernel<T, true><<<g4, b.C * maxout * tps4, sm4, s>>>(b);
      return cudaGetLastError();
    }
  }
  dim3 grid((a.ncols + a.C - 1) / a.C, a.njobs, a.nplanes > 1 ? a.nplanes : 1);
  const size_t smem = (size_t)sp_size(a.ny * a.C * maxout) * sizeof(cx<T>);
  col_kernel<T><<<grid, a.C * maxout * tps, smem, s>>>(a);
  return cudaGetLastError();
}

#define MJX_INST_ROW(T, RX) template cudaError_t launch_row<T, RX>(const RowArgs<T>&, cudaStream_t);
MJX_INST_ROW(float, RX_NONE)
MJX_INST_ROW(float, RX_GRAY_SCOTT)
MJX_INST_ROW(float, RX_FISHER)
MJX_INST_ROW(double, RX_NONE)
MJX_INST_ROW(double, RX_GRAY_SCOTT)
MJX_INST_ROW(double, RX_FISHER)
template cudaError_t launch_col<float>(const ColArgs<float>&, cudaStream_t);
template cudaError_t launch_col<double>(const ColArgs<double>&, cudaStream_t);

// Column tile width: ~256 threads per output, capped by 512 threads and ~200 KB smem.
int col_tile(int ny, int ncols, int nout, int elem) {
  const int tps = ny >= 16 ? ny / 16 : 1;
  int C = 256 / tps;
  if (C < 1) C = 1;
  // at least one 32-byte sector of every row per CTA (4 FP32 / 2 FP64 complex columns)
  const int cmin = 32 / (2 * elem);
  if (C < cmin) C = cmin;
  if (C > 16) C = 16;
  const int cap = elem == 4 ? 1024 : 512;  // col_kernel thread limit per precision
  while (C > 1 && (C * nout * tps > cap || (size_t)sp_size(ny * C * nout) * 2 * elem > 200 * 1024)) C >>= 1;
  (void)ncols;
  return C;
}

// Raises a kernel's dynamic shared-memory limit to the device's opt-in maximum
// minus the kernel's static shared memory.
template <typename K>
static mjx_status raise_smem(K kernel, int optin) {
  cudaFuncAttributes fa;
  MJX_CUDA_TRY(cudaFuncGetAttributes(&fa, kernel));
  MJX_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    optin - (int)fa.sharedSizeBytes));
  return MJX_OK;
}

// Raise the dynamic shared-memory limit of every kernel once per CUDA context
// (function attributes belong to the context the kernels are loaded in).
mjx_status ensure_kernel_attrs() {
  static ContextOnce once;
  return once.run([]() -> mjx_status {
    int dev = 0, optin = 0;
    MJX_CUDA_TRY(cudaGetDevice(&dev));
    MJX_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    MJX_TRY(raise_smem(row_kernel<float, RX_NONE>, optin));
    MJX_TRY(raise_smem(row_kernel<float, RX_GRAY_SCOTT>, optin));
    MJX_TRY(raise_smem(row_kernel<float, RX_FISHER>, optin));
    MJX_TRY(raise_smem(row_kernel<double, RX_NONE>, optin));
    MJX_TRY(raise_smem(row_kernel<double, RX_GRAY_SCOTT>, optin));
    MJX_TRY(raise_smem(row_kernel<double, RX_FISHER>, optin));
    MJX_TRY(raise_smem(row_kernel<float, RX_NONE, 11>, optin));
    MJX_TRY(raise_smem(row_kernel<float, RX_GRAY_SCOTT, 11>, optin));
    MJX_TRY(raise_smem(row_kernel<float, RX_FISHER, 11>, optin));
    MJX_TRY(raise_smem(row_kernel<float, RX_NONE, 12>, optin));
    MJX_TRY(raise_smem(row_kernel<float, RX_GRAY_SCOTT, 12>, optin));
    MJX_TRY(raise_smem(row_kernel<float, RX_FISHER, 12>, optin));

    MJX_TRY(raise_smem(col_kernel<float>, optin));
    MJX_TRY(raise_smem(col_kernel<double>, optin));
    MJX_TRY(raise_smem(col_kernel<double, true>, optin));
    MJX_TRY(raise_smem(row_kernel<double, RX_NONE, 0, true>, optin));
    MJX_TRY(raise_smem(row_kernel<double, RX_GRAY_SCOTT, 0, true>, optin));
    MJX_TRY(raise_smem(row_kernel<double, RX_FISHER, 0, true>, optin));
    return MJX_OK;
  });
}

typedef CUresult (*PfnTensorMapEncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                            const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                            CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                            CUtensorMapFloatOOBfill);

mjx_status make_tmap_2d_f32(CUtensorMap* map, const void* base, unsigned long long inner, unsigned long long rows,
                            unsigned long long row_bytes, unsigned box_inner, unsigned box_rows) {
  static PfnTensorMapEncodeTiled encode = nullptr;
  static std::once_flag resolved;
  std::call_once(resolved, []() {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      encode = (PfnTensorMapEncodeTiled)f;
  });
  if (encode == nullptr) return cuda_status(cudaErrorNotSupported);
  // the copy rules: 16-byte aligned base and row stride, inner box a multiple of 16 bytes
  if (((uintptr_t)base & 15) || (row_bytes & 15) || ((box_inner * 4) & 15) || box_rows < 1 || box_rows > 256 ||
      box_inner < 1 || box_inner > 256)
    return MJX_BAD_ARG;
  const cuuint64_t dims[2] = {inner, rows};
  const cuuint64_t strides[1] = {row_bytes};
  const cuuint32_t box[2] = {box_inner, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box,
                            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return cuda_status(cudaErrorInvalidValue);
  return MJX_OK;
}

mjx_status make_tmap_3d_f32(CUtensorMap* map, const void* base, unsigned long long nx, unsigned long long ny,
                            unsigned long long nz, unsigned box_x, unsigned box_y) {
  static PfnTensorMapEncodeTiled encode = nullptr;
  static std::once_flag resolved;
  std::call_once(resolved, []() {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      encode = (PfnTensorMapEncodeTiled)f;
  });
  if (encode == nullptr) return cuda_status(cudaErrorNotSupported);
  if (((uintptr_t)base & 15) || ((nx * 4) & 15) || ((box_x * 4) & 15) || box_x < 1 || box_x > 256 || box_y < 1 ||
      box_y > 256)
    return MJX_BAD_ARG;
  const cuuint64_t dims[3] = {nx, ny, nz};
  const cuuint64_t strides[2] = {nx * 4, nx * ny * 4};
  const cuuint32_t box[3] = {box_x, box_y, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dims, strides, box,
                            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return cuda_status(cudaErrorInvalidValue);
  return MJX_OK;
}

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

mjx_status current_context_id(unsigned long long* id) {
  static PfnCtxGetCurrent get_current = nullptr;
  static PfnCtxGetId get_id = nullptr;
  static std::once_flag resolved;
  std::call_once(resolved, []() {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (PfnCtxGetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (PfnCtxGetId)f;
  });
  if (get_current == nullptr || get_id == nullptr) return cuda_status(cudaErrorNotSupported);
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != 0) return cuda_status(cudaErrorDeviceUninitialized);
  if (ctx == nullptr) {  // nothing current yet: the runtime's default is the primary context
    int dev = 0;
    MJX_CUDA_TRY(cudaGetDevice(&dev));
    MJX_CUDA_TRY(cudaSetDevice(dev));
    if (get_current(&ctx) != 0 || ctx == nullptr) return cuda_status(cudaErrorDeviceUninitialized);
  }
  if (get_id(ctx, id) != 0) return cuda_status(cudaErrorDeviceUninitialized);
  return MJX_OK;
}

static thread_local char g_last_error[256] = "";

void set_last_error(cudaError_t e, const char* file, int line) {
  const char* f = strrchr(file, '/');
  snprintf(g_last_error, sizeof(g_last_error), "%s (%s) at %s:%d", cudaGetErrorName(e),
           cudaGetErrorString(e), f ? f + 1 : file, line);
}

mjx_status check_grid(const mjx_grid2d* g) {
  if (g == nullptr) return MJX_BAD_ARG;
  if (ilog2_exact(g->nx) < 1 || ilog2_exact(g->ny) < 1) return MJX_BAD_SHAPE;
  if (g->nx > 4096 || g->ny > 4096) return MJX_BAD_SHAPE;
  if (!(g->dx > 0) || !(g->dy > 0)) return MJX_BAD_ARG;
  return MJX_OK;
}

int elem_size(int dtype) { return dtype == MJX_F32 ? 4 : (dtype == MJX_F64 ? 8 : 0); }

// Row pass over nfields single fields, pairing rows y and y + ny/2 of each field.
template <typename T>
RowArgs<T> field_rows(const mjx_grid2d* g, int nfields, const PlanView& pv, cx<T>* spec) {
  RowArgs<T> r;
  memset(&r, 0, sizeof(r));
  r.n = g->nx; r.log2n = ilog2_exact(g->nx); r.ldc = spec_ldc(g->nx);
  r.nrows = g->ny / 2; r.npairs = nfields; r.nseq = row_nseq(g->nx, r.nrows);
  r.rstride = g->nx; r.rin_sel = -1; r.rout_sel = -1;
  r.spec = spec; r.tw = (const cx<T>*)pv.twx; r.inv_scale = (T)1;
  for (int f = 0; f < nfields; ++f) {
    r.pr[f].ra = (long long)f * g->ny * g->nx;
    r.pr[f].rb = r.pr[f].ra + (long long)(g->ny / 2) * g->nx;
    r.pr[f].sa = (long long)f * g->ny * r.ldc;
    r.pr[f].sb = r.pr[f].sa + (long long)(g->ny / 2) * r.ldc;
    r.pr[f].hfac = 1.0;
  }
  return r;
}

template <typename T>
ColArgs<T> field_cols(const mjx_grid2d* g, const PlanView& pv, cx<T>* spec, int nout) {
  ColArgs<T> c;
  memset(&c, 0, sizeof(c));
  c.ny = g->ny; c.log2ny = ilog2_exact(g->ny); c.ncols = g->nx / 2 + 1; c.ldc = spec_ldc(g->nx);
  c.C = col_tile(g->ny, c.ncols, nout, sizeof(T));
  c.spec = spec; c.lamx = (const T*)pv.lamx; c.lamy = (const T*)pv.lamy;
  c.tw = (const cx<T>*)pv.twy; c.scale = (T)(1.0 / ((double)g->nx * (double)g->ny));
  return c;
}

template <typename T>
mjx_status spectral_apply(const void* plan, const mjx_grid2d* g, int nfields, const double* D,
                          double h, int mult, const T* in, T* out, void* ws, cudaStream_t s,
                          const double* vx = nullptr, const double* vy = nullptr,
                          const T* mtab = nullptr) {
  const PlanView pv = plan_view(plan, g->ny, g->nx, sizeof(T));
  cx<T>* spec = (cx<T>*)ws;
  const size_t fsz = (size_t)g->ny * g->nx;
  // gather the fields that diffuse (or, for MUL_ADVDIFF, move); pass the others through
  auto moves = [&](int f) { return vx && vy && (fabs(vx[f]) > 1e-14 || fabs(vy[f]) > 1e-14); };
  int idx[4], nd = 0;
  for (int f = 0; f < nfields; ++f) {
    if (mult == MUL_TABLE || D[f] > 1e-14 || moves(f)) idx[nd++] = f;
    else if (mult == MUL_LAP || mult == MUL_ADV_LAP)  // L u = 0
      MJX_CUDA_TRY(cudaMemsetAsync(out + f * fsz, 0, fsz * sizeof(T), s));
    else if (in != out)
      MJX_CUDA_TRY(cudaMemcpyAsync(out + f * fsz, in + f * fsz, fsz * sizeof(T), cudaMemcpyDeviceToDevice, s));
  }
  if (nd == 0) return MJX_OK;
  RowArgs<T> r = field_rows<T>(g, nd, pv, spec);
  for (int i = 0; i < nd; ++i) {
    const long long off = (long long)idx[i] * fsz;
    r.pr[i].ra += off - (long long)i * fsz;
    r.pr[i].rb += off - (long long)i * fsz;
  }
  r.rin[0] = in; r.rout[0] = out;
  for (int i = 0; i < nd; ++i) r.pr[i].flags = ROW_STORE_SPEC;
  MJX_CUDA_TRY((launch_row<T, RX_NONE>(r, s)));
  ColArgs<T> c = field_cols<T>(g, pv, spec, 1);
  c.hfixed = h; c.njobs = nd; c.mtab = mtab;
  c.kxs = 6.283185307179586476925286766559 / ((double)g->nx * g->dx);
  c.kys = 6.283185307179586476925286766559 / ((double)g->ny * g->dy);
  for (int i = 0; i < nd; ++i) {
    ColJob& j = c.job[i];
    j.sin = j.sout[0] = j.sout[1] = (long long)i * g->ny * spec_ldc(g->nx);
    j.D = D[idx[i]]; j.hfac[0] = j.hfac[1] = 1.0; j.pow[0] = j.pow[1] = 1; j.nout = 1; j.mul = mult;
    if (vx && vy) { j.vx = vx[idx[i]]; j.vy = vy[idx[i]]; }
  }
  MJX_CUDA_TRY(launch_col<T>(c, s));
  for (int i = 0; i < nd; ++i) r.pr[i].flags = ROW_LOAD_SPEC | ROW_STORE_REAL;
  MJX_CUDA_TRY((launch_row<T, RX_NONE>(r, s)));
  return MJX_OK;
}

template <typename T>
mjx_status fft_cn(const void* plan, const mjx_grid2d* g, double D, double dt, int n_steps,
                  const T* u_in, T* u_out, void* ws, cudaStream_t s) {
  const PlanView pv = plan_view(plan, g->ny, g->nx, sizeof(T));
  cx<T>* spec = (cx<T>*)ws;
  RowArgs<T> fwd = field_rows<T>(g, 1, pv, spec);
  RowArgs<T> inv = fwd;
  fwd.pr[0].flags = ROW_STORE_SPEC;
  inv.pr[0].flags = ROW_LOAD_SPEC | ROW_STORE_REAL;
  inv.rout[0] = u_out;
  ColArgs<T> c = field_cols<T>(g, pv, spec, 1);
  c.hfixed = dt; c.njobs = 1;
  c.job[0].D = D; c.job[0].hfac[0] = c.job[0].hfac[1] = 1.0; c.job[0].pow[0] = c.job[0].pow[1] = 1;
  c.job[0].nout = 1; c.job[0].mul = MUL_CN;
  if (n_steps <= 0) {
    if (u_in != u_out)
      MJX_CUDA_TRY(cudaMemcpyAsync(u_out, u_in, sizeof(T) * g->ny * g->nx, cudaMemcpyDeviceToDevice, s));
    return MJX_OK;
  }
  for (int i = 0; i < n_steps; ++i) {
    fwd.rin[0] = i == 0 ? u_in : u_out;
    MJX_CUDA_TRY((launch_row<T, RX_NONE>(fwd, s)));
    MJX_CUDA_TRY(launch_col<T>(c, s));
    MJX_CUDA_TRY((launch_row<T, RX_NONE>(inv, s)));
  }
  return MJX_OK;
}

// Fixed device scratch for mjx_fft_cn2d_noalloc.  It lives in the library's
// own device memory: every GPU that loads the library holds these bytes until
// the process exits.  Host code must not pass the symbol itself to a kernel
// (in host code it is only a stand-in); the device address comes from
// cudaGetSymbolAddress, once per CUDA context.
static __device__ __align__(256) unsigned char g_noalloc_scratch[MJX_NOALLOC_SCRATCH_BYTES];

// Scratch addresses by CUDA context.  A __device__ array has a separate
// address in every context that loads the library (the primary context, a
// driver-API context of an embedding host, the new primary context after
// cudaDeviceReset), so the lookup is cached per context id, never per device.
static std::mutex g_noalloc_mu;
static unsigned long long g_noalloc_ctx[32];
static void* g_noalloc_ptr[32];
static int g_noalloc_n = 0;

static mjx_status noalloc_scratch(void** out) {
  unsigned long long ctx = 0;
  MJX_TRY(current_context_id(&ctx));
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  const int m = g_noalloc_n < 32 ? g_noalloc_n : 32;
  for (int i = 0; i < m; ++i)
    if (g_noalloc_ctx[i] == ctx) {
      *out = g_noalloc_ptr[i];
      return MJX_OK;
    }
  void* p = nullptr;
  MJX_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  g_noalloc_ctx[g_noalloc_n % 32] = ctx;
  g_noalloc_ptr[g_noalloc_n % 32] = p;
  ++g_noalloc_n;
  *out = p;
  return MJX_OK;
}

}  // namespace mjx

using namespace mjx;

extern "C" {

const char* mjx_version(void) { return "moljax_gb300 0.1.0 (sm_103a)"; }

const char* mjx_last_error(void) { return g_last_error; }

const char* mjx_status_string(int st) {
  switch (st) {
    case MJX_OK: return "ok";
    case MJX_BAD_SHAPE: return "unsupported or inconsistent shape";
    case MJX_BAD_DTYPE: return "unsupported dtype";
    case MJX_NOT_FINITE: return "non-finite values";
    case MJX_MAX_ITERS: return "maximum steps/iterations reached";
    case MJX_DT_TOO_SMALL: return "time step below dt_min";
    case MJX_NK_FAILED: return "Newton-Krylov failed";
    case MJX_OOM: return "out of memory";
    case MJX_CUDA_ERROR: return "CUDA error";
    case MJX_BAD_ARG: return "bad argument";
    case MJX_WORKSPACE: return "workspace too small";
    default: return "unknown status";
  }
}

size_t mjx_spec2d_plan_bytes(int ny, int nx, int dtype) {
  const int e = elem_size(dtype);
  if (!e || ilog2_exact(nx) < 1 || ilog2_exact(ny) < 1) return 0;
  return plan_bytes(ny, nx, e);
}

size_t mjx_spec2d_ws_bytes(int ny, int nx, int nfields, int dtype) {
  const int e = elem_size(dtype);
  if (!e || ilog2_exact(nx) < 1 || ilog2_exact(ny) < 1 || nfields < 1) return 0;
  return (size_t)nfields * ny * spec_ldc(nx) * 2 * e;
}

mjx_status mjx_spec2d_plan_init(void* plan, const mjx_grid2d* g, int symbol, int dtype,
                                void* stream) {
  MJX_TRY(check_grid(g));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (plan == nullptr) return MJX_BAD_ARG;
  if (symbol != MJX_SYMBOL_FD && symbol != MJX_SYMBOL_SPECTRAL) return MJX_BAD_ARG;
  const int nx = g->nx, ny = g->ny, ldc = spec_ldc(nx);
  const size_t bytes = plan_bytes(ny, nx, e);
  std::vector<unsigned char> host(bytes, 0);
  PlanView pv = plan_view(host.data(), ny, nx, e);
  const double twopi = 6.283185307179586476925286766559;
  auto put_tw = [&](const void* dst, int n) {
    for (int j = 0; j < n; ++j) {
      const double ang = twopi * (double)j / (double)n;
      const double c = cos(ang), s = -sin(ang);
      if (e == 4) { float* p = (float*)dst; p[2 * j] = (float)c; p[2 * j + 1] = (float)s; }
      else { double* p = (double*)dst; p[2 * j] = c; p[2 * j + 1] = s; }
    }
  };
  // eigenvalue of the 1D periodic Laplacian for integer frequency m on n points of spacing d
  auto lam1 = [&](int m, int n, double d) {
    if (symbol == MJX_SYMBOL_FD) return (2.0 * cos(twopi * (double)m / (double)n) - 2.0) / (d * d);
    const double k = twopi * (double)m / ((double)n * d);
    return -k * k;
  };
  put_tw(pv.twx, nx);
  if (twx_count(nx, e) != nx) {  // the transposed copy for the one-warp 1024-point transform
    float* p = (float*)pv.twx;
    for (int k1 = 0; k1 < 32; ++k1)
      for (int l = 0; l < 32; ++l) {
        p[2 * (1024 + 32 * k1 + l)] = p[2 * (l * k1)];
        p[2 * (1024 + 32 * k1 + l) + 1] = p[2 * (l * k1) + 1];
      }
  }
  put_tw(pv.twy, ny);
  for (int kx = 0; kx < ldc; ++kx) {
    const double v = kx <= nx / 2 ? lam1(kx, nx, g->dx) : 0.0;
    if (e == 4) ((float*)pv.lamx)[kx] = (float)v; else ((double*)pv.lamx)[kx] = v;
  }
  for (int ky = 0; ky < ny; ++ky) {
    const int m = ky < ny / 2 ? ky : ky - ny;  // fftfreq order
    const double v = lam1(m, ny, g->dy);
    if (e == 4) ((float*)pv.lamy)[ky] = (float)v; else ((double*)pv.lamy)[ky] = v;
  }
  MJX_CUDA_TRY(cudaMemcpyAsync(plan, host.data(), bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  MJX_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return MJX_OK;
}

mjx_status mjx_spectral_apply2d(const void* plan, const mjx_grid2d* g, int dtype, int nfields,
                                const double* D, double h, int mult, const void* in, void* out,
                                void* ws, size_t ws_bytes, void* stream) {
  MJX_TRY(check_grid(g));
  if (nfields < 1 || nfields > 4 || D == nullptr || plan == nullptr || in == nullptr || out == nullptr)
    return MJX_BAD_ARG;
  if ((mult < MJX_MULT_SCALE || mult > MJX_MULT_EXP) && mult != MJX_MULT_LAP) return MJX_BAD_ARG;
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (ws == nullptr || ws_bytes < mjx_spec2d_ws_bytes(g->ny, g->nx, nfields, dtype)) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4) return spectral_apply<float>(plan, g, nfields, D, h, mult, (const float*)in, (float*)out, ws, s);
  return spectral_apply<double>(plan, g, nfields, D, h, mult, (const double*)in, (double*)out, ws, s);
}

mjx_status mjx_advdiff_op2d(const void* plan, const mjx_grid2d* g, int dtype, int nfields,
                            const double* D, const double* vx, const double* vy, double h, int op,
                            const void* in, void* out, void* ws, size_t ws_bytes, void* stream) {
  MJX_TRY(check_grid(g));
  if (nfields < 1 || nfields > 4 || D == nullptr || vx == nullptr || vy == nullptr || plan == nullptr ||
      in == nullptr || out == nullptr || op < 0 || op > 3)
    return MJX_BAD_ARG;
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (ws == nullptr || ws_bytes < mjx_spec2d_ws_bytes(g->ny, g->nx, nfields, dtype)) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  const int mul = op == 0 ? MUL_ADVDIFF : (op == 1 ? MUL_ADV_LAP : (op == 2 ? MUL_ADV_EXP : MUL_ADV_CN));
  if (e == 4)
    return spectral_apply<float>(plan, g, nfields, D, h, mul, (const float*)in, (float*)out, ws, s, vx, vy);
  return spectral_apply<double>(plan, g, nfields, D, h, mul, (const double*)in, (double*)out, ws, s, vx, vy);
}

mjx_status mjx_spectral_filter2d(const void* plan, const mjx_grid2d* g, int dtype, int nfields,
                                 const void* table, const void* in, void* out, void* ws, size_t ws_bytes,
                                 void* stream) {
  MJX_TRY(check_grid(g));
  if (nfields < 1 || nfields > 4 || plan == nullptr || table == nullptr || in == nullptr || out == nullptr)
    return MJX_BAD_ARG;
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (ws == nullptr || ws_bytes < mjx_spec2d_ws_bytes(g->ny, g->nx, nfields, dtype)) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  const double D[4] = {1.0, 1.0, 1.0, 1.0};
  if (e == 4)
    return spectral_apply<float>(plan, g, nfields, D, 1.0, MUL_TABLE, (const float*)in, (float*)out, ws, s,
                                 nullptr, nullptr, (const float*)table);
  return spectral_apply<double>(plan, g, nfields, D, 1.0, MUL_TABLE, (const double*)in, (double*)out, ws, s,
                                nullptr, nullptr, (const double*)table);
}

mjx_status mjx_advdiff_apply2d(const void* plan, const mjx_grid2d* g, int dtype, int nfields,
                               const double* D, const double* vx, const double* vy, double h,
                               const void* in, void* out, void* ws, size_t ws_bytes, void* stream) {
  MJX_TRY(check_grid(g));
  if (nfields < 1 || nfields > 4 || D == nullptr || vx == nullptr || vy == nullptr || plan == nullptr ||
      in == nullptr || out == nullptr)
    return MJX_BAD_ARG;
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (ws == nullptr || ws_bytes < mjx_spec2d_ws_bytes(g->ny, g->nx, nfields, dtype)) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4)
    return spectral_apply<float>(plan, g, nfields, D, h, MUL_ADVDIFF, (const float*)in, (float*)out, ws, s, vx, vy);
  return spectral_apply<double>(plan, g, nfields, D, h, MUL_ADVDIFF, (const double*)in, (double*)out, ws, s, vx, vy);
}

mjx_status mjx_fft_cn2d(const void* plan, const mjx_grid2d* g, int dtype, double D, double dt,
                        int n_steps, const void* u_in, void* u_out, void* ws, size_t ws_bytes,
                        void* stream) {
  MJX_TRY(check_grid(g));
  if (plan == nullptr || u_in == nullptr || u_out == nullptr || n_steps < 0) return MJX_BAD_ARG;
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (ws == nullptr || ws_bytes < mjx_spec2d_ws_bytes(g->ny, g->nx, 1, dtype)) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4) return fft_cn<float>(plan, g, D, dt, n_steps, (const float*)u_in, (float*)u_out, ws, s);
  return fft_cn<double>(plan, g, D, dt, n_steps, (const double*)u_in, (double*)u_out, ws, s);
}

// FFT-CN stepping for callers that cannot allocate device memory: the
// spectrum scratch is the fixed library buffer above instead of a workspace.
mjx_status mjx_fft_cn2d_noalloc(const void* plan, const mjx_grid2d* g, int dtype, double D, double dt,
                                int n_steps, const void* u_in, void* u_out, void* stream) {
  MJX_TRY(check_grid(g));
  if (plan == nullptr || u_in == nullptr || u_out == nullptr || n_steps < 0) return MJX_BAD_ARG;
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  // the spectrum of one field must fit the fixed scratch
  if (mjx_spec2d_ws_bytes(g->ny, g->nx, 1, dtype) > (size_t)MJX_NOALLOC_SCRATCH_BYTES) return MJX_WORKSPACE;
  void* ws = nullptr;
  MJX_TRY(noalloc_scratch(&ws));  // first call on a device: symbol lookup (no allocation)
  MJX_TRY(ensure_kernel_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4) return fft_cn<float>(plan, g, D, dt, n_steps, (const float*)u_in, (float*)u_out, ws, s);
  return fft_cn<double>(plan, g, D, dt, n_steps, (const double*)u_in, (double*)u_out, ws, s);
}

}  // extern "C"
