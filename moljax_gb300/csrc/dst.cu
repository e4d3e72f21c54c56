// Batched DST-I and the Dirichlet spectral solvers built on it
// (moljax/core/fft_nonperiodic.py:97-162, 244-330, 360-398).
//
// DST-I of x[0..N-1]:  X[k] = sum_n x[n] sin(pi (k+1)(n+1) / (N+1)).
// As in dst_I_fast, it is read off the DFT of the odd extension of length
// M = 2(N+1):  z = [0, x, 0, -reverse(x)],  X[k] = -Im(DFT(z))[k+1] / 2.
// Two real rows a, b ride one complex sequence z = a_ext + i b_ext:
// DFT(z)[k] = 2 S_b[k] - 2i S_a[k], so S_a = -Im/2 and S_b = Re/2.
//
// When M is a power of two the DFT is the shared-memory Stockham FFT; for any
// other M it is Bluestein's chirp-z form, a circular convolution of length
// L = 2^ceil(log2(2M - 1)) done with two FFTs of length L:
//   DFT_M(z)[k] = c[k] * IFFT_L( FFT_L(z c) * FFT_L(b) )[k],
//   c[n] = exp(-i pi n^2 / M),  b[n] = conj(c[|n|]) for |n| < M (periodic in L).
// The plan holds the length-L twiddles, c, FFT_L(b) / L and sin^2(pi k / (2(N+1))).
//
// One CTA transforms nseq row pairs (each sequence in its own shared-memory
// segment); the Helmholtz, Poisson and ETD1 solvers multiply the coefficients
// and run the same transform again (DST-I is its own inverse up to 2/(N+1)).
#include <math.h>
#include <string.h>

#include <vector>

#include "fft.cuh"

namespace mjx {

mjx_status ensure_kernel_attrs();
int elem_size(int dtype);
void set_last_error(cudaError_t e, const char* file, int line);

enum { DST_PLAIN = 0, DST_HELMHOLTZ = 1, DST_POISSON = 2, DST_ETD1 = 3 };

static inline size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

struct Dst1Geom {
  int N, M, L, log2L, bluestein;
  size_t tw, chirp, bhat, shift, total;  // plan byte offsets (per element size)
};

// kind 0: DST-I, DFT length M = 2(N+1); kind 1: DCT-II, M = 2N (plus the N phase factors)
static Dst1Geom dst1_geom(int N, int elem, int kind = 0) {
  Dst1Geom g;
  g.N = N;
  g.M = kind == 0 ? 2 * (N + 1) : 2 * N;
  g.bluestein = ilog2_exact(g.M) < 0;
  g.L = g.M;
  if (g.bluestein) {
    g.L = 1;
    while (g.L < 2 * g.M - 1) g.L <<= 1;
  }
  g.log2L = ilog2_exact(g.L);
  const size_t c = 2 * (size_t)elem;
  size_t o = 0;
  g.tw = o; o += a256(g.L * c);
  g.chirp = o; o += a256(g.M * c);
  g.bhat = o; o += a256(g.L * c);
  g.shift = o; o += kind == 0 ? 0 : a256(N * c);
  g.total = o;
  return g;
}

template <typename T>
struct Dst1Args {
  const T* x;       // rows of N values (mode ETD1: rows u, then rows of N(u) at offset nrows*N)
  T* out;
  const T* lam;     // per-mode symbol of length N (Helmholtz/Poisson: laplacian_symbol; ETD1: eigenvalues)
  const cx<T>* tw;  // length-L twiddles
  const cx<T>* chirp;
  const cx<T>* bhat;
  long long nrows;  // rows to transform
  int N, M, L, log2L, bluestein, nseq, mode;
  T scale;          // output scale of a plain transform
  double h, D;      // Helmholtz: dt, D; ETD1: dt
};

// DFT of length M of each sequence in buf (segments of L), in place in [0, M).
template <typename T>
__device__ void dft_m(const Dst1Args<T>& a, cx<T>* buf, int s_loc, int lt, int tps, int tid) {
  typedef cx<T> C;
  const int L = a.L;
  if (!a.bluestein) {
    fft_smem<T, false, false>(buf, L, a.log2L, a.nseq, L, 1, a.tw, tid);
    return;
  }
  const int base = s_loc * L;
  const bool active = s_loc < a.nseq;
  if (active)
    for (int j = lt; j < L; j += tps) {
      const C v = buf[sp(base + j)];
      buf[sp(base + j)] = j < a.M ? cmul(v, __ldg(&a.chirp[j])) : mk<C>((T)0, (T)0);
    }
  __syncthreads();
  fft_smem<T, false, false>(buf, L, a.log2L, a.nseq, L, 1, a.tw, tid);
  if (active)
    for (int j = lt; j < L; j += tps) buf[sp(base + j)] = cmul(buf[sp(base + j)], __ldg(&a.bhat[j]));
  __syncthreads();
  fft_smem<T, true, false>(buf, L, a.log2L, a.nseq, L, 1, a.tw, tid);
  if (active)
    for (int j = lt; j < a.M; j += tps) buf[sp(base + j)] = cmul(buf[sp(base + j)], __ldg(&a.chirp[j]));
  __syncthreads();
}

// odd extension of (va, vb) into the sequence: z[0] = z[N+1] = 0, z[j] = v[j-1], z[M-j] = -v[j-1]
template <typename T>
__device__ __forceinline__ void put_odd(cx<T>* buf, int base, int N, int M, int j, T va, T vb) {
  typedef cx<T> C;
  buf[sp(base + j + 1)] = mk<C>(va, vb);
  buf[sp(base + M - 1 - j)] = mk<C>(-va, -vb);
}

template <typename T>
__global__ void __launch_bounds__(256) dst1_kernel(const __grid_constant__ Dst1Args<T> a) {
  typedef cx<T> C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const int L = a.L, M = a.M, N = a.N;
  const int tps = L >= 16 ? L / 16 : 1;
  const int tid = threadIdx.x, s_loc = tid / tps, lt = tid % tps;
  const bool active = s_loc < a.nseq;
  const int base = s_loc * L;
  // sequence q holds rows 2q and 2q+1 (ETD1: row q of u and of N(u))
  const long long q = (long long)blockIdx.x * a.nseq + s_loc;
  const bool etd = a.mode == DST_ETD1;
  const long long ra = etd ? q : 2 * q, rb = etd ? a.nrows + q : 2 * q + 1;
  const long long nr_a = a.nrows;  // rows available for a (and for b, except ETD1)
  const bool has_a = active && ra < nr_a;
  const bool has_b = active && (etd ? q < a.nrows : rb < nr_a);

  if (active) {
    if (lt == 0) { buf[sp(base)] = mk<C>((T)0, (T)0); buf[sp(base + N + 1)] = mk<C>((T)0, (T)0); }
    for (int j = lt; j < N; j += tps) {
      const T va = has_a ? a.x[ra * N + j] : (T)0;
      const T vb = has_b ? a.x[rb * N + j] : (T)0;
      put_odd<T>(buf, base, N, M, j, va, vb);
    }
  }
  __syncthreads();
  dft_m<T>(a, buf, s_loc, lt, tps, tid);

  if (a.mode != DST_PLAIN) {
    // coefficients S_a, S_b -> multiplied coefficients, written back as a new odd extension
    T ca[16], cb[16];  // N <= 2047 and tps >= L/16 >= N/8, so each thread owns <= 16 entries
    int cnt = 0;
    if (active)
      for (int j = lt; j < N; j += tps, ++cnt) {
        const C Z = buf[sp(base + j + 1)];
        const T sa = (T)-0.5 * Z.y, sb = (T)0.5 * Z.x;
        const T lam = a.lam[j];
        const T inv = (T)2 / (T)(N + 1);
        if (a.mode == DST_HELMHOLTZ) {
          const T m = (T)1 / ((T)1 - (T)(a.h * a.D) * lam);  // fft_nonperiodic.py:327-330
          ca[cnt] = sa * m * inv; cb[cnt] = sb * m * inv;
        } else if (a.mode == DST_POISSON) {
          ca[cnt] = sa / lam * inv; cb[cnt] = sb / lam * inv;  // 265-271
        } else {  // ETD1 (360-398): exp(z) u^ + dt phi1(z) N^, z = dt * eigenvalue
          const T z = (T)a.h * lam;
          const T ez = exp(z);
          const T phi1 = fabs(z) < (T)1e-4 ? (T)1 + z / (T)2 + z * z / (T)6 : (ez - (T)1) / z;
          ca[cnt] = (ez * sa + (T)a.h * phi1 * sb) * inv; cb[cnt] = (T)0;
        }
      }
    __syncthreads();
    if (active) {
      cnt = 0;
      for (int j = lt; j < N; j += tps, ++cnt) put_odd<T>(buf, base, N, M, j, ca[cnt], cb[cnt]);
      if (lt == 0) {
        buf[sp(base)] = mk<C>((T)0, (T)0);
        buf[sp(base + N + 1)] = mk<C>((T)0, (T)0);
      }
    }
    __syncthreads();
    dft_m<T>(a, buf, s_loc, lt, tps, tid);
  }

  if (active) {
    const T sc = a.mode == DST_PLAIN ? a.scale : (T)1;
    for (int j = lt; j < N; j += tps) {
      const C Z = buf[sp(base + j + 1)];
      if (has_a) a.out[ra * N + j] = (T)-0.5 * Z.y * sc;
      if (has_b && !etd) a.out[rb * N + j] = (T)0.5 * Z.x * sc;
    }
  }
}

// ---------------------------------------------------------------- DCT-II (orthonormal)
// jax.scipy.fft.dct(x, type=2, norm='ortho') and its inverse along rows of N values
// (the Neumann solvers, fft_nonperiodic.py:274-305, 333-355, 401-437).  Forward: the
// even extension v = [x, reverse(x)] of length M = 2N gives
//   2 sum_n x[n] cos(pi k (2n+1) / 2N) = Re(e^{-i pi k / 2N} DFT(v)[k]),
// and for a row pair z = a + i b the real and imaginary parts separate.  Inverse: the
// Hermitian spectrum Z[0] = w0 X0, Z[k] = (wk/2) e^{+i pi k/2N} Xk, Z[2N-k] = conj,
// transformed back (inverse DFT = conj(DFT(conj(.)))), returns both rows of a pair.
enum { DCT_FWD = 0, DCT_INV = 1, DCT_HELMHOLTZ = 2, DCT_POISSON = 3, DCT_ETD1 = 4 };

template <typename T>
__global__ void __launch_bounds__(256) dct2_kernel(const __grid_constant__ Dst1Args<T> a,
                                                   const cx<T>* __restrict__ shift) {
  typedef cx<T> C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const int L = a.L, M = a.M, N = a.N;
  const int tps = L >= 16 ? L / 16 : 1;
  const int tid = threadIdx.x, s_loc = tid / tps, lt = tid % tps;
  const bool active = s_loc < a.nseq;
  const int base = s_loc * L;
  const long long q = (long long)blockIdx.x * a.nseq + s_loc;
  const bool etd = a.mode == DCT_ETD1;
  const long long ra = etd ? q : 2 * q, rb = etd ? a.nrows + q : 2 * q + 1;
  const bool has_a = active && ra < a.nrows;
  const bool has_b = active && (etd ? q < a.nrows : rb < a.nrows);
  const T f0 = (T)sqrt(0.25 / N), fk = (T)sqrt(0.5 / N);  // forward ortho factors
  const T w0 = (T)sqrt(1.0 / N), wk = (T)sqrt(2.0 / N);   // inverse ortho factors
  T ca[16], cb[16];  // this thread's coefficients k = lt + m tps (N <= 8 tps)

  if (a.mode != DCT_INV) {
    if (active)
      for (int j = lt; j < N; j += tps) {
        const T va = has_a ? a.x[ra * N + j] : (T)0, vb = has_b ? a.x[rb * N + j] : (T)0;
        buf[sp(base + j)] = mk<C>(va, vb);
        buf[sp(base + M - 1 - j)] = mk<C>(va, vb);
      }
    __syncthreads();
    dft_m<T>(a, buf, s_loc, lt, tps, tid);
    int m = 0;
    if (active)
      for (int k = lt; k < N; k += tps, ++m) {
        const C t = cmul(buf[sp(base + k)], __ldg(&shift[k]));
        const T f = k == 0 ? f0 : fk;
        ca[m] = t.x * f; cb[m] = t.y * f;
      }
  } else {
    int m = 0;
    if (active)
      for (int k = lt; k < N; k += tps, ++m) {
        ca[m] = has_a ? a.x[ra * N + k] : (T)0;
        cb[m] = has_b ? a.x[rb * N + k] : (T)0;
      }
  }
  if (a.mode == DCT_FWD) {
    int m = 0;
    if (active)
      for (int k = lt; k < N; k += tps, ++m) {
        if (has_a) a.out[ra * N + k] = ca[m] * a.scale;
        if (has_b) a.out[rb * N + k] = cb[m] * a.scale;
      }
    return;
  }
  if (a.mode != DCT_INV) {  // spectral multipliers
    int m = 0;
    if (active)
      for (int k = lt; k < N; k += tps, ++m) {
        const T lam = a.lam[k];
        if (a.mode == DCT_HELMHOLTZ) {  // fft_nonperiodic.py:352-355
          const T mu = (T)1 / ((T)1 - (T)(a.h * a.D) * lam);
          ca[m] *= mu; cb[m] *= mu;
        } else if (a.mode == DCT_POISSON) {  // 297-303: the null mode is set to zero
          const bool null = fabs(lam) < (T)1e-14;
          ca[m] = null ? (T)0 : ca[m] / lam; cb[m] = null ? (T)0 : cb[m] / lam;
        } else {  // ETD1 (431-437): exp(z) u^ + dt phi1(z) N^
          const T z = (T)a.h * lam, ez = exp(z);
          const T phi1 = fabs(z) < (T)1e-4 ? (T)1 + z / (T)2 + z * z / (T)6 : (ez - (T)1) / z;
          ca[m] = ez * ca[m] + (T)a.h * phi1 * cb[m];
          cb[m] = (T)0;
        }
      }
  }
  // inverse: conj of the Hermitian spectrum, forward DFT, conj back
  __syncthreads();
  if (active) {
    for (int j = lt; j < L; j += tps) buf[sp(base + j)] = mk<C>((T)0, (T)0);
  }
  __syncthreads();
  if (active) {
    int m = 0;
    for (int k = lt; k < N; k += tps, ++m) {
      const C X = mk<C>(ca[m], cb[m]);
      if (k == 0) {
        buf[sp(base)] = cconj(cscale(X, w0));
      } else {
        const C sh = __ldg(&shift[k]);         // e^{-i pi k / 2N}
        const C zk = cscale(cmulc(X, sh), (T)0.5 * wk);  // (wk/2) e^{+i..} X
        const C zm = cscale(cmul(X, sh), (T)0.5 * wk);   // (wk/2) e^{-i..} X
        buf[sp(base + k)] = cconj(zk);
        buf[sp(base + M - k)] = cconj(zm);
      }
    }
  }
  __syncthreads();
  dft_m<T>(a, buf, s_loc, lt, tps, tid);
  if (active) {
    const T sc = a.mode == DCT_INV ? a.scale : (T)1;
    for (int j = lt; j < N; j += tps) {
      const C z = buf[sp(base + j)];  // conj(DFT(conj Z)) = inverse DFT of Z
      if (has_a) a.out[ra * N + j] = z.x * sc;
      if (has_b && !etd) a.out[rb * N + j] = -z.y * sc;
    }
  }
}

// In-place iterative radix-2 FFT on the host (FP64), for the Bluestein filter.
static void host_fft(std::vector<double>& re, std::vector<double>& im) {
  const int n = (int)re.size();
  for (int i = 1, j = 0; i < n; ++i) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) { std::swap(re[i], re[j]); std::swap(im[i], im[j]); }
  }
  const double twopi = 6.283185307179586476925286766559;
  for (int len = 2; len <= n; len <<= 1) {
    for (int i = 0; i < n; i += len)
      for (int k = 0; k < len / 2; ++k) {
        const double ang = -twopi * k / len;
        const double wr = cos(ang), wi = sin(ang);
        const int u = i + k, v = i + k + len / 2;
        const double xr = re[v] * wr - im[v] * wi, xi = re[v] * wi + im[v] * wr;
        re[v] = re[u] - xr; im[v] = im[u] - xi;
        re[u] += xr; im[u] += xi;
      }
  }
}

template <typename T>
static mjx_status dst1_run(const void* plan, int N, long long nrows, int mode, const T* x, T* out,
                           const T* lam, double h, double D, T scale, cudaStream_t s) {
  const Dst1Geom g = dst1_geom(N, sizeof(T));
  const char* p = (const char*)plan;
  Dst1Args<T> a;
  memset(&a, 0, sizeof(a));
  a.x = x; a.out = out; a.lam = lam;
  a.tw = (const cx<T>*)(p + g.tw); a.chirp = (const cx<T>*)(p + g.chirp); a.bhat = (const cx<T>*)(p + g.bhat);
  a.nrows = nrows; a.N = N; a.M = g.M; a.L = g.L; a.log2L = g.log2L; a.bluestein = g.bluestein;
  a.mode = mode; a.scale = scale; a.h = h; a.D = D;
  const int tps = g.L >= 16 ? g.L / 16 : 1;
  a.nseq = 256 / tps;
  if (a.nseq < 1) a.nseq = 1;
  const long long nseq_total = mode == DST_ETD1 ? nrows : (nrows + 1) / 2;
  if (nseq_total == 0) return MJX_OK;
  const long long nblk = (nseq_total + a.nseq - 1) / a.nseq;
  if (nblk > 0x7fffffffLL) return MJX_BAD_SHAPE;
  const size_t smem = (size_t)sp_size(a.nseq * g.L) * sizeof(cx<T>);
  dst1_kernel<T><<<(unsigned)nblk, 256, smem, s>>>(a);
  return cuda_status(cudaGetLastError());
}

static mjx_status dst1_attrs() {
  static ContextOnce once;
  return once.run([]() -> mjx_status {
    int dev = 0, optin = 0;
    MJX_CUDA_TRY(cudaGetDevice(&dev));
    MJX_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    MJX_CUDA_TRY(cudaFuncSetAttribute(dst1_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    MJX_CUDA_TRY(cudaFuncSetAttribute(dst1_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    MJX_CUDA_TRY(cudaFuncSetAttribute(dct2_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    MJX_CUDA_TRY(cudaFuncSetAttribute(dct2_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    return MJX_OK;
  });
}

template <typename T>
static mjx_status dct2_run(const void* plan, int n, long long nrows, int mode, const T* x, T* out,
                           const T* lam, double h, double D, T scale, cudaStream_t s) {
  const Dst1Geom g = dst1_geom(n, sizeof(T), 1);
  const char* p = (const char*)plan;
  Dst1Args<T> a;
  memset(&a, 0, sizeof(a));
  a.x = x; a.out = out; a.lam = lam;
  a.tw = (const cx<T>*)(p + g.tw); a.chirp = (const cx<T>*)(p + g.chirp); a.bhat = (const cx<T>*)(p + g.bhat);
  a.nrows = nrows; a.N = n; a.M = g.M; a.L = g.L; a.log2L = g.log2L; a.bluestein = g.bluestein;
  a.mode = mode; a.scale = scale; a.h = h; a.D = D;
  const int tps = g.L >= 16 ? g.L / 16 : 1;
  a.nseq = 256 / tps;
  if (a.nseq < 1) a.nseq = 1;
  const long long nseq_total = mode == DCT_ETD1 ? nrows : (nrows + 1) / 2;
  if (nseq_total == 0) return MJX_OK;
  const long long nblk = (nseq_total + a.nseq - 1) / a.nseq;
  if (nblk > 0x7fffffffLL) return MJX_BAD_SHAPE;
  const size_t smem = (size_t)sp_size(a.nseq * g.L) * sizeof(cx<T>);
  dct2_kernel<T><<<(unsigned)nblk, 256, smem, s>>>(a, (const cx<T>*)(p + g.shift));
  return cuda_status(cudaGetLastError());
}

// host-side tables of a length-N transform of the given kind (twiddles; Bluestein chirp and
// filter when M is not a power of two; DCT phase factors e^{-i pi k / 2N})
static void trig_tables(std::vector<unsigned char>& host, const Dst1Geom& g, int e, int kind) {
  const double twopi = 6.283185307179586476925286766559, pi = 0.5 * twopi;
  auto put = [&](size_t off, int i, double re, double im) {
    if (e == 4) { float* q = (float*)(host.data() + off); q[2 * i] = (float)re; q[2 * i + 1] = (float)im; }
    else { double* q = (double*)(host.data() + off); q[2 * i] = re; q[2 * i + 1] = im; }
  };
  for (int j = 0; j < g.L; ++j) put(g.tw, j, cos(twopi * j / g.L), -sin(twopi * j / g.L));
  if (g.bluestein) {
    // c[n] = exp(-i pi n^2 / M), with n^2 reduced mod 2M to keep the angle exact
    std::vector<double> cre(g.M), cim(g.M);
    for (int j = 0; j < g.M; ++j) {
      const long long r = ((long long)j * j) % (2LL * g.M);
      cre[j] = cos(pi * (double)r / g.M);
      cim[j] = -sin(pi * (double)r / g.M);
      put(g.chirp, j, cre[j], cim[j]);
    }
    std::vector<double> bre(g.L, 0.0), bim(g.L, 0.0);
    for (int j = 0; j < g.M; ++j) {
      bre[j] = cre[j]; bim[j] = -cim[j];
      if (j > 0) { bre[g.L - j] = cre[j]; bim[g.L - j] = -cim[j]; }
    }
    host_fft(bre, bim);
    for (int j = 0; j < g.L; ++j) put(g.bhat, j, bre[j] / g.L, bim[j] / g.L);
  }
  if (kind == 1)
    for (int k = 0; k < g.N; ++k) put(g.shift, k, cos(pi * k / (2.0 * g.N)), -sin(pi * k / (2.0 * g.N)));
}

}  // namespace mjx

using namespace mjx;

extern "C" {

// lengths the one-CTA transform handles: the FFT length L is at most 4096
static bool dst1_size_ok(int n) { return n >= 1 && n <= 2047 && dst1_geom(n, 8).L <= 4096; }

size_t mjx_dst1_plan_bytes(int n, int dtype) {
  const int e = elem_size(dtype);
  if (!e || !dst1_size_ok(n)) return 0;
  return dst1_geom(n, e).total;
}

mjx_status mjx_dst1_plan_init(void* plan, int n, int dtype, void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (plan == nullptr) return MJX_BAD_ARG;
  if (!dst1_size_ok(n)) return MJX_BAD_SHAPE;
  const Dst1Geom g = dst1_geom(n, e);
  std::vector<unsigned char> host(g.total, 0);
  trig_tables(host, g, e, 0);
  MJX_CUDA_TRY(cudaMemcpyAsync(plan, host.data(), g.total, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  MJX_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return MJX_OK;
}

mjx_status mjx_dst1(const void* plan, int n, long long nrows, int dtype, int mode, const void* x,
                    void* out, const void* lam, double h, double D, double scale, void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!dst1_size_ok(n) || nrows < 0) return MJX_BAD_SHAPE;
  if (plan == nullptr || x == nullptr || out == nullptr) return MJX_BAD_ARG;
  if (mode < DST_PLAIN || mode > DST_ETD1 || (mode != DST_PLAIN && lam == nullptr)) return MJX_BAD_ARG;
  MJX_TRY(dst1_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4)
    return dst1_run<float>(plan, n, nrows, mode, (const float*)x, (float*)out, (const float*)lam, h, D,
                           (float)scale, s);
  return dst1_run<double>(plan, n, nrows, mode, (const double*)x, (double*)out, (const double*)lam, h, D,
                          scale, s);
}

// DCT-II lengths: 2N a power of two up to 4096 or Bluestein with L <= 4096 (N <= 1024)
static bool dct2_size_ok(int n) { return n >= 1 && n <= 2048 && dst1_geom(n, 8, 1).L <= 4096; }

size_t mjx_dct2_plan_bytes(int n, int dtype) {
  const int e = elem_size(dtype);
  if (!e || !dct2_size_ok(n)) return 0;
  return dst1_geom(n, e, 1).total;
}

mjx_status mjx_dct2_plan_init(void* plan, int n, int dtype, void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (plan == nullptr) return MJX_BAD_ARG;
  if (!dct2_size_ok(n)) return MJX_BAD_SHAPE;
  const Dst1Geom g = dst1_geom(n, e, 1);
  std::vector<unsigned char> host(g.total, 0);
  trig_tables(host, g, e, 1);
  MJX_CUDA_TRY(cudaMemcpyAsync(plan, host.data(), g.total, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  MJX_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return MJX_OK;
}

mjx_status mjx_dct2(const void* plan, int n, long long nrows, int dtype, int mode, const void* x,
                    void* out, const void* lam, double h, double D, double scale, void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!dct2_size_ok(n) || nrows < 0) return MJX_BAD_SHAPE;
  if (plan == nullptr || x == nullptr || out == nullptr) return MJX_BAD_ARG;
  if (mode < DCT_FWD || mode > DCT_ETD1 || (mode >= DCT_HELMHOLTZ && lam == nullptr)) return MJX_BAD_ARG;
  MJX_TRY(dst1_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4)
    return dct2_run<float>(plan, n, nrows, mode, (const float*)x, (float*)out, (const float*)lam, h, D,
                           (float)scale, s);
  return dct2_run<double>(plan, n, nrows, mode, (const double*)x, (double*)out, (const double*)lam, h, D,
                          scale, s);
}

}  // extern "C"
