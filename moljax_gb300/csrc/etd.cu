// Exponential time differencing on a periodic box: ETDRK4 (Cox-Matthews),
// ETD1 (exponential Euler) and ETD2 (exponential Adams-Bashforth 2).
//
// Restates benchmarks/benchmark_gray_scott.py:336-417.  Coefficients E, E2,
// Q, f1, f2, f3 per Fourier mode come from the M = 32 point contour mean
// (compute_etdrk4_coeffs, 336-356), evaluated once on the GPU in FP64 (the
// contour sums cancel catastrophically in FP32) and stored in the state
// precision.  One step (etdrk4_step, 369-417) is 4 column passes that fuse
// forward FFT_y -> stage combination -> inverse FFT_y, and 4 row passes that
// fuse c2r -> N(u, v) -> r2c:
//
//   C1  N^u = F(ZN); a^ = E2 U^ + Q N^u; store N^u, a^; ZX = F^-1 a^
//   R1  ZX <- r2c N(c2r ZX)                                   (N^a in row space)
//   C2  N^a = F(ZX); b^ = E2 U^ + Q N^a; S = N^a; ZX = F^-1 b^
//   R2  ZX <- r2c N(c2r ZX)
//   C3  N^b = F(ZX); c^ = E2 a^ + Q (2 N^b - N^u); S += N^b; ZX = F^-1 c^
//   R3  ZX <- r2c N(c2r ZX)
//   C4  N^c = F(ZX); U^' = E U^ + f1 N^u + f2 S + f3 N^c; store U^'; ZU = F^-1 U^'
//   R4  ZN <- r2c N(c2r ZU)                                   (next step's N^u)
//
// ZU/ZN/ZX are row spectra (FFT along x only); U^, N^u, a^, S full 2D spectra.
// f2 is stored pre-multiplied by f2_factor: 2 gives Cox-Matthews / Kassam-
// Trefethen ETDRK4 (the library's b2 = 2 phi2 - 4 phi3, fft_integrators.py:110);
// 1 reproduces the benchmark script, whose update uses f2 (N^a + N^b) without
// the factor 2 (benchmark_gray_scott.py:415).
//
// The library form (moljax/core/fft_integrators.py) takes its coefficients from
// the phi functions instead (39-116: Taylor series below |z| = 1e-4, closed form
// above), and adds ETD1 (119-175) and ETD2 (178-249):
//
//   ETD1  N^ = F(ZN); U^' = E U^ + dt phi1 N^; store U^'; ZU = F^-1 U^'     + R4
//   ETD2  N^ = F(ZN); U^' = E U^ + dt phi1 N^ + dt phi2 (N^ - N^prev);
//         N^prev <- N^; store U^'; ZU = F^-1 U^'                            + R4
//
// (the first ETD2 step without a previous N is an ETD1 step that keeps N^, as
// etd2_step falls back to etd1_step, 207-209).  The nonlinear term is the
// coupled Gray-Scott reaction on (u, v), the logistic term r u (1 - u) on each
// field, or zero; one field pairs rows y and y + ny/2 in the row passes.
#include <math.h>
#include <string.h>

#include "spectral.cuh"

namespace mjx {

mjx_status ensure_kernel_attrs();
mjx_status check_grid(const mjx_grid2d* g);
int elem_size(int dtype);
void set_last_error(cudaError_t e, const char* file, int line);

// ------------------------------------------------------------------ FP64 contour coefficients
struct zc { double x, y; };
__device__ __forceinline__ zc zadd(zc a, zc b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ zc zsub(zc a, zc b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ zc zmul(zc a, zc b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ zc zsc(zc a, double s) { return {a.x * s, a.y * s}; }
__device__ __forceinline__ zc zdiv(zc a, zc b) {
  const double d = b.x * b.x + b.y * b.y;
  return {(a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d};
}
__device__ __forceinline__ zc zexp(zc a) {
  double s, c;
  sincos(a.y, &s, &c);
  const double e = exp(a.x);
  return {e * c, e * s};
}

// phi functions exactly as moljax/core/fft_integrators.py:39-78 evaluates them:
// a cubic Taylor polynomial for |z| < 1e-4, the closed form otherwise.
__device__ __forceinline__ double phi1_ref(double z) {
  if (fabs(z) < 1e-4) return 1.0 + z / 2.0 + z * z / 6.0 + z * z * z / 24.0;
  return (exp(z) - 1.0) / z;
}
__device__ __forceinline__ double phi2_ref(double z) {
  if (fabs(z) < 1e-4) return 0.5 + z / 6.0 + z * z / 24.0 + z * z * z / 120.0;
  return (exp(z) - 1.0 - z) / (z * z);
}
__device__ __forceinline__ double phi3_ref(double z) {
  if (fabs(z) < 1e-4) return 1.0 / 6.0 + z / 24.0 + z * z / 120.0 + z * z * z / 720.0;
  return (exp(z) - 1.0 - z - z * z / 2.0) / (z * z * z);
}

enum { FORM_CONTOUR_RK4 = 0, FORM_PHI_RK4 = 1, FORM_PHI_ETD12 = 2 };

// tab layout: [field][coef 0..5][ky][ldc]
//   RK4 forms: E, E2, Q, f1, f2, f3;   ETD1/ETD2: E, dt phi1, dt phi2
// xonly: the symbol has no y part (each row an independent 1D problem).
template <typename T>
__global__ void etd_coeff_kernel(T* tab, int ny, int nx, int ldc, int symbol, int xonly, double dy,
                                 double dx, double D0, double D1, int nf, double dt, int M,
                                 double f2_factor, int form) {
  const long long per = (long long)ny * ldc;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < per * nf;
       i += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(i / per);
    const long long r = i - f * per;
    const int ky = (int)(r / ldc), kx = (int)(r - (long long)ky * ldc);
    const int my = xonly ? 0 : (ky < ny / 2 ? ky : ky - ny);
    double lam;
    if (kx > nx / 2) {
      lam = 0.0;
    } else if (symbol == MJX_SYMBOL_FD) {
      lam = (2.0 * cospi(2.0 * kx / nx) - 2.0) / (dx * dx) + (2.0 * cospi(2.0 * my / ny) - 2.0) / (dy * dy);
    } else {
      const double kxx = 6.283185307179586476925 * kx / (nx * dx), kyy = 6.283185307179586476925 * my / (ny * dy);
      lam = -(kxx * kxx + kyy * kyy);
    }
    const double z = dt * (f == 0 ? D0 : D1) * lam;
    T* t = tab + (long long)f * 6 * per + r;
    if (form == FORM_PHI_ETD12) {
      t[0 * per] = (T)exp(z);
      t[1 * per] = (T)(dt * phi1_ref(z));
      t[2 * per] = (T)(dt * phi2_ref(z));
      continue;
    }
    if (form == FORM_PHI_RK4) {
      // _etdrk4_coefficients (fft_integrators.py:81-116): a = E2 u + (dt/2) phi1(z/2) N,
      // u' = E u + dt (b1 N + b2 (Na + Nb) + b4 Nc)
      const double p1 = phi1_ref(z), p2 = phi2_ref(z), p3 = phi3_ref(z);
      t[0 * per] = (T)exp(z);
      t[1 * per] = (T)exp(z / 2.0);
      t[2 * per] = (T)(dt / 2.0 * phi1_ref(z / 2.0));
      t[3 * per] = (T)(dt * (p1 - 3.0 * p2 + 4.0 * p3));
      t[4 * per] = (T)(dt * (2.0 * p2 - 4.0 * p3));
      t[5 * per] = (T)(dt * (-p2 + 4.0 * p3));
      continue;
    }
    zc Q = {0, 0}, f1 = {0, 0}, f2 = {0, 0}, f3 = {0, 0};
    for (int j = 1; j <= M; ++j) {
      double s, c;
      sincospi((j - 0.5) / M, &s, &c);
      const zc LR = {z + c, s};
      const zc eLR = zexp(LR), eLR2 = zexp(zsc(LR, 0.5));
      const zc LR2 = zmul(LR, LR), LR3 = zmul(LR2, LR);
      Q = zadd(Q, zdiv(zsub(eLR2, {1, 0}), LR));
      // (-4 - LR + e^LR (4 - 3 LR + LR^2)) / LR^3
      f1 = zadd(f1, zdiv(zadd(zsub({-4, 0}, LR), zmul(eLR, zadd(zsub({4, 0}, zsc(LR, 3)), LR2))), LR3));
      // (2 + LR + e^LR (-2 + LR)) / LR^3
      f2 = zadd(f2, zdiv(zadd(zadd({2, 0}, LR), zmul(eLR, zadd({-2, 0}, LR))), LR3));
      // (-4 - 3 LR - LR^2 + e^LR (4 - LR)) / LR^3
      f3 = zadd(f3, zdiv(zadd(zsub(zsub({-4, 0}, zsc(LR, 3)), LR2), zmul(eLR, zsub({4, 0}, LR))), LR3));
    }
    const double w = dt / M;
    t[0 * per] = (T)exp(z);
    t[1 * per] = (T)exp(0.5 * z);
    t[2 * per] = (T)(w * Q.x);
    t[3 * per] = (T)(w * f1.x);
    t[4 * per] = (T)(f2_factor * w * f2.x);
    t[5 * per] = (T)(w * f3.x);
  }
}

// ------------------------------------------------------------------ stage column pass
enum { E0 = 0, E1 = 1, E2S = 2, E3 = 3, E4 = 4, E5 = 5, E6 = 6, E7 = 7 };  // E5 ETD1, E6 ETD1 + keep N^, E7 ETD2

template <typename T> struct EArgs {
  int ny, log2ny, ncols, ldc, C, njobs;
  cx<T>* zu; cx<T>* zn; cx<T>* zx;
  cx<T>* uh; cx<T>* nu; cx<T>* ah; cx<T>* ss;
  const T* tab;
  long long fs;  // elements per field in every buffer (ny * ldc)
  const cx<T>* tw;
  T scale;
  int type;
  int pad;
};

// One CTA: C adjacent kx columns of one field (E1 transforms two inputs per column).
// FP32 CTAs take up to 1024 threads, so that at ny = 4096 a CTA still covers 2-4
// columns and each warp access reads whole 32-byte sectors of the row-major spectra;
// FP64 keeps 512 threads (its butterflies need the registers).
template <typename T> struct EThreads { static constexpr int v = sizeof(T) == 4 ? 1024 : 512; };

// The stage type is a template argument, so that each instance holds only its own operands.
// R4: radix-4 column transforms with ny/4 threads per column (short FP64 columns).
template <typename T, int TYPE, bool R4 = false>
__global__ void __launch_bounds__(EThreads<T>::v, 1) etd_col_kernel(const __grid_constant__ EArgs<T> a) {
  typedef cx<T> Cx;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cx* buf = reinterpret_cast<Cx*>(smem_raw);
  const int f = blockIdx.y;
  constexpr int type = TYPE;
  const int Cn = a.C, W = Cn;
  const int lc = __ffs(Cn) - 1;  // the tile width is a power of two (halved from 16)
  const int kx0 = blockIdx.x * Cn;
  const int ny = a.ny, tid = threadIdx.x, nth = blockDim.x;
  const long long ldc = a.ldc, fo = (long long)f * a.fs, per = a.fs;
  const T* tab = a.tab + (long long)f * 6 * per;

  // load the row-spectrum tile: E0 ZU, E1 and E5-E7 ZN, E2-E4 ZX
  const Cx* in0 = type == E0 ? a.zu : ((type == E1 || type >= E5) ? a.zn : a.zx);
  for (int e = tid; e < ny * Cn; e += nth) {
    const int ky = e >> lc, c = e & (Cn - 1), kx = kx0 + c;
    buf[sp(ky * W + c)] = kx < a.ncols ? in0[fo + ky * ldc + kx] : mk<Cx>((T)0, (T)0);
  }
  __syncthreads();
  if (R4) fft_smem_r4<T, false, true>(buf, ny, a.log2ny, Cn, 1, W, a.tw, tid);
  else fft_smem<T, false, true>(buf, ny, a.log2ny, Cn, 1, W, a.tw, tid);

  // The stage combination, two elements per thread at a time: the operands are read and
  // written in place, so the compiler cannot issue a later element's loads before an
  // earlier element's stores; loading both elements' operands first doubles the loads in
  // flight of the one CTA per SM (the 4096-row passes wait on DRAM).
  const T* tb0 = tab + 0 * per;
  const T* tb1 = tab + 1 * per;
  const T* tb2 = tab + 2 * per;
  const T* tb3 = tab + 3 * per;
  const T* tb4 = tab + 4 * per;
  const T* tb5 = tab + 5 * per;
  const Cx zero = mk<Cx>((T)0, (T)0);
  for (int e0 = tid; e0 < ny * Cn; e0 += 2 * nth) {
    Cx x[2], u[2], nu[2], s3[2];
    T c0[2], c1[2], c2[2], c3[2];
    long long g[2];
    int sidx[2];
    bool ok[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int e = e0 + h * nth;
      const int ky = e >> lc, c = e & (Cn - 1), kx = kx0 + c;
      ok[h] = e < ny * Cn && kx < a.ncols;
      sidx[h] = e < ny * Cn ? sp(ky * W + c) : -1;
      g[h] = fo + (long long)ky * ldc + kx;
      const long long tg = (long long)ky * ldc + kx;
      x[h] = u[h] = nu[h] = s3[h] = zero;
      c0[h] = c1[h] = c2[h] = c3[h] = (T)0;
      if (!ok[h]) continue;
      x[h] = buf[sidx[h]];
      if (type == E1 || type == E2S) {
        c0[h] = tb1[tg]; c1[h] = tb2[tg];
        u[h] = a.uh[g[h]];
      } else if (type == E3) {
        c0[h] = tb1[tg]; c1[h] = tb2[tg];
        u[h] = a.ah[g[h]]; nu[h] = a.nu[g[h]]; s3[h] = a.ss[g[h]];
      } else if (type >= E5) {
        c0[h] = tb0[tg]; c1[h] = tb1[tg];
        u[h] = a.uh[g[h]];
        if (type == E7) { c2[h] = tb2[tg]; nu[h] = a.nu[g[h]]; }
      } else if (type == E4) {
        c0[h] = tb0[tg]; c1[h] = tb3[tg]; c2[h] = tb4[tg]; c3[h] = tb5[tg];
        u[h] = a.uh[g[h]]; nu[h] = a.nu[g[h]]; s3[h] = a.ss[g[h]];
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (sidx[h] < 0) continue;
      if (!ok[h]) { buf[sidx[h]] = zero; continue; }
      const Cx xv = x[h];
      Cx out;
      if (type == E0) {  // the initial U^ (later steps get it from E4)
        a.uh[g[h]] = xv;
        continue;
      } else if (type == E1) {
        a.nu[g[h]] = xv;
        out = mk<Cx>(c0[h] * u[h].x + c1[h] * xv.x, c0[h] * u[h].y + c1[h] * xv.y);
        a.ah[g[h]] = out;
      } else if (type == E2S) {
        a.ss[g[h]] = xv;
        out = mk<Cx>(c0[h] * u[h].x + c1[h] * xv.x, c0[h] * u[h].y + c1[h] * xv.y);
      } else if (type == E3) {
        // u = a^, nu = N^u, s3 = S
        a.ss[g[h]] = cadd(s3[h], xv);
        out = mk<Cx>(c0[h] * u[h].x + c1[h] * ((T)2 * xv.x - nu[h].x),
                     c0[h] * u[h].y + c1[h] * ((T)2 * xv.y - nu[h].y));
      } else if (type >= E5) {
        // ETD1 (fft_integrators.py:165-166) / ETD2 (234-236): c0 = E, c1 = phi1, c2 = phi2
        T ox = c0[h] * u[h].x + c1[h] * xv.x, oy = c0[h] * u[h].y + c1[h] * xv.y;
        if (type == E7) {
          ox += c2[h] * (xv.x - nu[h].x);
          oy += c2[h] * (xv.y - nu[h].y);
        }
        if (type != E5) a.nu[g[h]] = xv;
        out = mk<Cx>(ox, oy);
        a.uh[g[h]] = out;
      } else {
        // E4: c0 = E, c1 = f1, c2 = f2, c3 = f3; next step's U^ (unnormalised, as the forward
        // transform leaves it)
        out = mk<Cx>(c0[h] * u[h].x + c1[h] * nu[h].x + c2[h] * s3[h].x + c3[h] * xv.x,
                     c0[h] * u[h].y + c1[h] * nu[h].y + c2[h] * s3[h].y + c3[h] * xv.y);
        a.uh[g[h]] = out;
      }
      buf[sidx[h]] = cscale(out, a.scale);
    }
  }
  if (type == E0) return;
  __syncthreads();
  if (R4) fft_smem_r4<T, true, true>(buf, ny, a.log2ny, Cn, 1, W, a.tw, tid);
  else fft_smem<T, true, true>(buf, ny, a.log2ny, Cn, 1, W, a.tw, tid);
  Cx* dst = type >= E4 ? a.zu : a.zx;
  for (int e = tid; e < ny * Cn; e += nth) {
    const int ky = e >> lc, c = e & (Cn - 1), kx = kx0 + c;
    if (kx < a.ncols) dst[fo + ky * ldc + kx] = buf[sp(ky * W + c)];
  }
}

// ------------------------------------------------------------------ driver
struct EtdLayout {
  size_t zu, zn, zx, uh, nu, ah, ss, tab, total;
  long long fs;
};

static inline size_t al(size_t b) { return (b + 255) & ~size_t(255); }

static EtdLayout etd_layout(int ny, int nx, int elem) {
  EtdLayout L;
  L.fs = (long long)ny * spec_ldc(nx);
  const size_t sc = (size_t)2 * L.fs * 2 * elem;  // 2 fields of complex
  size_t o = 0;
  L.zu = o; o += sc;  // ZU, ZN, ZX contiguous (row-kernel offsets are relative to ZU)
  L.zn = o; o += sc;
  L.zx = o; o += al(sc);
  L.uh = o; o += al(sc);
  L.nu = o; o += al(sc);
  L.ah = o; o += al(sc);
  L.ss = o; o += al(sc);
  L.tab = o; o += al((size_t)2 * 6 * L.fs * elem);
  L.total = o;
  return L;
}

template <typename T>
struct EtdPlan {
  EArgs<T> c[8];
  EArgs<T> c0n;                     // forward transform of N_prev (row spectra in ZX) into N^prev
  RowArgs<T> rN, r4, rin, rout;
  RowArgs<T> rprev, rnout;          // N_prev real -> ZX; ZU -> N(u) real
};

// nf = 2: fields u, v paired row by row; nf = 1: rows y and y + ny/2 of one field.
template <typename T>
static EtdPlan<T> build_etd(const void* plan, const mjx_grid2d* g, int nf, double F, double k, double r_,
                            char* ws, const EtdLayout& L, const T* y_in, T* y_out, const T* nprev_in,
                            T* n_out) {
  EtdPlan<T> P;
  const PlanView pv = plan_view(plan, g->ny, g->nx, sizeof(T));
  const int ldc = spec_ldc(g->nx);
  EArgs<T> e;
  memset(&e, 0, sizeof(e));
  e.ny = g->ny; e.log2ny = ilog2_exact(g->ny); e.ncols = g->nx / 2 + 1; e.ldc = ldc;
  const int tps = g->ny >= 16 ? g->ny / 16 : 1;
  // widest tile within the thread cap and ~200 KB of shared memory
  auto tile = [&](int nin) {
    int C = 16;
    while (C > 1 && (C * nin * tps > EThreads<T>::v ||
                     (size_t)sp_size(g->ny * nin * C) * 2 * sizeof(T) > 200 * 1024)) C >>= 1;
    return C;
  };
  e.njobs = nf;
  e.zu = (cx<T>*)(ws + L.zu); e.zn = (cx<T>*)(ws + L.zn); e.zx = (cx<T>*)(ws + L.zx);
  e.uh = (cx<T>*)(ws + L.uh); e.nu = (cx<T>*)(ws + L.nu); e.ah = (cx<T>*)(ws + L.ah); e.ss = (cx<T>*)(ws + L.ss);
  e.tab = (const T*)(ws + L.tab); e.fs = L.fs; e.tw = (const cx<T>*)pv.twy;
  // column inverses normalise by 1/ny and every c2r row pass by 1/nx, so the
  // row-space state ZU is an unnormalised row DFT both after the initial r2c and
  // after each step
  e.scale = (T)(1.0 / (double)g->ny);
  for (int t = E0; t <= E7; ++t) {
    P.c[t] = e;
    P.c[t].type = t;
    P.c[t].C = tile(1);
  }
  P.c0n = P.c[E0];
  P.c0n.zu = e.zx;
  P.c0n.uh = e.nu;

  RowArgs<T> r;
  memset(&r, 0, sizeof(r));
  r.n = g->nx; r.log2n = ilog2_exact(g->nx); r.ldc = ldc; r.nrows = nf == 2 ? g->ny : g->ny / 2; r.npairs = 1;
  r.nseq = row_nseq(g->nx, r.nrows); r.rstride = g->nx; r.rin_sel = -1; r.rout_sel = -1;
  r.spec = (cx<T>*)(ws + L.zu); r.tw = (const cx<T>*)pv.twx; r.inv_scale = (T)(1.0 / (double)g->nx);
  r.F = F; r.k = k; r.r = r_;
  r.rin[0] = y_in; r.rout[0] = y_out;
  const long long zx = (long long)((L.zx - L.zu) / sizeof(cx<T>)), zn = (long long)((L.zn - L.zu) / sizeof(cx<T>));
  const long long hr = nf == 2 ? (long long)g->ny * g->nx : (long long)(g->ny / 2) * g->nx;
  const long long hs = nf == 2 ? L.fs : (long long)(g->ny / 2) * ldc;
  RowPair p;
  memset(&p, 0, sizeof(p));
  p.ra = 0; p.rb = hr;
  P.rN = r; p.sa = zx; p.sb = zx + hs; p.flags = ROW_LOAD_SPEC | ROW_NONLIN | ROW_STORE_SPEC; P.rN.pr[0] = p;
  P.rprev = r; P.rprev.rin[0] = nprev_in; p.flags = ROW_STORE_SPEC; P.rprev.pr[0] = p;
  P.r4 = r; p.sa = 0; p.sb = hs; p.oa = zn; p.ob = zn + hs;
  p.flags = ROW_LOAD_SPEC | ROW_NONLIN | ROW_STORE_SPEC | ROW_SPEC_ALT; P.r4.pr[0] = p;
  P.rin = r; p.sa = 0; p.sb = hs; p.flags = ROW_STORE_SPEC; P.rin.pr[0] = p;
  P.rout = r; p.flags = ROW_LOAD_SPEC | ROW_STORE_REAL; P.rout.pr[0] = p;
  P.rnout = r; P.rnout.rout[0] = n_out; p.flags = ROW_LOAD_SPEC | ROW_NONLIN | ROW_STORE_REAL; P.rnout.pr[0] = p;
  return P;
}

template <typename T, bool R4>
static mjx_status etd_col_attrs(int optin) {
  const void* k[8] = {(const void*)etd_col_kernel<T, E0, R4>, (const void*)etd_col_kernel<T, E1, R4>,
                      (const void*)etd_col_kernel<T, E2S, R4>, (const void*)etd_col_kernel<T, E3, R4>,
                      (const void*)etd_col_kernel<T, E4, R4>, (const void*)etd_col_kernel<T, E5, R4>,
                      (const void*)etd_col_kernel<T, E6, R4>, (const void*)etd_col_kernel<T, E7, R4>};
  for (int i = 0; i < 8; ++i)
    MJX_CUDA_TRY(cudaFuncSetAttribute(k[i], cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  return MJX_OK;
}

template <typename T, int TYPE>
static void etd_col_launch(const EArgs<T>& e, cudaStream_t s) {
  const int tps = e.ny >= 16 ? e.ny / 16 : 1;
  if constexpr (sizeof(T) == 8) {
    // FP64 columns of at most 256 points on a small grid (fewer than four warps per SM at
    // radix 16): radix-4 transforms (ny/4 threads per column), narrower tiles within the cap
    if (e.ny >= 4 && e.ny <= 256 && (long long)e.ncols * e.njobs * tps < 152LL * 128) {
      EArgs<T> b = e;
      const int tps4 = e.ny / 4;
      while (b.C > 1 && b.C * tps4 > EThreads<T>::v) b.C >>= 1;
      dim3 g4((b.ncols + b.C - 1) / b.C, b.njobs);
      const size_t sm4 = (size_t)sp_size(b.ny * b.C) * 2 * sizeof(T);
      etd_col_kernel<T, TYPE, true><<<g4, b.C * tps4, sm4, s>>>(b);
      return;
    }
  }
  dim3 grid((e.ncols + e.C - 1) / e.C, e.njobs);
  const size_t smem = (size_t)sp_size(e.ny * e.C) * 2 * sizeof(T);
  etd_col_kernel<T, TYPE><<<grid, e.C * tps, smem, s>>>(e);
}

template <typename T>
static cudaError_t etd_col(const EArgs<T>& e, cudaStream_t s) {
  switch (e.type) {
    case E0: etd_col_launch<T, E0>(e, s); break;
    case E1: etd_col_launch<T, E1>(e, s); break;
    case E2S: etd_col_launch<T, E2S>(e, s); break;
    case E3: etd_col_launch<T, E3>(e, s); break;
    case E4: etd_col_launch<T, E4>(e, s); break;
    case E5: etd_col_launch<T, E5>(e, s); break;
    case E6: etd_col_launch<T, E6>(e, s); break;
    default: etd_col_launch<T, E7>(e, s); break;
  }
  return cudaGetLastError();
}

template <typename T>
static cudaError_t etd_row(const RowArgs<T>& r, int rx, cudaStream_t s) {
  if (rx == MJX_REACT_GRAY_SCOTT) return launch_row<T, RX_GRAY_SCOTT>(r, s);
  if (rx == MJX_REACT_FISHER) return launch_row<T, RX_FISHER>(r, s);
  return launch_row<T, RX_NONE>(r, s);
}

enum { K_RK4 = 0, K_ETD1 = 1, K_ETD1N = 2, K_ETD2 = 3 };

template <typename T>
static cudaError_t etd_step(const EtdPlan<T>& P, int kind, int rx, cudaStream_t s) {
  cudaError_t e;
  if (kind != K_RK4) {
    const int t = kind == K_ETD1 ? E5 : (kind == K_ETD1N ? E6 : E7);
    if ((e = etd_col<T>(P.c[t], s)) != cudaSuccess) return e;
    return etd_row<T>(P.r4, rx, s);
  }
  for (int t = 1; t <= 4; ++t) {
    if ((e = etd_col<T>(P.c[t], s)) != cudaSuccess) return e;
    if ((e = etd_row<T>(t < 4 ? P.rN : P.r4, rx, s)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// cnt steps of one kind: captured once into a graph, replayed cnt times.
template <typename T>
static cudaError_t etd_replay(const EtdPlan<T>& P, int kind, int rx, int cnt, cudaStream_t s) {
  cudaStream_t cs = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t ce = cudaSuccess;
  do {
    if ((ce = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) break;
    if ((ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) break;
    const cudaError_t le = etd_step<T>(P, kind, rx, cs);
    ce = cudaStreamEndCapture(cs, &graph);
    if (le != cudaSuccess) { ce = le; break; }
    if (ce != cudaSuccess) break;
    if ((ce = cudaGraphInstantiate(&exec, graph, 0)) != cudaSuccess) break;
    for (int i = 0; i < cnt && ce == cudaSuccess; ++i) ce = cudaGraphLaunch(exec, s);
  } while (0);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cs) cudaStreamDestroy(cs);
  return ce;
}

static int etd_form(const mjx_etd_problem* p) {
  if (p->method != MJX_ETD_RK4) return FORM_PHI_ETD12;
  return p->coeffs == MJX_ETD_COEFF_PHI ? FORM_PHI_RK4 : FORM_CONTOUR_RK4;
}

template <typename T>
static mjx_status etd_run(const void* plan, const mjx_grid2d* g, const mjx_etd_problem* pb, int n_steps,
                          const T* y_in, const T* nprev_in, T* y_out, T* n_out, char* ws, const EtdLayout& L,
                          int recompute, cudaStream_t s) {
  static ContextOnce attr;
  MJX_TRY(attr.run([]() -> mjx_status {
    int dev = 0, optin = 0;
    MJX_CUDA_TRY(cudaGetDevice(&dev));
    MJX_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    MJX_TRY((etd_col_attrs<float, false>(optin)));
    MJX_TRY((etd_col_attrs<double, false>(optin)));
    MJX_TRY((etd_col_attrs<double, true>(optin)));
    return MJX_OK;
  }));
  const int nf = pb->nfields, rx = pb->reaction;
  const int symbol = pb->symbol & 1, xonly = (pb->symbol & MJX_SYMBOL_X_ONLY) ? 1 : 0;
  if (recompute) {
    etd_coeff_kernel<T><<<152 * 8, 256, 0, s>>>((T*)(ws + L.tab), g->ny, g->nx, spec_ldc(g->nx), symbol, xonly,
                                                 g->dy, g->dx, pb->D[0], pb->D[1], nf, pb->dt, 32,
                                                 pb->f2_factor, etd_form(pb));
    MJX_CUDA_TRY(cudaGetLastError());
  }
  const EtdPlan<T> P = build_etd<T>(plan, g, nf, pb->F, pb->k, pb->r, ws, L, y_in, y_out, nprev_in, n_out);
  MJX_CUDA_TRY(etd_row<T>(P.rin, rx, s));
  MJX_CUDA_TRY(etd_col<T>(P.c[E0], s));  // U^ of the initial state
  const int method = pb->method;
  if (method == MJX_ETD_2 && nprev_in) {
    MJX_CUDA_TRY(etd_row<T>(P.rprev, rx, s));
    MJX_CUDA_TRY(etd_col<T>(P.c0n, s));  // N^prev
  }
  MJX_CUDA_TRY(etd_row<T>(P.r4, rx, s));  // ZN = row spectra of N(u0)
  const int regular = method == MJX_ETD_RK4 ? K_RK4 : (method == MJX_ETD_1 ? K_ETD1 : K_ETD2);
  int i = 0;
  while (i < n_steps) {
    const int kind = (method == MJX_ETD_2 && i == 0 && !nprev_in) ? K_ETD1N : regular;
    const bool last = i == n_steps - 1;
    if (last && n_out) MJX_CUDA_TRY(etd_row<T>(P.rnout, rx, s));  // N at the start of the last step
    const int cnt = n_steps - i - (n_out ? 1 : 0);
    if (kind != regular || last || cnt < 3) {
      MJX_CUDA_TRY(etd_step<T>(P, kind, rx, s));
      ++i;
      continue;
    }
    const cudaError_t ce = etd_replay<T>(P, kind, rx, cnt, s);
    if (ce != cudaSuccess) { set_last_error(ce, __FILE__, __LINE__); return MJX_CUDA_ERROR; }
    i += cnt;
  }
  MJX_CUDA_TRY(etd_row<T>(P.rout, rx, s));
  return MJX_OK;
}

// Row pass that replaces real rows by the nonlinear term (no spectra).
template <typename T>
static RowArgs<T> nonlin_rows(const void* plan, const mjx_grid2d* g, int nf, double F, double k, double r_,
                              const T* y, T* out) {
  const PlanView pv = plan_view(plan, g->ny, g->nx, sizeof(T));
  RowArgs<T> r;
  memset(&r, 0, sizeof(r));
  r.n = g->nx; r.log2n = ilog2_exact(g->nx); r.ldc = spec_ldc(g->nx); r.nrows = nf == 2 ? g->ny : g->ny / 2;
  r.npairs = 1; r.nseq = row_nseq(g->nx, r.nrows); r.rstride = g->nx; r.rin_sel = -1; r.rout_sel = -1;
  r.tw = (const cx<T>*)pv.twx; r.inv_scale = (T)1;
  r.F = F; r.k = k; r.r = r_;
  r.rin[0] = y; r.rout[0] = out;
  r.pr[0].ra = 0;
  r.pr[0].rb = nf == 2 ? (long long)g->ny * g->nx : (long long)(g->ny / 2) * g->nx;
  r.pr[0].flags = ROW_NONLIN | ROW_STORE_REAL;
  return r;
}

static mjx_status check_etd(const mjx_grid2d* g, const mjx_etd_problem* p) {
  if (!p) return MJX_BAD_ARG;
  if (p->method != MJX_ETD_1 && p->method != MJX_ETD_2 && p->method != MJX_ETD_RK4) return MJX_BAD_ARG;
  if (p->coeffs != MJX_ETD_COEFF_CONTOUR && p->coeffs != MJX_ETD_COEFF_PHI) return MJX_BAD_ARG;
  if ((p->symbol & ~MJX_SYMBOL_X_ONLY) != MJX_SYMBOL_FD && (p->symbol & ~MJX_SYMBOL_X_ONLY) != MJX_SYMBOL_SPECTRAL)
    return MJX_BAD_ARG;
  if (p->reaction != MJX_REACT_NONE && p->reaction != MJX_REACT_GRAY_SCOTT && p->reaction != MJX_REACT_FISHER)
    return MJX_BAD_ARG;
  if (p->nfields != 1 && p->nfields != 2) return MJX_BAD_ARG;
  if (p->reaction == MJX_REACT_GRAY_SCOTT && p->nfields != 2) return MJX_BAD_ARG;
  if (!(p->dt > 0.0)) return MJX_BAD_ARG;
  (void)g;
  return MJX_OK;
}

}  // namespace mjx

using namespace mjx;

extern "C" {

size_t mjx_etdrk4_ws_bytes(int ny, int nx, int dtype) {
  const int e = elem_size(dtype);
  if (!e || ilog2_exact(nx) < 1 || ilog2_exact(ny) < 1) return 0;
  return etd_layout(ny, nx, e).total;
}

mjx_status mjx_etd_integrate2d(const void* plan, const mjx_grid2d* g, int dtype, const mjx_etd_problem* p,
                               int n_steps, const void* y_in, const void* nprev_in, void* y_out, void* n_out,
                               void* ws, size_t ws_bytes, int recompute_coeffs, void* stream) {
  MJX_TRY(check_grid(g));
  MJX_TRY(check_etd(g, p));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!plan || !y_in || !y_out || n_steps < 0) return MJX_BAD_ARG;
  if (n_out && n_steps < 1) return MJX_BAD_ARG;
  if (nprev_in && p->method != MJX_ETD_2) return MJX_BAD_ARG;
  const EtdLayout L = etd_layout(g->ny, g->nx, e);
  if (!ws || ws_bytes < L.total) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4)
    return etd_run<float>(plan, g, p, n_steps, (const float*)y_in, (const float*)nprev_in, (float*)y_out,
                          (float*)n_out, (char*)ws, L, recompute_coeffs, s);
  return etd_run<double>(plan, g, p, n_steps, (const double*)y_in, (const double*)nprev_in, (double*)y_out,
                         (double*)n_out, (char*)ws, L, recompute_coeffs, s);
}

mjx_status mjx_etdrk4_gray_scott2d(const void* plan, const mjx_grid2d* g, int dtype, int symbol,
                                   const double* D, double F, double k, double dt, double f2_factor,
                                   int n_steps,
                                   const void* y_in, void* y_out, void* ws, size_t ws_bytes,
                                   int recompute_coeffs, void* stream) {
  if (!D) return MJX_BAD_ARG;
  mjx_etd_problem p;
  memset(&p, 0, sizeof(p));
  p.method = MJX_ETD_RK4; p.coeffs = MJX_ETD_COEFF_CONTOUR; p.symbol = symbol;
  p.reaction = MJX_REACT_GRAY_SCOTT; p.nfields = 2;
  p.D[0] = D[0]; p.D[1] = D[1]; p.F = F; p.k = k; p.dt = dt; p.f2_factor = f2_factor;
  return mjx_etd_integrate2d(plan, g, dtype, &p, n_steps, y_in, nullptr, y_out, nullptr, ws, ws_bytes,
                             recompute_coeffs, stream);
}

mjx_status mjx_etd_nonlinear2d(const void* plan, const mjx_grid2d* g, int dtype, int reaction, int nfields,
                               double F, double k, double r, const void* y, void* out, void* stream) {
  MJX_TRY(check_grid(g));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!plan || !y || !out) return MJX_BAD_ARG;
  if (nfields != 1 && nfields != 2) return MJX_BAD_ARG;
  if (reaction == MJX_REACT_GRAY_SCOTT && nfields != 2) return MJX_BAD_ARG;
  if (reaction != MJX_REACT_NONE && reaction != MJX_REACT_GRAY_SCOTT && reaction != MJX_REACT_FISHER)
    return MJX_BAD_ARG;
  MJX_TRY(ensure_kernel_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  // one row pass, real rows in and out
  const cudaError_t ce = e == 4
      ? etd_row<float>(nonlin_rows<float>(plan, g, nfields, F, k, r, (const float*)y, (float*)out), reaction, s)
      : etd_row<double>(nonlin_rows<double>(plan, g, nfields, F, k, r, (const double*)y, (double*)out), reaction, s);
  return cuda_status(ce);
}

mjx_status mjx_etdrk4_kernel2d(const void* plan, const mjx_grid2d* g, int dtype, double F, double k,
                               int which, void* ws, size_t ws_bytes, void* stream) {
  MJX_TRY(check_grid(g));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  const EtdLayout L = etd_layout(g->ny, g->nx, e);
  if (!ws || ws_bytes < L.total || which < 1 || which > 8) return MJX_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t ce;
  if (e == 4) {
    const EtdPlan<float> P = build_etd<float>(plan, g, 2, F, k, 0.0, (char*)ws, L, nullptr, nullptr, nullptr,
                                              nullptr);
    ce = (which & 1) ? etd_col<float>(P.c[(which + 1) / 2], s)
                     : launch_row<float, RX_GRAY_SCOTT>(which == 8 ? P.r4 : P.rN, s);
  } else {
    const EtdPlan<double> P = build_etd<double>(plan, g, 2, F, k, 0.0, (char*)ws, L, nullptr, nullptr, nullptr,
                                                nullptr);
    ce = (which & 1) ? etd_col<double>(P.c[(which + 1) / 2], s)
                     : launch_row<double, RX_GRAY_SCOTT>(which == 8 ? P.r4 : P.rN, s);
  }
  return cuda_status(ce);
}

}  // extern "C"
