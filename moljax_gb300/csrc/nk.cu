// Matrix-free Newton-Krylov for implicit steps of the nonlinear diffusion-
// reaction model F(u) = div((a + b u^2) grad u) - c u^3 on a cell-centred grid
// with homogeneous Dirichlet ghosts (ghost = -neighbour).
//
// Restates moljax/core/newton_krylov.py:171-448: Newton with the convergence
// flag evaluated before the update, left-preconditioned restarted GMRES on
// M^-1 J dx = -M^-1 R, 3-try backtracking (accept if |R(x + alpha dx)| <
// (1 - 1e-4 alpha) |R|, alpha halves; full damped step when no try is
// accepted), and the BE/CN/BDF2 residual builders (362-448; BDF2 alphas and
// beta as the reference, beta = dt (1 + w)/(1 + 2w)).
//
// Precision: state, residual (the Newton refinement) and the Hessenberg /
// Givens least squares in FP64; Krylov vectors, the hand-written JVP and the
// preconditioner in FP32.
//
// Preconditioner M^-1 = (alpha0 I - beta Dbar Lap_D)^-1, Dbar = a + b mean(u_n^2),
// exact in the DST-II basis of the cell-centred Dirichlet grid: a real DST-II /
// DST-III pair in Makhoul's n-point form (three passes, eigenvalues from the
// FD symbol of the (2N)^2 periodic plan, which the odd extension shares).
//
// The Arnoldi steps of a GMRES cycle run as one CUDA graph with a conditional
// while node, six kernels per step (the JVP; DST-II along x; DST-II along y, the
// multiplier and DST-III along y; DST-III along x; the Gram-Schmidt dots; the
// orthogonalisation + Givens step); the last CTA of the last kernel updates the
// residual estimate on the device and clears the loop flag.  In the default
// mode the whole Newton iteration is one graph of nested conditional loops.
#include <math.h>
#include <string.h>

#include <vector>

#include "mixed.cuh"
#include "spectral.cuh"

namespace mjx {

mjx_status ensure_kernel_attrs();
int elem_size(int dtype);
void set_last_error(cudaError_t e, const char* file, int line);

enum { NK_MAXM = 64 };
enum { NK_RING = 256 };  // steps of counts kept on the device between host reads

struct NKConsts {
  double a0, beta;      // residual R = a0 y + cst - beta F(y)
  double inv_a0;        // preconditioner output scale
  double pa, pb, pc;    // model a, b, c
  double alpha;         // line-search step for the trial point
  double dbar;          // preconditioner diffusivity
};

struct GmresState {
  int j, m, converged, k_used;
  double tol_abs, beta0, hnext_inv, res_est;
  double H[(NK_MAXM + 1) * NK_MAXM];
  double cs[NK_MAXM], sn[NK_MAXM], g[NK_MAXM + 1], y[NK_MAXM];
};

// --------------------------------------------------------------- stencils
// u at (i, j) with homogeneous Dirichlet ghosts (x ghosts first, then y: corners
// are not used by the 5-point stencil)
template <typename T>
__device__ __forceinline__ T dval(const T* u, int i, int j, int n) {
  const int ii = i < 0 ? 0 : (i >= n ? n - 1 : i);
  const int jj = j < 0 ? 0 : (j >= n ? n - 1 : j);
  const T v = u[(long long)ii * n + jj];
  return ((i < 0) != (i >= n)) || ((j < 0) != (j >= n)) ? -v : v;
}

// (row, column) of flat index p in rows of length n: 32-bit division whenever p fits
__device__ __forceinline__ void nk_rowcol(long long p, int n, int& i, int& j) {
  if (p < 4294967296LL) {
    const unsigned q = (unsigned)p / (unsigned)n;
    i = (int)q;
    j = (int)((unsigned)p - q * (unsigned)n);
  } else {
    i = (int)(p / n);
    j = (int)(p - (long long)i * n);
  }
}

// R = a0 u + cst - beta F(u) at (i, j); u(i, j) returns the ghosted value
template <class G>
__device__ __forceinline__ double vd_resid_at(G u, int i, int j, double cst_p, double a, double b, double c,
                                              double a0, double beta, double idx2, double idy2) {
  const double uc = u(i, j);
  const double ue = u(i, j + 1), uw = u(i, j - 1);
  const double un = u(i + 1, j), us = u(i - 1, j);
  const double Dc = a + b * uc * uc;
  const double De = a + b * ue * ue, Dw = a + b * uw * uw, Dn = a + b * un * un, Ds = a + b * us * us;
  const double fx = 0.5 * (Dc + De) * (ue - uc) - 0.5 * (Dw + Dc) * (uc - uw);
  const double fy = 0.5 * (Dc + Dn) * (un - uc) - 0.5 * (Ds + Dc) * (uc - us);
  const double F = fx * idx2 + fy * idy2 - c * uc * uc * uc;
  return a0 * uc + cst_p - beta * F;
}

// block sum of acc into part[blockIdx.x] (FP64)
__device__ __forceinline__ void block_partial(double acc, double* part) {
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    part[blockIdx.x] = s;
  }
}

// R = a0 y + cst - beta F(y); part[block] = sum R^2; b32 = -R (optional)
__global__ void vd_residual_kernel(const double* __restrict__ y, const double* __restrict__ cst,
                                   double* __restrict__ R, float* __restrict__ b32,
                                   double* __restrict__ part, const NKConsts* __restrict__ K,
                                   int n, double idx2, double idy2) {
  const double a = K->pa, b = K->pb, c = K->pc, a0 = K->a0, beta = K->beta;
  double acc = 0.0;
  const long long N2 = (long long)n * n;
  auto u = [&](int ii, int jj) { return dval(y, ii, jj, n); };
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j;
    nk_rowcol(p, n, i, j);
    const double r = vd_resid_at(u, i, j, cst[p], a, b, c, a0, beta, idx2, idy2);
    R[p] = r;
    if (b32) b32[p] = (float)(-r);
    acc += r * r;
  }
  block_partial(acc, part);
}

// out = s F(y) (the model right-hand side, scaled), constants by value
__global__ void vd_rhs_kernel(const double* __restrict__ y, double* __restrict__ out, double a,
                              double b, double c, double s, int n, double idx2, double idy2) {
  const long long N2 = (long long)n * n;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j;
    nk_rowcol(p, n, i, j);
    const double uc = y[p];
    const double ue = dval(y, i, j + 1, n), uw = dval(y, i, j - 1, n);
    const double un = dval(y, i + 1, j, n), us = dval(y, i - 1, j, n);
    const double Dc = a + b * uc * uc;
    const double De = a + b * ue * ue, Dw = a + b * uw * uw, Dn = a + b * un * un, Ds = a + b * us * us;
    const double fx = 0.5 * (Dc + De) * (ue - uc) - 0.5 * (Dw + Dc) * (uc - uw);
    const double fy = 0.5 * (Dc + Dn) * (un - uc) - 0.5 * (Ds + Dc) * (uc - us);
    out[p] = s * (fx * idx2 + fy * idy2 - c * uc * uc * uc);
  }
}

// partial dots <V_i, w>, i = 0..j, FP64 accumulation; part[i * nblk + block]
__global__ void gmres_dots_kernel(const float* __restrict__ V, const float* __restrict__ w,
                                  const GmresState* gs, double* part, long long N2) {
  if (gs->converged) return;
  const int j = gs->j;
  __shared__ double red[32];
  for (int i = 0; i <= j; ++i) {
    const float* vi = V + (long long)i * N2;
    double acc = 0.0;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
         p += (long long)gridDim.x * blockDim.x)
      acc += (double)vi[p] * (double)w[p];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
      part[(long long)i * gridDim.x + blockIdx.x] = s;
    }
    __syncthreads();
  }
}

// H[i][j] = sum of the partial dots
__global__ void gmres_hcol_kernel(const double* part, int nblk, GmresState* gs) {
  if (gs->converged) return;
  const int j = gs->j;
  __shared__ double red[32];
  for (int i = 0; i <= j; ++i) {
    double acc = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc += part[(long long)i * nblk + b];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
      gs->H[i * NK_MAXM + j] = s;
    }
    __syncthreads();
  }
}

// V_{j+1} = w - sum_i H[i][j] V_i (classical Gram-Schmidt), partial norms of V_{j+1}
__global__ void gmres_orth_kernel(float* __restrict__ V, const float* __restrict__ w,
                                  const GmresState* gs, double* part, long long N2) {
  if (gs->converged) return;
  const int j = gs->j;
  float h[NK_MAXM];
  for (int i = 0; i <= j; ++i) h[i] = (float)gs->H[i * NK_MAXM + j];
  float* vn = V + (long long)(j + 1) * N2;
  double acc = 0.0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    float x = w[p];
    for (int i = 0; i <= j; ++i) x -= h[i] * V[(long long)i * N2 + p];
    vn[p] = x;
    acc += (double)x * (double)x;
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
    part[blockIdx.x] = s;
  }
}

// one Givens step in FP64 (single thread) and the loop flag
__global__ void gmres_givens_kernel(const double* part, int nblk, GmresState* gs,
                                    cudaGraphConditionalHandle h, int use_handle) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc += part[b];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x != 0) return;
  if (gs->converged) {
    if (use_handle) cudaGraphSetConditional(h, 0u);
    return;
  }
  double s = 0.0;
  for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
  const int j = gs->j;
  const double hn = sqrt(s);
  double* H = gs->H;
  H[(j + 1) * NK_MAXM + j] = hn;
  for (int i = 0; i < j; ++i) {
    const double a = H[i * NK_MAXM + j], b = H[(i + 1) * NK_MAXM + j];
    H[i * NK_MAXM + j] = gs->cs[i] * a + gs->sn[i] * b;
    H[(i + 1) * NK_MAXM + j] = -gs->sn[i] * a + gs->cs[i] * b;
  }
  const double a = H[j * NK_MAXM + j], b = H[(j + 1) * NK_MAXM + j];
  const double den = hypot(a, b);
  const double c = den > 0 ? a / den : 1.0, sn = den > 0 ? b / den : 0.0;
  gs->cs[j] = c;
  gs->sn[j] = sn;
  H[j * NK_MAXM + j] = den;
  H[(j + 1) * NK_MAXM + j] = 0.0;
  gs->g[j + 1] = -sn * gs->g[j];
  gs->g[j] = c * gs->g[j];
  gs->k_used = j + 1;
  gs->res_est = fabs(gs->g[j + 1]);
  const bool conv = gs->res_est <= gs->tol_abs || hn == 0.0;
  gs->j = j + 1;
  gs->hnext_inv = hn > 0 ? 1.0 / hn : 0.0;
  const bool more = !conv && gs->j < gs->m;
  if (conv) gs->converged = 1;
  if (use_handle) cudaGraphSetConditional(h, more ? 1u : 0u);
}

// cycle start: beta0 = |V_0|, g = (beta0, 0, ...), tolerance on the first cycle
__global__ void gmres_init_kernel(const double* part, int nblk, GmresState* gs, int first, double tol,
                                  int m) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc += part[b];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x != 0) return;
  double s = 0.0;
  for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
  const double b0 = sqrt(s);
  if (first) gs->tol_abs = tol * b0;
  gs->beta0 = b0;
  gs->j = 0;
  gs->m = m;
  gs->k_used = 0;
  for (int i = 0; i <= m; ++i) gs->g[i] = 0.0;
  gs->g[0] = b0;
  gs->res_est = b0;
  gs->hnext_inv = b0 > 0 ? 1.0 / b0 : 0.0;
  gs->converged = (b0 <= gs->tol_abs || b0 == 0.0) ? 1 : 0;
}

// back substitution R y = g (FP64)
__global__ void gmres_solve_kernel(GmresState* gs) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int k = gs->k_used;
  for (int i = k - 1; i >= 0; --i) {
    double s = gs->g[i];
    for (int q = i + 1; q < k; ++q) s -= gs->H[i * NK_MAXM + q] * gs->y[q];
    const double d = gs->H[i * NK_MAXM + i];
    gs->y[i] = d != 0.0 ? s / d : 0.0;
  }
}

// dx += sum_i y_i V_i (V_0..V_{k-1} normalised)
__global__ void gmres_update_kernel(float* dx, const float* V, const GmresState* gs, long long N2) {
  const int k = gs->k_used;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    double x = dx[p];
    for (int i = 0; i < k; ++i) x += gs->y[i] * (double)V[(long long)i * N2 + p];
    dx[p] = (float)x;
  }
}

__global__ void sub_kernel(const float* b, const float* t, float* r, long long N2) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x)
    r[p] = b[p] - t[p];
}

// out = x + alpha dx (FP64 + FP32), alpha from K
__global__ void trial_kernel(const double* x, const float* dx, double* out, const NKConsts* K,
                             float* y32, long long N2) {
  const double al = K->alpha;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    const double v = x[p] + al * (double)dx[p];
    out[p] = v;
    if (y32) y32[p] = (float)v;
  }
}

__global__ void lincomb_kernel(const double* a, double ca, const double* b, double cb, double* out,
                               float* o32, long long N2) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    const double v = ca * a[p] + (b ? cb * b[p] : 0.0);
    out[p] = v;
    if (o32) o32[p] = (float)v;
  }
}

// partial sums of y^2 (preconditioner Dbar) and the 2N Helmholtz step for the spectral pass
__global__ void sumsq_kernel(const double* y, double* part, long long N2) {
  double acc = 0.0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x)
    acc += y[p] * y[p];
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
    part[blockIdx.x] = s;
  }
}

__global__ void sumsq32_kernel(const float* v, double* part, long long N2) {
  double acc = 0.0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x)
    acc += (double)v[p] * (double)v[p];
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
    part[blockIdx.x] = s;
  }
}

// scaled error partials: sum (E / (atol + rtol |y|))^2 and a non-finite flag on y
// (scaled_error_norm, moljax/core/state.py:312-343; is_finite, utils.py:186-197)
__global__ void errnorm_kernel(const double* E, const double* y, double atol, double rtol,
                               double* part, int* bad, long long N2) {
  double acc = 0.0;
  int nf = 0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    const double v = y[p];
    const double q = E[p] / (atol + rtol * fabs(v));
    acc += q * q;
    nf |= !isfinite(v);
  }
  __shared__ double red[32];
  __shared__ int redb[32];
  for (int o = 16; o > 0; o >>= 1) {
    acc += __shfl_xor_sync(0xffffffffu, acc, o);
    nf |= __shfl_xor_sync(0xffffffffu, nf, o);
  }
  if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = acc; redb[threadIdx.x >> 5] = nf; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    int b = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { s += red[q]; b |= redb[q]; }
    part[blockIdx.x] = s;
    bad[blockIdx.x] = b;
  }
}

__global__ void nk_consts_kernel(const double* part, int nblk, NKConsts* K, DevState* pst, double n2) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc += part[b];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x != 0) return;
  double s = 0.0;
  for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
  K->dbar = K->pa + K->pb * s / n2;
  K->inv_a0 = 1.0 / K->a0;
  // M^-1 = (1/a0) (I - (beta dbar / a0) Lap)^-1 : Helmholtz step h with D = 1
  pst->dtc = K->beta * K->dbar / K->a0;
  pst->done = 0;
}

// a0 (s v) - beta J_F(u) (s v) at (i, jj) in FP32: the hand-written JVP of the variable
// diffusion model (a + b u^2 faces averaged, - c u^3), Dirichlet ghosts on u and v
__device__ __forceinline__ float vd_jvp_at(const float* __restrict__ y32, const float* __restrict__ vin,
                                           float s, int i, int jj, int n, float a, float b, float c,
                                           float a0, float beta, float idx2, float idy2) {
  const long long p = (long long)i * n + jj;
  const float uc = y32[p], ue = dval(y32, i, jj + 1, n), uw = dval(y32, i, jj - 1, n);
  const float un = dval(y32, i + 1, jj, n), us = dval(y32, i - 1, jj, n);
  const float vc = s * vin[p], ve = s * dval(vin, i, jj + 1, n), vw = s * dval(vin, i, jj - 1, n);
  const float vn = s * dval(vin, i + 1, jj, n), vs = s * dval(vin, i - 1, jj, n);
  const float Dc = a + b * uc * uc, De = a + b * ue * ue, Dw = a + b * uw * uw;
  const float Dn = a + b * un * un, Ds = a + b * us * us;
  const float dc = 2.f * b * uc * vc, de = 2.f * b * ue * ve, dw = 2.f * b * uw * vw;
  const float dn = 2.f * b * un * vn, ds = 2.f * b * us * vs;
  const float gx = 0.5f * (Dc + De) * (ve - vc) + 0.5f * (dc + de) * (ue - uc)
                 - 0.5f * (Dw + Dc) * (vc - vw) - 0.5f * (dw + dc) * (uc - uw);
  const float gy = 0.5f * (Dc + Dn) * (vn - vc) + 0.5f * (dc + dn) * (un - uc)
                 - 0.5f * (Ds + Dc) * (vc - vs) - 0.5f * (ds + dc) * (uc - us);
  return a0 * vc - beta * (gx * idx2 + gy * idy2 - 3.f * c * uc * uc * vc);
}

// JVP of the current Arnoldi vector V_j (j read on the device)
// (gs == nullptr: t = J vin for the plain vector vin = V; with bsub, t = bsub - J vin)
__global__ void vd_jvp_j_kernel(const float* y32, float* V, const GmresState* gs, float* t,
                                const NKConsts* K, int n, float idx2, float idy2, long long N2,
                                const float* bsub = nullptr) {
  if (gs && gs->converged) return;
  const int j = gs ? gs->j : 0;
  const float* vin = V + (long long)j * N2;
  const float a = (float)K->pa, b = (float)K->pb, c = (float)K->pc;
  const float a0 = (float)K->a0, beta = (float)K->beta;
  const float s = gs ? (float)gs->hnext_inv : 1.0f;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    int i, jj;
    nk_rowcol(p, n, i, jj);
    const float jv = vd_jvp_at(y32, vin, s, i, jj, n, a, b, c, a0, beta, idx2, idy2);
    t[p] = bsub ? bsub[p] - jv : jv;
  }
}

// out = a0 v - beta J_F(u) v in FP64 (the exported JVP; J_F v itself with a0 = 0, beta = -1)
__global__ void vd_jvp64_kernel(const double* __restrict__ u, const double* __restrict__ v, double* __restrict__ out,
                                double a, double b, double c, double a0, double beta, int n, double idx2,
                                double idy2, long long N2) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    int i, jj;
    nk_rowcol(p, n, i, jj);
    const double uc = u[p], ue = dval(u, i, jj + 1, n), uw = dval(u, i, jj - 1, n);
    const double un = dval(u, i + 1, jj, n), us = dval(u, i - 1, jj, n);
    const double vc = v[p], ve = dval(v, i, jj + 1, n), vw = dval(v, i, jj - 1, n);
    const double vn = dval(v, i + 1, jj, n), vs = dval(v, i - 1, jj, n);
    const double Dc = a + b * uc * uc, De = a + b * ue * ue, Dw = a + b * uw * uw;
    const double Dn = a + b * un * un, Ds = a + b * us * us;
    const double dc = 2.0 * b * uc * vc, de = 2.0 * b * ue * ve, dw = 2.0 * b * uw * vw;
    const double dn = 2.0 * b * un * vn, ds = 2.0 * b * us * vs;
    const double gx = 0.5 * (Dc + De) * (ve - vc) + 0.5 * (dc + de) * (ue - uc)
                    - 0.5 * (Dw + Dc) * (vc - vw) - 0.5 * (dw + dc) * (uc - uw);
    const double gy = 0.5 * (Dc + Dn) * (vn - vc) + 0.5 * (dc + dn) * (un - uc)
                    - 0.5 * (Ds + Dc) * (vc - vs) - 0.5 * (ds + dc) * (uc - us);
    out[p] = a0 * vc - beta * (gx * idx2 + gy * idy2 - 3.0 * c * uc * uc * vc);
  }
}

__global__ void nk_scale_j_kernel(float* V, const GmresState* gs, long long N2) {
  if (gs->converged) return;
  float* v = V + (long long)gs->j * N2;
  const float s = (float)gs->hnext_inv;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x)
    v[p] *= s;
}


// --------------------------------------------------------------- device Newton loop
// The Newton iteration of newton_krylov_solve (newton_krylov.py:171-359) as one CUDA graph:
// while (iterating) { R(x) and its norm; restarted GMRES (while cycles { cycle set-up; while
// Arnoldi steps; solve and update }); backtracking line search (while tries { trial point
// and its residual; sufficient-decrease test }); accept or take the damped step }.  Every
// decision is made by a one-CTA kernel that sets the conditional flag of its loop; the host
// launches the graph once per solve and reads the counters once.
struct NewtonDev {
  int it, converged, cyc, bt, accepted, lits, max_newton, max_krylov, max_backtrack, restart;
  int rvalid;  // R and -R hold R(x) and rn its norm (initial residual, or an accepted trial point)
  double rn, rb, res, newton_tol, krylov_tol, damping, backtrack, min_decrease;
};

// sum of the block partials (one CTA of 256 threads)
__device__ __forceinline__ double nd_sum(const double* part, int nblk) {
  __shared__ double red[8];
  double acc = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc += part[b];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  double s = 0.0;
  for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
  return s;
}

// before the loop: |R(x0)|, converged (newton_krylov.py:338-346), the loop flag
__global__ void nd_init_kernel(const double* part, int nblk, NewtonDev* nd, cudaGraphConditionalHandle hN) {
  const double s = nd_sum(part, nblk);
  if (threadIdx.x != 0) return;
  nd->rn = sqrt(s);
  nd->res = nd->rn;
  nd->it = 0;
  nd->lits = 0;
  nd->rvalid = 1;
  nd->converged = nd->rn < nd->newton_tol;
  cudaGraphSetConditional(hN, (!nd->converged && nd->max_newton > 0) ? 1u : 0u);
}

// line search start (270-276): alpha = damping, reference norm |R(x)|
__global__ void nd_ls_begin_kernel(NewtonDev* nd, NKConsts* K, cudaGraphConditionalHandle hL) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  K->alpha = nd->damping;
  nd->rb = nd->rn;
  nd->bt = 0;
  nd->accepted = 0;
  cudaGraphSetConditional(hL, nd->max_backtrack > 0 ? 1u : 0u);
}


// --------------------------------------------------------------- fused Arnoldi step
// One GMRES iteration on M^-1 A in six kernels (the separate sequence above takes eleven):
//   JVP        t = A V_j / |V_j| (vd_jvp_j_kernel: elementwise, every SM busy);
//   DST rows   DST-II along x of t, two rows per complex n-point transform;
//   DST cols   DST-II along y, the Helmholtz inverse, DST-III along y (in place);
//   DST rows   DST-III along x and w = M^-1 A V_j (at a cycle start: V_0 = w and its |.|^2
//              partials, the last CTA starts the cycle);
//   nka_dots   V_j normalised in place and the Gram-Schmidt partial dots <V_i, w> (i <= j),
//              accumulated in float-float on the FP32 pipe; the last CTA sums them in a
//              fixed order into H[:, j];
//   nka_orth   V_{j+1} = w - sum_i H_ij V_i and |V_{j+1}|^2 partials; the last CTA applies
//              the Givens rotations, back-substitutes when the cycle ends and sets the loop
//              flag.
// The row passes have n/16 threads per row pair, i.e. few warps in all, so the stencil and
// the dot products, whose loads need many warps in flight, stay in the elementwise
// kernels.  "Last CTA" is a ticket: every CTA publishes its partials, fences and draws a
// ticket from a counter in the workspace; the CTA that draws the final ticket reads all
// partials and resets the counter.  No CTA ever waits for another.
enum { NKA_STORE_W = 0, NKA_START = 1 };

struct NkaArgs {
  int n, nseq;
  long long N2;
  const float* src;     // operand of the preconditioner (n x n)
  float* V;             // Krylov basis, m + 1 vectors of N2
  float* t;             // w = M^-1 A V_j (Arnoldi)
  GmresState* gs;
  const NKConsts* K;
  double* part;         // per-CTA partials
  unsigned* ticket;     // zero between kernels
  // cycle start: from nd (graph Newton loop) when set, else first / tol / m
  const NewtonDev* nd;
  int first, m;
  double tol;
  cudaGraphConditionalHandle h;
  int use_handle;
  int skip_converged;   // Arnoldi passes: return at entry once the cycle has converged
  // the DST passes
  int log2n, C;         // transform length n; column tile width (even)
  float* S;             // real DST coefficients, n x n
  const cx<float>* twn; // twiddles of length n
  const float2* ph;     // (cos, sin)(pi k / 2n), k < n
  const float* lamx;    // the plan's (2n)-point symbol along x (index = frequency 0..n)
  const float* lamy;    // along y (fftfreq order of 2n)
  const DevState* st;   // Helmholtz step dtc
};

// true in the CTA that finished last (block-uniform); its reads of the other CTAs'
// partials must bypass L1 (__ldcg)
__device__ __forceinline__ bool nka_last(unsigned* ticket) {
  __shared__ int last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  return last != 0;
}

// sum of nb partials read through L2, the same order in every call (all threads of the CTA)
__device__ __forceinline__ double nka_sum(const double* part, int nb) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) acc += __ldcg(&part[b]);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  double s = 0.0;
  for (int q = 0; q < (int)((blockDim.x + 31) >> 5); ++q) s += red[q];
  return s;
}

// (hi, lo) += a b: the FMA two-product and Knuth's two-sum on the FP32 pipe (the dot-product
// accumulation of Ogita, Rump and Oishi); hi + lo carries about twice the FP32 precision
__device__ __forceinline__ void ff_dot_acc(float& hi, float& lo, float a, float b) {
  const float p = __fmul_rn(a, b);
  const float pe = __fmaf_rn(a, b, -p);
  const float s = __fadd_rn(hi, p);
  lo = __fadd_rn(lo, __fadd_rn(ff_2sum_err(hi, p, s), pe));
  hi = s;
}

// warp sum of float-float values (hi, lo), a two-sum per step, the same order in every lane:
// the reduction stays on the FP32 pipe (an FP64 add per step waits on GB300's narrow FP64 units)
__device__ __forceinline__ void ff_warp_sum(float& hi, float& lo) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, o), ol = __shfl_xor_sync(0xffffffffu, lo, o);
    const float s = __fadd_rn(hi, oh);
    lo = __fadd_rn(lo, __fadd_rn(ol, ff_2sum_err(hi, oh, s)));
    hi = s;
  }
}

// cycle start from |V_0|^2 = s (as gmres_init_kernel; in the graph Newton loop the first-cycle
// flag, tolerance and restart come from NewtonDev)
__device__ void gmres_start(GmresState* gs, double s, int first, double tol, int m) {
  const double b0 = sqrt(s);
  if (first) gs->tol_abs = tol * b0;
  gs->beta0 = b0;
  gs->j = 0;
  gs->m = m;
  gs->k_used = 0;
  for (int i = 0; i <= m; ++i) gs->g[i] = 0.0;
  gs->g[0] = b0;
  gs->res_est = b0;
  gs->hnext_inv = b0 > 0 ? 1.0 / b0 : 0.0;
  gs->converged = (b0 <= gs->tol_abs || b0 == 0.0) ? 1 : 0;
}

// back substitution R y = g over the k_used columns (as gmres_solve_kernel)
__device__ void gmres_backsub(GmresState* gs) {
  const int k = gs->k_used;
  for (int i = k - 1; i >= 0; --i) {
    double s = gs->g[i];
    for (int q = i + 1; q < k; ++q) s -= gs->H[i * NK_MAXM + q] * gs->y[q];
    const double d = gs->H[i * NK_MAXM + i];
    gs->y[i] = d != 0.0 ? s / d : 0.0;
  }
}

// Work after the inverse transform: this thread holds w at columns x0 + m xs (m < M,
// x < n) of rows y and y + n/2.
template <int MODE, int M>
__device__ __forceinline__ void nka_finish(const NkaArgs& a, int y, int x0, int xs, const float (&wa)[M],
                                           const float (&wb)[M]) {
  const int n = a.n;
  const long long ra = (long long)y * n, rb = (long long)(y + (n >> 1)) * n;
  if (MODE == NKA_STORE_W) {
#pragma unroll
    for (int m = 0; m < M; ++m) {
      const int x = x0 + m * xs;
      if (x < n) { a.t[ra + x] = wa[m]; a.t[rb + x] = wb[m]; }
    }
    return;
  }
  // cycle start: V_0 = w, |V_0|^2
  __shared__ double red[8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
  double acc = 0.0;
#pragma unroll
  for (int m = 0; m < M; ++m) {
    const int x = x0 + m * xs;
    if (x < n) {
      a.V[ra + x] = wa[m]; a.V[rb + x] = wb[m];
      acc += (double)wa[m] * (double)wa[m];
      acc += (double)wb[m] * (double)wb[m];
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < nw; ++q) s += red[q];
    a.part[blockIdx.x] = s;
  }
  if (nka_last(a.ticket)) {
    const double s = nka_sum(a.part, gridDim.x);
    if (threadIdx.x == 0) {
      GmresState* gs = a.gs;
      const NewtonDev* nd = a.nd;
      if (nd) gmres_start(gs, s, nd->cyc == 0, nd->krylov_tol, nd->restart);
      else gmres_start(gs, s, a.first, a.tol, a.m);
      if (a.use_handle) cudaGraphSetConditional(a.h, gs->converged ? 0u : 1u);
      *a.ticket = 0u;
    }
  }
}

// ---- the preconditioner as a real DST-II / DST-III pair (Makhoul's n-point form)
// M^-1 = (1/a0) (I - (beta Dbar/a0) Lap_D)^-1 is diagonal in the DST-II basis of the
// cell-centred Dirichlet grid (the odd-extension form above carries the same coefficients
// with four times the transform work).  DST-II of a real row x of length n:
//   DST-II(x)[n-1-k] = DCT-II(y)[k], y_j = (-1)^j x_j,
//   DCT-II(y)[k] = Re(e^{-i pi k/2n} V_k), V = FFT_n(v), v_{j} = y_{2j}, v_{n-1-j} = y_{2j+1}
// (Makhoul 1980), two real rows (or columns) per complex FFT; the inverse runs the same
// steps backwards: V_k = e^{i pi k/2n} (C_k - i C_{n-k}) (C_n = 0), v = IFFT_n(V), y from v.
// DST index s has frequency s + 1: eigenvalue lam_2n(s + 1) of the plan's (2n)-point FD
// symbol, the same as the odd extension's.  Three kernels: rows forward (from the
// operand), columns forward * multiplier * inverse (in place), rows inverse (w, or the
// cycle start).

// position of element j in Makhoul's reordering
__device__ __forceinline__ int mk_pos(int j, int n) { return (j & 1) ? n - 1 - (j >> 1) : (j >> 1); }

// DCT-II coefficients of index k of the two sequences packed in Z (Zk = Z[k], Zm = Z[n-k])
__device__ __forceinline__ void dct_split(float2 Zk, float2 Zm, float2 p, float& ca, float& cb) {
  const float vax = 0.5f * (Zk.x + Zm.x), vay = 0.5f * (Zk.y - Zm.y);
  const float vbx = 0.5f * (Zk.y + Zm.y), vby = 0.5f * (Zm.x - Zk.x);
  ca = p.x * vax + p.y * vay;
  cb = p.x * vbx + p.y * vby;
}

// inverse input of index k from the coefficients (C_k, C_{n-k}) of the two sequences
__device__ __forceinline__ float2 dct_merge(float cak, float cam, float cbk, float cbm, float2 p) {
  const float vax = p.x * cak + p.y * cam, vay = p.y * cak - p.x * cam;
  const float vbx = p.x * cbk + p.y * cbm, vby = p.y * cbk - p.x * cbm;
  return make_float2(vax - vby, vay + vbx);
}

// Threads per sequence of the shared-memory transforms of the DST passes: n/16 for the
// radix-16 Stockham (fft_smem), n/4 for the radix-4 one (fft_smem_r4: a quarter of the
// dependent work per thread, for passes with few sequences)
template <bool R4>
__device__ __forceinline__ int dst_tps(int n) { return R4 ? (n >= 4 ? n >> 2 : 1) : (n >= 16 ? n >> 4 : 1); }

template <bool R4, bool INV, bool COLMAJOR>
__device__ __forceinline__ void dst_fft(float2* buf, const NkaArgs& a, int nseq, int ss, int es, int tid) {
  if (R4) fft_smem_r4<float, INV, COLMAJOR>(buf, a.n, a.log2n, nseq, ss, es, a.twn, tid);
  else fft_smem<float, INV, COLMAJOR>(buf, a.n, a.log2n, nseq, ss, es, a.twn, tid);
}

// forward DST-II along x of the row pairs (y, y + n/2) of a.src into a.S
template <bool R4>
__global__ void __launch_bounds__(256) dst_row_fwd_kernel(const __grid_constant__ NkaArgs a) {
  typedef float2 C;
  constexpr int PTS = R4 ? 4 : 16;  // elements per thread
  if (a.skip_converged && a.gs->converged) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const int n = a.n, hn = n >> 1;
  const int tps = dst_tps<R4>(n);
  const int tid = threadIdx.x, s_loc = pdiv(tid, tps), lt = tid - s_loc * tps;
  const bool active = s_loc < a.nseq;  // whole warps are launched
  const int y = blockIdx.x * a.nseq + s_loc;
  const int zb = s_loc * n;
  const float* ra = a.src + (long long)y * n;
  const float* rb = a.src + (long long)(y + hn) * n;
#pragma unroll
  for (int m = 0; m < PTS; ++m) {
    const int x = lt + m * tps;
    if (active && x < n) {
      const float sg = (x & 1) ? -1.f : 1.f;
      buf[sp(zb + mk_pos(x, n))] = make_float2(sg * ra[x], sg * rb[x]);
    }
  }
  __syncthreads();
  dst_fft<R4, false, false>(buf, a, a.nseq, n, 1, tid);
  if (!active) return;
  float* Sa = a.S + (long long)y * n;
  float* Sb = a.S + (long long)(y + hn) * n;
#pragma unroll
  for (int m = 0; m < PTS; ++m) {
    const int k = lt + m * tps;
    if (k < n) {
      float ca, cb;
      dct_split(buf[sp(zb + k)], buf[sp(zb + ((n - k) & (n - 1)))], a.ph[k], ca, cb);
      Sa[n - 1 - k] = ca;
      Sb[n - 1 - k] = cb;
    }
  }
}

// columns kx0 .. kx0 + C - 1 of a.S: DST-II along y, the Helmholtz inverse (with the 1/n^2
// of the two unnormalised inverse transforms), DST-III along y, in place
template <bool R4>
__global__ void __launch_bounds__(256) dst_col_kernel(const __grid_constant__ NkaArgs a) {
  typedef float2 C;
  if (a.skip_converged && a.gs->converged) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const int n = a.n, Cn = a.C, ns = Cn >> 1, lc = __ffs(Cn) - 1, ls = lc - 1;
  const int kx0 = blockIdx.x * Cn;
  const int tid = threadIdx.x, nth = blockDim.x;
  // load (sign and Makhoul position along y), columns 2q and 2q + 1 as sequence q
  for (int e = tid; e < n * Cn; e += nth) {
    const int y = e >> lc, c = e & (Cn - 1);
    const float v = a.S[(long long)y * n + kx0 + c];
    float* slot = reinterpret_cast<float*>(&buf[sp((c >> 1) + mk_pos(y, n) * ns)]) + (c & 1);
    *slot = (y & 1) ? -v : v;
  }
  __syncthreads();
  dst_fft<R4, false, true>(buf, a, ns, 1, ns, tid);
  // per (sequence, k <= n/2): the coefficients of k and n - k, the multiplier, the inverse
  // inputs of k and n - k (each item owns its two slots)
  const float hD = (float)a.st->dtc, inv_n2 = 1.0f / ((float)n * (float)n);
  for (int it = tid; it < ns * ((n >> 1) + 1); it += nth) {
    const int q = it & (ns - 1), k = it >> ls;
    const int km = (n - k) & (n - 1);
    const C Zk = buf[sp(q + k * ns)], Zm = buf[sp(q + km * ns)];
    float cak, cbk, cam = 0.f, cbm = 0.f;
    dct_split(Zk, Zm, a.ph[k], cak, cbk);
    if (k > 0) dct_split(Zm, Zk, a.ph[n - k], cam, cbm);
    const float lxa = a.lamx[kx0 + 2 * q + 1], lxb = a.lamx[kx0 + 2 * q + 2];
    auto mult = [&](float lam) {
      float den = 1.0f - hD * lam;
      if (fabsf(den) < 1e-14f) den = 1e-14f;
      return inv_n2 / den;
    };
    // DCT index k <-> frequency n - k along y (lamy in fftfreq order of 2n: index n - k)
    cak *= mult(lxa + a.lamy[n - k]);
    cbk *= mult(lxb + a.lamy[n - k]);
    if (k > 0) {
      cam *= mult(lxa + a.lamy[k]);
      cbm *= mult(lxb + a.lamy[k]);
    }
    buf[sp(q + k * ns)] = dct_merge(cak, cam, cbk, cbm, a.ph[k]);
    if (k > 0 && km != k) buf[sp(q + km * ns)] = dct_merge(cam, cak, cbm, cbk, a.ph[n - k]);
  }
  __syncthreads();
  dst_fft<R4, true, true>(buf, a, ns, 1, ns, tid);
  for (int e = tid; e < n * Cn; e += nth) {
    const int y = e >> lc, c = e & (Cn - 1);
    const float v = reinterpret_cast<const float*>(&buf[sp((c >> 1) + mk_pos(y, n) * ns)])[c & 1];
    a.S[(long long)y * n + kx0 + c] = (y & 1) ? -v : v;
  }
}

// inverse DST-III along x of the row pairs (y, y + n/2) of a.S; w = (1/a0) result
template <int MODE, bool R4>
__global__ void __launch_bounds__(256) dst_row_inv_kernel(const __grid_constant__ NkaArgs a) {
  typedef float2 C;
  constexpr int PTS = R4 ? 4 : 16, KPTS = PTS / 2 + 1;  // elements, coefficient pairs per thread
  if (a.skip_converged && a.gs->converged) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const int n = a.n, hn = n >> 1;
  const int tps = dst_tps<R4>(n);
  const int tid = threadIdx.x, s_loc = pdiv(tid, tps), lt = tid - s_loc * tps;
  const bool active = s_loc < a.nseq;  // whole warps are launched
  const int y = blockIdx.x * a.nseq + s_loc;
  const int zb = s_loc * n;
  const float* Ta = a.S + (long long)y * n;
  const float* Tb = a.S + (long long)(y + hn) * n;
  // DCT coefficient k of row r is T_r[n - 1 - k]; each k <= n/2 fills slots k and n - k
#pragma unroll
  for (int m = 0; m < KPTS; ++m) {
    const int k = lt + m * tps;
    if (active && k <= hn) {
      const float cak = Ta[n - 1 - k], cbk = Tb[n - 1 - k];
      const float cam = k > 0 ? Ta[k - 1] : 0.f, cbm = k > 0 ? Tb[k - 1] : 0.f;
      buf[sp(zb + k)] = dct_merge(cak, cam, cbk, cbm, a.ph[k]);
      if (k > 0 && k < n - k) buf[sp(zb + n - k)] = dct_merge(cam, cak, cbm, cbk, a.ph[n - k]);
    }
  }
  __syncthreads();
  dst_fft<R4, true, false>(buf, a, a.nseq, n, 1, tid);
  const float sc = (float)a.K->inv_a0;
  float wa[PTS], wb[PTS];
#pragma unroll
  for (int m = 0; m < PTS; ++m) {
    const int x = lt + m * tps;
    wa[m] = wb[m] = 0.f;
    if (active && x < n) {
      const C v = buf[sp(zb + mk_pos(x, n))];
      const float s = (x & 1) ? -sc : sc;
      wa[m] = s * v.x;
      wb[m] = s * v.y;
    }
  }
  // idle threads (x0 = n) contribute nothing
  nka_finish<MODE, PTS>(a, active ? y : 0, active ? lt : n, tps, wa, wb);
}

// twiddles exp(-2 pi i j/n) of the n-point transforms and the phases (cos, sin)(pi k/2n)
__global__ void dst_tables_kernel(cx<float>* twn, float2* ph, int n) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)j / (double)n, &s, &c);
    twn[j] = mk<cx<float>>((float)c, (float)(-s));
    sincospi((double)j / (2.0 * (double)n), &s, &c);
    ph[j] = make_float2((float)c, (float)s);
  }
}

// V_j /= |V_j| in place and the partial dots <V_i, w>, i = 0..j, in float-float per thread;
// the last CTA sums them (FP64, fixed order) into H[i][j]
__global__ void __launch_bounds__(256) nka_dots_kernel(const __grid_constant__ NkaArgs a) {
  GmresState* gs = a.gs;
  if (gs->converged) return;
  const int jv = gs->j;
  const long long N2 = a.N2;
  const float sj = (float)gs->hnext_inv;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  __shared__ double red[NK_MAXM][8];
  const long long p0 = blockIdx.x * (long long)blockDim.x + threadIdx.x, ps = (long long)gridDim.x * blockDim.x;
  float* vj = a.V + (long long)jv * N2;
  for (long long p = p0; p < N2; p += ps) vj[p] *= sj;  // as nk_scale_j_kernel
  // four vectors per sweep, so that their loads are in flight together
  for (int i0 = 0; i0 <= jv; i0 += 4) {
    float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
    for (long long p = p0; p < N2; p += ps) {
      const float tp = a.t[p];
      float v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = i0 + u <= jv ? a.V[(long long)(i0 + u) * N2 + p] : 0.f;
#pragma unroll
      for (int u = 0; u < 4; ++u) ff_dot_acc(hi[u], lo[u], v[u], tp);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) ff_warp_sum(hi[u], lo[u]);
    if (lane == 0) {
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (i0 + u <= jv) red[i0 + u][warp] = (double)hi[u] + (double)lo[u];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= jv; i += blockDim.x) {
    double s = 0.0;
    for (int q = 0; q < nw; ++q) s += red[i][q];
    a.part[(long long)i * gridDim.x + blockIdx.x] = s;
  }
  if (!nka_last(a.ticket)) return;
  // H[i][j]: one warp per i, lanes strided over the CTAs (a fixed order)
  for (int i = warp; i <= jv; i += nw) {
    double s = 0.0;
    for (int b = lane; b < (int)gridDim.x; b += 32) s += __ldcg(&a.part[(long long)i * gridDim.x + b]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) gs->H[i * NK_MAXM + jv] = s;
  }
  if (threadIdx.x == 0) *a.ticket = 0u;
}

// V_{j+1} = w - sum_i H_ij V_i (classical Gram-Schmidt), |V_{j+1}|^2; the last CTA runs the
// Givens step of gmres_givens_kernel and, at the end of a cycle, the back substitution
__global__ void __launch_bounds__(256) nka_orth_kernel(const __grid_constant__ NkaArgs a) {
  GmresState* gs = a.gs;
  if (gs->converged) {
    if (a.use_handle && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(a.h, 0u);
    return;
  }
  const int jv = gs->j;
  const long long N2 = a.N2;
  float hc[NK_MAXM];
  for (int i = 0; i <= jv; ++i) hc[i] = (float)gs->H[i * NK_MAXM + jv];
  float* vn = a.V + (long long)(jv + 1) * N2;
  float nh = 0.f, nl = 0.f;  // |V_{j+1}|^2 partial in float-float
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    float x = a.t[p];
    int i = 0;
    for (; i + 3 <= jv; i += 4) {  // loads of four vectors in flight, the same subtraction order
      const float v0 = a.V[(long long)i * N2 + p], v1 = a.V[(long long)(i + 1) * N2 + p];
      const float v2 = a.V[(long long)(i + 2) * N2 + p], v3 = a.V[(long long)(i + 3) * N2 + p];
      x -= hc[i] * v0;
      x -= hc[i + 1] * v1;
      x -= hc[i + 2] * v2;
      x -= hc[i + 3] * v3;
    }
    for (; i <= jv; ++i) x -= hc[i] * a.V[(long long)i * N2 + p];
    vn[p] = x;
    ff_dot_acc(nh, nl, x, x);
  }
  __shared__ double red[8];
  ff_warp_sum(nh, nl);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = (double)nh + (double)nl;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
    a.part[blockIdx.x] = s;
  }
  if (!nka_last(a.ticket)) return;
  const double s = nka_sum(a.part, gridDim.x);
  if (threadIdx.x != 0) return;
  const double hn = sqrt(s);
  double* H = gs->H;
  H[(jv + 1) * NK_MAXM + jv] = hn;
  for (int i = 0; i < jv; ++i) {
    const double x = H[i * NK_MAXM + jv], y = H[(i + 1) * NK_MAXM + jv];
    H[i * NK_MAXM + jv] = gs->cs[i] * x + gs->sn[i] * y;
    H[(i + 1) * NK_MAXM + jv] = -gs->sn[i] * x + gs->cs[i] * y;
  }
  const double x = H[jv * NK_MAXM + jv], y = H[(jv + 1) * NK_MAXM + jv];
  const double den = hypot(x, y);
  const double c = den > 0 ? x / den : 1.0, sn = den > 0 ? y / den : 0.0;
  gs->cs[jv] = c;
  gs->sn[jv] = sn;
  H[jv * NK_MAXM + jv] = den;
  H[(jv + 1) * NK_MAXM + jv] = 0.0;
  gs->g[jv + 1] = -sn * gs->g[jv];
  gs->g[jv] = c * gs->g[jv];
  gs->k_used = jv + 1;
  gs->res_est = fabs(gs->g[jv + 1]);
  const bool conv = gs->res_est <= gs->tol_abs || hn == 0.0;
  gs->j = jv + 1;
  gs->hnext_inv = hn > 0 ? 1.0 / hn : 0.0;
  const bool more = !conv && gs->j < gs->m;
  if (conv) gs->converged = 1;
  if (!more) gmres_backsub(gs);
  if (a.use_handle) cudaGraphSetConditional(a.h, more ? 1u : 0u);
  *a.ticket = 0u;
}

// dx += sum_i y_i V_i; with nd, the cycle-end bookkeeping of the graph Newton loop in one
// thread: Krylov iterations, the cycle count, the next cycle while not converged and cycles remain
__global__ void nka_update_kernel(float* dx, const float* V, const GmresState* gs, long long N2, NewtonDev* nd,
                                  cudaGraphConditionalHandle hG) {
  const int k = gs->k_used;
  if (nd != nullptr && blockIdx.x == 0 && threadIdx.x == 0) {
    nd->lits += k;
    nd->cyc += 1;
    cudaGraphSetConditional(hG, (!gs->converged && nd->cyc < nd->max_krylov) ? 1u : 0u);
  }
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    double x = dx[p];
    for (int i = 0; i < k; ++i) x += gs->y[i] * (double)V[(long long)i * N2 + p];
    dx[p] = (float)x;
  }
}

// ---- fused kernels of the graph Newton loop: each does a grid-wide pass and, in its last
// CTA (the ticket of nka_last), the one-thread decision that a separate control kernel made

// Newton iteration head: R(x), -R in FP32, |R|^2 partials, dx = 0; the last CTA sets
// |R|, converged (evaluated before the update, newton_krylov.py:249-254) and the cycle flag.
// When R(x) is already at hand (nd->rvalid) the pass only clears dx.
__global__ void nd_resid_head_kernel(const double* __restrict__ x, const double* __restrict__ cst,
                                     double* __restrict__ R, float* __restrict__ b32, float* __restrict__ dx,
                                     double* part, const NKConsts* __restrict__ K, int n, double idx2,
                                     double idy2, NewtonDev* nd, unsigned* ticket,
                                     cudaGraphConditionalHandle hG) {
  const long long N2 = (long long)n * n;
  if (nd->rvalid) {
    // R(x) is already in R and -R (the initial residual, or the trial point the line search
    // accepted): the same values this pass would compute, so only dx is cleared
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
         p += (long long)gridDim.x * blockDim.x)
      dx[p] = 0.0f;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      nd->converged = nd->rn < nd->newton_tol;
      nd->cyc = 0;
      cudaGraphSetConditional(hG, nd->max_krylov > 0 ? 1u : 0u);
    }
    return;
  }
  const double a = K->pa, b = K->pb, c = K->pc, a0 = K->a0, beta = K->beta;
  double acc = 0.0;
  auto u = [&](int ii, int jj) { return dval(x, ii, jj, n); };
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j;
    nk_rowcol(p, n, i, j);
    const double r = vd_resid_at(u, i, j, cst[p], a, b, c, a0, beta, idx2, idy2);
    R[p] = r;
    b32[p] = (float)(-r);
    dx[p] = 0.0f;
    acc += r * r;
  }
  block_partial(acc, part);
  if (!nka_last(ticket)) return;
  const double s = nka_sum(part, gridDim.x);
  if (threadIdx.x != 0) return;
  nd->rn = sqrt(s);
  nd->converged = nd->rn < nd->newton_tol;
  nd->cyc = 0;
  cudaGraphSetConditional(hG, nd->max_krylov > 0 ? 1u : 0u);
  *ticket = 0u;
}

// One line-search try (newton_krylov.py:277-316): the trial point xt = x + alpha dx (built on
// the fly at every stencil point), R(xt) and its partials; the last CTA accepts on
// sufficient decrease or halves alpha, and sets the loop flag
__global__ void nd_ls_try_kernel(const double* __restrict__ x, const float* __restrict__ dx,
                                 double* __restrict__ xt, const double* __restrict__ cst, double* __restrict__ R,
                                 float* __restrict__ b32, double* part, NKConsts* K, int n, double idx2,
                                 double idy2, NewtonDev* nd, unsigned* ticket, cudaGraphConditionalHandle hL) {
  const double a = K->pa, b = K->pb, c = K->pc, a0 = K->a0, beta = K->beta, al = K->alpha;
  double acc = 0.0;
  const long long N2 = (long long)n * n;
  auto u = [&](int ii, int jj) {
    const int i2 = ii < 0 ? 0 : (ii >= n ? n - 1 : ii);
    const int j2 = jj < 0 ? 0 : (jj >= n ? n - 1 : jj);
    const long long q = (long long)i2 * n + j2;
    const double v = x[q] + al * (double)dx[q];
    return ((ii < 0) != (ii >= n)) || ((jj < 0) != (jj >= n)) ? -v : v;
  };
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j;
    nk_rowcol(p, n, i, j);
    xt[p] = x[p] + al * (double)dx[p];
    const double r = vd_resid_at(u, i, j, cst[p], a, b, c, a0, beta, idx2, idy2);
    R[p] = r;
    b32[p] = (float)(-r);
    acc += r * r;
  }
  block_partial(acc, part);
  if (!nka_last(ticket)) return;
  const double s = nka_sum(part, gridDim.x);
  if (threadIdx.x != 0) return;
  const double rnn = sqrt(s);
  nd->bt += 1;
  if (rnn < (1.0 - nd->min_decrease * al) * nd->rb) {
    nd->accepted = 1;
    nd->rb = rnn;
    cudaGraphSetConditional(hL, 0u);
  } else {
    K->alpha = al * nd->backtrack;
    cudaGraphSetConditional(hL, nd->bt < nd->max_backtrack ? 1u : 0u);
  }
  *ticket = 0u;
}

// x <- the accepted trial point, or the full damped step when no try was accepted
// (318-322), and the FP32 copy; one thread closes the iteration (residual norm, count,
// the Newton loop flag)
__global__ void nd_update_tail_kernel(double* x, const double* xt, const float* dx, float* y32, NewtonDev* nd,
                                      long long N2, cudaGraphConditionalHandle hN) {
  const bool acc = nd->accepted != 0;
  const double al = nd->damping;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < N2;
       p += (long long)gridDim.x * blockDim.x) {
    const double v = acc ? xt[p] : x[p] + al * (double)dx[p];
    x[p] = v;
    y32[p] = (float)v;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    nd->res = nd->rb;
    nd->it += 1;
    // an accepted trial point left R(x_new) in R and -R (the host loop's have_r)
    nd->rvalid = acc ? 1 : 0;
    if (acc) nd->rn = nd->rb;
    cudaGraphSetConditional(hN, (nd->it < nd->max_newton && !nd->converged) ? 1u : 0u);
  }
}

// the step constants as a kernel argument (no host staging, no stream synchronisation)
__global__ void nk_put_consts_kernel(NKConsts* K, NKConsts h) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *K = h;
}

// Newton / GMRES counts and the converged flag of the solve just run, into a device slot
__global__ void nd_stats_kernel(const NewtonDev* nd, int* slot) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    slot[0] = nd->it;
    slot[1] = nd->lits;
    slot[2] = nd->converged;
  }
}

// --------------------------------------------------------------- host driver
struct NKLayout {
  size_t y0, y1, y2, y3, y4, cst, R, xt, xn, y32, b32, dx, t, V, S, dtab, part, gs, K, pst, nd, tick, ring, total;
  int nblk, m;
};
static inline size_t al(size_t b) { return (b + 255) & ~size_t(255); }

static NKLayout nk_layout(int n, int m) {
  NKLayout L;
  const size_t N2 = (size_t)n * n;
  L.nblk = 152 * 4;
  L.m = m;
  size_t o = 0;
  L.y0 = o; o += al(N2 * 8);
  L.y1 = o; o += al(N2 * 8);
  L.y2 = o; o += al(N2 * 8);
  L.y3 = o; o += al(N2 * 8);
  L.y4 = o; o += al(N2 * 8);
  L.cst = o; o += al(N2 * 8);
  L.R = o; o += al(N2 * 8);
  L.xt = o; o += al(N2 * 8);
  L.xn = o; o += al(N2 * 8);
  L.y32 = o; o += al(N2 * 4);
  L.b32 = o; o += al(N2 * 4);
  L.dx = o; o += al(N2 * 4);
  L.t = o; o += al(N2 * 4);
  L.V = o; o += al((size_t)(m + 1) * N2 * 4);
  L.S = o; o += al(N2 * 4);                              // real DST coefficients
  L.dtab = o; o += al((size_t)(2 * n) * sizeof(float2));  // n-point twiddles, phases
  // per-CTA partials: elementwise passes (nblk CTAs) and the fused row passes (up to n/2 CTAs)
  L.part = o; o += al((size_t)(m + 2) * (size_t)(L.nblk > n / 2 ? L.nblk : n / 2) * 8);
  L.gs = o; o += al(sizeof(GmresState));
  L.K = o; o += al(sizeof(NKConsts));
  L.pst = o; o += al(sizeof(DevState));
  static_assert(sizeof(NewtonDev) <= 256, "NewtonDev outgrew its workspace slot");
  L.nd = o; o += al(256);  // NewtonDev
  L.tick = o; o += al(sizeof(unsigned));  // last-CTA ticket of the fused Arnoldi passes
  L.ring = o; o += al(3 * NK_RING * sizeof(int));  // per-step counts of the fixed-step driver
  L.total = o;
  return L;
}

struct NKRun {
  const void* plan2;  // FP32 plan of the (2n)^2 periodic grid (FD symbol, same spacing)
  int n;
  double dy, dx;
  char* ws;
  NKLayout L;
  cudaStream_t s;
  int grid;  // elementwise grid
  cudaGraphExec_t arnoldi;
  cudaGraphExec_t newton;  // the device Newton loop (null: the host loop)
};

static double* P64(NKRun& r, size_t off) { return (double*)(r.ws + off); }
static float* P32(NKRun& r, size_t off) { return (float*)(r.ws + off); }

// Arguments of the fused Arnoldi passes for this run (mode fields left zero)
static NkaArgs nka_args(NKRun& r) {
  NkaArgs a;
  memset(&a, 0, sizeof(a));
  const int n = r.n;
  const PlanView pv = plan_view(r.plan2, 2 * n, 2 * n, 4);
  a.n = n;
  a.N2 = (long long)n * n;
  a.V = P32(r, r.L.V); a.t = P32(r, r.L.t); a.src = a.t;
  a.gs = (GmresState*)(r.ws + r.L.gs); a.K = (const NKConsts*)(r.ws + r.L.K);
  a.part = P64(r, r.L.part); a.ticket = (unsigned*)(r.ws + r.L.tick);
  a.log2n = ilog2_exact(n);
  a.S = P32(r, r.L.S);
  a.twn = (const cx<float>*)(r.ws + r.L.dtab);
  a.ph = (const float2*)(r.ws + r.L.dtab) + n;
  a.lamx = (const float*)pv.lamx; a.lamy = (const float*)pv.lamy;
  a.st = (const DevState*)(r.ws + r.L.pst);
  return a;
}

// CTA geometry of the DST passes: rows in pairs (y, y + n/2), tps threads per pair (n/16 for
// radix 16, n/4 for radix 4), fewer pairs per CTA until the pass covers every SM, at most 256
// threads, whole warps (the threads past nseq * tps idle); columns in tiles of C (even) real
// columns, C/2 complex sequences, at least 152 tiles where n allows and within the default
// 48 KB of shared memory
struct DstGeom { int nseq, ctas, threads, C, col_threads; size_t smem, col_smem; };
static DstGeom dst_geom(int n, bool r4) {
  DstGeom g;
  const int hn = n / 2, tps = r4 ? (n >= 4 ? n / 4 : 1) : (n >= 16 ? n / 16 : 1);
  int ns = row_nseq(n, hn);
  if (ns > hn) ns = hn;
  while (ns > 1 && (hn / ns < 152 || ns * tps > 256)) ns >>= 1;
  g.nseq = ns;
  g.ctas = hn / ns;
  g.threads = ((ns * tps + 31) / 32) * 32;
  g.smem = (size_t)sp_size(ns * n) * sizeof(float2);
  int C = 8 < n ? 8 : n;
  while (C > 2 && (n / C < 152 || (size_t)sp_size(n * (C / 2)) * sizeof(float2) > 48 * 1024 ||
                   (C / 2) * tps > 256))
    C >>= 1;
  g.C = C;
  g.col_threads = (((C / 2) * tps + 31) / 32) * 32;
  g.col_smem = (size_t)sp_size(n * (C / 2)) * sizeof(float2);
  return g;
}

// Radix 4 for the DST passes up to n = 512: at most n/2 row pairs and n/2 column pairs per
// pass, too few sequences for the radix-16 schedule's n/16 threads each to fill the SMs, so the
// pass lasts one sequence's dependent work, a quarter as long with n/4 threads per sequence
static bool dst_r4(int n) { return n <= 512; }

// w = M^-1 a.src: DST-II along x, along y with the multiplier and DST-III along y, DST-III
// along x (MODE: w into t, or the cycle start V_0 = w)
template <int MODE>
static cudaError_t nka_precond(NKRun& r, NkaArgs a) {
  const bool r4 = dst_r4(r.n);
  const DstGeom g = dst_geom(r.n, r4);
  a.nseq = g.nseq;
  a.C = g.C;
  if (r4) {
    dst_row_fwd_kernel<true><<<g.ctas, g.threads, g.smem, r.s>>>(a);
    dst_col_kernel<true><<<r.n / g.C, g.col_threads, g.col_smem, r.s>>>(a);
    dst_row_inv_kernel<MODE, true><<<g.ctas, g.threads, g.smem, r.s>>>(a);
  } else {
    dst_row_fwd_kernel<false><<<g.ctas, g.threads, g.smem, r.s>>>(a);
    dst_col_kernel<false><<<r.n / g.C, g.col_threads, g.col_smem, r.s>>>(a);
    dst_row_inv_kernel<MODE, false><<<g.ctas, g.threads, g.smem, r.s>>>(a);
  }
  return cudaGetLastError();
}

// The cycle start: V_0 = M^-1 (b - A dx) (first: M^-1 b), |V_0|, the GMRES header and, with a
// handle, the Arnoldi loop flag
static cudaError_t cycle_start(NKRun& r, NkaArgs a, bool first_plain) {
  const long long N2 = (long long)r.n * r.n;
  if (!first_plain) {
    vd_jvp_j_kernel<<<r.grid, 256, 0, r.s>>>(P32(r, r.L.y32), P32(r, r.L.dx), nullptr, P32(r, r.L.t),
                                             (const NKConsts*)(r.ws + r.L.K), r.n, (float)(1.0 / (r.dx * r.dx)),
                                             (float)(1.0 / (r.dy * r.dy)), N2, P32(r, r.L.b32));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    a.src = P32(r, r.L.t);
  } else {
    a.src = P32(r, r.L.b32);
  }
  a.skip_converged = 0;
  return nka_precond<NKA_START>(r, a);
}

// One Arnoldi step: t = A V_j/|V_j|, w = M^-1 t, V_j normalised and H[:, j], V_{j+1}, the
// Givens step and the loop flag, in six kernels (the index j lives on the device)
static cudaError_t arnoldi_step(NKRun& r, cudaGraphConditionalHandle h, int use_handle) {
  const long long N2 = (long long)r.n * r.n;
  NkaArgs a = nka_args(r);
  a.h = h;
  a.use_handle = use_handle;
  a.skip_converged = 1;
  vd_jvp_j_kernel<<<r.grid, 256, 0, r.s>>>(P32(r, r.L.y32), a.V, a.gs, a.t, a.K, r.n, (float)(1.0 / (r.dx * r.dx)),
                                           (float)(1.0 / (r.dy * r.dy)), N2);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if ((e = nka_precond<NKA_STORE_W>(r, a)) != cudaSuccess) return e;
  nka_dots_kernel<<<r.L.nblk, 256, 0, r.s>>>(a);
  nka_orth_kernel<<<r.L.nblk, 256, 0, r.s>>>(a);
  return cudaGetLastError();
}

static cudaError_t build_arnoldi_graph(NKRun& r) {
  cudaStream_t cs = nullptr;
  cudaGraph_t graph = nullptr;
  cudaError_t ce = cudaSuccess;
  r.arnoldi = nullptr;
  do {
    if ((ce = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) break;
    if ((ce = cudaGraphCreate(&graph, 0)) != cudaSuccess) break;
    cudaGraphConditionalHandle hdl;
    if ((ce = cudaGraphConditionalHandleCreate(&hdl, graph, 1, cudaGraphCondAssignDefault)) != cudaSuccess) break;
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = hdl;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if ((ce = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np)) != cudaSuccess) break;
    cudaGraph_t body = np.conditional.phGraph_out[0];
    NKRun rc = r;
    rc.s = cs;
    if ((ce = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) break;
    const cudaError_t le = arnoldi_step(rc, hdl, 1);
    cudaGraph_t captured = nullptr;
    ce = cudaStreamEndCapture(cs, &captured);
    if (le != cudaSuccess) { ce = le; break; }
    if (ce != cudaSuccess) break;
    ce = cudaGraphInstantiate(&r.arnoldi, graph, 0);
  } while (0);
  if (graph) cudaGraphDestroy(graph);
  if (cs) cudaStreamDestroy(cs);
  return ce;
}

struct NKParamsC {
  int max_newton, max_krylov, restart, max_backtrack;
  double newton_tol, krylov_tol, damping, backtrack, min_decrease;
};

// ---- the device Newton loop as one graph (nested conditional while nodes) ----
// Appends the work that seg() enqueues on the capture stream to graph g after deps and
// returns the nodes that end it.
template <typename F>
static cudaError_t capture_seg(cudaStream_t cs, cudaGraph_t g, std::vector<cudaGraphNode_t>& deps, F seg) {
  cudaError_t ce = cudaStreamBeginCaptureToGraph(cs, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                                                 cudaStreamCaptureModeThreadLocal);
  if (ce != cudaSuccess) return ce;
  const cudaError_t le = seg(cs);
  cudaStreamCaptureStatus stt;
  const cudaGraphNode_t* d = nullptr;
  size_t nd = 0;
  ce = cudaStreamGetCaptureInfo(cs, &stt, nullptr, nullptr, &d, nullptr, &nd);
  std::vector<cudaGraphNode_t> out;
  if (ce == cudaSuccess) out.assign(d, d + nd);
  cudaGraph_t captured = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(cs, &captured);
  if (le != cudaSuccess) return le;
  if (ce != cudaSuccess) return ce;
  if (ee != cudaSuccess) return ee;
  deps = out;
  return cudaSuccess;
}

// Builds r.newton: the Newton loop on the iterate buffer xn with the preconditioned
// restarted GMRES, line search and counters of NewtonDev (parameters written here).
static cudaError_t build_newton_graph(NKRun& r, const NKParamsC& P) {
  const long long N2 = (long long)r.n * r.n;
  NewtonDev h;
  memset(&h, 0, sizeof(h));
  h.max_newton = P.max_newton; h.max_krylov = P.max_krylov; h.max_backtrack = P.max_backtrack; h.restart = P.restart;
  h.newton_tol = P.newton_tol; h.krylov_tol = P.krylov_tol; h.damping = P.damping; h.backtrack = P.backtrack;
  h.min_decrease = P.min_decrease;
  NewtonDev* nd = (NewtonDev*)(r.ws + r.L.nd);
  cudaError_t ce = cudaMemcpyAsync(nd, &h, sizeof(h), cudaMemcpyHostToDevice, r.s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(r.s);  // h is a host stack value
  if (ce != cudaSuccess) return ce;
  NKConsts* K = (NKConsts*)(r.ws + r.L.K);
  GmresState* gs = (GmresState*)(r.ws + r.L.gs);
  double* x = P64(r, r.L.xn);
  double* xt = P64(r, r.L.xt);
  float* y32 = P32(r, r.L.y32);
  float* dx = P32(r, r.L.dx);
  float* V = P32(r, r.L.V);
  float* b32 = P32(r, r.L.b32);
  double* part = P64(r, r.L.part);
  double* R = P64(r, r.L.R);
  double* cst = P64(r, r.L.cst);
  unsigned* tick = (unsigned*)(r.ws + r.L.tick);
  const int nblk = r.L.nblk, grid = r.grid, n = r.n;
  const double idx2 = 1.0 / (r.dx * r.dx), idy2 = 1.0 / (r.dy * r.dy);
  cudaStream_t cs = nullptr;
  cudaGraph_t top = nullptr;
  do {
    if ((ce = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) break;
    if ((ce = cudaGraphCreate(&top, 0)) != cudaSuccess) break;
    NKRun rc = r;
    rc.s = cs;
    cudaGraphConditionalHandle hN, hG, hA, hL;
    cudaGraph_t bN, bG, bA, bL;
    std::vector<cudaGraphNode_t> d;
    // before the loop: y32 = x, R(x), converged
    if ((ce = capture_seg(cs, top, d, [&](cudaStream_t q) {
           lincomb_kernel<<<grid, 256, 0, q>>>(x, 1.0, nullptr, 0.0, x, y32, N2);
           vd_residual_kernel<<<nblk, 256, 0, q>>>(x, cst, R, b32, part, K, n, idx2, idy2);
           return cudaGetLastError();
         })) != cudaSuccess) break;
    if ((ce = cudaGraphConditionalHandleCreate(&hN, top, 0, 0)) != cudaSuccess) break;
    if ((ce = capture_seg(cs, top, d, [&](cudaStream_t q) {
           nd_init_kernel<<<1, 256, 0, q>>>(part, nblk, nd, hN);
           return cudaGetLastError();
         })) != cudaSuccess) break;
    {
      cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
      np.conditional.handle = hN;
      np.conditional.type = cudaGraphCondTypeWhile;
      np.conditional.size = 1;
      cudaGraphNode_t node;
      if ((ce = cudaGraphAddNode(&node, top, d.data(), nullptr, d.size(), &np)) != cudaSuccess) break;
      bN = np.conditional.phGraph_out[0];
    }
    // Newton body: R(x) and its norm, dx = 0, and the GMRES cycle loop flag
    std::vector<cudaGraphNode_t> dn;
    if ((ce = cudaGraphConditionalHandleCreate(&hG, bN, 0, 0)) != cudaSuccess) break;
    if ((ce = capture_seg(cs, bN, dn, [&](cudaStream_t q) {
           nd_resid_head_kernel<<<nblk, 256, 0, q>>>(x, cst, R, b32, dx, part, K, n, idx2, idy2, nd, tick, hG);
           return cudaGetLastError();
         })) != cudaSuccess) break;
    {
      cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
      np.conditional.handle = hG;
      np.conditional.type = cudaGraphCondTypeWhile;
      np.conditional.size = 1;
      cudaGraphNode_t node;
      if ((ce = cudaGraphAddNode(&node, bN, dn.data(), nullptr, dn.size(), &np)) != cudaSuccess) break;
      bG = np.conditional.phGraph_out[0];
      dn.assign(1, node);
    }
    // GMRES cycle: r = b - J dx, V_0 = M^-1 r, |V_0|; the Arnoldi loop; solve and update
    std::vector<cudaGraphNode_t> dg;
    if ((ce = cudaGraphConditionalHandleCreate(&hA, bG, 0, 0)) != cudaSuccess) break;
    if ((ce = capture_seg(cs, bG, dg, [&](cudaStream_t q) {
           // V_0 = M^-1 (b - A dx), |V_0|, the cycle start and the Arnoldi loop flag
           NkaArgs a = nka_args(rc);
           a.nd = nd;
           a.h = hA;
           a.use_handle = 1;
           return cycle_start(rc, a, false);
         })) != cudaSuccess) break;
    {
      cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
      np.conditional.handle = hA;
      np.conditional.type = cudaGraphCondTypeWhile;
      np.conditional.size = 1;
      cudaGraphNode_t node;
      if ((ce = cudaGraphAddNode(&node, bG, dg.data(), nullptr, dg.size(), &np)) != cudaSuccess) break;
      bA = np.conditional.phGraph_out[0];
      dg.assign(1, node);
    }
    std::vector<cudaGraphNode_t> da;
    if ((ce = capture_seg(cs, bA, da, [&](cudaStream_t) { return arnoldi_step(rc, hA, 1); })) != cudaSuccess) break;
    if ((ce = capture_seg(cs, bG, dg, [&](cudaStream_t q) {
           // y was back-substituted by the last Arnoldi step of the cycle
           nka_update_kernel<<<grid, 256, 0, q>>>(dx, V, gs, N2, nd, hG);
           return cudaGetLastError();
         })) != cudaSuccess) break;
    // line search
    if ((ce = cudaGraphConditionalHandleCreate(&hL, bN, 0, 0)) != cudaSuccess) break;
    if ((ce = capture_seg(cs, bN, dn, [&](cudaStream_t q) {
           nd_ls_begin_kernel<<<1, 32, 0, q>>>(nd, K, hL);
           return cudaGetLastError();
         })) != cudaSuccess) break;
    {
      cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
      np.conditional.handle = hL;
      np.conditional.type = cudaGraphCondTypeWhile;
      np.conditional.size = 1;
      cudaGraphNode_t node;
      if ((ce = cudaGraphAddNode(&node, bN, dn.data(), nullptr, dn.size(), &np)) != cudaSuccess) break;
      bL = np.conditional.phGraph_out[0];
      dn.assign(1, node);
    }
    std::vector<cudaGraphNode_t> dl;
    if ((ce = capture_seg(cs, bL, dl, [&](cudaStream_t q) {
           nd_ls_try_kernel<<<nblk, 256, 0, q>>>(x, dx, xt, cst, R, b32, part, K, n, idx2, idy2, nd, tick, hL);
           return cudaGetLastError();
         })) != cudaSuccess) break;
    // the step and the loop flag
    if ((ce = capture_seg(cs, bN, dn, [&](cudaStream_t q) {
           nd_update_tail_kernel<<<grid, 256, 0, q>>>(x, xt, dx, y32, nd, N2, hN);
           return cudaGetLastError();
         })) != cudaSuccess) break;
    ce = cudaGraphInstantiate(&r.newton, top, 0);
  } while (0);
  if (top) cudaGraphDestroy(top);
  if (cs) cudaStreamDestroy(cs);
  if (ce != cudaSuccess) {
    if (r.newton) cudaGraphExecDestroy(r.newton);
    r.newton = nullptr;
  }
  return ce;
}

// Newton on the device graph: x is copied into the iterate buffer, the graph runs the
// whole iteration, the counters come back with one synchronisation.
static cudaError_t newton_dev(NKRun& r, double* x, int* n_newton, int* n_lin, int* conv_out, double* res_out) {
  const long long N2 = (long long)r.n * r.n;
  double* xn = P64(r, r.L.xn);
  cudaError_t e = cudaMemcpyAsync(xn, x, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
  if (e == cudaSuccess) e = cudaGraphLaunch(r.newton, r.s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(x, xn, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
  NewtonDev h;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, r.ws + r.L.nd, sizeof(h), cudaMemcpyDeviceToHost, r.s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r.s);
  if (e != cudaSuccess) return e;
  *n_newton = h.it; *n_lin = h.lits; *conv_out = h.converged; *res_out = h.res;
  return cudaSuccess;
}

// The same without the read-back: the counts go to a device slot (fixed-step driver)
static cudaError_t newton_dev_async(NKRun& r, double* x, int* slot) {
  const long long N2 = (long long)r.n * r.n;
  double* xn = P64(r, r.L.xn);
  cudaError_t e = cudaMemcpyAsync(xn, x, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
  if (e == cudaSuccess) e = cudaGraphLaunch(r.newton, r.s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(x, xn, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
  if (e != cudaSuccess) return e;
  nd_stats_kernel<<<1, 32, 0, r.s>>>((const NewtonDev*)(r.ws + r.L.nd), slot);
  return cudaGetLastError();
}

static cudaError_t norm_of(NKRun& r, double* part_dev, double* host_out) {
  // the residual kernel already left per-block partial sums in part_dev
  double h[152 * 4];
  cudaError_t e = cudaMemcpyAsync(h, part_dev, sizeof(double) * r.L.nblk, cudaMemcpyDeviceToHost, r.s);
  if (e != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(r.s)) != cudaSuccess) return e;
  double s = 0.0;
  for (int i = 0; i < r.L.nblk; ++i) s += h[i];
  *host_out = sqrt(s);
  return cudaSuccess;
}

// R(x) into R (FP64), optionally -R into b32; returns |R|
static cudaError_t residual(NKRun& r, const double* x, double* rnorm, bool rhs) {
  NKConsts* K = (NKConsts*)(r.ws + r.L.K);
  vd_residual_kernel<<<r.L.nblk, 256, 0, r.s>>>(x, P64(r, r.L.cst), P64(r, r.L.R),
                                                rhs ? P32(r, r.L.b32) : nullptr, P64(r, r.L.part), K,
                                                r.n, 1.0 / (r.dx * r.dx), 1.0 / (r.dy * r.dy));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return norm_of(r, P64(r, r.L.part), rnorm);
}


// Newton on R(x) = 0 from the guess in x (FP64, updated in place)
static cudaError_t newton(NKRun& r, double* x, const NKParamsC& P, int* n_newton, int* n_lin,
                          int* conv_out, double* res_out) {
  const long long N2 = (long long)r.n * r.n;
  NKConsts* K = (NKConsts*)(r.ws + r.L.K);
  GmresState* gs = (GmresState*)(r.ws + r.L.gs);
  float* y32 = P32(r, r.L.y32);
  float* dx = P32(r, r.L.dx);
  float* V = P32(r, r.L.V);
  double* xt = P64(r, r.L.xt);
  cudaError_t e;
  double rn;
  lincomb_kernel<<<r.grid, 256, 0, r.s>>>(x, 1.0, nullptr, 0.0, x, y32, N2);
  if ((e = residual(r, x, &rn, true)) != cudaSuccess) return e;
  int converged = rn < P.newton_tol;  // initial state (newton_krylov.py:338-346)
  int it = 0, lits = 0;
  double res = rn;
  bool have_r = true;  // R and b32 hold R(x), y32 holds x
  while (it < P.max_newton && !converged) {
    if (!have_r) {
      lincomb_kernel<<<r.grid, 256, 0, r.s>>>(x, 1.0, nullptr, 0.0, x, y32, N2);
      if ((e = residual(r, x, &rn, true)) != cudaSuccess) return e;
    }
    converged = rn < P.newton_tol;  // evaluated before the update (newton_krylov.py:249-254)
    // restarted GMRES on M^-1 J dx = -M^-1 R
    if ((e = cudaMemsetAsync(dx, 0, sizeof(float) * N2, r.s)) != cudaSuccess) return e;
    for (int cyc = 0; cyc < P.max_krylov; ++cyc) {
      // V_0 = M^-1 b (first cycle) or M^-1 (b - J dx), |V_0| and the cycle start
      NkaArgs a = nka_args(r);
      a.first = cyc == 0;
      a.tol = P.krylov_tol;
      a.m = P.restart;
      if ((e = cycle_start(r, a, cyc == 0)) != cudaSuccess) return e;
      if (host_loop_mode()) {
        // MJX_HOST_LOOP=1: the host launches every Arnoldi step and reads the GMRES header
        // after it (the same kernels and decisions; profilers then see each launch)
        for (int k = 0; k < P.restart; ++k) {
          int g4[4];
          if ((e = cudaMemcpyAsync(g4, gs, sizeof(g4), cudaMemcpyDeviceToHost, r.s)) != cudaSuccess) return e;
          if ((e = cudaStreamSynchronize(r.s)) != cudaSuccess) return e;
          if (g4[2] || g4[0] >= g4[1]) break;  // converged, or j == m
          if ((e = arnoldi_step(r, 0, 0)) != cudaSuccess) return e;
        }
      } else if ((e = cudaGraphLaunch(r.arnoldi, r.s)) != cudaSuccess) {
        return e;
      }
      // the last Arnoldi step of the cycle back-substituted y
      nka_update_kernel<<<r.grid, 256, 0, r.s>>>(dx, V, gs, N2, nullptr, 0);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      int hdr[4];
      if ((e = cudaMemcpyAsync(hdr, gs, sizeof(hdr), cudaMemcpyDeviceToHost, r.s)) != cudaSuccess) return e;
      if ((e = cudaStreamSynchronize(r.s)) != cudaSuccess) return e;
      lits += hdr[3];  // k_used
      if (hdr[2]) break;  // converged
    }
    // backtracking line search (newton_krylov.py:270-316)
    double alpha = P.damping, rb = rn;
    bool acc = false;
    for (int bt = 0; bt < P.max_backtrack && !acc; ++bt) {
      if ((e = cudaMemcpyAsync(&K->alpha, &alpha, sizeof(double), cudaMemcpyHostToDevice, r.s)) != cudaSuccess) return e;
      trial_kernel<<<r.grid, 256, 0, r.s>>>(x, dx, xt, K, nullptr, N2);
      double rnn;
      if ((e = residual(r, xt, &rnn, true)) != cudaSuccess) return e;
      if (rnn < (1.0 - P.min_decrease * alpha) * rb) {
        acc = true;
        rb = rnn;
        if ((e = cudaMemcpyAsync(x, xt, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s)) != cudaSuccess) return e;
      } else {
        alpha *= P.backtrack;
      }
    }
    if (acc) {
      have_r = true;  // R/b32 hold R(x_new); refresh the FP32 copy
      lincomb_kernel<<<r.grid, 256, 0, r.s>>>(x, 1.0, nullptr, 0.0, x, y32, N2);
      rn = rb;
    } else {
      // no try accepted: full damped step (newton_krylov.py:318-322)
      if ((e = cudaMemcpyAsync(&K->alpha, &P.damping, sizeof(double), cudaMemcpyHostToDevice, r.s)) != cudaSuccess) return e;
      trial_kernel<<<r.grid, 256, 0, r.s>>>(x, dx, x, K, y32, N2);
      have_r = false;
    }
    res = rb;
    ++it;
  }
  if ((e = cudaStreamSynchronize(r.s)) != cudaSuccess) return e;
  *n_newton = it; *n_lin = lits; *conv_out = converged; *res_out = res;
  return cudaSuccess;
}

// One implicit step of the reference step functions: be_step (stepping.py:170-214),
// cn_step (217-260) or bdf2_step (263-310, omega = dt/dt_prev), residuals from
// create_implicit_residual / create_bdf2_residual (newton_krylov.py:362-448).
// yc = y_n, yp = y_{n-1} (BDF2 only); the solution is written to yout.
struct StepOut { int newton, lin, converged; double res; };

// With dev_slot (device Newton loop only) the step enqueues its work and leaves the counts
// in dev_slot without a host synchronisation; so is left untouched.
static cudaError_t implicit_step(NKRun& r, const NKParamsC& P, const double* abc, int method,
                                 double dt, double dt_prev, int guess_previous, const double* yc,
                                 const double* yp, double* yout, StepOut* so, int* dev_slot = nullptr) {
  const long long N2 = (long long)r.n * r.n;
  NKConsts* K = (NKConsts*)(r.ws + r.L.K);
  DevState* pst = (DevState*)(r.ws + r.L.pst);
  double* cst = P64(r, r.L.cst);
  const double idx2 = 1.0 / (r.dx * r.dx), idy2 = 1.0 / (r.dy * r.dy);
  NKConsts h;
  memset(&h, 0, sizeof(h));
  h.pa = abc[0]; h.pb = abc[1]; h.pc = abc[2];
  double a1 = -1.0, a2 = 0.0;
  if (method == MJX_METHOD_BE) {
    h.a0 = 1.0; h.beta = dt;
  } else if (method == MJX_METHOD_BDF2) {
    const double om = dt / dt_prev;
    h.a0 = (1 + 2 * om) / (1 + om); a1 = -(1 + om); a2 = om * om / (1 + om);
    h.beta = dt * (1 + om) / (1 + 2 * om);
  } else {  // CN: R = y - y_n - dt/2 (F_n + F(y)); F_n folded into cst below
    h.a0 = 1.0; h.beta = 0.5 * dt;
  }
  h.alpha = 1.0;
  nk_put_consts_kernel<<<1, 32, 0, r.s>>>(K, h);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (method == MJX_METHOD_CN) {
    // R(y_n) with cst = 0 is y_n - dt/2 F(y_n); cst = -y_n - dt/2 F(y_n) = R(y_n) - 2 y_n
    lincomb_kernel<<<r.grid, 256, 0, r.s>>>(yc, 0.0, nullptr, 0.0, cst, nullptr, N2);
    vd_residual_kernel<<<r.L.nblk, 256, 0, r.s>>>(yc, cst, P64(r, r.L.R), nullptr, P64(r, r.L.part), K,
                                                  r.n, idx2, idy2);
    lincomb_kernel<<<r.grid, 256, 0, r.s>>>(P64(r, r.L.R), 1.0, yc, -2.0, cst, nullptr, N2);
  } else {
    lincomb_kernel<<<r.grid, 256, 0, r.s>>>(yc, a1, yp, a2, cst, nullptr, N2);
  }
  // initial guess: BDF2 -> 2 y_n - y_{n-1}; BE/CN -> explicit Euler y_n + dt F(y_n)
  // (stepping.py:195-196, 242-243) or, with guess_previous == 1, y_n; guess_previous == 2
  // keeps the guess the caller left in yout (newton_krylov_solve's x0)
  if (guess_previous == 2) {
  } else if (method == MJX_METHOD_BDF2) {
    lincomb_kernel<<<r.grid, 256, 0, r.s>>>(yc, 2.0, yp, -1.0, yout, nullptr, N2);
  } else if (guess_previous) {
    lincomb_kernel<<<r.grid, 256, 0, r.s>>>(yc, 1.0, nullptr, 0.0, yout, nullptr, N2);
  } else {
    // the residual kernel with a0 = 0, beta = -dt, cst = y_n gives y_n + dt F(y_n)
    NKConsts ge = h;
    ge.a0 = 0.0; ge.beta = -dt;
    nk_put_consts_kernel<<<1, 32, 0, r.s>>>(K, ge);
    vd_residual_kernel<<<r.L.nblk, 256, 0, r.s>>>(yc, yc, yout, nullptr, P64(r, r.L.part), K, r.n, idx2, idy2);
    nk_put_consts_kernel<<<1, 32, 0, r.s>>>(K, h);
  }
  // preconditioner constants from y_n
  sumsq_kernel<<<r.L.nblk, 256, 0, r.s>>>(yc, P64(r, r.L.part), N2);
  nk_consts_kernel<<<1, 256, 0, r.s>>>(P64(r, r.L.part), r.L.nblk, K, pst, (double)N2);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (r.newton != nullptr && dev_slot != nullptr) return newton_dev_async(r, yout, dev_slot);
  if (r.newton != nullptr) return newton_dev(r, yout, &so->newton, &so->lin, &so->converged, &so->res);
  return newton(r, yout, P, &so->newton, &so->lin, &so->converged, &so->res);
}

// dt * F(y) into out (the BE error estimate of adaptive_integrate, stepping.py:823-826)
static cudaError_t scaled_rhs(NKRun& r, const double* abc, double dt, const double* y, double* out) {
  vd_rhs_kernel<<<r.grid, 256, 0, r.s>>>(y, out, abc[0], abc[1], abc[2], dt, r.n, 1.0 / (r.dx * r.dx),
                                         1.0 / (r.dy * r.dy));
  return cudaGetLastError();
}

// NaN-propagating min/max (jnp.minimum / jnp.maximum)
static inline double hmax(double a, double b) { return (a != a || b != b) ? a + b : (a > b ? a : b); }
static inline double hmin(double a, double b) { return (a != a || b != b) ? a + b : (a < b ? a : b); }
static inline double hclip(double x, double lo, double hi) { return hmin(hmax(x, lo), hi); }

static mjx_status nk_setup(NKRun& r, const void* plan2, int n, double dy, double dx,
                           const mjx_nk_params* nkp, void* ws, size_t ws_bytes, void* stream,
                           NKParamsC* P) {
  if (ilog2_exact(n) < 1 || n > 2048 || !(dx > 0) || !(dy > 0)) return MJX_BAD_SHAPE;
  if (nkp->restart < 1 || nkp->restart > NK_MAXM) return MJX_BAD_ARG;
  r.plan2 = plan2; r.n = n; r.dy = dy; r.dx = dx; r.ws = (char*)ws; r.L = nk_layout(n, nkp->restart);
  r.s = (cudaStream_t)stream;
  r.grid = 152 * 4;
  r.arnoldi = nullptr;
  r.newton = nullptr;
  if (ws == nullptr || ws_bytes < r.L.total) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  MJX_CUDA_TRY(cudaMemsetAsync(r.ws + r.L.pst, 0, sizeof(DevState), r.s));
  MJX_CUDA_TRY(cudaMemsetAsync(r.ws + r.L.tick, 0, sizeof(unsigned), r.s));
  dst_tables_kernel<<<(n + 255) / 256, 256, 0, r.s>>>((cx<float>*)(r.ws + r.L.dtab),
                                                      (float2*)(r.ws + r.L.dtab) + n, n);
  MJX_CUDA_TRY(cudaGetLastError());
  P->max_newton = nkp->max_newton_iters; P->max_krylov = nkp->max_krylov_iters; P->restart = nkp->restart;
  P->max_backtrack = nkp->max_backtrack; P->newton_tol = nkp->newton_tol; P->krylov_tol = nkp->krylov_tol;
  P->damping = nkp->damping; P->backtrack = nkp->backtrack_factor; P->min_decrease = nkp->min_residual_decrease;
  MJX_CUDA_TRY(build_arnoldi_graph(r));
  // the device Newton loop; without nested conditional graphs the host loop runs instead
  if (!host_loop_mode() && build_newton_graph(r, *P) != cudaSuccess) (void)cudaGetLastError();
  return MJX_OK;
}

}  // namespace mjx

using namespace mjx;

extern "C" {

size_t mjx_nk_vardiff_ws_bytes(int n, int restart) {
  if (ilog2_exact(n) < 1 || n > 2048 || restart < 1 || restart > NK_MAXM) return 0;
  return nk_layout(n, restart).total;
}

mjx_status mjx_nk_vardiff_integrate2d(const void* plan2, int n, double dy, double dx,
                                      const double* model_abc, int method, double dt, int n_steps,
                                      int be_guess_previous, const mjx_nk_params* nkp,
                                      const double* y0, double* y_out, int* stats, void* ws,
                                      size_t ws_bytes, void* stream) {
  if (plan2 == nullptr || model_abc == nullptr || nkp == nullptr || y0 == nullptr || y_out == nullptr)
    return MJX_BAD_ARG;
  if (n_steps < 0) return MJX_BAD_SHAPE;
  if (method != MJX_METHOD_BE && method != MJX_METHOD_CN && method != MJX_METHOD_BDF2) return MJX_BAD_ARG;
  NKRun r;
  NKParamsC P;
  MJX_TRY(nk_setup(r, plan2, n, dy, dx, nkp, ws, ws_bytes, stream, &P));
  const long long N2 = (long long)n * n;
  double* yp = P64(r, r.L.y0);   // y_{n-1}
  double* yc = P64(r, r.L.y1);   // y_n
  double* yn = P64(r, r.L.y2);   // Newton iterate
  mjx_status rc = MJX_OK;
  cudaError_t e = cudaMemcpyAsync(yc, y0, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(yp, y0, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
  if (e != cudaSuccess) { set_last_error(e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; }
  // integrate_fixed_dt (stepping.py:1028-1139): BDF2 takes a BE first step.  With the
  // device Newton loop no step reads anything back: the counts collect in a device ring
  // that the host reads every NK_RING steps.
  int* ring = (int*)(r.ws + r.L.ring);
  for (int step = 0; step < n_steps && rc == MJX_OK; ++step) {
    const int m = (method == MJX_METHOD_BDF2 && step == 0) ? MJX_METHOD_BE : method;
    StepOut so;
    int* slot = r.newton != nullptr ? ring + 3 * (step % NK_RING) : nullptr;
    e = implicit_step(r, P, model_abc, m, dt, dt, be_guess_previous, yc, yp, yn, &so, slot);
    if (e == cudaSuccess && slot != nullptr && (step % NK_RING == NK_RING - 1 || step == n_steps - 1)) {
      const int first = step - step % NK_RING, cnt = step - first + 1;
      if (stats) e = cudaMemcpyAsync(stats + 3 * first, ring, sizeof(int) * 3 * cnt, cudaMemcpyDeviceToHost, r.s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(r.s);
    }
    if (e != cudaSuccess) { set_last_error(e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; break; }
    if (stats && slot == nullptr) {
      stats[3 * step] = so.newton; stats[3 * step + 1] = so.lin; stats[3 * step + 2] = so.converged;
    }
    // rotate y_{n-1} <- y_n <- y_{n+1}
    double* tmp = yp; yp = yc; yc = yn; yn = tmp;
  }
  if (rc == MJX_OK) {
    e = cudaMemcpyAsync(y_out, yc, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r.s);
    if (e != cudaSuccess) { set_last_error(e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; }
  }
  if (r.arnoldi) cudaGraphExecDestroy(r.arnoldi);
  if (r.newton) cudaGraphExecDestroy(r.newton);
  return rc;
}

mjx_status mjx_vardiff_rhs2d(int n, double dy, double dx, const double* model_abc, const double* y,
                             double* out, void* stream) {
  if (model_abc == nullptr || y == nullptr || out == nullptr) return MJX_BAD_ARG;
  if (n < 1 || !(dx > 0) || !(dy > 0)) return MJX_BAD_SHAPE;
  vd_rhs_kernel<<<152 * 4, 256, 0, (cudaStream_t)stream>>>(y, out, model_abc[0], model_abc[1], model_abc[2],
                                                           1.0, n, 1.0 / (dx * dx), 1.0 / (dy * dy));
  return cuda_status(cudaGetLastError());
}

mjx_status mjx_vardiff_jvp2d(int n, double dy, double dx, const double* model_abc, double a0, double beta,
                             const double* u, const double* v, double* out, void* stream) {
  if (model_abc == nullptr || u == nullptr || v == nullptr || out == nullptr) return MJX_BAD_ARG;
  if (n < 1 || !(dx > 0) || !(dy > 0)) return MJX_BAD_SHAPE;
  vd_jvp64_kernel<<<152 * 4, 256, 0, (cudaStream_t)stream>>>(u, v, out, model_abc[0], model_abc[1], model_abc[2],
                                                             a0, beta, n, 1.0 / (dx * dx), 1.0 / (dy * dy),
                                                             (long long)n * n);
  return cuda_status(cudaGetLastError());
}

mjx_status mjx_nk_vardiff_step2d(const void* plan2, int n, double dy, double dx,
                                 const double* model_abc, int method, double dt, double dt_prev,
                                 int be_guess_previous, const mjx_nk_params* nkp, const double* y_n,
                                 const double* y_prev, double* y_out, int* stats, double* res_norm,
                                 void* ws, size_t ws_bytes, void* stream) {
  if (plan2 == nullptr || model_abc == nullptr || nkp == nullptr || y_n == nullptr || y_out == nullptr)
    return MJX_BAD_ARG;
  if (method != MJX_METHOD_BE && method != MJX_METHOD_CN && method != MJX_METHOD_BDF2) return MJX_BAD_ARG;
  if (method == MJX_METHOD_BDF2 && (y_prev == nullptr || !(dt_prev > 0))) return MJX_BAD_ARG;
  NKRun r;
  NKParamsC P;
  MJX_TRY(nk_setup(r, plan2, n, dy, dx, nkp, ws, ws_bytes, stream, &P));
  const long long N2 = (long long)n * n;
  double* yc = P64(r, r.L.y1);
  double* yp = P64(r, r.L.y0);
  double* yn = P64(r, r.L.y2);
  mjx_status rc = MJX_OK;
  cudaError_t e = cudaMemcpyAsync(yc, y_n, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(yp, y_prev ? y_prev : y_n, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
  if (e == cudaSuccess && be_guess_previous == 2)  // the caller's guess, in y_out on entry
    e = cudaMemcpyAsync(yn, y_out, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
  StepOut so;
  memset(&so, 0, sizeof(so));
  if (e == cudaSuccess) e = implicit_step(r, P, model_abc, method, dt, dt_prev, be_guess_previous, yc, yp, yn, &so);
  if (e == cudaSuccess) e = cudaMemcpyAsync(y_out, yn, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r.s);
  if (e != cudaSuccess) { set_last_error(e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; }
  if (stats) { stats[0] = so.newton; stats[1] = so.lin; stats[2] = so.converged; }
  if (res_norm) *res_norm = so.res;
  if (r.arnoldi) cudaGraphExecDestroy(r.arnoldi);
  if (r.newton) cudaGraphExecDestroy(r.newton);
  return rc;
}

mjx_status mjx_nk_vardiff_adaptive2d(const void* plan2, int n, double dy, double dx,
                                     const double* model_abc, int method,
                                     const mjx_pid_params* pid, double t0, double t_end, double dt0,
                                     int max_steps, int save_every, int be_guess_previous,
                                     const mjx_nk_params* nkp, const double* y0, double* y_final,
                                     double* hist_t, double* hist_dt, double* hist_y,
                                     int* nk_totals, double* attempt_log, int log_cap,
                                     mjx_adaptive_result* res, void* ws, size_t ws_bytes,
                                     void* stream) {
  if (plan2 == nullptr || model_abc == nullptr || nkp == nullptr || pid == nullptr || y0 == nullptr ||
      y_final == nullptr)
    return MJX_BAD_ARG;
  if (method != MJX_METHOD_BE && method != MJX_METHOD_CN && method != MJX_METHOD_BDF2) return MJX_BAD_ARG;
  if (max_steps < 0 || save_every < 1) return MJX_BAD_ARG;
  NKRun r;
  NKParamsC P;
  MJX_TRY(nk_setup(r, plan2, n, dy, dx, nkp, ws, ws_bytes, stream, &P));
  const long long N2 = (long long)n * n;
  // buffers: y_{n-1}, y_n, candidate, BE comparison solve, error
  double* yp = P64(r, r.L.y0);
  double* yc = P64(r, r.L.y1);
  double* yn = P64(r, r.L.y2);
  double* ybe = P64(r, r.L.y3);
  double* E = P64(r, r.L.y4);
  double* part = P64(r, r.L.part);
  int* bad = (int*)(part + r.L.nblk);  // the part buffer holds (m + 2) * nblk doubles
  const int max_saves = max_steps / save_every + 1;
  const int order = method == MJX_METHOD_BE ? 1 : 2;  // compute_error_order (dt_policy.py:411-423)
  // AdaptiveState initial values (stepping.py:778-813); implicit methods take dt0 as is
  double t = t0, dt = dt0, dt_prev = dt0, prev_err = 1.0;
  int step_count = 0, write_idx = 1, n_acc = 0, n_rej = 0, attempts = 0;
  int status = MJX_STATUS_RUNNING_CODE, all_finite = 1;
  int tot_newton = 0, tot_lin = 0, not_conv = 0;
  const int max_attempts = 20 * max_steps + 1000;  // bound on the host loop
  mjx_status rc = MJX_OK;
  cudaError_t e = cudaMemcpyAsync(yc, y0, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(yp, y0, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
  if (e == cudaSuccess && hist_y) e = cudaMemcpyAsync(hist_y, y0, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
  if (hist_t) { for (int i = 0; i < max_saves; ++i) hist_t[i] = 0.0; hist_t[0] = t0; }
  if (hist_dt) for (int i = 0; i < max_saves; ++i) hist_dt[i] = 0.0;
  if (e != cudaSuccess) { set_last_error(e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; }
  while (rc == MJX_OK && status == MJX_STATUS_RUNNING_CODE && t < t_end && write_idx < max_saves &&
         attempts < max_attempts) {
    ++attempts;
    const double dtc = hmin(dt, t_end - t);
    StepOut so, sb;
    // adaptive_integrate implicit branch (stepping.py:818-858)
    const bool be_only = method == MJX_METHOD_BE || (method == MJX_METHOD_BDF2 && step_count < 1);
    if (be_only) {
      e = implicit_step(r, P, model_abc, MJX_METHOD_BE, dtc, dt_prev, be_guess_previous, yc, yp, yn, &so);
      if (e == cudaSuccess) e = scaled_rhs(r, model_abc, dtc, yn, E);
    } else {
      e = implicit_step(r, P, model_abc, method, dtc, dt_prev, be_guess_previous, yc, yp, yn, &so);
      if (e == cudaSuccess)
        e = implicit_step(r, P, model_abc, MJX_METHOD_BE, dtc, dt_prev, be_guess_previous, yc, yp, ybe, &sb);
      if (e == cudaSuccess) {
        lincomb_kernel<<<r.grid, 256, 0, r.s>>>(yn, 1.0, ybe, -1.0, E, nullptr, N2);
        e = cudaGetLastError();
      }
    }
    double hp[152 * 4];
    int hb[152 * 4];
    if (e == cudaSuccess) {
      errnorm_kernel<<<r.L.nblk, 256, 0, r.s>>>(E, yn, pid->atol, pid->rtol, part, bad, N2);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hp, part, sizeof(double) * r.L.nblk, cudaMemcpyDeviceToHost, r.s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hb, bad, sizeof(int) * r.L.nblk, cudaMemcpyDeviceToHost, r.s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r.s);
    if (e != cudaSuccess) { set_last_error(e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; break; }
    double ssum = 0.0, c = 0.0;
    int nonfinite = 0;
    for (int i = 0; i < r.L.nblk; ++i) {  // Kahan
      const double yv = hp[i] - c, tv = ssum + yv;
      c = (tv - ssum) - yv;
      ssum = tv;
      nonfinite |= hb[i];
    }
    tot_newton += so.newton; tot_lin += so.lin; not_conv += !so.converged;
    const double err = hmax(sqrt(ssum / (double)N2), 1e-10);
    const bool finite = !nonfinite;
    const bool accept = (err <= 1.0) && finite && so.converged;
    // propose_dt (dt_policy.py:324-408) for an implicit method
    double dt_a, pe_new = prev_err;
    if (err <= 1.0) {  // pid_controller_dt (178-227)
      const double kI = pid->kI / order, kP = pid->kP / order;
      const double es = hmax(err, 1e-10), pes = hmax(prev_err, 1e-10);
      const double fac = hclip(pow(1.0 / es, kI) * pow(pes / es, kP) * pid->safety, pid->min_factor, pid->max_factor);
      dt_a = hclip(dtc * fac, pid->dt_min, pid->dt_max);
      pe_new = err;
    } else {  // handle_rejected_step (230-268)
      const double kI = pid->kI / order;
      const double fac = hclip(pid->safety * pow(1.0 / hmax(err, 1.0), kI), pid->min_factor, 1.0);
      dt_a = hclip(dtc * fac, pid->dt_min, pid->dt_max);
    }
    // implicit_robustness_dt (279-321) with its defaults, then the final clamp
    double dt_r = so.converged ? dt_a : dt_a * 0.5;
    if (so.converged && so.newton <= 3) dt_r = hmin(dt_r * 1.2, 1.0);
    dt_r = hclip(dt_r, 1e-12, 1.0);
    const double dt_new = hclip(dt_r, pid->dt_min, pid->dt_max);
    if (attempt_log && attempts <= log_cap) {
      double* L = attempt_log + 6 * (attempts - 1);
      L[0] = t; L[1] = dtc; L[2] = err; L[3] = so.converged; L[4] = so.newton; L[5] = accept;
    }
    if (accept) {  // stepping.py:931-964
      if (n_acc % save_every == 0) {
        if (hist_t) hist_t[write_idx] = t + dtc;
        if (hist_dt) hist_dt[write_idx - 1] = dtc;
        if (hist_y) {
          e = cudaMemcpyAsync(hist_y + (long long)write_idx * N2, yn, sizeof(double) * N2,
                              cudaMemcpyDeviceToDevice, r.s);
          if (e != cudaSuccess) { set_last_error(e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; break; }
        }
        ++write_idx;
      }
      t = t + dtc;
      double* tmp = yp; yp = yc; yc = yn; yn = tmp;  // y_prev <- y, y <- y_new
      dt = dt_new;
      dt_prev = dtc;
      ++step_count;
      prev_err = pe_new;
      ++n_acc;
    } else {  // stepping.py:966-992
      dt = hmax(dt_new * 0.5, pid->dt_min);
      if (dt <= pid->dt_min * 1.1) status = MJX_STATUS_DT_TOO_SMALL_CODE;
      ++n_rej;
    }
    if (!finite) { status = MJX_STATUS_NON_FINITE_CODE; all_finite = 0; }
  }
  if (rc == MJX_OK) {
    // final status (stepping.py:1003-1010)
    if (t >= t_end) status = MJX_STATUS_SUCCESS_CODE;
    else if (write_idx >= max_saves) status = MJX_STATUS_MAX_STEPS_CODE;
    else if (status == MJX_STATUS_RUNNING_CODE) status = MJX_STATUS_MAX_STEPS_CODE;
    e = cudaMemcpyAsync(y_final, yc, sizeof(double) * N2, cudaMemcpyDeviceToDevice, r.s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r.s);
    if (e != cudaSuccess) { set_last_error(e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; }
  }
  if (res) {
    res->t_final = t; res->dt_next = dt; res->prev_err = prev_err; res->last_err = 0.0;
    res->n_accepted = n_acc; res->n_rejected = n_rej; res->n_attempts = attempts;
    res->n_saved = write_idx; res->status = status; res->finite = all_finite;
  }
  if (nk_totals) { nk_totals[0] = tot_newton; nk_totals[1] = tot_lin; nk_totals[2] = not_conv; }
  if (r.arnoldi) cudaGraphExecDestroy(r.arnoldi);
  if (r.newton) cudaGraphExecDestroy(r.newton);
  return rc;
}

// ---- generic restarted GMRES over host callbacks ------------------------------------
// The Arnoldi basis (FP32, m + 1 vectors of n), the work vectors and the GMRES header live
// in the caller's workspace; the matvec / preconditioner callbacks enqueue their own work on
// the stream.  Per cycle: r = b - A x, V_0 = M^-1 r, its norm; per Arnoldi step: V_j
// normalised on the device, w = M^-1 A V_j, the Gram-Schmidt dots, the orthogonalisation and
// the Givens step on the device (the GMRES kernels of the Newton-Krylov solver above); after
// the m steps the small triangular solve and x += V y.  The host reads the header once per
// cycle.  Steps after the device has converged inside a cycle return at entry (the
// callbacks still run on the unused basis slots).
struct GLayout {
  size_t V, t, w, part, gs, total;
  int nblk;
};
static GLayout g_layout(long long n, int m) {
  GLayout L;
  L.nblk = 152 * 4;
  size_t o = 0;
  L.V = o; o += al((size_t)(m + 1) * (size_t)n * 4);
  L.t = o; o += al((size_t)n * 4);
  L.w = o; o += al((size_t)n * 4);
  L.part = o; o += al((size_t)(m + 2) * L.nblk * 8);
  L.gs = o; o += al(sizeof(GmresState));
  L.total = o;
  return L;
}

size_t mjx_gmres_ws_bytes(long long n, int restart) {
  if (n < 1 || restart < 1 || restart > NK_MAXM) return 0;
  return g_layout(n, restart).total;
}

mjx_status mjx_gmres_solve(long long n, mjx_vec_op matvec, mjx_vec_op precond, void* user, const float* b,
                           float* x, double tol, int restart, int max_cycles, int* iterations, double* rel_res,
                           int* converged, void* ws, size_t ws_bytes, void* stream) {
  if (n < 1 || matvec == nullptr || b == nullptr || x == nullptr || restart < 1 || restart > NK_MAXM ||
      max_cycles < 1 || !(tol >= 0))
    return MJX_BAD_ARG;
  const GLayout L = g_layout(n, restart);
  if (ws == nullptr || ws_bytes < L.total) return MJX_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  char* w8 = (char*)ws;
  float* V = (float*)(w8 + L.V);
  float* t = (float*)(w8 + L.t);
  float* w = (float*)(w8 + L.w);
  double* part = (double*)(w8 + L.part);
  GmresState* gs = (GmresState*)(w8 + L.gs);
  const int grid = L.nblk;
  auto fail = [&](cudaError_t e) -> mjx_status { set_last_error(e, __FILE__, __LINE__); return MJX_CUDA_ERROR; };
  auto pre = [&](const float* in, float* out) -> int {
    if (precond != nullptr) return precond(in, out, user, stream);
    return cudaMemcpyAsync(out, in, sizeof(float) * (size_t)n, cudaMemcpyDeviceToDevice, s) == cudaSuccess ? 0 : 1;
  };
  int its = 0, conv = 0;
  double res = 0.0, b0 = 0.0;
  for (int cyc = 0; cyc < max_cycles && !conv; ++cyc) {
    if (matvec(x, t, user, stream) != 0) return MJX_BAD_ARG;  // r = b - A x
    sub_kernel<<<grid, 256, 0, s>>>(b, t, t, n);
    if (pre(t, V) != 0) return MJX_BAD_ARG;                     // V_0 = M^-1 r
    sumsq32_kernel<<<grid, 256, 0, s>>>(V, part, n);
    gmres_init_kernel<<<1, 256, 0, s>>>(part, grid, gs, cyc == 0, tol, restart);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(e);
    for (int j = 0; j < restart; ++j) {
      nk_scale_j_kernel<<<grid, 256, 0, s>>>(V, gs, n);          // V_j /= |V_j|
      if (matvec(V + (size_t)j * n, t, user, stream) != 0) return MJX_BAD_ARG;
      if (pre(t, w) != 0) return MJX_BAD_ARG;                    // w = M^-1 A V_j
      gmres_dots_kernel<<<grid, 256, 0, s>>>(V, w, gs, part, n);
      gmres_hcol_kernel<<<1, 256, 0, s>>>(part, grid, gs);
      gmres_orth_kernel<<<grid, 256, 0, s>>>(V, w, gs, part, n);
      gmres_givens_kernel<<<1, 256, 0, s>>>(part, grid, gs, 0, 0);
      if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
    }
    gmres_solve_kernel<<<1, 1, 0, s>>>(gs);
    gmres_update_kernel<<<grid, 256, 0, s>>>(x, V, gs, n);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
    GmresState h;
    if ((e = cudaMemcpyAsync(&h, gs, sizeof(int) * 4 + sizeof(double) * 4, cudaMemcpyDeviceToHost, s)) !=
        cudaSuccess)
      return fail(e);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(e);
    its += h.k_used;
    conv = h.converged;
    if (cyc == 0) b0 = h.beta0;
    res = h.res_est;
  }
  if (iterations) *iterations = its;
  if (converged) *converged = conv;
  if (rel_res) *rel_res = b0 > 0 ? res / b0 : 0.0;
  return MJX_OK;
}

}  // extern "C"
