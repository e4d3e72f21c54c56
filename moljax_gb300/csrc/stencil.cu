// Ghost-cell boundary conditions and second-order finite-difference stencils
// on padded fields ([nfields][ny+2g][nx+2g], y on axis 0), fused with the
// reaction terms for the model right-hand side.
//
// Ghost values follow moljax/core/bc.py:202-307: x ghosts (columns) are filled
// first over every row, then y ghosts (rows) over every column, so a corner is
// BC_y(BC_x(interior)).  Periodic wraps, Dirichlet sets 2b - u_mirror,
// Neumann sets u_mirror -/+ 2 d q (left/bottom minus, right/top plus).
#include <string.h>

#include "common.cuh"

namespace mjx {

enum { MJX_ERRNORM_BLOCKS = 152 * 2 };

mjx_status check_grid(const mjx_grid2d* g);
int elem_size(int dtype);

struct BCSide { int kind; double v[4]; };  // v: left, right, bottom, top
struct BC2 { BCSide f[4]; };               // up to 4 fields

// padded index of the interior cell a ghost index reads from, along one axis
__device__ __forceinline__ int bc_src(int j, int n, int g, int kind) {
  if (j < g) return kind == MJX_BC_PERIODIC ? j + n : 2 * g - 1 - j;
  return kind == MJX_BC_PERIODIC ? j - n : 2 * (n + g) - 1 - j;
}

template <typename T>
__device__ __forceinline__ T bc_val(T src, int kind, bool lo, double b, double d) {
  if (kind == MJX_BC_DIRICHLET) return (T)(2.0 * b) - src;
  if (kind == MJX_BC_NEUMANN) return lo ? src - (T)(2.0 * d * b) : src + (T)(2.0 * d * b);
  return src;
}

// value of padded cell (y, x) after the reference's x-then-y ghost fill, reading interiors of f
template <typename T>
__device__ __forceinline__ T filled(const T* f, int y, int x, int ny, int nx, int g, int ldx,
                                    const BCSide& s, double dy, double dx) {
  const bool gy = (y < g) || (y >= ny + g), gx = (x < g) || (x >= nx + g);
  int yy = gy ? bc_src(y, ny, g, s.kind) : y;
  int xx = gx ? bc_src(x, nx, g, s.kind) : x;
  T v = f[(long long)yy * ldx + xx];
  if (gx) v = bc_val<T>(v, s.kind, x < g, x < g ? s.v[0] : s.v[1], dx);
  if (gy) v = bc_val<T>(v, s.kind, y < g, y < g ? s.v[2] : s.v[3], dy);
  return v;
}

// out (padded) = BC-filled copy of src; src interior-only (PAD) or padded (FILL).
template <typename T, bool FROM_INTERIOR>
__global__ void pad_kernel(const T* __restrict__ src, T* __restrict__ out, int nf, int ny, int nx,
                           int g, BC2 bc, double dy, double dx) {
  const int ldx = nx + 2 * g, ldy = ny + 2 * g;
  const long long per = (long long)ldx * ldy;
  const long long total = per * nf;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(i / per);
    const long long r = i - f * per;
    const int y = (int)(r / ldx), x = (int)(r - (long long)y * ldx);
    const bool ghost = y < g || y >= ny + g || x < g || x >= nx + g;
    T v;
    if (FROM_INTERIOR) {
      const T* fi = src + (long long)f * ny * nx;
      if (!ghost) {
        v = fi[(long long)(y - g) * nx + (x - g)];
      } else {
        // read interior cells through the padded index map
        const BCSide& s = bc.f[f];
        const bool gy = y < g || y >= ny + g, gx = x < g || x >= nx + g;
        const int yy = (gy ? bc_src(y, ny, g, s.kind) : y) - g;
        const int xx = (gx ? bc_src(x, nx, g, s.kind) : x) - g;
        v = fi[(long long)yy * nx + xx];
        if (gx) v = bc_val<T>(v, s.kind, x < g, x < g ? s.v[0] : s.v[1], dx);
        if (gy) v = bc_val<T>(v, s.kind, y < g, y < g ? s.v[2] : s.v[3], dy);
      }
    } else {
      const T* fp = src + f * per;
      v = ghost ? filled<T>(fp, y, x, ny, nx, g, ldx, bc.f[f], dy, dx) : fp[r];
    }
    out[i] = v;
  }
}

template <typename T>
__global__ void unpad_kernel(const T* __restrict__ src, T* __restrict__ out, int nf, int ny, int nx,
                             int g) {
  const long long per = (long long)ny * nx, total = per * nf;
  const int ldx = nx + 2 * g, ldy = ny + 2 * g;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(i / per);
    const long long r = i - f * per;
    const int y = (int)(r / nx), x = (int)(r - (long long)y * nx);
    out[i] = src[(long long)f * ldx * ldy + (long long)(y + g) * ldx + (x + g)];
  }
}

// out interior = coef_f * Lap(f) (+ reaction), ghosts of out = 0
// (moljax/core/operators.py:271-322; model.py:100-118 when FILL applies the BCs
// on the fly and RX adds the Gray-Scott terms of operators.py:644-667).
template <typename T, bool FILL, int RX>
__global__ void lap_kernel(const T* __restrict__ src, T* __restrict__ out, int nf, int ny, int nx,
                           int g, BC2 bc, double dy, double dx, double c0, double c1, double c2,
                           double c3, double F, double k) {
  const int ldx = nx + 2 * g, ldy = ny + 2 * g;
  const long long per = (long long)ldx * ldy;
  const long long total = per * (RX == 1 ? 1 : nf);
  const T idx2 = (T)(1.0 / (dx * dx)), idy2 = (T)(1.0 / (dy * dy));
  const double coef[4] = {c0, c1, c2, c3};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(i / per);
    const long long r = i - f * per;
    const int y = (int)(r / ldx), x = (int)(r - (long long)y * ldx);
    const bool ghost = y < g || y >= ny + g || x < g || x >= nx + g;
    if (RX == 1) {  // Gray-Scott: both fields at once
      if (ghost) { out[r] = (T)0; out[per + r] = (T)0; continue; }
      T lap[2], c[2];
      for (int q = 0; q < 2; ++q) {
        const T* fp = src + q * per;
        auto at = [&](int yy, int xx) -> T {
          if (FILL) {
            const bool gh = yy < g || yy >= ny + g || xx < g || xx >= nx + g;
            return gh ? filled<T>(fp, yy, xx, ny, nx, g, ldx, bc.f[q], dy, dx) : fp[(long long)yy * ldx + xx];
          }
          return fp[(long long)yy * ldx + xx];
        };
        c[q] = fp[r];
        lap[q] = (at(y + 1, x) - (T)2 * c[q] + at(y - 1, x)) * idy2 +
                 (at(y, x + 1) - (T)2 * c[q] + at(y, x - 1)) * idx2;
      }
      const T uvv = c[0] * c[1] * c[1];
      out[r] = (T)coef[0] * lap[0] + (-uvv + (T)F * ((T)1 - c[0]));
      out[per + r] = (T)coef[1] * lap[1] + (uvv - (T)(F + k) * c[1]);
      continue;
    }
    if (ghost) { out[i] = (T)0; continue; }
    const T* fp = src + f * per;
    auto at = [&](int yy, int xx) -> T {
      if (FILL) {
        const bool gh = yy < g || yy >= ny + g || xx < g || xx >= nx + g;
        return gh ? filled<T>(fp, yy, xx, ny, nx, g, ldx, bc.f[f], dy, dx) : fp[(long long)yy * ldx + xx];
      }
      return fp[(long long)yy * ldx + xx];
    };
    const T cc = fp[r];
    T v = (at(y + 1, x) - (T)2 * cc + at(y - 1, x)) * idy2 + (at(y, x + 1) - (T)2 * cc + at(y, x - 1)) * idx2;
    v = (T)coef[f] * v;
    if (RX == 2) v += (T)F * cc * ((T)1 - cc);  // Fisher-KPP, F carries r
    out[i] = v;
  }
}

static BC2 make_bc(int nf, const int* kinds, const double* values) {
  BC2 b;
  memset(&b, 0, sizeof(b));
  for (int f = 0; f < nf; ++f) {
    b.f[f].kind = kinds ? kinds[f] : MJX_BC_PERIODIC;
    for (int s = 0; s < 4; ++s) b.f[f].v[s] = values ? values[4 * f + s] : 0.0;
  }
  return b;
}

static int grid_for(long long total) {
  long long b = (total + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

static mjx_status check_pad(int nf, int ny, int nx, int g, const int* kinds) {
  if (nf < 1 || nf > 4 || ny < 1 || nx < 1 || g < 1 || g > ny || g > nx) return MJX_BAD_SHAPE;
  if (kinds)
    for (int f = 0; f < nf; ++f)
      if (kinds[f] < MJX_BC_PERIODIC || kinds[f] > MJX_BC_NEUMANN) return MJX_BAD_ARG;
  return MJX_OK;
}

// 1D stencils on padded fields [nf][nx+2g] (ghosts read as stored; output ghosts 0):
// op 0: Laplacian (operators.py:113-152), 1: upwind d/dx with velocity v (64-110),
// 2: central d/dx (35-61)
template <typename T>
__global__ void stencil1d_kernel(const T* __restrict__ in, T* __restrict__ out, int nf, int nx, int g,
                                 int op, double v, double dx) {
  const int ld = nx + 2 * g;
  const long long total = (long long)nf * ld;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total;
       p += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(p % ld);
    if (i < g || i >= nx + g) { out[p] = (T)0; continue; }
    const T c = in[p], l = in[p - 1], r = in[p + 1];
    T res;
    if (op == 0) res = (r - (T)2 * c + l) / (T)(dx * dx);
    else if (op == 1) res = v >= 0 ? (c - l) / (T)dx : (r - c) / (T)dx;
    else res = (r - l) / (T)(2.0 * dx);
    out[p] = res;
  }
}

// 2D first derivatives on padded fields, ghosts read as stored, output ghosts 0:
// op 1: upwind along axis with scalar velocity v (d1_upwind_2d, operators.py:200-268),
// op 2: central (d1_central_2d, 155-197).  axis 0: y, 1: x.
template <typename T>
__global__ void stencil2d_kernel(const T* __restrict__ in, T* __restrict__ out, int nf, int ny, int nx,
                                 int g, int op, int axis, double v, double d) {
  const int ldx = nx + 2 * g, ldy = ny + 2 * g;
  const long long per = (long long)ldx * ldy, total = per * nf;
  const long long step = axis == 0 ? ldx : 1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i % per;
    const int y = (int)(r / ldx), x = (int)(r - (long long)y * ldx);
    if (y < g || y >= ny + g || x < g || x >= nx + g) { out[i] = (T)0; continue; }
    const T c = in[i], lo = in[i - step], hi = in[i + step];
    if (op == 1) out[i] = v >= 0 ? (c - lo) / (T)d : (hi - c) / (T)d;
    else if (op == 2) out[i] = (hi - lo) / (T)(2.0 * d);
    else out[i] = (hi - (T)2 * c + lo) / (T)(d * d);
  }
}

// div(D grad u) with face averages D_{i+1/2} = (D_i + D_{i+1})/2 on the interior, ghosts zero
// (apply_variable_diffusion_2d, moljax/core/variable_coeff.py:232-287).  D is padded like u, or
// interior-shaped (d_interior != 0) and then edge-extended as jnp.pad(mode='edge') does.
template <typename T>
__global__ void vardiff2d_kernel(const T* __restrict__ u, const T* __restrict__ D, T* __restrict__ out,
                                 int ny, int nx, int g, int d_interior, double dy, double dx) {
  const int ldx = nx + 2 * g, ldy = ny + 2 * g;
  const long long total = (long long)ldx * ldy;
  const T idx2 = (T)(1.0 / (dx * dx)), idy2 = (T)(1.0 / (dy * dy));
  auto Dat = [&](int y, int x) -> T {
    if (!d_interior) return D[(long long)y * ldx + x];
    int yi = y - g, xi = x - g;
    yi = yi < 0 ? 0 : (yi >= ny ? ny - 1 : yi);
    xi = xi < 0 ? 0 : (xi >= nx ? nx - 1 : xi);
    return D[(long long)yi * nx + xi];
  };
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(i / ldx), x = (int)(i - (long long)y * ldx);
    if (y < g || y >= ny + g || x < g || x >= nx + g) { out[i] = (T)0; continue; }
    const T c = u[i], Dc = Dat(y, x);
    const T dxp = (T)0.5 * (Dc + Dat(y, x + 1)), dxm = (T)0.5 * (Dc + Dat(y, x - 1));
    const T dyp = (T)0.5 * (Dc + Dat(y + 1, x)), dym = (T)0.5 * (Dc + Dat(y - 1, x));
    const T Lx = (dxp * (u[i + 1] - c) - dxm * (c - u[i - 1])) * idx2;
    const T Ly = (dyp * (u[i + ldx] - c) - dym * (c - u[i - ldx])) * idy2;
    out[i] = Lx + Ly;
  }
}

// Reaction step of length h on interior fields [nf][n]: Heun R1 = N(y), R2 = N(y + h R1),
// y + h/2 (R1 + R2) (the reaction stage of imex_strang_step, moljax/core/stepping.py:370-435),
// explicit Euler y + h N(y) (imex_euler_step, 317-367), or the rates N(y) (mode 2);
// Gray-Scott couples fields 0 and 1, Fisher-KPP acts on each field, none has N = 0.
template <typename T>
__global__ void heun2d_kernel(const T* __restrict__ in, T* __restrict__ out, int nf, long long n, int rx,
                              double F, double k, double r, double h, int euler) {
  const T pF = (T)F, pK = (T)k, pR = (T)r, th = (T)h, hh = (T)(0.5 * h);
  const long long total = rx == MJX_REACT_GRAY_SCOTT ? n : n * nf;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    if (rx == MJX_REACT_GRAY_SCOTT) {
      const T u = in[i], v = in[n + i];
      const T a = u * v * v;
      const T r1u = -a + pF * ((T)1 - u), r1v = a - (pF + pK) * v;
      if (euler == 2) { out[i] = r1u; out[n + i] = r1v; continue; }
      const T ut = u + th * r1u, vt = v + th * r1v;
      if (euler) { out[i] = ut; out[n + i] = vt; continue; }
      const T b = ut * vt * vt;
      const T r2u = -b + pF * ((T)1 - ut), r2v = b - (pF + pK) * vt;
      out[i] = u + hh * (r1u + r2u);
      out[n + i] = v + hh * (r1v + r2v);
    } else if (rx == MJX_REACT_FISHER) {
      const T u = in[i];
      const T r1 = pR * u * ((T)1 - u);
      if (euler == 2) { out[i] = r1; continue; }
      const T ut = u + th * r1;
      if (euler) { out[i] = ut; continue; }
      const T r2 = pR * ut * ((T)1 - ut);
      out[i] = u + hh * (r1 + r2);
    } else {
      out[i] = euler == 2 ? (T)0 : in[i];
    }
  }
}

// scaled error partials over n values: sum (e / (atol + rtol |y|))^2 and non-finite flags of y
template <typename T>
__global__ void errnorm_partials(const T* __restrict__ e, const T* __restrict__ y, long long n,
                                 double atol, double rtol, double* part, int* bad) {
  double acc = 0.0;
  int nf = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double yv = (double)y[i];
    const double q = (double)e[i] / (atol + rtol * fabs(yv));
    acc += q * q;
    nf |= !isfinite(yv);
  }
  __shared__ double red[8];
  __shared__ int rb[8];
  for (int o = 16; o > 0; o >>= 1) {
    acc += __shfl_xor_sync(0xffffffffu, acc, o);
    nf |= __shfl_xor_sync(0xffffffffu, nf, o);
  }
  if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = acc; rb[threadIdx.x >> 5] = nf; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    int b = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { s += red[w]; b |= rb[w]; }
    part[blockIdx.x] = s;
    bad[blockIdx.x] = b;
  }
}

}  // namespace mjx

using namespace mjx;

extern "C" {

mjx_status mjx_stencil2d(const void* padded_in, void* padded_out, int nfields, int ny, int nx,
                        int n_ghost, int op, int axis, double v, double d, int dtype, void* stream) {
  MJX_TRY(check_pad(nfields, ny, nx, n_ghost, nullptr));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!padded_in || !padded_out || padded_in == padded_out) return MJX_BAD_ARG;
  if (op < 1 || op > 3 || axis < 0 || axis > 1 || !(d > 0)) return MJX_BAD_ARG;
  const long long total = (long long)nfields * (ny + 2 * n_ghost) * (nx + 2 * n_ghost);
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4) stencil2d_kernel<float><<<grid_for(total), 256, 0, s>>>((const float*)padded_in, (float*)padded_out, nfields, ny, nx, n_ghost, op, axis, v, d);
  else stencil2d_kernel<double><<<grid_for(total), 256, 0, s>>>((const double*)padded_in, (double*)padded_out, nfields, ny, nx, n_ghost, op, axis, v, d);
  return cuda_status(cudaGetLastError());
}

mjx_status mjx_variable_diffusion2d(const void* u_padded, const void* D, int d_interior, void* out_padded,
                                    int ny, int nx, int n_ghost, double dy, double dx, int dtype, void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!u_padded || !D || !out_padded || u_padded == out_padded || ny < 1 || nx < 1 || n_ghost < 1 ||
      !(dx > 0) || !(dy > 0))
    return MJX_BAD_ARG;
  const long long total = (long long)(ny + 2 * n_ghost) * (nx + 2 * n_ghost);
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4)
    vardiff2d_kernel<float><<<grid_for(total), 256, 0, s>>>((const float*)u_padded, (const float*)D,
                                                            (float*)out_padded, ny, nx, n_ghost, d_interior, dy, dx);
  else
    vardiff2d_kernel<double><<<grid_for(total), 256, 0, s>>>((const double*)u_padded, (const double*)D,
                                                             (double*)out_padded, ny, nx, n_ghost, d_interior, dy, dx);
  return cuda_status(cudaGetLastError());
}

mjx_status mjx_reaction_step2d(const void* in, void* out, int nfields, long long n, int reaction, double F,
                               double k, double r, double h, int euler, int dtype, void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!in || !out || nfields < 1 || n < 1) return MJX_BAD_ARG;
  if (reaction != MJX_REACT_NONE && reaction != MJX_REACT_GRAY_SCOTT && reaction != MJX_REACT_FISHER)
    return MJX_BAD_ARG;
  if (reaction == MJX_REACT_GRAY_SCOTT && nfields != 2) return MJX_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const long long total = (long long)nfields * n;
  if (e == 4)
    heun2d_kernel<float><<<grid_for(total), 256, 0, s>>>((const float*)in, (float*)out, nfields, n, reaction, F, k, r, h,
                                                         euler);
  else
    heun2d_kernel<double><<<grid_for(total), 256, 0, s>>>((const double*)in, (double*)out, nfields, n, reaction, F, k, r,
                                                          h, euler);
  return cuda_status(cudaGetLastError());
}

size_t mjx_error_norm_ws_bytes(void) { return (size_t)MJX_ERRNORM_BLOCKS * (sizeof(double) + sizeof(int)); }

mjx_status mjx_scaled_error_norm(const void* err, const void* y, long long n, int dtype, double atol,
                                 double rtol, double* result, void* ws, size_t ws_bytes, void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!err || !y || !result || n < 1) return MJX_BAD_ARG;
  if (!ws || ws_bytes < mjx_error_norm_ws_bytes()) return MJX_WORKSPACE;
  double* part = (double*)ws;
  int* bad = (int*)(part + MJX_ERRNORM_BLOCKS);
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4) errnorm_partials<float><<<MJX_ERRNORM_BLOCKS, 256, 0, s>>>((const float*)err, (const float*)y, n, atol, rtol, part, bad);
  else errnorm_partials<double><<<MJX_ERRNORM_BLOCKS, 256, 0, s>>>((const double*)err, (const double*)y, n, atol, rtol, part, bad);
  MJX_CUDA_TRY(cudaGetLastError());
  double hp[MJX_ERRNORM_BLOCKS];
  int hb[MJX_ERRNORM_BLOCKS];
  MJX_CUDA_TRY(cudaMemcpyAsync(hp, part, sizeof(hp), cudaMemcpyDeviceToHost, s));
  MJX_CUDA_TRY(cudaMemcpyAsync(hb, bad, sizeof(hb), cudaMemcpyDeviceToHost, s));
  MJX_CUDA_TRY(cudaStreamSynchronize(s));
  double sum = 0.0, c = 0.0;
  int nonfinite = 0;
  for (int i = 0; i < MJX_ERRNORM_BLOCKS; ++i) {  // Kahan
    const double yv = hp[i] - c, tv = sum + yv;
    c = (tv - sum) - yv;
    sum = tv;
    nonfinite |= hb[i];
  }
  result[0] = sqrt(sum / (double)n);
  result[1] = nonfinite ? 0.0 : 1.0;
  return MJX_OK;
}

mjx_status mjx_bc_pad2d(const void* interior, void* padded, int nfields, int ny, int nx, int n_ghost,
                        const int* kinds, const double* values, double dy, double dx, int dtype,
                        void* stream) {
  MJX_TRY(check_pad(nfields, ny, nx, n_ghost, kinds));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!interior || !padded) return MJX_BAD_ARG;
  const BC2 bc = make_bc(nfields, kinds, values);
  const long long total = (long long)nfields * (ny + 2 * n_ghost) * (nx + 2 * n_ghost);
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4) pad_kernel<float, true><<<grid_for(total), 256, 0, s>>>((const float*)interior, (float*)padded, nfields, ny, nx, n_ghost, bc, dy, dx);
  else pad_kernel<double, true><<<grid_for(total), 256, 0, s>>>((const double*)interior, (double*)padded, nfields, ny, nx, n_ghost, bc, dy, dx);
  return cuda_status(cudaGetLastError());
}

mjx_status mjx_bc_fill2d(const void* padded_in, void* padded_out, int nfields, int ny, int nx,
                         int n_ghost, const int* kinds, const double* values, double dy, double dx,
                         int dtype, void* stream) {
  MJX_TRY(check_pad(nfields, ny, nx, n_ghost, kinds));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!padded_in || !padded_out || padded_in == padded_out) return MJX_BAD_ARG;
  const BC2 bc = make_bc(nfields, kinds, values);
  const long long total = (long long)nfields * (ny + 2 * n_ghost) * (nx + 2 * n_ghost);
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4) pad_kernel<float, false><<<grid_for(total), 256, 0, s>>>((const float*)padded_in, (float*)padded_out, nfields, ny, nx, n_ghost, bc, dy, dx);
  else pad_kernel<double, false><<<grid_for(total), 256, 0, s>>>((const double*)padded_in, (double*)padded_out, nfields, ny, nx, n_ghost, bc, dy, dx);
  return cuda_status(cudaGetLastError());
}

mjx_status mjx_unpad2d(const void* padded, void* interior, int nfields, int ny, int nx, int n_ghost,
                       int dtype, void* stream) {
  MJX_TRY(check_pad(nfields, ny, nx, n_ghost, nullptr));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!padded || !interior) return MJX_BAD_ARG;
  const long long total = (long long)nfields * ny * nx;
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4) unpad_kernel<float><<<grid_for(total), 256, 0, s>>>((const float*)padded, (float*)interior, nfields, ny, nx, n_ghost);
  else unpad_kernel<double><<<grid_for(total), 256, 0, s>>>((const double*)padded, (double*)interior, nfields, ny, nx, n_ghost);
  return cuda_status(cudaGetLastError());
}

mjx_status mjx_laplacian2d(const void* padded_in, void* padded_out, int nfields, int ny, int nx,
                           int n_ghost, const double* coef, int fill_bc, const int* kinds,
                           const double* values, double dy, double dx, int dtype, void* stream) {
  MJX_TRY(check_pad(nfields, ny, nx, n_ghost, kinds));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!padded_in || !padded_out || padded_in == padded_out) return MJX_BAD_ARG;
  const BC2 bc = make_bc(nfields, kinds, values);
  double c[4] = {1, 1, 1, 1};
  if (coef) for (int f = 0; f < nfields; ++f) c[f] = coef[f];
  const long long total = (long long)nfields * (ny + 2 * n_ghost) * (nx + 2 * n_ghost);
  cudaStream_t s = (cudaStream_t)stream;
#define MJX_LAP(T, FILL) lap_kernel<T, FILL, 0><<<grid_for(total), 256, 0, s>>>((const T*)padded_in, (T*)padded_out, nfields, ny, nx, n_ghost, bc, dy, dx, c[0], c[1], c[2], c[3], 0.0, 0.0)
  if (e == 4) { if (fill_bc) MJX_LAP(float, true); else MJX_LAP(float, false); }
  else { if (fill_bc) MJX_LAP(double, true); else MJX_LAP(double, false); }
#undef MJX_LAP
  return cuda_status(cudaGetLastError());
}

mjx_status mjx_stencil1d(const void* padded_in, void* padded_out, int nfields, int nx, int n_ghost,
                        int op, double v, double dx, int dtype, void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!padded_in || !padded_out || padded_in == padded_out) return MJX_BAD_ARG;
  if (nfields < 1 || nx < 1 || n_ghost < 1 || op < 0 || op > 2 || !(dx > 0)) return MJX_BAD_ARG;
  const long long total = (long long)nfields * (nx + 2 * n_ghost);
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4) stencil1d_kernel<float><<<grid_for(total), 256, 0, s>>>((const float*)padded_in, (float*)padded_out, nfields, nx, n_ghost, op, v, dx);
  else stencil1d_kernel<double><<<grid_for(total), 256, 0, s>>>((const double*)padded_in, (double*)padded_out, nfields, nx, n_ghost, op, v, dx);
  return cuda_status(cudaGetLastError());
}

mjx_status mjx_rhs2d(const void* padded_in, void* padded_out, int nfields, int ny, int nx,
                     int n_ghost, int reaction, const double* D, double F, double k,
                     const int* kinds, const double* values, double dy, double dx, int dtype,
                     void* stream) {
  MJX_TRY(check_pad(nfields, ny, nx, n_ghost, kinds));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!padded_in || !padded_out || padded_in == padded_out || !D) return MJX_BAD_ARG;
  if (reaction == MJX_REACT_GRAY_SCOTT && nfields != 2) return MJX_BAD_ARG;
  if (reaction < MJX_REACT_NONE || reaction > MJX_REACT_FISHER) return MJX_BAD_ARG;
  const BC2 bc = make_bc(nfields, kinds, values);
  double c[4] = {0, 0, 0, 0};
  for (int f = 0; f < nfields; ++f) c[f] = D[f];
  const long long per = (long long)(ny + 2 * n_ghost) * (nx + 2 * n_ghost);
  cudaStream_t s = (cudaStream_t)stream;
  const long long total = reaction == MJX_REACT_GRAY_SCOTT ? per : per * nfields;
#define MJX_RHS(T, RX) lap_kernel<T, true, RX><<<grid_for(total), 256, 0, s>>>((const T*)padded_in, (T*)padded_out, nfields, ny, nx, n_ghost, bc, dy, dx, c[0], c[1], c[2], c[3], F, k)
  if (e == 4) {
    if (reaction == MJX_REACT_GRAY_SCOTT) MJX_RHS(float, 1); else if (reaction == MJX_REACT_FISHER) MJX_RHS(float, 2); else MJX_RHS(float, 0);
  } else {
    if (reaction == MJX_REACT_GRAY_SCOTT) MJX_RHS(double, 1); else if (reaction == MJX_REACT_FISHER) MJX_RHS(double, 2); else MJX_RHS(double, 0);
  }
#undef MJX_RHS
  return cuda_status(cudaGetLastError());
}

}  // extern "C"
