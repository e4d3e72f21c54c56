// Classical RK4 of periodic Gray-Scott with the Laplacian by FFT, as the explicit method
// of benchmarks/benchmark_gray_scott.py:93-131 (rk4_rhs / rk4_step / rk4_solve):
//   k = D Lap(y) + R(y),  Lap = real(ifft2(lam fft2(y))),
//   y_{n+1} = y_n + dt/6 (k1 + 2 k2 + 2 k3 + k4),  stage inputs y_n + dt/2 k1, ..., y_n + dt k3.
// A stage is two passes: a column pass (forward, times D lam, inverse: the row spectra of
// D Lap(y_s), csrc/spectral.cu col_kernel) and a row pass that inverts them to D Lap(y_s),
// adds the reaction of y_s, updates the running sum, writes the next stage input (or
// y_{n+1}) and transforms it forward for the next column pass.  Eight launches per step,
// replayed from a CUDA graph of up to 16 steps; no host synchronisation inside the loop.
#include <math.h>
#include <string.h>

#include "spectral.cuh"

namespace mjx {

mjx_status ensure_kernel_attrs();
mjx_status check_grid(const mjx_grid2d* g);
int elem_size(int dtype);

template <typename T>
struct GrkRowArgs {
  int n, log2n, ldc, nrows, nseq, stage;
  long long fs, fr;  // spectrum / real field strides (elements)
  const cx<T>* tw;
  cx<T>* spec;       // row spectra [2][ny][ldc]: in, D Lap(y_s); out, the next input's
  const T* Ys;       // stage input y_s [2][ny][nx]
  const T* Yn;       // step start y_n
  T* acc;            // k1 + 2 k2 + 2 k3
  T* out;            // next stage input (stages 0-2) or y_{n+1} (stage 3)
  double dt, F, k;
};

// R4: radix-4 transforms with n/4 threads per row (short FP64 rows, fft_smem_r4)
template <typename T, bool R4 = false>
__global__ void __launch_bounds__(256) grk_row_kernel(const __grid_constant__ GrkRowArgs<T> a) {
  typedef cx<T> C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const int n = a.n, half = n >> 1;
  const int tps = R4 ? (n >= 4 ? n / 4 : 1) : (n >= 16 ? n / 16 : 1);
  const int tid = threadIdx.x;
  const int s_loc = tid / tps, lt = tid % tps;
  const bool active = s_loc < a.nseq;
  const long long y = (long long)blockIdx.x * a.nseq + s_loc;
  const int zb = s_loc * n;
#define Z(x) buf[sp(zb + (x))]
  if (active) {  // the two fields' row spectra as one complex row u + i v
    const C* A = a.spec + y * a.ldc;
    const C* B = a.spec + a.fs + y * a.ldc;
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
        Z(kk) = mk<C>(Ak[m].x - Bk[m].y, Ak[m].y + Bk[m].x);
        if (kk > 0 && kk < half) Z(n - kk) = mk<C>(Ak[m].x + Bk[m].y, Bk[m].x - Ak[m].y);
      }
    }
  }
  __syncthreads();
  if (R4) fft_smem_r4<T, true, false>(buf, n, a.log2n, a.nseq, n, 1, a.tw, tid);
  else fft_smem<T, true, false>(buf, n, a.log2n, a.nseq, n, 1, a.tw, tid);
  const T dt = (T)a.dt, hh = (T)(0.5 * a.dt), d6 = (T)(a.dt / 6.0);
  const T F = (T)a.F, FK = (T)(a.F + a.k);
  const int stage = a.stage;
  if (active) {
    const long long ro = y * n;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int x = lt + m * tps;
      if (x >= n) continue;
      const C z = Z(x);  // (Du Lap u_s, Dv Lap v_s)
      const long long iu = ro + x, iv = a.fr + ro + x;
      const T us = a.Ys[iu], vs = a.Ys[iv];
      const T uvv = us * vs * vs;
      const T ku = z.x - uvv + F * ((T)1 - us);
      const T kv = z.y + uvv - FK * vs;
      const T un = a.Yn[iu], vn = a.Yn[iv];
      T ou, ov;
      if (stage == 0) {
        a.acc[iu] = ku; a.acc[iv] = kv;
        ou = un + hh * ku; ov = vn + hh * kv;
      } else if (stage < 3) {
        a.acc[iu] += (T)2 * ku; a.acc[iv] += (T)2 * kv;
        const T c = stage == 1 ? hh : dt;
        ou = un + c * ku; ov = vn + c * kv;
      } else {
        ou = un + d6 * (a.acc[iu] + ku); ov = vn + d6 * (a.acc[iv] + kv);
      }
      a.out[iu] = ou; a.out[iv] = ov;
      Z(x) = mk<C>(ou, ov);
    }
  }
  __syncthreads();
  if (R4) fft_smem_r4<T, false, false>(buf, n, a.log2n, a.nseq, n, 1, a.tw, tid);
  else fft_smem<T, false, false>(buf, n, a.log2n, a.nseq, n, 1, a.tw, tid);
  if (active) {
    C* A = a.spec + y * a.ldc;
    C* B = a.spec + a.fs + y * a.ldc;
#pragma unroll
    for (int m = 0; m < 9; ++m) {
      const int kk = lt + m * tps;
      if (kk > half) continue;
      const C Zk = Z(kk), Zm = Z((n - kk) & (n - 1));
      A[kk] = mk<C>((T)0.5 * (Zk.x + Zm.x), (T)0.5 * (Zk.y - Zm.y));
      B[kk] = mk<C>((T)0.5 * (Zk.y + Zm.y), (T)0.5 * (Zm.x - Zk.x));
    }
  }
#undef Z
}

struct GrkLayout {
  size_t spec, S, acc, total;
};
static inline size_t al256r(size_t b) { return (b + 255) & ~size_t(255); }

static GrkLayout grk_layout(int ny, int nx, int elem) {
  GrkLayout L;
  const size_t fr = (size_t)ny * nx * elem, fsb = (size_t)ny * spec_ldc(nx) * 2 * elem;
  size_t o = 0;
  L.spec = o; o += al256r(2 * fsb);
  L.S = o; o += al256r(2 * fr);
  L.acc = o; o += al256r(2 * fr);
  L.total = o;
  return L;
}

template <typename T>
static mjx_status grk_run(const void* plan, const mjx_grid2d* g, const double* D, double F, double k, double dt,
                          int n_steps, const T* y_in, T* y_out, char* ws, const GrkLayout& L, cudaStream_t s) {
  const int ny = g->ny, nx = g->nx, ldc = spec_ldc(nx);
  const long long fr = (long long)ny * nx, fs = (long long)ny * ldc;
  const PlanView pv = plan_view(plan, ny, nx, sizeof(T));
  cx<T>* spec = (cx<T>*)(ws + L.spec);
  T* S = (T*)(ws + L.S);
  T* acc = (T*)(ws + L.acc);
  if (y_out != y_in) MJX_CUDA_TRY(cudaMemcpyAsync(y_out, y_in, sizeof(T) * 2 * fr, cudaMemcpyDeviceToDevice, s));
  if (n_steps <= 0) return cuda_status(cudaStreamSynchronize(s));
  // initial r2c of y_0 (the (u, v) pair)
  RowArgs<T> r;
  memset(&r, 0, sizeof(r));
  r.n = nx; r.log2n = ilog2_exact(nx); r.ldc = ldc; r.nrows = ny; r.npairs = 1;
  r.nseq = row_nseq(nx, ny); r.rstride = nx; r.rin_sel = -1; r.rout_sel = -1;
  r.rin[0] = y_out; r.rout[0] = y_out; r.spec = spec; r.tw = (const cx<T>*)pv.twx; r.inv_scale = (T)1;
  r.pr[0].ra = 0; r.pr[0].rb = fr; r.pr[0].sa = 0; r.pr[0].sb = fs; r.pr[0].flags = ROW_STORE_SPEC;
  // column pass: D lam (h = 1), the 1/(nx ny) of the inverse applied here
  ColArgs<T> c;
  memset(&c, 0, sizeof(c));
  c.ny = ny; c.log2ny = ilog2_exact(ny); c.ncols = nx / 2 + 1; c.ldc = ldc;
  c.C = col_tile(ny, c.ncols, 1, sizeof(T)); c.spec = spec; c.lamx = (const T*)pv.lamx;
  c.lamy = (const T*)pv.lamy; c.tw = (const cx<T>*)pv.twy; c.scale = (T)(1.0 / ((double)nx * ny));
  c.njobs = 2; c.hfixed = 1.0;
  for (int f = 0; f < 2; ++f) {
    ColJob& j = c.job[f];
    j.sin = j.sout[0] = j.sout[1] = f * fs;
    j.nout = 1; j.D = D[f]; j.pow[0] = j.pow[1] = 1; j.mul = MUL_LAP; j.hfac[0] = j.hfac[1] = 1.0;
  }
  // row passes of the four stages; small grids take fewer rows per CTA to cover every SM
  GrkRowArgs<T> ra;
  memset(&ra, 0, sizeof(ra));
  ra.n = nx; ra.log2n = ilog2_exact(nx); ra.ldc = ldc; ra.nrows = ny;
  int nseq = row_nseq(nx, ny);
  while (nseq > 1 && ny / nseq < 152) nseq >>= 1;
  ra.nseq = nseq;
  ra.fs = fs; ra.fr = fr; ra.tw = (const cx<T>*)pv.twx; ra.spec = spec; ra.Yn = y_out; ra.acc = acc;
  ra.dt = dt; ra.F = F; ra.k = k;
  GrkRowArgs<T> st[4];
  for (int q = 0; q < 4; ++q) {
    st[q] = ra;
    st[q].stage = q;
    st[q].Ys = q == 0 ? y_out : S;
    st[q].out = q == 3 ? y_out : S;
  }
  // FP64 rows of at most 256 points on a small grid (fewer than four warps per SM at radix
  // 16): radix-4 transforms (nx/4 threads per row)
  const bool r4 = sizeof(T) == 8 && nx >= 4 && nx <= 256 && nseq * (nx / 4) <= 256 &&
                  (long long)ny * (nx / 16) < 152LL * 128;
  const int tps = r4 ? nx / 4 : (nx >= 16 ? nx / 16 : 1);
  const unsigned rblocks = (unsigned)(ny / nseq), rthreads = (unsigned)(nseq * tps);
  const size_t rsmem = (size_t)sp_size(nseq * nx) * sizeof(cx<T>);
  static ContextOnce attr;
  MJX_TRY(attr.run([]() -> mjx_status {
    int dev = 0, optin = 0;
    MJX_CUDA_TRY(cudaGetDevice(&dev));
    MJX_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    MJX_CUDA_TRY(cudaFuncSetAttribute(grk_row_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    MJX_CUDA_TRY(cudaFuncSetAttribute(grk_row_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    MJX_CUDA_TRY(cudaFuncSetAttribute(grk_row_kernel<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    return MJX_OK;
  }));
  auto one_step = [&](cudaStream_t q) -> cudaError_t {
    for (int i = 0; i < 4; ++i) {
      cudaError_t e = launch_col<T>(c, q);
      if (e != cudaSuccess) return e;
      if (r4) grk_row_kernel<T, true><<<rblocks, rthreads, rsmem, q>>>(st[i]);
      else grk_row_kernel<T><<<rblocks, rthreads, rsmem, q>>>(st[i]);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
  };
  cudaError_t ce = launch_row<T, RX_NONE>(r, s);
  const int B = n_steps < 16 ? n_steps : 16;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cs = nullptr;
  if (ce == cudaSuccess && n_steps / B > 1) {  // a graph of B steps
    ce = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
      cudaError_t le = cudaSuccess;
      for (int i = 0; i < B && le == cudaSuccess; ++i) le = one_step(cs);
      ce = cudaStreamEndCapture(cs, &graph);
      if (le != cudaSuccess) ce = le;
    }
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(&exec, graph, 0);
  }
  int done = 0;
  if (exec != nullptr)
    for (; done + B <= n_steps && ce == cudaSuccess; done += B) ce = cudaGraphLaunch(exec, s);
  for (; done < n_steps && ce == cudaSuccess; ++done) ce = one_step(s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cs) cudaStreamDestroy(cs);
  return cuda_status(ce);
}

}  // namespace mjx

using namespace mjx;

extern "C" {

size_t mjx_gs_rk4_spectral_ws_bytes(int ny, int nx, int dtype) {
  const int e = elem_size(dtype);
  if (!e || ilog2_exact(nx) < 4 || ilog2_exact(ny) < 1) return 0;
  return grk_layout(ny, nx, e).total;
}

mjx_status mjx_gs_rk4_spectral2d(const void* plan, const mjx_grid2d* g, int dtype, const double* D, double F,
                                 double k, double dt, int n_steps, const void* y_in, void* y_out, void* ws,
                                 size_t ws_bytes, void* stream) {
  MJX_TRY(check_grid(g));
  if (g->nx < 16) return MJX_BAD_SHAPE;
  if (plan == nullptr || D == nullptr || y_in == nullptr || y_out == nullptr || n_steps < 0) return MJX_BAD_ARG;
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  const GrkLayout L = grk_layout(g->ny, g->nx, e);
  if (ws == nullptr || ws_bytes < L.total) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4)
    return grk_run<float>(plan, g, D, F, k, dt, n_steps, (const float*)y_in, (float*)y_out, (char*)ws, L, s);
  return grk_run<double>(plan, g, D, F, k, dt, n_steps, (const double*)y_in, (double*)y_out, (char*)ws, L, s);
}

}  // extern "C"
