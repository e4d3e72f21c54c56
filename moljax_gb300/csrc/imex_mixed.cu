// Adaptive IMEX-Strang with an extended-precision spectral state and FP32
// transforms.
//
// The state is kept as its half spectrum Y^ in float-float form: every real
// component is the unevaluated sum hi + lo of two FP32 numbers (about 48
// significant bits; GB300 runs FP32 at 64x its FP64 rate, so all state
// arithmetic stays on the FP32 pipe).  Diffusion half steps are pointwise in
// spectral space, Y^ += Y^ * mu with mu = m - 1 = x/(1 - x), x = h D lam
// (computed in FP32: mu is small wherever Y^ carries energy, so its FP32
// rounding stays far below the state's).  Only the reaction increments
// Delta = R_heun(y*) - y* go through FP32 transforms:
//   y*  = IFFT32(M(h/2) Y^)          (c2r in FP32)
//   Y^' = M(h/2) (M(h/2) Y^ + FFT32(Delta(y*)))
// so the FP32 rounding enters in proportion to |Delta|, not |y|.  The error
// estimate y_half - y_full = IFFT32(Y^_half - Y^_full) is a transform of a small
// difference taken in float-float.  Same step doubling / PI controller /
// accept-reject loop as the FP32 path (csrc/imex.cu), six kernels per attempt:
//
//   C1 col  Y^[cur] -> PA = M(dt/2)Y^, PB = M(dt/4)Y^;  ZA = IFFT_y(PA), ZB = IFFT_y(PB)
//   R1 row  ZA: c2r, Delta(dt), r2c;  ZB: c2r, Delta(dt/2), r2c
//   C2 col  PA = M(dt/2)(PA + FFT_y ZA);  PB = M(dt/4)M(dt/4)(PB + FFT_y ZB);  ZB = IFFT_y(PB)
//   R2 row  ZB: c2r, Delta(dt/2), r2c
//   C3 col  Y^[1-cur] = M(dt/4)(PB + FFT_y ZB);  ZA = IFFT_y(Y^[1-cur] - PA), ZB = IFFT_y(Y^[1-cur])
//   R3 row  c2r of (ZA, ZB) pairs -> scaled error partials
#include <math.h>
#include <string.h>

#include "mixed.cuh"

namespace mjx {

mjx_status ensure_kernel_attrs();
mjx_status check_grid(const mjx_grid2d* g);
int elem_size(int dtype);
void set_last_error(cudaError_t e, const char* file, int line);

struct MJob {
  int type;
  int pad;
  long long off;  // field offset (complex elements) shared by every buffer
  double D;
};

// Float-float complex element in HBM: {re_hi, im_hi, re_lo, im_lo}.
struct MColArgs {
  int ny, log2ny, ncols, ldc, C, njobs;
  float4* ys[2];
  float4* pa;
  float4* pb;
  float2* za;
  float2* zb;
  const float* lamx;
  const float* lamy;
  const float2* tw;
  float inv_norm;
  double hfixed;
  const DevState* st;
  MJob job[8];
};

// LOG2NY, CN: compile-time column length and tile width (mcol_tile), launched with NT threads
template <int NT, int MINB, int LOG2NY = 0, int CN = 0>
__global__ void __launch_bounds__(NT, MINB) mcol_kernel(const __grid_constant__ MColArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* buf = reinterpret_cast<float2*>(smem_raw);
  const DevState* st = a.st;
  if (st != nullptr && st->done) return;
  const MJob jb = a.job[blockIdx.y];
  const int cur = st != nullptr ? st->cur : 0;
  const double h = st != nullptr ? st->dtc : a.hfixed;
  MColTile t;
  t.ny = a.ny; t.log2ny = a.log2ny; t.ncols = a.ncols; t.C = a.C; t.type = jb.type;
  t.kx0 = blockIdx.x * a.C;
  t.ldc = a.ldc; t.off = jb.off;
  t.ys_cur = a.ys[cur]; t.ys_next = a.ys[1 - cur];
  t.pa = a.pa; t.pb = a.pb; t.za = a.za; t.zb = a.zb;
  t.lamx = a.lamx; t.lamy = a.lamy; t.tw = a.tw;
  t.hA = (float)(0.5 * h * jb.D); t.hB = (float)(0.25 * h * jb.D); t.nrm = a.inv_norm;
  mcol_tile<LOG2NY, CN, LOG2NY ? NT : 0>(buf, t, threadIdx.x, blockDim.x);
}

__global__ void f32_to_f64(const float* in, double* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}
__global__ void f64_to_f32(const double* in, float* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}
// FP64 complex -> float-float complex, in place (each element is 16 bytes either way)
__global__ void c64_to_ff(double2* data, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double2 z = data[i];
    const float rh = __double2float_rn(z.x), ih = __double2float_rn(z.y);
    const float rl = __double2float_rn(z.x - (double)rh), il = __double2float_rn(z.y - (double)ih);
    reinterpret_cast<float4*>(data)[i] = make_float4(rh, ih, rl, il);
  }
}
// current float-float state -> FP64 complex
__global__ void select_state_kernel(const DevState* st, const float4* y0, const float4* y1, double2* out, long long n) {
  const float4* src = (st == nullptr || st->cur == 0) ? y0 : y1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float4 v = src[i];
    double2 z; z.x = (double)v.x + (double)v.z; z.y = (double)v.y + (double)v.w;
    out[i] = z;
  }
}


struct MixLayout {
  size_t ys0, ys1, pa, pb, za, zb, part, bad, st, total;
  int nparts;
  long long fs;  // complex elements per field spectrum
};

static inline size_t al256m(size_t b) { return (b + 255) & ~size_t(255); }

static MixLayout mix_layout(int ny, int nx, int nf, int nparts) {
  MixLayout L;
  L.fs = (long long)ny * spec_ldc(nx);
  const size_t s64 = (size_t)nf * L.fs * 16, s32 = (size_t)nf * L.fs * 8;
  size_t o = 0;
  L.ys0 = o; o += al256m(s64);
  L.ys1 = o; o += al256m(s64);
  L.pa = o; o += al256m(s64);
  L.pb = o; o += al256m(s64);
  L.za = o; o += al256m(s32);
  L.zb = o; o += al256m(s32);
  L.nparts = nparts;
  L.part = o; o += al256m(sizeof(double) * (size_t)nparts);
  L.bad = o; o += al256m(sizeof(int) * (size_t)nparts);
  L.st = o; o += al256m(sizeof(DevState));
  L.total = o;
  return L;
}

static int mix_nparts(int ny, int nx, int nf) { return row_ctas(nx, ny, nf); }

// thread caps of the C1 / C2 / C3 column tiles: 512 -> four columns per CTA at 1024 rows
// (whole 32-byte sectors of the FP32 tile; two 64-register CTAs per SM), 256 -> two columns
// (four CTAs per SM).  Measured at 1024^2: 881 ms per solve with 512 for all three passes,
// 901 ms with 256; mixed choices in between.
static constexpr int kColCap[3] = {512, 512, 512};

struct MixAttempt {
  MColArgs c1, c2, c3;
  RowArgs<float> r1, r2, r3;
  int rx;
};

static MixAttempt build_mix(const void* plan32, const mjx_grid2d* g, const mjx_imex_problem* pb,
                            const mjx_pid_params* pid, char* ws, const MixLayout& L, DevState* st) {
  MixAttempt A;
  const int nf = pb->nfields, ldc = spec_ldc(g->nx);
  const PlanView pv = plan_view(plan32, g->ny, g->nx, 4);
  A.rx = pb->reaction == MJX_REACT_GRAY_SCOTT ? RX_GRAY_SCOTT : (pb->reaction == MJX_REACT_FISHER ? RX_FISHER : RX_NONE);
  MColArgs c;
  memset(&c, 0, sizeof(c));
  c.ny = g->ny; c.log2ny = ilog2_exact(g->ny); c.ncols = g->nx / 2 + 1; c.ldc = ldc;
  const int tps = g->ny >= 16 ? g->ny / 16 : 1;
  // column tile width: the widest C with 2 C ny/16 <= cap threads and <= 200 KB of smem
  auto tile = [&](int cap) {
    int C = 8;
    while (C > 1 && (2 * C * tps > cap || (size_t)sp_size(g->ny * 2 * C) * 8 > 200 * 1024)) C >>= 1;
    return C;
  };
  c.C = tile(kColCap[1]);
  c.ys[0] = (float4*)(ws + L.ys0); c.ys[1] = (float4*)(ws + L.ys1);
  c.pa = (float4*)(ws + L.pa); c.pb = (float4*)(ws + L.pb);
  c.za = (float2*)(ws + L.za); c.zb = (float2*)(ws + L.zb);
  c.lamx = (const float*)pv.lamx; c.lamy = (const float*)pv.lamy; c.tw = (const float2*)pv.twy;
  c.inv_norm = (float)(1.0 / ((double)g->nx * (double)g->ny));
  c.st = st;
  A.c1 = c; A.c2 = c; A.c3 = c;
  A.c1.C = tile(kColCap[0]);
  A.c3.C = tile(kColCap[2]);
  for (int f = 0; f < nf; ++f) {
    const double D = pb->D[f] > 1e-14 ? pb->D[f] : 0.0;
    MJob j;
    memset(&j, 0, sizeof(j));
    j.off = (long long)f * L.fs; j.D = D;
    j.type = MC_SPLIT; A.c1.job[A.c1.njobs++] = j;
    j.type = MC_MID_BOTH; A.c2.job[A.c2.njobs++] = j;  // MC_FULL_END + MC_HALF_MID, one tile
    j.type = MC_HALF_END; A.c3.job[A.c3.njobs++] = j;
  }
  // row passes over the FP32 row spectra ZA/ZB (contiguous: ZB = ZA + zoff)
  const long long zoff = (long long)((L.zb - L.za) / sizeof(float2));
  RowArgs<float> r;
  memset(&r, 0, sizeof(r));
  r.n = g->nx; r.log2n = ilog2_exact(g->nx); r.ldc = ldc; r.rstride = g->nx;
  r.rin_sel = -1; r.rout_sel = -1;
  r.spec = (cx<float>*)(ws + L.za); r.tw = (const cx<float>*)pv.twx; r.inv_scale = 1.0f;
  r.F = pb->F; r.k = pb->k; r.r = pb->r; r.atol = pid->atol; r.rtol = pid->rtol;
  r.partial = (double*)(ws + L.part); r.nonfinite = (int*)(ws + L.bad); r.st = st;
  const long long fs = L.fs;
  auto reaction_pairs = [&](RowArgs<float>& rr, int b0, int nb, const double* hf) {
    const int fl = ROW_LOAD_SPEC | ROW_REACT | ROW_DELTA | ROW_STORE_SPEC;
    int q = 0;
    for (int b = b0; b < b0 + nb; ++b) {
      const long long base = b == 0 ? 0 : zoff;
      if (A.rx == RX_GRAY_SCOTT) {  // (u_y, v_y)
        RowPair& p = rr.pr[q++];
        p.sa = base; p.sb = base + fs; p.hfac = hf[b - b0]; p.flags = fl;
      } else {                      // (f_y, f_{y+ny/2})
        for (int f = 0; f < nf; ++f) {
          RowPair& p = rr.pr[q++];
          p.sa = base + f * fs; p.sb = p.sa + (long long)(g->ny / 2) * ldc; p.hfac = hf[b - b0]; p.flags = fl;
        }
      }
    }
    rr.npairs = q;
    rr.nrows = A.rx == RX_GRAY_SCOTT ? g->ny : g->ny / 2;
    rr.nseq = row_nseq(g->nx, rr.nrows);
  };
  const double h2[2] = {1.0, 0.5};
  A.r1 = r; reaction_pairs(A.r1, 0, 2, h2);
  const double hh[1] = {0.5};
  A.r2 = r; reaction_pairs(A.r2, 1, 1, hh);
  A.r3 = r;  // pairs (error row, solution row) of each field
  for (int f = 0; f < nf; ++f) {
    RowPair& p = A.r3.pr[f];
    p.sa = f * fs; p.sb = zoff + f * fs; p.hfac = 0.0; p.flags = ROW_LOAD_SPEC | ROW_ERRPAIR;
  }
  A.r3.npairs = nf; A.r3.nrows = g->ny; A.r3.nseq = row_nseq(g->nx, g->ny);
  return A;
}

static cudaError_t mcol(const MColArgs& c, cudaStream_t s) {
  const int tps = c.ny >= 16 ? c.ny / 16 : 1;
  const size_t smem = (size_t)sp_size(c.ny * 2 * c.C) * sizeof(float2);
  dim3 grid((c.ncols + c.C - 1) / c.C, c.njobs);
  const int nt = 2 * c.C * tps;
  if (c.ny == 1024 && c.C == 4 && nt == 512) mcol_kernel<512, 2, 10, 4><<<grid, nt, smem, s>>>(c);
  else if (nt <= 256) mcol_kernel<256, 4><<<grid, nt, smem, s>>>(c);
  else mcol_kernel<512, 2><<<grid, nt, smem, s>>>(c);
  return cudaGetLastError();
}

static cudaError_t mrow(const RowArgs<float>& r, int rx, cudaStream_t s) {
  return rx == RX_GRAY_SCOTT ? launch_row<float, RX_GRAY_SCOTT>(r, s)
         : (rx == RX_FISHER ? launch_row<float, RX_FISHER>(r, s) : launch_row<float, RX_NONE>(r, s));
}

// attempts per iteration of the conditional while node
static constexpr int kCondUnroll = 4;

static cudaError_t launch_mix_attempt(const MixAttempt& A, cudaStream_t s) {
  cudaError_t e;
  if ((e = mcol(A.c1, s)) != cudaSuccess) return e;
  if ((e = mrow(A.r1, A.rx, s)) != cudaSuccess) return e;
  if ((e = mcol(A.c2, s)) != cudaSuccess) return e;
  if ((e = mrow(A.r2, A.rx, s)) != cudaSuccess) return e;
  if ((e = mcol(A.c3, s)) != cudaSuccess) return e;
  return mrow(A.r3, RX_NONE, s);
}

// FP64 transform helpers for the initial and final conversions (split pairing, FP64 plan)
static mjx_status to_spectrum64(const void* plan64, const mjx_grid2d* g, int nf, const double* real,
                                double2* spec, cudaStream_t s) {
  const PlanView pv = plan_view(plan64, g->ny, g->nx, 8);
  const int ldc = spec_ldc(g->nx);
  RowArgs<double> r;
  memset(&r, 0, sizeof(r));
  r.n = g->nx; r.log2n = ilog2_exact(g->nx); r.ldc = ldc; r.nrows = g->ny / 2; r.npairs = nf;
  r.nseq = row_nseq(g->nx, r.nrows); r.rstride = g->nx; r.rin_sel = -1; r.rout_sel = -1;
  r.rin[0] = real; r.spec = (cx<double>*)spec; r.tw = (const cx<double>*)pv.twx; r.inv_scale = 1.0;
  for (int f = 0; f < nf; ++f) {
    r.pr[f].ra = (long long)f * g->ny * g->nx; r.pr[f].rb = r.pr[f].ra + (long long)(g->ny / 2) * g->nx;
    r.pr[f].sa = (long long)f * g->ny * ldc; r.pr[f].sb = r.pr[f].sa + (long long)(g->ny / 2) * ldc;
    r.pr[f].flags = ROW_STORE_SPEC;
  }
  MJX_CUDA_TRY((launch_row<double, RX_NONE>(r, s)));
  ColArgs<double> c;
  memset(&c, 0, sizeof(c));
  c.ny = g->ny; c.log2ny = ilog2_exact(g->ny); c.ncols = g->nx / 2 + 1; c.ldc = ldc;
  c.C = col_tile(g->ny, c.ncols, 1, 8); c.spec = (cx<double>*)spec; c.lamx = (const double*)pv.lamx;
  c.lamy = (const double*)pv.lamy; c.tw = (const cx<double>*)pv.twy; c.scale = 1.0; c.njobs = nf;
  for (int f = 0; f < nf; ++f) {
    ColJob& j = c.job[f];
    j.sin = j.sout[0] = j.sout[1] = (long long)f * g->ny * ldc;
    j.nout = 1; j.mul = MUL_SCALE; j.dirs = 1; j.scale = 1.0; j.pow[0] = j.pow[1] = 1;
  }
  MJX_CUDA_TRY(launch_col<double>(c, s));
  return MJX_OK;
}

static mjx_status from_spectrum64(const void* plan64, const mjx_grid2d* g, int nf, double2* spec,
                                  double* real, cudaStream_t s) {
  const PlanView pv = plan_view(plan64, g->ny, g->nx, 8);
  const int ldc = spec_ldc(g->nx);
  ColArgs<double> c;
  memset(&c, 0, sizeof(c));
  c.ny = g->ny; c.log2ny = ilog2_exact(g->ny); c.ncols = g->nx / 2 + 1; c.ldc = ldc;
  c.C = col_tile(g->ny, c.ncols, 1, 8); c.spec = (cx<double>*)spec; c.lamx = (const double*)pv.lamx;
  c.lamy = (const double*)pv.lamy; c.tw = (const cx<double>*)pv.twy; c.njobs = nf;
  for (int f = 0; f < nf; ++f) {
    ColJob& j = c.job[f];
    j.sin = j.sout[0] = j.sout[1] = (long long)f * g->ny * ldc;
    j.nout = 1; j.mul = MUL_SCALE; j.dirs = 2; j.scale = 1.0 / ((double)g->nx * (double)g->ny);
    j.pow[0] = j.pow[1] = 1;
  }
  MJX_CUDA_TRY(launch_col<double>(c, s));
  RowArgs<double> r;
  memset(&r, 0, sizeof(r));
  r.n = g->nx; r.log2n = ilog2_exact(g->nx); r.ldc = ldc; r.nrows = g->ny / 2; r.npairs = nf;
  r.nseq = row_nseq(g->nx, r.nrows); r.rstride = g->nx; r.rin_sel = -1; r.rout_sel = -1;
  r.rout[0] = real; r.spec = (cx<double>*)spec; r.tw = (const cx<double>*)pv.twx; r.inv_scale = 1.0;
  for (int f = 0; f < nf; ++f) {
    r.pr[f].ra = (long long)f * g->ny * g->nx; r.pr[f].rb = r.pr[f].ra + (long long)(g->ny / 2) * g->nx;
    r.pr[f].sa = (long long)f * g->ny * ldc; r.pr[f].sb = r.pr[f].sa + (long long)(g->ny / 2) * ldc;
    r.pr[f].flags = ROW_LOAD_SPEC | ROW_STORE_REAL;
  }
  MJX_CUDA_TRY((launch_row<double, RX_NONE>(r, s)));
  return MJX_OK;
}

mjx_status mix_state_from_real(const void* plan64, const mjx_grid2d* g, int nf, int io_dtype, const void* y,
                               double* real64, float4* ys, cudaStream_t s) {
  const long long nelem = (long long)nf * g->ny * g->nx;
  if (io_dtype == MJX_F32) {
    f32_to_f64<<<304, 256, 0, s>>>((const float*)y, real64, nelem);
    MJX_CUDA_TRY(cudaGetLastError());
  } else {
    MJX_CUDA_TRY(cudaMemcpyAsync(real64, y, nelem * 8, cudaMemcpyDeviceToDevice, s));
  }
  MJX_TRY(to_spectrum64(plan64, g, nf, real64, (double2*)ys, s));
  c64_to_ff<<<304, 256, 0, s>>>((double2*)ys, (long long)nf * g->ny * spec_ldc(g->nx));
  MJX_CUDA_TRY(cudaGetLastError());
  return MJX_OK;
}

mjx_status mix_real_from_state(const void* plan64, const mjx_grid2d* g, int nf, const DevState* st,
                               const float4* ys0, const float4* ys1, double2* spec64, double* real64,
                               int io_dtype, void* y_out, cudaStream_t s) {
  const long long nelem = (long long)nf * g->ny * g->nx;
  select_state_kernel<<<304, 256, 0, s>>>(st, ys0, ys1, spec64, (long long)nf * g->ny * spec_ldc(g->nx));
  MJX_CUDA_TRY(cudaGetLastError());
  MJX_TRY(from_spectrum64(plan64, g, nf, spec64, real64, s));
  if (io_dtype == MJX_F32) {
    f64_to_f32<<<304, 256, 0, s>>>(real64, (float*)y_out, nelem);
    MJX_CUDA_TRY(cudaGetLastError());
  } else if ((void*)real64 != y_out) {
    MJX_CUDA_TRY(cudaMemcpyAsync(y_out, real64, nelem * 8, cudaMemcpyDeviceToDevice, s));
  }
  return MJX_OK;
}

mjx_status ensure_mix_attrs() {
  static ContextOnce once;
  return once.run([]() -> mjx_status {
    int dev = 0, optin = 0;
    MJX_CUDA_TRY(cudaGetDevice(&dev));
    MJX_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    MJX_CUDA_TRY(cudaFuncSetAttribute(mcol_kernel<256, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    MJX_CUDA_TRY(cudaFuncSetAttribute(mcol_kernel<512, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    MJX_CUDA_TRY(cudaFuncSetAttribute(mcol_kernel<512, 2, 10, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    return MJX_OK;
  });
}

}  // namespace mjx

using namespace mjx;

extern "C" {

mjx_status mjx_imex_mixed_attempt_kernel2d(const void* plan32, const void* plan64,
                                           const mjx_grid2d* g, const mjx_imex_problem* pb,
                                           const mjx_pid_params* pid, int which, double dt,
                                           const void* y, void* ws, size_t ws_bytes, void* stream) {
  MJX_TRY(check_grid(g));
  if (pb == nullptr || pid == nullptr || plan32 == nullptr || plan64 == nullptr) return MJX_BAD_ARG;
  if (pb->nfields < 1 || pb->nfields > 4) return MJX_BAD_ARG;
  const int nf = pb->nfields;
  const MixLayout L = mix_layout(g->ny, g->nx, nf, mix_nparts(g->ny, g->nx, nf));
  if (ws == nullptr || ws_bytes < L.total) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  MJX_TRY(ensure_mix_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  char* w = (char*)ws;
  DevState* st = (DevState*)(w + L.st);
  if (which == 0) {  // seed: FP32 y -> FP64 spectral state, step dt
    if (y == nullptr) return MJX_BAD_ARG;
    const long long nelem = (long long)nf * g->ny * g->nx;
    double* real64 = (double*)(w + L.pa);
    f32_to_f64<<<304, 256, 0, s>>>((const float*)y, real64, nelem);
    MJX_CUDA_TRY(cudaGetLastError());
    MJX_TRY(to_spectrum64(plan64, g, nf, real64, (double2*)(w + L.ys0), s));
    c64_to_ff<<<304, 256, 0, s>>>((double2*)(w + L.ys0), (long long)nf * L.fs);
    MJX_CUDA_TRY(cudaGetLastError());
    MJX_CUDA_TRY(cudaMemcpyAsync(w + L.ys1, w + L.ys0, (size_t)nf * L.fs * 16, cudaMemcpyDeviceToDevice, s));
    DevState h;
    memset(&h, 0, sizeof(h));
    h.dt = dt; h.dtc = dt; h.t_end = 1e300; h.prev_err = 1.0; h.status = MJX_STATUS_RUNNING_CODE;
    h.order = 2; h.save_slot = -1; h.max_saves = 1 << 30; h.save_every = 1 << 30; h.max_attempts = 1 << 30;
    MJX_CUDA_TRY(cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
    MJX_CUDA_TRY(cudaStreamSynchronize(s));
    return MJX_OK;
  }
  const MixAttempt A = build_mix(plan32, g, pb, pid, w, L, st);
  cudaError_t e;
  switch (which) {
    case 1: e = mcol(A.c1, s); break;
    case 2: e = mrow(A.r1, A.rx, s); break;
    case 3: e = mcol(A.c2, s); break;
    case 4: e = mrow(A.r2, A.rx, s); break;
    case 5: e = mcol(A.c3, s); break;
    case 6: e = mrow(A.r3, RX_NONE, s); break;
    case 7: {  // the controller
      CtlArgs ca;
      memset(&ca, 0, sizeof(ca));
      ca.st = st; ca.partial = (const double*)(w + L.part); ca.nonfinite = (const int*)(w + L.bad);
      ca.nparts = L.nparts; ca.n_dof = (double)nf * g->ny * g->nx; ca.pid = *pid;
      e = launch_controller(ca, s);
      break;
    }
    default: return MJX_BAD_ARG;
  }
  return cuda_status(e);
}

size_t mjx_imex2d_mixed_ws_bytes(int ny, int nx, int nfields) {
  if (ilog2_exact(nx) < 1 || ilog2_exact(ny) < 1 || nfields < 1 || nfields > 4) return 0;
  return mix_layout(ny, nx, nfields, mix_nparts(ny, nx, nfields)).total;
}

}  // extern "C"

namespace mjx {

// The captured adaptive loop of one mixed-precision problem: the workspace layout, the
// attempt kernels' arguments and the instantiated conditional graph, built once and
// replayed by every run.  The t/dt history lives in the plan's workspace (after the
// mixed layout) so the captured controller writes a fixed address.
struct ImexMixedPlan {
  const void* plan32;
  const void* plan64;
  mjx_grid2d g;
  mjx_imex_problem pb;
  mjx_pid_params pid;
  int max_steps, save_every, max_saves;
  char* ws;
  MixLayout L;
  double* ht = nullptr;     // t/dt history written by the captured controller (may be null)
  double* hdt = nullptr;
  bool own_hist = false;    // the history lives in the plan's workspace (copied out per run)
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

static size_t plan_hist_offset(const MixLayout& L) { return L.total; }

static void free_mixed_plan(ImexMixedPlan* P) {
  if (P->exec) cudaGraphExecDestroy(P->exec);
  if (P->graph) cudaGraphDestroy(P->graph);
  if (P->cap) cudaStreamDestroy(P->cap);
  delete P;
}

static mjx_status check_mixed_problem(const mjx_grid2d* g, const mjx_imex_problem* pb, const mjx_pid_params* pid,
                                      const void* plan32, const void* plan64, int max_steps, int save_every) {
  MJX_TRY(check_grid(g));
  if (pb == nullptr || pid == nullptr || plan32 == nullptr || plan64 == nullptr) return MJX_BAD_ARG;
  if (pb->nfields < 1 || pb->nfields > 4 || !pb->use_strang) return MJX_BAD_ARG;
  if (pb->reaction == MJX_REACT_GRAY_SCOTT && pb->nfields != 2) return MJX_BAD_ARG;
  if (max_steps < 0 || save_every < 1) return MJX_BAD_ARG;
  return MJX_OK;
}

// Captures kCondUnroll attempts (each followed by the controller) into the body of a
// conditional while node and instantiates the graph.
static mjx_status capture_mixed(ImexMixedPlan& P) {
  DevState* st = (DevState*)(P.ws + P.L.st);
  const MixAttempt A = build_mix(P.plan32, &P.g, &P.pb, &P.pid, P.ws, P.L, st);
  CtlArgs ca;
  memset(&ca, 0, sizeof(ca));
  ca.st = st; ca.partial = (const double*)(P.ws + P.L.part); ca.nonfinite = (const int*)(P.ws + P.L.bad);
  ca.nparts = P.L.nparts; ca.n_dof = (double)P.pb.nfields * P.g.ny * P.g.nx; ca.pid = P.pid;
  ca.hist_t = P.ht; ca.hist_dt = P.hdt;
  cudaError_t ce = cudaSuccess;
  do {
    if ((ce = cudaStreamCreateWithFlags(&P.cap, cudaStreamNonBlocking)) != cudaSuccess) break;
    if ((ce = cudaGraphCreate(&P.graph, 0)) != cudaSuccess) break;
    cudaGraphConditionalHandle hdl;
    if ((ce = cudaGraphConditionalHandleCreate(&hdl, P.graph, 1, cudaGraphCondAssignDefault)) != cudaSuccess) break;
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = hdl;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if ((ce = cudaGraphAddNode(&node, P.graph, nullptr, nullptr, 0, &np)) != cudaSuccess) break;
    cudaGraph_t body = np.conditional.phGraph_out[0];
    if ((ce = cudaStreamBeginCaptureToGraph(P.cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) break;
    ca.handle = hdl; ca.use_handle = 1;
    // the body holds kCondUnroll attempts (each followed by the controller), so the
    // conditional node is evaluated once per kCondUnroll attempts; once the
    // controller marks the solve done, the rest of the body's kernels return at entry
    cudaError_t le = cudaSuccess;
    for (int u = 0; u < kCondUnroll && le == cudaSuccess; ++u) {
      le = launch_mix_attempt(A, P.cap);
      if (le == cudaSuccess) le = launch_controller(ca, P.cap);
    }
    cudaGraph_t captured = nullptr;
    ce = cudaStreamEndCapture(P.cap, &captured);
    if (le != cudaSuccess) { ce = le; break; }
    if (ce != cudaSuccess) break;
    ce = cudaGraphInstantiate(&P.exec, P.graph, 0);
  } while (0);
  if (ce != cudaSuccess) { set_last_error(ce, __FILE__, __LINE__); return MJX_CUDA_ERROR; }
  return MJX_OK;
}

static mjx_status run_mixed(ImexMixedPlan& P, int io_dtype, double t0, double t_end, double dt0, const void* y0,
                            void* y_final, double* hist_t, double* hist_dt, mjx_adaptive_result* res,
                            cudaStream_t s, bool host_loop) {
  const int nf = P.pb.nfields;
  char* w = P.ws;
  DevState* st = (DevState*)(w + P.L.st);
  const int max_saves = P.max_saves;
  double* real64 = (double*)(w + P.L.pa);
  double* ht = P.ht;
  double* hdt = P.hdt;
  // initial spectral state in FP64 (real input staged in PA)
  MJX_TRY(mix_state_from_real(P.plan64, &P.g, nf, io_dtype, y0, real64, (float4*)(w + P.L.ys0), s));
  DevState h;
  memset(&h, 0, sizeof(h));
  const double dt_init = (dt0 < P.pb.dt_cfl || dt0 != dt0) ? dt0 : P.pb.dt_cfl;
  h.t = t0; h.dt = dt_init; h.t_end = t_end; h.prev_err = 1.0; h.dt_cfl = P.pb.dt_cfl;
  h.status = MJX_STATUS_RUNNING_CODE; h.write_idx = 1; h.finite = 1;
  h.max_saves = max_saves; h.save_every = P.save_every; h.order = 2; h.save_slot = -1;
  h.max_attempts = P.pb.max_attempts > 0 ? P.pb.max_attempts : 20 * P.max_steps + 1000;
  const bool running = (t0 < t_end) && (1 < max_saves);
  if (running) h.dtc = dt_init < t_end - t0 ? dt_init : t_end - t0;
  else { h.done = 1; h.status = (t0 >= t_end) ? MJX_STATUS_SUCCESS_CODE : MJX_STATUS_MAX_STEPS_CODE; }
  MJX_CUDA_TRY(cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  if (ht) {
    MJX_CUDA_TRY(cudaMemsetAsync(ht, 0, sizeof(double) * max_saves, s));
    MJX_CUDA_TRY(cudaMemcpyAsync(ht, &t0, sizeof(double), cudaMemcpyHostToDevice, s));
  }
  if (hdt) MJX_CUDA_TRY(cudaMemsetAsync(hdt, 0, sizeof(double) * max_saves, s));
  MJX_CUDA_TRY(cudaStreamSynchronize(s));  // h and t0 are host stack values
  if (running && host_loop) {
    const MixAttempt A = build_mix(P.plan32, &P.g, &P.pb, &P.pid, w, P.L, st);
    CtlArgs ca;
    memset(&ca, 0, sizeof(ca));
    ca.st = st; ca.partial = (const double*)(w + P.L.part); ca.nonfinite = (const int*)(w + P.L.bad);
    ca.nparts = P.L.nparts; ca.n_dof = (double)nf * P.g.ny * P.g.nx; ca.pid = P.pid; ca.hist_t = ht; ca.hist_dt = hdt;
    const cudaError_t he = run_host_loop([&](cudaStream_t ls) -> cudaError_t {
      const cudaError_t le = launch_mix_attempt(A, ls);
      return le == cudaSuccess ? launch_controller(ca, ls) : le;
    }, st, h.max_attempts, s);
    MJX_CUDA_TRY(he);
  } else if (running) {
    MJX_CUDA_TRY(cudaGraphLaunch(P.exec, s));
  }
  // final real state: select Y^[cur] into PB, inverse FP64 transform, write real into PA
  MJX_TRY(mix_real_from_state(P.plan64, &P.g, nf, st, (const float4*)(w + P.L.ys0), (const float4*)(w + P.L.ys1),
                              (double2*)(w + P.L.pb), real64, io_dtype, y_final, s));
  if (P.own_hist && hist_t) MJX_CUDA_TRY(cudaMemcpyAsync(hist_t, ht, sizeof(double) * max_saves, cudaMemcpyDefault, s));
  if (P.own_hist && hist_dt) MJX_CUDA_TRY(cudaMemcpyAsync(hist_dt, hdt, sizeof(double) * max_saves, cudaMemcpyDefault, s));
  DevState out;
  MJX_CUDA_TRY(cudaMemcpyAsync(&out, st, sizeof(out), cudaMemcpyDeviceToHost, s));
  MJX_CUDA_TRY(cudaStreamSynchronize(s));
  if (res) {
    res->t_final = out.t; res->dt_next = out.dt; res->prev_err = out.prev_err; res->last_err = out.err_last;
    res->n_accepted = out.n_acc; res->n_rejected = out.n_rej; res->n_attempts = out.attempts;
    res->n_saved = out.write_idx; res->status = out.status; res->finite = out.finite;
  }
  return MJX_OK;
}

// hist_t / hist_dt: the caller's history arrays for a one-shot plan; null for a
// persistent plan, whose history lives after the mixed layout in its workspace.
static mjx_status make_mixed_plan(ImexMixedPlan** out, const void* plan32, const void* plan64, const mjx_grid2d* g,
                                  const mjx_imex_problem* pb, const mjx_pid_params* pid, int max_steps,
                                  int save_every, void* ws, size_t ws_bytes, bool persistent, double* hist_t,
                                  double* hist_dt) {
  MJX_TRY(check_mixed_problem(g, pb, pid, plan32, plan64, max_steps, save_every));
  const int nf = pb->nfields;
  const MixLayout L = mix_layout(g->ny, g->nx, nf, mix_nparts(g->ny, g->nx, nf));
  const int max_saves = max_steps / save_every + 1;
  const size_t ht = plan_hist_offset(L), hdt = ht + al256m(sizeof(double) * (size_t)max_saves);
  const size_t total = persistent ? hdt + al256m(sizeof(double) * (size_t)max_saves) : L.total;
  if (ws == nullptr || ws_bytes < total) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  MJX_TRY(ensure_mix_attrs());
  ImexMixedPlan* P = new ImexMixedPlan();
  P->plan32 = plan32; P->plan64 = plan64; P->g = *g; P->pb = *pb; P->pid = *pid;
  P->max_steps = max_steps; P->save_every = save_every; P->max_saves = max_saves;
  P->ws = (char*)ws; P->L = L;
  if (persistent) {
    P->ht = (double*)((char*)ws + ht); P->hdt = (double*)((char*)ws + hdt); P->own_hist = true;
  } else {
    P->ht = hist_t; P->hdt = hist_dt;
  }
  if (persistent || !host_loop_mode()) {
    const mjx_status st = capture_mixed(*P);
    if (st != MJX_OK) { free_mixed_plan(P); return st; }
  }
  *out = P;
  return MJX_OK;
}

}  // namespace mjx

extern "C" {

size_t mjx_imex_plan_ws_bytes(int ny, int nx, int nfields, int max_saves) {
  if (ilog2_exact(nx) < 1 || ilog2_exact(ny) < 1 || nfields < 1 || nfields > 4 || max_saves < 1) return 0;
  const MixLayout L = mix_layout(ny, nx, nfields, mix_nparts(ny, nx, nfields));
  return plan_hist_offset(L) + 2 * al256m(sizeof(double) * (size_t)max_saves);
}

mjx_status mjx_imex_plan_create(void** plan, const void* plan32, const void* plan64, const mjx_grid2d* g,
                                const mjx_imex_problem* pb, const mjx_pid_params* pid, int max_steps,
                                int save_every, void* ws, size_t ws_bytes) {
  if (plan == nullptr) return MJX_BAD_ARG;
  *plan = nullptr;
  ImexMixedPlan* P = nullptr;
  MJX_TRY(make_mixed_plan(&P, plan32, plan64, g, pb, pid, max_steps, save_every, ws, ws_bytes, true, nullptr,
                          nullptr));
  *plan = P;
  return MJX_OK;
}

mjx_status mjx_imex_plan_run(void* plan, int io_dtype, double t0, double t_end, double dt0, const void* y0,
                             void* y_final, double* hist_t, double* hist_dt, mjx_adaptive_result* res,
                             void* stream) {
  ImexMixedPlan* P = (ImexMixedPlan*)plan;
  if (P == nullptr || y0 == nullptr || y_final == nullptr) return MJX_BAD_ARG;
  if (!elem_size(io_dtype)) return MJX_BAD_DTYPE;
  return run_mixed(*P, io_dtype, t0, t_end, dt0, y0, y_final, hist_t, hist_dt, res, (cudaStream_t)stream,
                   host_loop_mode());
}

mjx_status mjx_imex_plan_destroy(void* plan) {
  if (plan == nullptr) return MJX_BAD_ARG;
  free_mixed_plan((ImexMixedPlan*)plan);
  return MJX_OK;
}

mjx_status mjx_imex_adaptive2d_mixed(const void* plan32, const void* plan64, const mjx_grid2d* g,
                                     int io_dtype, const mjx_imex_problem* pb,
                                     const mjx_pid_params* pid, double t0, double t_end, double dt0,
                                     int max_steps, int save_every, const void* y0, void* y_final,
                                     double* hist_t, double* hist_dt, void* ws, size_t ws_bytes,
                                     mjx_adaptive_result* res, void* stream) {
  if (!y0 || !y_final) return MJX_BAD_ARG;
  if (!elem_size(io_dtype)) return MJX_BAD_DTYPE;
  // one shot: capture, run once, release (the persistent form is mjx_imex_plan_create)
  ImexMixedPlan* P = nullptr;
  MJX_TRY(make_mixed_plan(&P, plan32, plan64, g, pb, pid, max_steps, save_every, ws, ws_bytes, false, hist_t,
                          hist_dt));
  const mjx_status st = run_mixed(*P, io_dtype, t0, t_end, dt0, y0, y_final, nullptr, nullptr, res,
                                  (cudaStream_t)stream, host_loop_mode());
  free_mixed_plan(P);
  return st;
}

}  // extern "C"
