// Crank-Nicolson steps of the periodic Gray-Scott system solved by the
// preconditioned Newton iteration of benchmarks/benchmark_gray_scott.py:162-228:
// per step, with h = dt/2 and R the Gray-Scott reaction,
//   res(u) = u - u_old - h (D Lap(u) + D Lap(u_old) + R(u) + R(u_old))
//   u <- u - (I - h D Lap)^-1 res(u)      (the exact periodic inverse by FFT)
// from u = u_old, while max|res_u| + max|res_v| > tol and fewer than max_iter
// iterations ran (the residual is taken before each update, as the reference's
// while_loop does).
//
// With c_old = u_old + h (D Lap(u_old) + R(u_old)) and w(u) = h R(u) + c_old the
// update is u' = (I - h D Lap)^-1 w(u), and (I - h D Lap) u' = w(u) makes the
// residual of the next iterate a pointwise difference, res(u') = w(u) - w(u'); the
// first residual is res(u_old) = -2 h (D Lap(u_old) + R(u_old)).  So an iteration is
// one row pass (c2r of u's row spectra, w and the residual maxima, r2c of w) and one
// column pass (forward, times 1/(1 - h D lam), inverse), and a one-CTA controller
// reduces the maxima and sets the loop flag of a conditional while node: the whole
// Newton loop stays on the device.  A step is
//   S1 row r2c of u_old;  S2 col D lam u^ (inverse) -> row spectra of D Lap(u_old);
//   while { R row;  C col;  K controller }  (one graph, captured once);  E row c2r -> u_new
// enqueued by the host with no synchronisation between steps.
#include <math.h>
#include <string.h>

#include "spectral.cuh"

namespace mjx {

mjx_status ensure_kernel_attrs();
mjx_status check_grid(const mjx_grid2d* g);
int elem_size(int dtype);

struct GcnState {
  int it;          // iteration of the current step
  int step;        // steps completed
  int iters_sum;   // Newton iterations over all steps
  int max_iter;
  double tol;
  double res;      // last residual norm
};

template <typename T>
struct GcnRowArgs {
  int n, log2n, ldc, nrows, nseq;
  long long fs, fr;  // spectrum / real field strides (elements)
  const cx<T>* tw;
  cx<T>* spec;       // row spectra [2][ny][ldc]
  const T* Y;        // u_old, v_old [2][ny][nx]
  T* Cb;             // c_old
  T* W;              // w of the previous iterate
  double h, F, k;
  double* part;      // 2 maxima per CTA
  GcnState* gs;
};

// R4: radix-4 transforms, n/4 threads per row (short FP64 rows on a small grid, where the
// radix-16 pass leaves most SMs idle and each row's FP64 work is the pass's length)
template <typename T, bool R4 = false>
__global__ void __launch_bounds__(256) gcn_row_kernel(const __grid_constant__ GcnRowArgs<T> a) {
  typedef cx<T> C;
  constexpr int PTS = R4 ? 4 : 16, KPTS = PTS / 2 + 1;  // elements, half-spectrum bins per thread
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const int n = a.n, half = n >> 1;
  const int tps = R4 ? (n >= 4 ? n / 4 : 1) : (n >= 16 ? n / 16 : 1);
  const int tid = threadIdx.x;
  const int s_loc = tid / tps, lt = tid % tps;
  const bool active = s_loc < a.nseq;
  const long long y = (long long)blockIdx.x * a.nseq + s_loc;
  const int first = a.gs->it == 0;
  const int zb = s_loc * n;
#define Z(x) buf[sp(zb + (x))]
  if (active) {
    const C* A = a.spec + y * a.ldc;
    const C* B = a.spec + a.fs + y * a.ldc;
    C Ak[KPTS], Bk[KPTS];
#pragma unroll
    for (int m = 0; m < KPTS; ++m) {
      const int kk = lt + m * tps;
      if (kk <= half) { Ak[m] = A[kk]; Bk[m] = B[kk]; }
    }
#pragma unroll
    for (int m = 0; m < KPTS; ++m) {
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
  const T h = (T)a.h, F = (T)a.F, FK = (T)(a.F + a.k);
  T mu = (T)0, mv = (T)0;
  if (active) {
    const long long ro = y * n;
#pragma unroll
    for (int m = 0; m < PTS; ++m) {
      const int x = lt + m * tps;
      if (x >= n) continue;
      const C z = Z(x);
      T u, v, ru, rv, wu, wv, resu, resv;
      if (first) {  // z = D Lap(u_old); the old state from Y
        u = a.Y[ro + x];
        v = a.Y[a.fr + ro + x];
        const T uvv = u * v * v;
        ru = -uvv + F * ((T)1 - u);
        rv = uvv - FK * v;
        const T cu = u + h * (z.x + ru), cv = v + h * (z.y + rv);
        a.Cb[ro + x] = cu;
        a.Cb[a.fr + ro + x] = cv;
        wu = h * ru + cu;
        wv = h * rv + cv;
        resu = (T)-2 * h * (z.x + ru);
        resv = (T)-2 * h * (z.y + rv);
      } else {      // z = the current iterate
        u = z.x;
        v = z.y;
        const T uvv = u * v * v;
        ru = -uvv + F * ((T)1 - u);
        rv = uvv - FK * v;
        wu = h * ru + a.Cb[ro + x];
        wv = h * rv + a.Cb[a.fr + ro + x];
        resu = a.W[ro + x] - wu;
        resv = a.W[a.fr + ro + x] - wv;
      }
      a.W[ro + x] = wu;
      a.W[a.fr + ro + x] = wv;
      // NaN-propagating maxima (a NaN residual keeps the loop going to max_iter, as jnp.max)
      mu = (fabs(resu) > mu || resu != resu) ? fabs(resu) : mu;
      mv = (fabs(resv) > mv || resv != resv) ? fabs(resv) : mv;
      Z(x) = mk<C>(wu, wv);
    }
  }
  __syncthreads();
  if (R4) fft_smem_r4<T, false, false>(buf, n, a.log2n, a.nseq, n, 1, a.tw, tid);
  else fft_smem<T, false, false>(buf, n, a.log2n, a.nseq, n, 1, a.tw, tid);
  if (active) {
    C* A = a.spec + y * a.ldc;
    C* B = a.spec + a.fs + y * a.ldc;
#pragma unroll
    for (int m = 0; m < KPTS; ++m) {
      const int kk = lt + m * tps;
      if (kk > half) continue;
      const C Zk = Z(kk), Zm = Z((n - kk) & (n - 1));
      A[kk] = mk<C>((T)0.5 * (Zk.x + Zm.x), (T)0.5 * (Zk.y - Zm.y));
      B[kk] = mk<C>((T)0.5 * (Zk.y + Zm.y), (T)0.5 * (Zm.x - Zk.x));
    }
  }
#undef Z
  // block maxima of the two residuals
  __shared__ double red[2][8];
  double du = (double)mu, dv = (double)mv;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ou = __shfl_xor_sync(0xffffffffu, du, o), ov = __shfl_xor_sync(0xffffffffu, dv, o);
    du = (ou > du || ou != ou) ? ou : du;
    dv = (ov > dv || ov != ov) ? ov : dv;
  }
  if ((tid & 31) == 0) { red[0][tid >> 5] = du; red[1][tid >> 5] = dv; }
  __syncthreads();
  if (tid == 0) {
    double bu = 0.0, bv = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      bu = (red[0][i] > bu || red[0][i] != red[0][i]) ? red[0][i] : bu;
      bv = (red[1][i] > bv || red[1][i] != red[1][i]) ? red[1][i] : bv;
    }
    a.part[2 * blockIdx.x] = bu;
    a.part[2 * blockIdx.x + 1] = bv;
  }
}

// One CTA: the residual norm max|res_u| + max|res_v|, the iteration count and the loop
// flag; at the end of a step the step's iteration count goes to iters (optional).
__global__ void __launch_bounds__(256) gcn_ctl_kernel(const double* part, int nparts, GcnState* gs, int* iters,
                                                       cudaGraphConditionalHandle handle) {
  __shared__ double red[2][8];
  double mu = 0.0, mv = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    const double pu = part[2 * i], pv = part[2 * i + 1];
    mu = (pu > mu || pu != pu) ? pu : mu;
    mv = (pv > mv || pv != pv) ? pv : mv;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ou = __shfl_xor_sync(0xffffffffu, mu, o), ov = __shfl_xor_sync(0xffffffffu, mv, o);
    mu = (ou > mu || ou != ou) ? ou : mu;
    mv = (ov > mv || ov != ov) ? ov : mv;
  }
  if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = mu; red[1][threadIdx.x >> 5] = mv; }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double bu = 0.0, bv = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
    bu = (red[0][i] > bu || red[0][i] != red[0][i]) ? red[0][i] : bu;
    bv = (red[1][i] > bv || red[1][i] != red[1][i]) ? red[1][i] : bv;
  }
  const double res = bu + bv;
  gs->res = res;
  gs->it += 1;
  // cond_fn of the reference: res > tol and i < max_iter (a NaN residual fails res > tol)
  const bool go_on = res > gs->tol && gs->it < gs->max_iter;
  if (!go_on) {
    if (iters) iters[gs->step] = gs->it;
    gs->iters_sum += gs->it;
    gs->step += 1;
    gs->it = 0;
  }
  cudaGraphSetConditional(handle, go_on ? 1u : 0u);
}

struct GcnLayout {
  size_t spec, C, W, part, st, total;
  int nparts;
};
static inline size_t al256g(size_t b) { return (b + 255) & ~size_t(255); }

static GcnLayout gcn_layout(int ny, int nx, int elem) {
  GcnLayout L;
  const size_t fr = (size_t)ny * nx * elem, fsb = (size_t)ny * spec_ldc(nx) * 2 * elem;
  L.nparts = ny;  // at most one row per CTA
  size_t o = 0;
  L.spec = o; o += al256g(2 * fsb);
  L.C = o; o += al256g(2 * fr);
  L.W = o; o += al256g(2 * fr);
  L.part = o; o += al256g(2 * sizeof(double) * (size_t)L.nparts);
  L.st = o; o += al256g(sizeof(GcnState));
  L.total = o;
  return L;
}

template <typename T>
static mjx_status gcn_run(const void* plan, const mjx_grid2d* g, const double* D, double F, double k, double dt,
                          int n_steps, double tol, int max_iter, const T* y_in, T* y_out, int* iters, char* ws,
                          const GcnLayout& L, cudaStream_t s) {
  const int ny = g->ny, nx = g->nx, ldc = spec_ldc(nx);
  const long long fr = (long long)ny * nx, fs = (long long)ny * ldc;
  const PlanView pv = plan_view(plan, ny, nx, sizeof(T));
  cx<T>* spec = (cx<T>*)(ws + L.spec);
  GcnState* gs = (GcnState*)(ws + L.st);
  if (y_out != y_in) MJX_CUDA_TRY(cudaMemcpyAsync(y_out, y_in, sizeof(T) * 2 * fr, cudaMemcpyDeviceToDevice, s));
  GcnState h0;
  memset(&h0, 0, sizeof(h0));
  h0.max_iter = max_iter; h0.tol = tol;
  MJX_CUDA_TRY(cudaMemcpyAsync(gs, &h0, sizeof(h0), cudaMemcpyHostToDevice, s));
  if (n_steps <= 0) return cuda_status(cudaStreamSynchronize(s));
  // S1: r2c of (u_y, v_y) pairs of y_out; E: c2r back into y_out
  RowArgs<T> r;
  memset(&r, 0, sizeof(r));
  r.n = nx; r.log2n = ilog2_exact(nx); r.ldc = ldc; r.nrows = ny; r.npairs = 1;
  r.nseq = row_nseq(nx, ny); r.rstride = nx; r.rin_sel = -1; r.rout_sel = -1;
  r.rin[0] = y_out; r.rout[0] = y_out; r.spec = spec; r.tw = (const cx<T>*)pv.twx; r.inv_scale = (T)1;
  r.pr[0].ra = 0; r.pr[0].rb = fr; r.pr[0].sa = 0; r.pr[0].sb = fs;
  RowArgs<T> s1 = r, e1 = r;
  s1.pr[0].flags = ROW_STORE_SPEC;
  e1.pr[0].flags = ROW_LOAD_SPEC | ROW_STORE_REAL;
  // S2 (D lam, h = 1) and C (Helmholtz with h = dt/2) column passes on both fields
  ColArgs<T> c;
  memset(&c, 0, sizeof(c));
  c.ny = ny; c.log2ny = ilog2_exact(ny); c.ncols = nx / 2 + 1; c.ldc = ldc;
  c.C = col_tile(ny, c.ncols, 1, sizeof(T)); c.spec = spec; c.lamx = (const T*)pv.lamx;
  c.lamy = (const T*)pv.lamy; c.tw = (const cx<T>*)pv.twy; c.scale = (T)(1.0 / ((double)nx * ny));
  c.njobs = 2;
  for (int f = 0; f < 2; ++f) {
    ColJob& j = c.job[f];
    j.sin = j.sout[0] = j.sout[1] = f * fs;
    j.nout = 1; j.D = D[f]; j.pow[0] = j.pow[1] = 1;
  }
  ColArgs<T> s2 = c, cc = c;
  for (int f = 0; f < 2; ++f) {
    s2.job[f].mul = MUL_LAP; s2.job[f].hfac[0] = s2.job[f].hfac[1] = 1.0;
    cc.job[f].mul = MUL_HELMHOLTZ; cc.job[f].hfac[0] = cc.job[f].hfac[1] = 0.5;
  }
  s2.hfixed = 1.0;  // D lam itself
  cc.hfixed = dt;   // 1/(1 - (dt/2) D lam) with hfac 1/2
  GcnRowArgs<T> ra;
  memset(&ra, 0, sizeof(ra));
  ra.n = nx; ra.log2n = ilog2_exact(nx); ra.ldc = ldc; ra.nrows = ny; ra.nseq = row_nseq(nx, ny);
  ra.fs = fs; ra.fr = fr; ra.tw = (const cx<T>*)pv.twx; ra.spec = spec; ra.Y = y_out;
  ra.Cb = (T*)(ws + L.C); ra.W = (T*)(ws + L.W); ra.h = 0.5 * dt; ra.F = F; ra.k = k;
  ra.part = (double*)(ws + L.part); ra.gs = gs;
  // FP64 rows of at most 256 points on a small grid (the rule of the spectral row passes):
  // radix 4, at most 256 threads per CTA, fewer rows per CTA until every SM has one
  const bool r4 = sizeof(T) == 8 && nx >= 4 && nx <= 256 && (long long)ny * (nx / 16) < 152LL * 128;
  int rthreads = 256;
  if (r4) {
    const int tps4 = nx / 4;
    while (ra.nseq > 1 && ra.nseq * tps4 > 256) ra.nseq >>= 1;
    while (ra.nseq > 1 && ny / ra.nseq < 152) ra.nseq >>= 1;
    rthreads = ((ra.nseq * tps4 + 31) / 32) * 32;
  }
  const unsigned rblocks = (unsigned)(ny / ra.nseq);
  const size_t rsmem = (size_t)sp_size(ra.nseq * nx) * sizeof(cx<T>);
  static ContextOnce attr;
  MJX_TRY(attr.run([]() -> mjx_status {
    int dev = 0, optin = 0;
    MJX_CUDA_TRY(cudaGetDevice(&dev));
    MJX_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    // the opt-in maximum less each kernel's static shared memory (the block reduction)
    cudaFuncAttributes fa;
    MJX_CUDA_TRY(cudaFuncGetAttributes(&fa, gcn_row_kernel<float>));
    MJX_CUDA_TRY(cudaFuncSetAttribute(gcn_row_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      optin - (int)fa.sharedSizeBytes));
    MJX_CUDA_TRY(cudaFuncGetAttributes(&fa, gcn_row_kernel<double>));
    MJX_CUDA_TRY(cudaFuncSetAttribute(gcn_row_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      optin - (int)fa.sharedSizeBytes));
    MJX_CUDA_TRY(cudaFuncGetAttributes(&fa, gcn_row_kernel<double, true>));
    MJX_CUDA_TRY(cudaFuncSetAttribute(gcn_row_kernel<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      optin - (int)fa.sharedSizeBytes));
    return MJX_OK;
  }));
  // the Newton loop: a graph whose conditional while node repeats (R, C, K), captured once;
  // per step the host enqueues S1, S2, the loop graph and E (no synchronisation)
  cudaStream_t cs = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t ce = cudaSuccess;
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
    if ((ce = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) break;
    if (r4) gcn_row_kernel<T, true><<<rblocks, rthreads, rsmem, cs>>>(ra);
    else gcn_row_kernel<T><<<rblocks, 256, rsmem, cs>>>(ra);
    cudaError_t le = cudaGetLastError();
    if (le == cudaSuccess) le = launch_col<T>(cc, cs);
    if (le == cudaSuccess) {
      gcn_ctl_kernel<<<1, 256, 0, cs>>>(ra.part, (int)rblocks, gs, iters, hdl);
      le = cudaGetLastError();
    }
    cudaGraph_t captured = nullptr;
    ce = cudaStreamEndCapture(cs, &captured);
    if (le != cudaSuccess) { ce = le; break; }
    if (ce != cudaSuccess) break;
    if ((ce = cudaGraphInstantiate(&exec, graph, 0)) != cudaSuccess) break;
    for (int i = 0; i < n_steps && ce == cudaSuccess; ++i) {
      ce = launch_row<T, RX_NONE>(s1, s);
      if (ce == cudaSuccess) ce = launch_col<T>(s2, s);
      if (ce == cudaSuccess) ce = cudaGraphLaunch(exec, s);
      if (ce == cudaSuccess) ce = launch_row<T, RX_NONE>(e1, s);
    }
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  } while (0);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cs) cudaStreamDestroy(cs);
  return cuda_status(ce);
}

// Fixed-step Strang splitting of the same benchmark (benchmarks/benchmark_gray_scott.py:
// 268-296): explicit Euler half step of the reaction, exact exponential diffusion
// exp(dt D lam) by FFT, explicit Euler half step.  The second half step of step i and
// the first of step i+1 are two consecutive pointwise Euler steps, so a step is one column
// pass (forward, times exp(dt D lam), inverse) and one row pass (c2r, two Euler half
// steps, r2c); the first half step rides the initial r2c and the last step's row pass
// stores the real fields.  The middle steps are replayed from a graph of up to 64 steps.
template <typename T>
static mjx_status gse_run(const void* plan, const mjx_grid2d* g, const double* D, double F, double k, double dt,
                          int n_steps, const T* y_in, T* y_out, char* ws, cudaStream_t s) {
  const int ny = g->ny, nx = g->nx, ldc = spec_ldc(nx);
  const long long fr = (long long)ny * nx, fs = (long long)ny * ldc;
  const PlanView pv = plan_view(plan, ny, nx, sizeof(T));
  cx<T>* spec = (cx<T>*)ws;
  if (y_out != y_in) MJX_CUDA_TRY(cudaMemcpyAsync(y_out, y_in, sizeof(T) * 2 * fr, cudaMemcpyDeviceToDevice, s));
  if (n_steps <= 0) return cuda_status(cudaStreamSynchronize(s));
  RowArgs<T> r;
  memset(&r, 0, sizeof(r));
  r.n = nx; r.log2n = ilog2_exact(nx); r.ldc = ldc; r.nrows = ny; r.npairs = 1;
  r.nseq = row_nseq(nx, ny); r.rstride = nx; r.rin_sel = -1; r.rout_sel = -1;
  r.rin[0] = y_out; r.rout[0] = y_out; r.spec = spec; r.tw = (const cx<T>*)pv.twx; r.inv_scale = (T)1;
  r.hfixed = dt; r.F = F; r.k = k;
  r.pr[0].ra = 0; r.pr[0].rb = fr; r.pr[0].sa = 0; r.pr[0].sb = fs; r.pr[0].hfac = 0.5;
  const int RE = ROW_REACT | ROW_EULER;
  RowArgs<T> first = r, mid = r, last = r;
  first.pr[0].flags = RE | ROW_STORE_SPEC;
  mid.pr[0].flags = ROW_LOAD_SPEC | RE | ROW_EULER2 | ROW_STORE_SPEC;
  last.pr[0].flags = ROW_LOAD_SPEC | RE | ROW_STORE_REAL;
  ColArgs<T> c;
  memset(&c, 0, sizeof(c));
  c.ny = ny; c.log2ny = ilog2_exact(ny); c.ncols = nx / 2 + 1; c.ldc = ldc;
  c.C = col_tile(ny, c.ncols, 1, sizeof(T)); c.spec = spec; c.lamx = (const T*)pv.lamx;
  c.lamy = (const T*)pv.lamy; c.tw = (const cx<T>*)pv.twy; c.scale = (T)(1.0 / ((double)nx * ny));
  c.njobs = 2; c.hfixed = dt;
  for (int f = 0; f < 2; ++f) {
    ColJob& j = c.job[f];
    j.sin = j.sout[0] = j.sout[1] = f * fs;
    j.nout = 1; j.D = D[f]; j.pow[0] = j.pow[1] = 1; j.mul = MUL_EXP; j.hfac[0] = j.hfac[1] = 1.0;
  }
  cudaError_t ce = launch_row<T, RX_GRAY_SCOTT>(first, s);
  const int nmid = n_steps - 1;
  const int B = nmid < 64 ? nmid : 64;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cs = nullptr;
  if (ce == cudaSuccess && B > 0 && nmid / B > 1) {  // a graph of B middle steps
    ce = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
      cudaError_t le = cudaSuccess;
      for (int i = 0; i < B && le == cudaSuccess; ++i) {
        le = launch_col<T>(c, cs);
        if (le == cudaSuccess) le = launch_row<T, RX_GRAY_SCOTT>(mid, cs);
      }
      ce = cudaStreamEndCapture(cs, &graph);
      if (le != cudaSuccess) ce = le;
    }
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(&exec, graph, 0);
  }
  int done = 0;
  if (exec != nullptr)
    for (; done + B <= nmid && ce == cudaSuccess; done += B) ce = cudaGraphLaunch(exec, s);
  for (; done < nmid && ce == cudaSuccess; ++done) {
    ce = launch_col<T>(c, s);
    if (ce == cudaSuccess) ce = launch_row<T, RX_GRAY_SCOTT>(mid, s);
  }
  if (ce == cudaSuccess) ce = launch_col<T>(c, s);
  if (ce == cudaSuccess) ce = launch_row<T, RX_GRAY_SCOTT>(last, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cs) cudaStreamDestroy(cs);
  return cuda_status(ce);
}

}  // namespace mjx

using namespace mjx;

extern "C" {

size_t mjx_gs_cn_ws_bytes(int ny, int nx, int dtype) {
  const int e = elem_size(dtype);
  if (!e || ilog2_exact(nx) < 4 || ilog2_exact(ny) < 1) return 0;
  return gcn_layout(ny, nx, e).total;
}

mjx_status mjx_gs_cn_newton2d(const void* plan, const mjx_grid2d* g, int dtype, const double* D, double F, double k,
                              double dt, int n_steps, double tol, int max_iter, const void* y_in, void* y_out,
                              int* iters, int* iters_total, double* last_res, void* ws, size_t ws_bytes,
                              void* stream) {
  MJX_TRY(check_grid(g));
  if (g->nx < 16) return MJX_BAD_SHAPE;
  if (plan == nullptr || D == nullptr || y_in == nullptr || y_out == nullptr || n_steps < 0 || max_iter < 1)
    return MJX_BAD_ARG;
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  const GcnLayout L = gcn_layout(g->ny, g->nx, e);
  if (ws == nullptr || ws_bytes < L.total) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  mjx_status st;
  if (e == 4)
    st = gcn_run<float>(plan, g, D, F, k, dt, n_steps, tol, max_iter, (const float*)y_in, (float*)y_out, iters,
                        (char*)ws, L, s);
  else
    st = gcn_run<double>(plan, g, D, F, k, dt, n_steps, tol, max_iter, (const double*)y_in, (double*)y_out, iters,
                         (char*)ws, L, s);
  if (st != MJX_OK) return st;
  GcnState out;
  MJX_CUDA_TRY(cudaMemcpyAsync(&out, (char*)ws + L.st, sizeof(out), cudaMemcpyDeviceToHost, s));
  MJX_CUDA_TRY(cudaStreamSynchronize(s));
  if (iters_total) *iters_total = out.iters_sum;
  if (last_res) *last_res = out.res;
  return MJX_OK;
}

size_t mjx_gs_strang_exp_ws_bytes(int ny, int nx, int dtype) {
  const int e = elem_size(dtype);
  if (!e || ilog2_exact(nx) < 4 || ilog2_exact(ny) < 1) return 0;
  return (size_t)2 * ny * spec_ldc(nx) * 2 * e;
}

mjx_status mjx_gs_strang_exp2d(const void* plan, const mjx_grid2d* g, int dtype, const double* D, double F,
                               double k, double dt, int n_steps, const void* y_in, void* y_out, void* ws,
                               size_t ws_bytes, void* stream) {
  MJX_TRY(check_grid(g));
  if (g->nx < 16) return MJX_BAD_SHAPE;
  if (plan == nullptr || D == nullptr || y_in == nullptr || y_out == nullptr || n_steps < 0) return MJX_BAD_ARG;
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (ws == nullptr || ws_bytes < mjx_gs_strang_exp_ws_bytes(g->ny, g->nx, dtype)) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4)
    return gse_run<float>(plan, g, D, F, k, dt, n_steps, (const float*)y_in, (float*)y_out, (char*)ws, s);
  return gse_run<double>(plan, g, D, F, k, dt, n_steps, (const double*)y_in, (double*)y_out, (char*)ws, s);
}

}  // extern "C"
