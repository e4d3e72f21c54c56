// IMEX-Strang step, step-doubling error estimate, PI controller and the
// device-resident adaptive loop (CUDA graph with a conditional while node).
//
// One attempt of adaptive_integrate_imex (moljax/core/stepping.py:1231-1345)
// runs the full step S(dt) and two half steps S(dt/2) S(dt/2) of
// imex_strang_step (stepping.py:370-435), S(h) = H(h/2) R(h) H(h/2) with
// H(h) = (I - h D Lap)^-1 by FFT and R(h) the Heun reaction step.  The fused
// schedule shares the first forward transform between the two branches and
// merges the adjacent H(dt/4) H(dt/4) of the half-step branch into one
// column multiply by m(dt/4)^2 (both are exact identities in exact arithmetic):
//
//   K1 row  Y[cur] -> SA                       (r2c)
//   K2 col  SA -> SA * m(dt/2), SB = SA * m(dt/4)
//   K3 row  SA: c2r, R(dt), r2c;  SB: c2r, R(dt/2), r2c
//   K4 col  SA *= m(dt/2);  SB *= m(dt/4)^2
//   K5 row  SA: c2r -> YF (full step);  SB: c2r, R(dt/2), r2c
//   K6 col  SB *= m(dt/4)
//   K7 row  SB: c2r -> Y[1-cur] (two half steps) + scaled error vs YF
//   K8      controller: error norm, accept/reject, PI dt, counters, loop flag
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "controller.cuh"
#include "spectral.cuh"

namespace mjx {

mjx_status ensure_kernel_attrs();
mjx_status check_grid(const mjx_grid2d* g);
int elem_size(int dtype);

struct ImexLayout {
  size_t y0, y1, yf, sa, sb, part, bad, st, total;
  int nparts;
};

static inline size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

// Pairing of real rows for the row transforms: Gray-Scott couples u and v at
// the same row (pair = (u_y, v_y)); otherwise each field pairs rows y, y+ny/2.
struct Pairing { int coupled, nrows, npairs_per_branch; };

static Pairing pairing_for(const mjx_imex_problem* p, const mjx_grid2d* g) {
  Pairing r;
  if (p->reaction == MJX_REACT_GRAY_SCOTT) { r.coupled = 1; r.nrows = g->ny; r.npairs_per_branch = 1; }
  else { r.coupled = 0; r.nrows = g->ny / 2; r.npairs_per_branch = p->nfields; }
  return r;
}

// npairs: pairs of ONE branch (the error pass K7 writes one partial per CTA).
static ImexLayout imex_layout(int ny, int nx, int nf, int elem, int nrows, int npairs) {
  ImexLayout L;
  const size_t fb = (size_t)nf * ny * nx * elem;
  const size_t sbytes = (size_t)nf * ny * spec_ldc(nx) * 2 * elem;
  L.nparts = row_ctas(nx, nrows, npairs);
  size_t o = 0;
  L.y0 = o; o += al256(fb);
  L.y1 = o; o += al256(fb);
  L.yf = o; o += al256(fb);
  L.sa = o; o += al256(sbytes);
  L.sb = o; o += al256(sbytes);
  L.part = o; o += al256(sizeof(double) * (size_t)L.nparts);
  L.bad = o; o += al256(sizeof(int) * (size_t)L.nparts);
  L.st = o; o += al256(sizeof(DevState));
  L.total = o;
  return L;
}

// ------------------------------------------------------------------ controller


__global__ void __launch_bounds__(256) controller_kernel(CtlArgs a) {
  DevState* st = a.st;
  if (st->done) {
    if (threadIdx.x == 0 && a.use_handle) cudaGraphSetConditional(a.handle, 0u);
    return;
  }
  __shared__ double red[8];
  __shared__ int redbad[8];
  double s = 0.0, c = 0.0;
  int bad = 0;
  for (int i = threadIdx.x; i < a.nparts; i += blockDim.x) {  // Kahan per thread
    const double yv = a.partial[i] - c;
    const double tv = s + yv;
    c = (tv - s) - yv;
    s = tv;
    bad |= a.nonfinite[i];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = s; redbad[threadIdx.x >> 5] = bad; }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double tot = 0.0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { tot += red[i]; bad |= redbad[i]; }

  const bool running = ctl_update(st, tot, bad, a.n_dof, a.pid, a.hist_t, a.hist_dt);
  if (a.use_handle) cudaGraphSetConditional(a.handle, running ? 1u : 0u);
}

// attempts per iteration of the conditional while node of the adaptive loops
static constexpr int kCondUnroll = 4;

bool host_loop_mode() {
  static const int mode = [] {
    const char* v = getenv("MJX_HOST_LOOP");
    return (v != nullptr && v[0] == '1') ? 1 : 0;
  }();
  return mode == 1;
}

cudaError_t launch_controller(const CtlArgs& a, cudaStream_t s) {
  controller_kernel<<<1, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// Copies the current state into the history slot chosen by the controller.
template <typename T>
__global__ void hist_copy_kernel(const DevState* st, const T* y0, const T* y1, T* hist, long long nelem) {
  const int slot = st->save_slot;
  if (slot < 0) return;
  const T* src = st->cur == 0 ? y0 : y1;
  T* dst = hist + (long long)slot * nelem;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nelem;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

template <typename T>
__global__ void select_copy_kernel(const DevState* st, const T* y0, const T* y1, T* out, long long nelem) {
  const T* src = st->cur == 0 ? y0 : y1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nelem;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = src[i];
}

// ------------------------------------------------------------------ attempt builder
template <typename T>
struct Attempt {
  RowArgs<T> k1, k3, k5, k7;
  ColArgs<T> k2, k4, k6;
  int rx;
  int euler;  // IMEX-Euler attempt: k1..k5 only
};

template <typename T>
static void make_pairs(RowArgs<T>& r, const Pairing& pg, const mjx_grid2d* g, int nf, int branch0,
                       int nbranch, const double* hfac, const int* flags, long long s_off[2]) {
  const int ldc = spec_ldc(g->nx);
  const long long fr = (long long)g->ny * g->nx, fs = (long long)g->ny * ldc;
  int q = 0;
  for (int b = 0; b < nbranch; ++b) {
    const long long so = s_off[branch0 + b];
    if (pg.coupled) {
      RowPair& p = r.pr[q++];
      p.ra = 0; p.rb = fr; p.sa = so; p.sb = so + fs; p.hfac = hfac[b]; p.flags = flags[b];
    } else {
      for (int f = 0; f < nf; ++f) {
        RowPair& p = r.pr[q++];
        p.ra = f * fr; p.rb = f * fr + (long long)(g->ny / 2) * g->nx;
        p.sa = so + f * fs; p.sb = so + f * fs + (long long)(g->ny / 2) * ldc;
        p.hfac = hfac[b]; p.flags = flags[b];
      }
    }
  }
  r.npairs = q;
}

template <typename T>
static Attempt<T> build_attempt(const void* plan, const mjx_grid2d* g, const mjx_imex_problem* pb,
                                const mjx_pid_params* pid, char* ws, const ImexLayout& L,
                                DevState* st) {
  Attempt<T> A;
  const Pairing pg = pairing_for(pb, g);
  const int nf = pb->nfields, ldc = spec_ldc(g->nx);
  const PlanView pv = plan_view(plan, g->ny, g->nx, sizeof(T));
  T* Y0 = (T*)(ws + L.y0);
  T* Y1 = (T*)(ws + L.y1);
  T* YF = (T*)(ws + L.yf);
  cx<T>* S = (cx<T>*)(ws + L.sa);  // SA and SB are consecutive; offsets below are from SA
  long long s_off[2] = {0, (long long)((L.sb - L.sa) / sizeof(cx<T>))};
  A.rx = pb->reaction == MJX_REACT_GRAY_SCOTT ? RX_GRAY_SCOTT : (pb->reaction == MJX_REACT_FISHER ? RX_FISHER : RX_NONE);

  RowArgs<T> base;
  memset(&base, 0, sizeof(base));
  base.n = g->nx; base.log2n = ilog2_exact(g->nx); base.ldc = ldc; base.nrows = pg.nrows;
  base.nseq = row_nseq(g->nx, pg.nrows); base.rstride = g->nx;
  base.rin[0] = Y0; base.rin[1] = Y1; base.rout[0] = Y0; base.rout[1] = Y1;
  base.rin_sel = 0; base.rout_sel = 1;
  base.eref = YF; base.spec = S; base.tw = (const cx<T>*)pv.twx; base.inv_scale = (T)1;
  base.F = pb->F; base.k = pb->k; base.r = pb->r;
  base.atol = pid->atol; base.rtol = pid->rtol;
  base.partial = (double*)(ws + L.part); base.nonfinite = (int*)(ws + L.bad);
  base.st = st;

  const double h1[2] = {1.0, 0.5};
  {  // K1: r2c of Y[cur] into SA
    A.k1 = base;
    const double hf[1] = {1.0};
    const int fl[1] = {ROW_STORE_SPEC};
    make_pairs(A.k1, pg, g, nf, 0, 1, hf, fl, s_off);
  }
  {  // K3: both branches, c2r -> Heun -> r2c
    A.k3 = base;
    const int fl[2] = {ROW_LOAD_SPEC | ROW_REACT | ROW_STORE_SPEC, ROW_LOAD_SPEC | ROW_REACT | ROW_STORE_SPEC};
    make_pairs(A.k3, pg, g, nf, 0, 2, h1, fl, s_off);
  }
  {  // K5: SA -> YF; SB: c2r -> Heun(dt/2) -> r2c
    A.k5 = base;
    A.k5.rout[0] = YF; A.k5.rout_sel = -1;
    const int fl[2] = {ROW_LOAD_SPEC | ROW_STORE_REAL, ROW_LOAD_SPEC | ROW_REACT | ROW_STORE_SPEC};
    make_pairs(A.k5, pg, g, nf, 0, 2, h1, fl, s_off);
  }
  {  // K7: SB -> Y[1-cur] + error
    A.k7 = base;
    const double hf[1] = {1.0};
    const int fl[1] = {ROW_LOAD_SPEC | ROW_STORE_REAL | ROW_ERRNORM};
    make_pairs(A.k7, pg, g, nf, 1, 1, hf, fl, s_off);
  }

  ColArgs<T> cb;
  memset(&cb, 0, sizeof(cb));
  cb.ny = g->ny; cb.log2ny = ilog2_exact(g->ny); cb.ncols = g->nx / 2 + 1; cb.ldc = ldc;
  cb.spec = S; cb.lamx = (const T*)pv.lamx; cb.lamy = (const T*)pv.lamy; cb.tw = (const cx<T>*)pv.twy;
  cb.scale = (T)(1.0 / ((double)g->nx * (double)g->ny)); cb.st = st;
  const long long fs = (long long)g->ny * ldc;
  auto job = [&](long long sin, long long o0, long long o1, int nout, double D, double h0, double hB,
                 int p0, int p1) {
    ColJob j;
    memset(&j, 0, sizeof(j));
    j.sin = sin; j.sout[0] = o0; j.sout[1] = o1; j.nout = nout; j.D = D;
    j.hfac[0] = h0; j.hfac[1] = hB; j.pow[0] = p0; j.pow[1] = p1; j.mul = MUL_HELMHOLTZ;
    return j;
  };
  const double D0 = 1e-14;
  A.k2 = cb; A.k2.C = col_tile(g->ny, cb.ncols, 2, sizeof(T));
  A.k4 = cb; A.k4.C = col_tile(g->ny, cb.ncols, 1, sizeof(T));
  A.k6 = cb; A.k6.C = A.k4.C;
  for (int f = 0; f < nf; ++f) {
    const double D = pb->D[f] > D0 ? pb->D[f] : 0.0;
    const long long a = s_off[0] + f * fs, b = s_off[1] + f * fs;
    A.k2.job[A.k2.njobs++] = job(a, a, b, 2, D, 0.5, 0.25, 1, 1);
    A.k4.job[A.k4.njobs++] = job(a, a, a, 1, D, 0.5, 0.5, 1, 1);
    A.k4.job[A.k4.njobs++] = job(b, b, b, 1, D, 0.25, 0.25, 2, 2);
    A.k6.job[A.k6.njobs++] = job(b, b, b, 1, D, 0.25, 0.25, 1, 1);
  }
  A.euler = 0;
  return A;
}

// IMEX-Euler step E(h) = H(h) (y + h N(y)) (imex_euler_step, stepping.py:317-367)
// under step doubling: the full step E(dt) on branch A, E(dt/2) E(dt/2) on branch B.
//
//   E1 row  Y[cur]: Euler(dt) -> r2c SA;  Euler(dt/2) -> r2c SB
//   E2 col  SA *= m(dt);  SB *= m(dt/2)
//   E3 row  SA: c2r -> YF (full step);  SB: c2r, Euler(dt/2), r2c
//   E4 col  SB *= m(dt/2)
//   E5 row  SB: c2r -> Y[1-cur] (two half steps) + scaled error vs YF
template <typename T>
static Attempt<T> build_attempt_euler(const void* plan, const mjx_grid2d* g, const mjx_imex_problem* pb,
                                      const mjx_pid_params* pid, char* ws, const ImexLayout& L,
                                      DevState* st) {
  Attempt<T> A = build_attempt<T>(plan, g, pb, pid, ws, L, st);
  const Pairing pg = pairing_for(pb, g);
  const int nf = pb->nfields, ldc = spec_ldc(g->nx);
  long long s_off[2] = {0, (long long)((L.sb - L.sa) / sizeof(cx<T>))};
  const RowArgs<T> base = A.k1;  // shared geometry; pairs are rebuilt below
  const double h1[2] = {1.0, 0.5};
  const int RE = ROW_REACT | ROW_EULER;
  {  // E1: both branches from the real state
    A.k1 = base;
    const int fl[2] = {RE | ROW_STORE_SPEC, RE | ROW_STORE_SPEC};
    make_pairs(A.k1, pg, g, nf, 0, 2, h1, fl, s_off);
  }
  {  // E3: SA -> YF; SB: c2r -> Euler(dt/2) -> r2c
    A.k3 = base;
    A.k3.rout[0] = (T*)(ws + L.yf); A.k3.rout_sel = -1;
    const int fl[2] = {ROW_LOAD_SPEC | ROW_STORE_REAL, ROW_LOAD_SPEC | RE | ROW_STORE_SPEC};
    make_pairs(A.k3, pg, g, nf, 0, 2, h1, fl, s_off);
  }
  {  // E5: SB -> Y[1-cur] + error
    A.k5 = base;
    const double hf[1] = {1.0};
    const int fl[1] = {ROW_LOAD_SPEC | ROW_STORE_REAL | ROW_ERRNORM};
    make_pairs(A.k5, pg, g, nf, 1, 1, hf, fl, s_off);
  }
  const long long fs = (long long)g->ny * ldc;
  ColArgs<T> cb = A.k4;
  cb.njobs = 0;
  cb.C = col_tile(g->ny, cb.ncols, 1, sizeof(T));
  A.k2 = cb; A.k4 = cb;
  for (int f = 0; f < nf; ++f) {
    const double D = pb->D[f] > 1e-14 ? pb->D[f] : 0.0;
    const long long a = s_off[0] + f * fs, b = s_off[1] + f * fs;
    ColJob j;
    memset(&j, 0, sizeof(j));
    j.nout = 1; j.D = D; j.mul = MUL_HELMHOLTZ; j.pow[0] = j.pow[1] = 1;
    j.sin = j.sout[0] = j.sout[1] = a; j.hfac[0] = j.hfac[1] = 1.0;
    A.k2.job[A.k2.njobs++] = j;
    j.sin = j.sout[0] = j.sout[1] = b; j.hfac[0] = j.hfac[1] = 0.5;
    A.k2.job[A.k2.njobs++] = j;
    A.k4.job[A.k4.njobs++] = j;
  }
  A.euler = 1;
  return A;
}

template <typename T>
static Attempt<T> make_attempt(const void* plan, const mjx_grid2d* g, const mjx_imex_problem* pb,
                               const mjx_pid_params* pid, char* ws, const ImexLayout& L, DevState* st) {
  return pb->use_strang ? build_attempt<T>(plan, g, pb, pid, ws, L, st)
                        : build_attempt_euler<T>(plan, g, pb, pid, ws, L, st);
}

template <typename T>
static cudaError_t launch_attempt(const Attempt<T>& A, cudaStream_t s) {
  cudaError_t e;
#define MJX_ROW(args)                                                                           \
  e = A.rx == RX_GRAY_SCOTT ? launch_row<T, RX_GRAY_SCOTT>(args, s)                              \
      : (A.rx == RX_FISHER ? launch_row<T, RX_FISHER>(args, s) : launch_row<T, RX_NONE>(args, s)); \
  if (e != cudaSuccess) return e;
  MJX_ROW(A.k1);
  if ((e = launch_col<T>(A.k2, s)) != cudaSuccess) return e;
  MJX_ROW(A.k3);
  if ((e = launch_col<T>(A.k4, s)) != cudaSuccess) return e;
  MJX_ROW(A.k5);
  if (A.euler) return cudaSuccess;
  if ((e = launch_col<T>(A.k6, s)) != cudaSuccess) return e;
  MJX_ROW(A.k7);
#undef MJX_ROW
  return cudaSuccess;
}

static mjx_status check_problem(const mjx_imex_problem* pb, const mjx_grid2d* g) {
  if (pb == nullptr) return MJX_BAD_ARG;
  if (pb->nfields < 1 || pb->nfields > 4) return MJX_BAD_ARG;
  if (pb->reaction == MJX_REACT_GRAY_SCOTT && pb->nfields != 2) return MJX_BAD_ARG;
  if (pb->reaction < MJX_REACT_NONE || pb->reaction > MJX_REACT_FISHER) return MJX_BAD_ARG;
  (void)g;
  return MJX_OK;
}

template <typename T>
static mjx_status adaptive_run(const void* plan, const mjx_grid2d* g, const mjx_imex_problem* pb,
                               const mjx_pid_params* pid, double t0, double t_end, double dt0,
                               int max_steps, int save_every, const T* y0, T* y_final,
                               double* hist_t, double* hist_dt, T* hist_y, char* ws,
                               const ImexLayout& L, mjx_adaptive_result* res, cudaStream_t s) {
  const long long nelem = (long long)pb->nfields * g->ny * g->nx;
  DevState* st = (DevState*)(ws + L.st);
  const int max_saves = max_steps / save_every + 1;

  // initial state (stepping.py:1186-1223)
  DevState h;
  memset(&h, 0, sizeof(h));
  const double dt_init = (dt0 < pb->dt_cfl || dt0 != dt0) ? dt0 : pb->dt_cfl;  // jnp.minimum
  h.t = t0; h.dt = dt_init; h.t_end = t_end; h.prev_err = 1.0; h.dt_cfl = pb->dt_cfl;
  h.cur = 0; h.status = MJX_STATUS_RUNNING_CODE; h.write_idx = 1; h.finite = 1;
  h.max_saves = max_saves; h.save_every = save_every; h.order = pb->use_strang ? 2 : 1;  // stepping.py:1193
  h.save_slot = -1;
  h.max_attempts = pb->max_attempts > 0 ? pb->max_attempts : 20 * max_steps + 1000;
  const bool running = (t0 < t_end) && (1 < max_saves);
  if (running) {
    h.dtc = dt_init < t_end - t0 ? dt_init : t_end - t0;
  } else {
    h.done = 1;
    h.status = (t0 >= t_end) ? MJX_STATUS_SUCCESS_CODE : MJX_STATUS_MAX_STEPS_CODE;
  }
  MJX_CUDA_TRY(cudaMemcpyAsync(ws + L.y0, y0, nelem * sizeof(T), cudaMemcpyDeviceToDevice, s));
  MJX_CUDA_TRY(cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  if (hist_t) {
    MJX_CUDA_TRY(cudaMemsetAsync(hist_t, 0, sizeof(double) * max_saves, s));
    MJX_CUDA_TRY(cudaMemcpyAsync(hist_t, &t0, sizeof(double), cudaMemcpyHostToDevice, s));
  }
  if (hist_dt) MJX_CUDA_TRY(cudaMemsetAsync(hist_dt, 0, sizeof(double) * max_saves, s));
  if (hist_y) MJX_CUDA_TRY(cudaMemcpyAsync(hist_y, y0, nelem * sizeof(T), cudaMemcpyDefault, s));
  // the host copies above read host memory: make sure they are done before it goes away
  MJX_CUDA_TRY(cudaStreamSynchronize(s));

  const Attempt<T> A = make_attempt<T>(plan, g, pb, pid, ws, L, st);
  CtlArgs ca;
  memset(&ca, 0, sizeof(ca));
  ca.st = st; ca.partial = (const double*)(ws + L.part); ca.nonfinite = (const int*)(ws + L.bad);
  ca.nparts = L.nparts; ca.n_dof = (double)nelem; ca.pid = *pid; ca.hist_t = hist_t; ca.hist_dt = hist_dt;

  if (running && host_loop_mode()) {
    const cudaError_t e = run_host_loop([&](cudaStream_t ls) -> cudaError_t {
      cudaError_t le = launch_attempt<T>(A, ls);
      if (le == cudaSuccess) le = launch_controller(ca, ls);
      if (le == cudaSuccess && hist_y) {
        hist_copy_kernel<T><<<304, 256, 0, ls>>>(st, (const T*)(ws + L.y0), (const T*)(ws + L.y1), hist_y, nelem);
        le = cudaGetLastError();
      }
      return le;
    }, st, h.max_attempts, s);
    MJX_CUDA_TRY(e);
  } else if (running) {
    // Graph: while (cond) { attempt; controller sets cond }.
    cudaStream_t cs = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    mjx_status rc = MJX_OK;
    do {
      { const cudaError_t _e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking); if (_e != cudaSuccess) { set_last_error(_e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; break; } }
      { const cudaError_t _e = cudaGraphCreate(&graph, 0); if (_e != cudaSuccess) { set_last_error(_e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; break; } }
      cudaGraphConditionalHandle hdl;
      { const cudaError_t _e = cudaGraphConditionalHandleCreate(&hdl, graph, 1, cudaGraphCondAssignDefault); if (_e != cudaSuccess) { set_last_error(_e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; break; } }
      cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
      np.conditional.handle = hdl;
      np.conditional.type = cudaGraphCondTypeWhile;
      np.conditional.size = 1;
      cudaGraphNode_t node;
      { const cudaError_t _e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np); if (_e != cudaSuccess) { set_last_error(_e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; break; } }
      cudaGraph_t body = np.conditional.phGraph_out[0];
      { const cudaError_t _e = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal); if (_e != cudaSuccess) { set_last_error(_e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; break; } }
      ca.handle = hdl; ca.use_handle = 1;
      // kCondUnroll attempts per iteration of the while node; after the controller
      // marks the solve done the remaining kernels of the body return at entry (a
      // repeated history copy rewrites the same slot with the same state)
      cudaError_t le = cudaSuccess;
      for (int u = 0; u < kCondUnroll && le == cudaSuccess; ++u) {
        le = launch_attempt<T>(A, cs);
        if (le == cudaSuccess) {
          controller_kernel<<<1, 256, 0, cs>>>(ca);
          le = cudaGetLastError();
        }
        if (le == cudaSuccess && hist_y) {
          hist_copy_kernel<T><<<304, 256, 0, cs>>>(st, (const T*)(ws + L.y0), (const T*)(ws + L.y1), hist_y, nelem);
          le = cudaGetLastError();
        }
      }
      cudaGraph_t captured = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(cs, &captured);
      if (le != cudaSuccess || ce != cudaSuccess) {
        set_last_error(le != cudaSuccess ? le : ce, __FILE__, __LINE__);
        rc = MJX_CUDA_ERROR;
        break;
      }
      { const cudaError_t _e = cudaGraphInstantiate(&exec, graph, 0); if (_e != cudaSuccess) { set_last_error(_e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; break; } }
      { const cudaError_t _e = cudaGraphLaunch(exec, s); if (_e != cudaSuccess) { set_last_error(_e, __FILE__, __LINE__); rc = MJX_CUDA_ERROR; break; } }
    } while (0);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (cs) cudaStreamDestroy(cs);
    if (rc != MJX_OK) return rc;
  }
  select_copy_kernel<T><<<304, 256, 0, s>>>(st, (const T*)(ws + L.y0), (const T*)(ws + L.y1), y_final, nelem);
  MJX_CUDA_TRY(cudaGetLastError());
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

template <typename T>
static mjx_status strang_step(const void* plan, const mjx_grid2d* g, const mjx_imex_problem* pb,
                              double dt, const T* y_in, T* y_out, char* ws, const ImexLayout& L,
                              cudaStream_t s) {
  // S(dt) = H(dt/2) R(dt) H(dt/2) on branch A only, with a fixed step.
  mjx_pid_params pid;
  memset(&pid, 0, sizeof(pid));
  pid.atol = 1.0; pid.rtol = 0.0;
  if (!pb->use_strang) {
    // E(dt) = H(dt) (y + dt N(y)): E1 and E2 on branch A, then c2r of SA into y_out
    Attempt<T> E = build_attempt_euler<T>(plan, g, pb, &pid, ws, L, nullptr);
    const Pairing pg = pairing_for(pb, g);
    E.k1.rin[0] = y_in; E.k1.rin_sel = -1; E.k1.hfixed = dt; E.k1.npairs = pg.npairs_per_branch;
    E.k2.hfixed = dt;
    int nj = 0;
    for (int j = 0; j < E.k2.njobs; j += 2) E.k2.job[nj++] = E.k2.job[j];
    E.k2.njobs = nj;
    RowArgs<T> fin = E.k3;
    fin.npairs = pg.npairs_per_branch;
    fin.rout[0] = y_out; fin.rout_sel = -1;
    cudaError_t e;
#define MJX_ROW(args)                                                                           \
  e = E.rx == RX_GRAY_SCOTT ? launch_row<T, RX_GRAY_SCOTT>(args, s)                              \
      : (E.rx == RX_FISHER ? launch_row<T, RX_FISHER>(args, s) : launch_row<T, RX_NONE>(args, s)); \
  if (e != cudaSuccess) return cuda_status(e);
    MJX_ROW(E.k1);
    MJX_CUDA_TRY(launch_col<T>(E.k2, s));
    MJX_ROW(fin);
#undef MJX_ROW
    return MJX_OK;
  }
  Attempt<T> A = build_attempt<T>(plan, g, pb, &pid, ws, L, nullptr);
  const long long nelem = (long long)pb->nfields * g->ny * g->nx;
  A.k1.rin[0] = y_in; A.k1.rin_sel = -1;
  A.k1.hfixed = dt; A.k3.hfixed = dt;
  A.k2.hfixed = dt; A.k4.hfixed = dt;
  // K2 with a single output (SA * m(dt/2)), K3 restricted to branch A, K4 branch A jobs only,
  // then c2r of SA straight into y_out.
  for (int j = 0; j < A.k2.njobs; ++j) A.k2.job[j].nout = 1;
  A.k2.C = A.k4.C;
  const Pairing pg = pairing_for(pb, g);
  A.k3.npairs = pg.npairs_per_branch;
  int nj = 0;
  for (int j = 0; j < A.k4.njobs; j += 2) A.k4.job[nj++] = A.k4.job[j];
  A.k4.njobs = nj;
  RowArgs<T> fin = A.k5;
  fin.npairs = pg.npairs_per_branch;
  fin.rout[0] = y_out; fin.rout_sel = -1;
  (void)nelem;
  cudaError_t e;
#define MJX_ROW(args)                                                                           \
  e = A.rx == RX_GRAY_SCOTT ? launch_row<T, RX_GRAY_SCOTT>(args, s)                              \
      : (A.rx == RX_FISHER ? launch_row<T, RX_FISHER>(args, s) : launch_row<T, RX_NONE>(args, s)); \
  if (e != cudaSuccess) return cuda_status(e);
  MJX_ROW(A.k1);
  MJX_CUDA_TRY(launch_col<T>(A.k2, s));
  MJX_ROW(A.k3);
  MJX_CUDA_TRY(launch_col<T>(A.k4, s));
  MJX_ROW(fin);
#undef MJX_ROW
  return MJX_OK;
}

// Launches one kernel of the fused attempt (timing and profiling entry).
template <typename T>
static mjx_status attempt_kernel(const void* plan, const mjx_grid2d* g, const mjx_imex_problem* pb,
                                 const mjx_pid_params* pid, int which, double dt, const T* y,
                                 char* ws, const ImexLayout& L, cudaStream_t s) {
  DevState* st = (DevState*)(ws + L.st);
  if (which == 0) {
    DevState h;
    memset(&h, 0, sizeof(h));
    h.t = 0.0; h.dt = dt; h.dtc = dt; h.t_end = 1e300; h.prev_err = 1.0; h.dt_cfl = pb->dt_cfl;
    h.status = MJX_STATUS_RUNNING_CODE; h.write_idx = 1; h.finite = 1; h.max_saves = 1 << 30;
    h.save_every = 1 << 30; h.max_attempts = 1 << 30; h.order = pb->use_strang ? 2 : 1; h.save_slot = -1;
    const long long nelem = (long long)pb->nfields * g->ny * g->nx;
    MJX_CUDA_TRY(cudaMemcpyAsync(ws + L.y0, y, nelem * sizeof(T), cudaMemcpyDeviceToDevice, s));
    MJX_CUDA_TRY(cudaMemcpyAsync(ws + L.y1, y, nelem * sizeof(T), cudaMemcpyDeviceToDevice, s));
    MJX_CUDA_TRY(cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
    MJX_CUDA_TRY(cudaStreamSynchronize(s));
    return MJX_OK;
  }
  const Attempt<T> A = make_attempt<T>(plan, g, pb, pid, ws, L, st);
  if (A.euler && which > 5) return MJX_BAD_ARG;
  cudaError_t e = cudaSuccess;
  auto row = [&](const RowArgs<T>& r) {
    return A.rx == RX_GRAY_SCOTT ? launch_row<T, RX_GRAY_SCOTT>(r, s)
           : (A.rx == RX_FISHER ? launch_row<T, RX_FISHER>(r, s) : launch_row<T, RX_NONE>(r, s));
  };
  switch (which) {
    case 1: e = row(A.k1); break;
    case 2: e = launch_col<T>(A.k2, s); break;
    case 3: e = row(A.k3); break;
    case 4: e = launch_col<T>(A.k4, s); break;
    case 5: e = row(A.k5); break;
    case 6: e = launch_col<T>(A.k6, s); break;
    case 7: e = row(A.k7); break;
    default: return MJX_BAD_ARG;
  }
  return cuda_status(e);
}

}  // namespace mjx

using namespace mjx;

extern "C" {

mjx_status mjx_imex_attempt_kernel2d(const void* plan, const mjx_grid2d* g, int dtype,
                                     const mjx_imex_problem* pb, const mjx_pid_params* pid,
                                     int which, double dt, const void* y, void* ws,
                                     size_t ws_bytes, void* stream) {
  MJX_TRY(check_grid(g));
  MJX_TRY(check_problem(pb, g));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (plan == nullptr || pid == nullptr || (which == 0 && y == nullptr)) return MJX_BAD_ARG;
  if (ws == nullptr || ws_bytes < mjx_imex2d_ws_bytes(g->ny, g->nx, pb->nfields, dtype)) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  const Pairing pg = pairing_for(pb, g);
  const ImexLayout L = imex_layout(g->ny, g->nx, pb->nfields, e, pg.nrows, pg.npairs_per_branch);
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4) return attempt_kernel<float>(plan, g, pb, pid, which, dt, (const float*)y, (char*)ws, L, s);
  return attempt_kernel<double>(plan, g, pb, pid, which, dt, (const double*)y, (char*)ws, L, s);
}

size_t mjx_imex2d_ws_bytes(int ny, int nx, int nfields, int dtype) {
  const int e = elem_size(dtype);
  if (!e || ilog2_exact(nx) < 1 || ilog2_exact(ny) < 1 || nfields < 1 || nfields > 4) return 0;
  // the larger of the two pairings (coupled: ny rows x 1 pair; split: ny/2 rows x nfields pairs)
  const ImexLayout a = imex_layout(ny, nx, nfields, e, ny, 1);
  const ImexLayout b = imex_layout(ny, nx, nfields, e, ny / 2, nfields);
  return a.total > b.total ? a.total : b.total;
}

mjx_status mjx_imex_strang_step2d(const void* plan, const mjx_grid2d* g, int dtype,
                                  const mjx_imex_problem* pb, double dt, const void* y_in,
                                  void* y_out, void* ws, size_t ws_bytes, void* stream) {
  MJX_TRY(check_grid(g));
  MJX_TRY(check_problem(pb, g));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (plan == nullptr || y_in == nullptr || y_out == nullptr) return MJX_BAD_ARG;
  if (ws == nullptr || ws_bytes < mjx_imex2d_ws_bytes(g->ny, g->nx, pb->nfields, dtype)) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  const Pairing pg = pairing_for(pb, g);
  const ImexLayout L = imex_layout(g->ny, g->nx, pb->nfields, e, pg.nrows, pg.npairs_per_branch);
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4) return strang_step<float>(plan, g, pb, dt, (const float*)y_in, (float*)y_out, (char*)ws, L, s);
  return strang_step<double>(plan, g, pb, dt, (const double*)y_in, (double*)y_out, (char*)ws, L, s);
}

mjx_status mjx_imex_adaptive2d(const void* plan, const mjx_grid2d* g, int dtype,
                               const mjx_imex_problem* pb, const mjx_pid_params* pid, double t0,
                               double t_end, double dt0, int max_steps, int save_every,
                               const void* y0, void* y_final, double* hist_t, double* hist_dt,
                               void* hist_y, void* ws, size_t ws_bytes,
                               mjx_adaptive_result* result, void* stream) {
  MJX_TRY(check_grid(g));
  MJX_TRY(check_problem(pb, g));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (plan == nullptr || pid == nullptr || y0 == nullptr || y_final == nullptr) return MJX_BAD_ARG;
  if (max_steps < 0 || save_every < 1) return MJX_BAD_ARG;
  if (ws == nullptr || ws_bytes < mjx_imex2d_ws_bytes(g->ny, g->nx, pb->nfields, dtype)) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  // hist_y in pinned host memory: the history kernel writes it directly (NVLink-C2C on
  // Grace-Blackwell), through the device view of the allocation
  if (hist_y) {
    cudaPointerAttributes pa;
    MJX_CUDA_TRY(cudaPointerGetAttributes(&pa, hist_y));
    if (pa.type == cudaMemoryTypeHost) {
      void* d = nullptr;
      MJX_CUDA_TRY(cudaHostGetDevicePointer(&d, hist_y, 0));
      hist_y = d;
    } else if (pa.type != cudaMemoryTypeDevice && pa.type != cudaMemoryTypeManaged) {
      return MJX_BAD_ARG;  // pageable host memory cannot be written by the GPU
    }
  }
  const Pairing pg = pairing_for(pb, g);
  const ImexLayout L = imex_layout(g->ny, g->nx, pb->nfields, e, pg.nrows, pg.npairs_per_branch);
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4)
    return adaptive_run<float>(plan, g, pb, pid, t0, t_end, dt0, max_steps, save_every, (const float*)y0,
                               (float*)y_final, hist_t, hist_dt, (float*)hist_y, (char*)ws, L, result, s);
  return adaptive_run<double>(plan, g, pb, pid, t0, t_end, dt0, max_steps, save_every, (const double*)y0,
                              (double*)y_final, hist_t, hist_dt, (double*)hist_y, (char*)ws, L, result, s);
}

}  // extern "C"
