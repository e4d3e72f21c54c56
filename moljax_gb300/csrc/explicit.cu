// Explicit Runge-Kutta time stepping for reaction-advection-diffusion models
// on the 5-point stencil, with ghost-cell BCs evaluated on the fly.
//
// Restates moljax/core/stepping.py:64-163 (euler_step, ssprk3_step, rk4_step),
// the step doubling of estimate_error_doubling / step_explicit_with_error
// (566-608, 648-682) and the explicit branch of adaptive_integrate (723-1021)
// with propose_dt's CFL limit (dt_policy.py:324-408; heisenberg_cfl_dt is
// computed on the host).  The right-hand side is MOLModel.rhs (model.py:100-118)
// of the built-in models: D_f Lap(u_f) - vx du_f/dx - vy du_f/dy (upwind,
// operators.py:200-268, or central) plus the Gray-Scott or Fisher-KPP reaction.
//
// Every Runge-Kutta stage is one fused kernel over interior points: it reads
// the stage input w with its 5-point neighbourhood (ghost values from the BC
// formulas of moljax/core/bc.py:202-307, never stored), evaluates F(w) for all
// fields of the point, and writes up to two linear combinations
//   o1 = cp1 P + cq1 Q + cf1 h F(w),   o2 = cp2 P + cq2 Q + cf2 h F(w)
// (RK4 keeps its running sum in o2).  The last stage of the second half step
// also accumulates the scaled error against the full step for the controller.
// An attempt (full step + two half steps) is 3, 9 or 12 stage kernels plus the
// controller, repeated on the device by the same conditional-graph loop as the
// IMEX driver.
#include <math.h>
#include <string.h>

#include "spectral.cuh"

namespace mjx {

mjx_status ensure_kernel_attrs();
int elem_size(int dtype);
void set_last_error(cudaError_t e, const char* file, int line);

enum { XB_YCUR = 0, XB_YNEXT = 1, XB_YF = 2, XB_YH = 3, XB_W1 = 4, XB_W2 = 5, XB_ACC = 6, XB_IN = 7,
       XB_NBUF = 8, XB_NONE = -1 };

struct XModel {
  int nf, ny, nx, reaction, advection;  // advection: 0 none, 1 upwind, 2 central
  int kind[4];
  double bv[4][4];  // per field: left, right, bottom, top
  double D[4];
  double F, k, r, vx, vy, dy, dx;
};

template <typename T>
struct XStage {
  XModel m;
  T* buf[XB_NBUF];
  int w, p, q, o1, o2;
  double cp1, cq1, cf1, cp2, cq2, cf2;
  double hfac, hfixed;
  const DevState* st;
  int err;  // accumulate the scaled error of o1 against buf[XB_YF]
  double atol, rtol;
  double* partial;
  int* nonfinite;
};

template <typename T>
__device__ __forceinline__ T* xbuf(const XStage<T>& a, int id, int cur) {
  if (id == XB_YCUR) return a.buf[cur];
  if (id == XB_YNEXT) return a.buf[1 - cur];
  return a.buf[id];
}

// w at (y, x) for interior or one-cell ghost positions of field f
template <typename T>
__device__ __forceinline__ T xat(const T* w, int y, int x, const XModel& m, int f) {
  const int ny = m.ny, nx = m.nx, kind = m.kind[f];
  if (x < 0 || x >= nx) {
    const bool lo = x < 0;
    const int xs = kind == MJX_BC_PERIODIC ? (lo ? nx - 1 : 0) : (lo ? 0 : nx - 1);
    const T s = w[(long long)y * nx + xs];
    const double b = lo ? m.bv[f][0] : m.bv[f][1];
    if (kind == MJX_BC_DIRICHLET) return (T)(2.0 * b) - s;
    if (kind == MJX_BC_NEUMANN) return lo ? s - (T)(2.0 * m.dx * b) : s + (T)(2.0 * m.dx * b);
    return s;
  }
  if (y < 0 || y >= ny) {
    const bool lo = y < 0;
    const int ys = kind == MJX_BC_PERIODIC ? (lo ? ny - 1 : 0) : (lo ? 0 : ny - 1);
    const T s = w[(long long)ys * nx + x];
    const double b = lo ? m.bv[f][2] : m.bv[f][3];
    if (kind == MJX_BC_DIRICHLET) return (T)(2.0 * b) - s;
    if (kind == MJX_BC_NEUMANN) return lo ? s - (T)(2.0 * m.dy * b) : s + (T)(2.0 * m.dy * b);
    return s;
  }
  return w[(long long)y * nx + x];
}

template <typename T, int RX>
__global__ void __launch_bounds__(256) rk_stage_kernel(const __grid_constant__ XStage<T> a) {
  const DevState* st = a.st;
  if (st != nullptr && st->done) return;
  const XModel& m = a.m;
  const int cur = st != nullptr ? st->cur : 0;
  const T h = (T)((st != nullptr ? st->dtc : a.hfixed) * a.hfac);
  const T* W = xbuf(a, a.w, cur);
  const T* P = a.p >= 0 ? xbuf(a, a.p, cur) : nullptr;
  const T* Q = a.q >= 0 ? xbuf(a, a.q, cur) : nullptr;
  T* O1 = xbuf(a, a.o1, cur);
  T* O2 = a.o2 >= 0 ? xbuf(a, a.o2, cur) : nullptr;
  const T* YF = a.buf[XB_YF];
  const long long per = (long long)m.ny * m.nx;
  const T idx2 = (T)(1.0 / (m.dx * m.dx)), idy2 = (T)(1.0 / (m.dy * m.dy));
  const T idx = (T)(1.0 / m.dx), idy = (T)(1.0 / m.dy);
  double esum = 0.0;
  int bad = 0;
  for (long long pt = blockIdx.x * (long long)blockDim.x + threadIdx.x; pt < per;
       pt += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(pt / m.nx), x = (int)(pt - (long long)y * m.nx);
    T c[4], Fv[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      if (f >= m.nf) break;
      const T* wf = W + f * per;
      const T cc = wf[pt];
      const T xm = xat(wf, y, x - 1, m, f), xp = xat(wf, y, x + 1, m, f);
      const T ym = xat(wf, y - 1, x, m, f), yp = xat(wf, y + 1, x, m, f);
      T v = (T)m.D[f] * ((xp - (T)2 * cc + xm) * idx2 + (yp - (T)2 * cc + ym) * idy2);
      if (m.advection == 1) {  // d1_upwind_2d: v >= 0 backward, else forward
        const T gx = m.vx >= 0.0 ? (cc - xm) * idx : (xp - cc) * idx;
        const T gy = m.vy >= 0.0 ? (cc - ym) * idy : (yp - cc) * idy;
        v = v - (T)m.vx * gx - (T)m.vy * gy;
      } else if (m.advection == 2) {
        v = v - (T)m.vx * (xp - xm) * (T)0.5 * idx - (T)m.vy * (yp - ym) * (T)0.5 * idy;
      }
      c[f] = cc;
      Fv[f] = v;
    }
    if (RX == RX_GRAY_SCOTT) {  // operators.py:644-667
      const T uvv = c[0] * c[1] * c[1];
      Fv[0] += -uvv + (T)m.F * ((T)1 - c[0]);
      Fv[1] += uvv - (T)(m.F + m.k) * c[1];
    } else if (RX == RX_FISHER) {  // operators.py:680-705
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        if (f >= m.nf) break;
        Fv[f] += (T)m.r * c[f] * ((T)1 - c[f]);
      }
    }
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      if (f >= m.nf) break;
      const long long i = f * per + pt;
      const T pv = P ? P[i] : (T)0, qv = Q ? Q[i] : (T)0;
      const T o1 = (T)a.cp1 * pv + (T)a.cq1 * qv + (T)a.cf1 * h * Fv[f];
      if (O2) O2[i] = (T)a.cp2 * pv + (T)a.cq2 * qv + (T)a.cf2 * h * Fv[f];
      O1[i] = o1;
      if (a.err) {  // moljax/core/state.py:335-339
        const double e = ((double)o1 - (double)YF[i]) / (a.atol + a.rtol * fabs((double)o1));
        esum += e * e;
        bad |= !isfinite(o1);
      }
    }
  }
  if (a.err) {
    __shared__ double red[8];
    __shared__ int redb[8];
    for (int o = 16; o > 0; o >>= 1) {
      esum += __shfl_xor_sync(0xffffffffu, esum, o);
      bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = esum; redb[threadIdx.x >> 5] = bad; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0, cc = 0.0;
      int b = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {  // Kahan
        const double yv = red[w] - cc, tv = s + yv;
        cc = (tv - s) - yv;
        s = tv;
        b |= redb[w];
      }
      a.partial[blockIdx.x] = s;
      a.nonfinite[blockIdx.x] = b;
    }
  }
}

template <typename T>
__global__ void xhist_copy_kernel(const DevState* st, const T* y0, const T* y1, T* hist, long long nelem) {
  const int slot = st->save_slot;
  if (slot < 0) return;
  const T* src = st->cur == 0 ? y0 : y1;
  T* dst = hist + (long long)slot * nelem;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nelem;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

template <typename T>
__global__ void xselect_kernel(const DevState* st, const T* y0, const T* y1, T* out, long long n) {
  const T* src = st->cur == 0 ? y0 : y1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = src[i];
}

// ------------------------------------------------------------------ host side
enum { XNPARTS = 152 * 4 };

struct XLayout {
  size_t b[7], part, bad, st, total;
};

static inline size_t xal(size_t v) { return (v + 255) & ~size_t(255); }

static XLayout x_layout(int nf, int ny, int nx, int elem) {
  XLayout L;
  const size_t fb = (size_t)nf * ny * nx * elem;
  size_t o = 0;
  for (int i = 0; i < 7; ++i) { L.b[i] = o; o += xal(fb); }
  L.part = o; o += xal(sizeof(double) * XNPARTS);
  L.bad = o; o += xal(sizeof(int) * XNPARTS);
  L.st = o; o += xal(sizeof(DevState));
  L.total = o;
  return L;
}

static mjx_status x_model(const mjx_explicit_problem* pb, const mjx_grid2d* g, XModel* m) {
  if (pb == nullptr || g == nullptr) return MJX_BAD_ARG;
  if (pb->nfields < 1 || pb->nfields > 4 || g->ny < 1 || g->nx < 1 || !(g->dx > 0) || !(g->dy > 0))
    return MJX_BAD_SHAPE;
  if (pb->reaction < MJX_REACT_NONE || pb->reaction > MJX_REACT_FISHER) return MJX_BAD_ARG;
  if (pb->reaction == MJX_REACT_GRAY_SCOTT && pb->nfields != 2) return MJX_BAD_ARG;
  if (pb->advection < 0 || pb->advection > 2) return MJX_BAD_ARG;
  if (pb->method < 0 || pb->method > 2) return MJX_BAD_ARG;
  memset(m, 0, sizeof(*m));
  m->nf = pb->nfields; m->ny = g->ny; m->nx = g->nx; m->reaction = pb->reaction;
  m->advection = pb->advection;
  for (int f = 0; f < pb->nfields; ++f) {
    if (pb->bc_kind[f] < MJX_BC_PERIODIC || pb->bc_kind[f] > MJX_BC_NEUMANN) return MJX_BAD_ARG;
    m->kind[f] = pb->bc_kind[f];
    for (int s = 0; s < 4; ++s) m->bv[f][s] = pb->bc_values[4 * f + s];
    m->D[f] = pb->D[f];
  }
  m->F = pb->F; m->k = pb->k; m->r = pb->r; m->vx = pb->vx; m->vy = pb->vy;
  m->dy = g->dy; m->dx = g->dx;
  return MJX_OK;
}

template <typename T>
struct XAttempt {
  XStage<T> s[12];
  int n;
  int rx;
};

// stages of one step of `method` from buffer src to dst with step hfac * dt
template <typename T>
static void add_step(XAttempt<T>& A, const XStage<T>& base, int method, int src, int dst, double hfac,
                     int err_last) {
  auto push = [&](int w, int p, int q, int o1, int o2, double cp1, double cq1, double cf1,
                  double cp2, double cq2, double cf2) {
    XStage<T> s = base;
    s.w = w; s.p = p; s.q = q; s.o1 = o1; s.o2 = o2;
    s.cp1 = cp1; s.cq1 = cq1; s.cf1 = cf1; s.cp2 = cp2; s.cq2 = cq2; s.cf2 = cf2;
    s.hfac = hfac; s.err = 0;
    A.s[A.n++] = s;
  };
  if (method == 0) {         // euler_step (stepping.py:64-84)
    push(src, src, XB_NONE, dst, XB_NONE, 1, 0, 1, 0, 0, 0);
  } else if (method == 1) {  // ssprk3_step (87-123), Shu-Osher stages
    push(src, src, XB_NONE, XB_W1, XB_NONE, 1, 0, 1, 0, 0, 0);
    push(XB_W1, src, XB_W1, XB_W2, XB_NONE, 0.75, 0.25, 0.25, 0, 0, 0);
    push(XB_W2, src, XB_W2, dst, XB_NONE, 1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0, 0, 0, 0);
  } else {                   // rk4_step (126-163): running sum y + h/6 (k1 + 2k2 + 2k3) in ACC
    push(src, src, XB_NONE, XB_W1, XB_ACC, 1, 0, 0.5, 1, 0, 1.0 / 6.0);
    push(XB_W1, src, XB_ACC, XB_W2, XB_ACC, 1, 0, 0.5, 0, 1, 1.0 / 3.0);
    push(XB_W2, src, XB_ACC, XB_W1, XB_ACC, 1, 0, 1, 0, 1, 1.0 / 3.0);
    push(XB_W1, XB_NONE, XB_ACC, dst, XB_NONE, 0, 1, 1.0 / 6.0, 0, 0, 0);
  }
  if (err_last) A.s[A.n - 1].err = 1;
}

template <typename T>
static XAttempt<T> build_x(const XModel& m, int method, char* ws, const XLayout& L, DevState* st,
                           double atol, double rtol) {
  XAttempt<T> A;
  memset(&A, 0, sizeof(A));
  XStage<T> base;
  memset(&base, 0, sizeof(base));
  base.m = m;
  for (int i = 0; i < 7; ++i) base.buf[i] = (T*)(ws + L.b[i]);
  base.st = st;
  base.atol = atol; base.rtol = rtol;
  base.partial = (double*)(ws + L.part); base.nonfinite = (int*)(ws + L.bad);
  A.rx = m.reaction == MJX_REACT_GRAY_SCOTT ? RX_GRAY_SCOTT : (m.reaction == MJX_REACT_FISHER ? RX_FISHER : RX_NONE);
  // estimate_error_doubling: full step -> YF; half steps -> YH -> Y[1-cur] (+ error)
  add_step(A, base, method, XB_YCUR, XB_YF, 1.0, 0);
  add_step(A, base, method, XB_YCUR, XB_YH, 0.5, 0);
  add_step(A, base, method, XB_YH, XB_YNEXT, 0.5, 1);
  return A;
}

template <typename T>
static cudaError_t launch_stage(const XStage<T>& s, int rx, cudaStream_t st) {
  const long long per = (long long)s.m.ny * s.m.nx;
  long long blocks = (per + 255) / 256;
  if (s.err || blocks > XNPARTS) blocks = XNPARTS;  // the error pass always fills XNPARTS partials
  if (rx == RX_GRAY_SCOTT) rk_stage_kernel<T, RX_GRAY_SCOTT><<<(int)blocks, 256, 0, st>>>(s);
  else if (rx == RX_FISHER) rk_stage_kernel<T, RX_FISHER><<<(int)blocks, 256, 0, st>>>(s);
  else rk_stage_kernel<T, RX_NONE><<<(int)blocks, 256, 0, st>>>(s);
  return cudaGetLastError();
}

template <typename T>
static cudaError_t launch_x_attempt(const XAttempt<T>& A, cudaStream_t s) {
  for (int i = 0; i < A.n; ++i) {
    const cudaError_t e = launch_stage<T>(A.s[i], A.rx, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename T>
static mjx_status x_integrate(const XModel& m, int method, double dt, int n_steps, const T* y0, T* y_out,
                              char* ws, const XLayout& L, cudaStream_t s) {
  const long long nelem = (long long)m.nf * m.ny * m.nx;
  XAttempt<T> A;
  memset(&A, 0, sizeof(A));
  XStage<T> base;
  memset(&base, 0, sizeof(base));
  base.m = m;
  for (int i = 0; i < 7; ++i) base.buf[i] = (T*)(ws + L.b[i]);
  base.hfixed = dt;
  A.rx = m.reaction == MJX_REACT_GRAY_SCOTT ? RX_GRAY_SCOTT : (m.reaction == MJX_REACT_FISHER ? RX_FISHER : RX_NONE);
  MJX_CUDA_TRY(cudaMemcpyAsync(base.buf[0], y0, nelem * sizeof(T), cudaMemcpyDeviceToDevice, s));
  int src = 0;
  for (int step = 0; step < n_steps; ++step) {
    A.n = 0;
    // with st == nullptr the buffer ids XB_YCUR/XB_YNEXT address buf[0]/buf[1] directly
    add_step(A, base, method, src == 0 ? XB_YCUR : XB_YNEXT, src == 0 ? XB_YNEXT : XB_YCUR, 1.0, 0);
    const cudaError_t e = launch_x_attempt<T>(A, s);
    if (e != cudaSuccess) { set_last_error(e, __FILE__, __LINE__); return MJX_CUDA_ERROR; }
    src = 1 - src;
  }
  MJX_CUDA_TRY(cudaMemcpyAsync(y_out, base.buf[src], nelem * sizeof(T), cudaMemcpyDeviceToDevice, s));
  return MJX_OK;
}

template <typename T>
static mjx_status x_adaptive(const XModel& m, const mjx_explicit_problem* pb, const mjx_pid_params* pid,
                             double t0, double t_end, double dt0, int max_steps, int save_every,
                             const T* y0, T* y_final, double* hist_t, double* hist_dt, T* hist_y,
                             char* ws, const XLayout& L, mjx_adaptive_result* res, cudaStream_t s) {
  const long long nelem = (long long)m.nf * m.ny * m.nx;
  DevState* st = (DevState*)(ws + L.st);
  const int max_saves = max_steps / save_every + 1;
  static const int order_of[3] = {1, 3, 4};  // compute_error_order (dt_policy.py:411-423)
  DevState h;
  memset(&h, 0, sizeof(h));
  const double dt_init = (dt0 < pb->dt_cfl || dt0 != dt0) ? dt0 : pb->dt_cfl;  // explicit: min(dt0, dt_cfl)
  h.t = t0; h.dt = dt_init; h.t_end = t_end; h.prev_err = 1.0; h.dt_cfl = pb->dt_cfl;
  h.cur = 0; h.status = MJX_STATUS_RUNNING_CODE; h.write_idx = 1; h.finite = 1;
  h.max_saves = max_saves; h.save_every = save_every; h.order = order_of[pb->method];
  h.save_slot = -1;
  h.max_attempts = pb->max_attempts > 0 ? pb->max_attempts : 20 * max_steps + 1000;
  const bool running = (t0 < t_end) && (1 < max_saves);
  if (running) h.dtc = dt_init < t_end - t0 ? dt_init : t_end - t0;
  else { h.done = 1; h.status = (t0 >= t_end) ? MJX_STATUS_SUCCESS_CODE : MJX_STATUS_MAX_STEPS_CODE; }
  T* Y0 = (T*)(ws + L.b[0]);
  T* Y1 = (T*)(ws + L.b[1]);
  MJX_CUDA_TRY(cudaMemcpyAsync(Y0, y0, nelem * sizeof(T), cudaMemcpyDeviceToDevice, s));
  MJX_CUDA_TRY(cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  if (hist_t) {
    MJX_CUDA_TRY(cudaMemsetAsync(hist_t, 0, sizeof(double) * max_saves, s));
    MJX_CUDA_TRY(cudaMemcpyAsync(hist_t, &t0, sizeof(double), cudaMemcpyHostToDevice, s));
  }
  if (hist_dt) MJX_CUDA_TRY(cudaMemsetAsync(hist_dt, 0, sizeof(double) * max_saves, s));
  if (hist_y) MJX_CUDA_TRY(cudaMemcpyAsync(hist_y, y0, nelem * sizeof(T), cudaMemcpyDefault, s));
  MJX_CUDA_TRY(cudaStreamSynchronize(s));  // the host copies above read host memory

  const XAttempt<T> A = build_x<T>(m, pb->method, ws, L, st, pid->atol, pid->rtol);
  CtlArgs ca;
  memset(&ca, 0, sizeof(ca));
  ca.st = st; ca.partial = (const double*)(ws + L.part); ca.nonfinite = (const int*)(ws + L.bad);
  ca.nparts = XNPARTS; ca.n_dof = (double)nelem; ca.pid = *pid; ca.hist_t = hist_t; ca.hist_dt = hist_dt;
  auto body = [&](cudaStream_t ls) -> cudaError_t {
    cudaError_t le = launch_x_attempt<T>(A, ls);
    if (le == cudaSuccess) le = launch_controller(ca, ls);
    if (le == cudaSuccess && hist_y) {
      xhist_copy_kernel<T><<<304, 256, 0, ls>>>(st, Y0, Y1, hist_y, nelem);
      le = cudaGetLastError();
    }
    return le;
  };
  if (running && host_loop_mode()) {
    MJX_CUDA_TRY(run_host_loop(body, st, h.max_attempts, s));
  } else if (running) {
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
      cudaGraph_t gbody = np.conditional.phGraph_out[0];
      if ((ce = cudaStreamBeginCaptureToGraph(cs, gbody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) break;
      ca.handle = hdl; ca.use_handle = 1;
      const cudaError_t le = body(cs);
      cudaGraph_t captured = nullptr;
      ce = cudaStreamEndCapture(cs, &captured);
      if (le != cudaSuccess) { ce = le; break; }
      if (ce != cudaSuccess) break;
      if ((ce = cudaGraphInstantiate(&exec, graph, 0)) != cudaSuccess) break;
      ce = cudaGraphLaunch(exec, s);
    } while (0);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (cs) cudaStreamDestroy(cs);
    if (ce != cudaSuccess) { set_last_error(ce, __FILE__, __LINE__); return MJX_CUDA_ERROR; }
  }
  xselect_kernel<T><<<304, 256, 0, s>>>(st, Y0, Y1, y_final, nelem);
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

static mjx_status resolve_host_hist(void** hist_y) {
  if (*hist_y == nullptr) return MJX_OK;
  cudaPointerAttributes pa;
  MJX_CUDA_TRY(cudaPointerGetAttributes(&pa, *hist_y));
  if (pa.type == cudaMemoryTypeHost) {
    void* d = nullptr;
    MJX_CUDA_TRY(cudaHostGetDevicePointer(&d, *hist_y, 0));
    *hist_y = d;
  } else if (pa.type != cudaMemoryTypeDevice && pa.type != cudaMemoryTypeManaged) {
    return MJX_BAD_ARG;
  }
  return MJX_OK;
}

}  // namespace mjx

using namespace mjx;

extern "C" {

size_t mjx_explicit_ws_bytes(int ny, int nx, int nfields, int dtype) {
  const int e = elem_size(dtype);
  if (!e || ny < 1 || nx < 1 || nfields < 1 || nfields > 4) return 0;
  return x_layout(nfields, ny, nx, e).total;
}

mjx_status mjx_explicit_integrate2d(const mjx_grid2d* grid, int dtype, const mjx_explicit_problem* prob,
                                    double dt, int n_steps, const void* y0, void* y_out, void* ws,
                                    size_t ws_bytes, void* stream) {
  XModel m;
  MJX_TRY(x_model(prob, grid, &m));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (y0 == nullptr || y_out == nullptr || n_steps < 0) return MJX_BAD_ARG;
  const XLayout L = x_layout(m.nf, m.ny, m.nx, e);
  if (ws == nullptr || ws_bytes < L.total) return MJX_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4) return x_integrate<float>(m, prob->method, dt, n_steps, (const float*)y0, (float*)y_out, (char*)ws, L, s);
  return x_integrate<double>(m, prob->method, dt, n_steps, (const double*)y0, (double*)y_out, (char*)ws, L, s);
}

mjx_status mjx_explicit_rhs2d(const mjx_grid2d* grid, int dtype, const mjx_explicit_problem* prob,
                              const void* y, void* out, void* stream) {
  XModel m;
  MJX_TRY(x_model(prob, grid, &m));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (y == nullptr || out == nullptr || y == out) return MJX_BAD_ARG;
  const int rx = m.reaction == MJX_REACT_GRAY_SCOTT ? RX_GRAY_SCOTT : (m.reaction == MJX_REACT_FISHER ? RX_FISHER : RX_NONE);
  cudaStream_t s = (cudaStream_t)stream;
  auto run = [&](auto tag) -> cudaError_t {
    typedef decltype(tag) T;
    XStage<T> st;
    memset(&st, 0, sizeof(st));
    st.m = m;
    st.buf[XB_IN] = (T*)y;
    st.buf[XB_YF] = (T*)out;
    st.w = XB_IN; st.p = XB_NONE; st.q = XB_NONE; st.o1 = XB_YF; st.o2 = XB_NONE;
    st.cf1 = 1.0; st.hfac = 1.0; st.hfixed = 1.0;
    return launch_stage<T>(st, rx, s);
  };
  const cudaError_t ce = e == 4 ? run(0.0f) : run(0.0);
  return cuda_status(ce);
}

mjx_status mjx_explicit_adaptive2d(const mjx_grid2d* grid, int dtype, const mjx_explicit_problem* prob,
                                   const mjx_pid_params* pid, double t0, double t_end, double dt0,
                                   int max_steps, int save_every, const void* y0, void* y_final,
                                   double* hist_t, double* hist_dt, void* hist_y, void* ws,
                                   size_t ws_bytes, mjx_adaptive_result* result, void* stream) {
  XModel m;
  MJX_TRY(x_model(prob, grid, &m));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (pid == nullptr || y0 == nullptr || y_final == nullptr) return MJX_BAD_ARG;
  if (max_steps < 0 || save_every < 1) return MJX_BAD_ARG;
  const XLayout L = x_layout(m.nf, m.ny, m.nx, e);
  if (ws == nullptr || ws_bytes < L.total) return MJX_WORKSPACE;
  MJX_TRY(resolve_host_hist(&hist_y));
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4)
    return x_adaptive<float>(m, prob, pid, t0, t_end, dt0, max_steps, save_every, (const float*)y0,
                             (float*)y_final, hist_t, hist_dt, (float*)hist_y, (char*)ws, L, result, s);
  return x_adaptive<double>(m, prob, pid, t0, t_end, dt0, max_steps, save_every, (const double*)y0,
                            (double*)y_final, hist_t, hist_dt, (double*)hist_y, (char*)ws, L, result, s);
}

}  // extern "C"
