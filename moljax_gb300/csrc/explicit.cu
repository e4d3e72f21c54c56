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
#include <stdint.h>
#include <type_traits>

#include "spectral.cuh"
#include "autotune.cuh"
#include "tma.cuh"

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
  mjx_kinetics kin;  // MJX_REACT_KINETICS
};

// A mass-action network in the state type.
template <typename T>
struct XKin {
  int nr;
  int order[MJX_KIN_MAXR][4];
  T rate[MJX_KIN_MAXR];
  T stoich[MJX_KIN_MAXR][4];
  T linear[4][4];
  T source[4];
};

// Adds the network's rates at concentrations c (NF fields, nf used) to Fv.
template <typename T, int NF>
__device__ __forceinline__ void kinetics_add(T* Fv, const T* c, int nf, const XKin<T>& q) {
#pragma unroll
  for (int s = 0; s < NF; ++s) {
    if (s >= nf) break;
    T acc = q.source[s];
#pragma unroll
    for (int j = 0; j < NF; ++j)
      if (j < nf) acc += q.linear[s][j] * c[j];
    Fv[s] += acc;
  }
  for (int r = 0; r < q.nr; ++r) {
    T w = q.rate[r];
#pragma unroll
    for (int j = 0; j < NF; ++j) {
      if (j >= nf) break;
      const int o = q.order[r][j];
      if (o >= 1) w *= c[j];
      if (o >= 2) w *= c[j];
      if (o >= 3) w *= c[j];
    }
#pragma unroll
    for (int s = 0; s < NF; ++s)
      if (s < nf) Fv[s] += q.stoich[r][s] * w;
  }
}

// The coefficients of a stage in the state type, converted on the host: FP64 arithmetic
// is rare on this part, so an FP32 stage kernel performs none per point.
template <typename T>
struct XCoef {
  T idx2, idy2, idx, idy, vx, vy, F, Fk, r;
  T D[4];
  T gv[4][4];  // ghost constants per field and side (left, right, bottom, top):
               // Dirichlet 2 b, Neumann 2 d b
  T cp1, cq1, cf1, cp2, cq2, cf2, hfac, hfixed;  // hfixed = fixed h * hfac
  T atol, rtol;
  int vxpos, vypos;
  XKin<T> kin;
};

template <typename T>
struct XStage {
  XModel m;
  XCoef<T> k;
  T* buf[XB_NBUF];
  int w, p, q, o1, o2;
  double cp1, cq1, cf1, cp2, cq2, cf2;
  double hfac, hfixed;
  const DevState* st;
  int err;  // accumulate the scaled error of o1 against buf[XB_YF]
  double atol, rtol;
  double* partial;
  int* nonfinite;
  int rows;  // rows per warp strip (tile height / XWARPS); 0: the tuned or default value
};

template <typename T>
__device__ __forceinline__ T* xbuf(const XStage<T>& a, int id, int cur) {
  if (id == XB_YCUR) return a.buf[cur];
  if (id == XB_YNEXT) return a.buf[1 - cur];
  return a.buf[id];
}

// Tiles of 32 columns x (rows x XWARPS) rows; block (32, 8): each warp owns a strip of
// `rows` rows (autotuned per grid size, default 8) and slides a three-row window down it.  The loads of a row are issued one
// row ahead (row y+2 of the stage input and row y+1 of the combine operands while row y
// is computed), with the BC ghosts applied by selects after branch-free index choices;
// the x-neighbours come from the lanes by shuffle (lanes 0 and 31 and the grid edges
// read theirs directly).  Coefficients arrive in the state type (XCoef).
enum { XROWS_DEFAULT = 8, XWARPS = 8 };

// the ghost formula of moljax/core/bc.py:202-307 on the boundary-adjacent value s
template <typename T>
__device__ __forceinline__ T xghost(T s, int kind, T g, bool lo) {
  if (kind == MJX_BC_DIRICHLET) return g - s;
  if (kind == MJX_BC_NEUMANN) return lo ? s - g : s + g;
  return s;
}

// row yy in [-1, ny] of field f at column xc (ghost rows from the BC formulas)
template <typename T>
__device__ __forceinline__ T xrow(const T* wf, int yy, int xc, const XModel& m, const XCoef<T>& k, int f) {
  const int ny = m.ny, kind = m.kind[f];
  const bool lo = yy < 0, hi = yy >= ny;
  const int ys = lo ? (kind == MJX_BC_PERIODIC ? ny - 1 : 0) : (hi ? (kind == MJX_BC_PERIODIC ? 0 : ny - 1) : yy);
  const T s = wf[(long long)ys * m.nx + xc];
  return (lo || hi) ? xghost(s, kind, lo ? k.gv[f][2] : k.gv[f][3], lo) : s;
}

template <typename T, int RX, int NF>
__global__ void __launch_bounds__(256, sizeof(T) == 8 ? 2 : (NF == 4 ? 3 : 4)) rk_stage_kernel(const __grid_constant__ XStage<T> a) {
  const DevState* st = a.st;
  if (st != nullptr && st->done) return;
  const XModel& m = a.m;
  const int cur = st != nullptr ? st->cur : 0;
  const XCoef<T>& k = a.k;
  const T h = st != nullptr ? (T)st->dtc * k.hfac : k.hfixed;  // hfac is 1 or 1/2: exact
  const T* W = xbuf(a, a.w, cur);
  const bool hasP = a.p >= 0, hasQ = a.q >= 0;
  const T* P = hasP ? xbuf(a, a.p, cur) : W;  // an absent operand reads W (cached) and is zeroed
  const T* Q = hasQ ? xbuf(a, a.q, cur) : W;
  T* O1 = xbuf(a, a.o1, cur);
  T* O2 = a.o2 >= 0 ? xbuf(a, a.o2, cur) : nullptr;
  const T* YF = a.buf[XB_YF];
  const int nf = m.nf, ny = m.ny, nx = m.nx, adv = m.advection;
  const long long per = (long long)ny * nx;
  const T idx2 = k.idx2, idy2 = k.idy2, idx = k.idx, idy = k.idy, vx = k.vx, vy = k.vy;
  const bool vxpos = k.vxpos != 0, vypos = k.vypos != 0;
  const T cp1 = k.cp1, cq1 = k.cq1, cf1h = k.cf1 * h;
  const T cp2 = k.cp2, cq2 = k.cq2, cf2h = k.cf2 * h;
  const T rF = k.F, rFk = k.Fk, rr = k.r;
  const int lane = threadIdx.x;
  const int rows = a.rows, tile_rows = rows * XWARPS;
  const int ntx = (nx + 31) >> 5, nty = (ny + tile_rows - 1) / tile_rows;
  const int ntiles = ntx * nty;
  T esum = (T)0;  // per thread in the state type; FP64 across threads (as the row kernels)
  int bad = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int ty = tile / ntx, tx = tile - ty * ntx;
    const int x = tx * 32 + lane;
    const int xc = x < nx ? x : nx - 1;
    const int y0 = ty * tile_rows + threadIdx.y * rows;
    if (y0 >= ny) continue;  // warp-uniform: a warp is one threadIdx.y
    const int y1 = y0 + rows < ny ? y0 + rows : ny;
    // x-neighbour columns of the lane that reads one directly (lane 0: left, others: right)
    T up[NF], cc[NF], dn[NF], pn[NF], qn[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      if (f >= nf) break;
      const T* wf = W + f * per;
      up[f] = xrow(wf, y0 - 1, xc, m, k, f);
      cc[f] = wf[(long long)y0 * nx + xc];
      dn[f] = xrow(wf, y0 + 1, xc, m, k, f);
      const long long i0 = f * per + (long long)y0 * nx + xc;
      pn[f] = P[i0];
      qn[f] = Q[i0];
    }
    for (int y = y0; y < y1; ++y) {
      const long long row = (long long)y * nx;
      const int yn = y + 1 < y1 ? y + 1 : y;         // the next row of this strip (or y again)
      const int y2 = y + 2 <= ny ? y + 2 : ny;       // two rows down, clamped to the ghost row
      T c[NF], Fv[NF], pc[NF], qc[NF], d2[NF];
#pragma unroll
      for (int f = 0; f < NF; ++f) {  // the loads of the next row, issued first
        if (f >= nf) break;
        const T* wf = W + f * per;
        pc[f] = pn[f];
        qc[f] = qn[f];
        d2[f] = xrow(wf, y2, xc, m, k, f);
        const long long i1 = f * per + (long long)yn * nx + xc;
        pn[f] = P[i1];
        qn[f] = Q[i1];
      }
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        if (f >= nf) break;
        const T* wf = W + f * per;
        const int kind = m.kind[f];
        const T cv = cc[f], ym = up[f], yp = dn[f];
        // lane 0 reads its left neighbour, the other lanes their right one (only lane 31
        // and the last column use it); edges take the BC ghost
        const bool left = lane == 0;
        const int xn = left ? (xc > 0 ? xc - 1 : (kind == MJX_BC_PERIODIC ? nx - 1 : 0))
                            : (xc < nx - 1 ? xc + 1 : (kind == MJX_BC_PERIODIC ? 0 : nx - 1));
        T e = wf[row + xn];
        if (left ? xc == 0 : xc >= nx - 1) e = xghost(e, kind, left ? k.gv[f][0] : k.gv[f][1], left);
        T xm = __shfl_up_sync(0xffffffffu, cv, 1), xp = __shfl_down_sync(0xffffffffu, cv, 1);
        if (left) xm = e;
        else if (lane == 31 || xc >= nx - 1) xp = e;
        if (left && xc >= nx - 1) {  // a one-lane last tile: the right ghost as well
          const int xr = kind == MJX_BC_PERIODIC ? 0 : nx - 1;
          xp = xghost(wf[row + xr], kind, k.gv[f][1], false);
        }
        T v = k.D[f] * ((xp - (T)2 * cv + xm) * idx2 + (yp - (T)2 * cv + ym) * idy2);
        if (adv == 1) {  // d1_upwind_2d: v >= 0 backward, else forward
          const T gx = vxpos ? (cv - xm) * idx : (xp - cv) * idx;
          const T gy = vypos ? (cv - ym) * idy : (yp - cv) * idy;
          v = v - vx * gx - vy * gy;
        } else if (adv == 2) {
          v = v - vx * (xp - xm) * (T)0.5 * idx - vy * (yp - ym) * (T)0.5 * idy;
        }
        c[f] = cv;
        Fv[f] = v;
        up[f] = cv;
        cc[f] = yp;
        dn[f] = d2[f];
      }
      if (RX == RX_GRAY_SCOTT) {  // operators.py:644-667
        const T uvv = c[0] * c[1] * c[1];
        Fv[0] += -uvv + rF * ((T)1 - c[0]);
        Fv[1] += uvv - rFk * c[1];
      } else if (RX == RX_FISHER) {  // operators.py:680-705
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          if (f >= nf) break;
          Fv[f] += rr * c[f] * ((T)1 - c[f]);
        }
      } else if (RX == RX_KINETICS) {
        kinetics_add<T, NF>(Fv, c, nf, k.kin);
      }
      if (x < nx) {
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          if (f >= nf) break;
          const long long i = f * per + row + x;
          const T pv = hasP ? pc[f] : (T)0, qv = hasQ ? qc[f] : (T)0;
          const T o1 = cp1 * pv + cq1 * qv + cf1h * Fv[f];
          if (O2) O2[i] = cp2 * pv + cq2 * qv + cf2h * Fv[f];
          O1[i] = o1;
          if (a.err) {  // moljax/core/state.py:335-339
            const T e = (o1 - YF[i]) / (k.atol + k.rtol * (o1 < (T)0 ? -o1 : o1));
            esum += e * e;
            bad |= !isfinite(o1);
          }
        }
      }
    }
  }
  if (a.err) {
    __shared__ double red[XWARPS];
    __shared__ int redb[XWARPS];
    double esd = (double)esum;
    for (int o = 16; o > 0; o >>= 1) {
      esd += __shfl_xor_sync(0xffffffffu, esd, o);
      bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if (lane == 0) { red[threadIdx.y] = esd; redb[threadIdx.y] = bad; }
    __syncthreads();
    if (lane == 0 && threadIdx.y == 0) {
      double s = 0.0, cc = 0.0;
      int b = 0;
      for (int w = 0; w < XWARPS; ++w) {  // Kahan
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
  if (pb->reaction < MJX_REACT_NONE || pb->reaction > MJX_REACT_KINETICS) return MJX_BAD_ARG;
  if (pb->reaction == MJX_REACT_KINETICS) {
    if (pb->kin.nreactions < 0 || pb->kin.nreactions > MJX_KIN_MAXR) return MJX_BAD_ARG;
    for (int r = 0; r < pb->kin.nreactions; ++r)
      for (int j = 0; j < 4; ++j)
        if (pb->kin.order[r][j] < 0 || pb->kin.order[r][j] > 3) return MJX_BAD_ARG;
  }
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
  if (pb->reaction == MJX_REACT_KINETICS) m->kin = pb->kin;
  return MJX_OK;
}

// compile-time reaction kind of an mjx_reaction
static int rx_of(int reaction) {
  switch (reaction) {
    case MJX_REACT_GRAY_SCOTT: return RX_GRAY_SCOTT;
    case MJX_REACT_FISHER: return RX_FISHER;
    case MJX_REACT_KINETICS: return RX_KINETICS;
    default: return RX_NONE;
  }
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
  A.rx = rx_of(m.reaction);
  // estimate_error_doubling: full step -> YF; half steps -> YH -> Y[1-cur] (+ error)
  add_step(A, base, method, XB_YCUR, XB_YF, 1.0, 0);
  add_step(A, base, method, XB_YCUR, XB_YH, 0.5, 0);
  add_step(A, base, method, XB_YH, XB_YNEXT, 0.5, 1);
  return A;
}

// 128-bit form of rk_stage_kernel: a thread owns V = 16 / sizeof(T) consecutive columns
// (one float4 / double2 per row, field and operand), a warp 32 V columns; the x-neighbours
// of a lane's first and last column come from the neighbouring lanes by shuffle (lanes 0
// and 31 and the grid edges read theirs, or the BC ghost, directly).  Used when nx is a
// multiple of V and every buffer is 16-byte aligned; same arithmetic per point as the
// scalar kernel, so the results are identical.
template <typename T> struct Vec16;
template <> struct Vec16<float> { typedef float4 t; enum { V = 4 }; };
template <> struct Vec16<double> { typedef double2 t; enum { V = 2 }; };

template <typename T, int V>
__device__ __forceinline__ void vload(const T* p, T (&v)[V]) {
  typedef typename Vec16<T>::t VT;
  const VT q = *reinterpret_cast<const VT*>(p);
  const T* e = reinterpret_cast<const T*>(&q);
#pragma unroll
  for (int k = 0; k < V; ++k) v[k] = e[k];
}

template <typename T, int V>
__device__ __forceinline__ void vstore(T* p, const T (&v)[V]) {
  typedef typename Vec16<T>::t VT;
  VT q;
  T* e = reinterpret_cast<T*>(&q);
#pragma unroll
  for (int k = 0; k < V; ++k) e[k] = v[k];
  *reinterpret_cast<VT*>(p) = q;
}

// row yy in [-1, ny] of field f at columns xb .. xb+V-1 (ghost rows from the BC formulas)
template <typename T, int V>
__device__ __forceinline__ void xrow_v(const T* wf, int yy, int xb, const XModel& m, const XCoef<T>& k, int f,
                                       T (&v)[V]) {
  const int ny = m.ny, kind = m.kind[f];
  const bool lo = yy < 0, hi = yy >= ny;
  const int ys = lo ? (kind == MJX_BC_PERIODIC ? ny - 1 : 0) : (hi ? (kind == MJX_BC_PERIODIC ? 0 : ny - 1) : yy);
  vload<T, V>(wf + (long long)ys * m.nx + xb, v);
  if (lo || hi) {
    const T g = lo ? k.gv[f][2] : k.gv[f][3];
#pragma unroll
    for (int q = 0; q < V; ++q) v[q] = xghost(v[q], kind, g, lo);
  }
}

template <typename T, int RX, int NF>
__global__ void __launch_bounds__(256, NF == 4 ? 1 : 2)
rk_stage_vec_kernel(const __grid_constant__ XStage<T> a) {
  constexpr int V = Vec16<T>::V;
  const DevState* st = a.st;
  if (st != nullptr && st->done) return;
  const XModel& m = a.m;
  const int cur = st != nullptr ? st->cur : 0;
  const XCoef<T>& k = a.k;
  const T h = st != nullptr ? (T)st->dtc * k.hfac : k.hfixed;
  const T* W = xbuf(a, a.w, cur);
  const bool hasP = a.p >= 0, hasQ = a.q >= 0;
  const T* P = hasP ? xbuf(a, a.p, cur) : W;
  const T* Q = hasQ ? xbuf(a, a.q, cur) : W;
  T* O1 = xbuf(a, a.o1, cur);
  T* O2 = a.o2 >= 0 ? xbuf(a, a.o2, cur) : nullptr;
  const T* YF = a.buf[XB_YF];
  const int nf = m.nf, ny = m.ny, nx = m.nx, adv = m.advection;
  const long long per = (long long)ny * nx;
  const T idx2 = k.idx2, idy2 = k.idy2, idx = k.idx, idy = k.idy, vx = k.vx, vy = k.vy;
  const bool vxpos = k.vxpos != 0, vypos = k.vypos != 0;
  const T cp1 = k.cp1, cq1 = k.cq1, cf1h = k.cf1 * h;
  const T cp2 = k.cp2, cq2 = k.cq2, cf2h = k.cf2 * h;
  const T rF = k.F, rFk = k.Fk, rr = k.r;
  const int lane = threadIdx.x;
  const int rows = a.rows, tile_rows = rows * XWARPS, tcols = 32 * V;
  const int ntx = (nx + tcols - 1) / tcols, nty = (ny + tile_rows - 1) / tile_rows;
  const int ntiles = ntx * nty;
  T esum = (T)0;
  int bad = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int ty = tile / ntx, tx = tile - ty * ntx;
    const int xb0 = (tx * 32 + lane) * V;
    const bool valid = xb0 < nx;
    const int xb = valid ? xb0 : nx - V;  // nx is a multiple of V
    const int y0 = ty * tile_rows + threadIdx.y * rows;
    if (y0 >= ny) continue;  // warp-uniform
    const int y1 = y0 + rows < ny ? y0 + rows : ny;
    T up[NF][V], cc[NF][V], dn[NF][V], pn[NF][V], qn[NF][V];
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      if (f >= nf) break;
      const T* wf = W + f * per;
      xrow_v<T, V>(wf, y0 - 1, xb, m, k, f, up[f]);
      vload<T, V>(wf + (long long)y0 * nx + xb, cc[f]);
      xrow_v<T, V>(wf, y0 + 1, xb, m, k, f, dn[f]);
      const long long i0 = f * per + (long long)y0 * nx + xb;
      vload<T, V>(P + i0, pn[f]);
      vload<T, V>(Q + i0, qn[f]);
    }
    for (int y = y0; y < y1; ++y) {
      const long long row = (long long)y * nx;
      const int yn = y + 1 < y1 ? y + 1 : y;
      const int y2 = y + 2 <= ny ? y + 2 : ny;
      T c[NF][V], Fv[NF][V], pc[NF][V], qc[NF][V], d2[NF][V];
#pragma unroll
      for (int f = 0; f < NF; ++f) {  // the loads of the next row, issued first
        if (f >= nf) break;
        const T* wf = W + f * per;
#pragma unroll
        for (int q = 0; q < V; ++q) { pc[f][q] = pn[f][q]; qc[f][q] = qn[f][q]; }
        xrow_v<T, V>(wf, y2, xb, m, k, f, d2[f]);
        const long long i1 = f * per + (long long)yn * nx + xb;
        vload<T, V>(P + i1, pn[f]);
        vload<T, V>(Q + i1, qn[f]);
      }
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        if (f >= nf) break;
        const T* wf = W + f * per;
        const int kind = m.kind[f];
        // left neighbour of column xb and right neighbour of column xb + V - 1
        T lft = __shfl_up_sync(0xffffffffu, cc[f][V - 1], 1);
        T rgt = __shfl_down_sync(0xffffffffu, cc[f][0], 1);
        if (lane == 0 || xb == 0) {
          const int xl = xb > 0 ? xb - 1 : (kind == MJX_BC_PERIODIC ? nx - 1 : 0);
          lft = wf[row + xl];
          if (xb == 0) lft = xghost(lft, kind, k.gv[f][0], true);
        }
        if (lane == 31 || xb + V >= nx) {
          const int xr = xb + V < nx ? xb + V : (kind == MJX_BC_PERIODIC ? 0 : nx - 1);
          rgt = wf[row + xr];
          if (xb + V >= nx) rgt = xghost(rgt, kind, k.gv[f][1], false);
        }
#pragma unroll
        for (int q = 0; q < V; ++q) {
          const T cv = cc[f][q], ym = up[f][q], yp = dn[f][q];
          const T xm = q > 0 ? cc[f][q > 0 ? q - 1 : 0] : lft;
          const T xp = q < V - 1 ? cc[f][q < V - 1 ? q + 1 : 0] : rgt;
          T v = k.D[f] * ((xp - (T)2 * cv + xm) * idx2 + (yp - (T)2 * cv + ym) * idy2);
          if (adv == 1) {
            const T gx = vxpos ? (cv - xm) * idx : (xp - cv) * idx;
            const T gy = vypos ? (cv - ym) * idy : (yp - cv) * idy;
            v = v - vx * gx - vy * gy;
          } else if (adv == 2) {
            v = v - vx * (xp - xm) * (T)0.5 * idx - vy * (yp - ym) * (T)0.5 * idy;
          }
          c[f][q] = cv;
          Fv[f][q] = v;
        }
#pragma unroll
        for (int q = 0; q < V; ++q) { up[f][q] = cc[f][q]; cc[f][q] = dn[f][q]; dn[f][q] = d2[f][q]; }
      }
#pragma unroll
      for (int q = 0; q < V; ++q) {
        if (RX == RX_GRAY_SCOTT) {  // operators.py:644-667
          const T uvv = c[0][q] * c[1][q] * c[1][q];
          Fv[0][q] += -uvv + rF * ((T)1 - c[0][q]);
          Fv[1][q] += uvv - rFk * c[1][q];
        } else if (RX == RX_FISHER) {  // operators.py:680-705
#pragma unroll
          for (int f = 0; f < NF; ++f) {
            if (f >= nf) break;
            Fv[f][q] += rr * c[f][q] * ((T)1 - c[f][q]);
          }
        } else if (RX == RX_KINETICS) {
          T cq[NF], fq[NF];
#pragma unroll
          for (int f = 0; f < NF; ++f) { cq[f] = c[f][q]; fq[f] = Fv[f][q]; }
          kinetics_add<T, NF>(fq, cq, nf, k.kin);
#pragma unroll
          for (int f = 0; f < NF; ++f) Fv[f][q] = fq[f];
        }
      }
      if (valid) {
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          if (f >= nf) break;
          const long long i = f * per + row + xb;
          T o1[V], o2[V];
#pragma unroll
          for (int q = 0; q < V; ++q) {
            const T pv = hasP ? pc[f][q] : (T)0, qv = hasQ ? qc[f][q] : (T)0;
            o1[q] = cp1 * pv + cq1 * qv + cf1h * Fv[f][q];
            o2[q] = cp2 * pv + cq2 * qv + cf2h * Fv[f][q];
          }
          if (O2) vstore<T, V>(O2 + i, o2);
          vstore<T, V>(O1 + i, o1);
          if (a.err) {  // moljax/core/state.py:335-339
            T yf[V];
            vload<T, V>(YF + i, yf);
#pragma unroll
            for (int q = 0; q < V; ++q) {
              const T e = (o1[q] - yf[q]) / (k.atol + k.rtol * (o1[q] < (T)0 ? -o1[q] : o1[q]));
              esum += e * e;
              bad |= !isfinite(o1[q]);
            }
          }
        }
      }
    }
  }
  if (a.err) {
    __shared__ double red[XWARPS];
    __shared__ int redb[XWARPS];
    double esd = (double)esum;
    for (int o = 16; o > 0; o >>= 1) {
      esd += __shfl_xor_sync(0xffffffffu, esd, o);
      bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if (lane == 0) { red[threadIdx.y] = esd; redb[threadIdx.y] = bad; }
    __syncthreads();
    if (lane == 0 && threadIdx.y == 0) {
      double s = 0.0, cc = 0.0;
      int b = 0;
      for (int w = 0; w < XWARPS; ++w) {  // Kahan
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

// the state-type coefficients of a stage (XCoef), from its FP64 description
template <typename T>
static void x_coef(XStage<T>& s) {
  const XModel& m = s.m;
  XCoef<T>& k = s.k;
  memset(&k, 0, sizeof(k));
  k.idx2 = (T)(1.0 / (m.dx * m.dx)); k.idy2 = (T)(1.0 / (m.dy * m.dy));
  k.idx = (T)(1.0 / m.dx); k.idy = (T)(1.0 / m.dy);
  k.vx = (T)m.vx; k.vy = (T)m.vy; k.vxpos = m.vx >= 0.0; k.vypos = m.vy >= 0.0;
  k.F = (T)m.F; k.Fk = (T)(m.F + m.k); k.r = (T)m.r;
  for (int f = 0; f < 4; ++f) {
    k.D[f] = (T)m.D[f];
    for (int side = 0; side < 4; ++side) {
      const double d = side < 2 ? m.dx : m.dy, b = m.bv[f][side];
      k.gv[f][side] = m.kind[f] == MJX_BC_NEUMANN ? (T)(2.0 * d * b) : (T)(2.0 * b);
    }
  }
  k.cp1 = (T)s.cp1; k.cq1 = (T)s.cq1; k.cf1 = (T)s.cf1;
  k.cp2 = (T)s.cp2; k.cq2 = (T)s.cq2; k.cf2 = (T)s.cf2;
  k.hfac = (T)s.hfac; k.hfixed = (T)(s.hfixed * s.hfac);
  k.atol = (T)s.atol; k.rtol = (T)s.rtol;
  if (m.reaction == MJX_REACT_KINETICS) {
    k.kin.nr = m.kin.nreactions;
    for (int r = 0; r < MJX_KIN_MAXR; ++r) {
      k.kin.rate[r] = (T)m.kin.rate[r];
      for (int j = 0; j < 4; ++j) { k.kin.order[r][j] = m.kin.order[r][j]; k.kin.stoich[r][j] = (T)m.kin.stoich[r][j]; }
    }
    for (int i = 0; i < 4; ++i) {
      k.kin.source[i] = (T)m.kin.source[i];
      for (int j = 0; j < 4; ++j) k.kin.linear[i][j] = (T)m.kin.linear[i][j];
    }
  }
}

// TMA-staged form of the stage kernel (FP32, nx a multiple of 4): a CTA loops over tiles of
// XT_H rows by XT_W columns; the stage input W of every field comes into shared memory as one
// 3D box per field with a one-row and a four-column halo (four columns keep the box start on a
// 16-byte boundary), two tiles in flight (the next tile's copies are issued before the
// current one is computed).  Boxes that reach past the grid are zero-filled by the copy; the
// ghost cells the 5-point stencil needs there are written from the BC formulas (periodic:
// the wrapped row or column from global memory).  The combine operands and the outputs use
// 128-bit loads and stores.  Same arithmetic per point as the scalar kernel.  A tile whose
// copies never arrive (a bounded wait) produces NaN, which the error norm reports.
enum { XT_W = 128, XT_H = 32, XT_SW = XT_W + 8, XT_SH = XT_H + 2, XT_TMA_ROWS = 64 };
// a tensor copy writes shared memory at 128-byte aligned addresses: each field's box
// (XT_SH x XT_SW floats, 18 496 bytes) sits in a slot rounded up to 128 bytes
enum { XT_BOX = XT_SH * XT_SW, XT_SLOT = (XT_BOX + 31) / 32 * 32 };
static_assert((XT_SLOT * 4) % 128 == 0, "TMA slots must keep 128-byte alignment");

struct XTmaMaps {
  CUtensorMap m[XB_NBUF];  // [nf][ny][nx] FP32 views of the stage buffers, boxes XT_SW x XT_SH x 1
};

// 128 bytes of alignment slack, 128 for the barriers, two tiles of NF field slots
static size_t x_tma_smem(int NF) { return 256 + 2 * (size_t)NF * XT_SLOT * sizeof(float); }

template <int RX, int NF>
__global__ void __launch_bounds__(256, NF == 2 ? 3 : 1)
rk_stage_tma_kernel(const __grid_constant__ XStage<float> a, const __grid_constant__ XTmaMaps tm) {
  typedef float T;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  // the dynamic region follows the static arrays: align its use to 128 bytes explicitly
  unsigned char* smem_base = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem_base);  // two barriers
  float* stg = reinterpret_cast<float*>(smem_base + 128);  // [2][NF] slots of [XT_SH][XT_SW]
  const DevState* st = a.st;
  if (st != nullptr && st->done) return;
  const XModel& m = a.m;
  const int cur = st != nullptr ? st->cur : 0;
  const XCoef<T>& k = a.k;
  const T h = st != nullptr ? (T)st->dtc * k.hfac : k.hfixed;
  const T* W = xbuf(a, a.w, cur);
  const int wid = a.w == XB_YCUR ? cur : (a.w == XB_YNEXT ? 1 - cur : a.w);
  const bool hasP = a.p >= 0, hasQ = a.q >= 0;
  const T* P = hasP ? xbuf(a, a.p, cur) : W;
  const T* Q = hasQ ? xbuf(a, a.q, cur) : W;
  T* O1 = xbuf(a, a.o1, cur);
  T* O2 = a.o2 >= 0 ? xbuf(a, a.o2, cur) : nullptr;
  const T* YF = a.buf[XB_YF];
  const int nf = m.nf, ny = m.ny, nx = m.nx, adv = m.advection;
  const long long per = (long long)ny * nx;
  const T idx2 = k.idx2, idy2 = k.idy2, idx = k.idx, idy = k.idy, vx = k.vx, vy = k.vy;
  const bool vxpos = k.vxpos != 0, vypos = k.vypos != 0;
  const T cp1 = k.cp1, cq1 = k.cq1, cf1h = k.cf1 * h;
  const T cp2 = k.cp2, cq2 = k.cq2, cf2h = k.cf2 * h;
  const T rF = k.F, rFk = k.Fk, rr = k.r;
  const int lane = threadIdx.x, warp = threadIdx.y, tid = warp * 32 + lane;
  const int ntx = (nx + XT_W - 1) / XT_W, nty = (ny + XT_H - 1) / XT_H, ntiles = ntx * nty;
  const int fsz = XT_SLOT;
  const CUtensorMap* mw = &tm.m[wid];
  if ((smem_u32(stg) & 127u) != 0) {  // guard: no tensor copy to a misaligned slot
    if (a.err && tid == 0) {
      a.partial[blockIdx.x] = __longlong_as_double(0x7ff8000000000000ll);
      a.nonfinite[blockIdx.x] = 1;
    }
    return;
  }
  if (tid == 0) { mbar_init(&bar[0], 1); mbar_init(&bar[1], 1); }
  __syncthreads();
  auto issue = [&](int tile, int sb) {  // thread 0: the boxes of every field of a tile
    const int ty = tile / ntx, tx = tile - ty * ntx;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // earlier ghost stores first
    mbar_arrive_expect_tx(&bar[sb], (unsigned)(nf * XT_BOX * sizeof(float)));
    for (int f = 0; f < nf; ++f)
      tma_load_3d(stg + (size_t)(sb * NF + f) * fsz, mw, tx * XT_W - 4, ty * XT_H - 1, f, &bar[sb]);
  };
  if (tid == 0 && (int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
  T esum = (T)0;
  int bad = 0;
  int it = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int sb = it & 1;
    if (tid == 0 && tile + (int)gridDim.x < ntiles) issue(tile + gridDim.x, sb ^ 1);
    // block-uniform: every thread leaves the loop together when the copies never land
    const bool arrived = __syncthreads_and(mbar_wait(&bar[sb], (it >> 1) & 1, 1 << 22)) != 0;
    const int ty = tile / ntx, tx = tile - ty * ntx;
    const int x0 = tx * XT_W, y0 = ty * XT_H;
    const int lxe = nx - x0 < XT_W ? nx - x0 : XT_W;  // valid columns / rows of the tile
    const int lye = ny - y0 < XT_H ? ny - y0 : XT_H;
    // ghost cells at the grid edges (the box holds zeros there)
    for (int f = 0; f < nf && arrived; ++f) {
      T* S = stg + (size_t)(sb * NF + f) * fsz;
      const int kind = m.kind[f];
      const T* wf = W + f * per;
      if (y0 == 0 && tid < lxe) {  // row -1
        const T v = kind == MJX_BC_PERIODIC ? wf[(long long)(ny - 1) * nx + x0 + tid] : S[XT_SW + 4 + tid];
        S[4 + tid] = kind == MJX_BC_PERIODIC ? v : xghost(v, kind, k.gv[f][2], true);
      }
      if (y0 + lye == ny && tid >= 128 && tid - 128 < lxe) {  // row ny
        const int c = tid - 128;
        const T v = kind == MJX_BC_PERIODIC ? wf[x0 + c] : S[lye * XT_SW + 4 + c];
        S[(lye + 1) * XT_SW + 4 + c] = kind == MJX_BC_PERIODIC ? v : xghost(v, kind, k.gv[f][3], false);
      }
      if (x0 == 0 && tid < lye) {  // column -1
        const T v = kind == MJX_BC_PERIODIC ? wf[(long long)(y0 + tid) * nx + nx - 1] : S[(tid + 1) * XT_SW + 4];
        S[(tid + 1) * XT_SW + 3] = kind == MJX_BC_PERIODIC ? v : xghost(v, kind, k.gv[f][0], true);
      }
      if (x0 + lxe == nx && tid >= 64 && tid - 64 < lye) {  // column nx
        const int r = tid - 64;
        const T v = kind == MJX_BC_PERIODIC ? wf[(long long)(y0 + r) * nx] : S[(r + 1) * XT_SW + 4 + lxe - 1];
        S[(r + 1) * XT_SW + 4 + lxe] = kind == MJX_BC_PERIODIC ? v : xghost(v, kind, k.gv[f][1], false);
      }
    }
    __syncthreads();
    const int lx = lane * 4;
    const bool colv = lx < lxe;
    const T nanv = __int_as_float(0x7fc00000);
#pragma unroll
    for (int j = 0; j < XT_H / XWARPS; ++j) {
      const int ly = warp * (XT_H / XWARPS) + j;
      const bool valid = colv && ly < lye;
      const long long row = (long long)(y0 + ly) * nx;
      T c[NF][4], Fv[NF][4];
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        if (f >= nf) break;
        const T* S = stg + (size_t)(sb * NF + f) * fsz;
        const float4 cv4 = *reinterpret_cast<const float4*>(S + (ly + 1) * XT_SW + 4 + lx);
        const float4 up4 = *reinterpret_cast<const float4*>(S + ly * XT_SW + 4 + lx);
        const float4 dn4 = *reinterpret_cast<const float4*>(S + (ly + 2) * XT_SW + 4 + lx);
        T lft = __shfl_up_sync(0xffffffffu, cv4.w, 1);
        T rgt = __shfl_down_sync(0xffffffffu, cv4.x, 1);
        if (lane == 0) lft = S[(ly + 1) * XT_SW + 3];
        if (lane == 31 || lx + 4 >= lxe) rgt = S[(ly + 1) * XT_SW + 4 + lx + 4];
        const T cc[4] = {cv4.x, cv4.y, cv4.z, cv4.w};
        const T uu[4] = {up4.x, up4.y, up4.z, up4.w};
        const T dd[4] = {dn4.x, dn4.y, dn4.z, dn4.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const T cvq = cc[q], ym = uu[q], yp = dd[q];
          const T xm = q > 0 ? cc[q > 0 ? q - 1 : 0] : lft;
          const T xp = q < 3 ? cc[q < 3 ? q + 1 : 0] : rgt;
          T v = k.D[f] * ((xp - (T)2 * cvq + xm) * idx2 + (yp - (T)2 * cvq + ym) * idy2);
          if (adv == 1) {
            const T gx = vxpos ? (cvq - xm) * idx : (xp - cvq) * idx;
            const T gy = vypos ? (cvq - ym) * idy : (yp - cvq) * idy;
            v = v - vx * gx - vy * gy;
          } else if (adv == 2) {
            v = v - vx * (xp - xm) * (T)0.5 * idx - vy * (yp - ym) * (T)0.5 * idy;
          }
          c[f][q] = arrived ? cvq : nanv;
          Fv[f][q] = arrived ? v : nanv;
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (RX == RX_GRAY_SCOTT) {  // operators.py:644-667
          const T uvv = c[0][q] * c[1][q] * c[1][q];
          Fv[0][q] += -uvv + rF * ((T)1 - c[0][q]);
          Fv[1][q] += uvv - rFk * c[1][q];
        } else if (RX == RX_FISHER) {  // operators.py:680-705
#pragma unroll
          for (int f = 0; f < NF; ++f) {
            if (f >= nf) break;
            Fv[f][q] += rr * c[f][q] * ((T)1 - c[f][q]);
          }
        } else if (RX == RX_KINETICS) {
          T cq[NF], fq[NF];
#pragma unroll
          for (int f = 0; f < NF; ++f) { cq[f] = c[f][q]; fq[f] = Fv[f][q]; }
          kinetics_add<T, NF>(fq, cq, nf, k.kin);
#pragma unroll
          for (int f = 0; f < NF; ++f) Fv[f][q] = fq[f];
        }
      }
      if (valid) {
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          if (f >= nf) break;
          const long long i = f * per + row + x0 + lx;
          T pc[4], qc[4], o1[4], o2[4];
          vload<T, 4>(P + i, pc);
          vload<T, 4>(Q + i, qc);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const T pv = hasP ? pc[q] : (T)0, qv = hasQ ? qc[q] : (T)0;
            o1[q] = cp1 * pv + cq1 * qv + cf1h * Fv[f][q];
            o2[q] = cp2 * pv + cq2 * qv + cf2h * Fv[f][q];
          }
          if (O2) vstore<T, 4>(O2 + i, o2);
          vstore<T, 4>(O1 + i, o1);
          if (a.err) {  // moljax/core/state.py:335-339
            T yf[4];
            vload<T, 4>(YF + i, yf);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const T e = (o1[q] - yf[q]) / (k.atol + k.rtol * (o1[q] < (T)0 ? -o1[q] : o1[q]));
              esum += e * e;
              bad |= !isfinite(o1[q]);
            }
          }
        }
      }
    }
    __syncthreads();  // the buffer is refilled by the copy issued two tiles later
    if (!arrived) {
      // the next tile's copies may still be in flight into the other buffer: wait for
      // them (bounded) before the block's shared memory is released
      if (tile + (int)gridDim.x < ntiles) mbar_wait(&bar[sb ^ 1], ((it + 1) >> 1) & 1, 1 << 22);
      break;
    }
  }
  if (a.err) {
    __shared__ double red[XWARPS];
    __shared__ int redb[XWARPS];
    double esd = (double)esum;
    for (int o = 16; o > 0; o >>= 1) {
      esd += __shfl_xor_sync(0xffffffffu, esd, o);
      bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if (lane == 0) { red[warp] = esd; redb[warp] = bad; }
    __syncthreads();
    if (tid == 0) {
      double s2 = 0.0, cc = 0.0;  // Kahan
      int b = 0;
      for (int w = 0; w < XWARPS; ++w) {
        const double yv = red[w] - cc;
        const double tv = s2 + yv;
        cc = (tv - s2) - yv;
        s2 = tv;
        b |= redb[w];
      }
      a.partial[blockIdx.x] = s2;
      a.nonfinite[blockIdx.x] = b;
    }
  }
}

// The TMA form applies when the stage is FP32, nx is a multiple of 4 (16-byte rows) and
// every buffer is 16-byte aligned; the maps cover the buffers the stage can read as W.
static bool x_tma_ok(const XStage<float>& s) {
  if (s.m.nx % 4 != 0) return false;
  for (int i = 0; i < XB_NBUF; ++i)
    if (s.buf[i] && ((uintptr_t)s.buf[i] & 15)) return false;
  return true;
}

template <int RX>
static cudaError_t launch_stage_tma_rx(const XStage<float>& s, cudaStream_t st) {
  XTmaMaps tm;
  memset(&tm, 0, sizeof(tm));
  // maps of the buffers the stage can read as W (the current state resolves on the device)
  for (int i = 0; i < XB_NBUF; ++i) {
    const bool wcand = s.w == XB_YCUR || s.w == XB_YNEXT ? i <= XB_YNEXT : i == s.w;
    if (wcand && s.buf[i] != nullptr &&
        make_tmap_3d_f32(&tm.m[i], s.buf[i], s.m.nx, s.m.ny, s.m.nf, XT_SW, XT_SH) != MJX_OK)
      return cudaErrorInvalidValue;
  }
  const int NFa = s.m.nf <= 2 ? 2 : 4;
  const size_t smem = x_tma_smem(NFa);
  const long long tiles = (long long)((s.m.nx + XT_W - 1) / XT_W) * ((s.m.ny + XT_H - 1) / XT_H);
  // one resident wave over the tiles; the error pass fills every partial slot
  const int res = (NFa == 2 ? 3 : 1) * 152;
  const int blocks = s.err ? XNPARTS : (int)(tiles < res ? tiles : res);
  const dim3 blk(32, XWARPS);
  static ContextOnce attr;
  cudaError_t e = cudaSuccess;
  const mjx_status as = attr.run([&]() -> mjx_status {
    e = cudaFuncSetAttribute(rk_stage_tma_kernel<RX, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)x_tma_smem(2));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(rk_stage_tma_kernel<RX, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)x_tma_smem(4));
    return e == cudaSuccess ? MJX_OK : MJX_CUDA_ERROR;
  });
  if (as != MJX_OK) return e != cudaSuccess ? e : cudaErrorInvalidValue;
  if (NFa == 2) rk_stage_tma_kernel<RX, 2><<<blocks, blk, smem, st>>>(s, tm);
  else rk_stage_tma_kernel<RX, 4><<<blocks, blk, smem, st>>>(s, tm);
  return cudaGetLastError();
}

static cudaError_t x_launch_tma(const XStage<float>& s, int rx, cudaStream_t st) {
  switch (rx) {
    case RX_GRAY_SCOTT: return launch_stage_tma_rx<RX_GRAY_SCOTT>(s, st);
    case RX_FISHER: return launch_stage_tma_rx<RX_FISHER>(s, st);
    case RX_KINETICS: return launch_stage_tma_rx<RX_KINETICS>(s, st);
    default: return launch_stage_tma_rx<RX_NONE>(s, st);
  }
}
static cudaError_t x_launch_tma(const XStage<double>&, int, cudaStream_t) { return cudaErrorInvalidValue; }
static bool x_tma_able(const XStage<float>& s) { return x_tma_ok(s); }
static bool x_tma_able(const XStage<double>&) { return false; }

template <typename T>
static cudaError_t launch_stage(const XStage<T>& s0, int rx, cudaStream_t st) {
  XStage<T> s = s0;
  x_coef(s);
  if (s.rows <= 0) {
    const int tuned = tune_rows_get(s.m.ny, s.m.nx, s.m.nf, (int)sizeof(T));
    s.rows = tuned > 0 ? tuned : XROWS_DEFAULT;
  }
  if (s.rows == XT_TMA_ROWS) {  // the TMA-staged form (selected by the autotuner)
    if (x_tma_able(s)) return x_launch_tma(s, rx, st);
    s.rows = XROWS_DEFAULT;
  }
  const int tile_rows = s.rows * XWARPS;
  // the 128-bit form when nx is a multiple of the vector width and every buffer is
  // 16-byte aligned (offsets f * ny * nx elements keep the alignment then)
  constexpr int V = Vec16<T>::V;
  bool vec = s.m.nx % V == 0;
  for (int i = 0; i < XB_NBUF && vec; ++i) vec = ((uintptr_t)s.buf[i] & 15) == 0;
  const int tcols = vec ? 32 * V : 32;
  const long long tiles = (long long)((s.m.nx + tcols - 1) / tcols) * ((s.m.ny + tile_rows - 1) / tile_rows);
  // one resident wave (4 blocks of 256 threads per SM) looping over the tiles; the error
  // pass always fills XNPARTS partials
  const int blocks = s.err ? XNPARTS : (int)(tiles < XNPARTS ? tiles : XNPARTS);
  const dim3 blk(32, XWARPS);
  if (vec) {
    // two resident blocks per SM (one with four fields): one wave looping over the tiles
    const int res = (s.m.nf <= 2 ? 2 : 1) * 152;
    const int vblocks = s.err ? XNPARTS : (int)(tiles < res ? tiles : res);
    if (rx == RX_GRAY_SCOTT) rk_stage_vec_kernel<T, RX_GRAY_SCOTT, 2><<<vblocks, blk, 0, st>>>(s);
    else if (s.m.nf <= 2) {
      if (rx == RX_FISHER) rk_stage_vec_kernel<T, RX_FISHER, 2><<<vblocks, blk, 0, st>>>(s);
      else if (rx == RX_KINETICS) rk_stage_vec_kernel<T, RX_KINETICS, 2><<<vblocks, blk, 0, st>>>(s);
      else rk_stage_vec_kernel<T, RX_NONE, 2><<<vblocks, blk, 0, st>>>(s);
    } else {
      if (rx == RX_FISHER) rk_stage_vec_kernel<T, RX_FISHER, 4><<<vblocks, blk, 0, st>>>(s);
      else if (rx == RX_KINETICS) rk_stage_vec_kernel<T, RX_KINETICS, 4><<<vblocks, blk, 0, st>>>(s);
      else rk_stage_vec_kernel<T, RX_NONE, 4><<<vblocks, blk, 0, st>>>(s);
    }
    return cudaGetLastError();
  }
  if (rx == RX_GRAY_SCOTT) rk_stage_kernel<T, RX_GRAY_SCOTT, 2><<<blocks, blk, 0, st>>>(s);
  else if (s.m.nf <= 2) {
    if (rx == RX_FISHER) rk_stage_kernel<T, RX_FISHER, 2><<<blocks, blk, 0, st>>>(s);
    else if (rx == RX_KINETICS) rk_stage_kernel<T, RX_KINETICS, 2><<<blocks, blk, 0, st>>>(s);
    else rk_stage_kernel<T, RX_NONE, 2><<<blocks, blk, 0, st>>>(s);
  } else {
    if (rx == RX_FISHER) rk_stage_kernel<T, RX_FISHER, 4><<<blocks, blk, 0, st>>>(s);
    else if (rx == RX_KINETICS) rk_stage_kernel<T, RX_KINETICS, 4><<<blocks, blk, 0, st>>>(s);
    else rk_stage_kernel<T, RX_NONE, 4><<<blocks, blk, 0, st>>>(s);
  }
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

// ---------------------------------------------------------------------------
// One whole SSPRK3 or RK4 step per kernel (temporal blocking).  A block owns an
// FTX x FTY tile of the output; it stages the step's input over the tile plus a halo
// of NST cells (one per stage: every stage's 5-point stencil eats one ring) in shared
// memory and runs the stages there, each over the region its successors still need,
// so that the step reads the state once and writes it once (8 B per point and field in
// FP32 instead of the 64 B of four separate RK4 stage passes).  The stage formulas are
// those of the separate passes (add_step) compiled in per method, with the buffers in
// shared memory: 0 step input, 1 and 2 the stage ping-pong, 3 the RK4 running sum (kept
// on the tile only, where the last stage reads it).
// Periodic halos wrap; for Dirichlet and Neumann fields the ring of ghost cells just
// outside the domain is refilled from the BC formula after every stage, and cells
// further out are never read by a domain point.
enum { FTX = 64, FTY = 32, FOUT = -2 };

template <typename T>
struct XFused {
  XModel m;
  XCoef<T> k;
  const T* in;
  T* out;
  int nst;     // 3: SSPRK3, 4: RK4 (the stage formulas are compiled in per method)
  int any_bc;  // some field is Dirichlet or Neumann
};

// periodic index: one add or subtract within a halo of the domain, a remainder beyond
__device__ __forceinline__ int xwrap(int v, int n) {
  v = v < 0 ? v + n : (v >= n ? v - n : v);
  return (v >= 0 && v < n) ? v : ((v % n) + n) % n;
}

enum { FTHREADS = 512 };

// one region cell of the step input: a wrapped periodic cell, a domain cell, a ghost of
// the ring (the BC formula on its adjacent domain cell) or an unused outer cell (0)
template <typename T>
__device__ __forceinline__ long long fcell_src(int gy, int gx, const XModel& m, int kind, int* side) {
  const int ny = m.ny, nx = m.nx;
  *side = -1;
  if (kind == MJX_BC_PERIODIC) return (long long)xwrap(gy, ny) * nx + xwrap(gx, nx);
  const bool iny = gy >= 0 && gy < ny, inx = gx >= 0 && gx < nx;
  if (iny && inx) return (long long)gy * nx + gx;
  if (iny && (gx == -1 || gx == nx)) { *side = gx < 0 ? 0 : 1; return (long long)gy * nx + (gx < 0 ? 0 : nx - 1); }
  if (inx && (gy == -1 || gy == ny)) { *side = gy < 0 ? 2 : 3; return (long long)(gy < 0 ? 0 : ny - 1) * nx + gx; }
  *side = 4;
  return -1;
}

template <typename T, int RX, int NF, int NST>
__global__ void __launch_bounds__(FTHREADS, (sizeof(T) * NF <= 8) ? 2 : 1)
fused_step_kernel(const __grid_constant__ XFused<T> a) {
  extern __shared__ __align__(16) unsigned char fsm_raw[];
  T* sm = reinterpret_cast<T*>(fsm_raw);
  const XModel& m = a.m;
  const XCoef<T>& k = a.k;
  constexpr int R = NST, RW = FTX + 2 * R, RH = FTY + 2 * R, RS = RW * RH;
  constexpr int NL = (RS + FTHREADS - 1) / FTHREADS;
  const int nf = m.nf, ny = m.ny, nx = m.nx, adv = m.advection;
  const long long per = (long long)ny * nx;
  const int ntx = (nx + FTX - 1) / FTX;
  const int ty = blockIdx.x / ntx, tx = blockIdx.x - ty * ntx;
  const int X0 = tx * FTX - R, Y0 = ty * FTY - R;  // domain coordinates of region cell (0, 0)
  const int tid = threadIdx.x;
  const T h = k.hfixed;
  const T idx2 = k.idx2, idy2 = k.idy2, idx = k.idx, idy = k.idy, vx = k.vx, vy = k.vy;
  const bool vxpos = k.vxpos != 0, vypos = k.vypos != 0;
  auto buf = [&](int b, int f) -> T* { return sm + (size_t)(b * NF + f) * RS; };

  // 1. the step input over the region: all loads of a thread are issued before any store
  {
    T v[NL][NF];
#pragma unroll
    for (int j = 0; j < NL; ++j) {
      const int i = tid + j * FTHREADS;
      const int ry = i / RW, rx = i - ry * RW;
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        v[j][f] = (T)0;
        if (f >= nf || i >= RS) continue;
        int side;
        const long long si = fcell_src<T>(Y0 + ry, X0 + rx, m, m.kind[f], &side);
        if (si >= 0) v[j][f] = a.in[f * per + si];
      }
    }
#pragma unroll
    for (int j = 0; j < NL; ++j) {
      const int i = tid + j * FTHREADS;
      if (i >= RS) continue;
      const int ry = i / RW, rx = i - ry * RW;
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        if (f >= nf) break;
        int side;
        const int kind = m.kind[f];
        (void)fcell_src<T>(Y0 + ry, X0 + rx, m, kind, &side);
        T x = v[j][f];
        if (side >= 0 && side < 4) x = xghost(x, kind, k.gv[f][side], side == 0 || side == 2);
        buf(0, f)[i] = x;
      }
    }
  }
  __syncthreads();

  // stage constants of add_step's SSPRK3 (NST 3) and RK4 (NST 4) tables, in the state type
  const T h2 = (T)0.5 * h, h3 = (T)(1.0 / 3.0) * h, h6 = (T)(1.0 / 6.0) * h;
  const T c75 = (T)0.75, c25 = (T)0.25, h25 = (T)0.25 * h;
  const T c13 = (T)(1.0 / 3.0), c23 = (T)(2.0 / 3.0), h23 = (T)(2.0 / 3.0) * h;
#pragma unroll
  for (int s = 0; s < NST; ++s) {
    const int lo = s + 1;
    const int SW = RW - 2 * lo, SH = RH - 2 * lo;  // this stage's output region (compile time)
    // stage input: buffer 0 (step input), then 1, 2, 1 (RK4) or 1, 2 (SSPRK3); output the
    // other ping-pong buffer, the RK4 running sum in buffer 3, the last stage to global
    const int wb = s == 0 ? 0 : (s == 2 ? 2 : 1);
    const int o1b = s == NST - 1 ? FOUT : (s == 1 ? 2 : 1);
    // cells in pairs (rx, rx + 1) from an even column (64-bit shared-memory accesses; RW and
    // every buffer offset are even): when lo is odd the pairs start one column left of the
    // region and may end one right of it; those extra cells are read by no later stage and
    // write no output (the global store is limited to the tile)
    const int x0 = lo & ~1;
    const int SWP = (RW - lo - x0 + 1) >> 1;
    typedef typename Vec16<T>::t V16;
    typedef typename std::conditional<sizeof(T) == 4, float2, double2>::type T2;
    (void)sizeof(V16);
    for (int i = tid; i < SWP * SH; i += FTHREADS) {
      const int sy = i / SWP, sp = i - sy * SWP;
      const int ry = sy + lo, rx = x0 + 2 * sp;
      const int gy = Y0 + ry, gx = X0 + rx;
      const int c0 = ry * RW + rx;
      // the running sum is read only on the tile (the last stage's region)
      const bool rin = ry >= R && ry < R + FTY;
      const bool t0 = rin && rx >= R && rx < R + FTX, t1 = rin && rx + 1 >= R && rx + 1 < R + FTX;
      T c[NF][2], Fv[NF][2];
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        if (f >= nf) break;
        const T* wv = buf(wb, f);
        const T2 cc = *reinterpret_cast<const T2*>(wv + c0);
        const T2 up = *reinterpret_cast<const T2*>(wv + c0 - RW);
        const T2 dn = *reinterpret_cast<const T2*>(wv + c0 + RW);
        const T xl = wv[c0 - 1], xr = wv[c0 + 2];
        const T cvs[2] = {cc.x, cc.y}, xms[2] = {xl, cc.x}, xps[2] = {cc.y, xr};
        const T yms[2] = {up.x, up.y}, yps[2] = {dn.x, dn.y};
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const T cv = cvs[q], xm = xms[q], xp = xps[q], ym = yms[q], yp = yps[q];
          T v = k.D[f] * ((xp - (T)2 * cv + xm) * idx2 + (yp - (T)2 * cv + ym) * idy2);
          if (adv == 1) {  // d1_upwind_2d
            const T gxv = vxpos ? (cv - xm) * idx : (xp - cv) * idx;
            const T gyv = vypos ? (cv - ym) * idy : (yp - cv) * idy;
            v = v - vx * gxv - vy * gyv;
          } else if (adv == 2) {
            v = v - vx * (xp - xm) * (T)0.5 * idx - vy * (yp - ym) * (T)0.5 * idy;
          }
          c[f][q] = cv;
          Fv[f][q] = v;
        }
      }
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        if (RX == RX_GRAY_SCOTT) {  // operators.py:644-667
          const T uvv = c[0][q] * c[1][q] * c[1][q];
          Fv[0][q] += -uvv + k.F * ((T)1 - c[0][q]);
          Fv[1][q] += uvv - k.Fk * c[1][q];
        } else if (RX == RX_FISHER) {  // operators.py:680-705
#pragma unroll
          for (int f = 0; f < NF; ++f) {
            if (f >= nf) break;
            Fv[f][q] += k.r * c[f][q] * ((T)1 - c[f][q]);
          }
        }
      }
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        if (f >= nf) break;
        T o1[2];
        if (NST == 4) {  // rk4_step (stepping.py:126-163), running sum in buffer 3
          T* acc = buf(3, f);
          const T2 av = *reinterpret_cast<const T2*>(acc + c0);
          const T avs[2] = {av.x, av.y};
          if (s == 3) {
#pragma unroll
            for (int q = 0; q < 2; ++q) o1[q] = avs[q] + h6 * Fv[f][q];
          } else {
            const T2 yv = *reinterpret_cast<const T2*>(buf(0, f) + c0);
            const T ys[2] = {yv.x, yv.y};
            T an[2];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
              o1[q] = ys[q] + (s == 2 ? h : h2) * Fv[f][q];
              an[q] = s == 0 ? ys[q] + h6 * Fv[f][q] : avs[q] + h3 * Fv[f][q];
            }
            if (t0 && t1) {
              T2 w2;
              w2.x = an[0];
              w2.y = an[1];
              *reinterpret_cast<T2*>(acc + c0) = w2;
            } else {
              if (t0) acc[c0] = an[0];
              if (t1) acc[c0 + 1] = an[1];
            }
          }
        } else {  // ssprk3_step (stepping.py:87-123), Shu-Osher form
          const T2 yv = *reinterpret_cast<const T2*>(buf(0, f) + c0);
          const T ys[2] = {yv.x, yv.y};
#pragma unroll
          for (int q = 0; q < 2; ++q)
            o1[q] = s == 0 ? ys[q] + h * Fv[f][q]
                           : (s == 1 ? c75 * ys[q] + c25 * c[f][q] + h25 * Fv[f][q]
                                     : c13 * ys[q] + c23 * c[f][q] + h23 * Fv[f][q]);
        }
        if (o1b == FOUT) {
          T* orow = a.out + f * per + (long long)gy * nx;
          if (gy < ny) {
            if (t0 && gx < nx) orow[gx] = o1[0];
            if (t1 && gx + 1 < nx) orow[gx + 1] = o1[1];
          }
        } else {
          T2 w2;
          w2.x = o1[0];
          w2.y = o1[1];
          *reinterpret_cast<T2*>(buf(o1b, f) + c0) = w2;
        }
      }
    }
    if (s + 1 < NST) {
      __syncthreads();
      if (a.any_bc) {  // the ghost ring of the new stage values
        for (int i = tid; i < SW * SH; i += FTHREADS) {
          const int sy = i / SW, sx = i - sy * SW;
          const int ry = sy + lo, rx = sx + lo;
          const int gy = Y0 + ry, gx = X0 + rx;
          const bool iny = gy >= 0 && gy < ny, inx = gx >= 0 && gx < nx;
          const bool gxr = iny && (gx == -1 || gx == nx), gyr = inx && (gy == -1 || gy == ny);
          if (!gxr && !gyr) continue;
          const int c0 = ry * RW + rx;
          // the adjacent domain cell lies one step inward, inside this stage's region
          const int cin = gxr ? (gx < 0 ? c0 + 1 : c0 - 1) : (gy < 0 ? c0 + RW : c0 - RW);
#pragma unroll
          for (int f = 0; f < NF; ++f) {
            if (f >= nf) break;
            const int kind = m.kind[f];
            if (kind == MJX_BC_PERIODIC) continue;
            T* ob = buf(o1b, f);
            ob[c0] = gxr ? xghost(ob[cin], kind, gx < 0 ? k.gv[f][0] : k.gv[f][1], gx < 0)
                         : xghost(ob[cin], kind, gy < 0 ? k.gv[f][2] : k.gv[f][3], gy < 0);
          }
        }
        __syncthreads();
      }
    }
  }
}

template <typename T>
static size_t fused_smem(int nst, int nfa) {
  const int nbuf = nst == 4 ? 4 : 3;
  return (size_t)nbuf * nfa * (FTX + 2 * nst) * (FTY + 2 * nst) * sizeof(T);
}

// whether a fused step of `method` fits the shared memory of a block
template <typename T>
static bool fused_ok(const XModel& m, int method) {
  if (method != 1 && method != 2) return false;
  if (m.reaction == MJX_REACT_KINETICS) return false;  // the stage kernels take the network
  const int nfa = m.nf <= 2 ? 2 : 4;
  return fused_smem<T>(method == 2 ? 4 : 3, nfa) <= 200 * 1024;
}

template <typename T, int RX, int NF, int NST>
static cudaError_t launch_fused_t(const XFused<T>& f, size_t smem, unsigned blocks, cudaStream_t s) {
  // the dynamic shared-memory limit is a function attribute of the CUDA context: set it
  // once for each context this instantiation runs in
  static ContextOnce attr;
  cudaError_t e = cudaSuccess;
  const mjx_status st = attr.run([&]() -> mjx_status {
    e = cudaFuncSetAttribute(fused_step_kernel<T, RX, NF, NST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return e == cudaSuccess ? MJX_OK : MJX_CUDA_ERROR;
  });
  if (st != MJX_OK) return e != cudaSuccess ? e : cudaErrorDeviceUninitialized;
  fused_step_kernel<T, RX, NF, NST><<<blocks, FTHREADS, smem, s>>>(f);
  return cudaGetLastError();
}

template <typename T, int RX>
static cudaError_t launch_fused_rx(const XFused<T>& f, cudaStream_t s) {
  const int nfa = f.m.nf <= 2 ? 2 : 4;
  const size_t smem = fused_smem<T>(f.nst, nfa);
  const unsigned blocks = (unsigned)(((f.m.nx + FTX - 1) / FTX) * ((f.m.ny + FTY - 1) / FTY));
  if constexpr (RX == RX_GRAY_SCOTT) {  // two fields only
    return f.nst == 4 ? launch_fused_t<T, RX, 2, 4>(f, smem, blocks, s) : launch_fused_t<T, RX, 2, 3>(f, smem, blocks, s);
  } else {
    if (f.nst == 4) {
      return nfa == 2 ? launch_fused_t<T, RX, 2, 4>(f, smem, blocks, s) : launch_fused_t<T, RX, 4, 4>(f, smem, blocks, s);
    }
    return nfa == 2 ? launch_fused_t<T, RX, 2, 3>(f, smem, blocks, s) : launch_fused_t<T, RX, 4, 3>(f, smem, blocks, s);
  }
}

template <typename T>
static cudaError_t launch_fused(const XFused<T>& f, cudaStream_t s) {
  if (f.m.reaction == MJX_REACT_GRAY_SCOTT) return launch_fused_rx<T, RX_GRAY_SCOTT>(f, s);
  if (f.m.reaction == MJX_REACT_FISHER) return launch_fused_rx<T, RX_FISHER>(f, s);
  return launch_fused_rx<T, RX_NONE>(f, s);
}

// the fused step of `method` (1 SSPRK3, 2 RK4; in / out set per step)
template <typename T>
static XFused<T> make_fused(const XModel& m, int method, double dt) {
  XStage<T> s0;
  memset(&s0, 0, sizeof(s0));
  s0.m = m;
  s0.hfixed = dt;
  s0.hfac = 1.0;
  x_coef(s0);
  XFused<T> f;
  memset(&f, 0, sizeof(f));
  f.m = m;
  f.k = s0.k;
  f.nst = method == 2 ? 4 : 3;
  for (int q = 0; q < m.nf; ++q) f.any_bc |= m.kind[q] != MJX_BC_PERIODIC;
  return f;
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
  A.rx = rx_of(m.reaction);
  MJX_CUDA_TRY(cudaMemcpyAsync(base.buf[0], y0, nelem * sizeof(T), cudaMemcpyDeviceToDevice, s));
  int src = 0;
  if (fused_ok<T>(m, method)) {  // SSPRK3 / RK4: one kernel per step
    XFused<T> f = make_fused<T>(m, method, dt);
    for (int step = 0; step < n_steps; ++step) {
      f.in = base.buf[src];
      f.out = base.buf[1 - src];
      const cudaError_t e = launch_fused<T>(f, s);
      if (e != cudaSuccess) { set_last_error(e, __FILE__, __LINE__); return MJX_CUDA_ERROR; }
      src = 1 - src;
    }
    MJX_CUDA_TRY(cudaMemcpyAsync(y_out, base.buf[src], nelem * sizeof(T), cudaMemcpyDeviceToDevice, s));
    return MJX_OK;
  }
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
  const int rx = rx_of(m.reaction);
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

// Autotuner of the stencil stage's tile height: one RK4 middle stage (stage input,
// step start and running sum read; two outputs) of the problem is timed for strips of
// 2, 4, 8, 16 and 32 rows per warp and, for FP32 with 16-byte rows, the TMA-staged form
// (one warm-up launch, then reps launches between CUDA events) on the workspace
// buffers, and the fastest is installed for this grid size, field count and element size.
template <typename T>
static mjx_status tune_stencil(const XModel& m, char* ws, const XLayout& L, int reps, double* times, int max_times,
                               int* best_rows, cudaStream_t s) {
  static const int cand[6] = {2, 4, 8, 16, 32, XT_TMA_ROWS};
  XStage<T> st;
  memset(&st, 0, sizeof(st));
  st.m = m;
  for (int i = 0; i < 7; ++i) st.buf[i] = (T*)(ws + L.b[i]);
  st.w = XB_W1; st.p = XB_YCUR; st.q = XB_ACC; st.o1 = XB_W2; st.o2 = XB_ACC;
  st.cp1 = 1; st.cf1 = 0.5; st.cq2 = 1; st.cf2 = 1.0 / 3.0;
  st.hfac = 1.0; st.hfixed = 1e-6;
  const int rx = rx_of(m.reaction);
  cudaEvent_t e0, e1;
  MJX_CUDA_TRY(cudaEventCreate(&e0));
  MJX_CUDA_TRY(cudaEventCreate(&e1));
  double best_t = 1e300;
  int bi = -1;
  cudaError_t ce = cudaSuccess;
  const int ncand = x_tma_able(st) ? 6 : 5;  // the TMA form: FP32 with aligned 16-byte rows
  for (int i = 0; i < ncand && ce == cudaSuccess; ++i) {
    st.rows = cand[i];
    ce = launch_stage<T>(st, rx, s);
    if (ce == cudaSuccess) ce = cudaEventRecord(e0, s);
    for (int r = 0; r < reps && ce == cudaSuccess; ++r) ce = launch_stage<T>(st, rx, s);
    if (ce == cudaSuccess) ce = cudaEventRecord(e1, s);
    if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
    if (ce != cudaSuccess) break;
    const double tpl = (double)ms / reps;
    if (times && i < max_times) times[i] = tpl;
    if (tpl < best_t) { best_t = tpl; bi = i; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ce != cudaSuccess) { set_last_error(ce, __FILE__, __LINE__); return MJX_CUDA_ERROR; }
  tune_rows_put(m.ny, m.nx, m.nf, (int)sizeof(T), cand[bi]);
  if (best_rows) *best_rows = cand[bi];
  return MJX_OK;
}

mjx_status mjx_autotune_stencil2d(const mjx_grid2d* grid, int dtype, const mjx_explicit_problem* prob, void* ws,
                                  size_t ws_bytes, int reps, double* times, int max_times, int* best_rows,
                                  void* stream) {
  XModel m;
  MJX_TRY(x_model(prob, grid, &m));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (reps < 1) return MJX_BAD_ARG;
  const XLayout L = x_layout(m.nf, m.ny, m.nx, e);
  if (ws == nullptr || ws_bytes < L.total) return MJX_WORKSPACE;
  cudaStream_t s = (cudaStream_t)stream;
  MJX_CUDA_TRY(cudaMemsetAsync(ws, 0, L.part, s));  // the state buffers: finite values to time on
  if (e == 4) return tune_stencil<float>(m, (char*)ws, L, reps, times, max_times, best_rows, s);
  return tune_stencil<double>(m, (char*)ws, L, reps, times, max_times, best_rows, s);
}
