// Spectral multipliers on periodic 3D boxes: u <- real(ifftn(m(k) fftn(u))), applied
// n_steps times, each a full forward and inverse transform as the 3D FFT-CN of
// benchmarks/sisc/bench_3d_feasibility.py:71-87 (cn_step_3d inside a fori_loop).
//
// Layout: real u[nz][ny][nx]; half spectrum S[nz][ny][ldc] (ldc = spec_ldc(nx)).
// One application is five passes over HBM:
//   X   r2c of every (z, y) row (rows r and r + nz*ny/2 share one complex FFT)
//   Y   forward FFT along y, one plane per gridDim.z
//   Z   forward FFT along z -> m(lamx + lamy + lamz) / (nx ny nz) -> inverse FFT along z;
//       the "columns" are the ny*ldc points of one z-plane, row stride ny*ldc
//   Y'  inverse FFT along y
//   X'  c2r
// The plan is two 2D plans: (ny, nx) for the x twiddles and the x / y symbols, and
// (nz, nx) whose "y" tables serve z.
#include <string.h>

#include "spectral.cuh"

namespace mjx {

void set_last_error(cudaError_t e, const char* file, int line);
mjx_status ensure_kernel_attrs();
int elem_size(int dtype);

static inline size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

static mjx_status check_grid3(const mjx_grid3d* g) {
  if (g == nullptr) return MJX_BAD_ARG;
  if (ilog2_exact(g->nx) < 1 || ilog2_exact(g->ny) < 1 || ilog2_exact(g->nz) < 1) return MJX_BAD_SHAPE;
  if (g->nx > 4096 || g->ny > 4096 || g->nz > 4096) return MJX_BAD_SHAPE;
  if (!(g->dx > 0) || !(g->dy > 0) || !(g->dz > 0)) return MJX_BAD_ARG;
  // the z pass indexes columns of one plane with int
  if ((long long)g->ny * spec_ldc(g->nx) > (1LL << 30)) return MJX_BAD_SHAPE;
  return MJX_OK;
}

template <typename T>
static mjx_status apply3d(const void* plan, const mjx_grid3d* g, double D, double h, int mult, int n_steps,
                          const T* in, T* out, void* ws, cudaStream_t s) {
  const int nx = g->nx, ny = g->ny, nz = g->nz, ldc = spec_ldc(nx);
  const PlanView pa = plan_view(plan, ny, nx, sizeof(T));
  const PlanView pz = plan_view((const char*)plan + al256(plan_bytes(ny, nx, sizeof(T))), nz, nx, sizeof(T));
  cx<T>* spec = (cx<T>*)ws;
  const long long plane = (long long)ny * ldc;
  const int rows = nz * ny;

  RowArgs<T> r;
  memset(&r, 0, sizeof(r));
  r.n = nx; r.log2n = ilog2_exact(nx); r.ldc = ldc; r.nrows = rows / 2; r.npairs = 1;
  r.nseq = row_nseq(nx, r.nrows); r.rstride = nx; r.rin_sel = -1; r.rout_sel = -1;
  r.spec = spec; r.tw = (const cx<T>*)pa.twx; r.inv_scale = (T)1;
  r.pr[0].ra = 0; r.pr[0].rb = (long long)(rows / 2) * nx;
  r.pr[0].sa = 0; r.pr[0].sb = (long long)(rows / 2) * ldc;
  r.pr[0].hfac = 1.0;
  RowArgs<T> rf = r, rb = r;
  rf.rin[0] = in; rf.pr[0].flags = ROW_STORE_SPEC;
  rb.rout[0] = out; rb.pr[0].flags = ROW_LOAD_SPEC | ROW_STORE_REAL;

  ColArgs<T> cy;
  memset(&cy, 0, sizeof(cy));
  cy.ny = ny; cy.log2ny = ilog2_exact(ny); cy.ncols = nx / 2 + 1; cy.ldc = ldc;
  cy.C = col_tile(ny, cy.ncols, 1, sizeof(T));
  cy.spec = spec; cy.lamx = (const T*)pa.lamx; cy.lamy = (const T*)pa.lamy; cy.tw = (const cx<T>*)pa.twy;
  cy.scale = (T)1; cy.njobs = 1; cy.pstride = plane; cy.nplanes = nz; cy.hfixed = h;
  cy.job[0].nout = 1; cy.job[0].mul = MUL_SCALE; cy.job[0].scale = 1.0; cy.job[0].hfac[0] = 1.0;
  cy.job[0].pow[0] = 1;
  ColArgs<T> cyf = cy, cyb = cy;
  cyf.job[0].dirs = 1;
  cyb.job[0].dirs = 2;

  ColArgs<T> cz;
  memset(&cz, 0, sizeof(cz));
  cz.ny = nz; cz.log2ny = ilog2_exact(nz); cz.ncols = (int)plane; cz.ldc = (int)plane;
  cz.C = col_tile(nz, cz.ncols, 1, sizeof(T));
  cz.spec = spec; cz.lamx = (const T*)pa.lamx; cz.lamy2 = (const T*)pa.lamy; cz.lamy = (const T*)pz.lamy;
  cz.ldc3 = ldc; cz.tw = (const cx<T>*)pz.twy; cz.hfixed = h; cz.njobs = 1; cz.nplanes = 1;
  cz.scale = (T)(1.0 / ((double)nx * (double)ny * (double)nz));
  cz.job[0].nout = 1; cz.job[0].mul = mult; cz.job[0].D = D; cz.job[0].hfac[0] = 1.0; cz.job[0].pow[0] = 1;
  cz.job[0].dirs = 3;

  auto one = [&](const RowArgs<T>& first, cudaStream_t st) -> cudaError_t {
    cudaError_t e;
    if ((e = launch_row<T, RX_NONE>(first, st)) != cudaSuccess) return e;
    if ((e = launch_col<T>(cyf, st)) != cudaSuccess) return e;
    if ((e = launch_col<T>(cz, st)) != cudaSuccess) return e;
    if ((e = launch_col<T>(cyb, st)) != cudaSuccess) return e;
    return launch_row<T, RX_NONE>(rb, st);
  };
  MJX_CUDA_TRY(one(rf, s));
  if (n_steps > 1) {
    // later applications read the previous output: captured once, replayed
    RowArgs<T> rf2 = rf;
    rf2.rin[0] = out;
    cudaStream_t cs = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaError_t ce = cudaSuccess;
    do {
      if ((ce = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) break;
      if ((ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) break;
      const cudaError_t le = one(rf2, cs);
      ce = cudaStreamEndCapture(cs, &graph);
      if (le != cudaSuccess) { ce = le; break; }
      if (ce != cudaSuccess) break;
      if ((ce = cudaGraphInstantiate(&exec, graph, 0)) != cudaSuccess) break;
      for (int i = 1; i < n_steps && ce == cudaSuccess; ++i) ce = cudaGraphLaunch(exec, s);
    } while (0);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (cs) cudaStreamDestroy(cs);
    if (ce != cudaSuccess) { set_last_error(ce, __FILE__, __LINE__); return MJX_CUDA_ERROR; }
  }
  return MJX_OK;
}

}  // namespace mjx

using namespace mjx;

extern "C" {

size_t mjx_spec3d_plan_bytes(int nz, int ny, int nx, int dtype) {
  const int e = elem_size(dtype);
  if (!e || ilog2_exact(nx) < 1 || ilog2_exact(ny) < 1 || ilog2_exact(nz) < 1) return 0;
  return al256(plan_bytes(ny, nx, e)) + plan_bytes(nz, nx, e);
}

mjx_status mjx_spec3d_plan_init(void* plan, const mjx_grid3d* g, int symbol, int dtype, void* stream) {
  MJX_TRY(check_grid3(g));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!plan) return MJX_BAD_ARG;
  const mjx_grid2d a = {g->ny, g->nx, g->dy, g->dx};
  const mjx_grid2d z = {g->nz, g->nx, g->dz, g->dx};
  MJX_TRY(mjx_spec2d_plan_init(plan, &a, symbol, dtype, stream));
  return mjx_spec2d_plan_init((char*)plan + al256(plan_bytes(g->ny, g->nx, e)), &z, symbol, dtype, stream);
}

size_t mjx_spec3d_ws_bytes(int nz, int ny, int nx, int dtype) {
  const int e = elem_size(dtype);
  if (!e || ilog2_exact(nx) < 1 || ilog2_exact(ny) < 1 || ilog2_exact(nz) < 1) return 0;
  return (size_t)nz * ny * spec_ldc(nx) * 2 * e;
}

mjx_status mjx_spectral_apply3d(const void* plan, const mjx_grid3d* g, int dtype, double D, double h, int mult,
                                int n_steps, const void* in, void* out, void* ws, size_t ws_bytes,
                                void* stream) {
  MJX_TRY(check_grid3(g));
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!plan || !in || !out || n_steps < 1) return MJX_BAD_ARG;
  if ((mult < MJX_MULT_SCALE || mult > MJX_MULT_EXP) && mult != MJX_MULT_LAP) return MJX_BAD_ARG;
  if (!ws || ws_bytes < mjx_spec3d_ws_bytes(g->nz, g->ny, g->nx, dtype)) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4)
    return apply3d<float>(plan, g, D, h, mult, n_steps, (const float*)in, (float*)out, ws, s);
  return apply3d<double>(plan, g, D, h, mult, n_steps, (const double*)in, (double*)out, ws, s);
}

}  // extern "C"
