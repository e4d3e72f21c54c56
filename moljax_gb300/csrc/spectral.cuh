// Row and column spectral passes over 2D periodic fields (internal interface).
//
// Data layout in HBM (all interior-only, no ghost cells):
//   real field   f[y][x], row stride `rstride` elements, fields `fstride` apart
//   half spectrum S[ky][kx], kx in [0, nx/2], row stride ldc (complex elements)
// Two real rows (a, b) are packed as one complex row z = a + i b for every
// row transform ("pair"), which gives two real FFTs for the price of one.
#pragma once

#include "common.cuh"
#include "fft.cuh"

namespace mjx {

// Device-resident state of an adaptive run (lives in the caller's workspace).
struct DevState {
  double t, dt, dtc, t_end, prev_err, err_last, dt_cfl, dt_last_accepted;
  int cur, status, n_acc, n_rej, write_idx, attempts, done, finite;
  int max_saves, save_every, max_attempts, order;
  int save_slot, pad0, pad1, pad2;
};

enum { MJX_MAXPAIR = 8, MJX_MAXJOB = 8 };

// moljax StatusCode values (moljax/core/utils.py:265-272), kept in DevState.status
enum {
  MJX_STATUS_SUCCESS_CODE = 0,
  MJX_STATUS_RUNNING_CODE = 1,
  MJX_STATUS_MAX_STEPS_CODE = 2,
  MJX_STATUS_DT_TOO_SMALL_CODE = 3,
  MJX_STATUS_NON_FINITE_CODE = 4,
  MJX_STATUS_NK_FAILED_CODE = 5
};

// per-pair runtime flags of a row pass
enum {
  ROW_LOAD_SPEC = 1,   // input is a half spectrum (c2r first); else real rows
  ROW_STORE_REAL = 2,  // store the real rows (after the pointwise op)
  ROW_REACT = 4,       // Heun reaction step of length hfac*dt on (a, b)
  ROW_STORE_SPEC = 8,  // r2c at the end and store the half spectrum
  ROW_ERRNORM = 16,    // accumulate the scaled error of (a, b) against eref
  ROW_DELTA = 32,      // with ROW_REACT: keep only the reaction increment (new - old)
  ROW_ERRPAIR = 64,    // accumulate (a / (atol + rtol |b|))^2: a = error row, b = solution row
  ROW_NONLIN = 128,    // replace (a, b) by the reaction terms N(a, b) (exponential integrators)
  ROW_SPEC_ALT = 256,  // store the spectrum at (oa, ob) instead of (sa, sb)
  ROW_EULER = 512,     // with ROW_REACT: explicit Euler reaction step instead of Heun
  ROW_EULER2 = 1024,   // with ROW_EULER: a second Euler step of the same length after the first
};

// pointwise reaction kinds (compile-time)
enum { RX_NONE = 0, RX_GRAY_SCOTT = 1, RX_FISHER = 2, RX_LINEAR = 3, RX_KINETICS = 4 };

// The Heun increment y** - y* computed without forming y** (no cancellation).
template <typename T, int RX>
__device__ __forceinline__ void react_delta(T& a, T& b, T h, T F, T k, T r) {
  const T hh = (T)0.5 * h;
  if (RX == RX_GRAY_SCOTT) {
    const T uvv = a * b * b;
    const T fu = -uvv + F * ((T)1 - a);
    const T fv = uvv - (F + k) * b;
    const T ua = a + h * fu, va = b + h * fv;
    const T uvv2 = ua * va * va;
    const T gu = -uvv2 + F * ((T)1 - ua);
    const T gv = uvv2 - (F + k) * va;
    a = hh * (fu + gu);
    b = hh * (fv + gv);
  } else if (RX == RX_FISHER) {
    const T fa = r * a * ((T)1 - a), fb = r * b * ((T)1 - b);
    const T ta = a + h * fa, tb = b + h * fb;
    a = hh * (fa + r * ta * ((T)1 - ta));
    b = hh * (fb + r * tb * ((T)1 - tb));
  } else {
    a = (T)0;
    b = (T)0;
  }
}

struct RowPair {
  long long ra, rb;    // real row offsets (elements) of rows a and b at y = 0
  long long sa, sb;    // spectrum offsets (complex elements) at ky = 0
  long long oa, ob;    // output spectrum offsets with ROW_SPEC_ALT
  double hfac;         // reaction step = hfac * (dt from state, or hfixed)
  int flags;
  int pad;
};

template <typename T> struct RowArgs {
  int n, log2n, ldc, nrows, npairs, nseq;
  long long rstride;
  const T* rin[2];     // real input bases; rin_sel: -1 -> rin[0], 0 -> rin[cur], 1 -> rin[1-cur]
  T* rout[2];
  int rin_sel, rout_sel;
  const T* eref;       // error reference base (same offsets as the real output)
  cx<T>* spec;         // spectrum base (read and/or written in place)
  const cx<T>* tw;     // twiddles for n
  T inv_scale;         // scale applied after the inverse transform
  double hfixed;       // reaction step when st == nullptr
  double F, k, r;      // reaction parameters
  double atol, rtol;
  double* partial;     // per-CTA error partial sums (ROW_ERRNORM)
  int* nonfinite;      // per-CTA non-finite flags (ROW_ERRNORM)
  const DevState* st;
  RowPair pr[MJX_MAXPAIR];
};

enum { MUL_SCALE = 0, MUL_HELMHOLTZ = 1, MUL_CN = 2, MUL_EXP = 3, MUL_ADVDIFF = 4, MUL_LAP = 5,
       MUL_ADV_LAP = 6,   // h (D lam - i v.k): the advection-diffusion operator itself
       MUL_ADV_EXP = 7,   // exp(h (D lam - i v.k))
       MUL_TABLE = 8,     // a real multiplier per half-spectrum point (ColArgs::mtab)
       MUL_ADV_CN = 9 };  // (1 + z/2)/(1 - z/2), z = h (D lam - i v.k): one Crank-Nicolson step

struct ColJob {
  long long sin;         // spectrum offset of the input column block (ky=0, kx=0)
  long long sout[2];     // outputs (may equal sin)
  double D;              // diffusivity of this field
  double hfac[2];        // step = hfac * dt
  int pow[2];            // multiplier power (1 or 2)
  int nout;
  int mul;               // MUL_*
  int dirs;              // bit 0: forward transform first, bit 1: inverse after (0 means both)
  double scale;          // multiplier scale (0: use ColArgs::scale)
  double vx, vy;         // MUL_ADVDIFF: advection velocity of this field
};

template <typename T> struct ColArgs {
  int ny, log2ny, ncols, ldc, C, njobs;
  cx<T>* spec;
  const T* lamx;         // symbol along x, length ldc (kx = 0..nx/2)
  const T* lamy;         // symbol along y, length ny (fftfreq order)
  const cx<T>* tw;       // twiddles for ny
  T scale;               // normalisation 1/(nx*ny)
  double kxs, kys;       // MUL_ADVDIFF: wavenumber units 2 pi/(nx dx), 2 pi/(ny dy)
  double hfixed;
  const DevState* st;
  // 3D grids: gridDim.z planes pstride complex elements apart; in the z pass (ldc3 > 0)
  // column c is (ky, kx) = (c / ldc3, c % ldc3) and lam = lamx[kx] + lamy2[ky] + lamy[row]
  long long pstride;
  int nplanes;
  int ldc3;
  const T* lamy2;
  const T* mtab;         // MUL_TABLE: [ny][ldc] real multipliers
  // odd extension along the column: rows ky >= ny/2 are not stored; they are loaded as
  // the negated mirror -row(ny-1-ky) and only rows ky < ny/2 are written back (the
  // cell-centred odd extension of a Dirichlet DST-II solve)
  int oddy;
  ColJob job[MJX_MAXJOB];
};

// Plan layout (device bytes): twx[nx] twy[ny] lamx[ldc] lamy[ny], 256-byte aligned parts;
// FP32 plans of 1024-point rows hold 2048 x twiddles (the second half transposed, wfft.cuh).
struct PlanView {
  const void* twx; const void* twy; const void* lamx; const void* lamy;
};
size_t plan_bytes(int ny, int nx, int elem);
PlanView plan_view(const void* plan, int ny, int nx, int elem);
int spec_ldc(int nx);

template <typename T, int RX>
cudaError_t launch_row(const RowArgs<T>& a, cudaStream_t s);
template <typename T>
cudaError_t launch_col(const ColArgs<T>& a, cudaStream_t s);

// Arguments of the adaptive controller kernel (csrc/imex.cu).
struct CtlArgs {
  DevState* st;
  const double* partial;
  const int* nonfinite;
  int nparts;
  double n_dof;
  mjx_pid_params pid;
  double* hist_t;
  double* hist_dt;
  cudaGraphConditionalHandle handle;
  int use_handle;
};
cudaError_t launch_controller(const CtlArgs& a, cudaStream_t s);
int col_tile(int ny, int ncols, int nout, int elem);

// Adaptive-loop driver selection.  The default keeps the whole loop on the
// device (a CUDA graph whose conditional while node repeats attempt +
// controller).  With MJX_HOST_LOOP=1 in the environment the host launches the
// attempts itself, in batches, and reads the done flag between batches:
// profilers that cannot see kernels inside conditional graphs (Nsight Compute)
// then see every launch.  Results are identical: every attempt kernel returns
// at once when the state is done, so the attempts after the end of a batch do
// nothing.
bool host_loop_mode();

// Host-driven loop: launch_attempt(stream) enqueues one attempt and its
// controller (no conditional handle).  At most max_attempts + batch attempts
// are launched; the controller ends the run at max_attempts.
template <typename F>
cudaError_t run_host_loop(F&& launch_attempt, const DevState* st, int max_attempts, cudaStream_t s) {
  const int batch = 32;
  int done = 0;
  for (long long launched = 0; !done && launched <= (long long)max_attempts + batch; launched += batch) {
    for (int k = 0; k < batch; ++k) {
      const cudaError_t e = launch_attempt(s);
      if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaMemcpyAsync(&done, &st->done, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Row-pass CTA geometry helpers (sequences per CTA and CTA count).
int row_nseq(int n, int nrows);
int row_ctas(int n, int nrows, int npairs);

}  // namespace mjx
