/*
 * moljax_gb300 -- C ABI of the GB300 (sm_103a) method-of-lines step path.
 *
 * Every entry point takes plain device pointers, sizes, host-side parameter
 * structs and a CUDA stream handle (passed as void*; NULL = legacy default
 * stream).  The caller owns all device memory: plans (twiddle and symbol
 * tables) and workspaces are caller-provided buffers whose sizes come from
 * the *_bytes() queries, so no step call allocates device memory.
 * Numerical failure is reported through status codes (never a device trap).
 *
 * Layout: fields are interior-only (no ghost cells), row-major [ny][nx] with
 * y on axis 0 (the reference's convention), several fields stored back to
 * back ([nfields][ny][nx]).  dtype MJX_F32 or MJX_F64 for every buffer.
 *
 * Each function names the reference (gogipav14/moljax) interface it replaces.
 */
#ifndef MOLJAX_GB300_H
#define MOLJAX_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mjx_status {
  MJX_OK = 0,
  MJX_BAD_SHAPE = 1,     /* unsupported or inconsistent sizes */
  MJX_BAD_DTYPE = 2,
  MJX_NOT_FINITE = 3,    /* moljax StatusCode.NON_FINITE_VALUES */
  MJX_MAX_ITERS = 4,     /* moljax StatusCode.MAX_STEPS_REACHED */
  MJX_DT_TOO_SMALL = 5,  /* moljax StatusCode.DT_TOO_SMALL */
  MJX_NK_FAILED = 6,     /* moljax StatusCode.NK_FAILED */
  MJX_OOM = 7,
  MJX_CUDA_ERROR = 8,
  MJX_BAD_ARG = 9,
  MJX_WORKSPACE = 10     /* workspace smaller than the *_bytes() query */
} mjx_status;

typedef enum mjx_dtype { MJX_F32 = 0, MJX_F64 = 1 } mjx_dtype;

/* Periodic Laplacian eigenvalues: FD 5-point symbol (moljax/core/fft_solvers.py:124-154)
 * or pseudo-spectral -(kx^2+ky^2) (benchmarks/benchmark_vs_scipy.py:77-80). */
typedef enum mjx_symbol { MJX_SYMBOL_FD = 0, MJX_SYMBOL_SPECTRAL = 1 } mjx_symbol;
/* OR-ed into an ETD symbol: the symbol has no y part, so each grid row is an
 * independent periodic 1D problem (moljax's 1D DiffusionOperator, fft_operators.py:80-176). */
#define MJX_SYMBOL_X_ONLY 0x10

/* Spectral multipliers applied between forward and inverse transform. */
typedef enum mjx_mult {
  MJX_MULT_SCALE = 0,      /* identity (round trip) */
  MJX_MULT_HELMHOLTZ = 1,  /* 1/(1 - h D lam), |denominator| clamped at 1e-14 */
  MJX_MULT_CN = 2,         /* (1 + h D lam/2)/(1 - h D lam/2) */
  MJX_MULT_EXP = 3,        /* exp(h D lam) */
  MJX_MULT_LAP = 5,        /* h D lam (the operator itself, DiffusionOperator.matvec) */
  /* general-size path only (mjx_spectral_apply_general2d), z = h (D lam - i (vx kx + vy ky)): */
  MJX_MULT_ADV_SOLVE = 16, /* 1/(1 - z), |1 - z| clamped at 1e-14 */
  MJX_MULT_ADV_LAP = 17,   /* z */
  MJX_MULT_ADV_EXP = 18,   /* exp(z) */
  MJX_MULT_ADV_CN = 20,    /* (1 + z/2)/(1 - z/2) */
  MJX_MULT_TABLE = 19      /* a real table [ny][nx] on the full spectrum */
} mjx_mult;

typedef enum mjx_reaction {
  MJX_REACT_NONE = 0,
  MJX_REACT_GRAY_SCOTT = 1, /* u: -uv^2 + F(1-u); v: uv^2 - (F+k)v  (operators.py:644-677) */
  MJX_REACT_FISHER = 2,     /* r u (1-u) on every field          (operators.py:680-705) */
  MJX_REACT_KINETICS = 3    /* a mass-action network (mjx_kinetics): the multispecies reaction
                               terms of make_reaction_op (operators.py:623-641) in native form */
} mjx_reaction;

/* Mass-action kinetics of up to 4 species (the fields, in order) and up to 8 reactions:
 *   dc_s/dt += source[s] + sum_j linear[s][j] c_j + sum_r stoich[r][s] rate[r] prod_q c_q^order[r][q]
 * First-order networks need only `linear`; a zeroth-order feed goes in `source`. */
#define MJX_KIN_MAXR 8
typedef struct mjx_kinetics {
  int nreactions;        /* 0..8 */
  int pad;
  int order[8][4];       /* reactant order of each species in each reaction, 0..3 */
  double rate[8];        /* rate constant of each reaction */
  double stoich[8][4];   /* net change of each species per reaction event (products - reactants) */
  double linear[4][4];   /* first-order rate matrix */
  double source[4];      /* zeroth-order source of each species */
} mjx_kinetics;

/* Ghost-cell BC kinds (moljax/core/bc.py:26-30 BCType). */
typedef enum mjx_bc_kind { MJX_BC_PERIODIC = 0, MJX_BC_DIRICHLET = 1, MJX_BC_NEUMANN = 2 } mjx_bc_kind;

typedef struct mjx_grid2d {
  int ny, nx;          /* interior points, powers of two in [2, 4096] */
  double dy, dx;
} mjx_grid2d;

typedef struct mjx_grid3d {
  int nz, ny, nx;      /* interior points, powers of two in [2, 4096]; arrays [nz][ny][nx] */
  int pad;
  double dz, dy, dx;
} mjx_grid3d;

/* moljax/core/dt_policy.py:49-78 (PIDParams) */
typedef struct mjx_pid_params {
  double safety, kI, kP, dt_min, dt_max, max_factor, min_factor, atol, rtol;
} mjx_pid_params;

typedef struct mjx_imex_problem {
  int reaction;        /* mjx_reaction */
  int nfields;         /* 1..4 (Gray-Scott: 2, fields u then v) */
  double D[4];         /* per-field diffusivity; D <= 1e-14 passes the field through */
  double F, k, r;      /* reaction parameters */
  double dt_cfl;       /* imex_cfl_dt (moljax/core/dt_policy.py:430-502), host-computed */
  int use_strang;      /* 1: IMEX-Strang (order 2); 0: IMEX-Euler (order 1, not in the mixed form) */
  int max_attempts;    /* hard cap on step attempts (accepted + rejected); <= 0 -> default */
} mjx_imex_problem;

/* moljax/core/stepping.py:710-720 (AdaptiveResult scalars) */
typedef struct mjx_adaptive_result {
  double t_final, dt_next, prev_err, last_err;
  int n_accepted, n_rejected, n_attempts, n_saved, status, finite;
} mjx_adaptive_result;

const char* mjx_version(void);
const char* mjx_status_string(int status);
/* Text of the last CUDA error seen by this host thread ("" if none), with the source location. */
const char* mjx_last_error(void);

/* ---- periodic 2D spectral plans ------------------------------------------------ */
/* Device bytes of a plan: twiddle tables for nx and ny plus the 1D symbols.
 * Replaces FFTCache2D / create_fft_cache_2d (moljax/core/fft_solvers.py:38-42, 181-198). */
size_t mjx_spec2d_plan_bytes(int ny, int nx, int dtype);
mjx_status mjx_spec2d_plan_init(void* plan, const mjx_grid2d* grid, int symbol, int dtype,
                                void* stream);
/* Spectrum workspace for nfields fields: nfields * ny * (nx/2+1 padded) complex. */
size_t mjx_spec2d_ws_bytes(int ny, int nx, int nfields, int dtype);

/* out_f = IFFT2( m(h, D_f, lam) * FFT2(in_f) ) for each of nfields fields.
 * Generic spectral pass: Helmholtz (solve_helmholtz_2d, fft_solvers.py:261-294,
 * apply_diffusion_inverse_fft 406-445), CN factor, exponential.  in may equal out.
 * Fields with D <= 1e-14 are copied unchanged (fft_solvers.py:435-443). */
mjx_status mjx_spectral_apply2d(const void* plan, const mjx_grid2d* grid, int dtype, int nfields,
                                const double* D, double h, int mult, const void* in, void* out,
                                void* ws, size_t ws_bytes, void* stream);

/* ---- periodic grids of any size (numpy / jnp.fft lengths) ------------------------- */
/* Plan of a length-n DFT: n a power of two <= 4096 (Stockham) or any n <= 2048
 * (Bluestein chirp-z with a power-of-two convolution <= 4096); 0 bytes if unsupported. */
size_t mjx_dftn_plan_bytes(int n, int dtype);
mjx_status mjx_dftn_plan_init(void* plan, int n, int dtype, void* stream);
size_t mjx_spectral_general2d_ws_bytes(int ny, int nx, int nfields, int dtype);
/* out_f = real(IFFT2( m FFT2(in_f) )) for ny x nx interiors of any supported size, on the
 * full complex spectrum (row DFTs, transpose, column DFTs, multiplier, and back).  mult:
 * MJX_MULT_SCALE/HELMHOLTZ/CN/EXP/LAP with lam the FD or spectral symbol and D_f, the
 * advection forms MJX_MULT_ADV_* with vx_f, vy_f (may be NULL: zero), or MJX_MULT_TABLE with
 * table [ny][nx].  The same operations as mjx_spectral_apply2d / mjx_advdiff_op2d /
 * mjx_spectral_filter2d (fft_solvers.py:222-616, fft_operators.py:80-260). */
mjx_status mjx_spectral_apply_general2d(const void* plan_y, const void* plan_x, const mjx_grid2d* grid, int symbol,
                                        int dtype, int nfields, const double* D, const double* vx,
                                        const double* vy, double h, int mult, const void* table,
                                        const void* in, void* out, void* ws, size_t ws_bytes, void* stream);

size_t mjx_spectral_general3d_ws_bytes(int nz, int ny, int nx, int dtype);
/* n_steps times u <- real(IFFTN( m(h, D, lam) FFTN(u) )) on an [nz][ny][nx] box of any
 * supported lengths (the general form of mjx_spectral_apply3d; the 3D FFT-CN of
 * bench_3d_feasibility.py at its 48^3, 80^3, 100^3 cases).  mult: SCALE/HELMHOLTZ/CN/EXP/LAP. */
mjx_status mjx_spectral_apply_general3d(const void* plan_z, const void* plan_y, const void* plan_x,
                                        const mjx_grid3d* grid, int symbol, int dtype, double D, double h, int mult,
                                        int n_steps, const void* in, void* out, void* ws, size_t ws_bytes,
                                        void* stream);

/* ---- periodic 3D boxes (benchmarks/sisc/bench_3d_feasibility.py) ------------------ */
/* Plan: x / y / z twiddles and 1D symbols (FD or spectral) of an [nz][ny][nx] box. */
size_t mjx_spec3d_plan_bytes(int nz, int ny, int nx, int dtype);
mjx_status mjx_spec3d_plan_init(void* plan, const mjx_grid3d* grid, int symbol, int dtype, void* stream);
/* Spectrum workspace: nz * ny * (nx/2+1 padded) complex. */
size_t mjx_spec3d_ws_bytes(int nz, int ny, int nx, int dtype);
/* n_steps times u <- real(IFFTN( m(h, D, lam_x + lam_y + lam_z) FFTN(u) )), each a full
 * forward and inverse transform: with MJX_MULT_CN the 3D FFT-CN loop of
 * bench_3d_feasibility.py:71-87 (cn_step_3d in a fori_loop); also Helmholtz, exp, D Lap. */
mjx_status mjx_spectral_apply3d(const void* plan, const mjx_grid3d* grid, int dtype, double D, double h, int mult,
                                int n_steps, const void* in, void* out, void* ws, size_t ws_bytes,
                                void* stream);

/* out_f = real(IFFT2( FFT2(in_f) / (1 - h (D_f lam - i (vx_f kx + vy_f ky))) )): the exact
 * periodic advection-diffusion inverse of FFTAdvectionDiffusionPreconditioner
 * (moljax/core/preconditioners.py:297-420; kx, ky = 2 pi fftfreq, |denominator| clamped at
 * 1e-14).  Fields with D <= 1e-14 and |v| <= 1e-14 are copied unchanged. */
mjx_status mjx_advdiff_apply2d(const void* plan, const mjx_grid2d* grid, int dtype, int nfields,
                               const double* D, const double* vx, const double* vy, double h,
                               const void* in, void* out, void* ws, size_t ws_bytes, void* stream);

/* The periodic advection-diffusion operator L = D Lap - v.grad with the symbol
 * D lam - i (vx kx + vy ky) (kx, ky = 2 pi fftfreq): op 0 solves (I - h L) u = in
 * (as mjx_advdiff_apply2d), op 1 applies h L, op 2 applies exp(h L), op 3 one
 * Crank-Nicolson step (I - h L/2)^-1 (I + h L/2); out = the real part
 * (AdvectionDiffusionOperator, moljax/core/fft_operators.py:179-260: solve, matvec with
 * h = 1, exp_matvec; the 1D advective FFT-CN of
 * benchmarks/benchmark_solver_comparison.py:152-163).  Fields with D <= 1e-14 and |v| <= 1e-14 are copied (ops 0, 2)
 * or zeroed (op 1). */
mjx_status mjx_advdiff_op2d(const void* plan, const mjx_grid2d* grid, int dtype, int nfields,
                            const double* D, const double* vx, const double* vy, double h, int op,
                            const void* in, void* out, void* ws, size_t ws_bytes, void* stream);

/* out_f = real(IFFT2( sigma * FFT2(in_f) )) with sigma a real multiplier per point of the
 * half spectrum: table [ny][ldc] (ldc = nx/2+1 rounded up to a multiple of 4), the
 * Hermitian part (K(k) + K(-k))/2 of a full-spectrum kernel K
 * (apply_spectral_filter_interior, moljax/core/fft_solvers.py:534-556). */
mjx_status mjx_spectral_filter2d(const void* plan, const mjx_grid2d* grid, int dtype, int nfields,
                                 const void* table, const void* in, void* out, void* ws, size_t ws_bytes,
                                 void* stream);

/* n_steps Crank-Nicolson steps u <- real(IFFT2(G * FFT2(u))) executed one by one;
 * G = (1 + dt D lam/2)/(1 - dt D lam/2).  Replaces the benchmark FFT-CN step
 * (benchmarks/benchmark_vs_scipy.py:74-91) behind fft_solvers.fft_cn_step. */
mjx_status mjx_fft_cn2d(const void* plan, const mjx_grid2d* grid, int dtype, double D, double dt,
                        int n_steps, const void* u_in, void* u_out, void* ws, size_t ws_bytes,
                        void* stream);

/* Workspace of mjx_gs_cn_newton2d: the two fields' row spectra, c_old, w and the residual
 * maxima (nx >= 16). */
size_t mjx_gs_cn_ws_bytes(int ny, int nx, int dtype);
/* n_steps Crank-Nicolson steps of periodic Gray-Scott (fields u then v, [2][ny][nx]; D =
 * {Du, Dv}) solved by the preconditioned Newton iteration of the reference's Gray-Scott
 * benchmark (benchmarks/benchmark_gray_scott.py:162-228, cn_newton_step_jit): residual
 * u - u_old - dt/2 (D Lap u + D Lap u_old + R(u) + R(u_old)), update by the exact periodic
 * inverse of (I - dt/2 D Lap) applied to -res, while max|res_u| + max|res_v| > tol and
 * fewer than max_iter iterations ran.  The Laplacian is the plan's symbol (the benchmark
 * uses the pseudo-spectral -(kx^2 + ky^2)).  The Newton loop of each step is a CUDA graph
 * with a conditional while node (no host synchronisation per iteration or step).  iters
 * (optional, DEVICE int[n_steps]): Newton iterations per step; iters_total / last_res
 * (optional, host): their sum and the last residual norm.  y_in may equal y_out.  FP64 is
 * the benchmark's precision; in FP32 the residual cannot fall below ~1e-7 relative. */
mjx_status mjx_gs_cn_newton2d(const void* plan, const mjx_grid2d* grid, int dtype, const double* D, double F,
                              double k, double dt, int n_steps, double tol, int max_iter, const void* y_in,
                              void* y_out, int* iters, int* iters_total, double* last_res, void* ws,
                              size_t ws_bytes, void* stream);

/* Workspace of mjx_gs_strang_exp2d: the two fields' half spectra. */
size_t mjx_gs_strang_exp_ws_bytes(int ny, int nx, int dtype);
/* n_steps fixed Strang steps of periodic Gray-Scott (imex_step / imex_solve of
 * benchmarks/benchmark_gray_scott.py:268-296): explicit Euler half step of the reaction,
 * exact exp(dt D lam) diffusion (lam from plan: FD or pseudo-spectral), explicit Euler half
 * step.  y_in / y_out: [u; v] interiors [2][ny][nx] (may alias); D[2] = (Du, Dv).  One row
 * and one column pass per step (nx >= 16, powers of two). */
mjx_status mjx_gs_strang_exp2d(const void* plan, const mjx_grid2d* grid, int dtype, const double* D, double F,
                               double k, double dt, int n_steps, const void* y_in, void* y_out, void* ws,
                               size_t ws_bytes, void* stream);

/* Workspace of mjx_gs_rk4_spectral2d: half spectra, stage input and running sum. */
size_t mjx_gs_rk4_spectral_ws_bytes(int ny, int nx, int dtype);
/* n_steps classical RK4 steps of periodic Gray-Scott with the Laplacian by FFT
 * (rk4_rhs / rk4_step / rk4_solve of benchmarks/benchmark_gray_scott.py:93-131; lam from
 * plan: pseudo-spectral as the benchmark, or FD).  Per stage one column pass (D lam) and
 * one row pass (inverse, reaction, running sum, next stage input, forward).  Same
 * arguments as mjx_gs_strang_exp2d. */
mjx_status mjx_gs_rk4_spectral2d(const void* plan, const mjx_grid2d* grid, int dtype, const double* D, double F,
                                 double k, double dt, int n_steps, const void* y_in, void* y_out, void* ws,
                                 size_t ws_bytes, void* stream);

/* Size of the fixed device scratch used by mjx_fft_cn2d_noalloc (8 MiB). */
#define MJX_NOALLOC_SCRATCH_BYTES (8u << 20)

/* mjx_fft_cn2d for callers that cannot call cudaMalloc: an allocator-free
 * host (an embedded driver loop, a signal-safe or real-time context, a host
 * whose device memory is owned by another framework's allocator) can still
 * run FFT-CN steps with only its input and output buffers.  The spectrum
 * scratch is a fixed 8 MiB array inside the library (held by every GPU that
 * loads the library until process exit), so the grid must satisfy
 * mjx_spec2d_ws_bytes(ny, nx, 1, dtype) <= MJX_NOALLOC_SCRATCH_BYTES (e.g.
 * 1024^2 FP32, 512^2 FP64); larger grids return MJX_WORKSPACE.  The first call
 * in each CUDA context looks up the scratch address of that context (make that
 * call before any stream capture): the array has its own address in the
 * device's primary context, in a driver-API context that an embedding host
 * made current, and in the new primary context after cudaDeviceReset, and the
 * lookup is cached per context, never per device.  No device memory is
 * allocated or freed.  All calls share
 * the one scratch array, so calls that overlap on the GPU (different streams,
 * or different host threads without ordering) race; nothing in the scratch
 * needs to start at zero, because each step writes every spectrum entry it
 * later reads.  No counterpart in the reference. */
mjx_status mjx_fft_cn2d_noalloc(const void* plan, const mjx_grid2d* grid, int dtype, double D,
                                double dt, int n_steps, const void* u_in, void* u_out,
                                void* stream);

/* ---- ghost cells and finite-difference stencils on padded fields ---------------- */
/* Padded layout: [nfields][ny+2g][nx+2g].  kinds[f] is an mjx_bc_kind; values holds
 * 4 constants per field (left, right, bottom, top): Dirichlet boundary values or
 * Neumann fluxes (NULL = homogeneous).  Ghost fill follows moljax/core/bc.py:202-307
 * (x ghosts first, then y ghosts, so corners are BC_y(BC_x(u))). */

/* interior [nf][ny][nx] -> padded with ghosts filled (create_state_from_interior +
 * apply_bc; state.py:268-295, bc.py:358-404). */
mjx_status mjx_bc_pad2d(const void* interior, void* padded, int nfields, int ny, int nx, int n_ghost,
                        const int* kinds, const double* values, double dy, double dx, int dtype,
                        void* stream);
/* padded -> padded with ghosts refilled (apply_bc, bc.py:358-404); in != out. */
mjx_status mjx_bc_fill2d(const void* padded_in, void* padded_out, int nfields, int ny, int nx,
                         int n_ghost, const int* kinds, const double* values, double dy, double dx,
                         int dtype, void* stream);
/* padded -> interior copy (get_interior_state, state.py:298-309). */
mjx_status mjx_unpad2d(const void* padded, void* interior, int nfields, int ny, int nx, int n_ghost,
                       int dtype, void* stream);
/* out = coef_f * Laplacian(in_f) on the interior, ghosts of out zero
 * (laplacian_2d, operators.py:311-322).  fill_bc != 0 evaluates the BC ghosts
 * on the fly instead of reading the input's ghost cells. */
mjx_status mjx_laplacian2d(const void* padded_in, void* padded_out, int nfields, int ny, int nx,
                           int n_ghost, const double* coef, int fill_bc, const int* kinds,
                           const double* values, double dy, double dx, int dtype, void* stream);
/* Reaction step of length h on interior fields [nfields][n]: Heun (euler = 0, the reaction
 * stage of imex_strang_step, moljax/core/stepping.py:370-435), explicit Euler (euler = 1,
 * imex_euler_step 317-367) or the rates N(y) themselves (euler = 2); Gray-Scott (nfields 2),
 * Fisher-KPP r u (1-u) per field, or none (a copy; rates zero).  in may equal out. */
mjx_status mjx_reaction_step2d(const void* in, void* out, int nfields, long long n, int reaction, double F,
                               double k, double r, double h, int euler, int dtype, void* stream);

/* div(D grad u) with face-averaged D on the interior of one padded field, ghosts zero
 * (apply_variable_diffusion_2d, moljax/core/variable_coeff.py:232-287).  D is padded like u,
 * or interior-shaped [ny][nx] (d_interior = 1) and edge-extended.  out must not alias u. */
mjx_status mjx_variable_diffusion2d(const void* u_padded, const void* D, int d_interior, void* out_padded,
                                    int ny, int nx, int n_ghost, double dy, double dx, int dtype, void* stream);

/* 2D one-axis differences on padded fields, ghosts read as stored, output ghosts zero:
 * op 1 upwind first derivative along axis with scalar velocity v (d1_upwind_2d,
 * operators.py:200-268), op 2 central first derivative (d1_central_2d, 155-197), op 3
 * central second derivative (d2_central_2d, 271-308); axis 0 = y, 1 = x; d = spacing. */
mjx_status mjx_stencil2d(const void* padded_in, void* padded_out, int nfields, int ny, int nx,
                        int n_ghost, int op, int axis, double v, double d, int dtype, void* stream);
/* result[0] = sqrt(sum((err/(atol + rtol |y|))^2) / n) (scaled_error_norm, state.py:312-343),
 * result[1] = 1 if every y is finite else 0 (is_finite, utils.py:186-197); n values each.
 * Host result, synchronises the stream; ws: mjx_error_norm_ws_bytes() device bytes. */
size_t mjx_error_norm_ws_bytes(void);
mjx_status mjx_scaled_error_norm(const void* err, const void* y, long long n, int dtype, double atol,
                                 double rtol, double* result, void* ws, size_t ws_bytes, void* stream);
/* Model right-hand side with BCs applied on the fly: D_f Lap(u_f) + reaction
 * (MOLModel.rhs, model.py:100-118; Gray-Scott operators.py:644-667; for
 * MJX_REACT_FISHER the parameter F carries r, operators.py:680-705). */
mjx_status mjx_rhs2d(const void* padded_in, void* padded_out, int nfields, int ny, int nx,
                     int n_ghost, int reaction, const double* D, double F, double k,
                     const int* kinds, const double* values, double dy, double dx, int dtype,
                     void* stream);

/* 1D stencils on padded fields [nfields][nx+2g], output ghosts 0: op 0 Laplacian
 * (laplacian_1d, operators.py:141-152), 1 first-order upwind d/dx for velocity v
 * (d1_upwind_1d, 64-110: backward if v >= 0), 2 central d/dx (d1_central_1d, 35-61). */
mjx_status mjx_stencil1d(const void* padded_in, void* padded_out, int nfields, int nx, int n_ghost,
                        int op, double v, double dx, int dtype, void* stream);

/* ---- IMEX-Strang (diffusion implicit by FFT, reaction explicit Heun) ------------- */
size_t mjx_imex2d_ws_bytes(int ny, int nx, int nfields, int dtype);

/* One fixed IMEX step of length dt: IMEX-Strang (moljax/core/stepping.py:370-435)
 * or, with prob->use_strang == 0, IMEX-Euler (317-367).  y_in may equal y_out. */
mjx_status mjx_imex_strang_step2d(const void* plan, const mjx_grid2d* grid, int dtype,
                                  const mjx_imex_problem* prob, double dt, const void* y_in,
                                  void* y_out, void* ws, size_t ws_bytes, void* stream);

/* Adaptive IMEX-Strang (or IMEX-Euler, prob->use_strang == 0, error order 1)
 * with step doubling and the PI controller, run as one
 * device-side loop (a CUDA graph with a conditional while node); no host
 * synchronisation per step.  Replaces adaptive_integrate_imex
 * (moljax/core/stepping.py:1146-1371) with estimate_error_imex_doubling (566-608),
 * scaled_error_norm (state.py:312-343) and propose_dt_imex (dt_policy.py:544-610).
 * hist_t/hist_dt (double[max_saves]) and hist_y ([max_saves][nfields][ny][nx])
 * may be NULL.  hist_y may be device memory or pinned host memory (cudaHostAlloc /
 * cudaHostRegister): the saved states then stream straight to the host as the loop
 * runs, so the device holds no history.  max_saves = max_steps // save_every + 1 as in the reference.
 * Blocks until the run finishes and fills *result. */
mjx_status mjx_imex_adaptive2d(const void* plan, const mjx_grid2d* grid, int dtype,
                               const mjx_imex_problem* prob, const mjx_pid_params* pid,
                               double t0, double t_end, double dt0, int max_steps, int save_every,
                               const void* y0, void* y_final, double* hist_t, double* hist_dt,
                               void* hist_y, void* ws, size_t ws_bytes,
                               mjx_adaptive_result* result, void* stream);

/* ---- Newton-Krylov implicit steps ------------------------------------------------ */
typedef enum mjx_method { MJX_METHOD_BE = 3, MJX_METHOD_CN = 4, MJX_METHOD_BDF2 = 5 } mjx_method;

/* moljax/core/newton_krylov.py:29-38 (NKParams) plus the GMRES restart length. */
typedef struct mjx_nk_params {
  int max_newton_iters, max_krylov_iters, restart, max_backtrack;
  double newton_tol, krylov_tol, damping, backtrack_factor, min_residual_decrease;
} mjx_nk_params;

size_t mjx_nk_vardiff_ws_bytes(int n, int restart);

/* n_steps fixed implicit steps (BE, CN, or BDF2 with a BE first step) of
 * u_t = div((a + b u^2) grad u) - c u^3 on an n x n cell-centred grid with
 * homogeneous Dirichlet ghosts (model_abc = {a, b, c}); y0/y_out are FP64
 * interiors.  Each step solves its residual (create_implicit_residual /
 * create_bdf2_residual, moljax/core/newton_krylov.py:362-448) with
 * newton_krylov_solve semantics (171-359): FP64 residual, FP32 hand-written
 * JVP and Krylov vectors, left-preconditioned restarted GMRES with the
 * Hessenberg/Givens least squares in FP64 on the GPU, preconditioner
 * (alpha0 I - beta Dbar Lap_D)^-1 (exact in the DST-II basis: a real DST-II /
 * DST-III pair of n-point transforms; plan2 = FP32 FD plan of the (2n)^2
 * periodic grid with the same spacing, whose symbols give the eigenvalues).
 * BE/CN initial guess: explicit Euler (stepping.py:195-196, 242-243) or, with
 * be_guess_previous != 0, y_n.  stats (optional, 3 ints per step): Newton
 * iterations, GMRES iterations, converged. */
mjx_status mjx_nk_vardiff_integrate2d(const void* plan2, int n, double dy, double dx,
                                      const double* model_abc, int method, double dt, int n_steps,
                                      int be_guess_previous, const mjx_nk_params* nkp,
                                      const double* y0, double* y_out, int* stats, void* ws,
                                      size_t ws_bytes, void* stream);

/* out = F(y) = div((a + b y^2) grad y) - c y^3 on the n x n interior with homogeneous
 * Dirichlet ghosts (MOLModel.rhs of this model, moljax/core/model.py:100-118 with
 * apply_variable_diffusion_2d, moljax/core/variable_coeff.py:232-287).  FP64. */
mjx_status mjx_vardiff_rhs2d(int n, double dy, double dx, const double* model_abc, const double* y,
                             double* out, void* stream);

/* ---- generic restarted GMRES (the Krylov cycle of newton_krylov_solve) ----------- */
/* A linear operator as a host callback: enqueues out = Op(v) on `stream` (device FP32
 * vectors of n elements) and returns 0, or non-zero to abort the solve. */
typedef int (*mjx_vec_op)(const float* v, float* out, void* user, void* stream);
/* Workspace of mjx_gmres_solve: the Arnoldi basis (restart + 1 vectors), two work vectors,
 * the partial sums and the GMRES header; 0 for restart outside [1, 64]. */
size_t mjx_gmres_ws_bytes(long long n, int restart);
/* Left-preconditioned restarted GMRES(restart) on A x = b: the Krylov solve of
 * newton_krylov_solve (moljax/core/newton_krylov.py:111-125, jax.scipy.sparse.linalg.gmres)
 * for any operator the host can enqueue.  precond may be NULL (identity).  x holds the initial
 * guess on entry and the solution on return.  Stops when the preconditioned residual estimate
 * falls to tol times the first cycle's |M^-1 (b - A x0)|, or after max_cycles cycles.
 * Orthogonalisation (classical Gram-Schmidt, FP64 dots), Givens steps and the update run on
 * the device; the host synchronises once per cycle.  iterations: Arnoldi steps used;
 * rel_res: final relative residual estimate; converged: 1 or 0. */
mjx_status mjx_gmres_solve(long long n, mjx_vec_op matvec, mjx_vec_op precond, void* user, const float* b,
                           float* x, double tol, int restart, int max_cycles, int* iterations, double* rel_res,
                           int* converged, void* ws, size_t ws_bytes, void* stream);

/* out = a0 v - beta J_F(u) v in FP64: the hand-written Jacobian-vector product of
 * F(u) = div((a + b u^2) grad u) - c u^3 (homogeneous Dirichlet ghosts), i.e. the JVP of
 * the residual a0 y + cst - beta F(y) at u (newton_krylov.py:61-80, _jvp_matvec, which
 * takes it with jax.jvp); a0 = 0, beta = -1 gives J_F(u) v.  u, v, out: n x n FP64. */
mjx_status mjx_vardiff_jvp2d(int n, double dy, double dx, const double* model_abc, double a0, double beta,
                             const double* u, const double* v, double* out, void* stream);

/* One implicit step of this model: be_step (moljax/core/stepping.py:170-214), cn_step
 * (217-260) or bdf2_step (263-310, omega = dt/dt_prev, y_prev = y_{n-1}), solved as in
 * mjx_nk_vardiff_integrate2d.  be_guess_previous: 0 the reference's guess (explicit Euler;
 * BDF2 2 y_n - y_{n-1}), 1 y_n, 2 the values y_out holds on entry (newton_krylov_solve's x0
 * for a residual of create_implicit_residual / create_bdf2_residual, newton_krylov.py:
 * 171-359).  stats (optional): Newton iterations, GMRES iterations, converged; res_norm
 * (optional): final residual norm (NKStats, newton_krylov.py:41-46). */
mjx_status mjx_nk_vardiff_step2d(const void* plan2, int n, double dy, double dx,
                                 const double* model_abc, int method, double dt, double dt_prev,
                                 int be_guess_previous, const mjx_nk_params* nkp, const double* y_n,
                                 const double* y_prev, double* y_out, int* stats, double* res_norm,
                                 void* ws, size_t ws_bytes, void* stream);

/* Adaptive implicit integration of this model: the implicit branch of adaptive_integrate
 * (moljax/core/stepping.py:723-1021).  BE error = dt F(y_BE); CN and BDF2 error =
 * y_method - y_BE (a second, BE solve per attempt; BDF2 takes BE steps while no step has
 * been accepted).  Acceptance also needs Newton convergence; the next dt follows
 * propose_dt (moljax/core/dt_policy.py:324-408) with implicit_robustness_dt (279-321).
 * The accept/reject loop runs on the host (one synchronisation per attempt, after the
 * Newton solves).  hist_t/hist_dt: HOST arrays of max_saves doubles (may be NULL);
 * hist_y: device array of max_saves n x n FP64 states (may be NULL).  nk_totals
 * (optional, 3 ints): Newton iterations, GMRES iterations and non-converged solves
 * summed over all attempts.  attempt_log (optional HOST array of 6 * log_cap doubles):
 * per attempt t, dt tried, error ratio, Newton converged, Newton iterations, accepted.
 * Workspace: mjx_nk_vardiff_ws_bytes. */
mjx_status mjx_nk_vardiff_adaptive2d(const void* plan2, int n, double dy, double dx,
                                     const double* model_abc, int method,
                                     const mjx_pid_params* pid, double t0, double t_end, double dt0,
                                     int max_steps, int save_every, int be_guess_previous,
                                     const mjx_nk_params* nkp, const double* y0, double* y_final,
                                     double* hist_t, double* hist_dt, double* hist_y,
                                     int* nk_totals, double* attempt_log, int log_cap,
                                     mjx_adaptive_result* res, void* ws, size_t ws_bytes,
                                     void* stream);

/* ---- explicit Runge-Kutta (Euler, SSPRK3, RK4) on the 5-point stencil ------------------ */
/* Reaction-advection-diffusion model for the explicit steppers: per field D_f Lap(u_f)
 * - vx du_f/dx - vy du_f/dy (advection 0: none, 1: upwind d1_upwind_2d, operators.py:200-268,
 * 2: central) plus the reaction, with ghost values from the field's BC (bc.py:202-307) computed
 * on the fly.  method: 0 Euler, 1 SSPRK3, 2 RK4 (IntegratorType, stepping.py:48-57). */
typedef struct mjx_explicit_problem {
  int reaction;          /* mjx_reaction */
  int nfields;           /* 1..4 */
  double D[4];
  double F, k, r;
  double vx, vy;
  int advection;
  int method;
  int bc_kind[4];        /* mjx_bc_kind per field */
  double bc_values[16];  /* per field: left, right, bottom, top (Dirichlet value / Neumann flux) */
  double dt_cfl;         /* heisenberg_cfl_dt (moljax/core/dt_policy.py:104-175), host-computed */
  int max_attempts;      /* <= 0 -> 20 * max_steps + 1000 */
  int pad;
  mjx_kinetics kin;      /* the network when reaction == MJX_REACT_KINETICS */
} mjx_explicit_problem;

/* Workspace of the explicit steppers: 7 state-sized buffers plus partials and the state. */
size_t mjx_explicit_ws_bytes(int ny, int nx, int nfields, int dtype);
/* n_steps fixed steps of euler_step / ssprk3_step / rk4_step (moljax/core/stepping.py:64-163,
 * integrate_fixed_dt 1028-1139) on interiors [nfields][ny][nx]; one fused kernel per stage. */
mjx_status mjx_explicit_integrate2d(const mjx_grid2d* grid, int dtype, const mjx_explicit_problem* prob,
                                    double dt, int n_steps, const void* y0, void* y_out, void* ws,
                                    size_t ws_bytes, void* stream);
/* out = F(y): MOLModel.rhs of this model on interiors (moljax/core/model.py:100-118). */
mjx_status mjx_explicit_rhs2d(const mjx_grid2d* grid, int dtype, const mjx_explicit_problem* prob,
                              const void* y, void* out, void* stream);
/* The explicit branch of adaptive_integrate (moljax/core/stepping.py:723-1021): step doubling
 * (step_explicit_with_error, 648-682), error order 1/3/4, PI controller with the CFL limit
 * (propose_dt, dt_policy.py:324-408), accept/reject on the device in a conditional-graph loop.
 * Same history, result and status semantics as mjx_imex_adaptive2d (hist_y may be pinned
 * host memory).  Any grid size; any BC per field. */
mjx_status mjx_explicit_adaptive2d(const mjx_grid2d* grid, int dtype, const mjx_explicit_problem* prob,
                                   const mjx_pid_params* pid, double t0, double t_end, double dt0,
                                   int max_steps, int save_every, const void* y0, void* y_final,
                                   double* hist_t, double* hist_dt, void* hist_y, void* ws,
                                   size_t ws_bytes, mjx_adaptive_result* result, void* stream);

/* ---- DST-I and the Dirichlet spectral solvers -------------------------------------- */
/* Plan of the length-n DST-I (twiddles; for 2(n+1) not a power of two, the Bluestein
 * chirp and filter).  Lengths: 1 <= n <= 1023, or n = 2^k - 1 <= 2047.  0 = unsupported. */
size_t mjx_dst1_plan_bytes(int n, int dtype);
mjx_status mjx_dst1_plan_init(void* plan, int n, int dtype, void* stream);

/* Row-batched transforms and solvers along rows of n values (nrows rows, contiguous):
 *  mode 0: out = scale * DST-I(x)   (dst_I_fast, moljax/core/fft_nonperiodic.py:97-122;
 *          scale 2/(n+1) gives idst_I_fast, 125-133)
 *  mode 1: out = IDST(DST(x) / (1 - h D lam))  (solve_helmholtz_dirichlet, 308-330)
 *  mode 2: out = IDST(DST(x) / lam)            (solve_poisson_dirichlet, 244-271)
 *  mode 3: out = IDST(exp(h lam) DST(u) + h phi1(h lam) DST(N))  (etd1_dirichlet, 360-398),
 *          x holds the nrows rows of u followed by the nrows rows of N(u).
 * lam: device array of n values in the data type (the symbol, or the eigenvalues for mode 3);
 * NULL for mode 0.  One kernel launch; out must not overlap x. */
mjx_status mjx_dst1(const void* plan, int n, long long nrows, int dtype, int mode, const void* x,
                    void* out, const void* lam, double h, double D, double scale, void* stream);

/* Orthonormal DCT-II (jax.scipy.fft.dct(type=2, norm='ortho')) and the Neumann spectral
 * solvers along rows of n values: plan of the length-n transform (1 <= n <= 1024, or n a
 * power of two <= 2048; 0 = unsupported).
 *  mode 0: out = scale * DCT(x);  mode 1: out = scale * IDCT(x) (DCT-III, the inverse)
 *  mode 2: out = IDCT(DCT(x) / (1 - h D lam))        (solve_helmholtz_neumann, 333-355)
 *  mode 3: out = IDCT(DCT(x) / lam), null modes -> 0 (solve_poisson_neumann, 274-305)
 *  mode 4: out = IDCT(exp(h lam) DCT(u) + h phi1(h lam) DCT(N)) (etd1_neumann, 401-437),
 *          x holds the nrows rows of u followed by the nrows rows of N(u). */
size_t mjx_dct2_plan_bytes(int n, int dtype);
mjx_status mjx_dct2_plan_init(void* plan, int n, int dtype, void* stream);
mjx_status mjx_dct2(const void* plan, int n, long long nrows, int dtype, int mode, const void* x,
                    void* out, const void* lam, double h, double D, double scale, void* stream);

/* ---- 1D tubular reactor, Crank-Nicolson, batched --------------------------------- */
typedef enum mjx_reactor_variant {
  MJX_REACTOR_DANCKWERTS = 0, /* benchmarks/benchmark_reactor_vs_diffrax.py:40-138 (dispersion CN,
                                 upwind advection and reaction explicit: needs dt <= dz) */
  MJX_REACTOR_DIRICHLET = 1,  /* benchmarks/benchmark_method_comparison.py:56-160 */
  MJX_REACTOR_DANCKWERTS_CN = 2, /* the Danckwerts discretisation of variant 0 advanced by the fully
                                   implicit CN of benchmark_method_comparison.py:134-160 (stable at
                                   its CN step dt = min(10 dz, 0.05, t_final/100), line 216) */
  /* benchmarks/benchmark_tubular_reactor.py:57-200: N nodes, dz = 1/(N-1), classical RK4 of
     (1/Pe) D2 c - D1 c - Da c with the end rows replaced by penalties 100 (target - c)
     (mjx_reactor_rk4_batch only) */
  MJX_REACTOR_RK4_DANCKWERTS = 3, /* inlet (c_in + k c1)/(1 + k), k = 1/(Pe dz); outlet c_{N-2} */
  MJX_REACTOR_RK4_ROBIN = 4,      /* alpha_in = 1, beta_in = 1/Pe, alpha_out = 0, beta_out = 1 */
  MJX_REACTOR_RK4_NEUMANN = 5     /* inlet c1, outlet c_{N-2} */
} mjx_reactor_variant;

/* One reactor solve of c_t = c_zz/Pe - c_z - Da c: n points, n_steps fixed CN
 * steps of dt from the uniform state c_init (the Dirichlet variant also sets
 * c[0] = c_inlet, as benchmark_method_comparison.py:188-190). */
typedef struct mjx_reactor_instance {
  int n, variant, n_steps, pad;
  long long offset;    /* element offset of this instance's final state in out */
  double Pe, Da, dt, c_init, c_inlet;
} mjx_reactor_instance;

/* Dynamic shared memory of one instance of size n. */
size_t mjx_reactor_smem_bytes(int n, int dtype);
/* n_inst independent reactor solves of different sizes and parameters in one
 * launch (one CTA per instance, every step of an instance in shared memory).
 * inst_dev: device array of instances; max_n: largest n in the batch (<= 4096
 * FP64, <= 8192 FP32).  Replaces solve_reactor_cn_jit
 * (benchmark_reactor_vs_diffrax.py:116-138) and run_reactor_cn
 * (benchmark_method_comparison.py:134-160), whose dense O(n^2) solves become
 * a tridiagonal factorisation plus two parallel substitution scans per step. */
mjx_status mjx_reactor_cn_batch(const mjx_reactor_instance* inst_dev, int n_inst, int max_n,
                                int dtype, void* out, void* stream);
/* n_inst penalty-BC RK4 reactor solves (variants MJX_REACTOR_RK4_*; c_init the uniform
 * initial state, c_inlet the inlet value c_in; 3 <= n <= max_n <= 1024) in one launch, one
 * CTA of four warps per instance with the whole state in registers.  Replaces solve_rk4 with
 * create_rhs_danckwerts / create_rhs_robin / create_rhs_neumann
 * (benchmarks/benchmark_tubular_reactor.py:84-192, 254-301), whose RHS is a dense n x n
 * matvec.  An instance of another variant or an n outside [3, max_n] comes back as NaN. */
mjx_status mjx_reactor_rk4_batch(const mjx_reactor_instance* inst_dev, int n_inst, int max_n,
                                 int dtype, void* out, void* stream);

/* ---- ETDRK4 (Cox-Matthews) for coupled Gray-Scott ------------------------------ */
/* Workspace: row spectra ZU/ZN/ZX, 2D spectra U^/N^u/a^/S and the coefficient tables. */
size_t mjx_etdrk4_ws_bytes(int ny, int nx, int dtype);

/* n_steps fixed ETDRK4 steps of the coupled Gray-Scott system (fields u then v,
 * interior [2][ny][nx]); restates benchmarks/benchmark_gray_scott.py:336-417.
 * The coefficient tables E, E2, Q, f1, f2, f3 are evaluated on the GPU in FP64
 * by the 32-point contour mean (336-356) when recompute_coeffs != 0 and kept in
 * the workspace (pass 0 to reuse them for the same grid, D, dt and symbol).
 * symbol: mjx_symbol (FD as DiffusionOperator, or pseudo-spectral as the benchmark).
 * f2_factor: 2 = Cox-Matthews ETDRK4 (as fft_integrators.py:110, b2 = 2 phi2 - 4 phi3);
 * 1 = the benchmark script's update, which omits that factor (benchmark_gray_scott.py:415).
 * Also backs fft_integrators.etdrk4_step (moljax/core/fft_integrators.py:252-341). */
mjx_status mjx_etdrk4_gray_scott2d(const void* plan, const mjx_grid2d* grid, int dtype, int symbol,
                                   const double* D, double F, double k, double dt, double f2_factor,
                                   int n_steps,
                                   const void* y_in, void* y_out, void* ws, size_t ws_bytes,
                                   int recompute_coeffs, void* stream);
/* ---- ETD1 / ETD2 / ETDRK4 (moljax/core/fft_integrators.py) ---------------------- */
typedef enum mjx_etd_method { MJX_ETD_1 = 1, MJX_ETD_2 = 2, MJX_ETD_RK4 = 4 } mjx_etd_method;
typedef enum mjx_etd_coeffs {
  MJX_ETD_COEFF_CONTOUR = 0, /* 32-point contour mean (benchmark_gray_scott.py:336-356); ETDRK4 only */
  MJX_ETD_COEFF_PHI = 1      /* phi functions, Taylor below |z| = 1e-4 (fft_integrators.py:39-116) */
} mjx_etd_coeffs;

typedef struct mjx_etd_problem {
  int method;       /* mjx_etd_method */
  int coeffs;       /* mjx_etd_coeffs (ETD1 and ETD2 always use the phi functions) */
  int symbol;       /* mjx_symbol, optionally | MJX_SYMBOL_X_ONLY */
  int reaction;     /* MJX_REACT_NONE (N = 0), MJX_REACT_GRAY_SCOTT (nfields 2), MJX_REACT_FISHER (r u (1-u)) */
  int nfields;      /* 1 or 2; interior fields [nfields][ny][nx] */
  int pad;
  double D[2];      /* diffusivity per field: L = D Lap */
  double F, k, r;   /* reaction parameters */
  double dt;
  double f2_factor; /* contour ETDRK4 only: 2 Cox-Matthews, 1 the benchmark script's update */
} mjx_etd_problem;

/* n_steps fixed steps of u_t = D Lap u + N(u) on a periodic grid, as etd_integrate
 * (fft_integrators.py:344-393) runs etd1_step (119-175), etd2_step (178-249) or
 * etdrk4_step (252-341); the nonlinear term of the Gray-Scott pair is evaluated
 * coupled.  ETD2 without nprev_in starts with an ETD1 step (207-209); with
 * nprev_in (real N(u_{n-1}), [nfields][ny][nx]) every step is ETD2.  n_out
 * (optional, n_steps >= 1) receives N at the start of the last step, the N_curr
 * that etd2_step returns.  The coefficient tables live in the workspace
 * (size mjx_etdrk4_ws_bytes); recompute_coeffs = 0 reuses them for the same grid,
 * problem and dt. */
mjx_status mjx_etd_integrate2d(const void* plan, const mjx_grid2d* grid, int dtype, const mjx_etd_problem* p,
                               int n_steps, const void* y_in, const void* nprev_in, void* y_out, void* n_out,
                               void* ws, size_t ws_bytes, int recompute_coeffs, void* stream);

/* N(y) of the ETD problem's reaction on interior fields [nfields][ny][nx] (one row
 * pass); the nonlinear_rhs of fft_integrators for a native reaction. */
mjx_status mjx_etd_nonlinear2d(const void* plan, const mjx_grid2d* grid, int dtype, int reaction, int nfields,
                               double F, double k, double r, const void* y, void* out, void* stream);

/* Launches one kernel of an ETDRK4 step for timing/profiling (which = 1..8:
 * C1, R1, C2, R2, C3, R3, C4, R4).  No reference counterpart. */
mjx_status mjx_etdrk4_kernel2d(const void* plan, const mjx_grid2d* grid, int dtype, double F,
                               double k, int which, void* ws, size_t ws_bytes, void* stream);

/* Workspace bytes of mjx_imex_adaptive2d_mixed. */
size_t mjx_imex2d_mixed_ws_bytes(int ny, int nx, int nfields);

/* Adaptive IMEX-Strang in mixed precision: the state is kept as its half
 * spectrum in float-float form (each real value an unevaluated sum of two FP32
 * numbers, about 48 significant bits, all arithmetic on the FP32 pipe), the
 * diffusion multipliers are applied to it in that form, and only the reaction
 * increments and the error estimate pass through FP32 transforms, so FP32
 * rounding scales with the increments instead of the state.  The initial and
 * final conversions between the real state and the spectrum run in FP64.  Same loop,
 * controller and result semantics as mjx_imex_adaptive2d (adaptive_integrate_imex,
 * moljax/core/stepping.py:1146-1371).  plan32/plan64: FD-symbol plans of the grid
 * in FP32 and FP64.  io_dtype: dtype of y0 and y_final.  No y history. */
mjx_status mjx_imex_adaptive2d_mixed(const void* plan32, const void* plan64, const mjx_grid2d* grid,
                                     int io_dtype, const mjx_imex_problem* prob,
                                     const mjx_pid_params* pid, double t0, double t_end, double dt0,
                                     int max_steps, int save_every, const void* y0, void* y_final,
                                     double* hist_t, double* hist_dt, void* ws, size_t ws_bytes,
                                     mjx_adaptive_result* result, void* stream);

/* Persistent plan of the mixed-precision adaptive loop for one problem: the attempt
 * kernels and controller of mjx_imex_adaptive2d_mixed captured ONCE into a CUDA graph
 * with a conditional while node and instantiated; every mjx_imex_plan_run replays it
 * (no graph capture, instantiation or device allocation per call).  The plan owns the
 * graph; the caller owns ws (mjx_imex_plan_ws_bytes: the mixed workspace plus the t/dt
 * history of max_saves = max_steps / save_every + 1 steps) and the FP32/FP64 grid plans,
 * which must outlive the plan.  The grid, problem, PID settings, max_steps and save_every
 * are fixed at creation; t0, t_end, dt0 and the state vary per run.  Runs of one plan
 * must not overlap (they share ws).  The steady loop of adaptive_integrate_imex
 * (moljax/core/stepping.py:1146-1371) as a reusable object; JAX re-traces per shape. */
size_t mjx_imex_plan_ws_bytes(int ny, int nx, int nfields, int max_saves);
mjx_status mjx_imex_plan_create(void** plan, const void* plan32, const void* plan64, const mjx_grid2d* grid,
                                const mjx_imex_problem* prob, const mjx_pid_params* pid, int max_steps,
                                int save_every, void* ws, size_t ws_bytes);
/* One adaptive solve from y0 ([nfields][ny][nx], io_dtype) to y_final; hist_t/hist_dt
 * (optional, device or host arrays of max_saves doubles) receive the t/dt history. */
mjx_status mjx_imex_plan_run(void* plan, int io_dtype, double t0, double t_end, double dt0, const void* y0,
                             void* y_final, double* hist_t, double* hist_dt, mjx_adaptive_result* result,
                             void* stream);
mjx_status mjx_imex_plan_destroy(void* plan);

/* Launches a single kernel of one mixed-precision attempt (timing/profiling):
 * which = 0 seeds the workspace from the FP32 state y with step dt; 1..6 launch
 * C1, R1, C2, R2, C3, R3 (see csrc/imex_mixed.cu); 7 the controller (it advances the
 * seeded state as an attempt would).  No reference counterpart. */
mjx_status mjx_imex_mixed_attempt_kernel2d(const void* plan32, const void* plan64,
                                           const mjx_grid2d* grid, const mjx_imex_problem* prob,
                                           const mjx_pid_params* pid, int which, double dt,
                                           const void* y, void* ws, size_t ws_bytes, void* stream);

/* Launches a single kernel of one fused adaptive attempt, for timing and
 * profiling: which = 0 seeds the workspace (both state buffers = y, step dt),
 * 1..7 launch the row/column passes K1..K7 of IMEX-Strang, or 1..5 the passes
 * E1..E5 of IMEX-Euler (see csrc/imex.cu).  No reference
 * counterpart: the reference has no per-kernel entry points. */
mjx_status mjx_imex_attempt_kernel2d(const void* plan, const mjx_grid2d* grid, int dtype,
                                     const mjx_imex_problem* prob, const mjx_pid_params* pid,
                                     int which, double dt, const void* y, void* ws,
                                     size_t ws_bytes, void* stream);

/* ---- batched adaptive IMEX-Strang: many Gray-Scott solves in one engine ------------ */
/* One Gray-Scott solve of the batch: grid, parameters, time span and controller
 * settings of adaptive_integrate_imex (moljax/core/stepping.py:1146-1371) for the
 * periodic model of create_gray_scott_periodic_fft (moljax/core/model.py:529-584). */
typedef struct mjx_gs_instance {
  int ny, nx;           /* powers of two, 16 <= ny <= 2048, 16 <= nx <= 4096 */
  double dy, dx;
  double Du, Dv, F, k;
  double t0, t_end, dt0;
  double dt_cfl;        /* imex_cfl_dt (moljax/core/dt_policy.py:430-502), host-computed */
  int max_steps, save_every, max_attempts, pad;  /* max_attempts <= 0: 20 max_steps + 1000 */
  mjx_pid_params pid;
} mjx_gs_instance;

/* Engine device bytes for up to max_instances solves and max_work work items per
 * pass (sum of mjx_gsbatch_work_items over the solves in flight). */
size_t mjx_gsbatch_bytes(int max_instances, int max_work);
/* Device bytes of one solve's workspace (float-float spectral state, FP32 and FP64
 * plans, error partials, t/dt history of max_saves = max_steps / save_every + 1). */
size_t mjx_gsbatch_instance_bytes(int ny, int nx, int max_saves);
/* Work items of one solve in the largest pass. */
int mjx_gsbatch_work_items(int ny, int nx);

/* Creates a batch engine in the caller's device workspace ws (mjx_gsbatch_bytes).
 * Every solve runs the mixed-precision attempt of mjx_imex_adaptive2d_mixed with
 * its own dt, controller state, accept mask and status; one persistent kernel per
 * attempt stage covers every solve in flight, and a batched controller (one warp per
 * solve) applies the PI / accept-reject update of each.  The attempt loop is a CUDA
 * graph with a conditional while node, captured once here; admissions and retirements
 * change only device memory.  The engine also holds one mapped pinned host flag
 * (mjx_gsbatch_request_stop).  Thread-compatible: one thread drives an engine.
 * The reference's only batching is stacking and vmap (moljax/core/jit_kernels.py:422-441,
 * fft_integrators.py:473-510); there is no engine counterpart. */
mjx_status mjx_gsbatch_create(void** batch, int max_instances, int max_work, void* ws, size_t ws_bytes);
mjx_status mjx_gsbatch_destroy(void* batch);
/* Admits one solve: y0 is [2][ny][nx] (u then v, io_dtype) and goes through an FP64
 * transform into the solve's float-float spectral state in ws
 * (mjx_gsbatch_instance_bytes); returns its slot.  MJX_OOM when no slot or no work-list
 * room is free.  Synchronises the stream. */
mjx_status mjx_gsbatch_admit(void* batch, const mjx_gs_instance* inst, int io_dtype, const void* y0, void* ws,
                             size_t ws_bytes, int* slot, void* stream);
/* Runs attempts of every admitted solve (one epoch) until none is running, until
 * stop_after_finished solves finished in this epoch (0: no such stop), after
 * max_attempts attempts, or when the stop flag is raised; blocks until the epoch ends.
 * n_running / n_finished (optional): solves still running, and finished solves waiting
 * for mjx_gsbatch_retire. */
mjx_status mjx_gsbatch_run(void* batch, int max_attempts, int stop_after_finished, int* n_running,
                           int* n_finished, void* stream);
/* Slots of the finished solves (up to cap of them) and their count. */
mjx_status mjx_gsbatch_finished(void* batch, int* slots, int cap, int* n);
/* Writes a finished solve's final state y_final ([2][ny][nx], io_dtype, by an FP64
 * inverse transform), its t/dt history (HOST arrays of n_saved doubles, may be NULL)
 * and its result (AdaptiveResult scalars), then frees the slot.  The solve's workspace
 * may be released afterwards. */
mjx_status mjx_gsbatch_retire(void* batch, int slot, int io_dtype, void* y_final, double* hist_t, double* hist_dt,
                              mjx_adaptive_result* res, void* stream);
/* Raises (stop != 0) or clears the stop flag from any host thread: a running epoch
 * ends at its next attempt boundary (the server uses it to admit arrivals). */
void mjx_gsbatch_request_stop(void* batch, int stop);

/* ---- Autotuning --------------------------------------------------------------
 * No reference counterpart: under jax.jit XLA chooses its own FFT and fusion
 * strategies (moljax/core/fft_solvers.py:33-80 calls jnp.fft.fft2 / ifft2 and
 * moljax/core/stepping.py:126-163 leaves the stencil passes to XLA).  Here the
 * tunable launch choices are timed on the device and the fastest is kept in a
 * process-wide registry that the launchers read. */

/* Candidate radix schedules of a mixed-radix DFT length n = 2^a 3^b 5^c (not a power of
 * two): up to max rows of 17 ints [nrad, r0 .. r15] (radices 2, 3, 4, 5 in pass order)
 * written to out; returns the count (0 for other lengths).  Host only. */
int mjx_dft_schedule_candidates(int n, int* out, int max);
/* Installs the radix schedule (nrad radices whose product is n) and the threads per
 * sequence (tpsm in [1, 256], 0 = n/8) used for length n in dtype; nrad = 0 clears the
 * entry (back to the default schedule 4s, 2s, 3s, 5s). */
mjx_status mjx_dft_schedule_set(int n, int dtype, int nrad, const int* rad, int tpsm);
/* The schedule in use for length n (tuned or default): nrad (0 for power-of-two and
 * Bluestein lengths), rad[16], tpsm. */
mjx_status mjx_dft_schedule_get(int n, int dtype, int* nrad, int* rad, int* tpsm);
/* Times every candidate schedule of length n with threads per sequence n/4, n/8, n/16
 * on nrows rows of scratch (>= nrows * n complex values of dtype; overwritten) with
 * CUDA events, reps launches each after a warm-up launch, installs the fastest and
 * returns the candidate count, the winner's index and up to max_times times (ms per
 * launch, candidate order: schedule-major).  plan is a mjx_dftn_plan_init plan of n.
 * Lengths without a schedule (powers of two, Bluestein) return n_cand = 0. */
mjx_status mjx_autotune_dft(const void* plan, int n, int dtype, long long nrows, void* scratch,
                            size_t scratch_bytes, int reps, double* times, int max_times, int* n_cand,
                            int* best, void* stream);
/* Installs the rows per warp strip (2, 4, 8, 16 or 32; 0 = default 8) of the explicit
 * stage kernel for this grid size, field count and dtype; 64 selects the TMA-staged
 * form (shared-memory tiles of 32 x 128 points loaded by cp.async.bulk.tensor), used
 * for FP32 stages whose rows are a multiple of 4 points (others run with 8). */
mjx_status mjx_stencil_rows_set(int ny, int nx, int nfields, int dtype, int rows);
/* The installed rows per warp strip (0 when untuned). */
int mjx_stencil_rows_get(int ny, int nx, int nfields, int dtype);
/* Times an RK4 middle stage of prob on grid for strips of 2, 4, 8, 16 and 32 rows and,
 * for FP32 with nx a multiple of 4, the TMA-staged form (64) (reps launches each, CUDA
 * events) in ws (mjx_explicit_ws_bytes; overwritten), installs the fastest and returns
 * it with up to max_times times (ms per launch, candidate order). */
mjx_status mjx_autotune_stencil2d(const mjx_grid2d* grid, int dtype, const mjx_explicit_problem* prob,
                                  void* ws, size_t ws_bytes, int reps, double* times, int max_times,
                                  int* best_rows, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MOLJAX_GB300_H */
