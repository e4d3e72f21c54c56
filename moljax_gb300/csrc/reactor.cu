// Batched 1D tubular-reactor Crank-Nicolson: one CTA per instance, the whole
// time loop of an instance in shared memory.
//
// Model c_t = (1/Pe) c_zz - c_z - Da c in two reference discretisations:
//  MJX_REACTOR_DANCKWERTS  benchmarks/benchmark_reactor_vs_diffrax.py:40-138:
//    N cells, dz = 1/N, diffusion implicit (CN), upwind advection and
//    reaction explicit, Danckwerts inlet flux -(c0 - 1)/dz, outlet Neumann row.
//  MJX_REACTOR_DIRICHLET   benchmarks/benchmark_method_comparison.py:56-160:
//    N nodes, dz = 1/(N-1), fully implicit CN of L = D2/Pe - D1 - Da with a
//    Dirichlet inlet row and the one-sided outlet row.
//  MJX_REACTOR_DANCKWERTS_CN  the Danckwerts discretisation above, advanced by
//    the fully implicit CN of benchmark_method_comparison.py:134-160: the whole
//    operator M c + s (dispersion, upwind advection with the inlet flux, and
//    reaction; s = e_0/dz) is implicit, so the step is stable at the CN step
//    size of that benchmark, dt = min(10 dz, 0.05, t_final/100) (line 216),
//    which the semi-implicit form above is not (its explicit upwind advection
//    needs dt <= dz).
//  MJX_REACTOR_RK4_DANCKWERTS / _ROBIN / _NEUMANN  benchmarks/benchmark_tubular_reactor.py:
//    N nodes, dz = 1/(N-1), explicit RK4 with penalty end rows (reactor_rk4_kernel).
// The reference solves with a dense inverse / LU (O(N^2) per step); the system
// matrix is tridiagonal and constant in time, so each CTA factorises it once
// (Thomas) and runs every step's two substitution sweeps as parallel affine
// scans over the CTA (x_i = alpha_i x_{i-1} + beta_i composes associatively).
#include <math.h>
#include <string.h>

#include "common.cuh"

namespace mjx {

int elem_size(int dtype);
void set_last_error(cudaError_t e, const char* file, int line);

struct ReactorArgs {
  const mjx_reactor_instance* inst;
  void* out;          // concatenated states, instance i at inst[i].offset
  int n_inst;
};

// shared-memory index with one pad word per 16: the scans give each thread a
// contiguous chunk (stride = chunk length), which would otherwise hit one bank
__device__ __forceinline__ int pz(int i) { return i + (i >> 4); }
__host__ __device__ __forceinline__ int pz_size(int n) { return n + (n >> 4) + 1; }

// affine map y -> a y + b, composition "first p then q"
template <typename T> struct Aff { T a, b; };
template <typename T> __device__ __forceinline__ Aff<T> comp(Aff<T> p, Aff<T> q) {
  Aff<T> r; r.a = q.a * p.a; r.b = q.a * p.b + q.b; return r;
}

// Inclusive scan of x_i = al[i] x_{i-1} + be[i] (x_{-1} = 0) over n elements in
// smem, processed in order ord(i) (forward, or reverse when REV).  Result in be[].
template <typename T, bool REV>
__device__ void affine_scan(T* al, T* be, int n, Aff<T>* wsum) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int per = (n + nt - 1) / nt;
  const int lo = tid * per, hi = min(n, lo + per);
  auto idx = [&](int i) { return pz(REV ? n - 1 - i : i); };
  Aff<T> acc; acc.a = (T)1; acc.b = (T)0;
  for (int i = lo; i < hi; ++i) {
    Aff<T> e; e.a = al[idx(i)]; e.b = be[idx(i)];
    acc = comp(acc, e);
  }
  // warp inclusive scan of the thread aggregates
  const int lane = tid & 31, w = tid >> 5;
  Aff<T> inc = acc;
  for (int o = 1; o < 32; o <<= 1) {
    Aff<T> up;
    up.a = __shfl_up_sync(0xffffffffu, inc.a, o);
    up.b = __shfl_up_sync(0xffffffffu, inc.b, o);
    if (lane >= o) inc = comp(up, inc);
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (tid == 0) {  // scan of the warp totals (<= 32 warps)
    Aff<T> run; run.a = (T)1; run.b = (T)0;
    for (int q = 0; q < (nt >> 5); ++q) { run = comp(run, wsum[q]); wsum[q] = run; }
  }
  __syncthreads();
  // exclusive prefix for this thread
  Aff<T> ex;
  Aff<T> up;
  up.a = __shfl_up_sync(0xffffffffu, inc.a, 1);
  up.b = __shfl_up_sync(0xffffffffu, inc.b, 1);
  if (lane == 0) { ex.a = (T)1; ex.b = (T)0; } else { ex = up; }
  if (w > 0) ex = comp(wsum[w - 1], ex);
  T y = ex.b;  // value x_{lo-1} (the composite applied to x_{-1} = 0)
  __syncthreads();
  for (int i = lo; i < hi; ++i) {
    y = al[idx(i)] * y + be[idx(i)];
    be[idx(i)] = y;
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(256) reactor_kernel(ReactorArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const mjx_reactor_instance I = A.inst[blockIdx.x];
  const int n = I.n;
  if (I.variant < MJX_REACTOR_DANCKWERTS || I.variant > MJX_REACTOR_DANCKWERTS_CN) {  // an RK4 instance
    T* o = reinterpret_cast<T*>(A.out) + I.offset;
    for (int i = threadIdx.x; i < n; i += blockDim.x) o[i] = (T)NAN;
    return;
  }
  const int np = pz_size(n);               // padded length (index through pz)
  T* c = reinterpret_cast<T*>(smem_raw);   // state
  T* d = c + np;                           // rhs / scan values
  T* al = d + np;                          // forward scan coefficients -a_i m_i
  T* m = al + np;                          // pivots 1/(b_i - a_i c'_{i-1})
  T* cp = m + np;                          // c'_i  (backward coefficients are -c'_i)
  Aff<T>* wsum = reinterpret_cast<Aff<T>*>(cp + np);
  const int tid = threadIdx.x, nt = blockDim.x;
  const double Pe = I.Pe, Da = I.Da, dt = I.dt;
  const bool dk = I.variant == MJX_REACTOR_DANCKWERTS;
  const bool dkcn = I.variant == MJX_REACTOR_DANCKWERTS_CN;
  const double dz = (dk || dkcn) ? 1.0 / n : 1.0 / (n - 1);
  // tridiagonal entries of the implicit matrix and of the explicit operator
  double kap = 0, Ls = 0, Ld = 0, Lp = 0, Lsl = 0, Ldl = 0;
  if (dk) {
    kap = 0.5 * dt / (Pe * dz * dz);
  } else if (dkcn) {
    // M: row 0 (-2q - 1/dz - Da, q), rows 1..N-2 (q + 1/dz, -2q - 1/dz - Da, q),
    // row N-1 (2q + 1/dz, -2q - 1/dz - Da)
    const double q = (1.0 / Pe) / (dz * dz);
    Ls = q + 1.0 / dz; Ld = -2.0 * q - 1.0 / dz - Da; Lp = q;
    Lsl = 2.0 * q + 1.0 / dz; Ldl = Ld;
  } else {
    const double q = (1.0 / Pe) / (dz * dz);
    Ls = q + 1.0 / dz; Ld = -2.0 * q - 1.0 / dz - Da; Lp = q;   // rows 1..N-2
    Lsl = q; Ldl = -q - 1.0 / dz - Da;                           // row N-1
  }
  auto sub = [&](int i) -> double {  // A[i][i-1]
    if (dk) return i == n - 1 ? -2.0 * kap : -kap;
    if (i == 0) return 0.0;
    return i == n - 1 ? -0.5 * dt * Lsl : -0.5 * dt * Ls;
  };
  auto dia = [&](int i) -> double {
    if (dk) return 1.0 + 2.0 * kap;
    if (i == 0) return dkcn ? 1.0 - 0.5 * dt * Ld : 1.0;
    return i == n - 1 ? 1.0 - 0.5 * dt * Ldl : 1.0 - 0.5 * dt * Ld;
  };
  auto sup = [&](int i) -> double {  // A[i][i+1]
    if (dk) return i == n - 1 ? 0.0 : -kap;
    if (i == n - 1 || (i == 0 && !dkcn)) return 0.0;
    return -0.5 * dt * Lp;
  };
  // Thomas factorisation once (sequential, FP64)
  if (tid == 0) {
    double cprev = 0.0;
    for (int i = 0; i < n; ++i) {
      const double mi = 1.0 / (dia(i) - sub(i) * cprev);
      m[pz(i)] = (T)mi;
      al[pz(i)] = (T)(-sub(i) * mi);
      cprev = sup(i) * mi;
      cp[pz(i)] = (T)cprev;
    }
  }
  for (int i = tid; i < n; i += nt) c[pz(i)] = (T)I.c_init;
  if (!dk && !dkcn && tid == 0) c[pz(0)] = (T)I.c_inlet;
  __syncthreads();
  const T idz = (T)(1.0 / dz), Dat = (T)Da, dtt = (T)dt, kp = (T)kap;
  const T half_dt = (T)(0.5 * dt);
  for (int step = 0; step < I.n_steps; ++step) {
    // right-hand side
    for (int i = tid; i < n; i += nt) {
      const T ci = c[pz(i)];
      T r;
      if (dk) {
        const T cl = i > 0 ? c[pz(i - 1)] : (T)0, cr = i < n - 1 ? c[pz(i + 1)] : (T)0;
        T lap;  // (L c)_i dz^2
        if (i == n - 1) lap = (T)2 * cl - (T)2 * ci;
        else lap = cl - (T)2 * ci + cr;
        const T adv = i == 0 ? -(ci - (T)1) * idz : -(ci - cl) * idz;
        r = ci + kp * lap + dtt * (adv - Dat * ci);
      } else if (dkcn) {  // c + dt/2 M c + dt s
        const T cl = i > 0 ? c[pz(i - 1)] : (T)0, cr = i < n - 1 ? c[pz(i + 1)] : (T)0;
        T Mc;
        if (i == 0) Mc = (T)Ld * ci + (T)Lp * cr;
        else if (i == n - 1) Mc = (T)Lsl * cl + (T)Ldl * ci;
        else Mc = (T)Ls * cl + (T)Ld * ci + (T)Lp * cr;
        r = ci + half_dt * Mc + (i == 0 ? dtt * idz : (T)0);
      } else {
        if (i == 0) {
          r = (T)I.c_inlet;
        } else {
          const T cl = c[pz(i - 1)];
          T Lc;
          if (i == n - 1) Lc = (T)Lsl * cl + (T)Ldl * ci;
          else Lc = (T)Ls * cl + (T)Ld * ci + (T)Lp * c[pz(i + 1)];
          r = ci + half_dt * Lc;
        }
      }
      d[pz(i)] = r * m[pz(i)];  // beta_i of the forward sweep
    }
    __syncthreads();
    affine_scan<T, false>(al, d, n, wsum);      // d'_i
    // backward: x_i = d'_i - c'_i x_{i+1}; reuse c[] for the -c' coefficients
    for (int i = tid; i < n; i += nt) c[pz(i)] = -cp[pz(i)];
    __syncthreads();
    affine_scan<T, true>(c, d, n, wsum);         // x in d[]
    for (int i = tid; i < n; i += nt) c[pz(i)] = d[pz(i)];
    __syncthreads();
  }
  T* out = reinterpret_cast<T*>(A.out) + I.offset;
  for (int i = tid; i < n; i += nt) out[i] = c[pz(i)];
}

// Penalty-BC RK4 of benchmarks/benchmark_tubular_reactor.py (57-200, 254-301): n nodes,
// dz = 1/(n-1), interior rows (1/Pe) D2 c - D1 c - Da c with central D1, and the end rows
// replaced by relaxations 100 (target - c) toward the BC value (Danckwerts / Robin inlet
// (c_in + k c_1)/(1 + k), k = (1/Pe)/dz; Neumann c_1; outlet c_{n-2}, Robin written as
// (c_{n-2}/dz)/(1/dz) like the reference).  The RHS is a 3-point stencil and the state fits
// in registers: one CTA of RW warps per instance, P contiguous nodes per lane
// (n <= 32 RW P).  The stages exchange only boundary nodes: by shuffle inside a warp and
// through two shared-memory slots (alternating by stage, one barrier per stage) between
// warps.  FP64 runs at a low rate on this part and each warp issues to one SM sub-
// partition, so spreading an instance over four warps uses all four FP64 units of the SM.
enum { RW = 4 };

template <typename T, int P>
__device__ __forceinline__ void rk4_rhs(T (&s)[P], int i0, int n, int bc, T iPe, T idz2, T hidz, T Da, T kin,
                                        T cin, T idz, T* xch, int stage) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T sl = __shfl_up_sync(0xffffffffu, s[P - 1], 1);
  T sr = __shfl_down_sync(0xffffffffu, s[0], 1);
  T* slot = xch + (stage & 1) * 2 * RW;
  if (lane == 0) slot[2 * warp] = s[0];
  if (lane == 31) slot[2 * warp + 1] = s[P - 1];
  __syncthreads();
  if (lane == 0 && warp > 0) sl = slot[2 * (warp - 1) + 1];
  if (lane == 31 && warp < RW - 1) sr = slot[2 * (warp + 1)];
  // f(s) in place: each node's left neighbour is carried from the previous iteration
  // (the value before it was overwritten), so one array holds both the stage input and k
  T cm = sl;
#pragma unroll
  for (int q = 0; q < P; ++q) {
    const int i = i0 + q;
    const T cc = s[q];
    const T cp = q < P - 1 ? s[q < P - 1 ? q + 1 : 0] : sr;
    T v = iPe * ((cm - (T)2 * cc + cp) * idz2) - (cp - cm) * hidz - Da * cc;
    if (i == 0) {
      const T tgt = bc == MJX_REACTOR_RK4_NEUMANN ? cp : (cin + kin * cp) / ((T)1 + kin);
      v = (T)100 * (tgt - cc);
    } else if (i == n - 1) {
      const T tgt = bc == MJX_REACTOR_RK4_ROBIN ? (idz * cm) / idz : cm;
      v = (T)100 * (tgt - cc);
    } else if (i >= n) {
      v = (T)0;
    }
    s[q] = v;
    cm = cc;
  }
}

template <typename T, int P>
__global__ void __launch_bounds__(32 * RW) reactor_rk4_kernel(ReactorArgs A) {
  __shared__ T xch[2 * 2 * RW];
  const mjx_reactor_instance I = A.inst[blockIdx.x];
  const int n = I.n, bc = I.variant;
  T* out = reinterpret_cast<T*>(A.out) + I.offset;
  const bool ok = n >= 3 && n <= 32 * RW * P && bc >= MJX_REACTOR_RK4_DANCKWERTS && bc <= MJX_REACTOR_RK4_NEUMANN;
  if (!ok) {  // not this kernel's instance: NaN, never an out-of-range write
    for (int i = threadIdx.x; i < n && i < 32 * RW * P; i += blockDim.x) out[i] = (T)NAN;
    return;
  }
  const double dz = 1.0 / (n - 1);
  const T iPe = (T)(1.0 / I.Pe), idz2 = (T)(1.0 / (dz * dz)), hidz = (T)(0.5 / dz), Da = (T)I.Da;
  const T idz = (T)(1.0 / dz), kin = (T)((1.0 / I.Pe) / dz), cin = (T)I.c_inlet;
  const T dt = (T)I.dt, hdt = (T)(0.5 * I.dt), dt6 = (T)(I.dt / 6.0);
  const int i0 = threadIdx.x * P;
  T c[P], acc[P], y[P];
#pragma unroll
  for (int q = 0; q < P; ++q) c[q] = i0 + q < n ? (T)I.c_init : (T)0;
  for (int step = 0; step < I.n_steps; ++step) {
#pragma unroll
    for (int q = 0; q < P; ++q) y[q] = c[q];
    rk4_rhs<T, P>(y, i0, n, bc, iPe, idz2, hidz, Da, kin, cin, idz, xch, 0);  // k1
#pragma unroll
    for (int q = 0; q < P; ++q) { acc[q] = y[q]; y[q] = c[q] + hdt * y[q]; }
    rk4_rhs<T, P>(y, i0, n, bc, iPe, idz2, hidz, Da, kin, cin, idz, xch, 1);  // k2
#pragma unroll
    for (int q = 0; q < P; ++q) { acc[q] += (T)2 * y[q]; y[q] = c[q] + hdt * y[q]; }
    rk4_rhs<T, P>(y, i0, n, bc, iPe, idz2, hidz, Da, kin, cin, idz, xch, 0);  // k3
#pragma unroll
    for (int q = 0; q < P; ++q) { acc[q] += (T)2 * y[q]; y[q] = c[q] + dt * y[q]; }
    rk4_rhs<T, P>(y, i0, n, bc, iPe, idz2, hidz, Da, kin, cin, idz, xch, 1);  // k4
#pragma unroll
    for (int q = 0; q < P; ++q) c[q] = c[q] + dt6 * (acc[q] + y[q]);
  }
#pragma unroll
  for (int q = 0; q < P; ++q)
    if (i0 + q < n) out[i0 + q] = c[q];
}

}  // namespace mjx

using namespace mjx;

extern "C" {

size_t mjx_reactor_smem_bytes(int n, int dtype) {
  const int e = elem_size(dtype);
  if (!e || n < 2) return 0;
  return (size_t)5 * pz_size(n) * e + 32 * 2 * e;
}

mjx_status mjx_reactor_cn_batch(const mjx_reactor_instance* inst_dev, int n_inst, int max_n,
                                int dtype, void* out, void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!inst_dev || !out || n_inst < 0 || max_n < 2) return MJX_BAD_ARG;
  if (n_inst == 0) return MJX_OK;
  const size_t smem = mjx_reactor_smem_bytes(max_n, dtype);
  static ContextOnce attr;
  MJX_TRY(attr.run([]() -> mjx_status {
    int dev = 0, optin = 0;
    MJX_CUDA_TRY(cudaGetDevice(&dev));
    MJX_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    MJX_CUDA_TRY(cudaFuncSetAttribute(reactor_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    MJX_CUDA_TRY(cudaFuncSetAttribute(reactor_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    return MJX_OK;
  }));
  if (smem > 227 * 1024) return MJX_BAD_SHAPE;
  ReactorArgs A;
  A.inst = inst_dev; A.out = out; A.n_inst = n_inst;
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4) reactor_kernel<float><<<n_inst, 256, smem, s>>>(A);
  else reactor_kernel<double><<<n_inst, 256, smem, s>>>(A);
  return cuda_status(cudaGetLastError());
}

mjx_status mjx_reactor_rk4_batch(const mjx_reactor_instance* inst_dev, int n_inst, int max_n, int dtype,
                                 void* out, void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!inst_dev || !out || n_inst < 0 || max_n < 3) return MJX_BAD_ARG;
  if (max_n > 32 * RW * 8) return MJX_BAD_SHAPE;  // at most 8 nodes per lane
  if (n_inst == 0) return MJX_OK;
  ReactorArgs A;
  A.inst = inst_dev; A.out = out; A.n_inst = n_inst;
  cudaStream_t s = (cudaStream_t)stream;
  const int per = (max_n + 32 * RW - 1) / (32 * RW);  // nodes per lane
#define MJX_RK4_LAUNCH(PP)                                                         \
  do {                                                                             \
    if (e == 4) reactor_rk4_kernel<float, PP><<<n_inst, 32 * RW, 0, s>>>(A);       \
    else reactor_rk4_kernel<double, PP><<<n_inst, 32 * RW, 0, s>>>(A);             \
  } while (0)
  if (per <= 1) MJX_RK4_LAUNCH(1);
  else if (per <= 2) MJX_RK4_LAUNCH(2);
  else if (per <= 4) MJX_RK4_LAUNCH(4);
  else MJX_RK4_LAUNCH(8);
#undef MJX_RK4_LAUNCH
  return cuda_status(cudaGetLastError());
}

}  // extern "C"
