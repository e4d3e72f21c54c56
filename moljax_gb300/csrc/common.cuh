// Shared helpers for the moljax_gb300 CUDA kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/moljax_gb300.h"

namespace mjx {

template <typename T> struct cplx_of;
template <> struct cplx_of<float> { typedef float2 type; };
template <> struct cplx_of<double> { typedef double2 type; };
template <typename T> using cx = typename cplx_of<T>::type;

template <typename C> __device__ __forceinline__ C mk(decltype(C::x) re, decltype(C::x) im) {
  C r; r.x = re; r.y = im; return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return mk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return mk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  return mk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename C> __device__ __forceinline__ C cmulc(C a, C b) {
  return mk<C>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename C> __device__ __forceinline__ C cconj(C a) { return mk<C>(a.x, -a.y); }
template <typename C, typename S> __device__ __forceinline__ C cscale(C a, S s) {
  return mk<C>(a.x * s, a.y * s);
}

// Remembers the last CUDA error (per host thread) for mjx_last_error().
void set_last_error(cudaError_t e, const char* file, int line);

// Records a CUDA launch/runtime error as an mjx status.
static inline mjx_status cuda_status_at(cudaError_t e, const char* file, int line) {
  if (e == cudaSuccess) return MJX_OK;
  set_last_error(e, file, line);
  return MJX_CUDA_ERROR;
}
#define cuda_status(e) cuda_status_at((e), __FILE__, __LINE__)

static inline int ilog2_exact(long long n) {
  if (n <= 0 || (n & (n - 1))) return -1;
  int l = 0;
  while ((1LL << l) < n) ++l;
  return l;
}

}  // namespace mjx

#define MJX_TRY(expr)                                   \
  do {                                                  \
    mjx_status _s = (expr);                             \
    if (_s != MJX_OK) return _s;                        \
  } while (0)

namespace mjx {

// Process-unique identity (cuCtxGetId) of the CUDA context current on the
// calling thread.  When no context is current yet, the device's primary
// context is made current first (cudaSetDevice), as any runtime call would.
// Function attributes and __device__ symbol addresses belong to a context, so
// one-time set-up is keyed on this id, not on the device number: a context
// created by a driver-API host, or the new primary context after
// cudaDeviceReset, gets its own set-up.
mjx_status current_context_id(unsigned long long* id);

// Runs a set-up function once per CUDA context (thread-safe).  A failed
// set-up leaves the context unmarked, so the next call retries it.
struct ContextOnce {
  std::mutex mu;
  unsigned long long ids[32] = {};
  int n = 0;
  template <class F>
  mjx_status run(F&& setup) {
    unsigned long long id = 0;
    MJX_TRY(current_context_id(&id));
    std::lock_guard<std::mutex> lk(mu);
    const int m = n < 32 ? n : 32;
    for (int i = 0; i < m; ++i)
      if (ids[i] == id) return MJX_OK;
    MJX_TRY(setup());
    ids[n % 32] = id;  // oldest entry replaced after 32 contexts
    ++n;
    return MJX_OK;
  }
};

}  // namespace mjx

#define MJX_CUDA_TRY(expr)                                          \
  do {                                                              \
    cudaError_t _e = (expr);                                        \
    if (_e != cudaSuccess) {                                        \
      mjx::set_last_error(_e, __FILE__, __LINE__);                  \
      return MJX_CUDA_ERROR;                                        \
    }                                                               \
  } while (0)
