// Spectral multipliers on periodic 2D grids of any size (numpy/jnp.fft accept any n; the
// fused row/column passes of spectral.cu take powers of two).
//
// out_f = real(IFFT2( m(kx, ky) FFT2(in_f) )) on the full complex spectrum:
//   R   real -> complex, row DFTs of length nx          [f][y][x]
//   T   transpose                                        [f][x][y]
//   C   row DFTs of length ny, multiplier, inverse DFTs  [f][x][y]
//   T   transpose back, inverse row DFTs of length nx, real part
// A DFT of length n is the shared-memory Stockham FFT when n is a power of two, a
// mixed-radix (2, 3, 4, 5) Stockham FFT when n has no other prime factor, and
// Bluestein's chirp-z form otherwise: with c[j] = exp(-i pi j^2 / n),
//   DFT_n(z)[k] = c[k] * IFFT_L( FFT_L(z c) * FFT_L(b) )[k],  b[j] = conj(c[|j|]),
// a circular convolution of length L = 2^ceil(log2(2n - 1)) <= 4096 (n <= 2048).
// Inverse DFTs use IDFT(z) = conj(DFT(conj(z))) / n.  The multiplier of the full
// spectrum needs no Hermitian averaging: the real part is taken at the end, as the
// reference's real(ifft2(.)) does.
#include <math.h>
#include <string.h>

#include <vector>

#include "fft.cuh"
#include "autotune.cuh"

namespace mjx {

mjx_status ensure_kernel_attrs();
int elem_size(int dtype);
void set_last_error(cudaError_t e, const char* file, int line);

static inline size_t g256(size_t b) { return (b + 255) & ~size_t(255); }

struct DftGeom {
  int n, L, log2L, bluestein, mixed, nrad;
  int rad[16];
  size_t tw, chirp, bhat, total;
};

// radices 4, 2, 3, 5 covering n, or 0 if n has another prime factor
static int radix_plan(int n, int* rad) {
  int m = n, k = 0;
  const int rs[4] = {4, 2, 3, 5};
  for (int i = 0; i < 4; ++i)
    while (m % rs[i] == 0 && k < 16) { rad[k++] = rs[i]; m /= rs[i]; }
  return m == 1 ? k : 0;
}

static DftGeom dft_geom(int n, int elem) {
  DftGeom g;
  memset(&g, 0, sizeof(g));
  g.n = n;
  const bool pow2 = ilog2_exact(n) >= 0;
  g.nrad = pow2 ? 0 : radix_plan(n, g.rad);
  g.mixed = !pow2 && g.nrad > 0;
  DftTune t;
  if (g.mixed && tune_dft_get(n, elem, &t) && t.nrad > 0) {  // an autotuned schedule
    g.nrad = t.nrad;
    for (int i = 0; i < 16; ++i) g.rad[i] = t.rad[i];
  }
  g.bluestein = !pow2 && !g.mixed;
  g.L = n;
  if (g.bluestein) {
    g.L = 1;
    while (g.L < 2 * n - 1) g.L <<= 1;
  }
  g.log2L = g.mixed ? 0 : ilog2_exact(g.L);
  const size_t c = 2 * (size_t)elem;
  size_t o = 0;
  g.tw = o; o += g256(g.L * c);
  g.chirp = o; o += g256(n * c);
  g.bhat = o; o += g256(g.L * c);
  g.total = o;
  return g;
}

static bool dft_len_ok(int n) {
  if (n < 1) return false;
  if (ilog2_exact(n) >= 0) return n <= 4096;
  return n <= 2048;
}

// in-place iterative radix-2 FFT on the host (FP64), for the Bluestein filter
static void host_fft2(std::vector<double>& re, std::vector<double>& im) {
  const int n = (int)re.size();
  for (int i = 1, j = 0; i < n; ++i) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) { std::swap(re[i], re[j]); std::swap(im[i], im[j]); }
  }
  const double twopi = 6.283185307179586476925286766559;
  for (int len = 2; len <= n; len <<= 1)
    for (int i = 0; i < n; i += len)
      for (int k = 0; k < len / 2; ++k) {
        const double ang = -twopi * k / len;
        const double wr = cos(ang), wi = sin(ang);
        const int u = i + k, v = i + k + len / 2;
        const double xr = re[v] * wr - im[v] * wi, xi = re[v] * wi + im[v] * wr;
        re[v] = re[u] - xr; im[v] = im[u] - xi;
        re[u] += xr; im[u] += xi;
      }
}

template <typename T>
struct DftArgs {
  cx<T>* data;        // rows of n complex values, row stride ld
  long long nrows, ld;
  const cx<T>* tw;    // length-L twiddles (mixed radix: exp(-2 pi i m / n), m < n)
  const cx<T>* chirp; // length n
  const cx<T>* bhat;  // length L, FFT_L(b) / L
  int n, L, log2L, bluestein, nseq, inverse;
  int mixed, nrad, tpsm;  // mixed radix: passes and threads per sequence
  int rad[16];
  T scale;
};

// small forward DFTs in registers (w = exp(-2 pi i / r)); the constants are cos/sin of
// 2 pi/3, 2 pi/5, 4 pi/5
template <typename C>
__device__ __forceinline__ void sdft(C* v, int r) {
  typedef decltype(C::x) R;
  if (r == 2) {
    const C a = v[0], b = v[1];
    v[0] = cadd(a, b); v[1] = csub(a, b);
  } else if (r == 3) {
    const R h = (R)0.86602540378443864676;  // sin(2 pi / 3)
    const C a = v[0], t = cadd(v[1], v[2]), d = csub(v[1], v[2]);
    const C m = mk<C>(a.x - (R)0.5 * t.x, a.y - (R)0.5 * t.y);
    const C q = mk<C>(h * d.y, -h * d.x);  // -i h d
    v[0] = cadd(a, t); v[1] = cadd(m, q); v[2] = csub(m, q);
  } else if (r == 4) {
    const C a = v[0], b = v[1], c = v[2], d = v[3];
    const C s0 = cadd(a, c), s1 = csub(a, c), t0 = cadd(b, d), t1 = csub(b, d);
    const C jt1 = mk<C>(t1.y, -t1.x);  // -i (b - d)
    v[0] = cadd(s0, t0); v[2] = csub(s0, t0); v[1] = cadd(s1, jt1); v[3] = csub(s1, jt1);
  } else {  // r == 5
    const R c1 = (R)0.30901699437494742410, c2 = (R)-0.80901699437494742410;
    const R s1 = (R)0.95105651629515357212, s2 = (R)0.58778525229247312917;
    const C a = v[0];
    const C t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]), t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
    const C m1 = mk<C>(a.x + c1 * t1.x + c2 * t2.x, a.y + c1 * t1.y + c2 * t2.y);
    const C m2 = mk<C>(a.x + c2 * t1.x + c1 * t2.x, a.y + c2 * t1.y + c1 * t2.y);
    const C n1 = mk<C>(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
    const C n2 = mk<C>(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
    v[0] = mk<C>(a.x + t1.x + t2.x, a.y + t1.y + t2.y);
    v[1] = mk<C>(m1.x + n1.y, m1.y - n1.x);  // m1 - i n1
    v[4] = mk<C>(m1.x - n1.y, m1.y + n1.x);  // m1 + i n1
    v[2] = mk<C>(m2.x + n2.y, m2.y - n2.x);
    v[3] = mk<C>(m2.x - n2.y, m2.y + n2.x);
  }
}

// Mixed-radix Stockham DFT of lengths n = 2^a 3^b 5^c: pass (r, p) maps butterfly j
// (k = j mod p) from src[j + t n/r] to dst[(j - k) r + k + t p] after the twiddles
// w^(k t), w = exp(-2 pi i / (p r)); two shared buffers alternate between passes.
template <typename T>
__global__ void __launch_bounds__(256) dft_mixed_kernel(const __grid_constant__ DftArgs<T> a) {
  typedef cx<T> C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = a.n, T_ = a.tpsm, tid = threadIdx.x;
  C* b0 = reinterpret_cast<C*>(smem_raw);
  C* b1 = b0 + (long long)a.nseq * n;
  const int s = tid / T_, lt = tid - s * T_;
  const long long row = (long long)blockIdx.x * a.nseq + s;
  const bool active = s < a.nseq && row < a.nrows;
  C* x = a.data + row * a.ld;
  C* src = b0 + s * n;
  C* dst = b1 + s * n;
  if (active)
    for (int j = lt; j < n; j += T_) {
      C v = x[j];
      if (a.inverse) v.y = -v.y;
      src[j] = v;
    }
  __syncthreads();
  int p = 1;
  for (int q = 0; q < a.nrad; ++q) {
    const int r = a.rad[q], nb = n / r, step = n / (p * r);
    if (active)
      for (int j = lt; j < nb; j += T_) {
        const int k = j % p;
        C v[5];
        for (int t = 0; t < r; ++t) v[t] = src[j + t * nb];
        if (p > 1)
          for (int t = 1; t < r; ++t) v[t] = cmul(v[t], __ldg(&a.tw[k * t * step]));
        sdft(v, r);
        const int base = (j - k) * r + k;
        for (int t = 0; t < r; ++t) dst[base + t * p] = v[t];
      }
    __syncthreads();
    C* tmp = src; src = dst; dst = tmp;
    p *= r;
  }
  if (active)
    for (int j = lt; j < n; j += T_) {
      C v = src[j];
      if (a.inverse) v.y = -v.y;
      x[j] = mk<C>(v.x * a.scale, v.y * a.scale);
    }
}

// nseq rows per CTA, each in its own shared-memory segment of length L
template <typename T>
__global__ void __launch_bounds__(256) dft_rows_kernel(const __grid_constant__ DftArgs<T> a) {
  typedef cx<T> C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* buf = reinterpret_cast<C*>(smem_raw);
  const int L = a.L, tps = L >= 16 ? L / 16 : 1, tid = threadIdx.x;
  const int s = tid / tps, lt = tid - s * tps;
  const long long row = (long long)blockIdx.x * a.nseq + s;
  const bool active = s < a.nseq && row < a.nrows;
  const int base = s * L;
  C* x = a.data + row * a.ld;
  if (active)
    for (int j = lt; j < L; j += tps) {
      C v = mk<C>((T)0, (T)0);
      if (j < a.n) {
        v = x[j];
        if (a.inverse) v.y = -v.y;
        if (a.bluestein) v = cmul(v, __ldg(&a.chirp[j]));
      }
      buf[sp(base + j)] = v;
    }
  __syncthreads();
  fft_smem<T, false, false>(buf, L, a.log2L, a.nseq, L, 1, a.tw, tid);
  if (a.bluestein) {
    if (active)
      for (int j = lt; j < L; j += tps) buf[sp(base + j)] = cmul(buf[sp(base + j)], __ldg(&a.bhat[j]));
    __syncthreads();
    fft_smem<T, true, false>(buf, L, a.log2L, a.nseq, L, 1, a.tw, tid);
    if (active)
      for (int j = lt; j < a.n; j += tps) buf[sp(base + j)] = cmul(buf[sp(base + j)], __ldg(&a.chirp[j]));
    __syncthreads();
  }
  if (active)
    for (int j = lt; j < a.n; j += tps) {
      C v = buf[sp(base + j)];
      if (a.inverse) v.y = -v.y;
      x[j] = mk<C>(v.x * a.scale, v.y * a.scale);
    }
}

// out[b][c][r] = in[b][r][c] for rows x cols matrices, 32 x 32 tiles
template <typename T>
__global__ void transpose_kernel(const cx<T>* __restrict__ in, cx<T>* __restrict__ out, int rows, int cols) {
  __shared__ cx<T> tile[32][33];
  const long long b = blockIdx.z;
  const cx<T>* src = in + b * (long long)rows * cols;
  cx<T>* dst = out + b * (long long)rows * cols;
  const int c0 = blockIdx.x * 32;
  // row tiles in a grid-stride loop (gridDim.y is capped at 65535)
  for (int r0 = blockIdx.y * 32; r0 < rows; r0 += gridDim.y * 32) {
    for (int i = threadIdx.y; i < 32; i += 8) {
      const int r = r0 + i, c = c0 + threadIdx.x;
      if (r < rows && c < cols) tile[i][threadIdx.x] = src[(long long)r * cols + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += 8) {
      const int c = c0 + i, r = r0 + threadIdx.x;
      if (r < rows && c < cols) dst[(long long)c * rows + r] = tile[threadIdx.x][i];
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void real_to_complex_kernel(const T* __restrict__ in, cx<T>* __restrict__ out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = mk<cx<T>>(in[i], (T)0);
}

template <typename T>
__global__ void complex_real_kernel(const cx<T>* __restrict__ in, T* __restrict__ out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = in[i].x;
}

struct GenMul {
  int nx, ny, symbol, mult, nf;
  double dx, dy, h;
  double D[4], vx[4], vy[4];
};

// multiplier on the transposed spectrum [f][kx][ky]
template <typename T>
__global__ void general_mult_kernel(cx<T>* __restrict__ s, const T* __restrict__ table, const GenMul m) {
  const long long per = (long long)m.nx * m.ny, total = per * m.nf;
  const double twopi = 6.283185307179586476925286766559;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(i / per);
    const long long r = i - f * per;
    const int kx = (int)(r / m.ny), ky = (int)(r - (long long)kx * m.ny);
    const cx<T> v = s[i];
    if (m.mult == MJX_MULT_TABLE) {
      const T t = table[(long long)ky * m.nx + kx];
      s[i] = mk<cx<T>>(v.x * t, v.y * t);
      continue;
    }
    // fftfreq indices (the Nyquist index of an even length negative)
    const int mx = kx < (m.nx + 1) / 2 ? kx : kx - m.nx, my = ky < (m.ny + 1) / 2 ? ky : ky - m.ny;
    double lam;
    if (m.symbol == MJX_SYMBOL_FD) {
      lam = (2.0 * cospi(2.0 * kx / m.nx) - 2.0) / (m.dx * m.dx) + (2.0 * cospi(2.0 * ky / m.ny) - 2.0) / (m.dy * m.dy);
    } else {
      const double ax = twopi * mx / (m.nx * m.dx), ay = twopi * my / (m.ny * m.dy);
      lam = -(ax * ax + ay * ay);
    }
    const double zr = m.h * m.D[f] * lam;
    const double zi = -m.h * (m.vx[f] * twopi * mx / (m.nx * m.dx) + m.vy[f] * twopi * my / (m.ny * m.dy));
    double fr, fi;
    switch (m.mult) {
      case MJX_MULT_SCALE: fr = 1.0; fi = 0.0; break;
      case MJX_MULT_HELMHOLTZ:
      case MJX_MULT_ADV_SOLVE: {
        double dr = 1.0 - zr, di = -zi;
        if (sqrt(dr * dr + di * di) < 1e-14) { dr = 1e-14; di = 0.0; }
        const double den = dr * dr + di * di;
        fr = dr / den; fi = -di / den;
        break;
      }
      case MJX_MULT_CN:
      case MJX_MULT_ADV_CN: {
        const double nr = 1.0 + 0.5 * zr, ni = 0.5 * zi, dr = 1.0 - 0.5 * zr, di = -0.5 * zi;
        const double den = dr * dr + di * di;
        fr = (nr * dr + ni * di) / den; fi = (ni * dr - nr * di) / den;
        break;
      }
      case MJX_MULT_LAP:
      case MJX_MULT_ADV_LAP: fr = zr; fi = zi; break;
      default: {  // exp
        double sn, cs;
        sincos(zi, &sn, &cs);
        const double ez = exp(zr);
        fr = ez * cs; fi = ez * sn;
      }
    }
    const T Fr = (T)fr, Fi = (T)fi;
    s[i] = mk<cx<T>>(v.x * Fr - v.y * Fi, v.x * Fi + v.y * Fr);
  }
}

// threads per sequence tp in [1, 256] (default n/8); sequences per CTA within 256
// threads and 96 KB of shared memory
template <typename T>
static void mixed_launch(DftArgs<T>& a, int tp) {
  int T_ = tp;
  if (T_ < 1) T_ = 1;
  if (T_ > 256) T_ = 256;
  a.tpsm = T_;
  int ns = 256 / T_;
  const int cap = (int)((96 * 1024) / (2 * (size_t)a.n * sizeof(cx<T>)));
  if (ns > cap) ns = cap;
  a.nseq = ns < 1 ? 1 : ns;
}

template <typename T>
static DftArgs<T> dft_args(const void* plan, int n, cx<T>* data, long long nrows, long long ld, int inverse) {
  const DftGeom g = dft_geom(n, sizeof(T));
  const char* p = (const char*)plan;
  DftArgs<T> a;
  memset(&a, 0, sizeof(a));
  a.data = data; a.nrows = nrows; a.ld = ld;
  a.tw = (const cx<T>*)(p + g.tw); a.chirp = (const cx<T>*)(p + g.chirp); a.bhat = (const cx<T>*)(p + g.bhat);
  a.n = n; a.L = g.L; a.log2L = g.log2L; a.bluestein = g.bluestein; a.inverse = inverse;
  a.mixed = g.mixed; a.nrad = g.nrad;
  for (int i = 0; i < 16; ++i) a.rad[i] = g.rad[i];
  if (g.mixed) {
    DftTune t;
    const int tp = (tune_dft_get(n, (int)sizeof(T), &t) && t.tpsm > 0) ? t.tpsm : n / 8;
    mixed_launch(a, tp);
  } else {
    const int tps = g.L >= 16 ? g.L / 16 : 1;
    a.nseq = tps >= 256 ? 1 : 256 / tps;
  }
  a.scale = (T)(inverse ? 1.0 / n : 1.0);
  return a;
}

template <typename T>
static cudaError_t dft_rows(const DftArgs<T>& a, cudaStream_t s) {
  if (a.mixed) {
    const long long grid = (a.nrows + a.nseq - 1) / a.nseq;
    const size_t smem = (size_t)2 * a.nseq * a.n * sizeof(cx<T>);
    dft_mixed_kernel<T><<<(unsigned)grid, a.nseq * a.tpsm, smem, s>>>(a);
    return cudaGetLastError();
  }
  const int tps = a.L >= 16 ? a.L / 16 : 1;
  const long long grid = (a.nrows + a.nseq - 1) / a.nseq;
  const size_t smem = (size_t)sp_size(a.nseq * a.L) * sizeof(cx<T>);
  dft_rows_kernel<T><<<(unsigned)grid, a.nseq * tps, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename T>
static cudaError_t transpose(const cx<T>* in, cx<T>* out, int rows, int cols, int batch, cudaStream_t s) {
  const int ty = (rows + 31) / 32;
  dim3 grid((cols + 31) / 32, ty < 65535 ? ty : 65535, batch), block(32, 8);
  transpose_kernel<T><<<grid, block, 0, s>>>(in, out, rows, cols);
  return cudaGetLastError();
}

template <typename T>
static mjx_status general_apply(const void* plan_y, const void* plan_x, const mjx_grid2d* g, int symbol, int nf,
                                const double* D, const double* vx, const double* vy, double h, int mult,
                                const T* table, const T* in, T* out, void* ws, cudaStream_t s) {
  const int ny = g->ny, nx = g->nx;
  const long long per = (long long)ny * nx, n = per * nf;
  cx<T>* A = (cx<T>*)ws;
  cx<T>* B = A + n;
  const int threads = 256, blocks = 152 * 8;
  real_to_complex_kernel<T><<<blocks, threads, 0, s>>>(in, A, n);
  MJX_CUDA_TRY(cudaGetLastError());
  MJX_CUDA_TRY(dft_rows<T>(dft_args<T>(plan_x, nx, A, (long long)nf * ny, nx, 0), s));
  MJX_CUDA_TRY(transpose<T>(A, B, ny, nx, nf, s));
  MJX_CUDA_TRY(dft_rows<T>(dft_args<T>(plan_y, ny, B, (long long)nf * nx, ny, 0), s));
  GenMul m;
  memset(&m, 0, sizeof(m));
  m.nx = nx; m.ny = ny; m.symbol = symbol; m.mult = mult; m.nf = nf; m.dx = g->dx; m.dy = g->dy; m.h = h;
  for (int f = 0; f < nf; ++f) {
    m.D[f] = D ? D[f] : 0.0;
    m.vx[f] = vx ? vx[f] : 0.0;
    m.vy[f] = vy ? vy[f] : 0.0;
  }
  general_mult_kernel<T><<<blocks, threads, 0, s>>>(B, table, m);
  MJX_CUDA_TRY(cudaGetLastError());
  MJX_CUDA_TRY(dft_rows<T>(dft_args<T>(plan_y, ny, B, (long long)nf * nx, ny, 1), s));
  MJX_CUDA_TRY(transpose<T>(B, A, nx, ny, nf, s));
  MJX_CUDA_TRY(dft_rows<T>(dft_args<T>(plan_x, nx, A, (long long)nf * ny, nx, 1), s));
  complex_real_kernel<T><<<blocks, threads, 0, s>>>(A, out, n);
  MJX_CUDA_TRY(cudaGetLastError());
  return MJX_OK;
}

struct GenMul3 {
  int nx, ny, nz, symbol, mult;
  double dx, dy, dz, h, D;
};

// multiplier on the spectrum laid out [kx][ky][kz]
template <typename T>
__global__ void general_mult3_kernel(cx<T>* __restrict__ s, const GenMul3 m) {
  const long long total = (long long)m.nx * m.ny * m.nz;
  const double twopi = 6.283185307179586476925286766559;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int kz = (int)(i % m.nz);
    const long long r = i / m.nz;
    const int ky = (int)(r % m.ny), kx = (int)(r / m.ny);
    double lam;
    if (m.symbol == MJX_SYMBOL_FD) {
      lam = (2.0 * cospi(2.0 * kx / m.nx) - 2.0) / (m.dx * m.dx) + (2.0 * cospi(2.0 * ky / m.ny) - 2.0) / (m.dy * m.dy) +
            (2.0 * cospi(2.0 * kz / m.nz) - 2.0) / (m.dz * m.dz);
    } else {
      const int mx = kx < (m.nx + 1) / 2 ? kx : kx - m.nx, my = ky < (m.ny + 1) / 2 ? ky : ky - m.ny;
      const int mz = kz < (m.nz + 1) / 2 ? kz : kz - m.nz;
      const double ax = twopi * mx / (m.nx * m.dx), ay = twopi * my / (m.ny * m.dy), az = twopi * mz / (m.nz * m.dz);
      lam = -(ax * ax + ay * ay + az * az);
    }
    const double z = m.h * m.D * lam;
    double f;
    switch (m.mult) {
      case MJX_MULT_SCALE: f = 1.0; break;
      case MJX_MULT_HELMHOLTZ: {
        double den = 1.0 - z;
        if (fabs(den) < 1e-14) den = 1e-14;
        f = 1.0 / den;
        break;
      }
      case MJX_MULT_CN: f = (1.0 + 0.5 * z) / (1.0 - 0.5 * z); break;
      case MJX_MULT_LAP: f = z; break;
      default: f = exp(z);
    }
    const cx<T> v = s[i];
    s[i] = mk<cx<T>>(v.x * (T)f, v.y * (T)f);
  }
}

// one application on [nz][ny][nx]: x DFTs, per-plane transpose -> [z][x][y], y DFTs,
// transpose (nz x nx ny) -> [x][y][z], z DFTs, multiplier, and back
template <typename T>
static mjx_status general_apply3(const void* pz, const void* py, const void* px, const mjx_grid3d* g, int symbol,
                                 double D, double h, int mult, const T* in, T* out, void* ws, cudaStream_t s) {
  const int nz = g->nz, ny = g->ny, nx = g->nx;
  const long long n = (long long)nz * ny * nx;
  cx<T>* A = (cx<T>*)ws;
  cx<T>* B = A + n;
  const int threads = 256, blocks = 152 * 8;
  real_to_complex_kernel<T><<<blocks, threads, 0, s>>>(in, A, n);
  MJX_CUDA_TRY(cudaGetLastError());
  MJX_CUDA_TRY(dft_rows<T>(dft_args<T>(px, nx, A, (long long)nz * ny, nx, 0), s));
  MJX_CUDA_TRY(transpose<T>(A, B, ny, nx, nz, s));                     // [z][x][y]
  MJX_CUDA_TRY(dft_rows<T>(dft_args<T>(py, ny, B, (long long)nz * nx, ny, 0), s));
  MJX_CUDA_TRY(transpose<T>(B, A, nz, nx * ny, 1, s));                 // [x][y][z]
  MJX_CUDA_TRY(dft_rows<T>(dft_args<T>(pz, nz, A, (long long)nx * ny, nz, 0), s));
  GenMul3 m;
  m.nx = nx; m.ny = ny; m.nz = nz; m.symbol = symbol; m.mult = mult;
  m.dx = g->dx; m.dy = g->dy; m.dz = g->dz; m.h = h; m.D = D;
  general_mult3_kernel<T><<<blocks, threads, 0, s>>>(A, m);
  MJX_CUDA_TRY(cudaGetLastError());
  MJX_CUDA_TRY(dft_rows<T>(dft_args<T>(pz, nz, A, (long long)nx * ny, nz, 1), s));
  MJX_CUDA_TRY(transpose<T>(A, B, nx * ny, nz, 1, s));                 // [z][x][y]
  MJX_CUDA_TRY(dft_rows<T>(dft_args<T>(py, ny, B, (long long)nz * nx, ny, 1), s));
  MJX_CUDA_TRY(transpose<T>(B, A, nx, ny, nz, s));                     // [z][y][x]
  MJX_CUDA_TRY(dft_rows<T>(dft_args<T>(px, nx, A, (long long)nz * ny, nx, 1), s));
  complex_real_kernel<T><<<blocks, threads, 0, s>>>(A, out, n);
  MJX_CUDA_TRY(cudaGetLastError());
  return MJX_OK;
}

static mjx_status set_dft_attrs() {
  static ContextOnce once;
  return once.run([]() -> mjx_status {
    int dev = 0, optin = 0;
    MJX_CUDA_TRY(cudaGetDevice(&dev));
    MJX_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    MJX_CUDA_TRY(cudaFuncSetAttribute(dft_rows_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    MJX_CUDA_TRY(cudaFuncSetAttribute(dft_rows_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    MJX_CUDA_TRY(cudaFuncSetAttribute(dft_mixed_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    MJX_CUDA_TRY(cudaFuncSetAttribute(dft_mixed_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    return MJX_OK;
  });
}

}  // namespace mjx

using namespace mjx;

extern "C" {

size_t mjx_dftn_plan_bytes(int n, int dtype) {
  const int e = elem_size(dtype);
  if (!e || !dft_len_ok(n)) return 0;
  return dft_geom(n, e).total;
}

mjx_status mjx_dftn_plan_init(void* plan, int n, int dtype, void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!plan || !dft_len_ok(n)) return MJX_BAD_ARG;
  const DftGeom g = dft_geom(n, e);
  std::vector<unsigned char> host(g.total, 0);
  auto put = [&](size_t off, int i, double re, double im) {
    if (e == 4) { float* q = (float*)(host.data() + off); q[2 * i] = (float)re; q[2 * i + 1] = (float)im; }
    else { double* q = (double*)(host.data() + off); q[2 * i] = re; q[2 * i + 1] = im; }
  };
  const double twopi = 6.283185307179586476925286766559, pi = 0.5 * twopi;
  for (int j = 0; j < g.L; ++j) put(g.tw, j, cos(twopi * j / g.L), -sin(twopi * j / g.L));  // L = n when mixed
  if (g.bluestein) {
    std::vector<double> cre(n), cim(n);
    for (int j = 0; j < n; ++j) {  // exp(-i pi j^2 / n), j^2 reduced mod 2n to keep the angle exact
      const long long r = ((long long)j * j) % (2LL * n);
      cre[j] = cos(pi * (double)r / n);
      cim[j] = -sin(pi * (double)r / n);
      put(g.chirp, j, cre[j], cim[j]);
    }
    std::vector<double> bre(g.L, 0.0), bim(g.L, 0.0);
    for (int j = 0; j < n; ++j) {
      bre[j] = cre[j]; bim[j] = -cim[j];
      if (j > 0) { bre[g.L - j] = cre[j]; bim[g.L - j] = -cim[j]; }
    }
    host_fft2(bre, bim);
    for (int j = 0; j < g.L; ++j) put(g.bhat, j, bre[j] / g.L, bim[j] / g.L);
  }
  cudaStream_t s = (cudaStream_t)stream;
  MJX_CUDA_TRY(cudaMemcpyAsync(plan, host.data(), g.total, cudaMemcpyHostToDevice, s));
  MJX_CUDA_TRY(cudaStreamSynchronize(s));
  return MJX_OK;
}

size_t mjx_spectral_general2d_ws_bytes(int ny, int nx, int nfields, int dtype) {
  const int e = elem_size(dtype);
  if (!e || !dft_len_ok(ny) || !dft_len_ok(nx) || nfields < 1 || nfields > 4) return 0;
  return (size_t)2 * nfields * ny * nx * 2 * e;
}

mjx_status mjx_spectral_apply_general2d(const void* plan_y, const void* plan_x, const mjx_grid2d* g, int symbol,
                                        int dtype, int nfields, const double* D, const double* vx,
                                        const double* vy, double h, int mult, const void* table,
                                        const void* in, void* out, void* ws, size_t ws_bytes, void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!g || !plan_y || !plan_x || !in || !out || nfields < 1 || nfields > 4) return MJX_BAD_ARG;
  if (!dft_len_ok(g->ny) || !dft_len_ok(g->nx)) return MJX_BAD_SHAPE;
  if (!(g->dx > 0) || !(g->dy > 0)) return MJX_BAD_ARG;
  if (symbol != MJX_SYMBOL_FD && symbol != MJX_SYMBOL_SPECTRAL) return MJX_BAD_ARG;
  const bool ok_mult = mult == MJX_MULT_SCALE || mult == MJX_MULT_HELMHOLTZ || mult == MJX_MULT_CN ||
                       mult == MJX_MULT_EXP || mult == MJX_MULT_LAP || mult == MJX_MULT_TABLE ||
                       mult == MJX_MULT_ADV_SOLVE || mult == MJX_MULT_ADV_LAP || mult == MJX_MULT_ADV_EXP ||
                       mult == MJX_MULT_ADV_CN;
  if (!ok_mult || (mult == MJX_MULT_TABLE && !table)) return MJX_BAD_ARG;
  if (!ws || ws_bytes < mjx_spectral_general2d_ws_bytes(g->ny, g->nx, nfields, dtype)) return MJX_WORKSPACE;
  MJX_TRY(set_dft_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  if (e == 4)
    return general_apply<float>(plan_y, plan_x, g, symbol, nfields, D, vx, vy, h, mult, (const float*)table,
                                (const float*)in, (float*)out, ws, s);
  return general_apply<double>(plan_y, plan_x, g, symbol, nfields, D, vx, vy, h, mult, (const double*)table,
                               (const double*)in, (double*)out, ws, s);
}

size_t mjx_spectral_general3d_ws_bytes(int nz, int ny, int nx, int dtype) {
  const int e = elem_size(dtype);
  if (!e || !dft_len_ok(nz) || !dft_len_ok(ny) || !dft_len_ok(nx)) return 0;
  return (size_t)2 * nz * ny * nx * 2 * e;
}

mjx_status mjx_spectral_apply_general3d(const void* plan_z, const void* plan_y, const void* plan_x,
                                        const mjx_grid3d* g, int symbol, int dtype, double D, double h, int mult,
                                        int n_steps, const void* in, void* out, void* ws, size_t ws_bytes,
                                        void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!g || !plan_z || !plan_y || !plan_x || !in || !out || n_steps < 1) return MJX_BAD_ARG;
  if (!dft_len_ok(g->nz) || !dft_len_ok(g->ny) || !dft_len_ok(g->nx)) return MJX_BAD_SHAPE;
  if (!(g->dx > 0) || !(g->dy > 0) || !(g->dz > 0)) return MJX_BAD_ARG;
  if (symbol != MJX_SYMBOL_FD && symbol != MJX_SYMBOL_SPECTRAL) return MJX_BAD_ARG;
  if (mult != MJX_MULT_SCALE && mult != MJX_MULT_HELMHOLTZ && mult != MJX_MULT_CN && mult != MJX_MULT_EXP &&
      mult != MJX_MULT_LAP)
    return MJX_BAD_ARG;
  if (!ws || ws_bytes < mjx_spectral_general3d_ws_bytes(g->nz, g->ny, g->nx, dtype)) return MJX_WORKSPACE;
  MJX_TRY(set_dft_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  for (int i = 0; i < n_steps; ++i) {  // each application a full transform pair
    const void* src = i == 0 ? in : out;
    mjx_status st = e == 4 ? general_apply3<float>(plan_z, plan_y, plan_x, g, symbol, D, h, mult, (const float*)src,
                                                   (float*)out, ws, s)
                           : general_apply3<double>(plan_z, plan_y, plan_x, g, symbol, D, h, mult,
                                                    (const double*)src, (double*)out, ws, s);
    if (st != MJX_OK) return st;
  }
  return MJX_OK;
}

}  // extern "C"

// Autotuner of the mixed-radix row DFT of length n: every candidate schedule
// (dft_schedules) with threads per sequence n/4, n/8 and n/16 is timed on nrows rows of
// scratch (one warm-up launch, then reps launches between CUDA events); the fastest is
// installed in the registry for n and this element size.
template <typename T>
static mjx_status tune_dft(const void* plan, int n, long long nrows, cx<T>* data, int reps, double* times,
                           int max_times, int* n_cand, int* best, cudaStream_t s) {
  int sched[64 * 17];
  const int ns = dft_schedules(n, sched, 64);
  if (ns == 0) return MJX_BAD_ARG;
  int tps[3] = {n / 4, n / 8, n / 16}, ntp = 0;
  int uniq[3];
  for (int i = 0; i < 3; ++i) {
    int v = tps[i] < 1 ? 1 : (tps[i] > 256 ? 256 : tps[i]);
    bool dup = false;
    for (int j = 0; j < ntp; ++j) dup |= uniq[j] == v;
    if (!dup) uniq[ntp++] = v;
  }
  tune_dft_clear(n, (int)sizeof(T));
  DftArgs<T> a = dft_args<T>(plan, n, data, nrows, n, 0);
  cudaEvent_t e0, e1;
  MJX_CUDA_TRY(cudaEventCreate(&e0));
  MJX_CUDA_TRY(cudaEventCreate(&e1));
  double best_t = 1e300;
  int best_i = -1, k = 0;
  mjx_status st = MJX_OK;
  for (int i = 0; i < ns && st == MJX_OK; ++i) {
    for (int j = 0; j < ntp && st == MJX_OK; ++j, ++k) {
      a.nrad = sched[17 * i];
      for (int q = 0; q < 16; ++q) a.rad[q] = sched[17 * i + 1 + q];
      mixed_launch(a, uniq[j]);
      cudaError_t ce = dft_rows<T>(a, s);
      if (ce == cudaSuccess) ce = cudaEventRecord(e0, s);
      for (int r = 0; r < reps && ce == cudaSuccess; ++r) ce = dft_rows<T>(a, s);
      if (ce == cudaSuccess) ce = cudaEventRecord(e1, s);
      if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
      if (ce != cudaSuccess) { set_last_error(ce, __FILE__, __LINE__); st = MJX_CUDA_ERROR; break; }
      const double tpl = (double)ms / reps;
      if (times && k < max_times) times[k] = tpl;
      if (tpl < best_t) { best_t = tpl; best_i = k; }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != MJX_OK) return st;
  const int bi = best_i / ntp, bj = best_i - bi * ntp;
  DftTune t;
  memset(&t, 0, sizeof(t));
  t.nrad = sched[17 * bi];
  for (int q = 0; q < 16; ++q) t.rad[q] = sched[17 * bi + 1 + q];
  t.tpsm = uniq[bj];
  tune_dft_put(n, (int)sizeof(T), t);
  if (n_cand) *n_cand = ns * ntp;
  if (best) *best = best_i;
  return MJX_OK;
}

mjx_status mjx_autotune_dft(const void* plan, int n, int dtype, long long nrows, void* scratch,
                            size_t scratch_bytes, int reps, double* times, int max_times, int* n_cand,
                            int* best, void* stream) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!plan || !scratch || !dft_len_ok(n) || nrows < 1 || reps < 1) return MJX_BAD_ARG;
  if (scratch_bytes < (size_t)nrows * n * 2 * e) return MJX_WORKSPACE;
  const DftGeom g = dft_geom(n, e);
  if (!g.mixed) {
    if (n_cand) *n_cand = 0;  // powers of two and Bluestein lengths have no schedule to tune
    if (best) *best = -1;
    return MJX_OK;
  }
  MJX_TRY(set_dft_attrs());
  cudaStream_t s = (cudaStream_t)stream;
  MJX_CUDA_TRY(cudaMemsetAsync(scratch, 0, (size_t)nrows * n * 2 * e, s));
  if (e == 4)
    return tune_dft<float>(plan, n, nrows, (cx<float>*)scratch, reps, times, max_times, n_cand, best, s);
  return tune_dft<double>(plan, n, nrows, (cx<double>*)scratch, reps, times, max_times, n_cand, best, s);
}

mjx_status mjx_dft_schedule_get(int n, int dtype, int* nrad, int* rad, int* tpsm) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (!nrad || !rad || !tpsm || !dft_len_ok(n)) return MJX_BAD_ARG;
  const DftGeom g = dft_geom(n, e);
  *nrad = g.mixed ? g.nrad : 0;
  for (int i = 0; i < 16; ++i) rad[i] = g.mixed ? g.rad[i] : 0;
  DftTune t;
  *tpsm = g.mixed ? ((tune_dft_get(n, e, &t) && t.tpsm > 0) ? t.tpsm : (n / 8 < 1 ? 1 : (n / 8 > 256 ? 256 : n / 8))) : 0;
  return MJX_OK;
}
