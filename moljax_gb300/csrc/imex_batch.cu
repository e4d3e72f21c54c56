// Batched adaptive IMEX-Strang for many Gray-Scott solves of different grid
// sizes (the served workload): one launch per attempt stage covers every
// admitted instance, each with its own step size, controller state, accept
// mask and status.
//
// Each instance runs the mixed-precision attempt of csrc/imex_mixed.cu (float-
// float spectral state, FP32 increment transforms, six passes C1 R1 C2 R2 C3 R3)
// and the same controller (csrc/controller.cuh).  An instance table in device
// memory holds every instance's geometry, buffers (in its own caller-provided
// workspace), parameters and DevState.  The host turns the table into a work
// list per pass: one entry per (instance, job, tile) for the column passes and
// per (instance, row kind, row block) for the row passes.  Each pass kernel
// runs one CTA per entry of its list; CTAs of instances that are done return
// at entry.  The batched controller (one warp
// per instance) reduces each instance's error partials, applies the PI /
// accept-reject update and decides whether the epoch goes on.
//
// The attempt loop is a CUDA graph with a conditional while node; the kernels
// read the table and the epoch header from device memory.  The graph is
// rebuilt only when the set of running instances changed since the last epoch
// (its launch grids are the work-list lengths).  An epoch ends, at an
// attempt boundary, when no instance is running, when a set number of
// instances has finished, after a cap of attempts, or when the host raises the
// stop flag (mapped pinned memory, read by the controller) to admit arrivals.
#include <math.h>
#include <string.h>

#include <vector>

#include "controller.cuh"
#include "mixed.cuh"

namespace mjx {

mjx_status ensure_kernel_attrs();
mjx_status check_grid(const mjx_grid2d* g);
int elem_size(int dtype);

enum { BT = 256 };           // threads per CTA of the batched pass kernels
enum { BPASS_C1 = 0, BPASS_R1 = 1, BPASS_C2 = 2, BPASS_R2 = 3, BPASS_C3 = 4, BPASS_R3 = 5, BNPASS = 6 };
enum { SLOT_FREE = 0, SLOT_RUNNING = 1, SLOT_FINISHED = 2 };

// One instance (device table entry).
struct BInst {
  DevState st;
  int ny, nx, log2ny, log2nx, ldc, ncols;
  int colC;                  // columns per column work item (2048 / ny, at most 32)
  int rseq;                  // row pairs per row work item (min(4096 / nx, ny))
  int nblk;                  // row blocks per row kind (ny / rseq)
  int nparts;                // R3 work items = error partials (2 nblk)
  long long fs;              // complex elements per field spectrum
  float4* ys[2];
  float4* pa;
  float4* pb;
  float2* za;
  float2* zb;
  const float2* twx;
  const float2* twy;
  const float* lamx;
  const float* lamy;
  double* partial;
  int* nonfinite;
  double* hist_t;
  double* hist_dt;
  double D[2];
  double F, k;
  double n_dof;
  float inv_norm;
  int pad;
  mjx_pid_params pid;
};

// Epoch header (device).
struct BEng {
  int halt;                  // set by the controller: the epoch is over, every kernel returns at entry
  int n_slots;               // table entries 0 .. n_slots-1 are scanned by the controller
  int attempts;              // attempts run in this epoch
  int max_attempts;          // epoch cap
  int stop_after_finished;   // end the epoch once this many instances finished in it (0: never)
  int finished;              // instances that finished in this epoch
  int running;               // instances still running after the last controller
  int pad;
  int nwork[BNPASS];
  const volatile int* host_stop;  // mapped pinned host flag (may be null)
};

struct BArgs {
  BInst* tab;
  BEng* eng;
  const unsigned* work[BNPASS];
};

// work item: instance (12 bits) | job or row kind (4 bits) | tile or row block (16 bits)
__host__ __device__ __forceinline__ unsigned witem(int inst, int job, int blk) {
  return ((unsigned)inst << 20) | ((unsigned)job << 16) | (unsigned)blk;
}

// ------------------------------------------------------------------ column passes
// One CTA per work item (the grid is the pass's work count, fixed when the engine's
// graph is built for the current set of solves).  A grid-stride loop over the items
// would keep the transforms from unrolling: their register arrays then go to local
// memory (measured with -Xptxas -v: kilobytes of spills per thread, none this way).
template <int PASS>
__device__ __forceinline__ void bcol_item(float2* buf, const BInst* I, unsigned it) {
  const int job = (it >> 16) & 15, tile = it & 0xffff;
  const int f = job;
  const int cur = I->st.cur;
  const double h = I->st.dtc;
  MColTile t;
  t.ny = I->ny; t.log2ny = I->log2ny; t.ncols = I->ncols; t.C = I->colC;
  t.type = PASS == BPASS_C1 ? MC_SPLIT : (PASS == BPASS_C3 ? MC_HALF_END : MC_MID_BOTH);
  t.kx0 = tile * I->colC;
  t.ldc = I->ldc; t.off = (long long)f * I->fs;
  t.ys_cur = I->ys[cur]; t.ys_next = I->ys[1 - cur];
  t.pa = I->pa; t.pb = I->pb; t.za = I->za; t.zb = I->zb;
  t.lamx = I->lamx; t.lamy = I->lamy; t.tw = I->twy;
  t.hA = (float)(0.5 * h * I->D[f]); t.hB = (float)(0.25 * h * I->D[f]); t.nrm = I->inv_norm;
  mcol_tile(buf, t, threadIdx.x, BT);
}

template <int PASS>
__global__ void __launch_bounds__(BT, 4) bcol_kernel(const __grid_constant__ BArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* buf = reinterpret_cast<float2*>(smem_raw);
  const BEng* eng = a.eng;
  if (eng->halt) return;
  const int nw = eng->nwork[PASS];
  const unsigned* work = a.work[PASS];
  const int w = blockIdx.x;
  if (w >= nw) return;
  const unsigned it = work[w];
  const BInst* I = a.tab + (it >> 20);
  if (I->st.done) return;  // uniform over the CTA
  bcol_item<PASS>(buf, I, it);
}

// ------------------------------------------------------------------ row passes
// One row work item: rseq row pairs of one instance.  R1 / R2: the pair (u_y, v_y) of a
// row spectrum (ZA or ZB) -> c2r -> Heun reaction increment of step hfac*dtc -> r2c.
// R3: the pair (error row, solution row) of one field -> (e / (atol + rtol |y|))^2 summed
// into the item's partial.
template <int PASS>
__device__ __forceinline__ void brow_item(float2* buf, const BInst* I, unsigned it) {
  const int tid = threadIdx.x;
  {
    const int kind = (it >> 16) & 15, blk = it & 0xffff;
    const int n = I->nx, half = n >> 1, log2n = I->log2nx;
    const int tps = n >> 4;
    const int nseq = I->rseq;
    const int s_loc = tid / tps, lt = tid - s_loc * tps;
    const bool active = s_loc < nseq;
    const long long y = (long long)blk * nseq + s_loc;
    const long long ldc = I->ldc, fs = I->fs;
    // spectrum rows of this pair
    const float2* base;
    long long sa, sb;
    if (PASS == BPASS_R3) {  // field kind: (ZA_f, ZB_f)
      base = I->za;
      sa = kind * fs;
      sb = (I->zb - I->za) + kind * fs;
    } else {                 // (u, v) of ZA (R1 kind 0) or ZB (R1 kind 1, R2)
      base = (PASS == BPASS_R1 && kind == 0) ? I->za : I->zb;
      sa = 0;
      sb = fs;
    }
    const int zb0 = s_loc * n;
#define Z(x) buf[sp(zb0 + (x))]
    if (active) {
      const float2* A = base + sa + y * ldc;
      const float2* B = base + sb + y * ldc;
      float2 Ak[9], Bk[9];
#pragma unroll
      for (int m = 0; m < 9; ++m) {
        const int kk = lt + m * tps;
        if (kk <= half) { Ak[m] = A[kk]; Bk[m] = B[kk]; }
      }
#pragma unroll
      for (int m = 0; m < 9; ++m) {
        const int kk = lt + m * tps;
        if (kk <= half) {
          Z(kk) = fmk(Ak[m].x - Bk[m].y, Ak[m].y + Bk[m].x);                                  // A_k + i B_k
          if (kk > 0 && kk < half) Z(n - kk) = fmk(Ak[m].x + Bk[m].y, Bk[m].x - Ak[m].y);    // conj(A_k) + i conj(B_k)
        }
      }
    }
    __syncthreads();
    fft_smem<float, true, false>(buf, n, log2n, nseq, n, 1, I->twx, tid);
    if (PASS == BPASS_R3) {
      const float atol = (float)I->pid.atol, rtol = (float)I->pid.rtol;
      float esum = 0.f;
      int bad = 0;
      if (active) {
#pragma unroll
        for (int m = 0; m < 16; ++m) {
          const int x = lt + m * tps;
          if (x >= n) continue;
          const float2 v = Z(x);
          const float d = v.x / (atol + rtol * fabsf(v.y));
          esum += d * d;
          bad |= !(isfinite(v.x) && isfinite(v.y));
        }
      }
      __shared__ double red[BT / 32];
      __shared__ int redbad[BT / 32];
      double v = (double)esum;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_xor_sync(0xffffffffu, v, o);
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
      }
      if ((tid & 31) == 0) { red[tid >> 5] = v; redbad[tid >> 5] = bad; }
      __syncthreads();
      if (tid == 0) {
        double s = 0.0, c = 0.0;  // Kahan over the warps
        int b2 = 0;
        for (int i = 0; i < BT / 32; ++i) {
          const double yv = red[i] - c;
          const double tv = s + yv;
          c = (tv - s) - yv;
          s = tv;
          b2 |= redbad[i];
        }
        I->partial[kind * I->nblk + blk] = s;
        I->nonfinite[kind * I->nblk + blk] = b2;
      }
    } else {
      const float h = (float)(I->st.dtc * ((PASS == BPASS_R1 && kind == 0) ? 1.0 : 0.5));
      const float pF = (float)I->F, pK = (float)I->k, pR = 0.f;
      if (active) {
#pragma unroll
        for (int m = 0; m < 16; ++m) {
          const int x = lt + m * tps;
          if (x >= n) continue;
          const float2 v = Z(x);
          float va = v.x, vb = v.y;
          react_delta<float, RX_GRAY_SCOTT>(va, vb, h, pF, pK, pR);
          Z(x) = fmk(va, vb);
        }
      }
      __syncthreads();
      fft_smem<float, false, false>(buf, n, log2n, nseq, n, 1, I->twx, tid);
      if (active) {
        float2* A = const_cast<float2*>(base) + sa + y * ldc;
        float2* B = const_cast<float2*>(base) + sb + y * ldc;
#pragma unroll
        for (int m = 0; m < 9; ++m) {
          const int kk = lt + m * tps;
          if (kk > half) continue;
          const float2 Zk = Z(kk), Zm = Z((n - kk) & (n - 1));
          A[kk] = fmk(0.5f * (Zk.x + Zm.x), 0.5f * (Zk.y - Zm.y));
          B[kk] = fmk(0.5f * (Zk.y + Zm.y), 0.5f * (Zm.x - Zk.x));
        }
      }
    }
#undef Z
  }
}

template <int PASS>
__global__ void __launch_bounds__(BT, 4) brow_kernel(const __grid_constant__ BArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* buf = reinterpret_cast<float2*>(smem_raw);
  const BEng* eng = a.eng;
  if (eng->halt) return;
  const int nw = eng->nwork[PASS];
  const unsigned* work = a.work[PASS];
  const int w = blockIdx.x;
  if (w >= nw) return;
  const unsigned it = work[w];
  const BInst* I = a.tab + (it >> 20);
  if (I->st.done) return;  // uniform over the CTA
  brow_item<PASS>(buf, I, it);
}

// ------------------------------------------------------------------ controller
// One CTA: warp i handles instances i, i + 32, ...; thread 0 then decides whether the
// epoch goes on and sets the conditional node.
__global__ void __launch_bounds__(1024) bctl_kernel(const __grid_constant__ BArgs a,
                                                   cudaGraphConditionalHandle handle) {
  BEng* eng = a.eng;
  __shared__ int s_run, s_fin;
  if (eng->halt) {
    if (threadIdx.x == 0) cudaGraphSetConditional(handle, 0u);
    return;
  }
  if (threadIdx.x == 0) { s_run = 0; s_fin = 0; }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  int run_local = 0, fin_local = 0;
  for (int i = wid; i < eng->n_slots; i += nwarps) {
    BInst* I = a.tab + i;
    if (I->st.done) continue;
    double s = 0.0, c = 0.0;
    int bad = 0;
    for (int p = lane; p < I->nparts; p += 32) {  // Kahan per lane
      const double yv = I->partial[p] - c;
      const double tv = s + yv;
      c = (tv - s) - yv;
      s = tv;
      bad |= I->nonfinite[p];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_xor_sync(0xffffffffu, s, o);
      bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if (lane == 0) {
      const bool running = ctl_update(&I->st, s, bad, I->n_dof, I->pid, I->hist_t, I->hist_dt);
      if (running) ++run_local; else ++fin_local;
    }
  }
  if (lane == 0) {
    if (run_local) atomicAdd(&s_run, run_local);
    if (fin_local) atomicAdd(&s_fin, fin_local);
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  eng->attempts += 1;
  eng->finished += s_fin;
  eng->running = s_run;
  const bool stop_req = eng->host_stop != nullptr && *eng->host_stop != 0;
  const bool go_on = s_run > 0 && eng->attempts < eng->max_attempts &&
                     !(eng->stop_after_finished > 0 && eng->finished >= eng->stop_after_finished) && !stop_req;
  if (!go_on) eng->halt = 1;
  cudaGraphSetConditional(handle, go_on ? 1u : 0u);
}

// ------------------------------------------------------------------ host engine
struct InstLayout {
  size_t ys0, ys1, pa, pb, za, zb, plan32, plan64, part, bad, ht, hdt, total;
};

static inline size_t al256b(size_t b) { return (b + 255) & ~size_t(255); }

static bool batch_size_ok(int ny, int nx) {
  return ilog2_exact(ny) >= 4 && ilog2_exact(nx) >= 4 && ny <= 2048 && nx <= 4096;
}
static int b_colC(int ny) { const int c = 2048 / ny; return c > 32 ? 32 : c; }
static int b_rseq(int ny, int nx) { const int q = 4096 / nx; return q > ny ? ny : q; }

static InstLayout inst_layout(int ny, int nx, int max_saves) {
  InstLayout L;
  const long long fs = (long long)ny * spec_ldc(nx);
  const size_t s64 = 2 * (size_t)fs * 16, s32 = 2 * (size_t)fs * 8;
  const int nparts = 2 * (ny / b_rseq(ny, nx));
  size_t o = 0;
  L.ys0 = o; o += al256b(s64);
  L.ys1 = o; o += al256b(s64);
  L.pa = o; o += al256b(s64);
  L.pb = o; o += al256b(s64);
  L.za = o; o += al256b(s32);
  L.zb = o; o += al256b(s32);
  L.plan32 = o; o += al256b(plan_bytes(ny, nx, 4));
  L.plan64 = o; o += al256b(plan_bytes(ny, nx, 8));
  L.part = o; o += al256b(sizeof(double) * (size_t)nparts);
  L.bad = o; o += al256b(sizeof(int) * (size_t)nparts);
  L.ht = o; o += al256b(sizeof(double) * (size_t)max_saves);
  L.hdt = o; o += al256b(sizeof(double) * (size_t)max_saves);
  L.total = o;
  return L;
}

// work items of one instance per pass
static void inst_items(const BInst& I, int slot, std::vector<unsigned>* w) {
  const int tiles = (I.ncols + I.colC - 1) / I.colC;
  for (int f = 0; f < 2; ++f)
    for (int t = 0; t < tiles; ++t) {
      w[BPASS_C1].push_back(witem(slot, f, t));
      w[BPASS_C2].push_back(witem(slot, f, t));  // both C2 jobs of the field in one tile
      w[BPASS_C3].push_back(witem(slot, f, t));
    }
  for (int b = 0; b < I.nblk; ++b) {
    w[BPASS_R1].push_back(witem(slot, 0, b));
    w[BPASS_R1].push_back(witem(slot, 1, b));
    w[BPASS_R2].push_back(witem(slot, 0, b));
    w[BPASS_R3].push_back(witem(slot, 0, b));
    w[BPASS_R3].push_back(witem(slot, 1, b));
  }
}

static size_t inst_item_count(int ny, int nx) {
  const int C = b_colC(ny), tiles = (nx / 2 + 1 + C - 1) / C, nblk = ny / b_rseq(ny, nx);
  const size_t c = (size_t)tiles * 2, r1 = (size_t)nblk * 2;
  return c > r1 ? c : r1;  // the largest pass (a column pass: one tile per field and tile; or R1)
}

struct EngLayout {
  size_t tab, eng, work[BNPASS], total;
};

static EngLayout eng_layout(int max_inst, int max_work) {
  EngLayout L;
  size_t o = 0;
  L.tab = o; o += al256b(sizeof(BInst) * (size_t)max_inst);
  L.eng = o; o += al256b(sizeof(BEng));
  for (int p = 0; p < BNPASS; ++p) { L.work[p] = o; o += al256b(sizeof(unsigned) * (size_t)max_work); }
  L.total = o;
  return L;
}

static constexpr int kBatchUnroll = 2;  // attempts per iteration of the conditional node

struct GsBatch {
  int max_inst = 0, max_work = 0;
  char* dws = nullptr;
  EngLayout L;
  BArgs args;
  std::vector<BInst> h_tab;         // host mirror of the table (geometry, pointers, last read state)
  std::vector<int> state;           // SLOT_*
  std::vector<const void*> plan64;  // per slot
  bool dirty = true;
  int* h_stop = nullptr;            // mapped pinned host flag
  int* d_stop = nullptr;
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  size_t smem = 0;
  BEng h_eng;
};

static mjx_status batch_attrs(size_t smem) {
  static ContextOnce once;
  return once.run([&]() -> mjx_status {
    MJX_CUDA_TRY(cudaFuncSetAttribute(bcol_kernel<BPASS_C1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MJX_CUDA_TRY(cudaFuncSetAttribute(bcol_kernel<BPASS_C2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MJX_CUDA_TRY(cudaFuncSetAttribute(bcol_kernel<BPASS_C3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MJX_CUDA_TRY(cudaFuncSetAttribute(brow_kernel<BPASS_R1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MJX_CUDA_TRY(cudaFuncSetAttribute(brow_kernel<BPASS_R2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MJX_CUDA_TRY(cudaFuncSetAttribute(brow_kernel<BPASS_R3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return MJX_OK;
  });
}

static cudaError_t launch_batch_attempt(const GsBatch& B, cudaGraphConditionalHandle hdl, cudaStream_t s) {
  const int* nw = B.h_eng.nwork;
  bcol_kernel<BPASS_C1><<<nw[BPASS_C1], BT, B.smem, s>>>(B.args);
  brow_kernel<BPASS_R1><<<nw[BPASS_R1], BT, B.smem, s>>>(B.args);
  bcol_kernel<BPASS_C2><<<nw[BPASS_C2], BT, B.smem, s>>>(B.args);
  brow_kernel<BPASS_R2><<<nw[BPASS_R2], BT, B.smem, s>>>(B.args);
  bcol_kernel<BPASS_C3><<<nw[BPASS_C3], BT, B.smem, s>>>(B.args);
  brow_kernel<BPASS_R3><<<nw[BPASS_R3], BT, B.smem, s>>>(B.args);
  bctl_kernel<<<1, 1024, 0, s>>>(B.args, hdl);
  return cudaGetLastError();
}

static void drop_graph(GsBatch& B) {
  if (B.exec) cudaGraphExecDestroy(B.exec);
  if (B.graph) cudaGraphDestroy(B.graph);
  B.exec = nullptr;
  B.graph = nullptr;
}

// (Re)builds the epoch graph for the current work lists (every count > 0).
static mjx_status build_graph(GsBatch& B) {
  drop_graph(B);
  cudaError_t ce = cudaSuccess;
  do {
    if (B.cap == nullptr && (ce = cudaStreamCreateWithFlags(&B.cap, cudaStreamNonBlocking)) != cudaSuccess) break;
    if ((ce = cudaGraphCreate(&B.graph, 0)) != cudaSuccess) break;
    cudaGraphConditionalHandle hdl;
    if ((ce = cudaGraphConditionalHandleCreate(&hdl, B.graph, 1, cudaGraphCondAssignDefault)) != cudaSuccess) break;
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = hdl;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if ((ce = cudaGraphAddNode(&node, B.graph, nullptr, nullptr, 0, &np)) != cudaSuccess) break;
    cudaGraph_t body = np.conditional.phGraph_out[0];
    if ((ce = cudaStreamBeginCaptureToGraph(B.cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) break;
    cudaError_t le = cudaSuccess;
    for (int u = 0; u < kBatchUnroll && le == cudaSuccess; ++u) le = launch_batch_attempt(B, hdl, B.cap);
    cudaGraph_t captured = nullptr;
    ce = cudaStreamEndCapture(B.cap, &captured);
    if (le != cudaSuccess) { ce = le; break; }
    if (ce != cudaSuccess) break;
    ce = cudaGraphInstantiate(&B.exec, B.graph, 0);
  } while (0);
  if (ce != cudaSuccess) { set_last_error(ce, __FILE__, __LINE__); return MJX_CUDA_ERROR; }
  return MJX_OK;
}

static void free_batch(GsBatch* B) {
  drop_graph(*B);
  if (B->cap) cudaStreamDestroy(B->cap);
  if (B->h_stop) cudaFreeHost(B->h_stop);
  delete B;
}

// uploads the work lists of every running instance
static mjx_status upload_work(GsBatch& B, cudaStream_t s) {
  std::vector<unsigned> w[BNPASS];
  int n_slots = 0;
  for (int i = 0; i < B.max_inst; ++i) {
    if (B.state[i] != SLOT_FREE) n_slots = i + 1;
    if (B.state[i] == SLOT_RUNNING) inst_items(B.h_tab[i], i, w);
  }
  for (int p = 0; p < BNPASS; ++p) {
    if ((int)w[p].size() > B.max_work) return MJX_BAD_SHAPE;
    B.h_eng.nwork[p] = (int)w[p].size();
    if (!w[p].empty())
      MJX_CUDA_TRY(cudaMemcpyAsync(B.dws + B.L.work[p], w[p].data(), sizeof(unsigned) * w[p].size(),
                                   cudaMemcpyHostToDevice, s));
  }
  B.h_eng.n_slots = n_slots;
  MJX_CUDA_TRY(cudaStreamSynchronize(s));  // the host vectors go out of scope
  MJX_TRY(build_graph(B));
  B.dirty = false;
  return MJX_OK;
}

}  // namespace mjx

using namespace mjx;

extern "C" {

size_t mjx_gsbatch_bytes(int max_instances, int max_work) {
  if (max_instances < 1 || max_instances > 4096 || max_work < 1) return 0;
  return eng_layout(max_instances, max_work).total;
}

size_t mjx_gsbatch_instance_bytes(int ny, int nx, int max_saves) {
  if (!batch_size_ok(ny, nx) || max_saves < 1) return 0;
  return inst_layout(ny, nx, max_saves).total;
}

int mjx_gsbatch_work_items(int ny, int nx) {
  if (!batch_size_ok(ny, nx)) return 0;
  return (int)inst_item_count(ny, nx);
}

mjx_status mjx_gsbatch_create(void** batch, int max_instances, int max_work, void* ws, size_t ws_bytes) {
  if (batch == nullptr || max_instances < 1 || max_instances > 4096 || max_work < 1 || ws == nullptr)
    return MJX_BAD_ARG;
  *batch = nullptr;
  const EngLayout L = eng_layout(max_instances, max_work);
  if (ws_bytes < L.total) return MJX_WORKSPACE;
  MJX_TRY(ensure_kernel_attrs());
  GsBatch* B = new GsBatch();
  B->max_inst = max_instances;
  B->max_work = max_work;
  B->dws = (char*)ws;
  B->L = L;
  B->h_tab.assign(max_instances, BInst());
  memset(B->h_tab.data(), 0, sizeof(BInst) * max_instances);
  for (int i = 0; i < max_instances; ++i) B->h_tab[i].st.done = 1;  // free slots never run
  B->state.assign(max_instances, SLOT_FREE);
  B->plan64.assign(max_instances, nullptr);
  B->args.tab = (BInst*)(B->dws + L.tab);
  B->args.eng = (BEng*)(B->dws + L.eng);
  for (int p = 0; p < BNPASS; ++p) B->args.work[p] = (const unsigned*)(B->dws + L.work[p]);
  memset(&B->h_eng, 0, sizeof(B->h_eng));
  mjx_status st = MJX_OK;
  cudaError_t ce = cudaHostAlloc((void**)&B->h_stop, sizeof(int), cudaHostAllocMapped);
  if (ce == cudaSuccess) { *B->h_stop = 0; ce = cudaHostGetDevicePointer((void**)&B->d_stop, B->h_stop, 0); }
  if (ce != cudaSuccess) { set_last_error(ce, __FILE__, __LINE__); free_batch(B); return MJX_CUDA_ERROR; }
  B->h_eng.host_stop = B->d_stop;
  B->smem = (size_t)sp_size(4096) * sizeof(float2);
  st = batch_attrs(B->smem);
  if (st == MJX_OK) {  // every slot of the device table starts free (done)
    ce = cudaMemcpy(B->args.tab, B->h_tab.data(), sizeof(BInst) * max_instances, cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) { set_last_error(ce, __FILE__, __LINE__); st = MJX_CUDA_ERROR; }
  }
  if (st != MJX_OK) { free_batch(B); return st; }
  *batch = B;
  return MJX_OK;
}

mjx_status mjx_gsbatch_destroy(void* batch) {
  if (batch == nullptr) return MJX_BAD_ARG;
  free_batch((GsBatch*)batch);
  return MJX_OK;
}

mjx_status mjx_gsbatch_admit(void* batch, const mjx_gs_instance* d, int io_dtype, const void* y0, void* ws,
                             size_t ws_bytes, int* slot_out, void* stream) {
  GsBatch* B = (GsBatch*)batch;
  if (B == nullptr || d == nullptr || y0 == nullptr || ws == nullptr || slot_out == nullptr) return MJX_BAD_ARG;
  if (!batch_size_ok(d->ny, d->nx)) return MJX_BAD_SHAPE;
  if (!elem_size(io_dtype)) return MJX_BAD_DTYPE;
  if (!(d->dx > 0) || !(d->dy > 0) || d->max_steps < 0 || d->save_every < 1) return MJX_BAD_ARG;
  const int max_saves = d->max_steps / d->save_every + 1;
  const InstLayout IL = inst_layout(d->ny, d->nx, max_saves);
  if (ws_bytes < IL.total) return MJX_WORKSPACE;
  int slot = -1;
  for (int i = 0; i < B->max_inst; ++i)
    if (B->state[i] == SLOT_FREE) { slot = i; break; }
  if (slot < 0) return MJX_OOM;
  // the work lists must still fit
  size_t items = inst_item_count(d->ny, d->nx);
  for (int i = 0; i < B->max_inst; ++i)
    if (B->state[i] == SLOT_RUNNING) items += inst_item_count(B->h_tab[i].ny, B->h_tab[i].nx);
  if (items > (size_t)B->max_work) return MJX_OOM;
  cudaStream_t s = (cudaStream_t)stream;
  char* w = (char*)ws;
  mjx_grid2d g;
  g.ny = d->ny; g.nx = d->nx; g.dy = d->dy; g.dx = d->dx;
  MJX_TRY(mjx_spec2d_plan_init(w + IL.plan32, &g, MJX_SYMBOL_FD, MJX_F32, stream));
  MJX_TRY(mjx_spec2d_plan_init(w + IL.plan64, &g, MJX_SYMBOL_FD, MJX_F64, stream));
  MJX_TRY(mix_state_from_real(w + IL.plan64, &g, 2, io_dtype, y0, (double*)(w + IL.pa), (float4*)(w + IL.ys0), s));
  BInst I;
  memset(&I, 0, sizeof(I));
  I.ny = g.ny; I.nx = g.nx; I.log2ny = ilog2_exact(g.ny); I.log2nx = ilog2_exact(g.nx);
  I.ldc = spec_ldc(g.nx); I.ncols = g.nx / 2 + 1;
  I.colC = b_colC(g.ny); I.rseq = b_rseq(g.ny, g.nx); I.nblk = g.ny / I.rseq; I.nparts = 2 * I.nblk;
  I.fs = (long long)g.ny * I.ldc;
  I.ys[0] = (float4*)(w + IL.ys0); I.ys[1] = (float4*)(w + IL.ys1);
  I.pa = (float4*)(w + IL.pa); I.pb = (float4*)(w + IL.pb);
  I.za = (float2*)(w + IL.za); I.zb = (float2*)(w + IL.zb);
  const PlanView pv = plan_view(w + IL.plan32, g.ny, g.nx, 4);
  I.twx = (const float2*)pv.twx; I.twy = (const float2*)pv.twy;
  I.lamx = (const float*)pv.lamx; I.lamy = (const float*)pv.lamy;
  I.partial = (double*)(w + IL.part); I.nonfinite = (int*)(w + IL.bad);
  I.hist_t = (double*)(w + IL.ht); I.hist_dt = (double*)(w + IL.hdt);
  I.D[0] = d->Du > 1e-14 ? d->Du : 0.0;
  I.D[1] = d->Dv > 1e-14 ? d->Dv : 0.0;
  I.F = d->F; I.k = d->k;
  I.n_dof = 2.0 * g.ny * g.nx;
  I.inv_norm = (float)(1.0 / ((double)g.nx * (double)g.ny));
  I.pid = d->pid;
  DevState& h = I.st;
  const double dt_init = (d->dt0 < d->dt_cfl || d->dt0 != d->dt0) ? d->dt0 : d->dt_cfl;
  h.t = d->t0; h.dt = dt_init; h.t_end = d->t_end; h.prev_err = 1.0; h.dt_cfl = d->dt_cfl;
  h.status = MJX_STATUS_RUNNING_CODE; h.write_idx = 1; h.finite = 1;
  h.max_saves = max_saves; h.save_every = d->save_every; h.order = 2; h.save_slot = -1;
  h.max_attempts = d->max_attempts > 0 ? d->max_attempts : 20 * d->max_steps + 1000;
  const bool running = (d->t0 < d->t_end) && (1 < max_saves);
  if (running) h.dtc = dt_init < d->t_end - d->t0 ? dt_init : d->t_end - d->t0;
  else { h.done = 1; h.status = (d->t0 >= d->t_end) ? MJX_STATUS_SUCCESS_CODE : MJX_STATUS_MAX_STEPS_CODE; }
  MJX_CUDA_TRY(cudaMemsetAsync(I.hist_t, 0, sizeof(double) * max_saves, s));
  MJX_CUDA_TRY(cudaMemsetAsync(I.hist_dt, 0, sizeof(double) * max_saves, s));
  MJX_CUDA_TRY(cudaMemcpyAsync(I.hist_t, &d->t0, sizeof(double), cudaMemcpyHostToDevice, s));
  B->h_tab[slot] = I;
  MJX_CUDA_TRY(cudaMemcpyAsync(B->args.tab + slot, &B->h_tab[slot], sizeof(BInst), cudaMemcpyHostToDevice, s));
  MJX_CUDA_TRY(cudaStreamSynchronize(s));
  B->plan64[slot] = w + IL.plan64;
  B->state[slot] = running ? SLOT_RUNNING : SLOT_FINISHED;
  B->dirty = true;
  *slot_out = slot;
  return MJX_OK;
}

mjx_status mjx_gsbatch_run(void* batch, int max_attempts, int stop_after_finished, int* n_running,
                           int* n_finished, void* stream) {
  GsBatch* B = (GsBatch*)batch;
  if (B == nullptr || max_attempts < 1) return MJX_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int running = 0;
  for (int i = 0; i < B->max_inst; ++i) running += B->state[i] == SLOT_RUNNING;
  if (running > 0) {
    if (B->dirty) MJX_TRY(upload_work(*B, s));
    MJX_TRY(batch_attrs(B->smem));
    B->h_eng.halt = 0;
    B->h_eng.attempts = 0;
    B->h_eng.finished = 0;
    B->h_eng.running = running;
    B->h_eng.max_attempts = max_attempts;
    B->h_eng.stop_after_finished = stop_after_finished;
    MJX_CUDA_TRY(cudaMemcpyAsync(B->args.eng, &B->h_eng, sizeof(BEng), cudaMemcpyHostToDevice, s));
    MJX_CUDA_TRY(cudaGraphLaunch(B->exec, s));
    // read back every slot's controller state
    const int n_slots = B->h_eng.n_slots;
    std::vector<BInst> tab(n_slots);
    MJX_CUDA_TRY(cudaMemcpyAsync(tab.data(), B->args.tab, sizeof(BInst) * n_slots, cudaMemcpyDeviceToHost, s));
    MJX_CUDA_TRY(cudaStreamSynchronize(s));
    running = 0;
    for (int i = 0; i < n_slots; ++i) {
      if (B->state[i] != SLOT_RUNNING) continue;
      B->h_tab[i].st = tab[i].st;
      if (tab[i].st.done) { B->state[i] = SLOT_FINISHED; B->dirty = true; }
      else ++running;
    }
  }
  int fin = 0;
  for (int i = 0; i < B->max_inst; ++i) fin += B->state[i] == SLOT_FINISHED;
  if (n_running) *n_running = running;
  if (n_finished) *n_finished = fin;
  return MJX_OK;
}

mjx_status mjx_gsbatch_finished(void* batch, int* slots, int cap, int* n) {
  GsBatch* B = (GsBatch*)batch;
  if (B == nullptr || n == nullptr || (cap > 0 && slots == nullptr)) return MJX_BAD_ARG;
  int k = 0;
  for (int i = 0; i < B->max_inst; ++i)
    if (B->state[i] == SLOT_FINISHED) {
      if (k < cap) slots[k] = i;
      ++k;
    }
  *n = k;
  return MJX_OK;
}

mjx_status mjx_gsbatch_retire(void* batch, int slot, int io_dtype, void* y_final, double* hist_t, double* hist_dt,
                              mjx_adaptive_result* res, void* stream) {
  GsBatch* B = (GsBatch*)batch;
  if (B == nullptr || slot < 0 || y_final == nullptr) return MJX_BAD_ARG;
  if (slot >= B->max_inst || B->state[slot] != SLOT_FINISHED) return MJX_BAD_ARG;
  if (!elem_size(io_dtype)) return MJX_BAD_DTYPE;
  const BInst& I = B->h_tab[slot];
  cudaStream_t s = (cudaStream_t)stream;
  mjx_grid2d g;
  g.ny = I.ny; g.nx = I.nx; g.dy = 1.0; g.dx = 1.0;  // the inverse transforms use only the twiddles
  // PB holds the FP64 spectrum and PA the FP64 real state (both free once the run ended)
  const DevState* st_dev = &B->args.tab[slot].st;
  MJX_TRY(mix_real_from_state(B->plan64[slot], &g, 2, st_dev, I.ys[0], I.ys[1], (double2*)I.pb, (double*)I.pa,
                              io_dtype, y_final, s));
  const int ns = I.st.write_idx;
  if (hist_t) MJX_CUDA_TRY(cudaMemcpyAsync(hist_t, I.hist_t, sizeof(double) * ns, cudaMemcpyDeviceToHost, s));
  if (hist_dt) MJX_CUDA_TRY(cudaMemcpyAsync(hist_dt, I.hist_dt, sizeof(double) * ns, cudaMemcpyDeviceToHost, s));
  MJX_CUDA_TRY(cudaStreamSynchronize(s));
  if (res) {
    const DevState& o = I.st;
    res->t_final = o.t; res->dt_next = o.dt; res->prev_err = o.prev_err; res->last_err = o.err_last;
    res->n_accepted = o.n_acc; res->n_rejected = o.n_rej; res->n_attempts = o.attempts;
    res->n_saved = o.write_idx; res->status = o.status; res->finite = o.finite;
  }
  B->state[slot] = SLOT_FREE;
  B->plan64[slot] = nullptr;
  B->dirty = true;
  return MJX_OK;
}

void mjx_gsbatch_request_stop(void* batch, int stop) {
  GsBatch* B = (GsBatch*)batch;
  if (B != nullptr && B->h_stop != nullptr) *(volatile int*)B->h_stop = stop ? 1 : 0;
}

}  // extern "C"
