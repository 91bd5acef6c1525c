// tdy_solver.cu -- device-resident backward-Euler Newton solve of one or many
// independent instances (the blocks of TDySetExtrudedMeshes) in one handle.
//
// Each Newton iteration evaluates the FP64 residual and the Jacobian with the
// handle's kernels for every instance at once, takes per-instance residual
// norms (the only values the host reads), and solves J y = F with
// right-preconditioned BiCGStab:
//   * Krylov vectors and the Jacobian copy in FP32 (default) or FP64; the
//     residual, the Newton update x -= y and the convergence test stay FP64;
//   * every instance keeps its own BiCGStab scalars and stops on its own
//     tolerance (device-side masks, no host round trip per iteration);
//   * preconditioner: exact solves of the vertical lines (the tridiagonal
//     coupling of each column of an extruded block, Thomas algorithm, one
//     thread per column), which carries the stiff vertical coupling of thin
//     layers;
//   * one BiCGStab iteration is built once as a CUDA graph with the explicit
//     graph API (kernel nodes in a chain, no stream capture, so device calls
//     that other threads make meanwhile cannot invalidate it) and replayed;
//   * the sparse matrix-vector product's threads per row (1, 4 or 8) are
//     picked by timing the candidates on the first solve.
// No reference counterpart: the reference hands F and J to PETSc's SNES/KSP.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <tuple>
#include <utility>
#include <vector>

#include "tdy_arena.h"
#include "tdy_device.h"
#include "tdy_emit.h"

namespace tdy {

namespace {

#define SCUDA(call)                                                                             \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      return set_error(TDY_ERR_GPU, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

inline unsigned nblk(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// per-instance scalars, [slot][nseg]
enum { S_RHO = 0, S_ALPHA, S_OMEGA, S_BETA, S_BNORM2, S_T1, S_T2, S_HALF, S_NSCAL };

struct Krylov {
  bool ready = false;
  void *Jv = nullptr;                                  // matrix values (T)
  void *b = nullptr, *r = nullptr, *r0 = nullptr, *p = nullptr, *v = nullptr, *s = nullptr, *t = nullptr,
       *ph = nullptr, *sh = nullptr, *y = nullptr;     // vectors (T)
  void *la = nullptr, *lcp = nullptr, *linv = nullptr; // line factors (T)
  void *cinv = nullptr;                                // clusters: 1/diagonal of the other cells (T)
  void *clu = nullptr;                                 // clusters: LU factors (T), grown on demand
  size_t clu_cap = 0;                                  // elements of clu
  cudaGraphExec_t graph = nullptr;
  int graph_precond = -1;  // preconditioner the graph was built with
  int graph_tpr = 0;       // spmv threads per row the graph was built with
  int tpr = 0;  // spmv threads per row (autotuned)
};

}  // namespace

struct SolverState {
  int n = 0, nnz = 0, nseg = 0, nlines = 0;
  std::vector<int> h_seg_off;
  int *rowptr = nullptr, *colidx = nullptr, *seg_off = nullptr, *cell_seg = nullptr;
  int *line_off = nullptr, *line_cells = nullptr, *pos_d = nullptr, *pos_lo = nullptr, *pos_hi = nullptr;
  double *x = nullptr, *xb = nullptr, *F = nullptr, *J = nullptr, *fn2 = nullptr, *scal = nullptr, *lam = nullptr;
  int *trial = nullptr, *commit = nullptr;
  int *newt_active = nullptr, *lin_active = nullptr, *lin_its = nullptr;
  int nchunks = 0;
  int *chunk_off = nullptr, *seg_chunk = nullptr;  // chunks of the per-instance reductions
  double *part = nullptr, *part2 = nullptr;
  double linear_rtol = -1.0;
  int *dpos = nullptr;  // position of each row's diagonal in the CSR values
  // strong-coupling clusters, rebuilt for every linear solve that uses them:
  // label per cell, a change flag, local index in its cluster (-1: the cell
  // takes its diagonal), the members of the 2..64-cell clusters (cluster by
  // cluster, ascending cell index), their offsets and LU offsets, pivots
  int *clab = nullptr, *cflag = nullptr, *cloc = nullptr, *cmem = nullptr, *coff = nullptr, *cpiv = nullptr;
  long long *cluoff = nullptr;
  int ncl = 0;  // clusters of 2..64 cells in the current solve
  int ncl_cells = 0, ncl_big_cells = 0;  // cells in them; cells of clusters over 64 cells
  int precond_used = 0;
  std::vector<int> h_lab, h_cnt, h_id, h_fill, h_loc, h_mem, h_off;
  std::vector<long long> h_luoff;
  Krylov k32, k64;
  // schedules of the line-preconditioned inner solve (block: one CTA per
  // instance; tile: the batch-wide graph): instances with at most
  // block_max_cells cells take the block schedule (-2: not chosen yet)
  int *inst_line_off = nullptr, *block_inst = nullptr, *block_mask = nullptr, *ticket = nullptr;
  std::vector<int> h_inst_line_off, h_order;  // h_order: instances by size, largest first
  long long block_max_cells = -2, mask_for = -3;
  int n_block = 0, n_tile = 0;
  std::vector<double> tune_ms;  // measured candidates of the last tuning (ms per linear solve)
  // evaluation of every instance: -1 not chosen, 0 three-stage launches,
  // 1 instance schedule (timed on the first evaluation; the same bits)
  int eval_mode = -1;
  double eval_ms[2] = {0.0, 0.0};
  // phase timers on the solve's stream: evaluation, Jacobian cast and
  // preconditioner set-up, Krylov iterations (events of the current phase)
  cudaEvent_t tev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  std::vector<long long> h_inst_cells;
  // device memory: stream-ordered on the handle's stream (allocated there and
  // synchronised at init; freed there when the solver is destroyed, after
  // every solve has synchronised its stream)
  cudaStream_t st = nullptr;
  std::vector<void *> allocs;
  ~SolverState() {
    for (cudaEvent_t e : tev)
      if (e) cudaEventDestroy(e);
    for (Krylov *k : {&k32, &k64}) {
      if (k->graph) cudaGraphExecDestroy(k->graph);
      if (k->clu) dmem_free(k->clu, st);
    }
    for (void *p : allocs) dmem_free(p, st);
  }
};

namespace {

template <class T>
int salloc(SolverState *s, T **p, size_t n) {
  int ierr = dmem_alloc((void **)p, std::max<size_t>(n, 1) * sizeof(T), s->st);
  if (ierr) return ierr;
  s->allocs.push_back(*p);
  return 0;
}
// (the host vector must stay alive until the stream is synchronised)
template <class T>
int sup(SolverState *s, T **p, const std::vector<T> &h) {
  int ierr = salloc(s, p, h.size());
  if (ierr) return ierr;
  if (h.empty()) return 0;
  cudaError_t e = cudaMemcpyAsync(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s->st);
  if (e != cudaSuccess) return set_error(TDY_ERR_GPU, "cudaMemcpyAsync: %s", cudaGetErrorString(e));
  return 0;
}

// ---------------------------------------------------------------------------
// kernels
//
// Two schedules run the BiCGStab iterations: "tile" (every kernel over all
// cells of the batch, instances masked as they converge; one iteration is a
// graph) and "block" (one CTA per instance runs its whole Krylov loop, see
// bicgstab_block_kernel).  Both perform every floating-point operation of an
// instance in the same order with explicit roundings (the element operations
// below, the chunked reductions, the per-row lane split of the product), so
// an instance gets the same bits from either schedule.

__device__ __forceinline__ float e_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double e_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float e_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double e_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float e_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double e_add(double a, double b) { return __dadd_rn(a, b); }

// p = r + beta (p - omega v)
template <class T>
__device__ __forceinline__ T op_p(T r, T p, T v, T beta, T omega) {
  return e_fma(beta, e_fma(-omega, v, p), r);
}
// y += alpha ph (+ omega sh)
template <class T>
__device__ __forceinline__ T op_y(T y, T ph, T alpha) {
  return e_fma(alpha, ph, y);
}
template <class T>
__device__ __forceinline__ T op_y2(T y, T ph, T sh, T alpha, T omega) {
  return e_fma(omega, sh, e_fma(alpha, ph, y));
}
// the per-cell terms of the chunked dot products, in FP64
template <class TA, class TB>
__device__ __forceinline__ double op_dot(double acc, TA a, TB b) {
  return __fma_rn((double)a, (double)b, acc);
}

template <class T>
__global__ void cast_kernel(long long n, const double *a, T *b) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (T)a[i];
}

// the cells of the flagged instances: b = (float)a
__global__ void cast_masked_kernel(int n, const int *cell_seg, const int *flag, const double *a, float *b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flag[cell_seg[i]]) b[i] = (float)a[i];
}

// Per-instance dot products in two deterministic passes: one block per chunk
// of at most kChunk cells (chunks counted from each instance's first cell, so
// an instance is reduced the same way alone and in a batch), then one thread
// per instance adding its chunks in order.
constexpr int kChunk = 4096;

template <class TA, class TB>
__global__ void __launch_bounds__(256) chunk_dot_kernel(const int *chunk_off, const TA *a, const TB *b, const TA *c,
                                                        const TB *d, double *part, double *part2) {
  __shared__ double sh[2][256];
  const int ch = blockIdx.x;
  const int i0 = chunk_off[ch], i1 = chunk_off[ch + 1];
  double acc = 0.0, acc2 = 0.0;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    acc = op_dot(acc, a[i], b[i]);
    if (c) acc2 = op_dot(acc2, c[i], d[i]);
  }
  sh[0][threadIdx.x] = acc;
  sh[1][threadIdx.x] = acc2;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[ch] = sh[0][0];
    if (c) part2[ch] = sh[1][0];
  }
}

__global__ void chunk_sum_kernel(int nseg, const int *seg_chunk, const double *part, const double *part2, double *out,
                                 double *out2) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  double acc = 0.0, acc2 = 0.0;
  for (int k = seg_chunk[s]; k < seg_chunk[s + 1]; k++) {
    acc += part[k];
    if (out2) acc2 += part2[k];
  }
  out[s] = acc;
  if (out2) out2[s] = acc2;
}

// y = A x over the CSR pattern with TPR threads per row
// One row of A x by TPR lanes (1, 2, 4 or 8) with the same bits for every
// TPR: the row's entries are split into 8 phases (entry k of the row in
// phase k mod 8), each phase summed by one FMA chain in entry order, and the
// 8 phase sums added by a fixed tree, ((P0+P4) + (P2+P6)) + ((P1+P5) +
// (P3+P7)).  Lane l holds phases l, l+TPR, ...; the tree levels whose pairs
// lie in one lane are added in registers, the others by shuffles, so the
// lane split can be tuned for speed without changing any result.  Lane 0
// returns the row's value.
template <class T, int TPR>
__device__ __forceinline__ T row_dot(bool valid, int k0, int k1, int lane, const int *colidx, const T *A, const T *x) {
  constexpr int NP = 8 / TPR;
  T P[NP];
#pragma unroll
  for (int q = 0; q < NP; q++) {
    T acc = 0;
    if (valid)
      for (int k = k0 + lane + TPR * q; k < k1; k += 8) acc = e_fma(A[k], x[colidx[k]], acc);
    P[q] = acc;
  }
#pragma unroll
  for (int o = 4; o >= TPR; o >>= 1) {  // pairs (p, p + o) within the lane: q and q + o / TPR
#pragma unroll
    for (int q = 0; q < o / TPR; q++) P[q] = e_add(P[q], P[q + o / TPR]);
  }
  T acc = P[0];
#pragma unroll
  for (int o = TPR / 2; o > 0; o >>= 1) acc = e_add(acc, __shfl_down_sync(0xffffffffu, acc, o, TPR));
  return acc;
}

template <class T, int TPR>
__global__ void __launch_bounds__(256) spmv_kernel(int n, const int *rowptr, const int *colidx, const T *A, const T *x,
                                                   T *y) {
  const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int row = (int)(gt / TPR), lane = (int)(gt % TPR);
  const T acc = row_dot<T, TPR>(row < n, row < n ? rowptr[row] : 0, row < n ? rowptr[row + 1] : 0, lane, colidx, A, x);
  if (row < n && lane == 0) y[row] = acc;
}

// Thomas factorisation of every vertical line from the FP64 Jacobian
template <class T>
__global__ void line_factor_kernel(int nlines, const int *line_off, const int *pd, const int *plo, const int *phi,
                                   const double *J, T *la, T *lcp, T *linv) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nlines) return;
  double cp = 0.0;
  for (int k = line_off[l]; k < line_off[l + 1]; k++) {
    const double b = J[pd[k]], a = plo[k] >= 0 ? J[plo[k]] : 0.0, c = phi[k] >= 0 ? J[phi[k]] : 0.0;
    double den = b - a * cp;
    if (den == 0.0) den = (b != 0.0) ? b : 1.0;  // singular line: fall back to its diagonal
    const double inv = 1.0 / den;
    cp = c * inv;
    la[k] = (T)a;
    lcp[k] = (T)cp;
    linv[k] = (T)inv;
  }
}

// out = (line-tridiagonal)^-1 in, line l
template <class T>
__device__ __forceinline__ void line_solve_one(int l, const int *line_off, const int *line_cells, const T *la,
                                               const T *lcp, const T *linv, const T *in, T *out) {
  const int k0 = line_off[l], k1 = line_off[l + 1];
  T prev = 0;
  for (int k = k0; k < k1; k++) {
    const int i = line_cells[k];
    prev = e_mul(e_fma(-la[k], prev, in[i]), linv[k]);
    out[i] = prev;
  }
  T next = 0;
  for (int k = k1 - 1; k >= k0; k--) {
    const int i = line_cells[k];
    next = e_fma(-lcp[k], next, out[i]);
    out[i] = next;
  }
}
template <class T>
__global__ void line_solve_kernel(int nlines, const int *line_off, const int *line_cells, const T *la, const T *lcp,
                                  const T *linv, const T *in, T *out) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nlines) return;
  line_solve_one(l, line_off, line_cells, la, lcp, linv, in, out);
}

template <class T>
__global__ void init_kernel(int n, const int *cell_seg, const int *active, const double *F, T *b, T *r, T *r0, T *p,
                            T *v, T *y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T f = active[cell_seg[i]] ? (T)F[i] : (T)0;
  b[i] = f;
  r[i] = f;
  r0[i] = f;
  p[i] = 0;
  v[i] = 0;
  y[i] = 0;
}

// (instances on the block schedule stay inactive in the tile iterations)
__global__ void init_scalars_kernel(int nseg, const int *newt_active, const int *block_mask, int *lin_active,
                                    int *lin_its, double *scal) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  scal[S_RHO * nseg + s] = 1.0;
  scal[S_ALPHA * nseg + s] = 1.0;
  scal[S_OMEGA * nseg + s] = 1.0;
  scal[S_HALF * nseg + s] = 0.0;
  lin_active[s] = newt_active[s] && scal[S_BNORM2 * nseg + s] > 0.0 && !block_mask[s];
}

// after rho_new = (r0, r) in T1
__global__ void scal_beta_kernel(int nseg, int *act, double *sc) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg || !act[s]) return;
  const double rn = sc[S_T1 * nseg + s];
  if (rn == 0.0) {
    act[s] = 0;
    return;
  }
  sc[S_BETA * nseg + s] = (rn / sc[S_RHO * nseg + s]) * (sc[S_ALPHA * nseg + s] / sc[S_OMEGA * nseg + s]);
  sc[S_RHO * nseg + s] = rn;
}
// after (r0, v) in T1
__global__ void scal_alpha_kernel(int nseg, int *act, double *sc) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg || !act[s]) return;
  const double d = sc[S_T1 * nseg + s];
  if (d == 0.0) {
    act[s] = 0;
    return;
  }
  sc[S_ALPHA * nseg + s] = sc[S_RHO * nseg + s] / d;
}
// after (s, s) in T1: converged already at the half step?
__global__ void scal_half_kernel(int nseg, const int *act, double *sc, double tol2) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg || !act[s]) return;
  sc[S_HALF * nseg + s] = (sc[S_T1 * nseg + s] <= tol2 * sc[S_BNORM2 * nseg + s]) ? 1.0 : 0.0;
}
// after (t, t) in T1 and (t, s) in T2
__global__ void scal_omega_kernel(int nseg, const int *act, double *sc) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg || !act[s]) return;
  const double tt = sc[S_T1 * nseg + s];
  sc[S_OMEGA * nseg + s] = tt > 0.0 ? sc[S_T2 * nseg + s] / tt : 0.0;
}
// after (r, r) in T1
__global__ void scal_check_kernel(int nseg, int *act, int *its, double *sc, double tol2) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg || !act[s]) return;
  its[s] += 1;
  if (sc[S_HALF * nseg + s] != 0.0 || sc[S_T1 * nseg + s] <= tol2 * sc[S_BNORM2 * nseg + s] ||
      sc[S_OMEGA * nseg + s] == 0.0)
    act[s] = 0;
}

template <class T>
__global__ void p_update_kernel(int n, const int *cs, const int *act, const double *sc, int nseg, const T *r, const T *v,
                                T *p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = cs[i];
  if (!act[s]) return;
  const T beta = (T)sc[S_BETA * nseg + s], omega = (T)sc[S_OMEGA * nseg + s];
  p[i] = op_p(r[i], p[i], v[i], beta, omega);
}
template <class T>
__global__ void s_update_kernel(int n, const int *cs, const int *act, const double *sc, int nseg, const T *r, const T *v,
                                T *sv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = cs[i];
  if (!act[s]) return;
  sv[i] = e_fma(-(T)sc[S_ALPHA * nseg + s], v[i], r[i]);
}
template <class T>
__global__ void xr_update_kernel(int n, const int *cs, const int *act, const double *sc, int nseg, const T *ph,
                                 const T *sh, const T *sv, const T *tv, T *y, T *r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = cs[i];
  if (!act[s]) return;
  const T alpha = (T)sc[S_ALPHA * nseg + s];
  if (sc[S_HALF * nseg + s] != 0.0) {
    y[i] = op_y(y[i], ph[i], alpha);
    return;
  }
  const T omega = (T)sc[S_OMEGA * nseg + s];
  y[i] = op_y2(y[i], ph[i], sh[i], alpha, omega);
  r[i] = e_fma(-omega, tv[i], sv[i]);
}

// ---------------------------------------------------------------------------
// Block schedule: one CTA of kBlockThreads threads per instance runs the
// instance's whole BiCGStab loop with the line preconditioner, performing the
// tile schedule's operations in the tile schedule's order (reductions in
// kChunk-cell chunks with the same per-chunk tree and in-order chunk sum, the
// product's rows split over TPR lanes the same way), so the two schedules
// give the same bits.  CTAs take instances from a ticket counter, largest
// first; an instance's result does not depend on which CTA takes it.
constexpr int kBlockThreads = 256;
static_assert(kBlockThreads == 256, "the block schedule's reductions mirror the 256-thread chunk reductions");

template <class T>
struct BlockSolve {
  int ninst;                 // instances on the block schedule
  const int *inst;           // their indices, largest first
  int *ticket;               // zeroed before the launch
  const int *seg_off;        // cells of instance g: [seg_off[g], seg_off[g + 1])
  const int *inst_line_off;  // lines of instance g: [inst_line_off[g], inst_line_off[g + 1])
  const int *line_off, *line_cells;
  const T *la, *lcp, *linv;
  const int *rowptr, *colidx;
  const T *A;
  T *b, *r, *r0, *p, *v, *s, *t, *ph, *sh, *y;
  const int *newt_active;
  int *lin_its;
  double tol2;
  int max_it;
};

// (a, b) and, with c, (c, d) over cells [i0, i1): chunk_dot_kernel's
// accumulation and tree per chunk, chunk_sum_kernel's in-order sum; every
// thread returns the result
template <class TA, class TB>
__device__ __forceinline__ void block_dot(int i0, int i1, const TA *a, const TB *b, const TA *c, const TB *d,
                                          double *red, double *out1, double *out2) {
  const int tid = threadIdx.x;
  double tot = 0.0, tot2 = 0.0;
  for (int k0 = i0; k0 < i1; k0 += kChunk) {
    const int k1 = min(k0 + kChunk, i1);
    double acc = 0.0, acc2 = 0.0;
    for (int i = k0 + tid; i < k1; i += kBlockThreads) {
      acc = op_dot(acc, a[i], b[i]);
      if (c) acc2 = op_dot(acc2, c[i], d[i]);
    }
    red[tid] = acc;
    red[kBlockThreads + tid] = acc2;
    __syncthreads();
    for (int w = kBlockThreads / 2; w > 0; w >>= 1) {
      if (tid < w) {
        red[tid] += red[tid + w];
        red[kBlockThreads + tid] += red[kBlockThreads + tid + w];
      }
      __syncthreads();
    }
    tot += red[0];
    tot2 += red[kBlockThreads];
    __syncthreads();  // every thread has read the chunk's sums
  }
  *out1 = tot;
  if (out2) *out2 = tot2;
}

// y = A x over rows [c0, c1): the row sums of spmv_kernel (row_dot)
template <class T, int TPR>
__device__ __forceinline__ void block_spmv(int c0, int c1, const int *rowptr, const int *colidx, const T *A,
                                           const T *x, T *y) {
  const int nrow = c1 - c0;
  for (int base = 0; base < nrow * TPR; base += kBlockThreads) {
    const int gt = base + (int)threadIdx.x, rl = gt / TPR, lane = gt % TPR, row = c0 + rl;
    const T acc = row_dot<T, TPR>(rl < nrow, rl < nrow ? rowptr[row] : 0, rl < nrow ? rowptr[row + 1] : 0, lane,
                                  colidx, A, x);
    if (rl < nrow && lane == 0) y[row] = acc;
  }
}

template <class T, int TPR>
__global__ void __launch_bounds__(kBlockThreads) bicgstab_block_kernel(BlockSolve<T> B) {
  __shared__ double red[2 * kBlockThreads];
  __shared__ int cur;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) cur = atomicAdd(B.ticket, 1);
    __syncthreads();
    const int k = cur;
    __syncthreads();  // every thread has read the ticket before the next one is drawn
    if (k >= B.ninst) return;
    const int g = B.inst[k];
    const int c0 = B.seg_off[g], c1 = B.seg_off[g + 1];
    const int l0 = B.inst_line_off[g], l1 = B.inst_line_off[g + 1];
    int its = 0;
    double bnorm2 = 0.0;
    if (B.newt_active[g]) block_dot<T, T>(c0, c1, B.b, B.b, nullptr, nullptr, red, &bnorm2, nullptr);
    if (bnorm2 > 0.0) {
      double rho = 1.0, alpha = 1.0, omega = 1.0;
      for (int it = 0; it < B.max_it; it++) {
        double rn;
        block_dot<T, T>(c0, c1, B.r0, B.r, nullptr, nullptr, red, &rn, nullptr);
        if (rn == 0.0) break;
        const double beta = (rn / rho) * (alpha / omega);
        rho = rn;
        {
          const T tb = (T)beta, to = (T)omega;
          for (int i = c0 + tid; i < c1; i += kBlockThreads) B.p[i] = op_p(B.r[i], B.p[i], B.v[i], tb, to);
        }
        __syncthreads();
        for (int l = l0 + tid; l < l1; l += kBlockThreads)
          line_solve_one(l, B.line_off, B.line_cells, B.la, B.lcp, B.linv, B.p, B.ph);
        __syncthreads();
        block_spmv<T, TPR>(c0, c1, B.rowptr, B.colidx, B.A, B.ph, B.v);
        __syncthreads();
        double dv;
        block_dot<T, T>(c0, c1, B.r0, B.v, nullptr, nullptr, red, &dv, nullptr);
        if (dv == 0.0) break;
        alpha = rho / dv;
        {
          const T ta = (T)alpha;
          for (int i = c0 + tid; i < c1; i += kBlockThreads) B.s[i] = e_fma(-ta, B.v[i], B.r[i]);
        }
        __syncthreads();
        double ss;
        block_dot<T, T>(c0, c1, B.s, B.s, nullptr, nullptr, red, &ss, nullptr);
        const bool half = ss <= B.tol2 * bnorm2;
        if (half) {
          const T ta = (T)alpha;
          for (int i = c0 + tid; i < c1; i += kBlockThreads) B.y[i] = op_y(B.y[i], B.ph[i], ta);
          __syncthreads();
          its++;
          break;
        }
        for (int l = l0 + tid; l < l1; l += kBlockThreads)
          line_solve_one(l, B.line_off, B.line_cells, B.la, B.lcp, B.linv, B.s, B.sh);
        __syncthreads();
        block_spmv<T, TPR>(c0, c1, B.rowptr, B.colidx, B.A, B.sh, B.t);
        __syncthreads();
        double tt, ts;
        block_dot<T, T>(c0, c1, B.t, B.t, B.t, B.s, red, &tt, &ts);
        omega = tt > 0.0 ? ts / tt : 0.0;
        {
          const T ta = (T)alpha, to = (T)omega;
          for (int i = c0 + tid; i < c1; i += kBlockThreads) {
            B.y[i] = op_y2(B.y[i], B.ph[i], B.sh[i], ta, to);
            B.r[i] = e_fma(-to, B.t[i], B.s[i]);
          }
        }
        __syncthreads();
        double rr;
        block_dot<T, T>(c0, c1, B.r, B.r, nullptr, nullptr, red, &rr, nullptr);
        its++;
        if (rr <= B.tol2 * bnorm2 || omega == 0.0) break;
      }
    }
    if (tid == 0) B.lin_its[g] = its;
    __syncthreads();
  }
}

// trial point of the line search: x = xb - lam_s y for the instances on
// trial, x = xb for the others (FP64 update)
template <class T>
__global__ void trial_kernel(int n, const int *cs, const int *trial, const double *lam, const T *y, const double *xb,
                             double *x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = cs[i];
  x[i] = trial[s] ? xb[i] - lam[s] * (double)y[i] : xb[i];
}
// accepted trial points become the base
__global__ void commit_kernel(int n, const int *cs, const int *commit, const double *x, double *xb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (commit[cs[i]]) xb[i] = x[i];
}

// ---------------------------------------------------------------------------
// Strong-coupling clusters.  A coupling with |a_ij| >= tau sqrt(|a_ii a_jj|)
// joins cells i and j; the connected clusters are found by label
// propagation (every strong coupling hooks the labels of both cells to the
// smaller one, then labels jump to their label's label).  The labels
// converge to each cluster's smallest cell index whatever the order of the
// atomic updates, so the clusters are deterministic.

__global__ void cl_init_kernel(int n, int *lab) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) lab[i] = i;
}

__global__ void cl_hook_kernel(int n, const int *rowptr, const int *colidx, const int *dpos, const double *J,
                               double tau, int *lab, int *flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double di = fabs(J[dpos[i]]);
  for (int k = rowptr[i]; k < rowptr[i + 1]; k++) {
    const int j = colidx[k];
    if (j == i) continue;
    const double aij = fabs(J[k]);
    if (!(aij > 0.0) || !(aij >= tau * sqrt(di * fabs(J[dpos[j]])))) continue;
    const int li = lab[i], lj = lab[j];
    if (li != lj) {
      const int m = li < lj ? li : lj;
      atomicMin(&lab[li], m);
      atomicMin(&lab[lj], m);
      *flag = 1;
    }
  }
}

__global__ void cl_jump_kernel(int n, int *lab, int *flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int l = lab[i], ll = lab[l];
  if (ll != l) {
    lab[i] = ll;
    *flag = 1;
  }
}

// cells outside the 2..64-cell clusters precondition with their diagonal
template <class T>
__global__ void cl_diag_kernel(int n, const int *loc, const int *dpos, const double *J, T *inv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || loc[i] >= 0) return;
  const double d = J[dpos[i]];
  inv[i] = d != 0.0 ? (T)(1.0 / d) : (T)1;
}

constexpr int kClusterMax = 64;
constexpr int kClusterLd = kClusterMax + 1;  // padded row of the staged block

// One warp per cluster: stage the cluster's block of J (every coupling
// between its cells) in shared memory, factor it by LU with partial pivoting
// (ties to the smaller row; a zero pivot becomes 1), store the factors.
template <class T>
__global__ void __launch_bounds__(32) cl_factor_kernel(int ncl, const int *coff, const long long *luoff,
                                                       const int *cmem, const int *loc, const int *lab,
                                                       const int *rowptr, const int *colidx, const double *J, T *lu,
                                                       int *piv) {
  extern __shared__ unsigned char cl_smem[];
  T *B = reinterpret_cast<T *>(cl_smem);  // [kClusterMax][kClusterLd]
  const int cl = blockIdx.x, lane = threadIdx.x;
  if (cl >= ncl) return;
  const int c0 = coff[cl], sz = coff[cl + 1] - c0;
  for (int e = lane; e < sz * kClusterLd; e += 32) B[e] = (T)0;
  __syncwarp();
  for (int r = lane; r < sz; r += 32) {
    const int m = cmem[c0 + r], L = lab[m];
    for (int k = rowptr[m]; k < rowptr[m + 1]; k++) {
      const int col = colidx[k];
      if (lab[col] == L) B[r * kClusterLd + loc[col]] = (T)J[k];
    }
  }
  __syncwarp();
  for (int kk = 0; kk < sz; kk++) {
    T best = (T)-1;
    int bi = kk;
    for (int i = kk + lane; i < sz; i += 32) {
      const T v = B[i * kClusterLd + kk] < (T)0 ? -B[i * kClusterLd + kk] : B[i * kClusterLd + kk];
      if (v > best) {
        best = v;
        bi = i;
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const T ob = __shfl_down_sync(0xffffffffu, best, off);
      const int oi = __shfl_down_sync(0xffffffffu, bi, off);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    bi = __shfl_sync(0xffffffffu, bi, 0);
    if (lane == 0) piv[c0 + kk] = bi;
    if (bi != kk)
      for (int j = lane; j < sz; j += 32) {
        const T t = B[kk * kClusterLd + j];
        B[kk * kClusterLd + j] = B[bi * kClusterLd + j];
        B[bi * kClusterLd + j] = t;
      }
    __syncwarp();
    T pv = B[kk * kClusterLd + kk];
    if (pv == (T)0) pv = (T)1;
    __syncwarp();
    if (lane == 0) B[kk * kClusterLd + kk] = pv;
    for (int i = kk + 1 + lane; i < sz; i += 32) {
      const T l = B[i * kClusterLd + kk] / pv;
      B[i * kClusterLd + kk] = l;
      for (int j = kk + 1; j < sz; j++) B[i * kClusterLd + j] -= l * B[kk * kClusterLd + j];
    }
    __syncwarp();
  }
  T *out = lu + luoff[cl];
  for (int e = lane; e < sz * sz; e += 32) out[e] = B[(e / sz) * kClusterLd + e % sz];
}

template <class T>
__global__ void cl_apply_diag_kernel(int n, const int *loc, const T *inv, const T *in, T *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && loc[i] < 0) out[i] = inv[i] * in[i];
}

// out = (cluster block)^-1 in, one warp per cluster: the row swaps, then the
// unit-lower and upper triangular solves
template <class T>
__global__ void __launch_bounds__(32) cl_apply_kernel(int ncl, const int *coff, const long long *luoff,
                                                      const int *cmem, const T *lu, const int *piv, const T *in,
                                                      T *out) {
  __shared__ T x[kClusterMax];
  const int cl = blockIdx.x, lane = threadIdx.x;
  if (cl >= ncl) return;
  const int c0 = coff[cl], sz = coff[cl + 1] - c0;
  for (int r = lane; r < sz; r += 32) x[r] = in[cmem[c0 + r]];
  __syncwarp();
  if (lane == 0)
    for (int kk = 0; kk < sz; kk++) {
      const int p = piv[c0 + kk];
      if (p != kk) {
        const T t = x[kk];
        x[kk] = x[p];
        x[p] = t;
      }
    }
  __syncwarp();
  const T *L = lu + luoff[cl];
  for (int kk = 0; kk < sz; kk++) {
    const T xk = x[kk];
    __syncwarp();
    for (int i = kk + 1 + lane; i < sz; i += 32) x[i] -= L[i * sz + kk] * xk;
    __syncwarp();
  }
  for (int kk = sz - 1; kk >= 0; kk--) {
    if (lane == 0) x[kk] /= L[kk * sz + kk];
    __syncwarp();
    const T xk = x[kk];
    for (int i = lane; i < kk; i += 32) x[i] -= L[i * sz + kk] * xk;
    __syncwarp();
  }
  for (int r = lane; r < sz; r += 32) out[cmem[c0 + r]] = x[r];
}

// ---------------------------------------------------------------------------
template <class T>
int spmv(SolverState *s, const Krylov &k, const T *x, T *y, Emit &e) {
  const T *A = (const T *)k.Jv;
  const unsigned g = nblk((long long)s->n * k.tpr, 256);
  switch (k.tpr) {
    case 1:
      e(spmv_kernel<T, 1>, g, 256, 0, s->n, (const int *)s->rowptr, (const int *)s->colidx, A, x, y);
      break;
    case 2:
      e(spmv_kernel<T, 2>, g, 256, 0, s->n, (const int *)s->rowptr, (const int *)s->colidx, A, x, y);
      break;
    case 4:
      e(spmv_kernel<T, 4>, g, 256, 0, s->n, (const int *)s->rowptr, (const int *)s->colidx, A, x, y);
      break;
    default:
      e(spmv_kernel<T, 8>, g, 256, 0, s->n, (const int *)s->rowptr, (const int *)s->colidx, A, x, y);
      break;
  }
  return 0;
}

template <class TA, class TB>
void seg_dot(SolverState *s, const TA *a, const TB *b, const TA *c, const TB *d, double *out, double *out2, Emit &e) {
  e(chunk_dot_kernel<TA, TB>, (unsigned)s->nchunks, 256, 0, (const int *)s->chunk_off, a, b, c, d, s->part,
    s->part2);
  e(chunk_sum_kernel, nblk(s->nseg, 128), 128, 0, s->nseg, (const int *)s->seg_chunk, (const double *)s->part,
    (const double *)s->part2, out, c ? out2 : (double *)nullptr);
}
template <class TA, class TB>
void seg_dot(SolverState *s, const TA *a, const TB *b, const TA *c, const TB *d, double *out, double *out2,
             cudaStream_t st) {
  Emit e(st);
  seg_dot<TA, TB>(s, a, b, c, d, out, out2, e);
}

template <class T>
int dot(SolverState *s, const T *a, const T *b, const T *c, const T *d, int slot1, int slot2, Emit &e) {
  seg_dot<T, T>(s, a, b, c, d, s->scal + (size_t)slot1 * s->nseg, c ? s->scal + (size_t)slot2 * s->nseg : nullptr, e);
  return 0;
}

// out = M^-1 in with the preconditioner of the current solve
template <class T>
void precondition(SolverState *s, Krylov &k, const T *in, T *out, Emit &e) {
  if (s->precond_used == TDY_PRECOND_CLUSTERS) {
    e(cl_apply_diag_kernel<T>, nblk(s->n, 256), 256, 0, s->n, (const int *)s->cloc, (const T *)k.cinv, in, out);
    e(cl_apply_kernel<T>, (unsigned)s->ncl, 32, 0, s->ncl, (const int *)s->coff, (const long long *)s->cluoff,
      (const int *)s->cmem, (const T *)k.clu, (const int *)s->cpiv, in, out);
  } else {
    e(line_solve_kernel<T>, nblk(s->nlines, 128), 128, 0, s->nlines, (const int *)s->line_off,
      (const int *)s->line_cells, (const T *)k.la, (const T *)k.lcp, (const T *)k.linv, in, out);
  }
}

// one BiCGStab iteration for every active instance (the graph body)
template <class T>
void bicgstab_iteration(SolverState *s, Krylov &k, double tol2, Emit &e) {
  const int n = s->n, ns = s->nseg;
  const unsigned gb = nblk(n, 256), sb = nblk(ns, 128);
  T *r = (T *)k.r, *r0 = (T *)k.r0, *p = (T *)k.p, *v = (T *)k.v, *sv = (T *)k.s, *tv = (T *)k.t;
  T *ph = (T *)k.ph, *sh = (T *)k.sh, *y = (T *)k.y;
  const int *cs = s->cell_seg;
  int *act = s->lin_active;
  const int *cact = s->lin_active;
  double *sc = s->scal;
  const double *csc = s->scal;
  dot<T>(s, r0, r, nullptr, nullptr, S_T1, 0, e);
  e(scal_beta_kernel, sb, 128, 0, ns, act, sc);
  e(p_update_kernel<T>, gb, 256, 0, n, cs, cact, csc, ns, (const T *)r, (const T *)v, p);
  precondition<T>(s, k, p, ph, e);
  spmv<T>(s, k, ph, v, e);
  dot<T>(s, r0, v, nullptr, nullptr, S_T1, 0, e);
  e(scal_alpha_kernel, sb, 128, 0, ns, act, sc);
  e(s_update_kernel<T>, gb, 256, 0, n, cs, cact, csc, ns, (const T *)r, (const T *)v, sv);
  dot<T>(s, sv, sv, nullptr, nullptr, S_T1, 0, e);
  e(scal_half_kernel, sb, 128, 0, ns, cact, sc, tol2);
  precondition<T>(s, k, sv, sh, e);
  spmv<T>(s, k, sh, tv, e);
  dot<T>(s, tv, tv, tv, sv, S_T1, S_T2, e);
  e(scal_omega_kernel, sb, 128, 0, ns, cact, sc);
  e(xr_update_kernel<T>, gb, 256, 0, n, cs, cact, csc, ns, (const T *)ph, (const T *)sh, (const T *)sv,
    (const T *)tv, y, r);
  dot<T>(s, r, r, nullptr, nullptr, S_T1, 0, e);
  e(scal_check_kernel, sb, 128, 0, ns, act, s->lin_its, sc, tol2);
}

// (one allocation for the Jacobian copy and every vector; ordered on the
// solve's stream, which uses them next)
template <class T>
int krylov_alloc(SolverState *s, Krylov &k, cudaStream_t st) {
  if (k.ready) return 0;
  Arena ar;
  T **vecs[] = {(T **)&k.b, (T **)&k.r,  (T **)&k.r0, (T **)&k.p,  (T **)&k.v,   (T **)&k.s,   (T **)&k.t,
                (T **)&k.ph, (T **)&k.sh, (T **)&k.y, (T **)&k.la, (T **)&k.lcp, (T **)&k.linv};
  ar.work((T **)&k.Jv, (size_t)s->nnz);
  for (T **vp : vecs) ar.work(vp, (size_t)s->n);
  int ierr = ar.commit(st);
  if (ierr) return ierr;
  s->allocs.push_back(ar.base);
  k.ready = true;
  return 0;
}

// Picks the spmv threads per row by timing the candidates on the handle's
// first solve in each precision (the best split depends on the rows and on
// the schedule); options.spmv_threads forces one.  The results do not depend
// on it (row_dot).
template <class T>
int autotune_spmv(SolverState *s, Krylov &k, int forced, cudaStream_t st) {
  if (forced > 0) {
    k.tpr = forced;
    return 0;
  }
  if (k.tpr) return 0;
  cudaEvent_t e0, e1;
  SCUDA(cudaEventCreate(&e0));
  SCUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int best_tpr = 1;
  Emit em(st);
  for (int tpr : {1, 2, 4, 8}) {
    k.tpr = tpr;
    spmv<T>(s, k, (const T *)k.b, (T *)k.v, em);  // warm-up
    cudaEventRecord(e0, st);
    for (int it = 0; it < 5; it++) spmv<T>(s, k, (const T *)k.b, (T *)k.v, em);
    cudaEventRecord(e1, st);
    SCUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      best_tpr = tpr;
    }
  }
  k.tpr = best_tpr;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return 0;
}

// Clusters for the current Jacobian: label propagation on the device (at
// most kClusterRounds rounds of one hook pass and four jump passes, until a
// round changes nothing), compaction on the host in cell order, then the
// factors.  Returns 0 with precond_used = TDY_PRECOND_LINES when the labels
// have not settled (the caller then factors the lines).
constexpr int kClusterRounds = 64;

template <class T>
int cluster_setup(SolverState *s, Krylov &k, double tau, cudaStream_t st) {
  int ierr;
  const int n = s->n;
  if (!s->clab) {
    if ((ierr = salloc(s, &s->clab, n))) return ierr;
    if ((ierr = salloc(s, &s->cflag, 1))) return ierr;
    if ((ierr = salloc(s, &s->cloc, n))) return ierr;
    if ((ierr = salloc(s, &s->cmem, n))) return ierr;
    if ((ierr = salloc(s, &s->coff, n + 1))) return ierr;
    if ((ierr = salloc(s, &s->cluoff, n + 1))) return ierr;
    if ((ierr = salloc(s, &s->cpiv, n))) return ierr;
  }
  if (!k.cinv) {
    T *p;
    if ((ierr = salloc(s, &p, n))) return ierr;
    k.cinv = p;
  }
  cl_init_kernel<<<nblk(n, 256), 256, 0, st>>>(n, s->clab);
  bool settled = false;
  for (int round = 0; round < kClusterRounds && !settled; round++) {
    SCUDA(cudaMemsetAsync(s->cflag, 0, sizeof(int), st));
    cl_hook_kernel<<<nblk(n, 128), 128, 0, st>>>(n, s->rowptr, s->colidx, s->dpos, s->J, tau, s->clab, s->cflag);
    for (int j = 0; j < 4; j++) cl_jump_kernel<<<nblk(n, 256), 256, 0, st>>>(n, s->clab, s->cflag);
    int flag = 1;
    SCUDA(cudaMemcpyAsync(&flag, s->cflag, sizeof(int), cudaMemcpyDeviceToHost, st));
    SCUDA(cudaStreamSynchronize(st));
    settled = flag == 0;
  }
  if (!settled) {
    s->precond_used = TDY_PRECOND_LINES;
    return 0;
  }
  // compaction: clusters of 2..kClusterMax cells in order of their smallest
  // cell, members in ascending cell order
  std::vector<int> &lab = s->h_lab, &cnt = s->h_cnt, &id = s->h_id, &fill = s->h_fill, &loc = s->h_loc,
                   &mem = s->h_mem, &off = s->h_off;
  std::vector<long long> &luoff = s->h_luoff;
  lab.resize(n);
  SCUDA(cudaMemcpyAsync(lab.data(), s->clab, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
  SCUDA(cudaStreamSynchronize(st));
  cnt.assign(n, 0);
  for (int i = 0; i < n; i++) {
    if (lab[i] < 0 || lab[i] >= n) return set_error(TDY_ERR_LIB, "solver: cluster label %d out of range", lab[i]);
    cnt[lab[i]]++;
  }
  id.assign(n, -1);
  off.assign(1, 0);
  luoff.assign(1, 0);
  int ncl = 0, big = 0;
  for (int r = 0; r < n; r++)
    if (cnt[r] >= 2 && cnt[r] <= kClusterMax) {
      id[r] = ncl++;
      off.push_back(off.back() + cnt[r]);
      luoff.push_back(luoff.back() + (long long)cnt[r] * cnt[r]);
    } else if (cnt[r] > kClusterMax) {
      big += cnt[r];
    }
  s->ncl_cells = off.back();
  s->ncl_big_cells = big;
  fill.assign(ncl, 0);
  loc.assign(n, -1);
  mem.resize(off.back());
  for (int i = 0; i < n; i++) {
    const int c = id[lab[i]];
    if (c < 0) continue;
    loc[i] = fill[c]++;
    mem[off[c] + loc[i]] = i;
  }
  s->ncl = ncl;
  SCUDA(cudaMemcpyAsync(s->cloc, loc.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
  if (ncl > 0) {
    SCUDA(cudaMemcpyAsync(s->cmem, mem.data(), sizeof(int) * mem.size(), cudaMemcpyHostToDevice, st));
    SCUDA(cudaMemcpyAsync(s->coff, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice, st));
    SCUDA(cudaMemcpyAsync(s->cluoff, luoff.data(), sizeof(long long) * luoff.size(), cudaMemcpyHostToDevice, st));
    const size_t need = (size_t)luoff.back();
    if (need > k.clu_cap) {  // stream-ordered: no device synchronisation
      if (k.clu) dmem_free(k.clu, st);
      k.clu = nullptr;
      k.clu_cap = 0;
      if ((ierr = dmem_alloc(&k.clu, need * sizeof(T), st))) return ierr;
      k.clu_cap = need;
    }
  }
  cl_diag_kernel<T><<<nblk(n, 256), 256, 0, st>>>(n, s->cloc, s->dpos, s->J, (T *)k.cinv);
  if (ncl > 0)
    cl_factor_kernel<T><<<ncl, 32, kClusterMax * kClusterLd * sizeof(T), st>>>(
        ncl, s->coff, s->cluoff, s->cmem, s->cloc, s->clab, s->rowptr, s->colidx, s->J, (T *)k.clu, s->cpiv);
  SCUDA(cudaGetLastError());
  // the host vectors above stay alive until the copies complete
  SCUDA(cudaStreamSynchronize(st));
  s->precond_used = TDY_PRECOND_CLUSTERS;
  return 0;
}

// Instances on the block schedule for a split at `thr` cells (-1: none,
// LLONG_MAX: all): the list (largest first) and the per-instance mask.
int set_block_split(SolverState *s, long long thr, cudaStream_t st) {
  if (s->mask_for == thr) return 0;
  std::vector<int> mask(s->nseg, 0), list;
  for (int g : s->h_order) {
    const long long nc = s->h_seg_off[g + 1] - s->h_seg_off[g];
    if (thr >= 0 && nc <= thr) {
      mask[g] = 1;
      list.push_back(g);
    }
  }
  s->n_block = (int)list.size();
  s->n_tile = s->nseg - s->n_block;
  SCUDA(cudaMemcpyAsync(s->block_mask, mask.data(), sizeof(int) * s->nseg, cudaMemcpyHostToDevice, st));
  if (!list.empty())
    SCUDA(cudaMemcpyAsync(s->block_inst, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice, st));
  SCUDA(cudaStreamSynchronize(st));  // the host vectors are read
  s->mask_for = thr;
  return 0;
}

template <class T, int TPR>
int launch_block(SolverState *s, Krylov &k, const TDyNewtonOptions &o, double tol2, cudaStream_t st) {
  BlockSolve<T> B;
  B.ninst = s->n_block;
  B.inst = s->block_inst;
  B.ticket = s->ticket;
  B.seg_off = s->seg_off;
  B.inst_line_off = s->inst_line_off;
  B.line_off = s->line_off;
  B.line_cells = s->line_cells;
  B.la = (const T *)k.la;
  B.lcp = (const T *)k.lcp;
  B.linv = (const T *)k.linv;
  B.rowptr = s->rowptr;
  B.colidx = s->colidx;
  B.A = (const T *)k.Jv;
  B.b = (T *)k.b;
  B.r = (T *)k.r;
  B.r0 = (T *)k.r0;
  B.p = (T *)k.p;
  B.v = (T *)k.v;
  B.s = (T *)k.s;
  B.t = (T *)k.t;
  B.ph = (T *)k.ph;
  B.sh = (T *)k.sh;
  B.y = (T *)k.y;
  B.newt_active = s->newt_active;
  B.lin_its = s->lin_its;
  B.tol2 = tol2;
  B.max_it = o.linear_max_it;
  int dev = 0, nsm = 0, per_sm = 0;
  SCUDA(cudaGetDevice(&dev));
  SCUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  SCUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bicgstab_block_kernel<T, TPR>, kBlockThreads, 0));
  const int grid = std::max(1, std::min(s->n_block, nsm * std::max(per_sm, 1)));
  SCUDA(cudaMemsetAsync(s->ticket, 0, sizeof(int), st));
  bicgstab_block_kernel<T, TPR><<<grid, kBlockThreads, 0, st>>>(B);
  SCUDA(cudaGetLastError());
  return 0;
}

// One linear solve with instances of at most `thr` cells on the block
// schedule and the others on the tile schedule; its = inner iterations.
template <class T>
int solve_scheduled(SolverState *s, Krylov &k, const TDyNewtonOptions &o, double tol2, long long thr,
                    cudaStream_t st, std::vector<int> &its) {
  int ierr;
  const int n = s->n, ns = s->nseg;
  if ((ierr = set_block_split(s, thr, st))) return ierr;
  init_kernel<T><<<nblk(n, 256), 256, 0, st>>>(n, s->cell_seg, s->newt_active, s->F, (T *)k.b, (T *)k.r, (T *)k.r0,
                                               (T *)k.p, (T *)k.v, (T *)k.y);
  {
    Emit em(st);
    dot<T>(s, (T *)k.b, (T *)k.b, nullptr, nullptr, S_BNORM2, 0, em);
  }
  SCUDA(cudaMemsetAsync(s->lin_its, 0, sizeof(int) * ns, st));
  init_scalars_kernel<<<nblk(ns, 128), 128, 0, st>>>(ns, s->newt_active, s->block_mask, s->lin_active, s->lin_its,
                                                     s->scal);
  SCUDA(cudaGetLastError());
  if (s->n_block > 0) {
    switch (k.tpr) {
      case 1:
        ierr = launch_block<T, 1>(s, k, o, tol2, st);
        break;
      case 2:
        ierr = launch_block<T, 2>(s, k, o, tol2, st);
        break;
      case 4:
        ierr = launch_block<T, 4>(s, k, o, tol2, st);
        break;
      default:
        ierr = launch_block<T, 8>(s, k, o, tol2, st);
        break;
    }
    if (ierr) return ierr;
  }
  if (s->n_tile > 0) {
    std::vector<int> act(ns);
    const int check_every = 8;
    for (int it = 0; it < o.linear_max_it; it += check_every) {
      for (int j = 0; j < check_every && it + j < o.linear_max_it; j++) SCUDA(cudaGraphLaunch(k.graph, st));
      SCUDA(cudaMemcpyAsync(act.data(), s->lin_active, sizeof(int) * ns, cudaMemcpyDeviceToHost, st));
      SCUDA(cudaStreamSynchronize(st));
      bool any = false;
      for (int a : act) any |= (a != 0);
      if (!any) break;
    }
  }
  its.resize(ns);
  SCUDA(cudaMemcpyAsync(its.data(), s->lin_its, sizeof(int) * ns, cudaMemcpyDeviceToHost, st));
  SCUDA(cudaStreamSynchronize(st));
  return 0;
}

// Schedule autotuner.  The first line-preconditioned solve of a size class
// (arithmetic, number of instances, largest instance) times the candidate
// splits on the solve at hand: all instances on the tile schedule, all on the
// block schedule, and splits at 4096, 16384 and 65536 cells where they
// separate the instances; the fastest split is kept for the class for the
// rest of the process.  The schedules give the same bits, so the choice
// changes only the time.
std::mutex g_sched_mutex;
std::vector<std::pair<long long, long long>> g_sched;  // (class key, split)

template <class T>
int tune_schedule(SolverState *s, Krylov &k, const TDyNewtonOptions &o, double tol2, cudaStream_t st,
                  long long *thr) {
  long long maxc = 0;
  for (int g = 0; g < s->nseg; g++) maxc = std::max<long long>(maxc, s->h_seg_off[g + 1] - s->h_seg_off[g]);
  int lg = 0;
  while ((1LL << lg) < maxc) lg++;
  const int cls = s->nseg == 1 ? 0 : (s->nseg < 64 ? 1 : 2);
  const long long key = ((long long)sizeof(T) << 16) | ((long long)cls << 8) | lg;
  if (s->block_max_cells != -2) {  // this handle's choice
    *thr = s->block_max_cells;
    return 0;
  }
  {
    std::lock_guard<std::mutex> lk(g_sched_mutex);
    for (auto &e : g_sched)
      if (e.first == key) {
        s->block_max_cells = *thr = e.second;
        return 0;
      }
  }
  std::vector<long long> cand = {-1, LLONG_MAX};
  for (long long c : {4096LL, 16384LL, 65536LL}) {
    int below = 0;
    for (int g = 0; g < s->nseg; g++) below += (s->h_seg_off[g + 1] - s->h_seg_off[g]) <= c;
    if (below > 0 && below < s->nseg) cand.push_back(c);
  }
  std::vector<int> its;
  s->tune_ms.clear();
  double best = 1e300;
  long long best_thr = -1;
  for (long long c : cand) {
    int ierr;
    if ((ierr = solve_scheduled<T>(s, k, o, tol2, c, st, its))) return ierr;  // warm-up
    const auto t0 = std::chrono::steady_clock::now();
    if ((ierr = solve_scheduled<T>(s, k, o, tol2, c, st, its))) return ierr;
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    s->tune_ms.push_back(ms);
    if (ms < best) {
      best = ms;
      best_thr = c;
    }
  }
  {
    std::lock_guard<std::mutex> lk(g_sched_mutex);
    g_sched.emplace_back(key, best_thr);
  }
  s->block_max_cells = *thr = best_thr;
  return 0;
}

template <class T>
int linear_solve(SolverState *s, Krylov &k, const TDyNewtonOptions &o, cudaStream_t st, long long *lin_total,
                 std::vector<int> &inst_lin_its) {
  int ierr;
  if ((ierr = krylov_alloc<T>(s, k, st))) return ierr;
  if ((ierr = autotune_spmv<T>(s, k, o.spmv_threads, st))) return ierr;  // uses b and v as scratch before they are set
  const int n = s->n, ns = s->nseg;
  SCUDA(cudaEventRecord(s->tev[2], st));
  cast_kernel<T><<<nblk(s->nnz, 256), 256, 0, st>>>(s->nnz, s->J, (T *)k.Jv);
  s->precond_used = TDY_PRECOND_LINES;
  if (o.precond == TDY_PRECOND_CLUSTERS && (ierr = cluster_setup<T>(s, k, o.cluster_threshold, st))) return ierr;
  if (s->precond_used == TDY_PRECOND_LINES)
    line_factor_kernel<T><<<nblk(s->nlines, 128), 128, 0, st>>>(s->nlines, s->line_off, s->pos_d, s->pos_lo,
                                                                 s->pos_hi, s->J, (T *)k.la, (T *)k.lcp, (T *)k.linv);
  SCUDA(cudaEventRecord(s->tev[3], st));
  const double tol2 = o.linear_rtol * o.linear_rtol;
  // The graph of one iteration is built with the explicit graph API, not by
  // stream capture: a capture is invalidated by device-wide operations that
  // other threads issue meanwhile (a cudaFree, a device synchronisation),
  // which a server running many handles at once cannot rule out.  The cluster
  // launches depend on this solve's cluster count: rebuild for every solve.
  if (!k.graph || s->linear_rtol != o.linear_rtol || k.graph_precond != s->precond_used || k.graph_tpr != k.tpr ||
      s->precond_used == TDY_PRECOND_CLUSTERS) {
    if (k.graph) cudaGraphExecDestroy(k.graph);
    k.graph = nullptr;
    cudaGraph_t g = nullptr;
    SCUDA(cudaGraphCreate(&g, 0));
    Emit em(st);
    em.g = g;
    bicgstab_iteration<T>(s, k, tol2, em);
    cudaError_t e = em.err;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&k.graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      k.graph = nullptr;
      return set_error(TDY_ERR_GPU, "BiCGStab iteration graph: %s", cudaGetErrorString(e));
    }
    k.graph_precond = s->precond_used;
    k.graph_tpr = k.tpr;
    s->linear_rtol = o.linear_rtol;
  }
  std::vector<int> its(ns);
  // the schedule split: chosen by timing on the first solve of this size
  // class (process-wide), or given by the options; clusters: tile only
  long long thr = -1;
  if (s->precond_used == TDY_PRECOND_LINES) {
    if (o.schedule == TDY_SCHEDULE_TILE)
      thr = -1;
    else if (o.schedule == TDY_SCHEDULE_BLOCK)
      thr = LLONG_MAX;
    else if ((ierr = tune_schedule<T>(s, k, o, tol2, st, &thr)))
      return ierr;
  }
  if ((ierr = solve_scheduled<T>(s, k, o, tol2, thr, st, its))) return ierr;
  SCUDA(cudaEventRecord(s->tev[4], st));
  for (int v : its) *lin_total += v;
  inst_lin_its = its;
  return 0;
}

int solver_init(_p_TDy *t) {
  if (t->solver) return 0;
  const MPFAOSetup &su = t->setup;
  SolverState *s = new SolverState();
  t->solver = s;
  s->st = (cudaStream_t)device_default_stream(t);
  for (cudaEvent_t &e : s->tev) SCUDA(cudaEventCreate(&e));
  s->n = t->mesh.nc;
  s->nnz = (int)su.colidx.size();
  // instances: the mesh blocks; lines: the columns of each block, bottom to top
  std::vector<int> seg_off(1, 0), cell_seg(s->n), line_off(1, 0), line_cells, pd, plo, phi;
  line_cells.reserve(s->n);
  auto find = [&](int i, int j) {
    const int *b = su.colidx.data() + su.rowptr[i], *e = su.colidx.data() + su.rowptr[i + 1];
    const int *q = std::lower_bound(b, e, j);
    return (q != e && *q == j) ? (int)(q - su.colidx.data()) : -1;
  };
  int c0 = 0;
  std::vector<int> inst_line_off(1, 0);
  for (const ExtrudedInput &blk : t->mesh_blocks) {
    const int nc2 = blk.nc2, nl = blk.nlayers;
    inst_line_off.push_back(inst_line_off.back() + nc2);
    for (int c2 = 0; c2 < nc2; c2++) {
      for (int k = 0; k < nl; k++) {
        const int i = c0 + k * nc2 + c2;
        line_cells.push_back(i);
        pd.push_back(find(i, i));
        plo.push_back(k > 0 ? find(i, i - nc2) : -1);
        phi.push_back(k + 1 < nl ? find(i, i + nc2) : -1);
        if (pd.back() < 0) return set_error(TDY_ERR_LIB, "solver: missing diagonal of cell %d", i);
      }
      line_off.push_back((int)line_cells.size());
    }
    for (int i = c0; i < c0 + nc2 * nl; i++) cell_seg[i] = (int)seg_off.size() - 1;
    c0 += nc2 * nl;
    seg_off.push_back(c0);
  }
  if (c0 != s->n) return set_error(TDY_ERR_LIB, "solver: blocks cover %d of %d cells", c0, s->n);
  s->nseg = (int)seg_off.size() - 1;
  s->nlines = (int)line_off.size() - 1;
  std::vector<int> chunk_off(1, 0), seg_chunk(1, 0);
  for (int g = 0; g < s->nseg; g++) {
    for (int i = seg_off[g]; i < seg_off[g + 1]; i += kChunk) chunk_off.push_back(std::min(i + kChunk, seg_off[g + 1]));
    seg_chunk.push_back((int)chunk_off.size() - 1);
  }
  s->nchunks = (int)chunk_off.size() - 1;
  s->h_seg_off = seg_off;
  s->h_inst_line_off = inst_line_off;
  s->h_order.resize(s->nseg);
  for (int g = 0; g < s->nseg; g++) s->h_order[g] = g;
  std::stable_sort(s->h_order.begin(), s->h_order.end(),
                   [&](int x, int y) { return seg_off[x + 1] - seg_off[x] > seg_off[y + 1] - seg_off[y]; });
  int ierr;
  // every array in one allocation, uploaded with one copy
  std::vector<int> dp(s->n);
  for (int i = 0; i < s->n; i++) dp[i] = find(i, i);  // every row has its diagonal (checked above per line cell)
  Arena ar;
  ar.up(&s->rowptr, su.rowptr);
  ar.up(&s->colidx, su.colidx);
  ar.up(&s->seg_off, seg_off);
  ar.up(&s->chunk_off, chunk_off);
  ar.up(&s->seg_chunk, seg_chunk);
  ar.work(&s->part, s->nchunks);
  ar.work(&s->part2, s->nchunks);
  ar.up(&s->cell_seg, cell_seg);
  ar.up(&s->line_off, line_off);
  ar.up(&s->line_cells, line_cells);
  ar.up(&s->pos_d, pd);
  ar.up(&s->dpos, dp);
  ar.up(&s->pos_lo, plo);
  ar.up(&s->pos_hi, phi);
  ar.work(&s->x, s->n);
  ar.work(&s->xb, s->n);
  ar.work(&s->lam, s->nseg);
  ar.work(&s->trial, s->nseg);
  ar.work(&s->commit, s->nseg);
  ar.work(&s->F, s->n);
  ar.work(&s->J, s->nnz);
  ar.work(&s->fn2, s->nseg);
  ar.work(&s->scal, (size_t)S_NSCAL * s->nseg);
  ar.work(&s->newt_active, s->nseg);
  ar.work(&s->lin_active, s->nseg);
  ar.work(&s->lin_its, s->nseg);
  ar.up(&s->inst_line_off, inst_line_off);
  ar.work(&s->block_inst, s->nseg);
  ar.work(&s->block_mask, s->nseg);
  ar.work(&s->ticket, 1);
  if ((ierr = ar.commit(s->st))) return ierr;
  s->allocs.push_back(ar.base);
  // the allocations and uploads complete before any other stream uses them
  // (and before the host vectors above go out of scope)
  SCUDA(cudaStreamSynchronize(s->st));
  return 0;
}

}  // namespace

void device_solver_destroy(_p_TDy *t) {
  delete t->solver;
  t->solver = nullptr;
}

int device_num_instances(_p_TDy *t) { return (int)t->mesh_blocks.size(); }

// the last linear_solve's set-up and Krylov times (ms), once its events completed
static int add_linear_times(SolverState *s, double *prec, double *kry) {
  SCUDA(cudaEventSynchronize(s->tev[4]));
  float m1 = 0.f, m2 = 0.f;
  SCUDA(cudaEventElapsedTime(&m1, s->tev[2], s->tev[3]));
  SCUDA(cudaEventElapsedTime(&m2, s->tev[3], s->tev[4]));
  *prec += m1;
  *kry += m2;
  return 0;
}

int device_be_solve(_p_TDy *t, double dt, double *dU, const TDyNewtonOptions &o, TDyNewtonStats *stats,
                    int *inst_its, double *inst_rel, void *stream) {
  int ierr;
  if ((ierr = solver_init(t))) {
    device_solver_destroy(t);
    return ierr;
  }
  SolverState *s = t->solver;
  // a capturable stream: the caller's, else the handle's own
  cudaStream_t st = (cudaStream_t)(stream ? stream : device_default_stream(t));
  const int n = s->n, ns = s->nseg;
  t->dtime = dt;
  if ((ierr = device_presolve(t, dU, st))) return ierr;
  SCUDA(cudaMemcpyAsync(s->x, dU, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  SCUDA(cudaMemcpyAsync(s->xb, dU, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  std::vector<double> f0(ns, 0.0), fn(ns, 0.0), g2(ns, 0.0), lam(ns, 1.0);
  std::vector<int> act(ns, 1), its(ns, 0), trial(ns, 0), commit(ns, 0), step_conv(ns, 0), failed(ns, 0);
  // instances retired by the caller are not advanced (TDySetActiveInstances)
  const bool masked = (int)t->inst_active.size() == ns;
  std::vector<int> live;
  for (int g = 0; g < ns; g++) {
    if (masked && !t->inst_active[g]) act[g] = 0;
    if (act[g]) live.push_back(g);
  }
  std::vector<double> y2(ns, 0.0), x2(ns, 0.0);
  std::vector<int> lin_its(ns, 0);  // inner iterations of the last solve, per instance
  long long lin_total = 0;
  int fell_back = 0;
  std::vector<int> trial_list;
  double t_eval = 0.0, t_prec = 0.0, t_kry = 0.0;  // ms on the stream
  int inner_redo = 0;  // FP32 inner solves redone in FP64 (instances x Newton iterations)
  // F and J at x (= xb for every instance after each evaluation below), and
  // the squared per-instance residual norms into g2
  // `sub` (host list of instances, or null for all): only those instances'
  // states changed since the last evaluation, the others keep F and J
  std::vector<int> all_inst(ns);
  for (int g = 0; g < ns; g++) all_inst[g] = g;
  auto eval_all = [&]() -> int {
    int e;
    if (s->eval_mode < 0 && device_inst_ok(t) && ns > 1) {
      // time both schedules once on this evaluation (they give the same bits)
      cudaEvent_t e0, e1;
      SCUDA(cudaEventCreate(&e0));
      SCUDA(cudaEventCreate(&e1));
      for (int mode = 0; mode < 2; mode++) {
        for (int rep = 0; rep < 2; rep++) {  // the first run warms up
          SCUDA(cudaEventRecord(e0, st));
          e = mode == 0 ? device_eval(t, FORM_SNES, 0.0, s->x, nullptr, 0.0, s->F, s->J, st)
                        : device_eval_instances(t, s->x, s->F, s->J, all_inst.data(), ns, st);
          if (e) return e;
          SCUDA(cudaEventRecord(e1, st));
          SCUDA(cudaEventSynchronize(e1));
          float ms = 0.f;
          SCUDA(cudaEventElapsedTime(&ms, e0, e1));
          s->eval_ms[mode] = ms;
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      s->eval_mode = s->eval_ms[1] < s->eval_ms[0] ? 1 : 0;
      return 0;
    }
    if (s->eval_mode < 0) s->eval_mode = 0;
    return s->eval_mode == 1 ? device_eval_instances(t, s->x, s->F, s->J, all_inst.data(), ns, st)
                             : device_eval(t, FORM_SNES, 0.0, s->x, nullptr, 0.0, s->F, s->J, st);
  };
  auto evaluate = [&](const std::vector<int> *sub = nullptr) -> int {
    int e;
    bool part = sub && (int)sub->size() < ns && device_inst_ok(t);
    if (part)  // one CTA per instance: only for instances small enough for one SM
      for (int g : *sub) part = part && s->h_seg_off[g + 1] - s->h_seg_off[g] <= 65536;
    SCUDA(cudaEventRecord(s->tev[0], st));
    if (part)
      e = device_eval_instances(t, s->x, s->F, s->J, sub->data(), (int)sub->size(), st);
    else
      e = eval_all();
    if (e) return e;
    SCUDA(cudaEventRecord(s->tev[1], st));
    seg_dot<double, double>(s, s->F, s->F, nullptr, nullptr, s->fn2, nullptr, st);
    SCUDA(cudaGetLastError());
    SCUDA(cudaMemcpyAsync(g2.data(), s->fn2, sizeof(double) * ns, cudaMemcpyDeviceToHost, st));
    SCUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    SCUDA(cudaEventElapsedTime(&ms, s->tev[0], s->tev[1]));
    t_eval += ms;
    return 0;
  };
  if ((ierr = evaluate(masked ? &live : nullptr))) return ierr;
  for (int g = 0; g < ns; g++) f0[g] = fn[g] = std::sqrt(g2[g]);
  const double alpha = 1e-4;  // sufficient-decrease constant of PETSc's backtracking line search
  constexpr double kMaxStep = 1e8;  // PETSc's default SNESLineSearch maxstep
  const int max_backtracks = 12;
  for (int it = 0;; it++) {
    bool any = false;
    for (int g = 0; g < ns; g++) {
      if (act[g]) {
        if (!std::isfinite(fn[g]) || !std::isfinite(f0[g])) {  // diverged: stop, reported as not converged
          act[g] = 0;
          failed[g] = 1;
          continue;
        }
        const bool done = !(fn[g] > o.atol) || fn[g] <= o.rtol * f0[g];
        if (done || it == o.max_it) act[g] = 0;  // converged, or out of iterations (reported below)
        else its[g] = it + 1;
      }
      any |= act[g] != 0;
    }
    if (!any) break;
    SCUDA(cudaMemcpyAsync(s->newt_active, act.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, st));
    // FP32 inner solves for the first fp32_max_it Newton iterations, FP64 after
    // (an instance still iterating then is one whose FP32 directions stall;
    // the switch depends only on the iteration number, so an instance takes it
    // at the same point alone and in a batch)
    const bool fp32 = o.linear_fp32 && (o.fp32_max_it < 0 || it < o.fp32_max_it);
    if (o.linear_fp32 && !fp32) fell_back = 1;
    const void *y;
    if (fp32) {
      // FP32 inner solves stop after a quarter of linear_max_it (at least 20
      // iterations); one that runs out (FP32 rounding can stall BiCGStab
      // above the tolerance on ill-conditioned Jacobians) is solved again in
      // FP64 with the full count, and the instance steps along that direction
      // (kept in the FP32 array).  The choice depends on the instance alone,
      // so it is the same alone and in a batch.
      TDyNewtonOptions o32 = o;
      o32.linear_max_it = std::min(o.linear_max_it, std::max(20, o.linear_max_it / 4));
      ierr = linear_solve<float>(s, s->k32, o32, st, &lin_total, lin_its);
      if (ierr) return ierr;
      if ((ierr = add_linear_times(s, &t_prec, &t_kry))) return ierr;
      std::vector<int> redo(ns, 0);
      bool any_redo = false;
      for (int g = 0; g < ns; g++)
        if (act[g] && lin_its[g] >= o32.linear_max_it) any_redo = redo[g] = 1;
      if (any_redo) {
        SCUDA(cudaMemcpyAsync(s->newt_active, redo.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, st));
        std::vector<int> lin64;
        if ((ierr = linear_solve<double>(s, s->k64, o, st, &lin_total, lin64))) return ierr;
        if ((ierr = add_linear_times(s, &t_prec, &t_kry))) return ierr;
        cast_masked_kernel<<<nblk(n, 256), 256, 0, st>>>(n, s->cell_seg, s->newt_active, (const double *)s->k64.y,
                                                         (float *)s->k32.y);
        SCUDA(cudaMemcpyAsync(s->newt_active, act.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, st));
        SCUDA(cudaStreamSynchronize(st));  // redo and act (host vectors) stay valid until here
        for (int g = 0; g < ns; g++)
          if (redo[g]) {
            lin_its[g] = lin64[g];
            inner_redo++;
          }
      }
      y = s->k32.y;
    } else {
      ierr = linear_solve<double>(s, s->k64, o, st, &lin_total, lin_its);
      if (!ierr) ierr = add_linear_times(s, &t_prec, &t_kry);
      y = s->k64.y;
    }
    if (ierr) return ierr;
    // ||y|| and ||x|| before the step: PETSc's backtracking line search caps
    // the step at maxstep and ends with convergence by the step test when the
    // full step fails and ||y|| < stol ||x||
    {
      if (fp32)
        seg_dot<float, float>(s, (const float *)y, (const float *)y, nullptr, nullptr, s->fn2, nullptr, st);
      else
        seg_dot<double, double>(s, (const double *)y, (const double *)y, nullptr, nullptr, s->fn2, nullptr, st);
      seg_dot<double, double>(s, s->xb, s->xb, nullptr, nullptr, s->scal + (size_t)S_T2 * ns, nullptr, st);
      SCUDA(cudaGetLastError());
      SCUDA(cudaMemcpyAsync(y2.data(), s->fn2, sizeof(double) * ns, cudaMemcpyDeviceToHost, st));
      SCUDA(cudaMemcpyAsync(x2.data(), s->scal + (size_t)S_T2 * ns, sizeof(double) * ns, cudaMemcpyDeviceToHost, st));
      SCUDA(cudaStreamSynchronize(st));
    }
    // backtracking per instance: accept when ||F(x - lam y)||^2 <= (1 - 2 alpha lam) ||F(x)||^2
    // (initial slope -||F||^2 of the Newton direction), else a quadratic fit of
    // lam clamped to [0.1 lam, 0.5 lam] (PETSc SNESLineSearchApply_BT)
    for (int g = 0; g < ns; g++) {
      trial[g] = act[g];
      // ||lam y|| <= maxstep (SNESLineSearch maxstep, PETSc default 1e8): a
      // direction from a diverged inner solve cannot throw the state away
      const double yn = std::sqrt(y2[g]);
      lam[g] = yn > kMaxStep ? kMaxStep / yn : 1.0;
    }
    for (int ls = 0; ls <= max_backtracks; ls++) {
      SCUDA(cudaMemcpyAsync(s->trial, trial.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, st));
      SCUDA(cudaMemcpyAsync(s->lam, lam.data(), sizeof(double) * ns, cudaMemcpyHostToDevice, st));
      if (fp32)
        trial_kernel<float><<<nblk(n, 256), 256, 0, st>>>(n, s->cell_seg, s->trial, s->lam, (const float *)y, s->xb,
                                                          s->x);
      else
        trial_kernel<double><<<nblk(n, 256), 256, 0, st>>>(n, s->cell_seg, s->trial, s->lam, (const double *)y, s->xb,
                                                           s->x);
      trial_list.clear();
      for (int g = 0; g < ns; g++)
        if (trial[g]) trial_list.push_back(g);
      if ((ierr = evaluate(&trial_list))) return ierr;
      bool pending = false;
      for (int g = 0; g < ns; g++) {
        commit[g] = 0;
        if (!trial[g]) continue;
        const double f = fn[g] * fn[g], gg = g2[g];
        const bool inner_ok = lin_its[g] < o.linear_max_it;
        if (std::isfinite(gg) &&
            (gg <= (1.0 - 2.0 * alpha * lam[g]) * f || (ls == max_backtracks && (inner_ok || gg <= 4.0 * f)))) {
          // sufficient decrease; or, at the smallest step, a Newton direction
          // from a converged inner solve (the next iteration's Jacobian at the
          // nearby state usually gives a better one; at the FP64 noise floor
          // no step lowers ||F|| and the step test ends the instance), or one
          // from an unconverged inner solve that at most doubles ||F||
          commit[g] = 1;
          trial[g] = 0;
          fn[g] = std::sqrt(gg);
        } else if (ls == max_backtracks) {
          // no finite residual along the step, or an unconverged inner solve
          // whose smallest step more than doubles ||F||: keep the last
          // accepted state and stop, converged by the step test if the step
          // is negligible, else failed
          trial[g] = 0;
          act[g] = 0;
          if (o.stol > 0.0 && std::sqrt(y2[g]) < o.stol * std::sqrt(x2[g]))
            step_conv[g] = 1;
          else
            failed[g] = 1;
        } else {
          const double slope = -f;
          double lt = std::isfinite(gg) ? -slope * lam[g] * lam[g] / (gg - f - 2.0 * slope * lam[g]) : 0.0;
          lt = std::min(lt, 0.5 * lam[g]);
          lam[g] = (lt <= 0.1 * lam[g]) ? 0.1 * lam[g] : lt;
          pending = true;
        }
      }
      SCUDA(cudaMemcpyAsync(s->commit, commit.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, st));
      commit_kernel<<<nblk(n, 256), 256, 0, st>>>(n, s->cell_seg, s->commit, s->x, s->xb);
      SCUDA(cudaGetLastError());
      if (!pending) break;
    }
    // every instance still active now has x == xb, so its F and J rows hold
    // the accepted state (instances do not couple).
    // Step test (SNESConvergedDefault): ||y|| < stol ||x|| per instance, with
    // y the full Newton step (PETSc's backtracking line search reports the
    // norm of the step before its lambda scaling), so a step cut short by the
    // line search does not count as convergence.
    if (o.stol > 0.0) {
      if (fp32)
        seg_dot<float, float>(s, (const float *)y, (const float *)y, nullptr, nullptr, s->fn2, nullptr, st);
      else
        seg_dot<double, double>(s, (const double *)y, (const double *)y, nullptr, nullptr, s->fn2, nullptr, st);
      seg_dot<double, double>(s, s->xb, s->xb, nullptr, nullptr, s->scal + (size_t)S_T2 * ns, nullptr, st);
      SCUDA(cudaGetLastError());
      SCUDA(cudaMemcpyAsync(y2.data(), s->fn2, sizeof(double) * ns, cudaMemcpyDeviceToHost, st));
      SCUDA(cudaMemcpyAsync(x2.data(), s->scal + (size_t)S_T2 * ns, sizeof(double) * ns, cudaMemcpyDeviceToHost, st));
      SCUDA(cudaStreamSynchronize(st));
      for (int g = 0; g < ns; g++)
        if (act[g] && std::sqrt(y2[g]) < o.stol * std::sqrt(x2[g])) {
          act[g] = 0;
          step_conv[g] = 1;
        }
    }
  }
  SCUDA(cudaMemcpyAsync(dU, s->xb, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  SCUDA(cudaStreamSynchronize(st));
  int conv = 0, conv_step = 0, maxit = 0;
  t->inst_status.assign(ns, TDY_INSTANCE_NOT_CONVERGED);
  double worst = 0.0;
  for (int g = 0; g < ns; g++) {
    const bool retired = masked && !t->inst_active[g];
    const double rel = (f0[g] > 0.0 && !retired) ? fn[g] / f0[g] : 0.0;
    const bool fin = !retired && !failed[g] && std::isfinite(fn[g]);
    const bool ok = fin && (!(fn[g] > o.atol) || rel <= o.rtol);
    conv += ok ? 1 : 0;
    conv_step += (fin && !ok && step_conv[g]) ? 1 : 0;
    t->inst_status[g] = retired ? TDY_INSTANCE_INACTIVE
                                : ok ? TDY_INSTANCE_CONVERGED
                                     : (fin && step_conv[g]) ? TDY_INSTANCE_STEP_TEST : TDY_INSTANCE_NOT_CONVERGED;
    worst = std::max(worst, rel);
    maxit = std::max(maxit, its[g]);
    if (inst_its) inst_its[g] = its[g];
    if (inst_rel) inst_rel[g] = rel;
  }
  if (stats) {
    stats->newton_iterations = maxit;
    stats->linear_iterations = lin_total;
    stats->converged = conv;
    stats->ninstances = ns;
    stats->max_rel_residual = worst;
    stats->step_converged = conv_step;
    stats->precond_used = s->precond_used;
    stats->clusters = s->precond_used == TDY_PRECOND_CLUSTERS ? s->ncl : 0;
    stats->cluster_cells = s->precond_used == TDY_PRECOND_CLUSTERS ? s->ncl_cells : 0;
    stats->cluster_cells_diagonal = s->precond_used == TDY_PRECOND_CLUSTERS ? s->ncl_big_cells : 0;
    stats->fp64_fallback = fell_back;
    stats->eval_schedule = s->eval_mode;
    stats->eval_s = 1e-3 * t_eval;
    stats->precond_s = 1e-3 * t_prec;
    stats->krylov_s = 1e-3 * t_kry;
    stats->fp64_inner_redo = inner_redo;
    stats->block_instances = s->precond_used == TDY_PRECOND_LINES ? s->n_block : 0;
    stats->block_max_cells = s->precond_used == TDY_PRECOND_LINES ? s->mask_for : -1;
  }
  return 0;
}

}  // namespace tdy
