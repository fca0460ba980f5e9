// sbm_solver.cu -- SBM operator and conjugate-gradient solvers on GB300.
//
// Replaces the three inline CG loops of the reference electrochemistry
// program SBMES_3D_MPI_CH_Gr_CONJG_VD_T05_01_BQ_hx3.f90 (SBMES below):
// CnE at SBMES:501-554, phP at :657-714, phE at :737-795.  The reference
// does per iteration: ghost exchange of PRJ, WMX = L PRJ, four allgather
// reductions, x/RES updates and PRJ = RES + bet PRJ.  Here one iteration is
// three fused kernels on one device-resident domain:
//   k_apply     q = A p (ghost rules applied while loading) + p.q  -> alpha
//   k_update    x += alpha p, r -= alpha q, r.r (+ stop norm)      -> beta, done
//   k_direction p = z + beta p
// Every scalar stays on the device; the last block of each reduction
// computes alpha / beta / the stopping norm in a fixed summation order
// (deterministic).  Chunks of iterations are captured once into a CUDA
// graph and replayed; a `done` flag turns the rest of a chunk into no-ops.
// The FP64 solver replays its chunk from the host (one chunk in flight
// while the host reads the previous one's state); the mixed solver loops
// its chunk on the device in a WHILE conditional node (one graph launch per
// solve), or from the host under SBM_TUNE_HOST_LOOP.
//
// Two precisions:
//   FP64  the drop-in: the reference's CG and stopping rules.
//   MIXED FP32 CG (FP32 stencil and vectors on a 16-byte-aligned internal
//         layout, per-thread FP32 partial sums promoted to FP64 for the grid
//         reduction) with FP64 iterative refinement by reliable updates: the
//         residual is periodically recomputed in FP64 and the correction
//         accumulated in FP64, without restarting the Krylov space.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "sbm_internal.cuh"
#include "sbm_net.cuh"

namespace sbm {

// --------------------------------------------------------------- helpers

int pick_zc(const Geo& g, int tuned) {
  if (tuned > 0) return tuned;
  const int64_t tiles = (int64_t)((g.ny + BX - 1) / BX) * ((g.nx + BY - 1) / BY);
  const int64_t target = 2 * 152 * 8;  // two waves of 8 resident 256-thread blocks per SM
  int zc = 1;
  for (int c = 2; c <= 16; c *= 2)
    if (tiles * ((g.nz + c - 1) / c) >= target) zc = c;
  return zc;
}

// Per-thread z-march over interior column (i, j), planes k0..k1.  Body is
// called with (c, k, pc, pzm, pzp_eff, kc, kzm, kzp) where p's z-neighbours
// already carry the ghost rule (RULE) or the stored ghosts (!RULE).
#define SBM_COLUMN_PROLOGUE(g, zc)                                   \
  const int i = blockIdx.x * BX + threadIdx.x + 1;                   \
  const int j = blockIdx.y * BY + threadIdx.y + 1;                   \
  const int k0 = blockIdx.z * (zc) + 1;                              \
  const int k1 = min(k0 + (zc)-1, (g).nz);                           \
  const bool active = (i <= (g).ny) && (j <= (g).nx);

// Loads the in-plane neighbours of p and hk at c and applies the ghost
// rules of the search direction when RULE: y faces copy the edge; x faces
// copy (SBM_BC_COPY) or read zero (SBM_BC_ZERO).
template <typename T, bool RULE>
__device__ __forceinline__ T stencil_at(const Geo& g, const T* __restrict__ hk,
                                        const T* __restrict__ fc, const T* __restrict__ p,
                                        int64_t c, int i, int j, T pc, T kc, T pzm, T pzp, T kzm,
                                        T kzp, int bcx0, int bcx1) {
  T pym = p[c - 1], pyp = p[c + 1], pxm = p[c - g.sx], pxp = p[c + g.sx];
  if (RULE) {
    if (i == 1) pym = pc;
    if (i == g.ny) pyp = pc;
    if (j == 1) pxm = bcx0 ? T(0) : pc;
    if (j == g.nx) pxp = bcx1 ? T(0) : pc;
  }
  if (fc) return face_sum_stored<T>(g, fc, c, pc, pyp, pym, pxp, pxm, pzp, pzm);
  const T kym = hk[c - 1], kyp = hk[c + 1], kxm = hk[c - g.sx], kxp = hk[c + g.sx];
  return face_sum<T>(kc, pc, kyp, pyp, kym, pym, kxp, pxp, kxm, pxm, kzp, pzp, kzm, pzm);
}

// ---------------------------------------------------------------- kernels

// q = A p.  DOT: also p.q -> pq, alpha = rho / pq.  RULE: ghost rules on p.
template <typename T, int FORM, bool DOT, bool RULE>
__global__ void __launch_bounds__(BX* BY) k_apply(OpArgs<T> op, int zc, const T* __restrict__ p,
                                                  T* __restrict__ q, double* partials,
                                                  CgState* st) {
  const Geo g = op.g;
  if (DOT && st->done) return;
  SBM_COLUMN_PROLOGUE(g, zc)
  T acc = T(0);
  if (active && k0 <= k1) {
    const bool sf = op.fc != nullptr;  // stored faces: no half coefficient reads
    int64_t c = g.ix(i, j, k0);
    T pc = p[c], kc = sf ? T(0) : op.hk[c];
    T pzm = p[c - g.sz], kzm = sf ? T(0) : op.hk[c - g.sz];
    if (RULE && k0 == 1) pzm = pc;
    for (int k = k0; k <= k1; ++k) {
      const T pzp_raw = p[c + g.sz];
      const T kzp = sf ? T(0) : op.hk[c + g.sz];
      const T pzp = (RULE && k == g.nz) ? pc : pzp_raw;
      const T s = stencil_at<T, RULE>(g, op.hk, op.fc, p, c, i, j, pc, kc, pzm, pzp, kzm, kzp,
                                      op.bcx0, op.bcx1);
      T qv;
      if (FORM == 0)
        qv = op.scale * s;
      else
        qv = op.diag[c] * pc - op.scale * s;
      q[c] = qv;
      if (DOT) acc += pc * qv;
      pzm = pc;
      kzm = kc;
      pc = pzp_raw;
      kc = kzp;
      c += g.sz;
    }
  }
  if (DOT) {
    double v[1] = {(double)acc}, tot[1];
    if (grid_reduce<1>(v, partials, &st->counter[0], tot)) {
      if (threadIdx.x == 0 && threadIdx.y == 0) {
        const double pq = tot[0];
        st->pq = pq;
        st->alpha = st->rho / pq;
        if (pq == 0.0) st->done = 4;
        else if (!isfinite(pq)) st->done = 3;
      }
    }
  }
}

// Start of a solve: r = b - A x with x's stored ghosts (SBMES:492-499,
// :649-655, :729-735), p = z (= invd*r with Jacobi, r otherwise), rho = r.z,
// rr = rr0 = r.r.
template <int FORM, bool PC>
__global__ void __launch_bounds__(BX* BY)
    k_residual_mem(OpArgs<double> op, int zc, const double* __restrict__ b,
                   const double* __restrict__ x, double* __restrict__ r,
                   double* __restrict__ p, const double* __restrict__ invd, double* partials,
                   CgState* st) {
  const Geo g = op.g;
  SBM_COLUMN_PROLOGUE(g, zc)
  double a_rr = 0.0, a_rz = 0.0;
  if (active && k0 <= k1) {
    const bool sf = op.fc != nullptr;
    int64_t c = g.ix(i, j, k0);
    double pc = x[c], kc = sf ? 0.0 : op.hk[c];
    double pzm = x[c - g.sz], kzm = sf ? 0.0 : op.hk[c - g.sz];
    for (int k = k0; k <= k1; ++k) {
      const double pzp = x[c + g.sz], kzp = sf ? 0.0 : op.hk[c + g.sz];
      const double s = stencil_at<double, false>(g, op.hk, op.fc, x, c, i, j, pc, kc, pzm, pzp,
                                                 kzm, kzp, 0, 0);
      const double ax = (FORM == 0) ? op.scale * s : op.diag[c] * pc - op.scale * s;
      const double rv = b[c] - ax;
      r[c] = rv;
      const double zv = PC ? invd[c] * rv : rv;
      p[c] = zv;
      a_rr += rv * rv;
      a_rz += rv * zv;
      pzm = pc;
      kzm = kc;
      pc = pzp;
      kc = kzp;
      c += g.sz;
    }
  }
  double v[2] = {a_rr, a_rz}, tot[2];
  if (grid_reduce<2>(v, partials, &st->counter[2], tot)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      st->rr = tot[0];
      st->rr0 = tot[0];
      st->rho = tot[1];
      st->iter = 0;
      st->rms = 1.0;
      st->done = (st->stop_rule == SBM_STOP_REL_RES && tot[0] == 0.0) ? 1 : 0;
    }
  }
}

// x += alpha p; r -= alpha q; rho = r.z, rr = r.r, stop norm; beta.
// STOP: SBM_STOP_REF_UPDATE (sum w*(x_new-x_old)^2, SBMES:699-705),
// SBM_STOP_REF_RESID (sum w*r^2, SBMES:545-547) or SBM_STOP_REL_RES.
template <typename T, int STOP, bool PC>
__global__ void __launch_bounds__(BX* BY)
    k_update(Geo g, int zc, T* __restrict__ x, const T* __restrict__ p, T* __restrict__ r,
             const T* __restrict__ q, const double* __restrict__ w, const T* __restrict__ invd,
             double* partials, CgState* st) {
  if (st->done) return;
  SBM_COLUMN_PROLOGUE(g, zc)
  const T alpha = (T)st->alpha;
  T a_rr = T(0), a_rz = T(0);
  double a_w = 0.0;
  if (active && k0 <= k1) {
    int64_t c = g.ix(i, j, k0);
    for (int k = k0; k <= k1; ++k, c += g.sz) {
      const T xo = x[c];
      const T xn = xo + alpha * p[c];
      x[c] = xn;
      const T rn = r[c] - alpha * q[c];
      r[c] = rn;
      a_rr += rn * rn;
      if (PC) a_rz += rn * (invd[c] * rn);
      if (STOP == SBM_STOP_REF_UPDATE) {
        const double d = (double)xn - (double)xo;
        a_w += (d * d) * w[c];
      } else if (STOP == SBM_STOP_REF_RESID) {
        a_w += ((double)rn * (double)rn) * w[c];
      }
    }
  }
  double v[3] = {(double)a_rr, PC ? (double)a_rz : (double)a_rr, a_w}, tot[3];
  if (grid_reduce<3>(v, partials, &st->counter[1], tot)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      const double rho_new = tot[1];
      const double beta = rho_new / st->rho;
      double rms;
      if (STOP == SBM_STOP_REL_RES)
        rms = sqrt(tot[0]) / sqrt(st->rr0);
      else
        rms = sqrt(tot[2] / st->wsum);
      st->rr = tot[0];
      st->rho = rho_new;
      st->beta = beta;
      st->rms = rms;
      const int it = st->iter + 1;
      st->iter = it;
      if (!isfinite(rms) || !isfinite(st->alpha)) st->done = 3;
      else if (!(rms > st->tol)) st->done = 1;
      else if (it >= st->max_it) st->done = 2;
    }
  }
}

// p = z + beta p, z = invd*r (Jacobi) or r.
template <typename T, bool PC>
__global__ void __launch_bounds__(BX* BY)
    k_direction(Geo g, int zc, const T* __restrict__ r, T* __restrict__ p,
                const T* __restrict__ invd, const CgState* st) {
  if (st->done) return;
  SBM_COLUMN_PROLOGUE(g, zc)
  const T beta = (T)st->beta;
  if (active && k0 <= k1) {
    int64_t c = g.ix(i, j, k0);
    for (int k = k0; k <= k1; ++k, c += g.sz) {
      const T z = PC ? invd[c] * r[c] : r[c];
      p[c] = z + beta * p[c];
    }
  }
}

// Inverse diagonal of the homogeneous operator (faces whose ghost copies the
// edge contribute nothing), for Jacobi preconditioning.
template <typename T>
__global__ void __launch_bounds__(BX* BY)
    k_invdiag(OpArgs<T> op, int zc, T* __restrict__ invd) {
  const Geo g = op.g;
  SBM_COLUMN_PROLOGUE(g, zc)
  if (!active) return;
  for (int k = k0; k <= k1; ++k) {
    const int64_t c = g.ix(i, j, k);
    const T kc = op.hk[c];
    T sum = T(0);
    if (i > 1) sum += op.hk[c - 1] + kc;
    if (i < g.ny) sum += op.hk[c + 1] + kc;
    if (j > 1 || op.bcx0) sum += op.hk[c - g.sx] + kc;
    if (j < g.nx || op.bcx1) sum += op.hk[c + g.sx] + kc;
    if (k > 1) sum += op.hk[c - g.sz] + kc;
    if (k < g.nz) sum += op.hk[c + g.sz] + kc;
    const T d = (op.form == 0) ? -op.scale * sum : op.diag[c] + op.scale * sum;
    invd[c] = (d != T(0)) ? T(1) / d : T(0);
  }
}

template <typename T>
__global__ void k_accum(Geo g, int zc, double* __restrict__ acc, const T* __restrict__ v) {
  SBM_COLUMN_PROLOGUE(g, zc)
  if (!active) return;
  for (int k = k0; k <= k1; ++k) {
    const int64_t c = g.ix(i, j, k);
    acc[c] = acc[c] + (double)v[c];
  }
}

__global__ void k_to_f32(int64_t n, const double* __restrict__ a, float* __restrict__ fa,
                         const double* __restrict__ b, float* __restrict__ fb) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    fa[c] = (float)a[c];
    if (b) fb[c] = (float)b[c];
  }
}

__global__ void k_half(int64_t n, const double* __restrict__ k, double* __restrict__ hk) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    hk[c] = k[c] * 0.5;
}

static dim3 flat_grid(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return dim3((unsigned)b);
}

// ------------------------------------------------------------ launchers

cudaError_t launch_apply_mem64(const OpArgs<double>& op, const double* x, double* q,
                               cudaStream_t s) {
  const Shape sh = stencil_shape(op.g, pick_zc(op.g, 0));
  if (op.form == 0)
    k_apply<double, 0, false, false><<<sh.grid, sh.block, 0, s>>>(op, sh.zc, x, q, nullptr,
                                                                   nullptr);
  else
    k_apply<double, 1, false, false><<<sh.grid, sh.block, 0, s>>>(op, sh.zc, x, q, nullptr,
                                                                   nullptr);
  SBM_LAUNCHED(1);
  return cudaGetLastError();
}

cudaError_t launch_half(const Geo& g, const double* k, double* hk, cudaStream_t s) {
  k_half<<<flat_grid(g.nh), 256, 0, s>>>(g.nh, k, hk);
  SBM_LAUNCHED(1);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- driver

__global__ void k_graph_loop(cudaGraphConditionalHandle h, CgState* st, int* rounds, int cap,
                             int init) {
  if (threadIdx.x) return;
  const int r = init ? 0 : *rounds + 1;
  *rounds = r;
  const bool more = st->done == 0 && r < cap;
  if (!more && st->done == 0) st->done = 2;
  cudaGraphSetConditional(h, more ? 1u : 0u);
}

int add_graph_loop_node(cudaGraph_t g, const cudaGraphNode_t* dep, cudaGraphConditionalHandle h,
                        CgState* st, int* rounds, int cap, int init, cudaGraphNode_t* out) {
  void* args[] = {&h, &st, &rounds, &cap, &init};
  cudaKernelNodeParams kp{};
  kp.func = reinterpret_cast<void*>(k_graph_loop);
  kp.gridDim = dim3(1);
  kp.blockDim = dim3(32);
  kp.sharedMemBytes = 0;
  kp.kernelParams = args;
  SBM_CUDA_TRY(cudaGraphAddKernelNode(out, g, dep, dep ? 1 : 0, &kp));
  return SBM_OK;
}

namespace {

template <typename T>
void launch_iteration(const OpArgs<T>& op, const Shape& sh, int stop, bool pc, T* x, T* p,
                      T* r, T* q, const double* w, const T* invd, double* partials,
                      CgState* st, cudaStream_t s) {
  const Geo& g = op.g;
  if (op.form == 0)
    k_apply<T, 0, true, true><<<sh.grid, sh.block, 0, s>>>(op, sh.zc, p, q, partials, st);
  else
    k_apply<T, 1, true, true><<<sh.grid, sh.block, 0, s>>>(op, sh.zc, p, q, partials, st);
#define SBM_UPD(STOPV, PCV)                                                                   \
  k_update<T, STOPV, PCV><<<sh.grid, sh.block, 0, s>>>(g, sh.zc, x, p, r, q, w, invd, partials, \
                                                        st)
  if (pc) {
    if (stop == SBM_STOP_REF_UPDATE) SBM_UPD(SBM_STOP_REF_UPDATE, true);
    else if (stop == SBM_STOP_REF_RESID) SBM_UPD(SBM_STOP_REF_RESID, true);
    else SBM_UPD(SBM_STOP_REL_RES, true);
    k_direction<T, true><<<sh.grid, sh.block, 0, s>>>(g, sh.zc, r, p, invd, st);
  } else {
    if (stop == SBM_STOP_REF_UPDATE) SBM_UPD(SBM_STOP_REF_UPDATE, false);
    else if (stop == SBM_STOP_REF_RESID) SBM_UPD(SBM_STOP_REF_RESID, false);
    else SBM_UPD(SBM_STOP_REL_RES, false);
    k_direction<T, false><<<sh.grid, sh.block, 0, s>>>(g, sh.zc, r, p, invd, st);
  }
#undef SBM_UPD
}

int chunk_len(const sbm_ctx* ctx) {
  if (ctx->chunk > 0) return ctx->chunk;
  const int64_t n = ctx->g.ninterior();
  if (n >= (int64_t)4 << 20) return 8;
  if (n >= (int64_t)256 << 10) return 16;
  return 32;
}

// Captures (once per key) a graph of chunk_len(ctx) iterations, each
// issued by body(stream), and returns it with its kernel-node count.
template <typename Body>
int capture_graph(sbm_ctx* ctx, const std::string& key, int nodes_per_iter, Body&& body,
                  cudaGraphExec_t* exec, int* nodes, int len_override = 0) {
  auto it = ctx->graphs.find(key);
  if (it != ctx->graphs.end()) {
    *exec = it->second.exec;
    *nodes = it->second.nodes;
    return SBM_OK;
  }
  const int len = len_override > 0 ? len_override : chunk_len(ctx);
  cudaGraph_t graph = nullptr;
  SBM_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  for (int c = 0; c < len; ++c) body(ctx->stream);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
  if (e != cudaSuccess) {
    set_error("cudaStreamEndCapture", e);
    return SBM_ERR_CUDA;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    set_error("capture launch", e);
    return SBM_ERR_CUDA;
  }
  cudaGraphExec_t ex = nullptr;
  e = cudaGraphInstantiate(&ex, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    set_error("cudaGraphInstantiate", e);
    return SBM_ERR_CUDA;
  }
  ctx->graphs[key] = {ex, graph, nodes_per_iter * len};
  *exec = ex;
  *nodes = nodes_per_iter * len;
  return SBM_OK;
}

// Runs the chunk graph on the device until the state at dst reports done:
// a parent graph (built once per chunk graph and round cap) holds a WHILE
// conditional node whose body is the chunk followed by k_graph_loop, so the
// loop stops after the chunk in which the solve finished, without a host
// round trip per chunk.  The round count is kept in dst->counter[7]; the
// final state is copied through the pinned hbuf[0] to *final_state.
int run_loop(sbm_ctx* ctx, cudaGraph_t chunk, int nodes, int max_it, CgState* dst, CgState* hbuf,
             CgState* final_state) {
  cudaStream_t s = ctx->stream;
  const int cap = max_it > INT_MAX - 2 ? INT_MAX : max_it + 2;  // each round >= 1 iteration
  sbm_ctx::LoopRec& L = ctx->loops[chunk];
  if (!L.exec || L.cap != cap) {
    if (L.exec) cudaGraphExecDestroy(L.exec);
    if (L.graph) cudaGraphDestroy(L.graph);
    L = sbm_ctx::LoopRec();
    SBM_CUDA_TRY(cudaGraphCreate(&L.graph, 0));
    cudaGraphConditionalHandle h;
    SBM_CUDA_TRY(cudaGraphConditionalHandleCreate(&h, L.graph, 0, cudaGraphCondAssignDefault));
    int* rounds = reinterpret_cast<int*>(&dst->counter[7]);
    cudaGraphNode_t first, loop, child, last;
    int rc = add_graph_loop_node(L.graph, nullptr, h, dst, rounds, cap, 1, &first);
    if (rc) return rc;
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    SBM_CUDA_TRY(cudaGraphAddNode(&loop, L.graph, &first, nullptr, 1, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    SBM_CUDA_TRY(cudaGraphAddChildGraphNode(&child, body, nullptr, 0, chunk));
    if ((rc = add_graph_loop_node(body, &child, h, dst, rounds, cap, 0, &last))) return rc;
    SBM_CUDA_TRY(cudaGraphInstantiate(&L.exec, L.graph, 0));
    L.cap = cap;
  }
  SBM_CUDA_TRY(cudaGraphLaunch(L.exec, s));
  SBM_CUDA_TRY(cudaMemcpyAsync(&hbuf[0], dst, sizeof(CgState), cudaMemcpyDeviceToHost, s));
  SBM_CUDA_TRY(cudaEventRecord(ctx->evq[0], s));
  SBM_CUDA_TRY(cudaEventSynchronize(ctx->evq[0]));
  *final_state = hbuf[0];
  const int rounds = (int)hbuf[0].counter[7];
  SBM_LAUNCHED((int64_t)rounds * (nodes + 1) + 1);
  return SBM_OK;
}

// Replays the chunk graph until the state reports done, keeping one chunk
// in flight while the host inspects the previous one.  `hbuf` = 2 pinned
// CgState slots; the final state is copied to *final.
int run_chunks(sbm_ctx* ctx, cudaGraphExec_t exec, int nodes, CgState* dst, CgState* hbuf,
               CgState* final_state) {
  cudaStream_t s = ctx->stream;
  int n = 0;
  SBM_CUDA_TRY(cudaGraphLaunch(exec, s));
  SBM_CUDA_TRY(cudaMemcpyAsync(&hbuf[0], dst, sizeof(CgState), cudaMemcpyDeviceToHost, s));
  SBM_CUDA_TRY(cudaEventRecord(ctx->evq[0], s));
  int launched = 1;
  for (n = 1;; ++n) {
    SBM_CUDA_TRY(cudaGraphLaunch(exec, s));
    SBM_CUDA_TRY(
        cudaMemcpyAsync(&hbuf[n & 1], dst, sizeof(CgState), cudaMemcpyDeviceToHost, s));
    SBM_CUDA_TRY(cudaEventRecord(ctx->evq[n & 1], s));
    ++launched;
    SBM_CUDA_TRY(cudaEventSynchronize(ctx->evq[(n - 1) & 1]));
    if (hbuf[(n - 1) & 1].done) break;
  }
  SBM_CUDA_TRY(cudaEventSynchronize(ctx->evq[n & 1]));
  *final_state = hbuf[n & 1];
  SBM_LAUNCHED((int64_t)launched * nodes);
  return SBM_OK;
}

int status_of(int done) {
  switch (done) {
    case 1: return SBM_OK;
    case 2: return SBM_ERR_MAXIT;
    case 3: return SBM_ERR_NONFINITE;
    case 4: return SBM_ERR_BREAKDOWN;
    case 5: return SBM_ERR_TIMEOUT;
    default: return SBM_ERR_STATE;
  }
}

std::string key_of(const char* tag, const void* a, const void* b, const void* c, const void* d,
                   const void* e, const void* f, const void* h, double scale, int form, int bcx0,
                   int bcx1, int stop, int pc, int zc, int len) {
  char buf[320];
  snprintf(buf, sizeof(buf), "%s|%p|%p|%p|%p|%p|%p|%p|%.17g|%d|%d|%d|%d|%d|%d|%d", tag, a, b, c,
           d, e, f, h, scale, form, bcx0, bcx1, stop, pc, zc, len);
  return std::string(buf);
}

// Stored faces: fc[0..nh) the y+ face of each cell, [nh, 2nh) the x+ face,
// [2nh, 3nh) the z+ face (hk_nb + hk_c), and [3nh, 4nh) the sum of the six
// faces of each interior cell (the residual replacement's diagonal form).
__global__ void k_faces(Geo g, const double* __restrict__ hk, double* __restrict__ fc) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.nh;
       c += (int64_t)gridDim.x * blockDim.x) {
    const double kc = hk[c];
    fc[c] = c + 1 < g.nh ? hk[c + 1] + kc : 0.0;
    fc[g.nh + c] = c + g.sx < g.nh ? hk[c + g.sx] + kc : 0.0;
    fc[2 * g.nh + c] = c + g.sz < g.nh ? hk[c + g.sz] + kc : 0.0;
    double dsum = 0.0;
    if (c - g.sz >= 0 && c + g.sz < g.nh) {  // every cell whose six neighbours exist
      dsum = (hk[c + 1] + kc) + (kc + hk[c - 1]);
      dsum += (hk[c + g.sx] + kc) + (kc + hk[c - g.sx]);
      dsum += (hk[c + g.sz] + kc) + (kc + hk[c - g.sz]);
    }
    fc[3 * g.nh + c] = dsum;
  }
}

// Stored faces of hk (OpArgs::fc) into ctx->fc64, allocated on first use.
int compute_faces(sbm_ctx* ctx, const double* hk, cudaStream_t s) {
  const Geo& g = ctx->g;
  if (!ctx->fc64) {
    const cudaError_t e = cudaMalloc(&ctx->fc64, sizeof(double) * 4 * (size_t)g.nh);
    if (e != cudaSuccess) {
      ctx->fc64 = nullptr;
      set_error("cudaMalloc faces", e);
      return SBM_ERR_NOMEM;
    }
  }
  k_faces<<<flat_grid(g.nh), 256, 0, s>>>(g, hk, ctx->fc64);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

int solve_fp64(sbm_ctx* ctx, const SolveSpec& sp, SolveResult* out) {
  const Geo& g = ctx->g;
  cudaStream_t s = ctx->stream;
  const Shape sh = stencil_shape(g, pick_zc(g, ctx->zc64));
  OpArgs<double> op{g, sp.hk64, sp.diag64, sp.scale, sp.form, sp.bcx0, sp.bcx1};
  int frc = compute_faces(ctx, sp.hk64, s);
  if (frc) return frc;
  op.fc = ctx->fc64;
  const bool pc = sp.precond == SBM_PC_JACOBI;
  CgState* h = &ctx->h_st[2];
  memset(h, 0, sizeof(CgState));
  h->tol = sp.tol;
  h->max_it = sp.max_it;
  h->stop_rule = sp.stop_rule;
  h->wsum = sp.wsum;
  SBM_CUDA_TRY(cudaEventRecord(ctx->ev0, s));
  SBM_CUDA_TRY(cudaMemcpyAsync(ctx->st, h, sizeof(CgState), cudaMemcpyHostToDevice, s));
  double* invd = ctx->d64;
  if (pc) {
    k_invdiag<double><<<sh.grid, sh.block, 0, s>>>(op, sh.zc, invd);
    SBM_LAUNCHED(1);
  }
  if (sp.form == 0) {
    if (pc)
      k_residual_mem<0, true><<<sh.grid, sh.block, 0, s>>>(op, sh.zc, sp.rhs, sp.x, ctx->r64,
                                                          ctx->p64, invd, ctx->partials, ctx->st);
    else
      k_residual_mem<0, false><<<sh.grid, sh.block, 0, s>>>(op, sh.zc, sp.rhs, sp.x, ctx->r64,
                                                           ctx->p64, invd, ctx->partials, ctx->st);
  } else {
    if (pc)
      k_residual_mem<1, true><<<sh.grid, sh.block, 0, s>>>(op, sh.zc, sp.rhs, sp.x, ctx->r64,
                                                          ctx->p64, invd, ctx->partials, ctx->st);
    else
      k_residual_mem<1, false><<<sh.grid, sh.block, 0, s>>>(op, sh.zc, sp.rhs, sp.x, ctx->r64,
                                                           ctx->p64, invd, ctx->partials, ctx->st);
  }
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  const std::string key =
      key_of("fp64", sp.hk64, sp.diag64, sp.x, sp.w, ctx->r64, ctx->p64, ctx->q64, sp.scale,
             sp.form, sp.bcx0, sp.bcx1, sp.stop_rule, pc, sh.zc, chunk_len(ctx));
  cudaGraphExec_t ex = nullptr;
  int nodes = 0;
  int rc = capture_graph(
      ctx, key, 3,
      [&](cudaStream_t s2) {
        launch_iteration<double>(op, sh, sp.stop_rule, pc, sp.x, ctx->p64, ctx->r64, ctx->q64,
                                 sp.w, invd, ctx->partials, ctx->st, s2);
      },
      &ex, &nodes);
  if (rc) return rc;
  CgState fin;
  rc = run_chunks(ctx, ex, nodes, ctx->st, ctx->h_st, &fin);
  if (rc) return rc;
  SBM_CUDA_TRY(cudaEventRecord(ctx->ev1, s));
  SBM_CUDA_TRY(cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  SBM_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  out->iters = fin.iter;
  out->outer = 1;
  out->final_res = fin.rms;
  out->ms = ms;
  out->status = status_of(fin.done);
  return SBM_OK;
}

}  // namespace

// =================================================================== MIXED
// FP32 CG with FP64 iterative refinement by reliable updates (residual
// replacement).  The FP32 iteration runs on an internal 16-byte-aligned
// layout (make_geo32); every time the FP32 recursive residual has dropped
// by delta^2 since the last replacement -- and whenever it claims
// convergence or the cap is reached -- the true residual
//     r = r0 - A (d + x32)
// is recomputed in double-float arithmetic (FP32 pairs, about 48
// significant bits; the initial residual r0 itself comes from the FP64
// stencil) from the double-float correction d and the FP32 partial
// correction x32, rounded to FP32 and substituted for the recursive
// residual; x32 is then folded into d.  The FP32 search direction is kept
// across replacements, so the Krylov space is not restarted (unlike
// restarted iterative refinement).  Convergence is decided only on the
// recomputed true residual: on return ||b - A x||_2 / ||b - A x0||_2 <= tol.

namespace {

__device__ __forceinline__ float4 ld4(const float* p) {
  return *reinterpret_cast<const float4*>(p);
}
__device__ __forceinline__ void st4(float* p, const float4& v) {
  *reinterpret_cast<float4*>(p) = v;
}

// p_new = z + beta p_old (z = invd*r with Jacobi, else r) at the centre
// and at the six neighbours (so p never needs a separate pass), then
// q = A p_new and p_new.q -> alpha.  p is double-buffered (p_old read at
// neighbours, p_new written at the centre).  Four y-consecutive voxels per
// thread (float4), threads flattened over (y-chunk, x-row) so short rows do
// not idle lanes; y-neighbours come from the adjacent lanes by shuffle, x-
// and z-neighbours by float4 loads, z kept in registers while marching.
template <int FORM, bool PC>
__global__ void __launch_bounds__(256, 4)
    k32v_apply_dir(OpArgs<float> op, int nchunk, int zc, const float* __restrict__ r,
                   const float* __restrict__ pold, const float* __restrict__ invd,
                   float* __restrict__ pnew, float* __restrict__ q, double* partials,
                   CgState* st) {
  pdl_begin();
  if (st->done) return;
  const Geo g = op.g;
  const float beta = (float)st->beta;
  const unsigned FULL = 0xffffffffu;
  const int64_t rows = (int64_t)nchunk * g.nx;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = t < rows;
  const int64_t tt = active ? t : rows - 1;
  const int lane = threadIdx.x & 31;
  const int chunk = (int)(tt % nchunk);
  const int j = (int)(tt / nchunk) + 1;
  const int k0 = blockIdx.y * zc + 1;
  const int k1 = min(k0 + zc - 1, g.nz);
  const bool lin = (lane > 0) && (chunk > 0);
  const bool rin = (lane < 31) && (chunk < nchunk - 1) && (t + 1 < rows);
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  auto P4 = [&](int64_t idx) -> float4 {
    const float4 rv = ld4(r + idx), pv = ld4(pold + idx);
    float4 z = rv;
    if (PC) {
      const float4 d = ld4(invd + idx);
      z = make_float4(d.x * rv.x, d.y * rv.y, d.z * rv.z, d.w * rv.w);
    }
    return make_float4(z.x + beta * pv.x, z.y + beta * pv.y, z.z + beta * pv.z,
                       z.w + beta * pv.w);
  };
  auto P1 = [&](int64_t idx) -> float {
    const float z = PC ? invd[idx] * r[idx] : r[idx];
    return z + beta * pold[idx];
  };
  int64_t c = g.ix(4 * chunk + 1, j, k0);
  float4 pc = P4(c), kc = ld4(op.hk + c);
  float4 pzm = (k0 == 1) ? pc : P4(c - g.sz);
  float4 kzm = ld4(op.hk + c - g.sz);
  float acc = 0.f;
  for (int k = k0; k <= k1; ++k) {
    const bool top = (k == g.nz);
    const float4 pzp = top ? pc : P4(c + g.sz);
    const float4 kzp = ld4(op.hk + c + g.sz);
    const float4 pxm = (j == 1) ? (op.bcx0 ? zero4 : pc) : P4(c - g.sx);
    const float4 pxp = (j == g.nx) ? (op.bcx1 ? zero4 : pc) : P4(c + g.sx);
    const float4 kxm = ld4(op.hk + c - g.sx), kxp = ld4(op.hk + c + g.sx);
    float pl = __shfl_up_sync(FULL, pc.w, 1), kl = __shfl_up_sync(FULL, kc.w, 1);
    float pr = __shfl_down_sync(FULL, pc.x, 1), kr = __shfl_down_sync(FULL, kc.x, 1);
    if (!lin) {
      kl = op.hk[c - 1];
      pl = (chunk == 0) ? pc.x : P1(c - 1);
    }
    if (!rin) {
      kr = op.hk[c + 4];
      pr = (chunk == nchunk - 1) ? pc.w : P1(c + 4);
    }
    const float pa[6] = {pl, pc.x, pc.y, pc.z, pc.w, pr};
    const float ka[6] = {kl, kc.x, kc.y, kc.z, kc.w, kr};
    const float pxa[4] = {pxm.x, pxm.y, pxm.z, pxm.w}, pxb[4] = {pxp.x, pxp.y, pxp.z, pxp.w};
    const float kxa[4] = {kxm.x, kxm.y, kxm.z, kxm.w}, kxb[4] = {kxp.x, kxp.y, kxp.z, kxp.w};
    const float pza[4] = {pzm.x, pzm.y, pzm.z, pzm.w}, pzb[4] = {pzp.x, pzp.y, pzp.z, pzp.w};
    const float kza[4] = {kzm.x, kzm.y, kzm.z, kzm.w}, kzb[4] = {kzp.x, kzp.y, kzp.z, kzp.w};
    float dg[4] = {0.f, 0.f, 0.f, 0.f};
    if (FORM == 1) {
      const float4 d4 = ld4(op.diag + c);
      dg[0] = d4.x; dg[1] = d4.y; dg[2] = d4.z; dg[3] = d4.w;
    }
    float qa[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float s = face_sum<float>(ka[e + 1], pa[e + 1], ka[e + 2], pa[e + 2], ka[e], pa[e],
                                      kxb[e], pxb[e], kxa[e], pxa[e], kzb[e], pzb[e], kza[e],
                                      pza[e]);
      qa[e] = (FORM == 0) ? op.scale * s : dg[e] * pa[e + 1] - op.scale * s;
    }
    if (active) {
      st4(pnew + c, pc);
      st4(q + c, make_float4(qa[0], qa[1], qa[2], qa[3]));
      acc += (pa[1] * qa[0] + pa[2] * qa[1]) + (pa[3] * qa[2] + pa[4] * qa[3]);
    }
    pzm = pc;
    kzm = kc;
    pc = pzp;
    kc = kzp;
    c += g.sz;
  }
  double v[1] = {(double)acc}, tot[1];
  if (grid_reduce<1>(v, partials, &st->counter[0], tot)) {
    if (threadIdx.x == 0) {
      const double pq = tot[0];
      st->pq = pq;
      st->alpha = st->rho / pq;
      if (pq == 0.0) st->done = 4;
      else if (!isfinite(pq)) st->done = 3;
    }
  }
}

// Scalar form of k32v_apply_dir for rows whose length is not a multiple of
// four (one voxel per thread, column z-march).
template <int FORM, bool PC>
__global__ void __launch_bounds__(BX* BY)
    k32s_apply_dir(OpArgs<float> op, int zc, const float* __restrict__ r,
                   const float* __restrict__ pold, const float* __restrict__ invd,
                   float* __restrict__ pnew, float* __restrict__ q, double* partials,
                   CgState* st) {
  if (st->done) return;
  const Geo g = op.g;
  const float beta = (float)st->beta;
  SBM_COLUMN_PROLOGUE(g, zc)
  auto P1 = [&](int64_t idx) -> float {
    const float z = PC ? invd[idx] * r[idx] : r[idx];
    return z + beta * pold[idx];
  };
  float acc = 0.f;
  if (active && k0 <= k1) {
    int64_t c = g.ix(i, j, k0);
    float pc = P1(c), kc = op.hk[c];
    float pzm = (k0 == 1) ? pc : P1(c - g.sz), kzm = op.hk[c - g.sz];
    for (int k = k0; k <= k1; ++k) {
      const float pzp = (k == g.nz) ? pc : P1(c + g.sz), kzp = op.hk[c + g.sz];
      const float pym = (i == 1) ? pc : P1(c - 1), pyp = (i == g.ny) ? pc : P1(c + 1);
      const float pxm = (j == 1) ? (op.bcx0 ? 0.f : pc) : P1(c - g.sx);
      const float pxp = (j == g.nx) ? (op.bcx1 ? 0.f : pc) : P1(c + g.sx);
      const float s = face_sum<float>(kc, pc, op.hk[c + 1], pyp, op.hk[c - 1], pym,
                                      op.hk[c + g.sx], pxp, op.hk[c - g.sx], pxm, kzp, pzp, kzm,
                                      pzm);
      const float qv = (FORM == 0) ? op.scale * s : op.diag[c] * pc - op.scale * s;
      pnew[c] = pc;
      q[c] = qv;
      acc += pc * qv;
      pzm = pc;
      kzm = kc;
      pc = pzp;
      kc = kzp;
      c += g.sz;
    }
  }
  double v[1] = {(double)acc}, tot[1];
  if (grid_reduce<1>(v, partials, &st->counter[0], tot)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      const double pq = tot[0];
      st->pq = pq;
      st->alpha = st->rho / pq;
      if (pq == 0.0) st->done = 4;
      else if (!isfinite(pq)) st->done = 3;
    }
  }
}

// Interior work item u -> index of its first voxel on layout g (VEC voxels
// along y per item).
template <int VEC>
__device__ __forceinline__ int64_t item_ix(const Geo& g, int nchunk, int64_t u, int* pi, int* pj,
                                           int* pk) {
  const int chunk = (int)(u % nchunk);
  const int64_t rr = u / nchunk;
  const int j = (int)(rr % g.nx) + 1;
  const int k = (int)(rr / g.nx) + 1;
  *pi = VEC * chunk + 1;
  *pj = j;
  *pk = k;
  return g.ix(*pi, j, k);
}

// x32 += alpha p; r32 -= alpha q; r.r and r.z (FP32 per thread, FP64 across
// threads); decides whether the next step is a reliable update.  After a
// reliable update the FP32 correction accumulated so far is first folded
// into the double-float one (d += x32, x32 = alpha p).
// FLEX (flexible CG with the learned preconditioner): rho and beta are left
// to the preconditioner kernel that follows.
template <bool PC, int VEC, bool FLEX = false>
__global__ void __launch_bounds__(256)
    k32_update(Geo g, int nchunk, float* __restrict__ x, const float* __restrict__ p,
               float* __restrict__ r, const float* __restrict__ q, const float* __restrict__ invd,
               float* __restrict__ dhi, float* __restrict__ dlo, double* partials, CgState* st) {
  if (st->done) return;
  const bool fold = st->accum_pending != 0;
  const float alpha = (float)st->alpha;
  const int64_t n = (int64_t)nchunk * g.nx * g.nz;
  float a_rr = 0.f, a_rz = 0.f;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n;
       u += (int64_t)gridDim.x * blockDim.x) {
    int i, j, k;
    const int64_t c = item_ix<VEC>(g, nchunk, u, &i, &j, &k);
    if (VEC == 4) {
      float4 xv = ld4(x + c);
      const float4 pv = ld4(p + c), qv = ld4(q + c);
      float4 rv = ld4(r + c);
      if (fold) {
        const float4 dh = ld4(dhi + c), dl = ld4(dlo + c);
        const DF d0 = df_add_f(DF{dh.x, dl.x}, xv.x), d1 = df_add_f(DF{dh.y, dl.y}, xv.y);
        const DF d2 = df_add_f(DF{dh.z, dl.z}, xv.z), d3 = df_add_f(DF{dh.w, dl.w}, xv.w);
        st4(dhi + c, make_float4(d0.hi, d1.hi, d2.hi, d3.hi));
        st4(dlo + c, make_float4(d0.lo, d1.lo, d2.lo, d3.lo));
        xv = make_float4(alpha * pv.x, alpha * pv.y, alpha * pv.z, alpha * pv.w);
      } else {
        xv.x += alpha * pv.x; xv.y += alpha * pv.y; xv.z += alpha * pv.z; xv.w += alpha * pv.w;
      }
      rv.x -= alpha * qv.x; rv.y -= alpha * qv.y; rv.z -= alpha * qv.z; rv.w -= alpha * qv.w;
      st4(x + c, xv);
      st4(r + c, rv);
      a_rr += (rv.x * rv.x + rv.y * rv.y) + (rv.z * rv.z + rv.w * rv.w);
      if (PC) {
        const float4 d = ld4(invd + c);
        a_rz += (rv.x * (d.x * rv.x) + rv.y * (d.y * rv.y)) +
                (rv.z * (d.z * rv.z) + rv.w * (d.w * rv.w));
      }
    } else {
      float xv = x[c];
      if (fold) {
        const DF d = df_add_f(DF{dhi[c], dlo[c]}, xv);
        dhi[c] = d.hi;
        dlo[c] = d.lo;
        xv = alpha * p[c];
      } else {
        xv += alpha * p[c];
      }
      x[c] = xv;
      const float rn = r[c] - alpha * q[c];
      r[c] = rn;
      a_rr += rn * rn;
      if (PC) a_rz += rn * (invd[c] * rn);
    }
  }
  double v[2] = {(double)a_rr, PC ? (double)a_rz : (double)a_rr}, tot[2];
  if (grid_reduce<2>(v, partials, &st->counter[1], tot)) {
    if (threadIdx.x == 0) {
      const double rr_new = tot[0], rho_new = tot[1];
      const int it = st->iter + 1;
      st->iter = it;
      st->accum_pending = 0;
      if (!isfinite(rho_new) || !isfinite(st->alpha)) {
        st->done = 3;
      } else {
        const double maxrr = fmax(st->maxrr, rr_new);
        const bool trig = (rr_new < st->delta2 * maxrr) ||
                          (rr_new <= st->tol * st->tol * st->aux[0]) || (it >= st->max_it);
        if (trig) {
          st->reliable = 1;
        } else if (!FLEX) {
          st->beta = rho_new / st->rho;
          st->rho = rho_new;
        }
        st->rr = rr_new;
        st->maxrr = maxrr;
      }
    }
  }
}

// Operands of the double-float residual replacement (FP32 layout, base +
// kOff32): hk = hkhi + hklo and, for the CnE form, diag = dghi + dglo split
// from the FP64 fields; r0 = r0hi + r0lo; the correction d = dhi + dlo
// plus x32.
struct DfResArgs {
  const float *hkhi, *hklo, *dghi, *dglo, *r0hi, *r0lo, *dhi, *dlo, *x32;
  float* r32;
  const float* invd32;
  float scale_hi, scale_lo;
  int bcx0, bcx1;
};

// Last-block bookkeeping of a residual replacement (tot = r.r, r.z): the
// stopping norm ||r|| / ||r0||, beta and rho (not FLEX, whose
// preconditioner kernel forms them), the replacement counters.
template <bool FLEX>
__device__ void df_rel_close(CgState* st, const double (&tot)[2]) {
  const double rms = (st->rr0 > 0.0) ? sqrt(tot[0] / st->rr0) : 0.0;
  st->rms = rms;
  st->n_reliable += 1;
  if (!isfinite(rms)) st->done = 3;
  else if (!(rms > st->tol)) st->done = 1;
  else if (st->iter >= st->max_it) st->done = 2;
  st->aux[1] = 0.0;  // the coarse residual of the learned preconditioner is stale
  if (!FLEX) {
    st->beta = tot[1] / st->rho;
    st->rho = tot[1];
  }
  st->rr = tot[0];
  st->maxrr = tot[0];
  st->reliable = 0;
  st->accum_pending = 1;
}

// Last-block state of a new solve after its initial residual (tot = r0.r0,
// r0.z0), which is also the solve's first residual replacement (the
// correction is still zero): rr0, the stopping norm (1, or 0 for a zero
// residual, or the non-finite value itself), rho and beta = 0 (not FLEX)
// and the replacement bookkeeping.
template <bool FLEX>
__device__ void df_init_close(CgState* st, const double (&tot)[2]) {
  const double rr = tot[0];
  const double rms = !isfinite(rr) ? rr : (rr > 0.0 ? 1.0 : 0.0);
  st->rr0 = rr;
  st->iter = 0;
  st->rms = rms;
  st->n_reliable = 1;
  st->done = 0;
  if (!isfinite(rr)) st->done = 3;
  else if (!(rms > st->tol)) st->done = 1;
  else if (st->max_it <= 0) st->done = 2;
  st->aux[0] = rr;
  st->aux[1] = 0.0;  // the learned preconditioner's coarse residual is stale
  st->rho = FLEX ? rr : tot[1];
  if (!FLEX) {
    st->beta = 0.0;
    st->initial = 0;
  }
  st->rr = rr;
  st->maxrr = rr;
  st->reliable = 0;
  st->accum_pending = 1;
}

// Reliable update in double-float arithmetic: r = r0 - A (d + x32) with
// every operand carried as an FP32 pair (about 48 significant bits, ample
// for residuals down to 1e-8 of r0 at 256^3), r32 = the high part, z =
// invd*r32 (Jacobi) and the norms as in k_rel_resid, whose FP64 stencil it
// replaces in the mixed solver: about 230 FP32 instructions per voxel
// instead of about 25 FP64 ones.  The correction V = d + x32 of each voxel
// is formed once and shared with the plane's other threads through a
// shared-memory tile (its column rolls along z); the half coefficients
// come from global memory (L1 / L2).  Tiles of BX x BY columns x zc planes
// are walked grid-stride by a few blocks per SM, as in k_rel_resid.
template <int FORM, bool PC, bool FLEX = false>
__global__ void __launch_bounds__(BX* BY)
    k_rel_resid_df(Geo g, int zc, DfResArgs a, double* partials, CgState* st) {
  pdl_begin();
  if (!st->reliable || st->done) return;
  const int nty = (g.ny + BX - 1) / BX, ntx = (g.nx + BY - 1) / BY;
  const int ntiles = nty * ntx * ((g.nz + zc - 1) / zc);
  double a_rr = 0.0, a_rz = 0.0;
  __shared__ float svh[BY + 2][BX + 2], svl[BY + 2][BX + 2];
  const DF scale{a.scale_hi, a.scale_lo};
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int ib = (t % nty) * BX, jb = ((t / nty) % ntx) * BY;
    const int i = ib + threadIdx.x + 1, j = jb + threadIdx.y + 1;
    const int k0 = (t / (nty * ntx)) * zc + 1;
    const int k1 = min(k0 + zc - 1, g.nz);
    const bool active = (i <= g.ny) && (j <= g.nx);
    float t_rr = 0.f, t_rz = 0.f;
    {
      const int tx = threadIdx.x, ty = threadIdx.y, tf = ty * BX + tx;
      int hrow = -1, hcol = -1;
      if (tf < 2 * BX) {  // rows 0 and BY + 1 (x halo)
        hcol = tf % BX + 1;
        hrow = tf < BX ? 0 : BY + 1;
      } else if (tf < 2 * BX + 2 * BY) {  // columns 0 and BX + 1 (y halo)
        const int u = tf - 2 * BX;
        hrow = u % BY + 1;
        hcol = u < BY ? 0 : BX + 1;
      }
      const int hi = ib + hcol, hj = jb + hrow;
      // only interior halo cells are read (the ghost rules replace the rest)
      const bool hact = hrow >= 0 && hi >= 1 && hi <= g.ny && hj >= 1 && hj <= g.nx;
      auto corr = [&](int ii, int jj, int kk) {
        const int64_t c = g.ix(ii, jj, kk);
        return df_add_f(DF{a.dhi[c], a.dlo[c]}, a.x32[c]);
      };
      auto hk = [&](int64_t c) { return DF{a.hkhi[c], a.hklo[c]}; };
      DF vc{0.f, 0.f}, vm{0.f, 0.f};
      if (active) {
        vc = corr(i, j, k0);
        vm = (k0 == 1) ? vc : corr(i, j, k0 - 1);
      }
      for (int k = k0; k <= k1; ++k) {
        DF vp{0.f, 0.f}, hv{0.f, 0.f};
        if (active) vp = (k == g.nz) ? vc : corr(i, j, k + 1);
        if (hact) hv = corr(hi, hj, k);
        __syncthreads();  // the previous plane's readers are done
        svh[ty + 1][tx + 1] = vc.hi;
        svl[ty + 1][tx + 1] = vc.lo;
        if (hrow >= 0) {
          svh[hrow][hcol] = hv.hi;
          svl[hrow][hcol] = hv.lo;
        }
        __syncthreads();
        if (active) {
          const int64_t c = g.ix(i, j, k);
          const DF zero{0.f, 0.f};
          const DF vym = (i == 1) ? vc : DF{svh[ty + 1][tx], svl[ty + 1][tx]};
          const DF vyp = (i == g.ny) ? vc : DF{svh[ty + 1][tx + 2], svl[ty + 1][tx + 2]};
          const DF vxm = (j == 1) ? (a.bcx0 ? zero : vc) : DF{svh[ty][tx + 1], svl[ty][tx + 1]};
          const DF vxp =
              (j == g.nx) ? (a.bcx1 ? zero : vc) : DF{svh[ty + 2][tx + 1], svl[ty + 2][tx + 1]};
          const DF kc = hk(c);
          // S(V) = sum_f (hk_nb + hk_c) (V_nb - V_c), faces y+, y-, x+, x-, z+, z-
          DF sum = df_mul(df_add(hk(c + 1), kc), df_sub(vyp, vc));
          sum = df_add(sum, df_mul(df_add(hk(c - 1), kc), df_sub(vym, vc)));
          sum = df_add(sum, df_mul(df_add(hk(c + g.sx), kc), df_sub(vxp, vc)));
          sum = df_add(sum, df_mul(df_add(hk(c - g.sx), kc), df_sub(vxm, vc)));
          sum = df_add(sum, df_mul(df_add(hk(c + g.sz), kc), df_sub(vp, vc)));
          sum = df_add(sum, df_mul(df_add(hk(c - g.sz), kc), df_sub(vm, vc)));
          DF av = df_mul(scale, sum);
          if (FORM == 1) av = df_sub(df_mul(DF{a.dghi[c], a.dglo[c]}, vc), av);
          const DF rv = df_sub(DF{a.r0hi[c], a.r0lo[c]}, av);
          const float rf = rv.hi;
          a.r32[c] = rf;
          t_rr += rf * rf;
          if (!FLEX) {  // the flexible solver takes rho from its preconditioner kernel
            const float zf = PC ? a.invd32[c] * rf : rf;
            t_rz += rf * zf;
          }
        }
        vm = vc;
        vc = vp;
      }
      __syncthreads();  // the next tile reuses the plane tile
    }
    a_rr += (double)t_rr;
    a_rz += (double)t_rz;
  }
  double v[2] = {a_rr, a_rz}, tot[2];
  if (grid_reduce<2>(v, partials, &st->counter[3], tot))
    if (threadIdx.x == 0 && threadIdx.y == 0) df_rel_close<FLEX>(st, tot);
}

// Initial residual of the mixed solve in double-float arithmetic:
// r0 = b - A x0 with x0's stored ghosts (Dirichlet / flux data: no ghost
// rules), from the hi + lo splits of x0 (xhi, xlo) and b (bhi, blo) in the
// FP32 layout; r0 is kept as the pair r0hi + r0lo for the replacements and
// its high part starts the FP32 residual (a.r32).  The last block sets
// rr0 = r0.r0 and the state of a new solve, including what the first
// residual replacement of k_rel_resid_df would set (the correction is still
// zero, so that replacement is this kernel's own result): the stopping
// norm, rho = r.z (PC: z = invd r; not FLEX, whose preconditioner kernel
// forms rho) and the replacement bookkeeping.  The operands of
// k_rel_resid_df, with hkhi / hklo / dghi / dglo / scale / r32 / invd32 of
// `a` used; same tiling.
template <int FORM, bool PC, bool FLEX>
__global__ void __launch_bounds__(BX* BY)
    k_residual_df(Geo g, int zc, DfResArgs a, const float* __restrict__ xhi,
                  const float* __restrict__ xlo, const float* __restrict__ bhi,
                  const float* __restrict__ blo, float* __restrict__ r0hi,
                  float* __restrict__ r0lo, double* partials, CgState* st) {
  const int nty = (g.ny + BX - 1) / BX, ntx = (g.nx + BY - 1) / BY;
  const int ntiles = nty * ntx * ((g.nz + zc - 1) / zc);
  double a_rr = 0.0, a_rz = 0.0;
  __shared__ float svh[BY + 2][BX + 2], svl[BY + 2][BX + 2];
  const DF scale{a.scale_hi, a.scale_lo};
  const int tx = threadIdx.x, ty = threadIdx.y, tf = ty * BX + tx;
  int hrow = -1, hcol = -1;
  if (tf < 2 * BX) {  // rows 0 and BY + 1 (x halo)
    hcol = tf % BX + 1;
    hrow = tf < BX ? 0 : BY + 1;
  } else if (tf < 2 * BX + 2 * BY) {  // columns 0 and BX + 1 (y halo)
    const int u = tf - 2 * BX;
    hrow = u % BY + 1;
    hcol = u < BY ? 0 : BX + 1;
  }
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int ib = (t % nty) * BX, jb = ((t / nty) % ntx) * BY;
    const int i = ib + tx + 1, j = jb + ty + 1;
    const int k0 = (t / (nty * ntx)) * zc + 1;
    const int k1 = min(k0 + zc - 1, g.nz);
    const bool active = (i <= g.ny) && (j <= g.nx);
    // a thread of a partial tile whose cell is in the ghost layer supplies
    // that ghost value to its neighbours through the plane tile
    const bool ghost = !active && (i <= g.ny + 1) && (j <= g.nx + 1);
    const int hi = ib + hcol, hj = jb + hrow;
    // halo cells up to and including the ghost layer: x0's ghosts are data
    const bool hact = hrow >= 0 && hi <= g.ny + 1 && hj <= g.nx + 1;
    auto xv = [&](int ii, int jj, int kk) {
      const int64_t c = g.ix(ii, jj, kk);
      return DF{xhi[c], xlo[c]};
    };
    auto hk = [&](int64_t c) { return DF{a.hkhi[c], a.hklo[c]}; };
    DF vc{0.f, 0.f}, vm{0.f, 0.f};
    if (active) {
      vc = xv(i, j, k0);
      vm = xv(i, j, k0 - 1);
    }
    float t_rr = 0.f, t_rz = 0.f;
    for (int k = k0; k <= k1; ++k) {
      DF vp{0.f, 0.f}, hv{0.f, 0.f};
      if (active) vp = xv(i, j, k + 1);
      else if (ghost) vc = xv(i, j, k);
      if (hact) hv = xv(hi, hj, k);
      __syncthreads();  // the previous plane's readers are done
      svh[ty + 1][tx + 1] = vc.hi;
      svl[ty + 1][tx + 1] = vc.lo;
      if (hrow >= 0) {
        svh[hrow][hcol] = hv.hi;
        svl[hrow][hcol] = hv.lo;
      }
      __syncthreads();
      if (active) {
        const int64_t c = g.ix(i, j, k);
        const DF vym{svh[ty + 1][tx], svl[ty + 1][tx]};
        const DF vyp{svh[ty + 1][tx + 2], svl[ty + 1][tx + 2]};
        const DF vxm{svh[ty][tx + 1], svl[ty][tx + 1]};
        const DF vxp{svh[ty + 2][tx + 1], svl[ty + 2][tx + 1]};
        const DF kc = hk(c);
        DF sum = df_mul(df_add(hk(c + 1), kc), df_sub(vyp, vc));
        sum = df_add(sum, df_mul(df_add(hk(c - 1), kc), df_sub(vym, vc)));
        sum = df_add(sum, df_mul(df_add(hk(c + g.sx), kc), df_sub(vxp, vc)));
        sum = df_add(sum, df_mul(df_add(hk(c - g.sx), kc), df_sub(vxm, vc)));
        sum = df_add(sum, df_mul(df_add(hk(c + g.sz), kc), df_sub(vp, vc)));
        sum = df_add(sum, df_mul(df_add(hk(c - g.sz), kc), df_sub(vm, vc)));
        DF av = df_mul(scale, sum);
        if (FORM == 1) av = df_sub(df_mul(DF{a.dghi[c], a.dglo[c]}, vc), av);
        const DF rv = df_sub(DF{bhi[c], blo[c]}, av);
        r0hi[c] = rv.hi;
        r0lo[c] = rv.lo;
        const float rf = rv.hi;
        a.r32[c] = rf;
        t_rr += rf * rf;
        if (!FLEX) {
          const float zf = PC ? a.invd32[c] * rf : rf;
          t_rz += rf * zf;
        }
      }
      vm = vc;
      vc = vp;
    }
    __syncthreads();  // the next tile reuses the plane tile
    a_rr += (double)t_rr;
    a_rz += (double)t_rz;
  }
  double v[2] = {a_rr, a_rz}, tot[2];
  if (grid_reduce<2>(v, partials, &st->counter[2], tot))
    if (threadIdx.x == 0 && threadIdx.y == 0) df_init_close<FLEX>(st, tot);
}

// The double-float residuals for grids whose y extent is a multiple of 4:
// INIT the initial residual of k_residual_df (from the splits of x0 and b,
// x0's ghosts read as data; also writes r0hi / r0lo and sets the state of
// the first replacement), else the replacement of k_rel_resid_df
// (V = d + x32 with the ghost rules of the correction).  Tiles of 64 (y) x
// 8 (x) cells x zc planes walked grid-stride by 128-thread blocks; each
// thread takes four y-consecutive cells (float4 loads of V, hk, the
// right-hand side) and runs the double-float arithmetic on pairs of FP32
// lanes: r (and r0) bit-identical to the one-cell kernels' (the same
// operations per cell), the norms summed in another order.  V of the
// plane's x / y neighbours comes from a shared-memory tile
// (12 lanes of every warp load its halo), V of the z neighbours rolls in
// registers, hk comes from global memory (L1 / L2).
constexpr int kDfTX = 64, kDfTY = 8, kDfThreads = kDfTX / 4 * kDfTY;
template <int FORM, bool PC, bool FLEX, bool INIT>
__global__ void __launch_bounds__(kDfThreads, 4)
    k_df_res4(Geo g, int zc, DfResArgs a, const float* __restrict__ xhi,
              const float* __restrict__ xlo, const float* __restrict__ bhi,
              const float* __restrict__ blo, float* __restrict__ r0hi, float* __restrict__ r0lo,
              double* partials, CgState* st) {
  if (!INIT) {
    pdl_begin();
    if (!st->reliable || st->done) return;
  }
  constexpr int Q = kDfTX / 4;  // float4 columns of the tile (16)
  constexpr int RF4 = Q + 2;    // with the y halo columns
  __shared__ float4 svh[kDfTY + 2][RF4], svl[kDfTY + 2][RF4];
  const int tid = threadIdx.x;
  const int q4 = tid % Q, row = tid / Q;
  const int nty = (g.ny + kDfTX - 1) / kDfTX, ntx = (g.nx + kDfTY - 1) / kDfTY;
  const int ntiles = nty * ntx * ((g.nz + zc - 1) / zc);
  // this thread's halo float4 (12 lanes of each warp): rows 0 / TY+1 at
  // columns 1..Q (the x neighbours of the tile's edge rows), columns 0 /
  // RF4-1 at rows 1..TY (the y neighbours of the row ends)
  constexpr int NH = 2 * Q + 2 * kDfTY;
  constexpr int HPW = NH / (kDfThreads / 32);
  const int hh = (tid & 31) < HPW ? (tid >> 5) * HPW + (tid & 31) : NH;
  int hrow = -1, hcol = -1;
  if (hh < 2 * Q) {
    hrow = hh < Q ? 0 : kDfTY + 1;
    hcol = hh % Q + 1;
  } else if (hh < NH) {
    const int u = hh - 2 * Q;
    hrow = u % kDfTY + 1;
    hcol = u < kDfTY ? 0 : RF4 - 1;
  }
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  auto lo2 = [](float4 v) { return make_float2(v.x, v.y); };
  auto hi2 = [](float4 v) { return make_float2(v.z, v.w); };
  // V (x0, or the correction d + x32) of the float4 starting at c
  auto vat = [&](int64_t c, float4& vh, float4& vl) {
    if (INIT) {
      vh = *reinterpret_cast<const float4*>(xhi + c);
      vl = *reinterpret_cast<const float4*>(xlo + c);
    } else {
      const float4 dh = *reinterpret_cast<const float4*>(a.dhi + c);
      const float4 dl = *reinterpret_cast<const float4*>(a.dlo + c);
      const float4 xx = *reinterpret_cast<const float4*>(a.x32 + c);
      const DF2 p0 = df2_add_f(DF2{lo2(dh), lo2(dl)}, lo2(xx));
      const DF2 p1 = df2_add_f(DF2{hi2(dh), hi2(dl)}, hi2(xx));
      vh = make_float4(p0.hi.x, p0.hi.y, p1.hi.x, p1.hi.y);
      vl = make_float4(p0.lo.x, p0.lo.y, p1.lo.x, p1.lo.y);
    }
  };
  auto hk2 = [&](int64_t c, float2* h0, float2* h1) {  // hk pairs (cells 0-1, 2-3) at c
    const float4 h = *reinterpret_cast<const float4*>(a.hkhi + c);
    const float4 l = *reinterpret_cast<const float4*>(a.hklo + c);
    h0[0] = lo2(h);
    h0[1] = lo2(l);
    h1[0] = hi2(h);
    h1[1] = hi2(l);
  };
  const DF2 scale2{make_float2(a.scale_hi, a.scale_hi), make_float2(a.scale_lo, a.scale_lo)};
  double a_rr = 0.0, a_rz = 0.0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int tyb = t % nty, txb = (t / nty) % ntx, tzb = t / (nty * ntx);
    const int i0 = kDfTX * tyb + 4 * q4 + 1, j = kDfTY * txb + row + 1;
    const int k0 = tzb * zc + 1, k1 = min(k0 + zc - 1, g.nz);
    // the own float4 lies in the padded layout (rows end at ny + 4), and
    // its cells are interior
    const bool inrow = i0 <= g.ny + 1 && j <= g.nx + 1;
    const bool active = i0 <= g.ny && j <= g.nx;
    const int hi_i = kDfTX * tyb + 4 * (hcol - 1) + 1, hj = kDfTY * txb + hrow;
    const bool hload = hrow >= 0 && hi_i <= g.ny + 1 && hj <= g.nx + 1;
    float4 vch = z4, vcl = z4, vmh = z4, vml = z4;
    if (inrow) {
      vat(g.ix(i0, j, k0), vch, vcl);
      vat(g.ix(i0, j, k0 - 1), vmh, vml);
    }
    float2 t_rr = make_float2(0.f, 0.f), t_rz = t_rr;
    for (int k = k0; k <= k1; ++k) {
      const int64_t c = g.ix(i0, j, k);
      float4 vph = z4, vpl = z4, hvh = z4, hvl = z4;
      if (inrow) vat(c + g.sz, vph, vpl);
      if (hload) vat(g.ix(hi_i, hj, k), hvh, hvl);
      __syncthreads();  // the previous plane's readers are done
      svh[row + 1][q4 + 1] = vch;
      svl[row + 1][q4 + 1] = vcl;
      if (hrow >= 0) {
        svh[hrow][hcol] = hvh;
        svl[hrow][hcol] = hvl;
      }
      __syncthreads();
      if (active) {
        // neighbours of V: y from the tile row, x from the rows beside, z in
        // registers; INIT reads x0's ghosts as data, otherwise the ghost
        // rules of the correction apply
        float ylh = svh[row + 1][q4].w, yll = svl[row + 1][q4].w;
        float yrh = svh[row + 1][q4 + 2].x, yrl = svl[row + 1][q4 + 2].x;
        float4 xmh = svh[row][q4 + 1], xml = svl[row][q4 + 1];
        float4 xph = svh[row + 2][q4 + 1], xpl = svl[row + 2][q4 + 1];
        float4 zmh = vmh, zml = vml, zph = vph, zpl = vpl;
        if (!INIT) {
          if (i0 == 1) {
            ylh = vch.x;
            yll = vcl.x;
          }
          if (i0 + 3 == g.ny) {
            yrh = vch.w;
            yrl = vcl.w;
          }
          if (j == 1) {
            xmh = a.bcx0 ? z4 : vch;
            xml = a.bcx0 ? z4 : vcl;
          }
          if (j == g.nx) {
            xph = a.bcx1 ? z4 : vch;
            xpl = a.bcx1 ? z4 : vcl;
          }
          if (k == 1) {
            zmh = vch;
            zml = vcl;
          }
          if (k == g.nz) {
            zph = vch;
            zpl = vcl;
          }
        }
        const DF2 vc0{lo2(vch), lo2(vcl)}, vc1{hi2(vch), hi2(vcl)};
        float2 kc0[2], kc1[2], n0[2], n1[2];
        hk2(c, kc0, kc1);
        const DF2 k0v{kc0[0], kc0[1]}, k1v{kc1[0], kc1[1]};
        // S(V) = sum_f (hk_nb + hk_c) (V_nb - V_c), faces y+, y-, x+, x-, z+, z-
        const float klh = a.hkhi[c - 1], kll = a.hklo[c - 1];
        const float krh = a.hkhi[c + 4], krl = a.hklo[c + 4];
        DF2 s0 = df2_mul(df2_add(DF2{make_float2(kc0[0].y, kc1[0].x), make_float2(kc0[1].y, kc1[1].x)}, k0v),
                         df2_sub(DF2{make_float2(vch.y, vch.z), make_float2(vcl.y, vcl.z)}, vc0));
        DF2 s1 = df2_mul(df2_add(DF2{make_float2(kc1[0].y, krh), make_float2(kc1[1].y, krl)}, k1v),
                         df2_sub(DF2{make_float2(vch.w, yrh), make_float2(vcl.w, yrl)}, vc1));
        s0 = df2_add(s0, df2_mul(df2_add(DF2{make_float2(klh, kc0[0].x), make_float2(kll, kc0[1].x)}, k0v),
                                 df2_sub(DF2{make_float2(ylh, vch.x), make_float2(yll, vcl.x)}, vc0)));
        s1 = df2_add(s1, df2_mul(df2_add(DF2{make_float2(kc0[0].y, kc1[0].x), make_float2(kc0[1].y, kc1[1].x)}, k1v),
                                 df2_sub(DF2{make_float2(vch.y, vch.z), make_float2(vcl.y, vcl.z)}, vc1)));
        auto face = [&](int64_t cn, float4 nh, float4 nl) {
          hk2(cn, n0, n1);
          s0 = df2_add(s0, df2_mul(df2_add(DF2{n0[0], n0[1]}, k0v),
                                   df2_sub(DF2{lo2(nh), lo2(nl)}, vc0)));
          s1 = df2_add(s1, df2_mul(df2_add(DF2{n1[0], n1[1]}, k1v),
                                   df2_sub(DF2{hi2(nh), hi2(nl)}, vc1)));
        };
        face(c + g.sx, xph, xpl);
        face(c - g.sx, xmh, xml);
        face(c + g.sz, zph, zpl);
        face(c - g.sz, zmh, zml);
        DF2 av0 = df2_mul(scale2, s0), av1 = df2_mul(scale2, s1);
        if (FORM == 1) {
          const float4 dh = *reinterpret_cast<const float4*>(a.dghi + c);
          const float4 dl = *reinterpret_cast<const float4*>(a.dglo + c);
          av0 = df2_sub(df2_mul(DF2{lo2(dh), lo2(dl)}, vc0), av0);
          av1 = df2_sub(df2_mul(DF2{hi2(dh), hi2(dl)}, vc1), av1);
        }
        const float* rh = INIT ? bhi : a.r0hi;
        const float* rl = INIT ? blo : a.r0lo;
        const float4 bh = *reinterpret_cast<const float4*>(rh + c);
        const float4 bl = *reinterpret_cast<const float4*>(rl + c);
        const DF2 rv0 = df2_sub(DF2{lo2(bh), lo2(bl)}, av0);
        const DF2 rv1 = df2_sub(DF2{hi2(bh), hi2(bl)}, av1);
        if (INIT) {
          *reinterpret_cast<float4*>(r0hi + c) = make_float4(rv0.hi.x, rv0.hi.y, rv1.hi.x, rv1.hi.y);
          *reinterpret_cast<float4*>(r0lo + c) = make_float4(rv0.lo.x, rv0.lo.y, rv1.lo.x, rv1.lo.y);
        }
        *reinterpret_cast<float4*>(a.r32 + c) = make_float4(rv0.hi.x, rv0.hi.y, rv1.hi.x, rv1.hi.y);
        t_rr = __ffma2_rn(rv1.hi, rv1.hi, __ffma2_rn(rv0.hi, rv0.hi, t_rr));
        if (!FLEX) {
          float2 z0 = rv0.hi, z1 = rv1.hi;
          if (PC) {
            const float4 iv = *reinterpret_cast<const float4*>(a.invd32 + c);
            z0 = __fmul2_rn(lo2(iv), z0);
            z1 = __fmul2_rn(hi2(iv), z1);
          }
          t_rz = __ffma2_rn(rv1.hi, z1, __ffma2_rn(rv0.hi, z0, t_rz));
        }
      }
      vmh = vch;
      vml = vcl;
      vch = vph;
      vcl = vpl;
    }
    a_rr += (double)t_rr.x + (double)t_rr.y;
    a_rz += (double)t_rz.x + (double)t_rz.y;
  }
  double v[2] = {a_rr, a_rz}, tot[2];
  if (grid_reduce<2>(v, partials, &st->counter[INIT ? 2 : 3], tot))
    if (threadIdx.x == 0) {
      if (INIT) df_init_close<FLEX>(st, tot);
      else df_rel_close<FLEX>(st, tot);
    }
}

// x += dhi + dlo + x32 on the interior (the total correction of the mixed
// solve; the FP32 parts summed in FP64).
__global__ void k_finish(Geo g, Geo g32, int zc, double* __restrict__ x,
                         const float* __restrict__ dhi, const float* __restrict__ dlo,
                         const float* __restrict__ x32) {
  SBM_COLUMN_PROLOGUE(g, zc)
  if (!active) return;
#pragma unroll 2
  for (int k = k0; k <= k1; ++k) {
    const int64_t c = g.ix(i, j, k), c3 = g32.ix(i, j, k);
    // d + x32 in double-float on the FP32 pipe, widened to FP64 with integer
    // instructions, then two FP64 additions
    const DF d = df_add_f(DF{dhi[c3], dlo[c3]}, x32[c3]);
    x[c] = (x[c] + f2d_int(d.hi)) + f2d_int(d.lo);
  }
}

// a32 = (float) a over the padded domain, FP64 layout -> FP32 layout, with
// the low part a - a32 in alo when given (and the same for b).
// A block of 64 x 2 threads takes two padded rows (j, k): each thread
// walks its row with stride 64, several independent loads in flight
// (launch with to32_grid / kTo32Block).
constexpr int kTo32Row = 64;
const dim3 kTo32Block(kTo32Row, 2);
__global__ void __launch_bounds__(2 * kTo32Row)
    k_to32(Geo g64, Geo g32, const double* __restrict__ a, float* __restrict__ a32,
           const double* __restrict__ b, float* __restrict__ b32, float* __restrict__ alo = nullptr,
           float* __restrict__ blo = nullptr) {
  const int j = 2 * blockIdx.x + threadIdx.y, k = blockIdx.y;
  if (j > g64.nx + 1) return;
  const int64_t c0 = g64.ix(0, j, k), c30 = g32.ix(0, j, k);
  const int n = g64.ny + 2;
#pragma unroll 4
  for (int i = threadIdx.x; i < n; i += kTo32Row) {
    const int64_t c = c0 + i, c3 = c30 + i;
    float h, l;
    df_split_int(a[c], &h, &l);
    a32[c3] = h;
    if (alo) alo[c3] = l;
    if (b) {
      df_split_int(b[c], &h, &l);
      b32[c3] = h;
      if (blo) blo[c3] = l;
    }
  }
}

// hi + lo splits of n FP64 values (sbm_split_f64), grid-stride.
__global__ void k_split_f64(int64_t n, const double* __restrict__ x, float* __restrict__ hi,
                            float* __restrict__ lo) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    float h, l;
    df_split_int(x[t], &h, &l);
    hi[t] = h;
    lo[t] = l;
  }
}

dim3 to32_grid(const Geo& g) {
  return dim3((unsigned)((g.nx + 2 + 1) / 2), (unsigned)(g.nz + 2));
}

int flat_blocks(int64_t items) {
  int64_t b = (items + 256 * 8 - 1) / (256 * 8);
  if (b < 1) b = 1;
  if (b > 152 * 16) b = 152 * 16;
  return (int)b;
}

}  // namespace

// sbm_tma.cu
struct TmaPlan;
bool tma_supported(const Geo& g32);
int tma_plan(const Geo& g32, const float* r, const float* pa, const float* pb, const float* hk,
             const float* iv, const float* dg, int pc, int form, int zct, int flex,
             TmaPlan* plan);
int tma_plan_size(void);
int tma_init();
void tma_launch(const TmaPlan& plan, bool fwd, const OpArgs<float>& op, float* pnew, float* q,
                double* partials, CgState* st, cudaStream_t s);
void tma_launch_fcg(const TmaPlan& plan, bool fwd, const OpArgs<float>& op, float* pnew, float* q,
                    const FcgDirArgs& fx, double* partials, CgState* st, cudaStream_t s);

int mixed_begin(sbm_ctx* ctx, const SolveSpec& sp, cudaGraphExec_t* ex_out, cudaGraph_t* graph_out,
                int* nodes_out) {
  if (sp.stop_rule != SBM_STOP_REL_RES) return SBM_ERR_ARG;
  if (ctx->g.nz + 2 > 65535) return SBM_ERR_ARG;  // to32_grid
  int rc = ensure_fp32_work(ctx);
  if (rc) return rc;
  const Geo& g = ctx->g;
  const Geo& g32 = ctx->g32;
  cudaStream_t s = ctx->stream;
  const Shape sh64 = stencil_shape(g, pick_zc(g, ctx->zc64));
  const int vec = (g.ny % 4 == 0) ? 4 : 1;
  const int nchunk = g.ny / vec;
  const int zc32 = ctx->zc32 > 0 ? ctx->zc32 : 8;
  const Shape sh32 = stencil_shape(g32, pick_zc(g32, ctx->zc32));
  float* const hk32 = ctx->hk32 + kOff32;
  float* const dg32 = ctx->dg32 + kOff32;
  float* const r32 = ctx->r32 + kOff32;
  float* const p32 = ctx->p32 + kOff32;
  float* const q32 = ctx->q32 + kOff32;
  float* const x32 = ctx->x32 + kOff32;
  float* const iv32 = ctx->z32 + kOff32;
  OpArgs<float> op32{g32, hk32, sp.form ? dg32 : nullptr, (float)sp.scale, sp.form, sp.bcx0,
                     sp.bcx1};
  // learned preconditioner when usable, else Jacobi (the documented fallback)
  // the flexible-CG loop runs on the TMA-staged direction kernel (it carries
  // the deferred x update and the restriction of q)
  const bool learned = sp.precond == SBM_PC_LEARNED && net_pc_usable(ctx, sp.form) && vec == 4 &&
                       tma_supported(g32);
  const bool pc = sp.precond == SBM_PC_JACOBI || (sp.precond == SBM_PC_LEARNED && !learned);
  ctx->last_precond = learned ? SBM_PC_LEARNED : (pc ? SBM_PC_JACOBI : SBM_PC_NONE);
  // Reliable-update factor: replace the residual once the FP32 residual
  // has fallen by 1e-2 (Jacobi / none; same iteration counts as 0.1 at
  // 256^3) or 1e-4 (flexible CG, which converges in far fewer iterations:
  // 256^3 headline solve 29.13 / 29.51 / 28.69 / 28.67 ms at 1e-3 / 3e-4 /
  // 1e-4 / 3e-5 with the FP64 replacement, 61-62 iterations each).
  const double delta = ctx->inner_tol > 0 ? ctx->inner_tol : (learned ? 1e-4 : 1e-2);
  CgState* h = &ctx->h_st[2];
  memset(h, 0, sizeof(CgState));
  h->tol = sp.tol;
  h->max_it = sp.max_it;
  h->stop_rule = SBM_STOP_REL_RES;
  h->delta2 = delta * delta;
  h->reliable = 1;
  h->initial = 1;
  SBM_CUDA_TRY(cudaEventRecord(ctx->ev0, s));
  SBM_CUDA_TRY(cudaMemcpyAsync(ctx->st, h, sizeof(CgState), cudaMemcpyHostToDevice, s));
  SBM_CUDA_TRY(cudaMemsetAsync(ctx->p32, 0, sizeof(float) * g32.nh, s));
  SBM_CUDA_TRY(cudaMemsetAsync(ctx->rold32, 0, sizeof(float) * g32.nh, s));
  // FP32 coefficients and, for the double-float replacement, their low parts
  k_to32<<<to32_grid(g), kTo32Block, 0, s>>>(g, g32, sp.hk64, hk32,
                                              sp.form ? sp.diag64 : nullptr, dg32,
                                              ctx->hklo32 + kOff32, ctx->dglo32 + kOff32);
  SBM_LAUNCHED(1);
  // the Jacobi weight: Jacobi-PCG and the learned preconditioner's additive
  // form read it (the multiplicative form forms it from hk itself)
  if (pc || (learned && ctx->pc_additive)) {
    k_invdiag<float><<<sh32.grid, sh32.block, 0, s>>>(op32, sh32.zc, iv32);
    SBM_LAUNCHED(1);
  }
  if (learned &&
      (rc = net_pc_begin(ctx, hk32, sp.form ? dg32 : nullptr, r32, q32, sp.scale, sp.bcx0,
                         sp.bcx1, s)))
    return rc;
  FcgDirArgs fx{};
  if (learned) {
    fx.x32 = x32;
    fx.dhi = ctx->dhi32 + kOff32;
    fx.dlo = ctx->dlo32 + kOff32;
    fx.rc = net_pc_rc(ctx);
    fx.rq = net_pc_rq(ctx);
    fx.scal = net_pc_scal(ctx);
    net_pc_rc_strides(ctx, &fx.rcy, &fx.rcx);
    fx.ncell = net_pc_ncell(ctx);
  }
  // with the learned preconditioner the direction kernels read z from its buffer
  float* const zl = learned ? net_pc_zbuf(ctx) : nullptr;
  const float* const rdir = learned ? zl : r32;
  // the double-float residual kernels walk their tiles grid-stride with four
  // blocks per SM (four fit at their 64 registers), so the usual no-op
  // launch of the replacement is cheap
  const int64_t rel_tiles = (int64_t)sh64.grid.x * sh64.grid.y * sh64.grid.z;
  const dim3 rgrid((unsigned)std::min<int64_t>(rel_tiles, 152 * 4));
  // the four-cell form when rows are whole float4s: tiles of 64 x 8 cells x
  // 16 planes, four 128-thread blocks per SM at most
  const bool df4 = vec == 4;
  constexpr int kDfZc = 16;
  const int64_t df_tiles = (int64_t)((g32.ny + kDfTX - 1) / kDfTX) *
                           ((g32.nx + kDfTY - 1) / kDfTY) * ((g32.nz + kDfZc - 1) / kDfZc);
  const dim3 dgrid((unsigned)std::min<int64_t>(df_tiles, 152 * 4));
  DfResArgs dfa{};
  dfa.hkhi = hk32;
  dfa.hklo = ctx->hklo32 + kOff32;
  dfa.dghi = dg32;
  dfa.dglo = ctx->dglo32 + kOff32;
  dfa.r0hi = ctx->r0hi32 + kOff32;
  dfa.r0lo = ctx->r0lo32 + kOff32;
  dfa.dhi = ctx->dhi32 + kOff32;
  dfa.dlo = ctx->dlo32 + kOff32;
  dfa.x32 = x32;
  dfa.r32 = r32;
  dfa.invd32 = iv32;
  df_split(sp.scale, &dfa.scale_hi, &dfa.scale_lo);
  dfa.bcx0 = sp.bcx0;
  dfa.bcx1 = sp.bcx1;
  // r0 = b - A x0 with x0's stored ghosts, in double-float from the hi + lo
  // splits of x0 (held meanwhile in q32 / x32) and b (in the correction's
  // arrays); x32 and the correction are cleared after it.  The initial
  // residual is also the first residual replacement: it writes r32 = r0's
  // high part (r32 is none of its inputs) and sets the stopping norm and rho.
  k_to32<<<to32_grid(g), kTo32Block, 0, s>>>(g, g32, sp.x, q32, sp.rhs, ctx->dhi32 + kOff32,
                                              x32, ctx->dlo32 + kOff32);
#define SBM_RES0(F, P, X)                                                                    \
  do {                                                                                       \
    if (df4)                                                                                 \
      k_df_res4<F, P, X, true><<<dgrid, kDfThreads, 0, s>>>(                                 \
          g32, kDfZc, dfa, q32, x32, ctx->dhi32 + kOff32, ctx->dlo32 + kOff32,               \
          ctx->r0hi32 + kOff32, ctx->r0lo32 + kOff32, ctx->partials, ctx->st);               \
    else                                                                                     \
      k_residual_df<F, P, X><<<rgrid, sh64.block, 0, s>>>(                                  \
          g32, sh64.zc, dfa, q32, x32, ctx->dhi32 + kOff32, ctx->dlo32 + kOff32,             \
          ctx->r0hi32 + kOff32, ctx->r0lo32 + kOff32, ctx->partials, ctx->st);               \
  } while (0)
  if (sp.form == 0) {
    if (learned) SBM_RES0(0, false, true);
    else if (pc) SBM_RES0(0, true, false);
    else SBM_RES0(0, false, false);
  } else {
    if (learned) SBM_RES0(1, false, true);
    else if (pc) SBM_RES0(1, true, false);
    else SBM_RES0(1, false, false);
  }
#undef SBM_RES0
  SBM_LAUNCHED(2);
  SBM_CUDA_TRY(cudaMemsetAsync(ctx->dhi32, 0, sizeof(float) * g32.nh, s));
  SBM_CUDA_TRY(cudaMemsetAsync(ctx->dlo32, 0, sizeof(float) * g32.nh, s));
  SBM_CUDA_TRY(cudaMemsetAsync(ctx->x32, 0, sizeof(float) * g32.nh, s));
  const int64_t items = (int64_t)nchunk * g.nx * g.nz;
  const dim3 fgrid(flat_blocks(items));
  const dim3 vgrid((unsigned)(((int64_t)nchunk * g.nx + 255) / 256), (g.nz + zc32 - 1) / zc32);
  float* const pbuf[2] = {p32, ctx->rold32 + kOff32};  // alternating direction buffers
  auto rel = [&](cudaStream_t s2) {
    const float* nf = nullptr;
    float* nw = nullptr;
#define SBM_REL(F, P)                                                                          \
  do {                                                                                         \
    if (df4)                                                                                   \
      k_df_res4<F, P, false, false><<<dgrid, kDfThreads, 0, s2>>>(                             \
          g32, kDfZc, dfa, nf, nf, nf, nf, nw, nw, ctx->partials, ctx->st);                    \
    else                                                                                       \
      k_rel_resid_df<F, P><<<rgrid, sh64.block, 0, s2>>>(g32, sh64.zc, dfa, ctx->partials,     \
                                                         ctx->st);                             \
  } while (0)
    if (learned) {
      launch_pdl(sp.form ? k_df_res4<1, false, true, false> : k_df_res4<0, false, true, false>,
                 dgrid, dim3(kDfThreads), 0, s2, g32, kDfZc, dfa, nf, nf, nf, nf, nw, nw,
                 ctx->partials, ctx->st);
    } else if (sp.form == 0) {
      if (pc) SBM_REL(0, true); else SBM_REL(0, false);
    } else {
      if (pc) SBM_REL(1, true); else SBM_REL(1, false);
    }
#undef SBM_REL
  };
  // TMA-staged stencil when the layout allows it (tensor maps of this solve)
  const bool use_tma = (vec == 4) && (learned || !ctx->no_tma) && tma_supported(g32);
  std::vector<unsigned char> plan_buf(use_tma ? tma_plan_size() : 1);
  TmaPlan* plan = reinterpret_cast<TmaPlan*>(plan_buf.data());
  if (use_tma) {
    if ((rc = tma_init())) return rc;
    if ((rc = tma_plan(g32, learned ? zl - kOff32 : ctx->r32, ctx->p32, ctx->rold32, ctx->hk32,
                       ctx->z32, ctx->dg32, pc ? 1 : 0, sp.form, ctx->zc32, learned ? 1 : 0,
                       plan)))
      return rc;
  }
  // one iteration reading direction buffer `in` and writing `out`
  auto iter = [&](cudaStream_t s2, const float* in, float* out) {
    if (learned) {
      // flexible CG: R r (when stale) and R r -= alpha R q, the U-Net, the
      // step that applies r -= alpha q and forms z, the direction kernel
      // (which applies x += alpha p_old), then the residual replacement
      net_pc_launch(ctx, r32, iv32, q32, ctx->partials, ctx->st, s2);
      tma_launch_fcg(*plan, in == pbuf[0], op32, out, q32, fx, ctx->partials, ctx->st, s2);
      rel(s2);
      return;
    }
#define SBM_AD(F, P)                                                                           \
  do {                                                                                         \
    if (use_tma)                                                                               \
      tma_launch(*plan, in == pbuf[0], op32, out, q32, ctx->partials, ctx->st, s2);            \
    else if (vec == 4)                                                                         \
      k32v_apply_dir<F, P><<<vgrid, 256, 0, s2>>>(op32, nchunk, zc32, rdir, in, iv32, out, q32, \
                                                   ctx->partials, ctx->st);                    \
    else                                                                                       \
      k32s_apply_dir<F, P><<<sh32.grid, sh32.block, 0, s2>>>(op32, sh32.zc, rdir, in, iv32,    \
                                                              out, q32, ctx->partials,         \
                                                              ctx->st);                        \
  } while (0)
    if (sp.form == 0) {
      if (pc) SBM_AD(0, true); else SBM_AD(0, false);
    } else {
      if (pc) SBM_AD(1, true); else SBM_AD(1, false);
    }
#undef SBM_AD
#define SBM_UP(P, V)                                                                         \
  k32_update<P, V><<<fgrid, 256, 0, s2>>>(g32, nchunk, x32, out, r32, q32, iv32,               \
                                          ctx->dhi32 + kOff32, ctx->dlo32 + kOff32,             \
                                          ctx->partials, ctx->st)
    if (vec == 4) {
      if (pc) SBM_UP(true, 4); else SBM_UP(false, 4);
    } else {
      if (pc) SBM_UP(true, 1); else SBM_UP(false, 1);
    }
#undef SBM_UP
    rel(s2);
  };
  // two iterations per captured unit so the direction buffers alternate
  auto body = [&](cudaStream_t s2) {
    iter(s2, pbuf[0], pbuf[1]);
    iter(s2, pbuf[1], pbuf[0]);
  };
  // (the first residual replacement -- r32 = r0, rho, beta = 0, with p32 = 0
  // so that the first p_new = z -- was made by k_residual_df)
  SBM_CUDA_TRY(cudaGetLastError());
  // bodies of 2 iterations per captured chunk: the flexible CG converges in
  // ~10x fewer iterations, so shorter chunks trim the no-op tail (256^3,
  // 61 iterations: 28.51 / 28.26 / 28.19 / 28.21 ms with 8 / 4 / 2 / 1
  // bodies per chunk)
  const int clen = ctx->chunk > 0 ? ctx->chunk : (learned ? 2 : chunk_len(ctx));
  const std::string key =
      key_of(learned ? (use_tma ? "mixfcg2-tma" : "mixfcg2") : (use_tma ? "mixrel2-tma" : "mixrel2"),
             hk32, dg32, x32, r32, pbuf[0], pbuf[1], learned ? (const void*)zl : iv32, sp.scale,
             sp.form, sp.bcx0, sp.bcx1, vec * 16 + zc32, pc, sh64.zc, clen);
  cudaGraphExec_t ex = nullptr;
  int nodes = 0;
  rc = capture_graph(ctx, key, learned ? 2 * (2 + net_pc_nodes()) : 6, body, &ex, &nodes, clen);
  if (rc) return rc;
  ctx->last_op32 = op32;
  ctx->last_pc = pc ? 1 : 0;
  *ex_out = ex;
  *nodes_out = nodes;
  *graph_out = ctx->graphs[key].graph;
  return SBM_OK;
}

int mixed_end(sbm_ctx* ctx, const SolveSpec& sp, const CgState& fin, SolveResult* out) {
  const Geo& g = ctx->g;
  const Geo& g32 = ctx->g32;
  cudaStream_t s = ctx->stream;
  const Shape sh64 = stencil_shape(g, pick_zc(g, ctx->zc64));
  float* const x32 = ctx->x32 + kOff32;
  // x += d + x32 (interior): the ghosts of x keep their Dirichlet / flux data.
  k_finish<<<sh64.grid, sh64.block, 0, s>>>(g, g32, sh64.zc, sp.x, ctx->dhi32 + kOff32,
                                            ctx->dlo32 + kOff32, x32);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  SBM_CUDA_TRY(cudaEventRecord(ctx->ev1, s));
  SBM_CUDA_TRY(cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  SBM_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  if (fin.pc_off && ctx->last_precond == SBM_PC_LEARNED) ctx->last_precond = SBM_PC_JACOBI;
  out->iters = fin.iter;
  out->outer = fin.n_reliable;
  out->final_res = fin.rms;
  out->ms = ms;
  out->status = status_of(fin.done);
  return SBM_OK;
}

// One application of the learned preconditioner to a host residual
// (halo-padded FP64, interior used) on the solve spec's operator; z gets
// the interior of M(r), ghosts zero.  For checking the preconditioner
// against an independent restatement.
int learned_pc_apply(sbm_ctx* ctx, const SolveSpec& sp, const double* r, double* z) {
  if (!net_pc_usable(ctx, sp.form) || ctx->g.ny % 4) return SBM_ERR_STATE;
  if (ctx->g.nz + 2 > 65535) return SBM_ERR_ARG;  // to32_grid
  int rc = ensure_fp32_work(ctx);
  if (rc) return rc;
  const Geo& g = ctx->g;
  const Geo& g32 = ctx->g32;
  cudaStream_t s = ctx->stream;
  float* const hk32 = ctx->hk32 + kOff32;
  float* const dg32 = ctx->dg32 + kOff32;
  float* const iv32 = ctx->z32 + kOff32;
  float* const r32 = ctx->r32 + kOff32;
  float* const q32 = ctx->q32 + kOff32;
  OpArgs<float> op32{g32, hk32, sp.form ? dg32 : nullptr, (float)sp.scale, sp.form, sp.bcx0,
                     sp.bcx1};
  const Shape sh32 = stencil_shape(g32, pick_zc(g32, ctx->zc32));
  k_to32<<<to32_grid(g), kTo32Block, 0, s>>>(g, g32, sp.hk64, hk32,
                                              sp.form ? sp.diag64 : nullptr, dg32);
  k_invdiag<float><<<sh32.grid, sh32.block, 0, s>>>(op32, sh32.zc, iv32);
  SBM_LAUNCHED(2);
  if ((rc = net_pc_begin(ctx, hk32, sp.form ? dg32 : nullptr, r32, q32, sp.scale, sp.bcx0,
                         sp.bcx1, s)))
    return rc;
  SBM_CUDA_TRY(cudaMemcpyAsync(ctx->r64, r, sizeof(double) * g.nh, cudaMemcpyHostToDevice, s));
  k_to32<<<to32_grid(g), kTo32Block, 0, s>>>(g, g32, ctx->r64, r32, nullptr, nullptr);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaMemsetAsync(ctx->q32, 0, sizeof(float) * g32.nh, s));
  CgState* h = &ctx->h_st[2];
  memset(h, 0, sizeof(CgState));
  h->initial = 1;
  SBM_CUDA_TRY(cudaMemcpyAsync(ctx->st32, h, sizeof(CgState), cudaMemcpyHostToDevice, s));
  net_pc_launch(ctx, r32, iv32, q32, ctx->partials, ctx->st32, s);
  SBM_CUDA_TRY(cudaGetLastError());
  std::vector<float> hz((size_t)g32.nh);
  SBM_CUDA_TRY(cudaMemcpyAsync(hz.data(), net_pc_zbuf(ctx) - kOff32, sizeof(float) * g32.nh,
                               cudaMemcpyDeviceToHost, s));
  SBM_CUDA_TRY(cudaMemcpyAsync(h, ctx->st32, sizeof(CgState), cudaMemcpyDeviceToHost, s));
  SBM_CUDA_TRY(cudaStreamSynchronize(s));
  if (h->done == 5) {
    set_error_msg("tensor-core convolution wait expired");
    return SBM_ERR_TIMEOUT;
  }
  memset(z, 0, sizeof(double) * g.nh);
  for (int k = 1; k <= g.nz; ++k)
    for (int j = 1; j <= g.nx; ++j)
      for (int i = 1; i <= g.ny; ++i) z[g.ix(i, j, k)] = hz[(size_t)(kOff32 + g32.ix(i, j, k))];
  return SBM_OK;
}

int solve_mixed(sbm_ctx* ctx, const SolveSpec& sp, SolveResult* out) {
  cudaGraphExec_t ex = nullptr;
  cudaGraph_t graph = nullptr;
  int nodes = 0;
  int rc = mixed_begin(ctx, sp, &ex, &graph, &nodes);
  if (rc) return rc;
  CgState fin;
  rc = ctx->host_loop ? run_chunks(ctx, ex, nodes, ctx->st, ctx->h_st, &fin)
                      : run_loop(ctx, graph, nodes, sp.max_it, ctx->st, ctx->h_st, &fin);
  if (rc) return rc;
  return mixed_end(ctx, sp, fin, out);
}


// Times `reps` back-to-back launches of one solver kernel on the context
// stream with CUDA events, on the buffers of the last mixed solve:
//   which 0: the FP32 fused direction + stencil kernel (its flexible-CG
//            variant after a learned solve)
//   which 1: the FP32 vector update kernel (Jacobi / no preconditioner)
//   which 2: the FP64 stencil + dot kernel of the plain CG
//   which 3: one application of the learned preconditioner (its r update
//            included); 5: its nine convolutions; 6: its multiplicative step
// and reports the algorithmic bytes one launch moves.
int bench_kernel(sbm_ctx* ctx, int which, int reps, float* ms_per_launch, double* bytes_per_launch) {
  if (reps < 1 || which < 0 || which > 6 || which == 4) return SBM_ERR_ARG;
  if (which != 2 && ctx->last_pc < 0) return SBM_ERR_STATE;
  if (which >= 3 && (ctx->last_precond != SBM_PC_LEARNED || !net_pc_usable(ctx, 0)))
    return SBM_ERR_STATE;
  const Geo& g = ctx->g;
  const Geo& g32 = ctx->g32;
  cudaStream_t s = ctx->stream;
  const double n = (double)g.ninterior();
  CgState* h = &ctx->h_st[3];
  memset(h, 0, sizeof(CgState));
  h->rho = 1.0;
  h->pq = 1.0;
  h->alpha = 1e-30;
  h->beta = 0.5;
  h->max_it = 1 << 30;
  h->tol = 0.0;
  h->delta2 = 0.0;
  h->aux[0] = 1.0;
  SBM_CUDA_TRY(cudaMemcpyAsync(ctx->st32, h, sizeof(CgState), cudaMemcpyHostToDevice, s));
  const OpArgs<float> op32 = ctx->last_op32;
  const bool pc = ctx->last_pc == 1;
  const int vec = (g.ny % 4 == 0) ? 4 : 1;
  const int nchunk = g.ny / vec;
  const int zc32 = ctx->zc32 > 0 ? ctx->zc32 : 8;
  const dim3 vgrid((unsigned)(((int64_t)nchunk * g.nx + 255) / 256), (g.nz + zc32 - 1) / zc32);
  const dim3 fgrid(flat_blocks((int64_t)nchunk * g.nx * g.nz));
  const Shape sh32 = stencil_shape(g32, pick_zc(g32, ctx->zc32));
  const Shape sh64 = stencil_shape(g, pick_zc(g, ctx->zc64));
  float* r32 = ctx->r32 + kOff32;
  float* pa = ctx->p32 + kOff32;
  float* pb = ctx->rold32 + kOff32;
  float* q32 = ctx->q32 + kOff32;
  float* x32 = ctx->x32 + kOff32;
  float* iv = ctx->z32 + kOff32;
  // the direction kernel of the last solve: the flexible-CG variant after a
  // learned solve (it also applies the deferred x update and restricts q)
  const bool flex = ctx->last_precond == SBM_PC_LEARNED && net_pc_usable(ctx, op32.form);
  const bool use_tma = (vec == 4) && (flex || !ctx->no_tma) && tma_supported(g32);
  std::vector<unsigned char> plan_buf(use_tma ? tma_plan_size() : 1);
  TmaPlan* plan = reinterpret_cast<TmaPlan*>(plan_buf.data());
  FcgDirArgs fx{};
  if (use_tma && which == 0) {
    int rc = tma_init();
    if (!rc) rc = tma_plan(g32, flex ? net_pc_zbuf(ctx) - kOff32 : ctx->r32, ctx->p32,
                           ctx->rold32, ctx->hk32, ctx->z32, ctx->dg32, pc ? 1 : 0, op32.form,
                           ctx->zc32, flex ? 1 : 0, plan);
    if (rc) return rc;
    if (flex) {
      fx.x32 = x32;
      fx.dhi = ctx->dhi32 + kOff32;
      fx.dlo = ctx->dlo32 + kOff32;
      fx.rc = net_pc_rc(ctx);
      fx.rq = net_pc_rq(ctx);
      fx.scal = net_pc_scal(ctx);
      net_pc_rc_strides(ctx, &fx.rcy, &fx.rcx);
      fx.ncell = net_pc_ncell(ctx);
    }
  }
  if (which == 2) {
    int rc = compute_faces(ctx, ctx->hk_gen, s);
    if (rc) return rc;
  }
  auto launch = [&]() {
    if (which == 0 && use_tma && flex) {
      tma_launch_fcg(*plan, true, op32, pb, q32, fx, ctx->partials, ctx->st32, s);
    } else if (which == 0 && use_tma) {
      tma_launch(*plan, true, op32, pb, q32, ctx->partials, ctx->st32, s);
    } else if (which == 0) {
      if (vec == 4) {
        if (op32.form == 0) {
          if (pc) k32v_apply_dir<0, true><<<vgrid, 256, 0, s>>>(op32, nchunk, zc32, r32, pa, iv, pb, q32, ctx->partials, ctx->st32);
          else k32v_apply_dir<0, false><<<vgrid, 256, 0, s>>>(op32, nchunk, zc32, r32, pa, iv, pb, q32, ctx->partials, ctx->st32);
        } else {
          if (pc) k32v_apply_dir<1, true><<<vgrid, 256, 0, s>>>(op32, nchunk, zc32, r32, pa, iv, pb, q32, ctx->partials, ctx->st32);
          else k32v_apply_dir<1, false><<<vgrid, 256, 0, s>>>(op32, nchunk, zc32, r32, pa, iv, pb, q32, ctx->partials, ctx->st32);
        }
      } else {
        if (op32.form == 0) k32s_apply_dir<0, false><<<sh32.grid, sh32.block, 0, s>>>(op32, sh32.zc, r32, pa, iv, pb, q32, ctx->partials, ctx->st32);
        else k32s_apply_dir<1, false><<<sh32.grid, sh32.block, 0, s>>>(op32, sh32.zc, r32, pa, iv, pb, q32, ctx->partials, ctx->st32);
      }
    } else if (which == 3) {
      net_pc_launch(ctx, r32, iv, q32, ctx->partials, ctx->st32, s);
    } else if (which == 5 || which == 6) {
      net_pc_launch_part(ctx, which - 5, r32, q32, ctx->partials, ctx->st32, s);
    } else if (which == 1) {
      if (vec == 4) {
        if (pc) k32_update<true, 4><<<fgrid, 256, 0, s>>>(g32, nchunk, x32, pb, r32, q32, iv, ctx->dhi32 + kOff32, ctx->dlo32 + kOff32, ctx->partials, ctx->st32);
        else k32_update<false, 4><<<fgrid, 256, 0, s>>>(g32, nchunk, x32, pb, r32, q32, iv, ctx->dhi32 + kOff32, ctx->dlo32 + kOff32, ctx->partials, ctx->st32);
      } else {
        k32_update<false, 1><<<fgrid, 256, 0, s>>>(g32, nchunk, x32, pb, r32, q32, iv, ctx->dhi32 + kOff32, ctx->dlo32 + kOff32, ctx->partials, ctx->st32);
      }
    } else {
      OpArgs<double> op{g, ctx->hk_gen, nullptr, 1.0, 0, SBM_BC_ZERO, SBM_BC_ZERO};
      op.fc = ctx->fc64;  // stored faces of the GENERIC operator (computed above)
      k_apply<double, 0, true, true><<<sh64.grid, sh64.block, 0, s>>>(op, sh64.zc, ctx->p64, ctx->q64, ctx->partials, ctx->st32);
    }
  };
  launch();  // warm
  SBM_CUDA_TRY(cudaEventRecord(ctx->ev0, s));
  for (int r = 0; r < reps; ++r) launch();
  SBM_CUDA_TRY(cudaEventRecord(ctx->ev1, s));
  SBM_CUDA_TRY(cudaEventSynchronize(ctx->ev1));
  SBM_CUDA_TRY(cudaGetLastError());
  SBM_LAUNCHED(reps + 1);
  float ms = 0.f;
  SBM_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  if (ms_per_launch) *ms_per_launch = ms / reps;
  double words;
  const double dgw = op32.form ? 1.0 : 0.0;
  if (which == 0 && flex) words = 7.0 + dgw;  // z,p_old,hk,x,[diag] -> p_new,q,x (+ R q)
  else if (which == 0) words = 5.0 + (pc ? 1.0 : 0.0) + dgw;  // r,p_old,hk,[invd],[diag] -> p_new,q
  else if (which == 1) words = 6.0 + (pc ? 1.0 : 0.0);        // x,p,r,q,[invd] -> x,r
  // one application: R r (only after a replacement) and the coarse grid not
  // counted; multiplicative r,q,hk,[diag] -> r,z; additive r,invd,q -> r,z
  else if (which == 3) words = ctx->pc_additive ? 5.0 : 5.0 + dgw;
  else if (which == 5) words = 0.0;  // convolutions: coarse grid only (flops, not fine bytes)
  else if (which == 6) words = 5.0 + dgw;  // r,q,hk,[diag] -> r,z
  else words = 3.0;                                                          // p,hk -> q (FP64)
  if (bytes_per_launch) *bytes_per_launch = words * (which == 2 ? 8.0 : 4.0) * n;
  return SBM_OK;
}

int solve(sbm_ctx* ctx, const SolveSpec& sp, SolveResult* out) {
  if (sp.precision == SBM_PREC_FP64) return solve_fp64(ctx, sp, out);
  if (sp.precision == SBM_PREC_MIXED) return solve_mixed(ctx, sp, out);
  return SBM_ERR_ARG;
}

void release_graphs(sbm_ctx* ctx) {
  for (auto& kv : ctx->loops) {
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    if (kv.second.graph) cudaGraphDestroy(kv.second.graph);
  }
  ctx->loops.clear();
  for (auto& kv : ctx->graphs) {
    cudaGraphExecDestroy(kv.second.exec);
    cudaGraphDestroy(kv.second.graph);
  }
  ctx->graphs.clear();
}

int status_of_done(int done) { return status_of(done); }

}  // namespace sbm

extern "C" int sbm_split_f64(int64_t n, const double* x, float* hi, float* lo, void* stream) {
  if (n < 0 || (n > 0 && (!x || !hi || !lo))) return SBM_ERR_ARG;
  if (n == 0) return SBM_OK;
  const int64_t b = std::min<int64_t>((n + 255) / 256, 152 * 16);
  sbm::k_split_f64<<<(unsigned)b, 256, 0, static_cast<cudaStream_t>(stream)>>>(n, x, hi, lo);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}
