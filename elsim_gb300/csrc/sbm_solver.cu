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
//
// Two precisions:
//   FP64  the drop-in: the reference's CG and stopping rules.
//   MIXED FP32 inner CG (FP32 stencil, FP32 vectors, per-thread FP32 partial
//         sums promoted to FP64 for the grid reduction) inside an FP64
//         iterative-refinement loop whose residual r = r0 - A d is always
//         recomputed in FP64.
#include <cmath>
#include <cstring>

#include "sbm_internal.cuh"

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

// Face terms of S(p) = sum_f c_f (p_nb - p_c) in the reference's order
// (y+, y-, x+, x-, z+, z-; SBMES:494-499), c_f = hk_nb + hk_c.
template <typename T>
__device__ __forceinline__ T face_sum(T kc, T pc, T kyp, T pyp, T kym, T pym, T kxp, T pxp,
                                      T kxm, T pxm, T kzp, T pzp, T kzm, T pzm) {
  T s = (kyp + kc) * (pyp - pc);
  s = s - (kym + kc) * (pc - pym);
  s = s + (kxp + kc) * (pxp - pc);
  s = s - (kxm + kc) * (pc - pxm);
  s = s + (kzp + kc) * (pzp - pc);
  s = s - (kzm + kc) * (pc - pzm);
  return s;
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
                                        const T* __restrict__ p, int64_t c, int i, int j, T pc,
                                        T kc, T pzm, T pzp, T kzm, T kzp, int bcx0, int bcx1) {
  T pym = p[c - 1], pyp = p[c + 1], pxm = p[c - g.sx], pxp = p[c + g.sx];
  const T kym = hk[c - 1], kyp = hk[c + 1], kxm = hk[c - g.sx], kxp = hk[c + g.sx];
  if (RULE) {
    if (i == 1) pym = pc;
    if (i == g.ny) pyp = pc;
    if (j == 1) pxm = bcx0 ? T(0) : pc;
    if (j == g.nx) pxp = bcx1 ? T(0) : pc;
  }
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
    int64_t c = g.ix(i, j, k0);
    T pc = p[c], kc = op.hk[c];
    T pzm = p[c - g.sz], kzm = op.hk[c - g.sz];
    if (RULE && k0 == 1) pzm = pc;
    for (int k = k0; k <= k1; ++k) {
      const T pzp_raw = p[c + g.sz];
      const T kzp = op.hk[c + g.sz];
      const T pzp = (RULE && k == g.nz) ? pc : pzp_raw;
      const T s = stencil_at<T, RULE>(g, op.hk, p, c, i, j, pc, kc, pzm, pzp, kzm, kzp, op.bcx0,
                                      op.bcx1);
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
    int64_t c = g.ix(i, j, k0);
    double pc = x[c], kc = op.hk[c];
    double pzm = x[c - g.sz], kzm = op.hk[c - g.sz];
    for (int k = k0; k <= k1; ++k) {
      const double pzp = x[c + g.sz], kzp = op.hk[c + g.sz];
      const double s = stencil_at<double, false>(g, op.hk, x, c, i, j, pc, kc, pzm, pzp, kzm,
                                                 kzp, 0, 0);
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

// Iterative refinement step: r = r0 - A_h d64 in FP64 (ghost rules on d64),
// rr = r.r and the outer stopping test; then start the inner FP32 solve:
// r32 = (float)r, x32 = 0, p32 = z32 (Jacobi) or r32, inner rho/rr/rr0.
template <int FORM, bool PC>
__global__ void __launch_bounds__(BX* BY)
    k_ir_resid(OpArgs<double> op, int zc, const double* __restrict__ d64,
               const double* __restrict__ r0, float* __restrict__ r32, float* __restrict__ p32,
               float* __restrict__ x32, const float* __restrict__ invd32, double* partials,
               CgState* st, CgState* st32, int max_outer) {
  const Geo g = op.g;
  SBM_COLUMN_PROLOGUE(g, zc)
  double a_rr = 0.0, a_r32 = 0.0, a_rz32 = 0.0;
  if (active && k0 <= k1) {
    int64_t c = g.ix(i, j, k0);
    double pc = d64[c], kc = op.hk[c];
    double pzm = d64[c - g.sz], kzm = op.hk[c - g.sz];
    if (k0 == 1) pzm = pc;
    for (int k = k0; k <= k1; ++k) {
      const double pzp_raw = d64[c + g.sz], kzp = op.hk[c + g.sz];
      const double pzp = (k == g.nz) ? pc : pzp_raw;
      const double s = stencil_at<double, true>(g, op.hk, d64, c, i, j, pc, kc, pzm, pzp, kzm,
                                                kzp, op.bcx0, op.bcx1);
      const double ad = (FORM == 0) ? op.scale * s : op.diag[c] * pc - op.scale * s;
      const double rv = r0[c] - ad;
      a_rr += rv * rv;
      const float rf = (float)rv;
      r32[c] = rf;
      x32[c] = 0.0f;
      const float zf = PC ? invd32[c] * rf : rf;
      p32[c] = zf;
      a_r32 += (double)rf * (double)rf;
      a_rz32 += (double)rf * (double)zf;
      pzm = pc;
      kzm = kc;
      pc = pzp_raw;
      kc = kzp;
      c += g.sz;
    }
  }
  double v[3] = {a_rr, a_r32, a_rz32}, tot[3];
  if (grid_reduce<3>(v, partials, &st->counter[3], tot)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      st->rr = tot[0];
      const double rms = sqrt(tot[0]) / sqrt(st->rr0);
      st->rms = rms;
      if (!isfinite(rms)) st->done = 3;
      else if (!(rms > st->tol) || st->rr0 == 0.0) st->done = 1;
      else if (st->iter >= max_outer) st->done = 2;
      st->iter = st->iter + 1;
      st32->rr = tot[1];
      st32->rr0 = tot[1];
      st32->rho = tot[2];
      st32->iter = 0;
      st32->rms = 1.0;
      st32->done = (tot[1] == 0.0 || st->done) ? 1 : 0;
    }
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

// Captures (once) and returns a graph of `len` iterations.
template <typename T>
int get_graph(sbm_ctx* ctx, const std::string& key, const OpArgs<T>& op, const Shape& sh,
              int stop, bool pc, T* x, T* p, T* r, T* q, const double* w, const T* invd,
              CgState* st, cudaGraphExec_t* exec, int* nodes) {
  auto it = ctx->graphs.find(key);
  if (it != ctx->graphs.end()) {
    *exec = it->second.first;
    *nodes = it->second.second;
    return SBM_OK;
  }
  const int len = chunk_len(ctx);
  cudaGraph_t graph = nullptr;
  SBM_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  for (int c = 0; c < len; ++c)
    launch_iteration<T>(op, sh, stop, pc, x, p, r, q, w, invd, ctx->partials, st, ctx->stream);
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
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    set_error("cudaGraphInstantiate", e);
    return SBM_ERR_CUDA;
  }
  ctx->graphs[key] = {ex, 3 * len};
  *exec = ex;
  *nodes = 3 * len;
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

int solve_fp64(sbm_ctx* ctx, const SolveSpec& sp, SolveResult* out) {
  const Geo& g = ctx->g;
  cudaStream_t s = ctx->stream;
  const Shape sh = stencil_shape(g, pick_zc(g, ctx->zc64));
  OpArgs<double> op{g, sp.hk64, sp.diag64, sp.scale, sp.form, sp.bcx0, sp.bcx1};
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
  int rc = get_graph<double>(ctx, key, op, sh, sp.stop_rule, pc, sp.x, ctx->p64, ctx->r64,
                             ctx->q64, sp.w, invd, ctx->st, &ex, &nodes);
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

int solve_mixed(sbm_ctx* ctx, const SolveSpec& sp, SolveResult* out) {
  if (sp.stop_rule != SBM_STOP_REL_RES) return SBM_ERR_ARG;
  int rc = ensure_fp32_work(ctx);
  if (rc) return rc;
  const Geo& g = ctx->g;
  cudaStream_t s = ctx->stream;
  const Shape sh64 = stencil_shape(g, pick_zc(g, ctx->zc64));
  const Shape sh32 = stencil_shape(g, pick_zc(g, ctx->zc32));
  OpArgs<double> op64{g, sp.hk64, sp.diag64, sp.scale, sp.form, sp.bcx0, sp.bcx1};
  OpArgs<float> op32{g, ctx->hk32, sp.form ? ctx->dg32 : nullptr, (float)sp.scale, sp.form,
                     sp.bcx0, sp.bcx1};
  const bool pc = sp.precond == SBM_PC_JACOBI;
  const int max_outer = 40;
  const double inner_tol = ctx->inner_tol > 0 ? ctx->inner_tol : 2e-5;
  CgState* h = &ctx->h_st[2];
  memset(h, 0, sizeof(CgState));
  h->tol = sp.tol;
  h->max_it = max_outer;
  h->stop_rule = SBM_STOP_REL_RES;
  CgState* h32 = &ctx->h_st[3];
  memset(h32, 0, sizeof(CgState));
  h32->tol = inner_tol;
  h32->max_it = ctx->inner_max > 0 ? ctx->inner_max : sp.max_it;
  h32->stop_rule = SBM_STOP_REL_RES;
  SBM_CUDA_TRY(cudaEventRecord(ctx->ev0, s));
  SBM_CUDA_TRY(cudaMemcpyAsync(ctx->st, h, sizeof(CgState), cudaMemcpyHostToDevice, s));
  SBM_CUDA_TRY(cudaMemcpyAsync(ctx->st32, h32, sizeof(CgState), cudaMemcpyHostToDevice, s));
  // FP32 copies of the operator
  k_to_f32<<<flat_grid(g.nh), 256, 0, s>>>(g.nh, sp.hk64, ctx->hk32, sp.form ? sp.diag64 : nullptr,
                                           ctx->dg32);
  SBM_LAUNCHED(1);
  float* invd32 = ctx->z32;
  if (pc) {
    k_invdiag<float><<<sh32.grid, sh32.block, 0, s>>>(op32, sh32.zc, invd32);
    SBM_LAUNCHED(1);
  }
  // r0 = b - A x (FP64, stored ghosts); the outer state's rr0.
  if (sp.form == 0)
    k_residual_mem<0, false><<<sh64.grid, sh64.block, 0, s>>>(op64, sh64.zc, sp.rhs, sp.x, ctx->r0,
                                                              ctx->p64, nullptr, ctx->partials,
                                                              ctx->st);
  else
    k_residual_mem<1, false><<<sh64.grid, sh64.block, 0, s>>>(op64, sh64.zc, sp.rhs, sp.x, ctx->r0,
                                                              ctx->p64, nullptr, ctx->partials,
                                                              ctx->st);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaMemsetAsync(ctx->d64, 0, sizeof(double) * g.nh, s));
  SBM_CUDA_TRY(cudaGetLastError());
  const std::string key =
      key_of("mix32", ctx->hk32, ctx->dg32, ctx->x32, ctx->r32, ctx->p32, ctx->q32, invd32,
             sp.scale, sp.form, sp.bcx0, sp.bcx1, SBM_STOP_REL_RES, pc, sh32.zc, chunk_len(ctx));
  cudaGraphExec_t ex = nullptr;
  int nodes = 0;
  rc = get_graph<float>(ctx, key, op32, sh32, SBM_STOP_REL_RES, pc, ctx->x32, ctx->p32,
                        ctx->r32, ctx->q32, nullptr, invd32, ctx->st32, &ex, &nodes);
  if (rc) return rc;
  int inner_total = 0, outer = 0;
  CgState fin{}, fin32{};
  for (;;) {
    if (sp.form == 0) {
      if (pc)
        k_ir_resid<0, true><<<sh64.grid, sh64.block, 0, s>>>(op64, sh64.zc, ctx->d64, ctx->r0,
                                                            ctx->r32, ctx->p32, ctx->x32, invd32,
                                                            ctx->partials, ctx->st, ctx->st32,
                                                            max_outer);
      else
        k_ir_resid<0, false><<<sh64.grid, sh64.block, 0, s>>>(op64, sh64.zc, ctx->d64, ctx->r0,
                                                             ctx->r32, ctx->p32, ctx->x32, invd32,
                                                             ctx->partials, ctx->st, ctx->st32,
                                                             max_outer);
    } else {
      if (pc)
        k_ir_resid<1, true><<<sh64.grid, sh64.block, 0, s>>>(op64, sh64.zc, ctx->d64, ctx->r0,
                                                            ctx->r32, ctx->p32, ctx->x32, invd32,
                                                            ctx->partials, ctx->st, ctx->st32,
                                                            max_outer);
      else
        k_ir_resid<1, false><<<sh64.grid, sh64.block, 0, s>>>(op64, sh64.zc, ctx->d64, ctx->r0,
                                                             ctx->r32, ctx->p32, ctx->x32, invd32,
                                                             ctx->partials, ctx->st, ctx->st32,
                                                             max_outer);
    }
    SBM_LAUNCHED(1);
    SBM_CUDA_TRY(cudaMemcpyAsync(&ctx->h_st[0], ctx->st, sizeof(CgState), cudaMemcpyDeviceToHost, s));
    SBM_CUDA_TRY(cudaStreamSynchronize(s));
    fin = ctx->h_st[0];
    if (fin.done) break;
    ++outer;
    rc = run_chunks(ctx, ex, nodes, ctx->st32, ctx->h_st, &fin32);
    if (rc) return rc;
    inner_total += fin32.iter;
    k_accum<float><<<sh64.grid, sh64.block, 0, s>>>(g, sh64.zc, ctx->d64, ctx->x32);
    SBM_LAUNCHED(1);
  }
  // x += d (interior): the ghosts of x keep their Dirichlet / flux data.
  k_accum<double><<<sh64.grid, sh64.block, 0, s>>>(g, sh64.zc, sp.x, ctx->d64);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  SBM_CUDA_TRY(cudaEventRecord(ctx->ev1, s));
  SBM_CUDA_TRY(cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  SBM_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  out->iters = inner_total;
  out->outer = outer;
  out->final_res = fin.rms;
  out->ms = ms;
  out->status = status_of(fin.done);
  return SBM_OK;
}

}  // namespace

int solve(sbm_ctx* ctx, const SolveSpec& sp, SolveResult* out) {
  if (sp.precision == SBM_PREC_FP64) return solve_fp64(ctx, sp, out);
  if (sp.precision == SBM_PREC_MIXED) return solve_mixed(ctx, sp, out);
  return SBM_ERR_ARG;
}

void release_graphs(sbm_ctx* ctx) {
  for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second.first);
  ctx->graphs.clear();
}

}  // namespace sbm
