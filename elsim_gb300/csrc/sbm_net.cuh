// sbm_net.cuh -- the learned coarse-grid preconditioner as seen by the
// solver (sbm_solver.cu): plan set-up outside graph capture, and the
// per-iteration launch sequence z = M(r) captured into the CG chunk graph.
#pragma once

#include "sbm_internal.cuh"

namespace sbm {

// True when the context has a network attached and the grid / operator
// suit it (every interior extent a multiple of 16; the FORM 0 operator, or
// FORM 1 with a network trained with the mass channel).
bool net_pc_usable(const sbm_ctx* ctx, int form);

// Per-solve set-up on the context stream (static features of the coarse
// grid from the FP32 half coefficient and, for FORM 1, the FP32 diagonal
// dg32 -- null for FORM 0; output scaling; the tensor maps the
// multiplicative step stages r, q and hk with).  hk32 / dg32 / r32 / q32 are
// the solver's FP32 fields (base + kOff32); later launches pass the same r32
// and q32.
int net_pc_begin(sbm_ctx* ctx, const float* hk32, const float* dg32, const float* r32,
                 const float* q32, double scale, int bcx0, int bcx1, cudaStream_t s);

// One application inside the flexible CG (no-op once st->done is set):
// R r when stale (first use, residual replacement), R r -= alpha R q and
// the network's input, the U-Net, then the kernel that applies the pending
// r -= alpha q of the previous direction (not on the first residual) and
// forms z = M(r) -- multiplicative: z1 + omega invd (r - A z1), z1 the
// prolonged network output; additive: invd r + z1.  Its last block sets
// st->rho = z.r and st->beta (Notay's FCG(1): beta = -z.q_old / pq_old; 0
// on the first use) and decides the reliable-update trigger from r.r.
// net_pc_zbuf returns the FP32 buffer (base + kOff32) receiving z.
float* net_pc_zbuf(sbm_ctx* ctx);
void net_pc_launch(sbm_ctx* ctx, float* r32, const float* iv32, const float* q32,
                   double* partials, CgState* st, cudaStream_t s);
// Coarse residual R r, the direction's R q (written by the flexible-CG
// direction kernel) and the scalars (s, 1/s, ...) the preconditioner reads.
float* net_pc_rc(sbm_ctx* ctx);
float* net_pc_rq(sbm_ctx* ctx);
// valid coarse cells (fine interior / 64)
int64_t net_pc_ncell(sbm_ctx* ctx);
// y and x strides of the coarse arrays (R r is stored with them)
void net_pc_rc_strides(sbm_ctx* ctx, int* sy, int* sx);
float* net_pc_scal(sbm_ctx* ctx);
// Kernel launches of one net_pc_launch.
int net_pc_nodes();
// One part of net_pc_launch for timing: 0 = the 9 U-Net convolutions on the
// current input, 1 = the multiplicative prolongation / Jacobi step.
void net_pc_launch_part(sbm_ctx* ctx, int part, float* r32, const float* q32,
                        double* partials, CgState* st, cudaStream_t s);

void net_pc_release(sbm_ctx* ctx);

}  // namespace sbm
