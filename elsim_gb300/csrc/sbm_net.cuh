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
// dg32 -- null for FORM 0; output scaling).  hk32 / dg32 are the solver's
// FP32 fields (base + kOff32).
int net_pc_begin(sbm_ctx* ctx, const float* hk32, const float* dg32, double scale, int bcx0,
                 int bcx1, cudaStream_t s);

// z = invd*r + P(e_c), e_c from the network on the restricted residual;
// the last block sets st->rho = z.r and st->beta (flexible CG, Notay's
// FCG(1): beta = -z.q_old / pq_old; 0 on the first use).  No-op once
// st->done is set.  Returns the FP32 buffer (base + kOff32) receiving z.
float* net_pc_zbuf(sbm_ctx* ctx);
void net_pc_launch(sbm_ctx* ctx, const float* r32, const float* iv32, const float* q32,
                   double* partials, CgState* st, cudaStream_t s);
// Coarse residual R r and the scalars (s, 1/s, ...) the preconditioner reads;
// the flexible-CG update kernel fills them (and marks them valid in
// CgState.aux[1]).
float* net_pc_rc(sbm_ctx* ctx);
// y and x strides of the coarse arrays (R r is stored with them)
void net_pc_rc_strides(sbm_ctx* ctx, int* sy, int* sx);
float* net_pc_scal(sbm_ctx* ctx);
// Kernel launches of one net_pc_launch.
int net_pc_nodes();
// One part of net_pc_launch for timing: 0 = the 9 U-Net convolutions on the
// current input, 1 = the multiplicative prolongation / Jacobi step.
void net_pc_launch_part(sbm_ctx* ctx, int part, const float* r32, const float* iv32,
                        const float* q32, double* partials, CgState* st, cudaStream_t s);

void net_pc_release(sbm_ctx* ctx);

}  // namespace sbm
