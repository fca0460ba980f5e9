/*
 * sbm_capi.h -- C-ABI of the GB300 smoothed-boundary-method (SBM) hot path.
 *
 * Every entry point is `extern "C"`, takes plain pointers, sizes and a plain
 * parameter struct, and returns an `int` status (SBM_OK == 0, negative on
 * error).  Nothing here aborts the process.  The types are bind(C)
 * compatible, so a Fortran host can declare them in an ISO_C_BINDING
 * interface block (INTEGER(C_INT), REAL(C_DOUBLE), TYPE(C_PTR)).
 *
 * Array layout is the reference's: Fortran column-major (y, x, z), y fastest.
 * A halo-padded field A(0:ny+1, 0:nx+1, 0:nz+1) has element (i, j, k) at
 *     i + (ny+2) * (j + (nx+2) * k)
 * and an interior-only field B(1:ny, 1:nx, 1:nz) has element (i, j, k) at
 *     (i-1) + ny * ((j-1) + nx * (k-1)).
 * The x axis (2nd index) carries the Dirichlet / flux faces, exactly as in
 * SBMES_3D_MPI_CH_Gr_CONJG_VD_T05_01_BQ_hx3.f90 (called SBMES below).
 *
 * The reference has no FFI of its own: its solver loops are inline in the
 * main program.  Each declaration below names the reference lines it
 * replaces.
 */
#ifndef SBM_CAPI_H
#define SBM_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define SBM_OK                 0
#define SBM_ERR_ARG           -1   /* bad dimension, null pointer, unknown id */
#define SBM_ERR_CUDA          -2   /* a CUDA runtime call failed               */
#define SBM_ERR_MAXIT         -3   /* iteration cap hit before tolerance       */
#define SBM_ERR_NONFINITE     -4   /* NaN/Inf in a reduction                   */
#define SBM_ERR_BREAKDOWN     -5   /* p.Ap == 0 in CG                          */
#define SBM_ERR_NOMEM         -6   /* device allocation failed                 */
#define SBM_ERR_STATE         -7   /* call made in a state that forbids it     */
#define SBM_ERR_TIMEOUT       -8   /* a bounded device-side wait expired       */

/* ---------------------------------------------------------- enumerations */
/* Ghost rule applied to the CG search direction at an x face
 * (SBMES:512-513, :667-668, :748-749).  y and z faces are always Neumann
 * (edge copy), as BcMpiYZ does at the physical boundary (SBMES:1043-1088). */
#define SBM_BC_COPY   0   /* PRJ(ghost) = PRJ(edge)   (Neumann)  */
#define SBM_BC_ZERO   1   /* PRJ(ghost) = 0           (Dirichlet) */

/* Operator families (SBMES:515-521 CnE, :670-676 phP, :751-757 phE).
 * GENERIC is the phP form on the context's COEF field with the x-face ghost
 * rules taken from the solve call (used for the plain potential solve);
 * GENERIC_DIAG the CnE form on the context's fields, q = DIAG p - scale
 * S(p) with faces from COEF (a concentration solve with its mass term). */
#define SBM_OP_CNE      0
#define SBM_OP_PHP      1
#define SBM_OP_PHE      2
#define SBM_OP_GENERIC  3
#define SBM_OP_GENERIC_DIAG 4

/* Stopping rules.  REF_UPDATE: sqrt(sum(w*dx^2)/sum(w)) < tol, the
 * potential loops (SBMES:699-705, :780-786).  REF_RESID:
 * sqrt(sum(w*r^2)/sum(w)) < tol, the CnE loop (SBMES:545-547).
 * REL_RES: ||r||_2 / ||r_0||_2 <= tol. */
#define SBM_STOP_REF_UPDATE  0
#define SBM_STOP_REF_RESID   1
#define SBM_STOP_REL_RES     2

/* Solver variants (no counterpart in the reference). */
#define SBM_PREC_FP64   0   /* plain FP64 CG: the drop-in                    */
#define SBM_PREC_MIXED  1   /* FP32 inner CG, double-float residual replacement */

#define SBM_PC_NONE     0
#define SBM_PC_JACOBI   1
#define SBM_PC_LEARNED  2

/* Butler-Volmer forms (SBMES:636-637). */
#define SBM_BV_EXP      0   /* reference exponential form        */
#define SBM_BV_LINEAR   1   /* first-order expansion in dPh      */

/* Cahn-Hilliard chemical potential (sbm_params.ch_mode) */
#define SBM_CH_TABLE        0   /* reference: mu = Tbl(c) - eps Lap c, SBMES:403-411 */
#define SBM_CH_DOUBLE_WELL  1   /* mu = ch_w 2c(1-c)(1-2c) - eps Lap c (the analytic
                                   double well of the 128^3 full-step workload);
                                   mobility still from tbl_mb (all ones: M = 1) */

/* Device-resident fields of a context.  All are halo-padded FP64. */
enum sbm_field {
  SBM_F_PSP = 0,   /* psP  particle domain parameter      SBMES:143 */
  SBM_F_PSE,       /* psE  electrolyte domain parameter   SBMES:144 */
  SBM_F_AVP,       /* AvP  interface measure              SBMES:273-289 */
  SBM_F_AVPX,      /* AvPx = AvP/dx                        SBMES:291 */
  SBM_F_CNP,       /* CnP  particle Li fraction           SBMES:295 */
  SBM_F_CNE,       /* CnE  salt concentration             SBMES:306 */
  SBM_F_PHP,       /* phP  particle potential             SBMES:316 */
  SBM_F_PHE,       /* phE  electrolyte potential          SBMES:336 */
  SBM_F_RXN,       /* Rxn  reaction rate                  SBMES:310 */
  SBM_F_COEF,      /* node coefficient of the GENERIC operator */
  SBM_F_RHS,       /* right-hand side of a GENERIC solve       */
  SBM_F_X,         /* unknown of a GENERIC solve (ghosts = Dirichlet data) */
  SBM_F_WEIGHT,    /* psi weight of the GENERIC stopping norm  */
  SBM_F_DIAG,      /* diagonal (mass) term of GENERIC_DIAG     */
  SBM_F_COUNT
};

#define SBM_TBL_MAX 128

/* Physical and numerical parameters of the electrochemical step.  Field
 * names follow the reference's variables; defaults (sbm_params_reference)
 * carry the reference's Fortran literals with their kinds preserved. */
typedef struct sbm_params {
  double dx;              /* SBMES:90 */
  double rho;             /* SBMES:100 (REAL(4) literal)     */
  double eps;             /* SBMES:136                        */
  double ch_mask;         /* 1e-5 update mask, SBMES:430      */
  double d0, tc1, tc2, t_minus;   /* SBMES:118-126 */
  double dab_c0, dab_c1, dab_c2, dab_c3; /* Dab = D0*EXP(c0 - c1*c + c2*(c3*c)**2), SBMES:474 */
  double cne_ref;         /* mean CnE target 1e-3, SBMES:567  */
  double cst1, frd;       /* SBMES:101-102                    */
  double bvp, bve;        /* SBMES:106-107                    */
  double kap_scale;       /* 3.3, SBMES:324                   */
  double avp_mask;        /* 1e-2, SBMES:287, :631            */
  double i0_scale;        /* 1e-3, SBMES:617                  */
  double kfw_c;           /* 0.001 in Kfw, SBMES:621          */
  double crt_cne, crt_php, crt_phe, crt_picard; /* SBMES:96-98, :627 */
  int    max_it_cne, max_it_php, max_it_phe, max_picard;
  int    cne_mean_every;  /* 100, SBMES:562 */
  int    bv_mode;         /* SBM_BV_EXP or SBM_BV_LINEAR */
  int    tbl_n;           /* table length (101), SBMES:210-242 */
  int    ch_mode;         /* SBM_CH_TABLE or SBM_CH_DOUBLE_WELL */
  double tbl_x[SBM_TBL_MAX];    /* Tbl(1,:)  coordinates   */
  double tbl_mu[SBM_TBL_MAX];   /* Tbl(2,:)  chemical potential, C_Li_M6 */
  double tbl_mb[SBM_TBL_MAX];   /* DTbl(2,:) mobility, C_Li_Mb5 (already scaled) */
  double tbl_i0[SBM_TBL_MAX];   /* iTbl(2,:) exchange current, C_Li_J2 */
  double tbl_ocv[SBM_TBL_MAX];  /* OTbl(2,:) open-circuit voltage, C_Li_O3 */
  double ch_w;                  /* double-well height W (SBM_CH_DOUBLE_WELL) */
} sbm_params;

/* Scalars of the electrochemical state that the reference keeps in
 * program variables (SBMES:248-262, :303, :341, :351, :443, :828). */
typedef struct sbm_scalars {
  double tPP, tPE;        /* sums of psP, psE */
  double xrf;             /* mean particle Li fraction */
  double infx;            /* Li influx */
  double scrnt, trgI;     /* current and target current */
  double bve;             /* electrolyte boundary potential (moves) */
  double cvgp, cvgl;      /* Picard convergence norms of the last step */
  int    it_cne, it_php, it_phe, n_picard; /* CG iterations of the last step */
} sbm_scalars;

typedef struct sbm_ctx sbm_ctx;

/* Fills *p with the reference's constants (SBMES:90-136) and flat tables. */
int sbm_params_reference(sbm_params* p);

/* Context: one device-resident domain (replaces the MPI decomposition
 * MyDmnCmpn_YZ, SBMES:947-982, and the halo exchange BcMpiYZ,
 * SBMES:1031-1090).  Owns device buffers and one CUDA stream. */
int sbm_ctx_create(int ny, int nx, int nz, const sbm_params* p, sbm_ctx** out);
int sbm_ctx_destroy(sbm_ctx* ctx);
int sbm_ctx_set_params(sbm_ctx* ctx, const sbm_params* p);
/* Launch-shape and mixed-precision knobs (0 = built-in choice): z planes
 * per thread of the FP64 / FP32 stencil kernels, CG iterations per captured
 * graph chunk, and `delta` of the mixed solver (its true residual is
 * recomputed in double-float arithmetic whenever the FP32 residual norm has
 * fallen by this factor; default 1e-2, 1e-4 with the learned
 * preconditioner).  flags bit 0
 * (SBM_TUNE_NO_TMA): use the register-tiled FP32 stencil instead of the
 * TMA-staged one; bit 1 (SBM_TUNE_PC_ADDITIVE): apply the learned
 * preconditioner in its additive form z = D^-1 r + P e_c instead of the
 * default multiplicative one z = z1 + 2.3 D^-1 (r - A z1), z1 = P e_c;
 * bit 2 (SBM_TUNE_HOST_LOOP): drive the mixed solver's captured iteration
 * chunks from the host (one chunk in flight while the host reads the
 * previous one's state) instead of looping them on the device in a
 * conditional graph node -- the same kernels, for profilers that cannot
 * see kernels inside conditional graphs.
 * No counterpart in the reference. */
#define SBM_TUNE_NO_TMA 1
#define SBM_TUNE_PC_ADDITIVE 2
#define SBM_TUNE_HOST_LOOP 4
int sbm_ctx_set_tuning(sbm_ctx* ctx, int zc64, int zc32, int chunk, double delta, int flags);
/* The context's CUDA stream as an opaque handle (cudaStream_t), and a wait
 * for everything enqueued on it (no counterpart in the reference: its work
 * is synchronous). */
int sbm_ctx_stream(sbm_ctx* ctx, void** stream);
int sbm_ctx_sync(sbm_ctx* ctx);
/* The context's parameters (the reference's parameter block, SBMES:90-136)
 * and electrochemical scalars (tPP, tPE, Xrf, the current and the boundary
 * potential of the reference's time loop, SBMES:357-877), host copies. */
int sbm_ctx_get_params(const sbm_ctx* ctx, sbm_params* p);
int sbm_ctx_get_scalars(const sbm_ctx* ctx, sbm_scalars* s);

/* Checkpoint / resume (no counterpart in the reference, whose periodic
 * REAL(4) dumps are outputs only).  A snapshot holds the parameters, the
 * electrochemical scalars and every halo-padded FP64 field a later solve or
 * time step reads: the 14 public fields and, after sbm_setup_domain, the 12
 * step buffers (operator half coefficients, Dab, mu, mobility, reaction
 * coefficients, rate constants, previous phP / phE).  A context restored
 * from it continues bit for bit like the one it was taken from.  The buffer
 * is host memory of sbm_ctx_snapshot_size bytes (pinned memory copies
 * fastest); restore requires the same grid and rejects any other buffer
 * with SBM_ERR_ARG.  The run's own counters (iteration, time, frame) are the
 * caller's to keep beside it. */
int sbm_ctx_snapshot_size(sbm_ctx* ctx, size_t* bytes);
int sbm_ctx_snapshot(sbm_ctx* ctx, void* buf, size_t bytes);
int sbm_ctx_restore(sbm_ctx* ctx, const void* buf, size_t bytes);

/* Host <-> device copies of a field.  `haloed` = 1: h has the halo-padded
 * shape (ny+2)(nx+2)(nz+2); 0: interior shape ny*nx*nz (ghosts untouched). */
int sbm_upload(sbm_ctx* ctx, int field, const double* h, int haloed);
int sbm_download(sbm_ctx* ctx, int field, double* h, int haloed);
/* Raw device pointer of a field (halo-padded FP64), for device-resident use. */
int sbm_field_ptr(sbm_ctx* ctx, int field, double** dptr);

/* Domain set-up, SBMES:154-168 + :173-176 + :247-262 + :273-291 +
 * :297-341: psi from two REAL(4) distance fields (interior shape), clamp,
 * edge ghosts, the 1e-7 / 1e-6 floors, AvP/AvPx, tPP/tPE, initial
 * concentrations and potentials, Kap, Xrf and the target current
 * (rate `cr`, SBMES:109, :341).  zeta: SBMES:94. */
int sbm_setup_domain(sbm_ctx* ctx, const float* dist_p, const float* dist_e,
                     double zeta, double cnp0, double cne0, double cr,
                     sbm_scalars* s);

/* CG solve on device-resident fields (SBMES:492-555, :647-714, :729-795).
 * op: SBM_OP_*.  For CNE/PHP/PHE the right-hand side is the context's
 * internal RHS buffer filled by the step routines; GENERIC uses
 * SBM_F_RHS, SBM_F_X, SBM_F_COEF and SBM_F_WEIGHT with x-face ghost rules
 * bc_x0 / bc_x1 and operator scale `scale` (q = scale * div(K grad p)).
 * precision: SBM_PREC_*; precond: SBM_PC_*.  `iters` receives the number
 * of CG iterations executed (inner iterations for MIXED); `final_res`
 * the last value of the stopping norm; `ms` the device time. */
int sbm_cg_solve(sbm_ctx* ctx, int op, int bc_x0, int bc_x1, double scale,
                 double tol, int max_it, int stop_rule, int precision,
                 int precond, int* iters, double* final_res, float* ms);

/* Benchmark hook (no counterpart in the reference): times `reps` launches
 * of one solver kernel on the context stream with CUDA events, replaying the
 * arguments of the last mixed-precision solve.  which 0: FP32 fused
 * direction + stencil kernel (after a learned-preconditioner solve its
 * flexible-CG variant, which also applies the deferred x update and
 * restricts q); 1: FP32 vector update; 2: FP64 stencil + dot; after a
 * learned-preconditioner solve also 3: one application of the
 * preconditioner (restriction, U-Net, the step that updates r and forms z:
 * 12 launches), 5: the 9 U-Net convolutions alone (0 fine-grid bytes) and
 * 6: the multiplicative step alone.  which 4 is not used.
 * Reports the mean time and the algorithmic bytes one launch (one
 * application) moves on the fine grid. */
int sbm_bench_kernel(sbm_ctx* ctx, int which, int reps, float* ms_per_launch,
                     double* bytes_per_launch);

/* Batched solves (no counterpart in the reference): n independent
 * contexts, each loaded with a GENERIC problem (COEF, X, RHS), solved by the
 * mixed-precision CG to rel-res tol together in ONE graph launch: a parent
 * CUDA graph holds per volume a WHILE conditional node whose body is the
 * volume's captured iteration chunk, re-armed on the device while the
 * volume is not done (at most max_it + 2 rounds), so converged volumes stop
 * launching work and the host waits once.  Per-volume iterations, final
 * rel-res and status go to the n-element arrays; ms_total is the device
 * time of the whole batch.  precond SBM_PC_LEARNED applies per volume (its
 * own attached network and grid permitting, else Jacobi;
 * sbm_ctx_last_precond of each context).  The library caches the parent
 * graph of the last batch (rebuilt when the set of volumes changes); batch
 * calls from several host threads are serialised by a lock around that
 * cache, and a context must not be used by another call while its batch
 * runs. */
int sbm_batch_solve(sbm_ctx** ctxs, int n, int bc_x0, int bc_x1, double scale, double tol,
                    int max_it, int precond, int* iters, double* final_res, int* status,
                    float* ms_total);

/* The same with one system per context of either GENERIC operator: ops[v]
 * is SBM_OP_GENERIC (potential form) or SBM_OP_GENERIC_DIAG (concentration
 * form, diagonal from the context's DIAG field), with its own x-face rules
 * and scale, so potential and concentration systems of many sub-volumes
 * advance in the same graph launches.  The learned preconditioner applies
 * to GENERIC systems only (GENERIC_DIAG ones use Jacobi). */
int sbm_batch_solve_ops(sbm_ctx** ctxs, const int* ops, const int* bc_x0, const int* bc_x1,
                        const double* scale, int n, double tol, int max_it, int precond,
                        int* iters, double* final_res, int* status, float* ms_total);

/* One electrochemical time step, the body of the reference's time loop
 * (SBMES:397-840) for a given dt, voltage-scan rate vsr and step index
 * iter: Cahn-Hilliard, CnE implicit solve with the flux BC and mean
 * correction, Dab/pce/pcN, tables, Butler-Volmer Picard loop with the phP
 * and phE solves, current sum and voltage control.  precision
 * SBM_PREC_FP64 runs the reference's plain CG with its stopping norms;
 * SBM_PREC_MIXED solves each system to rel-res 1e-10 with the mixed solver,
 * preconditioned by the attached network where it applies (see
 * SBM_PC_LEARNED below), else by Jacobi. */
int sbm_time_step(sbm_ctx* ctx, int iter, double dt, double vsr,
                  int precision, sbm_scalars* s);

/* Stages of the same step, callable one at a time. */
int sbm_ch_step(sbm_ctx* ctx, double dt, sbm_scalars* s);            /* SBMES:397-443 */
int sbm_cne_step(sbm_ctx* ctx, int iter, double dt, int precision,
                 sbm_scalars* s);                                     /* SBMES:461-572 */
int sbm_bv_update(sbm_ctx* ctx, int precision, sbm_scalars* s);      /* SBMES:577-812 */
int sbm_voltage_step(sbm_ctx* ctx, double dt, double vsr,
                     sbm_scalars* s);                                 /* SBMES:826-835 */

/* ---------------------------------------------------- stateless kernels
 * These take HOST arrays, copy to the device, run, and copy back, so a
 * Fortran host can swap them in for the named subroutines one for one. */

/* Tbl_Chk_Pln_3DA(py,px,pz,sz,Cord,Vals,Cn,fn), SBMES:987-1028.
 * n = py*px*pz voxels. */
int sbm_table_lookup(int64_t n, int sz, const double* cord, const double* vals,
                     const double* cn, double* fn);

/* ReDist3D_XYZ(lit,py,px,pz,sg,f), LevelSet_3D.f90:194-261 (dt = 1.0d-1)
 * and RM_UCNCT_3D.f90:209-276 (dt = 1.0e-1 REAL(4)): in place on f,
 * halo-padded.  Bit-exact with the reference arithmetic. */
int sbm_redist(int lit, int py, int px, int pz, double dt,
               const double* sg, double* f);

/* Allen-Cahn pre-smoothing of the stacked voxel field before the sign and
 * the reinitialisation, LevelSet_3D.f90:116-136: NoGrdBc3D, then `iters`
 * steps (the reference runs 50) of
 *   sgF = 2 f (1 - f)(1 - 2 f) - 0.64 (sum of the 6 neighbours - 6 f),
 *   f = f - 0.05 sgF   (0.64, 0.05 REAL(4)), NoGrdBc3D,
 * in place on the halo-padded (py+2)(px+2)(pz+2) array; bit-exact. */
int sbm_allen_cahn(int iters, int py, int px, int pz, double* f);

/* The stacked voxel field of LevelSet_3D.f90:80-122 for one tunnel radius:
 * vox = TmpA(yo,xo,zo) (Fortran order) is reoriented (TmpB(i,k,j) =
 * TmpA(i,j,zo-k+1)), cylindrical tunnels of radius tr about (i,k) = (1,zg)
 * and (yg,1) are zeroed by the reference's loop over j = 1..xg (its writes
 * past TmpB's second extent zo land where column-major storage puts them,
 * :87-106), and nthick thicknesses of zo columns (even ones straight, odd
 * ones mirrored) are stacked after xoff zero columns (:109-119; the
 * reference: yo,xo,zo = 500,520,170, yg = 93, zg = 160, xoff = 50,
 * nthick = 4, tr = TuRd(3..13)).  ds: the halo-padded
 * (yg+2)(xg+2)(zg+2) field, xg = xoff + nthick*zo, ghosts zero-gradient
 * (:122).  Requires yg <= yo, zg <= xo and (xg-1) + zo*(zg-1) < zo*xo (the
 * tunnel loop stays inside TmpB).  Bit-exact. */
int sbm_ls_geometry(const double* vox, int yo, int xo, int zo, int yg, int zg, int xoff,
                    int nthick, double tr, double* ds);

/* One frame of the LevelSet_3D front end on the GPU (:80-150): the stacked
 * field above, ac_iters Allen-Cahn steps (50), sign (> 0.5 -> +1, else -1,
 * ghosts included), lit reinitialisation steps (175) of time step dt (0.1)
 * from zero.  ds: the halo-padded distance (OutPut3D writes its interior).
 * Bit-exact with the reference arithmetic. */
int sbm_ls_frontend(const double* vox, int yo, int xo, int zo, int yg, int zg, int xoff,
                    int nthick, double tr, int ac_iters, int lit, double dt, double* ds);

/* The per-frame body of the AccDiff_3D program (AccDiff_3D.f90:76-243):
 * psi = 0.5*(1.0+TANH(dist/width)) (width 0.75; computed on the host with
 * the C library's tanh) with zero-gradient ghosts, then `term` (1501)
 * connectivity sweeps of the solid (Cn = 1 on the x = px+1 face) and of the
 * electrolyte (interior psi -> 1 - psi, the ghosts keeping the solid values
 * as in the reference; Cn = 1 on the x = 0 face), each from Cn = 0.
 * dist: interior py*px*pz; cn_solid / cn_elec: halo-padded outputs.
 * Bit-exact with the reference arithmetic. */
int sbm_connectivity(int py, int px, int pz, const double* dist, double width, int term,
                     double* cn_solid, double* cn_elec);

/* The per-frame body of the RM_UCNCT_3D program (RM_UCNCT_3D.f90:68-141):
 * for the solid (psA = 0.5*(1.0+TANH(dist/1.0))) and the electrolyte
 * (1 - psA), zero psA where the phase's Cn < 1.0e-4, sign (> 0.5) with
 * zero-gradient ghosts and `lit` (175) reinitialisation steps from zero with
 * dt = 1.0e-1 REAL(4): the distance of each phase with its disconnected
 * regions removed.  dist, cn_solid, cn_elec: interior py*px*pz;
 * d_solid / d_elec: halo-padded outputs.  Bit-exact. */
int sbm_rm_ucnct(int py, int px, int pz, const double* dist, const double* cn_solid,
                 const double* cn_elec, int lit, double* d_solid, double* d_elec);

/* sbm_ls_frontend on caller-owned DEVICE buffers: vox (yo*xo*zo doubles),
 * ds, sg, tmp (each (yg+2)(xg+2)(zg+2) doubles; ds receives the distance,
 * sg the sign field, tmp is scratch).  Enqueued on `stream` (cudaStream_t,
 * NULL = the default stream); returns without waiting. */
int sbm_ls_frontend_device(const double* vox, int yo, int xo, int zo, int yg, int zg, int xoff,
                           int nthick, double tr, int ac_iters, int lit, double dt, double* ds,
                           double* sg, double* tmp, void* stream);

/* One phase of the AccDiff_3D connectivity sweep, AccDiff_3D.f90:111-169
 * (solid, dirichlet_x = 1: Dirichlet 1 at x = px+1) and :185-243
 * (electrolyte, dirichlet_x = 0: Dirichlet 1 at x = 0), for iterations
 * 2..term.  psi and cn halo-padded; cn in/out.  Bit-exact. */
int sbm_accdiff(int py, int px, int pz, const double* psi, double* cn,
                int term, int dirichlet_x);

/* ReDist3D_XYZ without any device allocation.  No counterpart in the
 * reference.  Some callers cannot allocate device memory: a host program
 * whose GPU memory is all owned by another allocator or framework, or one
 * that runs under a fixed memory budget set at start-up.  This variant takes
 * DEVICE pointers sg and f (halo-padded, f in/out), enqueues the lit
 * iterations on `stream` (a cudaStream_t; NULL = the default stream) and
 * blocks the calling thread until that stream has finished them
 * (cudaStreamSynchronize).  Its scratch is a fixed array built into the
 * library (SBM_NOALLOC_REDIST_MAX_CELLS doubles, 8 MiB, held on every GPU
 * that loads the library until exit); grids of more padded cells, or with
 * pz + 2 > 65535, are rejected with SBM_ERR_ARG and a message in
 * sbm_last_error().  It calls no cudaMalloc or cudaFree.  Because it
 * synchronizes the stream, no call (first or later) may be made while that
 * stream is being captured into a graph.  All calls share the scratch: calls that
 * overlap on the GPU race.  Results are bit-identical to sbm_redist. */
#define SBM_NOALLOC_REDIST_MAX_CELLS (1 << 20)
int sbm_redist_noalloc(int lit, int py, int px, int pz, double dt, const double* sg, double* f,
                       void* stream);

/* RM_UCNCT_3D.f90:78-82 / :127-130: psB = psA, psB = 0 where Cn < 1e-4
 * (REAL(4) literal).  n voxels, bit-exact. */
int sbm_rm_mask(int64_t n, const double* psA, const double* cn, double* psB);

/* Sign function, LevelSet_3D.f90:140-144 / RM_UCNCT_3D.f90:92-96:
 * sg = 1 where ds > thr else -1; n values (halo-padded array). */
int sbm_sign(int64_t n, const double* ds, double thr, double* sg);

/* Text of the last error (CUDA failure or size rejection) seen by this thread. */
const char* sbm_last_error(void);
/* One BF16 3x3x3 convolution (zero padding) of a channels-last grid, the
 * building block of the learned preconditioner; no counterpart in the
 * reference.  x: (ny*nx*nz) x cin BF16 bit patterns, voxel v = i + ny*(j +
 * nx*k); w: cout x 27 x cin BF16 (tap t = (di+1) + 3(dj+1) + 9(dk+1));
 * bias: cout FP32 (may be NULL); y: (ny*nx*nz) x cout FP32.  flip = 1 reads
 * the neighbour at minus the tap offset (the transposed convolution of the
 * backward pass).  use_tc = 1: tcgen05 tensor-core kernel; 0: CUDA-core
 * kernel.  cin, cout multiples of 16, cout <= 256. */
int sbm_conv3d_bf16(int ny, int nx, int nz, int cin, int cout, const uint16_t* x,
                    const uint16_t* w, const float* bias, int relu, int flip, int use_tc,
                    float* y);

/* ---- Learned coarse-grid preconditioner (no counterpart in the reference).
 *
 * A 3D U-Net on the grid coarsened 4x per axis proposes the smooth part of
 * the error, z1 = P e_c with e_c = (s k_out / (scale c_ref)) N(f), followed
 * by one over-relaxed Jacobi step on the residual it leaves:
 * z = z1 + 2.3 D^-1 (r - A z1) (the default; z = D^-1 r + z1 with
 * SBM_TUNE_PC_ADDITIVE), R = 4x4x4 average, P = cell-centred trilinear
 * interpolation, s = RMS(R r),
 * c_ref = mean(R K); the input channels f (16 per coarse cell, voxel
 * v = i + ny*(j + nx*k)) are [R r / s, R K / c_ref, 1, x0-face Dirichlet
 * mask, x1-face Dirichlet mask, 0 x 11].  Because z is not linear in r the
 * solver runs flexible CG (beta = -z.q_old / p_old.q_old).
 * SBM_PC_LEARNED applies when a network is attached and ny, nx, nz are
 * multiples of 16 (the coarse grid, ny/4 x nx/4 x nz/4 cells, is padded with
 * zero cells to multiples of 16 for the U-Net, whose activations stay zero
 * there), to the phP / phE / GENERIC form, and to the CnE / GENERIC_DIAG
 * form q = diag p - scale S(p) when the network was trained with the mass
 * channel (input channel 5 = x / (1 + x), x = R diag / (scale c_ref); the
 * output's sign follows the operator's); otherwise the solve falls back to
 * Jacobi (sbm_ctx_last_precond reports which ran).
 * Only the mixed-precision solver takes it.  Training / forward calls on
 * one network come from one host thread at a time; any number of contexts
 * may share a network as their preconditioner (they only read its
 * weights). */
typedef struct sbm_net sbm_net;

/* Number of FP32 parameters of the network. */
int64_t sbm_net_param_count(void);
/* New network, He-normal initialised from `seed`. */
int sbm_net_create(uint64_t seed, sbm_net** out);
int sbm_net_destroy(sbm_net* net);
/* Master (FP32) parameters; set also resets the Adam state. */
int sbm_net_get_params(const sbm_net* net, float* host, int64_t count);
int sbm_net_set_params(sbm_net* net, const float* host, int64_t count);
/* Forward pass on nb samples of ny x nx x nz coarse cells (multiples of 16)
 * stacked along z: in (nb*ny*nx*nz) x 16 FP32 (rounded to BF16), out
 * nb*ny*nx*nz FP32. */
int sbm_net_forward(sbm_net* net, int ny, int nx, int nz, int nb, const float* in, float* out);
/* loss = mean (out - target)^2 and its gradient with respect to every
 * parameter (FP32, same order as the parameters; grad may be NULL). */
int sbm_net_loss_grad(sbm_net* net, int ny, int nx, int nz, int nb, const float* in,
                      const float* target, double* loss, float* grad);
/* Training set kept on the device until replaced or the network is
 * destroyed: nsamples input / target pairs of ny x nx x nz coarse cells. */
int sbm_net_set_data(sbm_net* net, int ny, int nx, int nz, int nsamples, const float* in,
                     const float* target);
/* `steps` Adam steps (learning rate lr) on mini-batches of `batch` samples
 * drawn (seeded) from the resident training set; loss_hist[steps] receives
 * each step's loss (may be NULL).  Adam's moments carry over between calls. */
int sbm_net_train_steps(sbm_net* net, int steps, int batch, float lr, uint64_t seed,
                        float* loss_hist);
/* sbm_net_set_data followed by sbm_net_train_steps. */
int sbm_net_train(sbm_net* net, int ny, int nx, int nz, int nsamples, const float* in,
                  const float* target, int steps, int batch, float lr, uint64_t seed,
                  float* loss_hist);
/* New network from a weights file (elsim_gb300/weights/pc_unet.bin: magic
 * "SBMNET01", or "SBMNET02" for a network trained with the mass channel,
 * int64 parameter count, float64 k_out, FP32 parameters); *out_scale
 * receives k_out for sbm_ctx_set_net. */
int sbm_net_load(const char* path, sbm_net** out, double* out_scale);
/* Whether the network reads input channel 5 (the CnE form's mass term): a
 * network trained on such systems sets it (1) before it is attached; the
 * getter returns 0 or 1. */
int sbm_net_set_mass_channel(sbm_net* net, int on);
int sbm_net_get_mass_channel(const sbm_net* net);
/* Attach `net` (NULL detaches) to a context with output scale k_out.  The
 * context does not own the network: keep it alive while attached. */
int sbm_ctx_set_net(sbm_ctx* ctx, sbm_net* net, double out_scale);
/* Preconditioner used by the last mixed-precision solve (SBM_PC_*).  A
 * learned-preconditioner solve whose FP32 residual norm stops halving
 * within 50 iterations continues as Jacobi-PCG and reports SBM_PC_JACOBI. */
int sbm_ctx_last_precond(const sbm_ctx* ctx);
/* One application z = M(r) of the learned preconditioner for the GENERIC
 * operator of the context's coefficient (halo-padded FP64 r and z). */
int sbm_learned_pc_apply(sbm_ctx* ctx, int bc_x0, int bc_x1, double scale, const double* r,
                         double* z);
/* The same for op = SBM_OP_GENERIC or SBM_OP_GENERIC_DIAG (diagonal from
 * the context's DIAG field). */
int sbm_learned_pc_apply_op(sbm_ctx* ctx, int op, int bc_x0, int bc_x1, double scale,
                            const double* r, double* z);

/* Test hook of the device-side bounded waits (no counterpart in the
 * reference): the number of attempts each consumer-side mbarrier wait of
 * the TMA-staged FP32 stencil kernel makes before the CTA gives up, records
 * the expiry (the solve returns SBM_ERR_TIMEOUT) and returns after waiting
 * out its own copies in flight with the full built-in bound.  tries < 0
 * restores the default (2^20 attempts, about a second); 0 makes every wait
 * give up at once.  Applies to the current device, for every context; call
 * it only while no solve runs. */
int sbm_set_wait_limit(int tries);

/* Double-float split (no counterpart in the reference): hi[i] = (float)x[i]
 * and lo[i] = (float)(x[i] - hi[i]) for n FP64 values, the hi + lo pairs
 * (about 48 significant bits) in which the mixed-precision solver carries
 * the operator, the initial iterate and the right-hand side.  Computed with
 * integer instructions, bit-identical to those FP64 expressions.  DEVICE
 * pointers; enqueued on `stream` (a cudaStream_t; NULL = the default
 * stream), asynchronous. */
int sbm_split_f64(int64_t n, const double* x, float* hi, float* lo, void* stream);

/* Version string of the compiled library. */
const char* sbm_version(void);
/* Number of kernel launches this process has issued through the library. */
int64_t sbm_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* SBM_CAPI_H */
