/*
 * sbm_oracle.h -- CPU oracle for the SBM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a line-by-line FP64 restatement of the
 * reference Fortran (AffanMalik90/Elsim, src/frtrn/ Fortran sources) in C, used as the
 * checker by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline leg.  The product path (elsim_gb300) never links or calls it.
 *
 * PARITY PINNED by the reference's own code: the reference ships no tests
 * or golden vectors and cannot be compiled here (no Fortran compiler, no
 * MPI), so tests/golden/fortran_subset.py interprets its Fortran sources
 * and tests/golden/reference_v1.npz holds what they compute on small seeded
 * cases.  This restatement matches them bit for bit (tests/
 * test_oracle_reference.py): every element-wise routine, and the coupled
 * time step too once the reference's SUMs run in this file's order of
 * reduction (below); with the reference's sequential SUMs the iteration
 * counts are identical and the fields agree to the solves' rounding.
 * Analytic known-answer tests (tests/test_oracle_pins.py) pin it as well.
 *
 * Rules kept from the reference:
 *   - Fortran evaluation order of every expression (left to right for
 *     + - and * /, ** before * /);
 *   - REAL(4) literals promoted as gfortran promotes them, e.g. 0.4 is
 *     (double)0.4f, and `1.05625e-02*0.125*0.75` is evaluated in float;
 *   - WHERE semantics: each masked assignment completes over the whole
 *     array before the next statement;
 *   - compiled with -ffp-contract=off (no fused multiply-add).
 * Reductions are summed per z plane, then over planes in order, so the
 * result does not depend on the OpenMP thread count.
 */
#ifndef SBM_ORACLE_H
#define SBM_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#include "../include/sbm_capi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ghost fills */
void orc_nogrdbc(int py, int px, int pz, double* f);
void orc_bc_yz(int ny, int nx, int nz, double* f);
void orc_bc_x(int ny, int nx, int nz, double* f, int k0, int k1,
              int mode0, double v0, int mode1, double v1);

/* level set / connectivity */
void orc_absgrd(int py, int px, int pz, const double* sg, const double* f, double* gr);
void orc_redist(int lit, double dt, int py, int px, int pz, const double* sg, double* f);
void orc_accdiff(int py, int px, int pz, const double* psi, double* cn,
                 int term, int dirichlet_x);
void orc_connectivity(int py, int px, int pz, const double* dist, double width,
                      int term, double* cn_solid, double* cn_elec);
void orc_rm_mask(int64_t n, const double* psA, const double* cn, double* psB);
void orc_sign(int64_t n, const double* ds, double thr, double* sg);
void orc_allen_cahn(int iters, int py, int px, int pz, double* f);
void orc_rm_ucnct(int py, int px, int pz, const double* dist, const double* cn_solid,
                  const double* cn_elec, int lit, double* d_solid, double* d_elec);
int orc_ls_geometry(const double* vox, int yo, int xo, int zo, int yg, int zg, int xoff,
                    int nthick, double tr, double* ds);

/* fields */
void orc_psi_from_dist(int ny, int nx, int nz, const float* d, double zeta, double* psi);
void orc_avp(int ny, int nx, int nz, const double* psP, const double* psE, double dx,
             double mask, double* avp, double* avpx);
void orc_table(int64_t n, int sz, const double* cord, const double* vals,
               const double* cn, double* fn);

/* operator and CG */
void orc_apply(int ny, int nx, int nz, const double* K, const double* diag,
               double scale, const double* p, double* q);
void orc_residual(int ny, int nx, int nz, const double* K, const double* diag,
                  double scale, const double* rhs, const double* x, double* r);
int  orc_cg(int ny, int nx, int nz, const double* K, const double* diag, double scale,
            int bc_x0, int bc_x1, const double* rhs, double* x, const double* w,
            double wsum, int stop_rule, double tol, int max_it,
            int* iters, double* final_res);
double orc_dot(int ny, int nx, int nz, const double* a, const double* b);

/* electrochemical state (host mirror of the reference program state) */
typedef struct orc_state orc_state;
orc_state* orc_state_new(int ny, int nx, int nz, const sbm_params* p);
void orc_state_free(orc_state* s);
double* orc_state_field(orc_state* s, int field);
int  orc_setup_domain(orc_state* s, const float* dist_p, const float* dist_e,
                      double zeta, double cnp0, double cne0, double cr, sbm_scalars* sc);
int  orc_ch_step(orc_state* s, double dt, sbm_scalars* sc);
int  orc_cne_step(orc_state* s, int iter, double dt, sbm_scalars* sc);
int  orc_bv_update(orc_state* s, sbm_scalars* sc);
int  orc_voltage_step(orc_state* s, double dt, double vsr, sbm_scalars* sc);
int  orc_time_step(orc_state* s, int iter, double dt, double vsr, sbm_scalars* sc);

int  orc_params_reference(sbm_params* p);
int  orc_num_threads(void);
void orc_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
