!! sbm_capi.f90 -- ISO_C_BINDING interface to libsbm_gb300.so (include/sbm_capi.h)
!!
!! The module a Fortran host uses to call the GB300 SBM library in place of
!! the inline solver blocks and subroutines of the reference program.
!! Arrays keep the reference layout: REAL(KIND=8) A(0:ny+1,0:nx+1,0:nz+1),
!! passed by reference (the first element's address).  Every function
!! returns an INTEGER(C_INT) status, 0 on success.
MODULE sbm_capi
  USE, INTRINSIC :: ISO_C_BINDING
  IMPLICIT NONE

  INTEGER(C_INT), PARAMETER :: SBM_OK = 0, SBM_ERR_MAXIT = -3
  INTEGER(C_INT), PARAMETER :: SBM_BC_COPY = 0, SBM_BC_ZERO = 1
  INTEGER(C_INT), PARAMETER :: SBM_OP_CNE = 0, SBM_OP_PHP = 1, SBM_OP_PHE = 2, SBM_OP_GENERIC = 3
  INTEGER(C_INT), PARAMETER :: SBM_OP_GENERIC_DIAG = 4
  INTEGER(C_INT), PARAMETER :: SBM_STOP_REF_UPDATE = 0, SBM_STOP_REF_RESID = 1, SBM_STOP_REL_RES = 2
  INTEGER(C_INT), PARAMETER :: SBM_PREC_FP64 = 0, SBM_PREC_MIXED = 1
  INTEGER(C_INT), PARAMETER :: SBM_PC_NONE = 0, SBM_PC_JACOBI = 1, SBM_PC_LEARNED = 2
  INTEGER(C_INT), PARAMETER :: SBM_BV_EXP = 0, SBM_BV_LINEAR = 1
  INTEGER(C_INT), PARAMETER :: SBM_CH_TABLE = 0, SBM_CH_DOUBLE_WELL = 1
  INTEGER(C_INT), PARAMETER :: SBM_F_PSP = 0, SBM_F_PSE = 1, SBM_F_AVP = 2, SBM_F_AVPX = 3, &
       SBM_F_CNP = 4, SBM_F_CNE = 5, SBM_F_PHP = 6, SBM_F_PHE = 7, SBM_F_RXN = 8, &
       SBM_F_COEF = 9, SBM_F_RHS = 10, SBM_F_X = 11, SBM_F_WEIGHT = 12, SBM_F_DIAG = 13
  INTEGER, PARAMETER :: SBM_TBL_MAX = 128

  TYPE, BIND(C) :: sbm_params
    REAL(C_DOUBLE) :: dx, rho, eps, ch_mask, d0, tc1, tc2, t_minus
    REAL(C_DOUBLE) :: dab_c0, dab_c1, dab_c2, dab_c3, cne_ref, cst1, frd, bvp, bve
    REAL(C_DOUBLE) :: kap_scale, avp_mask, i0_scale, kfw_c
    REAL(C_DOUBLE) :: crt_cne, crt_php, crt_phe, crt_picard
    INTEGER(C_INT) :: max_it_cne, max_it_php, max_it_phe, max_picard
    INTEGER(C_INT) :: cne_mean_every, bv_mode, tbl_n, ch_mode
    REAL(C_DOUBLE) :: tbl_x(SBM_TBL_MAX), tbl_mu(SBM_TBL_MAX), tbl_mb(SBM_TBL_MAX)
    REAL(C_DOUBLE) :: tbl_i0(SBM_TBL_MAX), tbl_ocv(SBM_TBL_MAX)
    REAL(C_DOUBLE) :: ch_w
  END TYPE sbm_params

  TYPE, BIND(C) :: sbm_scalars
    REAL(C_DOUBLE) :: tPP, tPE, xrf, infx, scrnt, trgI, bve, cvgp, cvgl
    INTEGER(C_INT) :: it_cne, it_php, it_phe, n_picard
  END TYPE sbm_scalars

  INTERFACE
    INTEGER(C_INT) FUNCTION sbm_params_reference(p) BIND(C, NAME='sbm_params_reference')
      IMPORT :: C_INT, sbm_params
      TYPE(sbm_params), INTENT(OUT) :: p
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_ctx_create(ny, nx, nz, p, ctx) BIND(C, NAME='sbm_ctx_create')
      IMPORT :: C_INT, C_PTR, sbm_params
      INTEGER(C_INT), VALUE :: ny, nx, nz
      TYPE(sbm_params), INTENT(IN) :: p
      TYPE(C_PTR), INTENT(OUT) :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_ctx_destroy(ctx) BIND(C, NAME='sbm_ctx_destroy')
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_ctx_snapshot_size(ctx, bytes) BIND(C, NAME='sbm_ctx_snapshot_size')
      IMPORT :: C_INT, C_PTR, C_SIZE_T
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_SIZE_T), INTENT(OUT) :: bytes
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_ctx_snapshot(ctx, buf, bytes) BIND(C, NAME='sbm_ctx_snapshot')
      IMPORT :: C_INT, C_PTR, C_SIZE_T
      TYPE(C_PTR), VALUE :: ctx, buf
      INTEGER(C_SIZE_T), VALUE :: bytes
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_ctx_restore(ctx, buf, bytes) BIND(C, NAME='sbm_ctx_restore')
      IMPORT :: C_INT, C_PTR, C_SIZE_T
      TYPE(C_PTR), VALUE :: ctx, buf
      INTEGER(C_SIZE_T), VALUE :: bytes
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_upload(ctx, field, h, haloed) BIND(C, NAME='sbm_upload')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: field, haloed
      REAL(C_DOUBLE), INTENT(IN) :: h(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_download(ctx, field, h, haloed) BIND(C, NAME='sbm_download')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: field, haloed
      REAL(C_DOUBLE), INTENT(OUT) :: h(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_setup_domain(ctx, dist_p, dist_e, zeta, cnp0, cne0, cr, s) &
         BIND(C, NAME='sbm_setup_domain')
      IMPORT :: C_INT, C_PTR, C_FLOAT, C_DOUBLE, sbm_scalars
      TYPE(C_PTR), VALUE :: ctx
      REAL(C_FLOAT), INTENT(IN) :: dist_p(*), dist_e(*)
      REAL(C_DOUBLE), VALUE :: zeta, cnp0, cne0, cr
      TYPE(sbm_scalars), INTENT(OUT) :: s
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_time_step(ctx, iter, dt, vsr, precision, s) &
         BIND(C, NAME='sbm_time_step')
      IMPORT :: C_INT, C_PTR, C_DOUBLE, sbm_scalars
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: iter, precision
      REAL(C_DOUBLE), VALUE :: dt, vsr
      TYPE(sbm_scalars), INTENT(OUT) :: s
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_cg_solve(ctx, op, bc_x0, bc_x1, scale, tol, max_it, stop_rule, &
         precision, precond, iters, final_res, ms) BIND(C, NAME='sbm_cg_solve')
      IMPORT :: C_INT, C_PTR, C_DOUBLE, C_FLOAT
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: op, bc_x0, bc_x1, max_it, stop_rule, precision, precond
      REAL(C_DOUBLE), VALUE :: scale, tol
      INTEGER(C_INT), INTENT(OUT) :: iters
      REAL(C_DOUBLE), INTENT(OUT) :: final_res
      REAL(C_FLOAT), INTENT(OUT) :: ms
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_table_lookup(n, sz, cord, vals, cn, fn) &
         BIND(C, NAME='sbm_table_lookup')
      IMPORT :: C_INT, C_INT64_T, C_DOUBLE
      INTEGER(C_INT64_T), VALUE :: n
      INTEGER(C_INT), VALUE :: sz
      REAL(C_DOUBLE), INTENT(IN) :: cord(*), vals(*), cn(*)
      REAL(C_DOUBLE), INTENT(OUT) :: fn(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_redist(lit, py, px, pz, dt, sg, f) BIND(C, NAME='sbm_redist')
      IMPORT :: C_INT, C_DOUBLE
      INTEGER(C_INT), VALUE :: lit, py, px, pz
      REAL(C_DOUBLE), VALUE :: dt
      REAL(C_DOUBLE), INTENT(IN) :: sg(*)
      REAL(C_DOUBLE), INTENT(INOUT) :: f(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_allen_cahn(iters, py, px, pz, f) BIND(C, NAME='sbm_allen_cahn')
      IMPORT :: C_INT, C_DOUBLE
      INTEGER(C_INT), VALUE :: iters, py, px, pz
      REAL(C_DOUBLE), INTENT(INOUT) :: f(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_ls_geometry(vox, yo, xo, zo, yg, zg, xoff, nthick, tr, ds) &
        BIND(C, NAME='sbm_ls_geometry')
      IMPORT :: C_INT, C_DOUBLE
      REAL(C_DOUBLE), INTENT(IN) :: vox(*)
      INTEGER(C_INT), VALUE :: yo, xo, zo, yg, zg, xoff, nthick
      REAL(C_DOUBLE), VALUE :: tr
      REAL(C_DOUBLE), INTENT(OUT) :: ds(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_ls_frontend(vox, yo, xo, zo, yg, zg, xoff, nthick, tr, &
        ac_iters, lit, dt, ds) BIND(C, NAME='sbm_ls_frontend')
      IMPORT :: C_INT, C_DOUBLE
      REAL(C_DOUBLE), INTENT(IN) :: vox(*)
      INTEGER(C_INT), VALUE :: yo, xo, zo, yg, zg, xoff, nthick, ac_iters, lit
      REAL(C_DOUBLE), VALUE :: tr, dt
      REAL(C_DOUBLE), INTENT(OUT) :: ds(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_ls_frontend_device(vox, yo, xo, zo, yg, zg, xoff, nthick, tr, &
        ac_iters, lit, dt, ds, sg, tmp, stream) BIND(C, NAME='sbm_ls_frontend_device')
      IMPORT :: C_INT, C_DOUBLE, C_PTR
      TYPE(C_PTR), VALUE :: vox, ds, sg, tmp, stream
      INTEGER(C_INT), VALUE :: yo, xo, zo, yg, zg, xoff, nthick, ac_iters, lit
      REAL(C_DOUBLE), VALUE :: tr, dt
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_connectivity(py, px, pz, dist, width, term, cn_solid, cn_elec) &
        BIND(C, NAME='sbm_connectivity')
      IMPORT :: C_INT, C_DOUBLE
      INTEGER(C_INT), VALUE :: py, px, pz, term
      REAL(C_DOUBLE), VALUE :: width
      REAL(C_DOUBLE), INTENT(IN) :: dist(*)
      REAL(C_DOUBLE), INTENT(OUT) :: cn_solid(*), cn_elec(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_rm_ucnct(py, px, pz, dist, cn_solid, cn_elec, lit, d_solid, &
        d_elec) BIND(C, NAME='sbm_rm_ucnct')
      IMPORT :: C_INT, C_DOUBLE
      INTEGER(C_INT), VALUE :: py, px, pz, lit
      REAL(C_DOUBLE), INTENT(IN) :: dist(*), cn_solid(*), cn_elec(*)
      REAL(C_DOUBLE), INTENT(OUT) :: d_solid(*), d_elec(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_accdiff(py, px, pz, psi, cn, term, dirichlet_x) &
         BIND(C, NAME='sbm_accdiff')
      IMPORT :: C_INT, C_DOUBLE
      INTEGER(C_INT), VALUE :: py, px, pz, term, dirichlet_x
      REAL(C_DOUBLE), INTENT(IN) :: psi(*)
      REAL(C_DOUBLE), INTENT(INOUT) :: cn(*)
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_rm_mask(n, psA, cn, psB) BIND(C, NAME='sbm_rm_mask')
      IMPORT :: C_INT, C_INT64_T, C_DOUBLE
      INTEGER(C_INT64_T), VALUE :: n
      REAL(C_DOUBLE), INTENT(IN) :: psA(*), cn(*)
      REAL(C_DOUBLE), INTENT(OUT) :: psB(*)
    END FUNCTION
    ! learned coarse-grid preconditioner (SBM_PC_LEARNED with SBM_PREC_MIXED)
    INTEGER(C_INT) FUNCTION sbm_net_load(path, net, out_scale) BIND(C, NAME='sbm_net_load')
      IMPORT :: C_INT, C_PTR, C_CHAR, C_DOUBLE
      CHARACTER(KIND=C_CHAR), INTENT(IN) :: path(*)   ! NUL-terminated
      TYPE(C_PTR), INTENT(OUT) :: net
      REAL(C_DOUBLE), INTENT(OUT) :: out_scale
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_net_destroy(net) BIND(C, NAME='sbm_net_destroy')
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: net
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_ctx_set_net(ctx, net, out_scale) BIND(C, NAME='sbm_ctx_set_net')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx, net
      REAL(C_DOUBLE), VALUE :: out_scale
    END FUNCTION
    INTEGER(C_INT) FUNCTION sbm_ctx_last_precond(ctx) BIND(C, NAME='sbm_ctx_last_precond')
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION
  END INTERFACE
END MODULE sbm_capi
