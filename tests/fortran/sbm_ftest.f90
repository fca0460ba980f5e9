! Fortran host calling libsbm_gb300 through the sbm_capi bind(C) module, as
! the reference program would: the Laplace problem between the Dirichlet x
! ghost planes (phi = 0 at j = 0, 1 at j = nx+1, Neumann in y and z), whose
! discrete solution is phi(j) = j / (nx+1), by the FP64 CG and by the mixed
! solver with Jacobi preconditioning; and one Tbl_Chk_Pln_3DA lookup.
program sbm_ftest
  use, intrinsic :: iso_c_binding
  use sbm_capi
  implicit none
  integer(c_int), parameter :: ny = 16, nx = 16, nz = 16
  type(sbm_params) :: p
  type(c_ptr) :: ctx
  real(c_double), allocatable :: coef(:,:,:), x(:,:,:), rhs(:,:,:)
  real(c_double) :: cord(11), vals(11), cn(3), fn(3), res, err
  real(c_float) :: ms
  integer(c_int) :: rc, it, prec
  integer :: j

  allocate(coef(0:ny+1, 0:nx+1, 0:nz+1), x(0:ny+1, 0:nx+1, 0:nz+1), rhs(0:ny+1, 0:nx+1, 0:nz+1))
  rc = sbm_params_reference(p)
  rc = sbm_ctx_create(ny, nx, nz, p, ctx)
  if (rc /= SBM_OK) stop 1
  coef = 1.0d0
  rhs = 0.0d0
  rc = sbm_upload(ctx, SBM_F_COEF, coef, 1)
  rc = sbm_upload(ctx, SBM_F_RHS, rhs, 1)
  do prec = SBM_PREC_FP64, SBM_PREC_MIXED
    x = 0.0d0
    x(:, nx + 1, :) = 1.0d0
    rc = sbm_upload(ctx, SBM_F_X, x, 1)
    rc = sbm_cg_solve(ctx, SBM_OP_GENERIC, SBM_BC_ZERO, SBM_BC_ZERO, 1.0d0, 1.0d-10, 10000, &
                      SBM_STOP_REL_RES, prec, SBM_PC_JACOBI * prec, it, res, ms)
    if (rc /= SBM_OK) stop 2
    rc = sbm_download(ctx, SBM_F_X, x, 1)
    err = 0.0d0
    do j = 1, nx
      err = max(err, maxval(abs(x(1:ny, j, 1:nz) - dble(j) / dble(nx + 1))))
    end do
    if (err > 1.0d-7) stop 3
    print '(a,i0,a,i0,a,es10.2)', 'fortran solve ok: precision ', prec, ', ', it, &
          ' iterations, max error ', err
  end do
  rc = sbm_ctx_destroy(ctx)
  do j = 1, 11
    cord(j) = 0.1d0 * (j - 1)
    vals(j) = 2.0d0 * cord(j) + 1.0d0
  end do
  cn = [0.05d0, 0.5d0, 0.95d0]
  rc = sbm_table_lookup(3_c_int64_t, 11, cord, vals, cn, fn)
  if (rc /= SBM_OK) stop 4
  print '(a,3f10.5)', 'fortran table ok: ', fn
end program sbm_ftest
