/* C host of libsbm_gb300 (the C-ABI of include/sbm_capi.h): loads the
 * learned preconditioner from its weights file and solves a potential
 * problem with it.  Conductivity layered in z (1 and 0.1 in bands of 4
 * planes), phi = 0 / 1 on the x ghost planes, Neumann in y and z: the
 * discrete solution is phi(j) = j / (n+1) in every layer. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "sbm_capi.h"

int main(int argc, char** argv) {
  const char* weights = argc > 1 ? argv[1] : "elsim_gb300/weights/pc_unet.bin";
  const int n = 64;
  const int64_t s = n + 2, nh = s * s * s;
  sbm_params p;
  sbm_ctx* ctx = NULL;
  sbm_net* net = NULL;
  double kout = 0.0, res = 0.0, err = 0.0;
  int it = 0;
  float ms = 0.f;
  double* coef = (double*)malloc(sizeof(double) * nh);
  double* x = (double*)calloc((size_t)nh, sizeof(double));
  double* rhs = (double*)calloc((size_t)nh, sizeof(double));
  if (!coef || !x || !rhs) return 10;
  for (int k = 0; k < s; ++k)
    for (int j = 0; j < s; ++j)
      for (int i = 0; i < s; ++i) {
        const int64_t c = i + s * (j + s * (int64_t)k);
        coef[c] = ((k / 4) % 2 == 0) ? 1.0 : 0.1;
        if (j == n + 1) x[c] = 1.0;
      }
  if (sbm_params_reference(&p) || sbm_ctx_create(n, n, n, &p, &ctx)) return 1;
  if (sbm_upload(ctx, SBM_F_COEF, coef, 1) || sbm_upload(ctx, SBM_F_X, x, 1) ||
      sbm_upload(ctx, SBM_F_RHS, rhs, 1))
    return 2;
  if (sbm_net_load(weights, &net, &kout) || sbm_ctx_set_net(ctx, net, kout)) return 3;
  int rc = sbm_cg_solve(ctx, SBM_OP_GENERIC, SBM_BC_ZERO, SBM_BC_ZERO, 1.0, 1e-8, 100000,
                        SBM_STOP_REL_RES, SBM_PREC_MIXED, SBM_PC_LEARNED, &it, &res, &ms);
  if (rc) {
    fprintf(stderr, "solve failed: %d %s\n", rc, sbm_last_error());
    return 4;
  }
  const int used = sbm_ctx_last_precond(ctx);
  if (sbm_download(ctx, SBM_F_X, x, 1)) return 5;
  for (int k = 1; k <= n; ++k)
    for (int j = 1; j <= n; ++j)
      for (int i = 1; i <= n; ++i) {
        const double e = fabs(x[i + s * (j + s * (int64_t)k)] - (double)j / (double)(n + 1));
        if (e > err) err = e;
      }
  sbm_ctx_destroy(ctx);
  sbm_net_destroy(net);
  free(coef);
  free(x);
  free(rhs);
  printf("c host ok: %d iterations, preconditioner %d, rel-res %.2e, max error %.2e\n", it, used,
         res, err);
  /* the learned preconditioner, or Jacobi if it was switched off for lack
   * of progress on this (untrained-for) layered problem */
  return (err < 1e-6 && (used == SBM_PC_LEARNED || used == SBM_PC_JACOBI) && res <= 1e-8) ? 0 : 6;
}
