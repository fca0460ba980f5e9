// sbm_capi.cu -- the extern "C" boundary of the GB300 SBM library.
//
// Context lifetime, host<->device copies, and the entry points that stand in
// for the reference's inline solver blocks and subroutines (each function
// names the reference lines it replaces in include/sbm_capi.h).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "sbm_internal.cuh"
#include "sbm_net.cuh"

namespace sbm {

std::atomic<int64_t> g_launches{0};
static thread_local char g_err[256] = "";

void set_error(const char* where, cudaError_t e) {
  snprintf(g_err, sizeof(g_err), "%s: %s", where, cudaGetErrorString(e));
}
void set_error_msg(const char* msg) { snprintf(g_err, sizeof(g_err), "%s", msg); }
const char* last_error() { return g_err; }

// defined in sbm_fields.cu / sbm_levelset.cu
int upload_tables(sbm_ctx* ctx);
int step_setup(sbm_ctx* ctx, const float* dp, const float* de, double zeta, double cnp0,
               double cne0, double cr, sbm_scalars* out);
int step_ch(sbm_ctx* ctx, double dt, sbm_scalars* out);
int step_cne(sbm_ctx* ctx, int iter, double dt, int precision, sbm_scalars* out);
int step_bv(sbm_ctx* ctx, int precision, sbm_scalars* out);
int step_voltage(sbm_ctx* ctx, double dt, double vsr, sbm_scalars* out);
int table_lookup_dev(cudaStream_t s, int64_t n, int sz, const double* dx, const double* dv,
                     const double* cn, double* fn);
int redist_dev(cudaStream_t s, const Geo& g, const double* sg, double* f, double* tmp, int lit,
               double dt);
int accdiff_dev(cudaStream_t s, const Geo& g, const double* psi, double* cn, double* tmp,
                int term, int dirichlet_x);
int rm_mask_dev(cudaStream_t s, int64_t n, const double* psA, const double* cn, double* psB);
int allen_cahn_dev(cudaStream_t s, const Geo& g, double* f, double* tmp, int iters);
int ls_geometry_dev(cudaStream_t s, const Geo& g, const double* vox, int yo, int xo, int zo,
                    int xoff, double tr, double* ds);
int ls_frontend_dev(cudaStream_t s, const Geo& g, const double* vox, int yo, int xo, int zo,
                    int xoff, double tr, int ac_iters, int lit, double dt, double* ds, double* sg,
                    double* tmp);
int sign_dev(cudaStream_t s, int64_t n, const double* ds, double thr, double* sg);
int ghost_after_solve(sbm_ctx* ctx, double* f, int bcx0, int bcx1);

static int dalloc(double** p, int64_t n) {
  cudaError_t e = cudaMalloc(p, sizeof(double) * (size_t)n);
  if (e != cudaSuccess) {
    set_error("cudaMalloc", e);
    *p = nullptr;
    return SBM_ERR_NOMEM;
  }
  e = cudaMemset(*p, 0, sizeof(double) * (size_t)n);
  if (e != cudaSuccess) {
    set_error("cudaMemset", e);
    return SBM_ERR_CUDA;
  }
  return SBM_OK;
}

int ensure_fp32_work(sbm_ctx* ctx) {
  if (ctx->hk32) return SBM_OK;
  float** bufs[] = {&ctx->hk32,   &ctx->dg32,   &ctx->r32,    &ctx->p32,    &ctx->q32,
                    &ctx->x32,    &ctx->z32,    &ctx->rold32, &ctx->hklo32, &ctx->dglo32,
                    &ctx->r0hi32, &ctx->r0lo32, &ctx->dhi32,  &ctx->dlo32};
  for (float** b : bufs) {
    cudaError_t e = cudaMalloc(b, sizeof(float) * (size_t)ctx->g32.nh);
    if (e != cudaSuccess) {
      set_error("cudaMalloc fp32", e);
      return SBM_ERR_NOMEM;
    }
    if (cudaMemset(*b, 0, sizeof(float) * (size_t)ctx->g32.nh) != cudaSuccess) return SBM_ERR_CUDA;
  }
  return SBM_OK;
}

static int ensure_step_work(sbm_ctx* ctx) {
  if (ctx->hk_kap) return SBM_OK;
  double** bufs[] = {&ctx->hk_kap, &ctx->hk_pce, &ctx->hk_pcc, &ctx->dab, &ctx->mu, &ctx->mb,
                     &ctx->rhe,    &ctx->rxc,    &ctx->kfw,    &ctx->kbw, &ctx->ppo, &ctx->peo};
  for (double** b : bufs) {
    int rc = dalloc(b, ctx->g.nh);
    if (rc) return rc;
  }
  return upload_tables(ctx);
}

}  // namespace sbm

using namespace sbm;

extern "C" {

const char* sbm_version(void) { return "elsim_gb300 sm_103a 0.1"; }
int64_t sbm_launch_count(void) { return g_launches.load(); }
const char* sbm_last_error(void) { return last_error(); }

int sbm_params_reference(sbm_params* p) {
  if (!p) return SBM_ERR_ARG;
  memset(p, 0, sizeof(*p));
  p->dx = 3.25e-5 * 0.5;                               // SBMES:90
  p->rho = (double)0.0312f;                             // :100
  p->eps = 6.7600e-10;                                  // :136
  p->ch_mask = 1.0e-5;                                  // :430
  p->cst1 = 1.6021766e-19 / (1.3806488e-23 * 300.0);   // :101
  p->frd = (double)96485.3365f;                         // :102
  p->bvp = (double)(-0.1f);                             // :106
  p->bve = (double)(-0.4495f);                          // :107
  const double de = 2.0 * (4.0e-6 * 1.25e-6) / (4.0e-6 + 1.25e-6);        // :118
  p->t_minus = 4.0e-6 / (4.0e-6 + 1.25e-6);                               // :121
  p->d0 = (de / 2.598606299407882e-06) * (double)0.006667f;               // :124
  p->tc1 = (2 * p->t_minus - 1.0) / (2 * p->t_minus * (1.0 - p->t_minus)); // :125
  p->tc2 = 1.0 / (2 * p->t_minus * (1.0 - p->t_minus)) * p->cst1;        // :126
  p->dab_c0 = (double)(-7.02f);                          // :474
  p->dab_c1 = 0.83e3;
  p->dab_c2 = (double)0.05f;
  p->dab_c3 = 1.0e3;
  p->cne_ref = 1.0e-3;                                   // :567
  p->kap_scale = (double)3.3f;                           // :324
  p->avp_mask = 1.0e-2;                                  // :287, :631
  p->i0_scale = 1.0e-3;                                  // :617
  p->kfw_c = (double)0.001f;                             // :621
  p->crt_cne = 1.0e-7;                                   // :96
  p->crt_php = 1.0e-7;                                   // :97
  p->crt_phe = 1.0e-6;                                   // :98
  p->crt_picard = 1.0e-8;                                // :627
  p->max_it_cne = 50001;                                 // :551 (EXIT after itlp > 50000)
  p->ch_mode = SBM_CH_TABLE;
  p->ch_w = 1.0;
  p->max_it_php = 30001;                                 // :710
  p->max_it_phe = 100001;                                // :791
  p->max_picard = 1000;
  p->cne_mean_every = 100;                               // :562
  p->bv_mode = SBM_BV_EXP;
  p->tbl_n = 101;
  for (int t = 0; t < 101; ++t) p->tbl_x[t] = t * 0.01;
  return SBM_OK;
}

int sbm_ctx_create(int ny, int nx, int nz, const sbm_params* p, sbm_ctx** out) {
  if (!out || ny < 1 || nx < 1 || nz < 1) return SBM_ERR_ARG;
  if ((int64_t)(ny + 2) * (nx + 2) * (nz + 2) > ((int64_t)1 << 36)) return SBM_ERR_ARG;
  if (p && (p->tbl_n < 2 || p->tbl_n > SBM_TBL_MAX)) return SBM_ERR_ARG;
  *out = nullptr;
  sbm_ctx* ctx = new (std::nothrow) sbm_ctx();
  if (!ctx) return SBM_ERR_NOMEM;
  ctx->g = make_geo(ny, nx, nz);
  ctx->g32 = make_geo32(ny, nx, nz);
  if (p) ctx->p = *p;
  else sbm_params_reference(&ctx->p);
  int rc = SBM_OK;
  auto fail = [&](int code) {
    sbm_ctx_destroy(ctx);
    return code;
  };
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(SBM_ERR_CUDA);
  if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->evq[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->evq[1], cudaEventDisableTiming) != cudaSuccess)
    return fail(SBM_ERR_CUDA);
  for (int f = 0; f < SBM_F_COUNT; ++f)
    if ((rc = dalloc(&ctx->f[f], ctx->g.nh))) return fail(rc);
  double** cg[] = {&ctx->hk_gen, &ctx->r64, &ctx->p64, &ctx->q64, &ctx->d64};
  for (double** b : cg)
    if ((rc = dalloc(b, ctx->g.nh))) return fail(rc);
  ctx->rhs = ctx->f[SBM_F_RHS];
  // reduction partials: enough for the finest launch shape (zc = 1), 4 values
  const Shape sh = stencil_shape(ctx->g, 1);
  int64_t nparts = (int64_t)sh.nblocks() * 4;
  if (nparts < 4 * 152 * 16) nparts = 4 * 152 * 16;
  if ((rc = dalloc(&ctx->partials, nparts))) return fail(rc);
  if (cudaMalloc(&ctx->st, sizeof(CgState)) != cudaSuccess ||
      cudaMalloc(&ctx->st32, sizeof(CgState)) != cudaSuccess)
    return fail(SBM_ERR_NOMEM);
  cudaMemset(ctx->st, 0, sizeof(CgState));
  cudaMemset(ctx->st32, 0, sizeof(CgState));
  if ((rc = dalloc(&ctx->d_scal, 64 + 5 * SBM_TBL_MAX))) return fail(rc);
  if (cudaMallocHost(&ctx->h_st, 4 * sizeof(CgState)) != cudaSuccess ||
      cudaMallocHost(&ctx->h_scal, sizeof(double) * (64 + 5 * SBM_TBL_MAX)) != cudaSuccess)
    return fail(SBM_ERR_NOMEM);
  if (cudaDeviceSynchronize() != cudaSuccess) return fail(SBM_ERR_CUDA);
  *out = ctx;
  return SBM_OK;
}

int sbm_ctx_destroy(sbm_ctx* ctx) {
  if (!ctx) return SBM_ERR_ARG;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  release_graphs(ctx);
  net_pc_release(ctx);
  for (int f = 0; f < SBM_F_COUNT; ++f) cudaFree(ctx->f[f]);
  double* d[] = {ctx->hk_kap, ctx->hk_pce, ctx->hk_pcc, ctx->hk_gen, ctx->dab, ctx->dab1,
                 ctx->mu,     ctx->mb,     ctx->pmn,    ctx->rhe,    ctx->rxc, ctx->kfw,
                 ctx->kbw,    ctx->ppo,    ctx->peo,    ctx->tmp,    ctx->r64, ctx->p64,
                 ctx->q64,    ctx->d64,    ctx->partials, ctx->d_scal,
                 ctx->fc64};
  for (double* q : d) cudaFree(q);
  float* fl[] = {ctx->hk32,   ctx->dg32,   ctx->r32,    ctx->p32,   ctx->q32,
                 ctx->x32,    ctx->z32,    ctx->rold32, ctx->hklo32, ctx->dglo32,
                 ctx->r0hi32, ctx->r0lo32, ctx->dhi32,  ctx->dlo32};
  for (float* q : fl) cudaFree(q);
  cudaFree(ctx->st);
  cudaFree(ctx->st32);
  if (ctx->h_st) cudaFreeHost(ctx->h_st);
  if (ctx->h_scal) cudaFreeHost(ctx->h_scal);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  for (cudaEvent_t e : ctx->evq)
    if (e) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return SBM_OK;
}

int sbm_ctx_set_params(sbm_ctx* ctx, const sbm_params* p) {
  if (!ctx || !p || p->tbl_n < 2 || p->tbl_n > SBM_TBL_MAX) return SBM_ERR_ARG;
  ctx->p = *p;
  if (ctx->hk_kap) return upload_tables(ctx);
  return SBM_OK;
}

int sbm_ctx_set_tuning(sbm_ctx* ctx, int zc64, int zc32, int chunk, double delta, int flags) {
  if (!ctx || zc64 < 0 || zc32 < 0 || chunk < 0 || zc64 > 64 || zc32 > 64 || chunk > 1024 ||
      !(delta >= 0.0 && delta < 1.0) ||
      (flags & ~(SBM_TUNE_NO_TMA | SBM_TUNE_PC_ADDITIVE | SBM_TUNE_HOST_LOOP)))
    return SBM_ERR_ARG;
  const int no_tma = (flags & SBM_TUNE_NO_TMA) ? 1 : 0;
  const int pc_add = (flags & SBM_TUNE_PC_ADDITIVE) ? 1 : 0;
  if (zc64 != ctx->zc64 || zc32 != ctx->zc32 || chunk != ctx->chunk || no_tma != ctx->no_tma ||
      pc_add != ctx->pc_additive) {
    cudaStreamSynchronize(ctx->stream);
    release_graphs(ctx);
  }
  ctx->zc64 = zc64;
  ctx->zc32 = zc32;
  ctx->chunk = chunk;
  ctx->inner_tol = delta;
  ctx->no_tma = no_tma;
  ctx->pc_additive = pc_add;
  ctx->host_loop = (flags & SBM_TUNE_HOST_LOOP) ? 1 : 0;
  return SBM_OK;
}

int sbm_ctx_stream(sbm_ctx* ctx, void** stream) {
  if (!ctx || !stream) return SBM_ERR_ARG;
  *stream = (void*)ctx->stream;
  return SBM_OK;
}

int sbm_ctx_sync(sbm_ctx* ctx) {
  if (!ctx) return SBM_ERR_ARG;
  SBM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SBM_OK;
}

int sbm_field_ptr(sbm_ctx* ctx, int field, double** dptr) {
  if (!ctx || !dptr || field < 0 || field >= SBM_F_COUNT) return SBM_ERR_ARG;
  *dptr = ctx->f[field];
  return SBM_OK;
}

int sbm_upload(sbm_ctx* ctx, int field, const double* h, int haloed) {
  if (!ctx || !h || field < 0 || field >= SBM_F_COUNT) return SBM_ERR_ARG;
  const Geo& g = ctx->g;
  if (haloed) {
    SBM_CUDA_TRY(cudaMemcpyAsync(ctx->f[field], h, sizeof(double) * g.nh, cudaMemcpyHostToDevice,
                                 ctx->stream));
  } else {
    // one 2D copy per z plane: interior rows j = 1..nx of ny doubles each
    for (int k = 1; k <= g.nz; ++k) {
      SBM_CUDA_TRY(cudaMemcpy2DAsync(ctx->f[field] + g.ix(1, 1, k), sizeof(double) * g.sx,
                                     h + (size_t)g.ny * g.nx * (k - 1), sizeof(double) * g.ny,
                                     sizeof(double) * g.ny, g.nx, cudaMemcpyHostToDevice,
                                     ctx->stream));
    }
  }
  SBM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SBM_OK;
}

int sbm_download(sbm_ctx* ctx, int field, double* h, int haloed) {
  if (!ctx || !h || field < 0 || field >= SBM_F_COUNT) return SBM_ERR_ARG;
  const Geo& g = ctx->g;
  if (haloed) {
    SBM_CUDA_TRY(cudaMemcpyAsync(h, ctx->f[field], sizeof(double) * g.nh, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  } else {
    for (int k = 1; k <= g.nz; ++k) {
      SBM_CUDA_TRY(cudaMemcpy2DAsync(h + (size_t)g.ny * g.nx * (k - 1), sizeof(double) * g.ny,
                                     ctx->f[field] + g.ix(1, 1, k), sizeof(double) * g.sx,
                                     sizeof(double) * g.ny, g.nx, cudaMemcpyDeviceToHost,
                                     ctx->stream));
    }
  }
  SBM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SBM_OK;
}

// ------------------------------------------------------------ snapshots
//
// A snapshot is a header followed by whole halo-padded FP64 fields: the 14
// public fields and, once the electrochemical state exists, the 12 step
// buffers (half coefficients of the kappa / pce / pcc operators, Dab, mu,
// mobility, CnE right-hand side, reaction coefficients, forward / backward
// rate constants and the previous phP / phE).  Everything a later time step
// or solve reads from the context is in it, so a restored context continues
// bit for bit; the CG work vectors are not, since every solve starts them
// afresh.
namespace {
constexpr char kSnapMagic[8] = {'S', 'B', 'M', 'S', 'N', 'A', 'P', '1'};
constexpr int kStepBufs = 12;

struct SnapHeader {
  char magic[8];
  int32_t version;
  int32_t ny, nx, nz;
  int32_t nfields;    // field records after the header
  int32_t step_work;  // 1 when the step buffers follow the public fields
  int64_t nh;         // doubles per field record
  sbm_params p;
  sbm_scalars sc;
};

constexpr size_t kSnapHead = (sizeof(SnapHeader) + 63) / 64 * 64;

int step_bufs(sbm_ctx* ctx, double** out) {
  double* b[kStepBufs] = {ctx->hk_kap, ctx->hk_pce, ctx->hk_pcc, ctx->dab, ctx->mu,  ctx->mb,
                          ctx->rhe,    ctx->rxc,    ctx->kfw,    ctx->kbw, ctx->ppo, ctx->peo};
  for (int i = 0; i < kStepBufs; ++i) out[i] = b[i];
  return ctx->hk_kap ? kStepBufs : 0;
}
}  // namespace

int sbm_ctx_get_params(const sbm_ctx* ctx, sbm_params* p) {
  if (!ctx || !p) return SBM_ERR_ARG;
  *p = ctx->p;
  return SBM_OK;
}

int sbm_ctx_get_scalars(const sbm_ctx* ctx, sbm_scalars* s) {
  if (!ctx || !s) return SBM_ERR_ARG;
  *s = ctx->sc;
  return SBM_OK;
}

int sbm_ctx_snapshot_size(sbm_ctx* ctx, size_t* bytes) {
  if (!ctx || !bytes) return SBM_ERR_ARG;
  const int nf = SBM_F_COUNT + (ctx->hk_kap ? kStepBufs : 0);
  *bytes = kSnapHead + (size_t)nf * sizeof(double) * (size_t)ctx->g.nh;
  return SBM_OK;
}

int sbm_ctx_snapshot(sbm_ctx* ctx, void* buf, size_t bytes) {
  size_t need = 0;
  if (!ctx || !buf || sbm_ctx_snapshot_size(ctx, &need) || bytes < need) return SBM_ERR_ARG;
  double* sb[kStepBufs];
  const int ns = step_bufs(ctx, sb);
  SnapHeader h;
  memset(&h, 0, sizeof(h));
  memcpy(h.magic, kSnapMagic, sizeof(h.magic));
  h.version = 2;
  h.ny = ctx->g.ny;
  h.nx = ctx->g.nx;
  h.nz = ctx->g.nz;
  h.nfields = SBM_F_COUNT + ns;
  h.step_work = ns ? 1 : 0;
  h.nh = ctx->g.nh;
  h.p = ctx->p;
  h.sc = ctx->sc;
  char* out = static_cast<char*>(buf);
  memset(out, 0, kSnapHead);
  memcpy(out, &h, sizeof(h));
  const size_t fb = sizeof(double) * (size_t)ctx->g.nh;
  for (int i = 0; i < h.nfields; ++i) {
    const double* src = i < SBM_F_COUNT ? ctx->f[i] : sb[i - SBM_F_COUNT];
    SBM_CUDA_TRY(cudaMemcpyAsync(out + kSnapHead + (size_t)i * fb, src, fb,
                                 cudaMemcpyDeviceToHost, ctx->stream));
  }
  SBM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SBM_OK;
}

int sbm_ctx_restore(sbm_ctx* ctx, const void* buf, size_t bytes) {
  if (!ctx || !buf || bytes < kSnapHead) return SBM_ERR_ARG;
  SnapHeader h;
  memcpy(&h, buf, sizeof(h));
  if (memcmp(h.magic, kSnapMagic, sizeof(h.magic)) != 0 || h.version != 2 ||
      h.ny != ctx->g.ny || h.nx != ctx->g.nx || h.nz != ctx->g.nz || h.nh != ctx->g.nh ||
      h.nfields != SBM_F_COUNT + (h.step_work ? kStepBufs : 0) || h.p.tbl_n < 2 ||
      h.p.tbl_n > SBM_TBL_MAX)
    return SBM_ERR_ARG;
  const size_t fb = sizeof(double) * (size_t)ctx->g.nh;
  if (bytes < kSnapHead + (size_t)h.nfields * fb) return SBM_ERR_ARG;
  SBM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  release_graphs(ctx);
  ctx->p = h.p;
  ctx->sc = h.sc;
  if (h.step_work) {
    int rc = ensure_step_work(ctx);
    if (rc) return rc;
  }
  double* sb[kStepBufs];
  step_bufs(ctx, sb);
  const char* in = static_cast<const char*>(buf);
  for (int i = 0; i < h.nfields; ++i) {
    double* dst = i < SBM_F_COUNT ? ctx->f[i] : sb[i - SBM_F_COUNT];
    SBM_CUDA_TRY(cudaMemcpyAsync(dst, in + kSnapHead + (size_t)i * fb, fb,
                                 cudaMemcpyHostToDevice, ctx->stream));
  }
  if (ctx->hk_kap) {
    int rc = upload_tables(ctx);
    if (rc) return rc;
  }
  SBM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SBM_OK;
}

int sbm_setup_domain(sbm_ctx* ctx, const float* dist_p, const float* dist_e, double zeta,
                     double cnp0, double cne0, double cr, sbm_scalars* s) {
  if (!ctx || !dist_p || !dist_e || !(zeta > 0.0) || !(cr != 0.0)) return SBM_ERR_ARG;
  int rc = ensure_step_work(ctx);
  if (rc) return rc;
  return step_setup(ctx, dist_p, dist_e, zeta, cnp0, cne0, cr, s);
}

int sbm_cg_solve(sbm_ctx* ctx, int op, int bc_x0, int bc_x1, double scale, double tol, int max_it,
                 int stop_rule, int precision, int precond, int* iters, double* final_res,
                 float* ms) {
  if (!ctx || max_it < 1 || !(tol >= 0.0)) return SBM_ERR_ARG;
  if (stop_rule < 0 || stop_rule > 2 || precision < 0 || precision > 1) return SBM_ERR_ARG;
  if (precond != SBM_PC_NONE && precond != SBM_PC_JACOBI && precond != SBM_PC_LEARNED)
    return SBM_ERR_ARG;
  if ((bc_x0 != SBM_BC_COPY && bc_x0 != SBM_BC_ZERO) || (bc_x1 != SBM_BC_COPY && bc_x1 != SBM_BC_ZERO))
    return SBM_ERR_ARG;
  const Geo& g = ctx->g;
  SolveSpec sp{};
  sp.op = op;
  sp.precision = precision;
  sp.precond = precond;
  sp.stop_rule = stop_rule;
  sp.tol = tol;
  sp.max_it = max_it;
  sp.rhs = ctx->f[SBM_F_RHS];
  const double idx2 = 1.0 / (ctx->p.dx * ctx->p.dx);
  (void)g;
  if (op == SBM_OP_GENERIC || op == SBM_OP_GENERIC_DIAG) {
    int rc = generic_spec(ctx, op, bc_x0, bc_x1, scale, tol, max_it, stop_rule, precision, precond,
                          &sp);
    if (rc) return rc;
  } else {
    if (!ctx->hk_kap) return SBM_ERR_STATE;
    if (op == SBM_OP_CNE) {
      sp.form = 1; sp.bcx0 = SBM_BC_COPY; sp.bcx1 = SBM_BC_COPY; sp.scale = scale;
      sp.hk64 = ctx->hk_pce; sp.diag64 = ctx->f[SBM_F_PSE];
      sp.x = ctx->f[SBM_F_CNE]; sp.w = ctx->f[SBM_F_PSE]; sp.wsum = ctx->sc.tPE;
    } else if (op == SBM_OP_PHP) {
      sp.form = 0; sp.bcx0 = SBM_BC_COPY; sp.bcx1 = SBM_BC_ZERO; sp.scale = idx2;
      sp.hk64 = ctx->hk_kap; sp.x = ctx->f[SBM_F_PHP]; sp.w = ctx->f[SBM_F_PSP];
      sp.wsum = ctx->sc.tPP;
    } else if (op == SBM_OP_PHE) {
      sp.form = 0; sp.bcx0 = SBM_BC_ZERO; sp.bcx1 = SBM_BC_COPY; sp.scale = idx2;
      sp.hk64 = ctx->hk_pcc; sp.x = ctx->f[SBM_F_PHE]; sp.w = ctx->f[SBM_F_PSE];
      sp.wsum = ctx->sc.tPE;
    } else {
      return SBM_ERR_ARG;
    }
  }
  SolveResult r{};
  int rc = solve(ctx, sp, &r);
  if (rc) return rc;
  if (op == SBM_OP_GENERIC || op == SBM_OP_GENERIC_DIAG) {
    if ((rc = ghost_after_solve(ctx, sp.x, sp.bcx0, sp.bcx1))) return rc;
    SBM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  }
  if (iters) *iters = r.iters;
  if (final_res) *final_res = r.final_res;
  if (ms) *ms = r.ms;
  return r.status;
}

int sbm_ctx_last_precond(const sbm_ctx* ctx) { return ctx ? ctx->last_precond : SBM_ERR_ARG; }

int sbm_learned_pc_apply(sbm_ctx* ctx, int bc_x0, int bc_x1, double scale, const double* r,
                         double* z) {
  return sbm_learned_pc_apply_op(ctx, SBM_OP_GENERIC, bc_x0, bc_x1, scale, r, z);
}

int sbm_learned_pc_apply_op(sbm_ctx* ctx, int op, int bc_x0, int bc_x1, double scale,
                            const double* r, double* z) {
  if (!ctx || !r || !z || (op != SBM_OP_GENERIC && op != SBM_OP_GENERIC_DIAG)) return SBM_ERR_ARG;
  SolveSpec sp{};
  int rc = generic_spec(ctx, op, bc_x0, bc_x1, scale, 1e-8, 1, SBM_STOP_REL_RES, SBM_PREC_MIXED,
                        SBM_PC_LEARNED, &sp);
  if (rc) return rc;
  return learned_pc_apply(ctx, sp, r, z);
}

}  // extern "C"

namespace sbm {
// Solve spec of the GENERIC / GENERIC_DIAG operator (coefficient, diagonal,
// unknown, right-hand side and weight from the context's public fields);
// also halves the coefficient.
int generic_spec(sbm_ctx* ctx, int op, int bc_x0, int bc_x1, double scale, double tol, int max_it,
                 int stop_rule, int precision, int precond, SolveSpec* out) {
  const Geo& g = ctx->g;
  if (op != SBM_OP_GENERIC && op != SBM_OP_GENERIC_DIAG) return SBM_ERR_ARG;
  SolveSpec sp{};
  sp.op = op;
  sp.precision = precision;
  sp.precond = precond;
  sp.stop_rule = stop_rule;
  sp.tol = tol;
  sp.max_it = max_it;
  sp.rhs = ctx->f[SBM_F_RHS];
  SBM_CUDA_TRY(launch_half(g, ctx->f[SBM_F_COEF], ctx->hk_gen, ctx->stream));
  sp.hk64 = ctx->hk_gen;
  sp.form = op == SBM_OP_GENERIC_DIAG ? 1 : 0;
  sp.diag64 = op == SBM_OP_GENERIC_DIAG ? ctx->f[SBM_F_DIAG] : nullptr;
  sp.scale = scale;
  sp.bcx0 = bc_x0;
  sp.bcx1 = bc_x1;
  sp.x = ctx->f[SBM_F_X];
  sp.w = ctx->f[SBM_F_WEIGHT];
  sp.wsum = 1.0;
  if (stop_rule != SBM_STOP_REL_RES) {
    // sum of the weight over the interior (host side, once per call)
    const size_t n = (size_t)g.nh;
    double* hw = (double*)malloc(sizeof(double) * n);
    if (!hw) return SBM_ERR_NOMEM;
    int rc = sbm_download(ctx, SBM_F_WEIGHT, hw, 1);
    double ws = 0.0;
    for (int k = 1; k <= g.nz; ++k)
      for (int j = 1; j <= g.nx; ++j)
        for (int i = 1; i <= g.ny; ++i) ws += hw[g.ix(i, j, k)];
    free(hw);
    if (rc) return rc;
    sp.wsum = ws;
  }
  *out = sp;
  return SBM_OK;
}
}  // namespace sbm

extern "C" {

int sbm_bench_kernel(sbm_ctx* ctx, int which, int reps, float* ms_per_launch,
                     double* bytes_per_launch) {
  if (!ctx) return SBM_ERR_ARG;
  return bench_kernel(ctx, which, reps, ms_per_launch, bytes_per_launch);
}

int sbm_ch_step(sbm_ctx* ctx, double dt, sbm_scalars* s) {
  if (!ctx) return SBM_ERR_ARG;
  if (!ctx->hk_kap) return SBM_ERR_STATE;
  return step_ch(ctx, dt, s);
}

int sbm_cne_step(sbm_ctx* ctx, int iter, double dt, int precision, sbm_scalars* s) {
  if (!ctx || precision < 0 || precision > 1) return SBM_ERR_ARG;
  if (!ctx->hk_kap) return SBM_ERR_STATE;
  return step_cne(ctx, iter, dt, precision, s);
}

int sbm_bv_update(sbm_ctx* ctx, int precision, sbm_scalars* s) {
  if (!ctx || precision < 0 || precision > 1) return SBM_ERR_ARG;
  if (!ctx->hk_kap) return SBM_ERR_STATE;
  return step_bv(ctx, precision, s);
}

int sbm_voltage_step(sbm_ctx* ctx, double dt, double vsr, sbm_scalars* s) {
  if (!ctx) return SBM_ERR_ARG;
  if (!ctx->hk_kap) return SBM_ERR_STATE;
  return step_voltage(ctx, dt, vsr, s);
}

int sbm_time_step(sbm_ctx* ctx, int iter, double dt, double vsr, int precision, sbm_scalars* s) {
  if (!ctx || precision < 0 || precision > 1) return SBM_ERR_ARG;
  if (!ctx->hk_kap) return SBM_ERR_STATE;
  int rc = step_ch(ctx, dt, nullptr);
  if (rc) return rc;
  if ((rc = step_cne(ctx, iter, dt, precision, nullptr))) return rc;
  if ((rc = step_bv(ctx, precision, nullptr))) return rc;
  if ((rc = step_voltage(ctx, dt, vsr, nullptr))) return rc;
  if (s) *s = ctx->sc;
  return SBM_OK;
}

}  // extern "C"

// ----------------------------------------------------- stateless kernels
// Each allocates its device buffers per call, runs on a stream of its own,
// and copies the result back.

namespace {
struct DevBufs {
  std::vector<void*> ptrs;
  ~DevBufs() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  T* get(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(T) * (n ? n : 1)) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return (T*)p;
  }
};
struct Stream {
  cudaStream_t s = nullptr;
  Stream() { cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking); }
  ~Stream() {
    if (s) cudaStreamDestroy(s);
  }
};
}  // namespace

extern "C" {

int sbm_table_lookup(int64_t n, int sz, const double* cord, const double* vals, const double* cn,
                     double* fn) {
  if (n < 0 || sz < 2 || sz > SBM_TBL_MAX || !cord || !vals || (n > 0 && (!cn || !fn)))
    return SBM_ERR_ARG;
  if (n == 0) return SBM_OK;
  DevBufs b;
  Stream st;
  double *dx = b.get<double>(sz), *dv = b.get<double>(sz), *dc = b.get<double>(n),
         *df = b.get<double>(n);
  if (!dx || !dv || !dc || !df || !st.s) return SBM_ERR_NOMEM;
  SBM_CUDA_TRY(cudaMemcpyAsync(dx, cord, sizeof(double) * sz, cudaMemcpyHostToDevice, st.s));
  SBM_CUDA_TRY(cudaMemcpyAsync(dv, vals, sizeof(double) * sz, cudaMemcpyHostToDevice, st.s));
  SBM_CUDA_TRY(cudaMemcpyAsync(dc, cn, sizeof(double) * n, cudaMemcpyHostToDevice, st.s));
  int rc = table_lookup_dev(st.s, n, sz, dx, dv, dc, df);
  if (rc) return rc;
  SBM_CUDA_TRY(cudaMemcpyAsync(fn, df, sizeof(double) * n, cudaMemcpyDeviceToHost, st.s));
  SBM_CUDA_TRY(cudaStreamSynchronize(st.s));
  return SBM_OK;
}

namespace {
// Arguments of the level-set geometry entry points; false when the stacked
// grid or the tunnel loop would leave the reference's arrays.
bool ls_args_ok(const double* vox, int yo, int xo, int zo, int yg, int zg, int xoff, int nthick,
                double tr, const double* ds) {
  if (!vox || !ds || yo < 1 || xo < 1 || zo < 1 || yg < 1 || zg < 1 || xoff < 0 || nthick < 1)
    return false;
  if (yg > yo || zg > xo || !(tr == tr)) return false;
  const int64_t xg = xoff + (int64_t)nthick * zo;
  if (xg > (1 << 24)) return false;
  return (xg - 1) + (int64_t)zo * (zg - 1) < (int64_t)zo * xo;
}
}  // namespace

int sbm_ls_geometry(const double* vox, int yo, int xo, int zo, int yg, int zg, int xoff,
                    int nthick, double tr, double* ds) {
  if (!ls_args_ok(vox, yo, xo, zo, yg, zg, xoff, nthick, tr, ds)) return SBM_ERR_ARG;
  const Geo g = make_geo(yg, xoff + nthick * zo, zg);
  const size_t nv = (size_t)yo * xo * zo;
  DevBufs b;
  Stream st;
  double *dv = b.get<double>(nv), *dd = b.get<double>(g.nh);
  if (!dv || !dd || !st.s) return SBM_ERR_NOMEM;
  SBM_CUDA_TRY(cudaMemcpyAsync(dv, vox, sizeof(double) * nv, cudaMemcpyHostToDevice, st.s));
  int rc = ls_geometry_dev(st.s, g, dv, yo, xo, zo, xoff, tr, dd);
  if (rc) return rc;
  SBM_CUDA_TRY(cudaMemcpyAsync(ds, dd, sizeof(double) * g.nh, cudaMemcpyDeviceToHost, st.s));
  SBM_CUDA_TRY(cudaStreamSynchronize(st.s));
  return SBM_OK;
}

int sbm_ls_frontend(const double* vox, int yo, int xo, int zo, int yg, int zg, int xoff,
                    int nthick, double tr, int ac_iters, int lit, double dt, double* ds) {
  if (!ls_args_ok(vox, yo, xo, zo, yg, zg, xoff, nthick, tr, ds) || ac_iters < 0 || lit < 0)
    return SBM_ERR_ARG;
  const Geo g = make_geo(yg, xoff + nthick * zo, zg);
  const size_t nv = (size_t)yo * xo * zo;
  DevBufs b;
  Stream st;
  double *dv = b.get<double>(nv), *dd = b.get<double>(g.nh), *dg = b.get<double>(g.nh),
         *dt2 = b.get<double>(g.nh);
  if (!dv || !dd || !dg || !dt2 || !st.s) return SBM_ERR_NOMEM;
  SBM_CUDA_TRY(cudaMemcpyAsync(dv, vox, sizeof(double) * nv, cudaMemcpyHostToDevice, st.s));
  int rc = ls_frontend_dev(st.s, g, dv, yo, xo, zo, xoff, tr, ac_iters, lit, dt, dd, dg, dt2);
  if (rc) return rc;
  SBM_CUDA_TRY(cudaMemcpyAsync(ds, dd, sizeof(double) * g.nh, cudaMemcpyDeviceToHost, st.s));
  SBM_CUDA_TRY(cudaStreamSynchronize(st.s));
  return SBM_OK;
}

namespace {
// Interior (py*px*pz, Fortran order) host array into the interior of a
// halo-padded device array, one 2-D copy per z plane.
int upload_interior(const Geo& g, const double* h, double* d, cudaStream_t s) {
  for (int k = 1; k <= g.nz; ++k)
    SBM_CUDA_TRY(cudaMemcpy2DAsync(d + g.ix(1, 1, k), sizeof(double) * g.sx,
                                   h + (size_t)g.ny * g.nx * (k - 1), sizeof(double) * g.ny,
                                   sizeof(double) * g.ny, g.nx, cudaMemcpyHostToDevice, s));
  return SBM_OK;
}

// 0.5*(1.0 + TANH(d/width)) on the host with the C library's tanh (the
// oracle's), so the thresholds the sweeps test see the same psi.
std::vector<double> psi_host(const double* dist, size_t n, double width) {
  std::vector<double> v(n);
  for (size_t c = 0; c < n; ++c) v[c] = 0.5 * (1.0 + std::tanh(dist[c] / width));
  return v;
}
}  // namespace

int sbm_connectivity(int py, int px, int pz, const double* dist, double width, int term,
                     double* cn_solid, double* cn_elec) {
  if (py < 1 || px < 1 || pz < 1 || !dist || !cn_solid || !cn_elec || term < 1 ||
      !(width != 0.0))
    return SBM_ERR_ARG;
  const Geo g = make_geo(py, px, pz);
  const size_t n = (size_t)py * px * pz;
  std::vector<double> psi = psi_host(dist, n, width);
  DevBufs b;
  Stream st;
  double *dp = b.get<double>(g.nh), *dc = b.get<double>(g.nh), *dt2 = b.get<double>(g.nh);
  if (!dp || !dc || !dt2 || !st.s) return SBM_ERR_NOMEM;
  int rc = upload_interior(g, psi.data(), dp, st.s);
  if (!rc) rc = allen_cahn_dev(st.s, g, dp, dt2, 0);  // NoGrdBc3D fill, AD:88-97
  if (rc) return rc;
  for (int phase = 0; phase < 2; ++phase) {
    if (phase == 1) {  // AD:175: interior 1 - psi, ghosts keep the solid values
      for (double& v : psi) v = 1.0e0 - v;
      if ((rc = upload_interior(g, psi.data(), dp, st.s))) return rc;
    }
    SBM_CUDA_TRY(cudaMemsetAsync(dc, 0, sizeof(double) * g.nh, st.s));
    if ((rc = accdiff_dev(st.s, g, dp, dc, dt2, term, phase == 0 ? 1 : 0))) return rc;
    SBM_CUDA_TRY(cudaMemcpyAsync(phase == 0 ? cn_solid : cn_elec, dc, sizeof(double) * g.nh,
                                 cudaMemcpyDeviceToHost, st.s));
    SBM_CUDA_TRY(cudaStreamSynchronize(st.s));
  }
  return SBM_OK;
}

int sbm_rm_ucnct(int py, int px, int pz, const double* dist, const double* cn_solid,
                 const double* cn_elec, int lit, double* d_solid, double* d_elec) {
  if (py < 1 || px < 1 || pz < 1 || !dist || !cn_solid || !cn_elec || !d_solid || !d_elec ||
      lit < 0)
    return SBM_ERR_ARG;
  const Geo g = make_geo(py, px, pz);
  const size_t n = (size_t)py * px * pz;
  std::vector<double> psa = psi_host(dist, n, 1.0);  // RM:70
  DevBufs b;
  Stream st;
  double *da = b.get<double>(g.nh), *dc = b.get<double>(g.nh), *dd = b.get<double>(g.nh),
         *dg = b.get<double>(g.nh), *dt2 = b.get<double>(g.nh);
  if (!da || !dc || !dd || !dg || !dt2 || !st.s) return SBM_ERR_NOMEM;
  SBM_CUDA_TRY(cudaMemsetAsync(da, 0, sizeof(double) * g.nh, st.s));
  SBM_CUDA_TRY(cudaMemsetAsync(dc, 0, sizeof(double) * g.nh, st.s));
  const double dt = (double)1.0e-1f;  // RM:236, dt = 1.0e-1 REAL(4)
  int rc;
  for (int phase = 0; phase < 2; ++phase) {
    if (phase == 1)
      for (double& v : psa) v = 1.0e0 - v;  // RM:114
    if ((rc = upload_interior(g, psa.data(), da, st.s))) return rc;
    if ((rc = upload_interior(g, phase == 0 ? cn_solid : cn_elec, dc, st.s))) return rc;
    // RM:79-82 / :127-130 mask, :86-88 dsF = psB with NoGrdBc3D, :91-96 sign,
    // :99-100 reinitialisation from zero
    if ((rc = rm_mask_dev(st.s, g.nh, da, dc, dd))) return rc;
    if ((rc = allen_cahn_dev(st.s, g, dd, dt2, 0))) return rc;
    if ((rc = sign_dev(st.s, g.nh, dd, 0.5, dg))) return rc;
    SBM_CUDA_TRY(cudaMemsetAsync(dd, 0, sizeof(double) * g.nh, st.s));
    if ((rc = redist_dev(st.s, g, dg, dd, dt2, lit, dt))) return rc;
    SBM_CUDA_TRY(cudaMemcpyAsync(phase == 0 ? d_solid : d_elec, dd, sizeof(double) * g.nh,
                                 cudaMemcpyDeviceToHost, st.s));
    SBM_CUDA_TRY(cudaStreamSynchronize(st.s));
  }
  return SBM_OK;
}

int sbm_ls_frontend_device(const double* vox, int yo, int xo, int zo, int yg, int zg, int xoff,
                           int nthick, double tr, int ac_iters, int lit, double dt, double* ds,
                           double* sg, double* tmp, void* stream) {
  if (!ls_args_ok(vox, yo, xo, zo, yg, zg, xoff, nthick, tr, ds) || !sg || !tmp ||
      ac_iters < 0 || lit < 0)
    return SBM_ERR_ARG;
  const Geo g = make_geo(yg, xoff + nthick * zo, zg);
  return ls_frontend_dev(static_cast<cudaStream_t>(stream), g, vox, yo, xo, zo, xoff, tr,
                         ac_iters, lit, dt, ds, sg, tmp);
}

int sbm_redist(int lit, int py, int px, int pz, double dt, const double* sg, double* f) {
  if (lit < 0 || py < 1 || px < 1 || pz < 1 || !sg || !f) return SBM_ERR_ARG;
  const Geo g = make_geo(py, px, pz);
  DevBufs b;
  Stream st;
  double *ds = b.get<double>(g.nh), *df = b.get<double>(g.nh), *dt2 = b.get<double>(g.nh);
  if (!ds || !df || !dt2 || !st.s) return SBM_ERR_NOMEM;
  SBM_CUDA_TRY(cudaMemcpyAsync(ds, sg, sizeof(double) * g.nh, cudaMemcpyHostToDevice, st.s));
  SBM_CUDA_TRY(cudaMemcpyAsync(df, f, sizeof(double) * g.nh, cudaMemcpyHostToDevice, st.s));
  int rc = redist_dev(st.s, g, ds, df, dt2, lit, dt);
  if (rc) return rc;
  SBM_CUDA_TRY(cudaMemcpyAsync(f, df, sizeof(double) * g.nh, cudaMemcpyDeviceToHost, st.s));
  SBM_CUDA_TRY(cudaStreamSynchronize(st.s));
  return SBM_OK;
}

int sbm_allen_cahn(int iters, int py, int px, int pz, double* f) {
  if (iters < 0 || py < 1 || px < 1 || pz < 1 || !f) return SBM_ERR_ARG;
  const Geo g = make_geo(py, px, pz);
  DevBufs b;
  Stream st;
  double *df = b.get<double>(g.nh), *dt2 = b.get<double>(g.nh);
  if (!df || !dt2 || !st.s) return SBM_ERR_NOMEM;
  SBM_CUDA_TRY(cudaMemcpyAsync(df, f, sizeof(double) * g.nh, cudaMemcpyHostToDevice, st.s));
  int rc = allen_cahn_dev(st.s, g, df, dt2, iters);
  if (rc) return rc;
  SBM_CUDA_TRY(cudaMemcpyAsync(f, df, sizeof(double) * g.nh, cudaMemcpyDeviceToHost, st.s));
  SBM_CUDA_TRY(cudaStreamSynchronize(st.s));
  return SBM_OK;
}

int sbm_accdiff(int py, int px, int pz, const double* psi, double* cn, int term, int dirichlet_x) {
  if (py < 1 || px < 1 || pz < 1 || !psi || !cn || term < 1 ||
      (dirichlet_x != 0 && dirichlet_x != 1))
    return SBM_ERR_ARG;
  const Geo g = make_geo(py, px, pz);
  DevBufs b;
  Stream st;
  double *dp = b.get<double>(g.nh), *dc = b.get<double>(g.nh), *dt2 = b.get<double>(g.nh);
  if (!dp || !dc || !dt2 || !st.s) return SBM_ERR_NOMEM;
  SBM_CUDA_TRY(cudaMemcpyAsync(dp, psi, sizeof(double) * g.nh, cudaMemcpyHostToDevice, st.s));
  SBM_CUDA_TRY(cudaMemcpyAsync(dc, cn, sizeof(double) * g.nh, cudaMemcpyHostToDevice, st.s));
  int rc = accdiff_dev(st.s, g, dp, dc, dt2, term, dirichlet_x);
  if (rc) return rc;
  SBM_CUDA_TRY(cudaMemcpyAsync(cn, dc, sizeof(double) * g.nh, cudaMemcpyDeviceToHost, st.s));
  SBM_CUDA_TRY(cudaStreamSynchronize(st.s));
  return SBM_OK;
}

int sbm_rm_mask(int64_t n, const double* psA, const double* cn, double* psB) {
  if (n < 0 || (n > 0 && (!psA || !cn || !psB))) return SBM_ERR_ARG;
  if (n == 0) return SBM_OK;
  DevBufs b;
  Stream st;
  double *da = b.get<double>(n), *dc = b.get<double>(n), *db = b.get<double>(n);
  if (!da || !dc || !db || !st.s) return SBM_ERR_NOMEM;
  SBM_CUDA_TRY(cudaMemcpyAsync(da, psA, sizeof(double) * n, cudaMemcpyHostToDevice, st.s));
  SBM_CUDA_TRY(cudaMemcpyAsync(dc, cn, sizeof(double) * n, cudaMemcpyHostToDevice, st.s));
  int rc = rm_mask_dev(st.s, n, da, dc, db);
  if (rc) return rc;
  SBM_CUDA_TRY(cudaMemcpyAsync(psB, db, sizeof(double) * n, cudaMemcpyDeviceToHost, st.s));
  SBM_CUDA_TRY(cudaStreamSynchronize(st.s));
  return SBM_OK;
}

int sbm_sign(int64_t n, const double* ds, double thr, double* sg) {
  if (n < 0 || (n > 0 && (!ds || !sg))) return SBM_ERR_ARG;
  if (n == 0) return SBM_OK;
  DevBufs b;
  Stream st;
  double *dd = b.get<double>(n), *dg = b.get<double>(n);
  if (!dd || !dg || !st.s) return SBM_ERR_NOMEM;
  SBM_CUDA_TRY(cudaMemcpyAsync(dd, ds, sizeof(double) * n, cudaMemcpyHostToDevice, st.s));
  int rc = sign_dev(st.s, n, dd, thr, dg);
  if (rc) return rc;
  SBM_CUDA_TRY(cudaMemcpyAsync(sg, dg, sizeof(double) * n, cudaMemcpyDeviceToHost, st.s));
  SBM_CUDA_TRY(cudaStreamSynchronize(st.s));
  return SBM_OK;
}

}  // extern "C"
