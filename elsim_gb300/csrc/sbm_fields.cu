// sbm_fields.cu -- element-wise and stencil kernels of the electrochemical
// step, and the step stages themselves.
//
// Each stage follows one block of the reference time loop in
// SBMES_3D_MPI_CH_Gr_CONJG_VD_T05_01_BQ_hx3.f90 (SBMES below), in the same
// order, on device-resident FP64 fields:
//   set-up           SBMES:154-168, :173-176, :247-262, :273-291, :297-341
//   Cahn-Hilliard    SBMES:397-443
//   CnE solve        SBMES:461-572
//   potentials + BV  SBMES:577-812
//   voltage control  SBMES:826-835
// Global sums (the reference's MPI_ALLGATHER + SUM) are deterministic
// device reductions.  Ghost cells follow the single-rank BcMpiYZ plus the
// x-face lines: every y/z ghost is the nearest interior value; the x faces
// copy, take a value, or take the CnE flux condition.
#include <cmath>
#include <cstring>

#include "sbm_internal.cuh"

namespace sbm {

namespace {

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

dim3 flat(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return dim3((unsigned)b);
}

#define SBM_GRID_STRIDE(c, n) \
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < (n); c += (int64_t)gridDim.x * blockDim.x)

// Interior index t in [0, ny*nx*nz) -> padded index.
__device__ __forceinline__ int64_t interior_ix(const Geo& g, int64_t t, int* pi, int* pj, int* pk) {
  const int i = (int)(t % g.ny) + 1;
  const int64_t r = t / g.ny;
  const int j = (int)(r % g.nx) + 1;
  const int k = (int)(r / g.nx) + 1;
  if (pi) { *pi = i; *pj = j; *pk = k; }
  return g.ix(i, j, k);
}

// -------------------------------------------------------------- tables
// Tbl_Chk_Pln_3DA, SBMES:987-1028, bit-exact: clamp, lb = FLOOR(c/ditv)
// with the 0 -> 1 and sz -> sz-1 fix-ups, then the one-segment-left
// interpolation, with no fused multiply-add.
__device__ __forceinline__ double table_at(double t, int sz, const double* __restrict__ x,
                                           const double* __restrict__ v, double ditv) {
  if (t < 0.0) t = 1.0e-6;
  if (t > 1.0) t = 1.0;
  const double fl = floor(__ddiv_rn(t, ditv));
  int lb = (fl >= 0.0 && fl < 2147483647.0) ? (int)fl : 0;
  if (lb == 0) lb = 1;
  else if (lb == sz) lb = sz - 1;
  // Beyond the table the reference reads outside its arrays; stay inside.
  if (lb > sz - 1) lb = sz - 1;
  const double a = __ddiv_rn(__dsub_rn(t, x[lb - 1]), ditv);
  return __dadd_rn(v[lb - 1], __dmul_rn(a, __dsub_rn(v[lb], v[lb - 1])));
}

struct Tbl {
  const double* x;
  const double* v;
  int n;
};

__global__ void k_table(int64_t n, Tbl t, const double* __restrict__ cn, double* __restrict__ fn) {
  __shared__ double sx[SBM_TBL_MAX], sv[SBM_TBL_MAX];
  for (int q = threadIdx.x; q < t.n; q += blockDim.x) {
    sx[q] = t.x[q];
    sv[q] = t.v[q];
  }
  __syncthreads();
  const double ditv = __dsub_rn(sx[1], sx[0]);
  SBM_GRID_STRIDE(c, n) fn[c] = table_at(cn[c], t.n, sx, sv, ditv);
}

// ------------------------------------------------------------- ghosts
// x-face modes for k_ghost.
constexpr int GX_COPY = 0, GX_VALUE = 1, GX_FLUX = 2, GX_KEEP = 3;

struct GhostArgs {
  Geo g;
  double* f;
  int m0, m1;       // x = 0 and x = nx+1 modes
  double v0, v1;    // values for GX_VALUE
  int k0, k1;       // planes of the x lines
  const double* dab;  // GX_FLUX: Dab field
  double flux;        // GX_FLUX: (infx*t_minus)*dx
};

// One thread per ghost cell of the six faces.  Copies read interior cells
// only (the clamped index), so there is no ordering hazard.
__global__ void k_ghost(GhostArgs a) {
  const Geo g = a.g;
  const int64_t nzf = (int64_t)(g.ny + 2) * (g.nx + 2);  // one z face, all cells
  const int64_t nxf = (int64_t)(g.ny + 2) * g.nz;        // one x face, k in 1..nz
  const int64_t nyf = (int64_t)g.nx * g.nz;              // one y face, j in 1..nx, k in 1..nz
  const int64_t total = 2 * (nzf + nxf + nyf);
  SBM_GRID_STRIDE(t, total) {
    int i, j, k;
    int64_t u = t;
    if (u < 2 * nzf) {
      k = (u < nzf) ? 0 : g.nz + 1;
      u %= nzf;
      i = (int)(u % (g.ny + 2));
      j = (int)(u / (g.ny + 2));
    } else if ((u -= 2 * nzf) < 2 * nxf) {
      j = (u < nxf) ? 0 : g.nx + 1;
      u %= nxf;
      i = (int)(u % (g.ny + 2));
      k = (int)(u / (g.ny + 2)) + 1;
    } else {
      u -= 2 * nxf;
      i = (u < nyf) ? 0 : g.ny + 1;
      u %= nyf;
      j = (int)(u % g.nx) + 1;
      k = (int)(u / g.nx) + 1;
    }
    const int64_t c = g.ix(i, j, k);
    const int ci = clampi(i, 1, g.ny), ck = clampi(k, 1, g.nz);
    if (j == 0 || j == g.nx + 1) {
      const int m = (j == 0) ? a.m0 : a.m1;
      if (k < a.k0 || k > a.k1 || m == GX_KEEP) continue;
      if (m == GX_VALUE) {
        a.f[c] = (j == 0) ? a.v0 : a.v1;
      } else if (m == GX_FLUX) {
        // SBMES:558: infx*t_minus*dx/(0.5*(Dab(0)+Dab(1))) + CnE(1)
        const double den = 0.5 * (a.dab[c] + a.dab[g.ix(i, 1, k)]);
        a.f[c] = a.flux / den + a.f[g.ix(ci, 1, ck)];
      } else {
        a.f[c] = a.f[g.ix(ci, (j == 0) ? 1 : g.nx, ck)];
      }
    } else {
      a.f[c] = a.f[g.ix(ci, j, ck)];
    }
  }
}

// ---------------------------------------------------------- reductions
// out[slot] = sum over the interior of MODE 0: a*b, 1: a, 2: (a-b)^2*w.
template <int MODE>
__global__ void __launch_bounds__(256) k_sum(Geo g, const double* __restrict__ a,
                                             const double* __restrict__ b,
                                             const double* __restrict__ w, double* partials,
                                             unsigned int* counter, double* out) {
  double acc = 0.0;
  const int64_t n = g.ninterior();
  SBM_GRID_STRIDE(t, n) {
    const int64_t c = interior_ix(g, t, nullptr, nullptr, nullptr);
    if (MODE == 0) acc += a[c] * b[c];
    else if (MODE == 1) acc += a[c];
    else {
      const double d = a[c] - b[c];
      acc += (d * d) * w[c];
    }
  }
  double v[1] = {acc}, tot[1];
  if (grid_reduce<1>(v, partials, counter, tot))
    if (threadIdx.x == 0) *out = tot[0];
}

// ------------------------------------------------------------- set-up
// SBMES:154-168 (+ the single-rank halo, :173-176, and the floor of
// :247 / :258): psi = clamp(0.5(1 + tanh(d/zeta)), 0, 1) + floor, with
// every ghost the nearest interior value.  d is REAL(4), interior shape.
__global__ void k_psi(Geo g, const float* __restrict__ d, double zeta, double floor_,
                      double* __restrict__ psi) {
  SBM_GRID_STRIDE(c, g.nh) {
    const int i = (int)(c % g.sx);
    const int64_t r = c / g.sx;
    const int j = (int)(r % (g.nx + 2));
    const int k = (int)(r / (g.nx + 2));
    const int ci = clampi(i, 1, g.ny), cj = clampi(j, 1, g.nx), ck = clampi(k, 1, g.nz);
    double v = (double)d[(ci - 1) + (int64_t)g.ny * ((cj - 1) + (int64_t)g.nx * (ck - 1))];
    v = 0.5 * (1.0 + tanh(v / zeta));
    if (v < 0.0) v = 0.0;
    if (v > 1.0) v = 1.0;
    psi[c] = v + floor_;
  }
}

// SBMES:273-291.
__global__ void k_avp(Geo g, const double* __restrict__ psP, const double* __restrict__ psE,
                      double dx, double mask, double* __restrict__ avp, double* __restrict__ avpx) {
  SBM_GRID_STRIDE(t, g.ninterior()) {
    int i, j, k;
    const int64_t c = interior_ix(g, t, &i, &j, &k);
    double a = (psP[c + 1] - psP[c - 1]) / 2.0;
    double b = (psP[c + g.sx] - psP[c - g.sx]) / 2.0;
    double e = (psP[c + g.sz] - psP[c - g.sz]) / 2.0;
    const double gp = sqrt((a * a + b * b) + e * e);
    a = (psE[c + 1] - psE[c - 1]) / 2.0;
    b = (psE[c + g.sx] - psE[c - g.sx]) / 2.0;
    e = (psE[c + g.sz] - psE[c - g.sz]) / 2.0;
    const double ge = sqrt((a * a + b * b) + e * e);
    double v = sqrt(gp * ge);
    if (v < mask) v = 0.0;
    avp[c] = v;
    avpx[c] = v / dx;
  }
}

// Fills every cell of the padded array with constant v.
__global__ void k_fill(int64_t n, double* __restrict__ f, double v) {
  SBM_GRID_STRIDE(c, n) f[c] = v;
}

// out = s * in over the padded array (Kap = 3.3 psP, SBMES:324, stored halved).
__global__ void k_scale(int64_t n, const double* __restrict__ in, double s, double* __restrict__ out) {
  SBM_GRID_STRIDE(c, n) out[c] = (s * in[c]) * 0.5;
}

// ------------------------------------------------------- Cahn-Hilliard
struct ChArgs {
  Geo g;
  const double* cnp;
  double* mu;
  double* mb;
  double dx2, eps;
  Tbl tmu, tmb;
  int double_well;  // SBM_CH_DOUBLE_WELL: mu from the analytic well of height w
  double w;
};

// SBMES:398-405, :411: Lap in the reference's term order (x, y, z),
// mu = Tbl(c) - eps*Lap, Mb = DTbl(c); with the double well
// mu = w*2*c*(1-c)*(1-2*c) - eps*Lap (left to right).
__global__ void k_ch_mu(ChArgs a) {
  __shared__ double sx[SBM_TBL_MAX], smu[SBM_TBL_MAX], smb[SBM_TBL_MAX];
  for (int q = threadIdx.x; q < a.tmu.n; q += blockDim.x) {
    sx[q] = a.tmu.x[q];
    smu[q] = a.tmu.v[q];
    smb[q] = a.tmb.v[q];
  }
  __syncthreads();
  const double ditv = __dsub_rn(sx[1], sx[0]);
  const Geo g = a.g;
  SBM_GRID_STRIDE(t, g.ninterior()) {
    const int64_t c = interior_ix(g, t, nullptr, nullptr, nullptr);
    const double u = a.cnp[c];
    double l = a.cnp[c - g.sx] - 2.0 * u;
    l = l + a.cnp[c + g.sx];
    l = l + a.cnp[c - 1];
    l = l - 2.0 * u;
    l = l + a.cnp[c + 1];
    l = l + a.cnp[c - g.sz];
    l = l - 2.0 * u;
    l = l + a.cnp[c + g.sz];
    l = l / a.dx2;
    const double f0 = a.double_well ? (((a.w * 2.0) * u) * (1.0 - u)) * (1.0 - 2.0 * u)
                                     : table_at(u, a.tmu.n, sx, smu, ditv);
    a.mu[c] = f0 - a.eps * l;
    a.mb[c] = table_at(u, a.tmb.n, sx, smb, ditv);
  }
}

// SBMES:419-433: pmN = psP*Mb, DvC, masked update of CnP.
__global__ void k_ch_update(Geo g, const double* __restrict__ psP, const double* __restrict__ mb,
                            const double* __restrict__ mu, const double* __restrict__ rxn,
                            const double* __restrict__ avpx, double* __restrict__ cnp, double dt,
                            double dx2, double rho, double mask) {
  SBM_GRID_STRIDE(t, g.ninterior()) {
    const int64_t c = interior_ix(g, t, nullptr, nullptr, nullptr);
    const double pc = psP[c] * mb[c];
    const double mc = mu[c];
#define PM(o) (psP[c + (o)] * mb[c + (o)])
    double s = (0.5 * (PM(1) + pc)) * (mu[c + 1] - mc);
    s = s - (0.5 * (pc + PM(-1))) * (mc - mu[c - 1]);
    s = s + (0.5 * (PM(g.sx) + pc)) * (mu[c + g.sx] - mc);
    s = s - (0.5 * (pc + PM(-g.sx))) * (mc - mu[c - g.sx]);
    s = s + (0.5 * (PM(g.sz) + pc)) * (mu[c + g.sz] - mc);
    s = s - (0.5 * (pc + PM(-g.sz))) * (mc - mu[c - g.sz]);
#undef PM
    const double dvc = s / dx2;
    const double ps = psP[c];
    if (ps > mask) cnp[c] = cnp[c] + (dt * (dvc + (rxn[c] / rho) * avpx[c])) / ps;
  }
}

// ------------------------------------------------------------ CnE stage
// SBMES:461-462: RHS = psE*CEo - dt*Rxn*AvPx*t_minus (interior).
__global__ void k_cne_rhs(Geo g, const double* __restrict__ psE, const double* __restrict__ cne,
                          const double* __restrict__ rxn, const double* __restrict__ avpx,
                          double dt, double tm, double* __restrict__ rhs) {
  SBM_GRID_STRIDE(t, g.ninterior()) {
    const int64_t c = interior_ix(g, t, nullptr, nullptr, nullptr);
    rhs[c] = psE[c] * cne[c] - ((dt * rxn[c]) * avpx[c]) * tm;
  }
}

// Dab = pre*EXP(c0 - c1*c + c2*(c3*c)**2) over the padded array
// (SBMES:474, :579, :601); hk = 0.5*(psE*Dab) (MODE 0) or
// 0.5*(psE*CnE*Dab) (MODE 1); dab_out optional.
template <int MODE>
__global__ void k_dab(int64_t n, const double* __restrict__ cne, const double* __restrict__ psE,
                      double pre, double c0, double c1, double c2, double c3,
                      double* __restrict__ dab_out, double* __restrict__ hk) {
  SBM_GRID_STRIDE(c, n) {
    const double u = cne[c];
    const double q = c3 * u;
    const double d = pre * exp((c0 - c1 * u) + c2 * (q * q));
    if (dab_out) dab_out[c] = d;
    hk[c] = (MODE == 0 ? psE[c] * d : (psE[c] * u) * d) * 0.5;
  }
}

// interior: f = f - s
__global__ void k_shift(Geo g, double* __restrict__ f, double s) {
  SBM_GRID_STRIDE(t, g.ninterior()) {
    const int64_t c = interior_ix(g, t, nullptr, nullptr, nullptr);
    f[c] = f[c] - s;
  }
}

// ------------------------------------------------------- BV stage
// SBMES:614-622: ioC = Tbl_i0(CnP)*1e-3, OCV = Tbl_O(CnP), Kfw, Kbw.
struct KArgs {
  Geo g;
  const double* cnp;
  double* kfw;
  double* kbw;
  Tbl ti0, tocv;
  double i0s, frd, kfwc, ac;
};

__global__ void k_bv_coef(KArgs a) {
  __shared__ double sx[SBM_TBL_MAX], si[SBM_TBL_MAX], so[SBM_TBL_MAX];
  for (int q = threadIdx.x; q < a.ti0.n; q += blockDim.x) {
    sx[q] = a.ti0.x[q];
    si[q] = a.ti0.v[q];
    so[q] = a.tocv.v[q];
  }
  __syncthreads();
  const double ditv = __dsub_rn(sx[1], sx[0]);
  const Geo g = a.g;
  SBM_GRID_STRIDE(t, g.ninterior()) {
    const int64_t c = interior_ix(g, t, nullptr, nullptr, nullptr);
    const double u = a.cnp[c];
    const double ioc = table_at(u, a.ti0.n, sx, si, ditv) * a.i0s;
    const double ocv = table_at(u, a.tocv.n, sx, so, ditv);
    a.kfw[c] = (ioc / (a.frd * a.kfwc)) * exp(a.ac * ocv);
    a.kbw[c] = (ioc / (a.frd * u)) * exp(-(a.ac * ocv));
  }
}

// SBMES:631-645 (and :727 for the phE right-hand side, written later):
// masked Rxn / RxC, then RHS_P = -RxC*AvPx.
__global__ void k_bv_rxn(Geo g, const double* __restrict__ avp, const double* __restrict__ avpx,
                         const double* __restrict__ php, const double* __restrict__ phe,
                         const double* __restrict__ kfw, const double* __restrict__ kbw,
                         const double* __restrict__ cne, const double* __restrict__ cnp,
                         double* __restrict__ rxn, double* __restrict__ rxc,
                         double* __restrict__ rhs, double mask, double ac, double frd, int linear) {
  SBM_GRID_STRIDE(t, g.ninterior()) {
    const int64_t c = interior_ix(g, t, nullptr, nullptr, nullptr);
    if (avp[c] > mask) {
      const double dph = php[c] - phe[c];
      double r;
      if (linear)
        r = (kfw[c] * cne[c]) * (1.0 - ac * dph) - (kbw[c] * cnp[c]) * (1.0 + ac * dph);
      else
        r = (kfw[c] * cne[c]) * exp(-(ac * dph)) - (kbw[c] * cnp[c]) * exp(ac * dph);
      rxn[c] = r;
      rxc[c] = r * frd;
    }
    rhs[c] = -rxc[c] * avpx[c];
  }
}

// SBMES:727: RHS = Rxn*AvPx + RHE.
__global__ void k_phe_rhs(Geo g, const double* __restrict__ rxn, const double* __restrict__ avpx,
                          const double* __restrict__ rhe, double* __restrict__ rhs) {
  SBM_GRID_STRIDE(t, g.ninterior()) {
    const int64_t c = interior_ix(g, t, nullptr, nullptr, nullptr);
    rhs[c] = rxn[c] * avpx[c] + rhe[c];
  }
}

}  // namespace

// =============================================================== host side

static int ghost(sbm_ctx* ctx, double* f, int m0, double v0, int m1, double v1, int k0, int k1,
                 const double* dab = nullptr, double flux = 0.0) {
  const Geo& g = ctx->g;
  GhostArgs a{g, f, m0, m1, v0, v1, k0, k1, dab, flux};
  const int64_t total = 2 * ((int64_t)(g.ny + 2) * (g.nx + 2) + (int64_t)(g.ny + 2) * g.nz +
                             (int64_t)g.nx * g.nz);
  k_ghost<<<flat(total), 256, 0, ctx->stream>>>(a);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

// Ghost refresh of a solved unknown: Dirichlet (ZERO-rule) x faces keep
// their data, copy-rule faces and all y/z faces copy the edge.
int ghost_after_solve(sbm_ctx* ctx, double* f, int bcx0, int bcx1) {
  return ghost(ctx, f, bcx0 == SBM_BC_ZERO ? GX_KEEP : GX_COPY, 0.0,
               bcx1 == SBM_BC_ZERO ? GX_KEEP : GX_COPY, 0.0, 0, ctx->g.nz + 1);
}

static int ghost_copy(sbm_ctx* ctx, double* f) {
  return ghost(ctx, f, GX_COPY, 0, GX_COPY, 0, 0, ctx->g.nz + 1);
}

// Interior sum into device slot `slot` of ctx->d_scal.
template <int MODE>
static int dsum(sbm_ctx* ctx, const double* a, const double* b, const double* w, int slot) {
  const Geo& g = ctx->g;
  const int64_t n = g.ninterior();
  int64_t nb = (n + 255) / 256;
  if (nb > 152 * 8) nb = 152 * 8;
  k_sum<MODE><<<(unsigned)nb, 256, 0, ctx->stream>>>(g, a, b, w, ctx->partials,
                                                     &ctx->st->counter[6], ctx->d_scal + slot);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

// Copies slots [0, n) of the device scalars to the host and waits.
static int fetch_scalars(sbm_ctx* ctx, int n) {
  SBM_CUDA_TRY(cudaMemcpyAsync(ctx->h_scal, ctx->d_scal, sizeof(double) * n,
                               cudaMemcpyDeviceToHost, ctx->stream));
  SBM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SBM_OK;
}

// Device copies of the five tables live in ctx->d_scal beyond slot 64.
static Tbl tbl_dev(const sbm_ctx* ctx, int which) {
  // layout: x, mu, mb, i0, ocv each SBM_TBL_MAX, starting at slot 64
  const double* base = ctx->d_scal + 64;
  Tbl t;
  t.x = base;
  t.v = base + (size_t)(which + 1) * SBM_TBL_MAX;
  t.n = ctx->p.tbl_n;
  return t;
}

int upload_tables(sbm_ctx* ctx) {
  double* h = ctx->h_scal + 64;
  memcpy(h + 0 * SBM_TBL_MAX, ctx->p.tbl_x, sizeof(double) * SBM_TBL_MAX);
  memcpy(h + 1 * SBM_TBL_MAX, ctx->p.tbl_mu, sizeof(double) * SBM_TBL_MAX);
  memcpy(h + 2 * SBM_TBL_MAX, ctx->p.tbl_mb, sizeof(double) * SBM_TBL_MAX);
  memcpy(h + 3 * SBM_TBL_MAX, ctx->p.tbl_i0, sizeof(double) * SBM_TBL_MAX);
  memcpy(h + 4 * SBM_TBL_MAX, ctx->p.tbl_ocv, sizeof(double) * SBM_TBL_MAX);
  SBM_CUDA_TRY(cudaMemcpyAsync(ctx->d_scal + 64, h, sizeof(double) * 5 * SBM_TBL_MAX,
                               cudaMemcpyHostToDevice, ctx->stream));
  SBM_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SBM_OK;
}

int step_setup(sbm_ctx* ctx, const float* dp, const float* de, double zeta, double cnp0,
               double cne0, double cr, sbm_scalars* out) {
  const Geo& g = ctx->g;
  cudaStream_t s = ctx->stream;
  const sbm_params& p = ctx->p;
  const size_t nin = (size_t)g.ninterior();
  float* dd = nullptr;
  SBM_CUDA_TRY(cudaMalloc(&dd, sizeof(float) * nin));
  int rc = SBM_OK;
  do {
    if (cudaMemcpyAsync(dd, dp, sizeof(float) * nin, cudaMemcpyHostToDevice, s) != cudaSuccess) { rc = SBM_ERR_CUDA; break; }
    k_psi<<<flat(g.nh), 256, 0, s>>>(g, dd, zeta, 1.0e-7, ctx->f[SBM_F_PSP]);
    if (cudaMemcpyAsync(dd, de, sizeof(float) * nin, cudaMemcpyHostToDevice, s) != cudaSuccess) { rc = SBM_ERR_CUDA; break; }
    k_psi<<<flat(g.nh), 256, 0, s>>>(g, dd, zeta, 1.0e-6, ctx->f[SBM_F_PSE]);
    SBM_LAUNCHED(2);
    if (cudaStreamSynchronize(s) != cudaSuccess) { rc = SBM_ERR_CUDA; break; }
  } while (0);
  cudaFree(dd);
  if (rc) return rc;
  if ((rc = dsum<1>(ctx, ctx->f[SBM_F_PSP], nullptr, nullptr, 0))) return rc;   // :248
  if ((rc = dsum<1>(ctx, ctx->f[SBM_F_PSE], nullptr, nullptr, 1))) return rc;   // :260
  k_avp<<<flat(g.ninterior()), 256, 0, s>>>(g, ctx->f[SBM_F_PSP], ctx->f[SBM_F_PSE], p.dx,
                                            p.avp_mask, ctx->f[SBM_F_AVP], ctx->f[SBM_F_AVPX]);
  k_fill<<<flat(g.nh), 256, 0, s>>>(g.nh, ctx->f[SBM_F_CNP], cnp0);
  k_fill<<<flat(g.nh), 256, 0, s>>>(g.nh, ctx->f[SBM_F_CNE], cne0);
  k_fill<<<flat(g.nh), 256, 0, s>>>(g.nh, ctx->f[SBM_F_RXN], 0.0);
  k_fill<<<flat(g.nh), 256, 0, s>>>(g.nh, ctx->rxc, 0.0);
  k_fill<<<flat(g.nh), 256, 0, s>>>(g.nh, ctx->f[SBM_F_PHP], p.bvp);
  k_fill<<<flat(g.nh), 256, 0, s>>>(g.nh, ctx->f[SBM_F_PHE], p.bve);
  k_scale<<<flat(g.nh), 256, 0, s>>>(g.nh, ctx->f[SBM_F_PSP], p.kap_scale, ctx->hk_kap);
  SBM_LAUNCHED(9);
  if ((rc = dsum<0>(ctx, ctx->f[SBM_F_CNP], ctx->f[SBM_F_PSP], nullptr, 2))) return rc;
  if ((rc = fetch_scalars(ctx, 3))) return rc;
  sbm_scalars& sc = ctx->sc;
  memset(&sc, 0, sizeof(sc));
  sc.tPP = ctx->h_scal[0];
  sc.tPE = ctx->h_scal[1];
  sc.xrf = ctx->h_scal[2] / sc.tPP;                                    // :303
  sc.trgI = (((double)0.95f * sc.tPP) * p.rho) / (3600 / cr);         // :341
  sc.scrnt = sc.trgI;                                                  // :351
  sc.bve = p.bve;
  if (out) *out = sc;
  return SBM_OK;
}

int step_ch(sbm_ctx* ctx, double dt, sbm_scalars* out) {
  const Geo& g = ctx->g;
  cudaStream_t s = ctx->stream;
  const sbm_params& p = ctx->p;
  const double dx2 = p.dx * p.dx;
  ChArgs a{g,      ctx->f[SBM_F_CNP], ctx->mu, ctx->mb, dx2, p.eps, tbl_dev(ctx, 0), tbl_dev(ctx, 1),
           p.ch_mode == SBM_CH_DOUBLE_WELL, p.ch_w};
  k_ch_mu<<<flat(g.ninterior()), 256, 0, s>>>(a);
  SBM_LAUNCHED(1);
  int rc;
  if ((rc = ghost_copy(ctx, ctx->mb))) return rc;   // :407-409
  if ((rc = ghost_copy(ctx, ctx->mu))) return rc;   // :413-415
  k_ch_update<<<flat(g.ninterior()), 256, 0, s>>>(g, ctx->f[SBM_F_PSP], ctx->mb, ctx->mu,
                                                  ctx->f[SBM_F_RXN], ctx->f[SBM_F_AVPX],
                                                  ctx->f[SBM_F_CNP], dt, dx2, p.rho, p.ch_mask);
  SBM_LAUNCHED(1);
  if ((rc = ghost_copy(ctx, ctx->f[SBM_F_CNP]))) return rc;  // :436-438
  if ((rc = dsum<0>(ctx, ctx->f[SBM_F_CNP], ctx->f[SBM_F_PSP], nullptr, 2))) return rc;
  if ((rc = fetch_scalars(ctx, 3))) return rc;
  ctx->sc.xrf = ctx->h_scal[2] / ctx->sc.tPP;                  // :441-443
  if (out) *out = ctx->sc;
  return SBM_OK;
}

// Mixed-precision solves of the step use rel-res with this tolerance.
static const double kMixedStepTol = 1.0e-10;

static int step_solve(sbm_ctx* ctx, int op, int precision, double cne_scale, int* iters) {
  const sbm_params& p = ctx->p;
  SolveSpec sp{};
  sp.op = op;
  sp.precision = precision;
  sp.precond = SBM_PC_NONE;
  sp.rhs = ctx->rhs;
  if (op == SBM_OP_CNE) {
    sp.bcx0 = SBM_BC_COPY; sp.bcx1 = SBM_BC_COPY; sp.form = 1;
    sp.scale = cne_scale;  // dt/dx**2, SBMES:515
    sp.hk64 = ctx->hk_pce; sp.diag64 = ctx->f[SBM_F_PSE];
    sp.x = ctx->f[SBM_F_CNE]; sp.w = ctx->f[SBM_F_PSE]; sp.wsum = ctx->sc.tPE;
    sp.stop_rule = SBM_STOP_REF_RESID; sp.tol = p.crt_cne; sp.max_it = p.max_it_cne;
  } else if (op == SBM_OP_PHP) {
    sp.bcx0 = SBM_BC_COPY; sp.bcx1 = SBM_BC_ZERO; sp.form = 0;
    sp.scale = 1.0 / (p.dx * p.dx);
    sp.hk64 = ctx->hk_kap; sp.diag64 = nullptr;
    sp.x = ctx->f[SBM_F_PHP]; sp.w = ctx->f[SBM_F_PSP]; sp.wsum = ctx->sc.tPP;
    sp.stop_rule = SBM_STOP_REF_UPDATE; sp.tol = p.crt_php; sp.max_it = p.max_it_php;
  } else {
    sp.bcx0 = SBM_BC_ZERO; sp.bcx1 = SBM_BC_COPY; sp.form = 0;
    sp.scale = 1.0 / (p.dx * p.dx);
    sp.hk64 = ctx->hk_pcc; sp.diag64 = nullptr;
    sp.x = ctx->f[SBM_F_PHE]; sp.w = ctx->f[SBM_F_PSE]; sp.wsum = ctx->sc.tPE;
    sp.stop_rule = SBM_STOP_REF_UPDATE; sp.tol = p.crt_phe; sp.max_it = p.max_it_phe;
  }
  if (precision == SBM_PREC_MIXED) {
    sp.stop_rule = SBM_STOP_REL_RES;
    sp.tol = kMixedStepTol;
    // the learned preconditioner where a network is attached and suits the
    // grid and the operator, else Jacobi (the FP64 path keeps the
    // reference's plain CG)
    sp.precond = SBM_PC_LEARNED;
  }
  SolveResult r{};
  int rc = solve(ctx, sp, &r);
  if (rc) return rc;
  if (iters) *iters = r.iters;
  if (r.status == SBM_ERR_NONFINITE || r.status == SBM_ERR_BREAKDOWN) return r.status;
  return SBM_OK;  // the reference continues after hitting its iteration cap
}

int step_cne(sbm_ctx* ctx, int iter, double dt, int precision, sbm_scalars* out) {
  const Geo& g = ctx->g;
  cudaStream_t s = ctx->stream;
  const sbm_params& p = ctx->p;
  double* cne = ctx->f[SBM_F_CNE];
  k_cne_rhs<<<flat(g.ninterior()), 256, 0, s>>>(g, ctx->f[SBM_F_PSE], cne, ctx->f[SBM_F_RXN],
                                                ctx->f[SBM_F_AVPX], dt, p.t_minus, ctx->rhs);
  SBM_LAUNCHED(1);
  int rc;
  if ((rc = dsum<0>(ctx, ctx->f[SBM_F_RXN], ctx->f[SBM_F_AVPX], nullptr, 3))) return rc;
  k_dab<0><<<flat(g.nh), 256, 0, s>>>(g.nh, cne, ctx->f[SBM_F_PSE], p.d0, p.dab_c0, p.dab_c1,
                                      p.dab_c2, p.dab_c3, ctx->dab, ctx->hk_pce);
  SBM_LAUNCHED(1);
  if ((rc = fetch_scalars(ctx, 4))) return rc;
  // :465-467
  const double lsm = ctx->h_scal[3] * ((p.dx * p.dx) * p.dx);
  ctx->sc.infx = lsm / ((double)(g.ny * g.nz) * (p.dx * p.dx));
  int it = 0;
  if (iter > 1)                                                           // :505-555
    if ((rc = step_solve(ctx, SBM_OP_CNE, precision, dt / (p.dx * p.dx), &it))) return rc;
  const double flux = (ctx->sc.infx * p.t_minus) * p.dx;
  if ((rc = ghost(ctx, cne, GX_FLUX, 0, GX_COPY, 0, 0, g.nz + 1, ctx->dab, flux))) return rc;
  if (iter % p.cne_mean_every == 1) {                                     // :562-572
    if ((rc = dsum<0>(ctx, ctx->f[SBM_F_PSE], cne, nullptr, 4))) return rc;
    if ((rc = fetch_scalars(ctx, 5))) return rc;
    const double av = ctx->h_scal[4] / ctx->sc.tPE;
    k_shift<<<flat(g.ninterior()), 256, 0, s>>>(g, cne, av - p.cne_ref);
    SBM_LAUNCHED(1);
    if ((rc = ghost(ctx, cne, GX_FLUX, 0, GX_COPY, 0, 0, g.nz + 1, ctx->dab, flux))) return rc;
  }
  ctx->sc.it_cne = it;
  if (out) *out = ctx->sc;
  return SBM_OK;
}

int step_bv(sbm_ctx* ctx, int precision, sbm_scalars* out) {
  const Geo& g = ctx->g;
  cudaStream_t s = ctx->stream;
  const sbm_params& p = ctx->p;
  double *cne = ctx->f[SBM_F_CNE], *php = ctx->f[SBM_F_PHP], *phe = ctx->f[SBM_F_PHE];
  const double idx2 = 1.0 / (p.dx * p.dx);
  int rc;
  // :579-596  (hk_pce is reused as scratch for the tc1 coefficient)
  k_dab<0><<<flat(g.nh), 256, 0, s>>>(g.nh, cne, ctx->f[SBM_F_PSE], p.tc1 * p.d0, p.dab_c0,
                                      p.dab_c1, p.dab_c2, p.dab_c3, nullptr, ctx->hk_pce);
  SBM_LAUNCHED(1);
  OpArgs<double> op{g, ctx->hk_pce, nullptr, idx2, 0, SBM_BC_COPY, SBM_BC_COPY};
  SBM_CUDA_TRY(launch_apply_mem64(op, cne, ctx->rhe, s));
  // :601-610
  k_dab<1><<<flat(g.nh), 256, 0, s>>>(g.nh, cne, ctx->f[SBM_F_PSE], p.tc2 * p.d0, p.dab_c0,
                                      p.dab_c1, p.dab_c2, p.dab_c3, nullptr, ctx->hk_pcc);
  // :614-622
  const double ac = 0.5 * p.cst1;
  KArgs ka{g, ctx->f[SBM_F_CNP], ctx->kfw, ctx->kbw, tbl_dev(ctx, 2), tbl_dev(ctx, 3),
           p.i0_scale, p.frd, p.kfw_c, ac};
  k_bv_coef<<<flat(g.ninterior()), 256, 0, s>>>(ka);
  SBM_LAUNCHED(2);
  double cvgp = 1.0, cvgl = 1.0;
  int nlp = 0, itp = 0, ite = 0;
  const size_t bytes = sizeof(double) * (size_t)g.nh;
  while (cvgp > p.crt_picard && cvgl > p.crt_picard && nlp < p.max_picard) {
    k_bv_rxn<<<flat(g.ninterior()), 256, 0, s>>>(g, ctx->f[SBM_F_AVP], ctx->f[SBM_F_AVPX], php,
                                                 phe, ctx->kfw, ctx->kbw, cne, ctx->f[SBM_F_CNP],
                                                 ctx->f[SBM_F_RXN], ctx->rxc, ctx->rhs,
                                                 p.avp_mask, ac, p.frd,
                                                 p.bv_mode == SBM_BV_LINEAR);
    SBM_LAUNCHED(1);
    SBM_CUDA_TRY(cudaMemcpyAsync(ctx->ppo, php, bytes, cudaMemcpyDeviceToDevice, s));
    if ((rc = ghost(ctx, php, GX_COPY, 0, GX_VALUE, p.bvp, 0, g.nz + 1))) return rc;  // :647
    if ((rc = step_solve(ctx, SBM_OP_PHP, precision, 0.0, &itp))) return rc;
    if ((rc = ghost(ctx, php, GX_COPY, 0, GX_VALUE, p.bvp, 0, g.nz + 1))) return rc;  // :717-719
    if ((rc = dsum<2>(ctx, php, ctx->ppo, ctx->f[SBM_F_PSP], 5))) return rc;
    SBM_CUDA_TRY(cudaMemcpyAsync(ctx->peo, phe, bytes, cudaMemcpyDeviceToDevice, s));
    k_phe_rhs<<<flat(g.ninterior()), 256, 0, s>>>(g, ctx->f[SBM_F_RXN], ctx->f[SBM_F_AVPX],
                                                  ctx->rhe, ctx->rhs);
    SBM_LAUNCHED(1);
    if ((rc = step_solve(ctx, SBM_OP_PHE, precision, 0.0, &ite))) return rc;
    if ((rc = ghost(ctx, phe, GX_VALUE, ctx->sc.bve, GX_COPY, 0, 0, g.nz + 1))) return rc;  // :798-800
    if ((rc = dsum<2>(ctx, phe, ctx->peo, ctx->f[SBM_F_PSE], 6))) return rc;
    if ((rc = fetch_scalars(ctx, 7))) return rc;
    cvgp = sqrt(ctx->h_scal[5] / ctx->sc.tPP);
    cvgl = sqrt(ctx->h_scal[6] / ctx->sc.tPE);
    ++nlp;
    if (!std::isfinite(cvgp) || !std::isfinite(cvgl)) return SBM_ERR_NONFINITE;
  }
  ctx->sc.cvgp = cvgp;
  ctx->sc.cvgl = cvgl;
  ctx->sc.it_php = itp;
  ctx->sc.it_phe = ite;
  ctx->sc.n_picard = nlp;
  if (out) *out = ctx->sc;
  return SBM_OK;
}

int step_voltage(sbm_ctx* ctx, double dt, double vsr, sbm_scalars* out) {
  const Geo& g = ctx->g;
  int rc;
  if ((rc = dsum<0>(ctx, ctx->f[SBM_F_RXN], ctx->f[SBM_F_AVPX], nullptr, 7))) return rc;
  if ((rc = fetch_scalars(ctx, 8))) return rc;
  ctx->sc.scrnt = ctx->h_scal[7];                                      // :826-828
  const double d = ctx->sc.trgI - ctx->sc.scrnt;
  const double sv = copysign(fabs(vsr), d);  // DSIGN(Vsr, d): a -0.0 difference is negative
  ctx->sc.bve = ctx->sc.bve + sv * dt;                                 // :830
  k_shift<<<flat(g.ninterior()), 256, 0, ctx->stream>>>(g, ctx->f[SBM_F_PHE], -(sv * dt));
  SBM_LAUNCHED(1);
  if ((rc = ghost(ctx, ctx->f[SBM_F_PHE], GX_VALUE, ctx->sc.bve, GX_COPY, 0, 1, g.nz))) return rc;
  if (out) *out = ctx->sc;
  return SBM_OK;
}

int table_lookup_dev(cudaStream_t s, int64_t n, int sz, const double* dx, const double* dv,
                     const double* cn, double* fn) {
  Tbl t{dx, dv, sz};
  k_table<<<flat(n), 256, 0, s>>>(n, t, cn, fn);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

}  // namespace sbm
