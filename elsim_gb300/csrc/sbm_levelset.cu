// sbm_levelset.cu -- level-set reinitialisation, connectivity diffusion and
// phase masks, bit-exact with the reference arithmetic.
//
//   ReDist3D_XYZ + AbsGrd3DUW_XYZ + NoGrdBc3D   LevelSet_3D.f90:164-322
//                                               (same code in RM_UCNCT_3D.f90:180-337)
//   AccDiff sweep (solid / electrolyte)         AccDiff_3D.f90:111-169, :185-243
//   disconnected-region mask                    RM_UCNCT_3D.f90:78-82, :127-130
//   sign function                               LevelSet_3D.f90:140-144
//
// Bit-exactness: every operation is an explicit IEEE round-to-nearest
// intrinsic (__dadd_rn, __dmul_rn, __ddiv_rn, __dsqrt_rn), so no multiply-add
// is ever contracted, and each expression keeps the Fortran evaluation
// order.  REAL(4) literals are passed in already promoted to double.
//
// Both sweeps are Jacobi (the reference computes the whole new field from
// the old one: nf/f in ReDist, the WHERE block in AccDiff), so each
// iteration is one kernel reading buffer A and writing buffer B.  Each is
// FP64-ALU-bound on GB300 (about 40 FP64 operations per voxel against 24
// bytes of traffic).
#include "sbm_internal.cuh"

namespace sbm {

namespace {

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
__device__ __forceinline__ double dmax0(double a) { return a > 0.0 ? a : 0.0; }
__device__ __forceinline__ double dmaxd(double a, double b) { return a > b ? a : b; }

// AbsGrd3DUW_XYZ at interior cell c (LevelSet_3D.f90:294-317).
__device__ __forceinline__ double godunov(const double* __restrict__ f, const Geo& g, int64_t c,
                                          double s) {
  const double fc = f[c];
  const double ag = __dsub_rn(fc, f[c - 1]);
  const double bg = __dsub_rn(f[c + 1], fc);
  const double cg = __dsub_rn(fc, f[c - g.sx]);
  const double dg = __dsub_rn(f[c + g.sx], fc);
  const double eg = __dsub_rn(fc, f[c - g.sz]);
  const double fg = __dsub_rn(f[c + g.sz], fc);
  if (s == 0.0) return 0.0;
  double a, b, cc, d, e, ff;
  if (s > 0.0) {
    a = dmax0(ag); b = dmax0(-bg); cc = dmax0(cg); d = dmax0(-dg); e = dmax0(eg); ff = dmax0(-fg);
  } else {
    a = dmax0(-ag); b = dmax0(bg); cc = dmax0(-cg); d = dmax0(dg); e = dmax0(-eg); ff = dmax0(fg);
  }
  const double m1 = dmaxd(__dmul_rn(a, a), __dmul_rn(b, b));
  const double m2 = dmaxd(__dmul_rn(cc, cc), __dmul_rn(d, d));
  const double m3 = dmaxd(__dmul_rn(e, e), __dmul_rn(ff, ff));
  return __dsqrt_rn(__dadd_rn(__dadd_rn(m1, m2), m3));
}

// One ReDist3D_XYZ iteration over every cell of the padded array
// (LevelSet_3D.f90:229-258): Gf on the interior, NoGrdBc3D (every ghost of
// Gf takes the nearest interior value), then
//   nf = f + sg*(1 - Gf)*dt;  if .NOT.(nf*f > 0): nf = f + dt*1e-7*sg.
__global__ void __launch_bounds__(256) k_redist(Geo g, const double* __restrict__ sg,
                                                const double* __restrict__ f,
                                                double* __restrict__ nf, double dt,
                                                double small) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.ny + 1 || j > g.nx + 1) return;
  const int64_t c = g.ix(i, j, k);
  const int64_t cc = g.ix(clampi(i, 1, g.ny), clampi(j, 1, g.nx), clampi(k, 1, g.nz));
  const double gf = godunov(f, g, cc, sg[cc]);
  const double fc = f[c], s = sg[c];
  double v = __dadd_rn(fc, __dmul_rn(__dmul_rn(s, __dsub_rn(1.0, gf)), dt));
  if (!(__dmul_rn(v, fc) > 0.0)) v = __dadd_rn(fc, __dmul_rn(small, s));
  nf[c] = v;
}

struct AccArgs {
  Geo g;
  const double* psi;
  const double* cn;
  double* cn_new;
  double dt, half_idh2, thr, cmin;
  int dirichlet_x;  // 1: Cn = 1 at x = nx+1 (solid); 0: at x = 0 (electrolyte)
  int stored;       // 1: read Cn's ghosts from memory (first iteration)
  int accel;        // MOD(iter,5) == 1
};

// One AccDiff iteration on the interior (AccDiff_3D.f90:118-134): Jacobi
// masked diffusion, then the acceleration step.  After the first iteration
// the ghosts are the boundary rule of AccDiff_3D.f90:138-148 / :212-222,
// applied while loading: a copy face reads the edge value (the cell itself)
// and the Dirichlet x face reads 1.
__global__ void __launch_bounds__(256) k_accdiff(AccArgs a) {
  const Geo g = a.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > g.ny || j > g.nx) return;
  const int64_t c = g.ix(i, j, k);
  const double p = a.psi[c];
  const double u = a.cn[c];
  double un = u;
  if (p >= a.thr) {
    double yp = a.cn[c + 1], ym = a.cn[c - 1];
    double xp = a.cn[c + g.sx], xm = a.cn[c - g.sx];
    double zp = a.cn[c + g.sz], zm = a.cn[c - g.sz];
    if (!a.stored) {
      if (i == g.ny) yp = u;
      if (i == 1) ym = u;
      if (j == g.nx) xp = a.dirichlet_x ? 1.0 : u;
      if (j == 1) xm = a.dirichlet_x ? u : 1.0;
      if (k == g.nz) zp = u;
      if (k == 1) zm = u;
    }
    const double* ps = a.psi;
    double s = __dmul_rn(__dadd_rn(ps[c + 1], p), __dsub_rn(yp, u));
    s = __dsub_rn(s, __dmul_rn(__dadd_rn(p, ps[c - 1]), __dsub_rn(u, ym)));
    s = __dadd_rn(s, __dmul_rn(__dadd_rn(ps[c + g.sx], p), __dsub_rn(xp, u)));
    s = __dsub_rn(s, __dmul_rn(__dadd_rn(p, ps[c - g.sx]), __dsub_rn(u, xm)));
    s = __dadd_rn(s, __dmul_rn(__dadd_rn(ps[c + g.sz], p), __dsub_rn(zp, u)));
    s = __dsub_rn(s, __dmul_rn(__dadd_rn(p, ps[c - g.sz]), __dsub_rn(u, zm)));
    const double div = __dmul_rn(__ddiv_rn(a.half_idh2, p), s);
    un = __dadd_rn(u, __dmul_rn(a.dt, div));
  }
  if (a.accel && un > a.cmin && p > a.thr) un = 1.0;
  a.cn_new[c] = un;
}

// Ghosts of Cn after an AccDiff iteration: the x Dirichlet face is 1, every
// other ghost the nearest interior value (AccDiff_3D.f90:138-148).
__global__ void k_acc_ghost(Geo g, double* __restrict__ cn, int dirichlet_x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.ny + 1 || j > g.nx + 1) return;
  const bool ghost = (i == 0 || i == g.ny + 1 || j == 0 || j == g.nx + 1 || k == 0 || k == g.nz + 1);
  if (!ghost) return;
  const int64_t c = g.ix(i, j, k);
  if ((dirichlet_x && j == g.nx + 1) || (!dirichlet_x && j == 0)) {
    cn[c] = 1.0;
  } else {
    cn[c] = cn[g.ix(clampi(i, 1, g.ny), clampi(j, 1, g.nx), clampi(k, 1, g.nz))];
  }
}

__global__ void k_rm_mask(int64_t n, const double* __restrict__ psA, const double* __restrict__ cn,
                          double* __restrict__ psB, double thr) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    psB[c] = (cn[c] < thr) ? 0.0 : psA[c];
}

__global__ void k_sign(int64_t n, const double* __restrict__ ds, double thr, double* __restrict__ sg) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    sg[c] = (ds[c] > thr) ? 1.0 : -1.0;
}

dim3 flat(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return dim3((unsigned)b);
}

}  // namespace

// lit Jacobi iterations of ReDist3D_XYZ on device buffers; f in/out, tmp
// scratch of the same size.
int redist_dev(cudaStream_t s, const Geo& g, const double* sg, double* f, double* tmp, int lit,
               double dt) {
  const dim3 blk(32, 8, 1);
  const dim3 grd((g.ny + 2 + 31) / 32, (g.nx + 2 + 7) / 8, g.nz + 2);
  const double small = dt * 1.0e-7;  // LevelSet_3D.f90:248: dt * 1.0d-7 * sg
  double* a = f;
  double* b = tmp;
  for (int m = 0; m < lit; ++m) {
    k_redist<<<grd, blk, 0, s>>>(g, sg, a, b, dt, small);
    double* t = a;
    a = b;
    b = t;
  }
  SBM_LAUNCHED(lit);
  if (a != f) SBM_CUDA_TRY(cudaMemcpyAsync(f, a, sizeof(double) * g.nh, cudaMemcpyDeviceToDevice, s));
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

// AccDiff iterations 2..term on device buffers; cn in/out (ghosts included),
// tmp scratch.
int accdiff_dev(cudaStream_t s, const Geo& g, const double* psi, double* cn, double* tmp,
                int term, int dirichlet_x) {
  const dim3 blk(32, 8, 1);
  const dim3 grd((g.ny + 31) / 32, (g.nx + 7) / 8, g.nz);
  AccArgs a;
  a.g = g;
  a.psi = psi;
  a.dt = (double)(1.25e-1f * 0.5f);   // AccDiff_3D.f90:51, REAL(4) product
  a.half_idh2 = 0.5 * (1.0 / (1.0 * 1.0));  // 0.5*idh2, AccDiff_3D.f90:49, :119
  a.thr = (double)4.0e-1f;            // :118, :133
  a.cmin = (double)1.0e-4f;           // :133
  a.dirichlet_x = dirichlet_x;
  double* src = cn;
  double* dst = tmp;
  // the interior of tmp must carry the ghosts too once we read it with
  // stored ghosts; only the first iteration does, and it reads cn.
  int n = 0;
  for (int iter = 2; iter <= term; ++iter, ++n) {
    a.cn = src;
    a.cn_new = dst;
    a.stored = (iter == 2);
    a.accel = (iter % 5 == 1);
    k_accdiff<<<grd, blk, 0, s>>>(a);
    double* t = src;
    src = dst;
    dst = t;
  }
  SBM_LAUNCHED(n);
  if (src != cn && n > 0)
    SBM_CUDA_TRY(cudaMemcpyAsync(cn, src, sizeof(double) * g.nh, cudaMemcpyDeviceToDevice, s));
  if (n > 0) {
    const dim3 gg((g.ny + 2 + 31) / 32, (g.nx + 2 + 7) / 8, g.nz + 2);
    k_acc_ghost<<<gg, blk, 0, s>>>(g, cn, dirichlet_x);
    SBM_LAUNCHED(1);
  }
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

int rm_mask_dev(cudaStream_t s, int64_t n, const double* psA, const double* cn, double* psB) {
  k_rm_mask<<<flat(n), 256, 0, s>>>(n, psA, cn, psB, (double)1.0e-4f);  // RM_UCNCT_3D.f90:80
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

int sign_dev(cudaStream_t s, int64_t n, const double* ds, double thr, double* sg) {
  k_sign<<<flat(n), 256, 0, s>>>(n, ds, thr, sg);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

}  // namespace sbm

// ================================================ no-allocation ReDist3D_XYZ
// sbm_redist_noalloc runs the same ReDist3D_XYZ iterations as sbm_redist on
// caller-owned device buffers, for callers that must not allocate device
// memory themselves or through this library.  Its only scratch -- the
// ping-pong field of the Jacobi sweep -- is the fixed array below: every GPU
// that loads this library holds it (SBM_NOALLOC_REDIST_MAX_CELLS doubles,
// 8 MiB) until the process exits.  All calls share it: two calls whose work
// overlaps on the GPU (different streams or host threads) race on it.  The
// sweep writes every cell of the scratch before reading it, so the contents
// a previous call left behind never matter and nothing is cleared.

#include <mutex>

namespace sbm {

static __device__ __align__(256) double g_redist_scratch[SBM_NOALLOC_REDIST_MAX_CELLS];

namespace {

std::mutex g_redist_scratch_mu;
double* g_redist_scratch_ptr[64] = {};

// Device address of the scratch array on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is asked of
// the runtime once per device (with that device current) and cached.
int redist_scratch(double** out) {
  int dev = 0;
  SBM_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return SBM_ERR_STATE;
  std::lock_guard<std::mutex> lock(g_redist_scratch_mu);
  if (!g_redist_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_redist_scratch);
    if (e != cudaSuccess) {
      set_error("cudaGetSymbolAddress", e);
      return SBM_ERR_CUDA;
    }
    g_redist_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_redist_scratch_ptr[dev];
  return SBM_OK;
}

}  // namespace
}  // namespace sbm

extern "C" int sbm_redist_noalloc(int lit, int py, int px, int pz, double dt, const double* sg,
                                  double* f, void* stream) {
  if (lit < 0 || py < 1 || px < 1 || pz < 1 || !sg || !f) return SBM_ERR_ARG;
  const int64_t cells = (int64_t)(py + 2) * (px + 2) * (pz + 2);
  if (cells > SBM_NOALLOC_REDIST_MAX_CELLS) {
    char msg[160];
    snprintf(msg, sizeof(msg),
             "sbm_redist_noalloc: %lld padded cells exceed the %d-cell built-in scratch",
             (long long)cells, SBM_NOALLOC_REDIST_MAX_CELLS);
    sbm::set_error_msg(msg);
    return SBM_ERR_ARG;
  }
  double* scratch = nullptr;
  int rc = sbm::redist_scratch(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  rc = sbm::redist_dev(s, sbm::make_geo(py, px, pz), sg, f, scratch, lit, dt);
  if (rc) return rc;
  SBM_CUDA_TRY(cudaStreamSynchronize(s));
  return SBM_OK;
}
