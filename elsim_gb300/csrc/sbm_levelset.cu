// sbm_levelset.cu -- level-set reinitialisation, connectivity diffusion and
// phase masks, bit-exact with the reference arithmetic.
//
//   ReDist3D_XYZ + AbsGrd3DUW_XYZ + NoGrdBc3D   LevelSet_3D.f90:164-322
//                                               (same code in RM_UCNCT_3D.f90:180-337)
//   AccDiff sweep (solid / electrolyte)         AccDiff_3D.f90:111-169, :185-243
//   disconnected-region mask                    RM_UCNCT_3D.f90:78-82, :127-130
//   sign function                               LevelSet_3D.f90:140-144
//   Allen-Cahn pre-smoothing                    LevelSet_3D.f90:116-136
//   reorient / tunnels / stacking               LevelSet_3D.f90:80-122
//
// Bit-exactness: every operation is an explicit IEEE round-to-nearest
// intrinsic (__dadd_rn, __dmul_rn, __ddiv_rn, __dsqrt_rn), so no multiply-add
// is ever contracted, and each expression keeps the Fortran evaluation
// order.  REAL(4) literals are passed in already promoted to double.
//
// Both sweeps are Jacobi (the reference computes the whole new field from
// the old one: nf/f in ReDist, the WHERE block in AccDiff), so each
// iteration is one kernel reading buffer A and writing buffer B.  They are
// bound by GB300's FP64 pipe, not by HBM (a ReDist step moves 24 bytes per
// voxel), so comparisons and clamps run on integer bit patterns and only
// the roundings the reference's result depends on stay FP64 (the identities
// are stated above godunov()).
#include "sbm_internal.cuh"

namespace sbm {

namespace {

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// GB300 issues FP64 arithmetic at a small fraction of its FP32 / integer
// rate, and these sweeps are bound by that pipe, so the kernels below keep
// only the FP64 operations whose rounding the reference's result depends
// on; comparisons, clamps at zero and sign flips run as integer operations
// on the bit patterns.  The results are unchanged for finite fields:
//
// * max(RN(fc - a), RN(fc - b)) = RN(fc - min(a, b)) and
//   max(RN(a - fc), RN(b - fc)) = RN(max(a, b) - fc), since x -> RN(fc - x)
//   and x -> RN(x - fc) are monotone (RN = round to nearest even);
// * RN(-x) = -RN(x), so MAX(-bg, 0) with bg = f(i+1) - f(i) is
//   MAX(RN(f(i) - f(i+1)), 0);
// * max(RN(u*u), RN(v*v)) = RN(max(u, v)^2) for u, v >= 0.
//
// Hence each direction's MAX(MAX(.,0)**2, MAX(.,0)**2) of AbsGrd3DUW_XYZ is
// one subtraction and one square.

// Order-preserving integer key of a non-NaN double.
__device__ __forceinline__ long long okey(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double imin(double a, double b) { return okey(a) <= okey(b) ? a : b; }
__device__ __forceinline__ double imax(double a, double b) { return okey(a) >= okey(b) ? a : b; }
// MAX(x, 0.0d0) for non-NaN x (a zero result is +0; it is only squared).
__device__ __forceinline__ double pos0(double x) { return __double_as_longlong(x) > 0 ? x : 0.0; }

// AbsGrd3DUW_XYZ at interior cell c (LevelSet_3D.f90:294-317).
__device__ __forceinline__ double godunov(const double* __restrict__ f, const Geo& g, int64_t c,
                                          double s) {
  const long long sb = __double_as_longlong(s);
  if ((sb << 1) == 0) return 0.0;  // sg == 0.0
  const double fc = f[c];
  const double ym = f[c - 1], yp = f[c + 1], xm = f[c - g.sx], xp = f[c + g.sx];
  const double zm = f[c - g.sz], zp = f[c + g.sz];
  double a, b, e;
  if (sb > 0) {  // MAX(ag,0), MAX(-bg,0) per direction
    a = pos0(__dsub_rn(fc, imin(ym, yp)));
    b = pos0(__dsub_rn(fc, imin(xm, xp)));
    e = pos0(__dsub_rn(fc, imin(zm, zp)));
  } else {       // MAX(-ag,0), MAX(bg,0) per direction
    a = pos0(__dsub_rn(imax(ym, yp), fc));
    b = pos0(__dsub_rn(imax(xm, xp), fc));
    e = pos0(__dsub_rn(imax(zm, zp), fc));
  }
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(e, e)));
}

// RN(s*x) with the common s = +-1 as a sign flip.
__device__ __forceinline__ double mul_sign(double s, double x) {
  const long long sb = __double_as_longlong(s);
  if (sb == 0x3ff0000000000000LL) return x;
  if (sb == (long long)0xbff0000000000000ULL) return -x;
  return __dmul_rn(s, x);
}

// (v*f > 0.0) of the reference: false for a zero factor or opposite signs;
// for two normal factors with biased exponents summing to at least 972 the
// product is at least 2^-1074 and rounds to a positive value; anything else
// (possible underflow, Inf, NaN) takes the FP64 product.
__device__ __forceinline__ bool prod_pos(double v, double f) {
  const long long a = __double_as_longlong(v), b = __double_as_longlong(f);
  if ((a << 1) == 0 || (b << 1) == 0 || (a ^ b) < 0) return false;
  const int ea = (int)((a >> 52) & 0x7ff), eb = (int)((b >> 52) & 0x7ff);
  if (ea != 0 && eb != 0 && ea != 0x7ff && eb != 0x7ff && ea + eb >= 972) return true;
  return __dmul_rn(v, f) > 0.0;
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
  double v = __dadd_rn(fc, __dmul_rn(mul_sign(s, __dsub_rn(1.0, gf)), dt));
  if (!prod_pos(v, fc)) v = __dadd_rn(fc, mul_sign(s, small));
  nf[c] = v;
}

// One Allen-Cahn pre-smoothing step (LevelSet_3D.f90:124-136) over every
// cell of the padded array: the new value of the nearest interior cell, so
// the ghosts leave as the NoGrdBc3D copies; neighbours are read at clamped
// indices, which are exactly the zero-gradient ghosts the reference fills
// before the loop and after every step.  step = 0 only fills the ghosts.
//   sgF = 2*d*(1.0-d)*(1.0-2*d) - 0.64*(yp + ym + xp + xm + zp + zm - 6*d)
//   d   = d - 0.05*sgF            (0.64, 0.05 REAL(4); no FMA contraction)
__global__ void __launch_bounds__(256) k_allen_cahn(Geo g, const double* __restrict__ f,
                                                    double* __restrict__ nf, int step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.ny + 1 || j > g.nx + 1) return;
  const int ci = clampi(i, 1, g.ny), cj = clampi(j, 1, g.nx), ck = clampi(k, 1, g.nz);
  const double d = f[g.ix(ci, cj, ck)];
  double v = d;
  if (step) {
    const double c064 = (double)0.64f, c005 = (double)0.05f;
    double nb = __dadd_rn(f[g.ix(clampi(ci + 1, 1, g.ny), cj, ck)],
                          f[g.ix(clampi(ci - 1, 1, g.ny), cj, ck)]);
    nb = __dadd_rn(nb, f[g.ix(ci, clampi(cj + 1, 1, g.nx), ck)]);
    nb = __dadd_rn(nb, f[g.ix(ci, clampi(cj - 1, 1, g.nx), ck)]);
    nb = __dadd_rn(nb, f[g.ix(ci, cj, clampi(ck + 1, 1, g.nz))]);
    nb = __dadd_rn(nb, f[g.ix(ci, cj, clampi(ck - 1, 1, g.nz))]);
    nb = __dsub_rn(nb, __dmul_rn(6.0, d));
    // 2*d exactly: one more in the exponent of a normal d below 2^1023
    const long long db = __double_as_longlong(d);
    const int de = (int)((db >> 52) & 0x7ff);
    const double dd = (de != 0 && de < 0x7fe) ? __longlong_as_double(db + (1LL << 52))
                                               : __dmul_rn(2.0, d);
    const double w = __dmul_rn(__dmul_rn(dd, __dsub_rn(1.0, d)), __dsub_rn(1.0, dd));
    const double sg = __dsub_rn(w, __dmul_rn(c064, nb));
    v = __dsub_rn(d, __dmul_rn(c005, sg));
  }
  nf[g.ix(i, j, k)] = v;
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
  // psi is the same in every iteration, so its face sums and the factor
  // 0.5*idh2/psi are formed once per call (the same operations, so the
  // same bits): fs[c] = psi(i+1)+psi(i), fs[nh+c] = psi(j+1)+psi(j),
  // fs[2nh+c] = psi(k+1)+psi(k); qd[c] = (0.5*idh2)/psi where psi >= 0.4
  const double* fs;
  const double* qd;
};

// The per-call constants of the AccDiff sweep (see AccArgs::fs, qd).
__global__ void k_acc_pre(Geo g, const double* __restrict__ psi, double half_idh2, double thr,
                          double* __restrict__ fs, double* __restrict__ qd) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.nh;
       c += (int64_t)gridDim.x * blockDim.x) {
    const double p = psi[c];
    fs[c] = c + 1 < g.nh ? __dadd_rn(psi[c + 1], p) : 0.0;
    fs[g.nh + c] = c + g.sx < g.nh ? __dadd_rn(psi[c + g.sx], p) : 0.0;
    fs[2 * g.nh + c] = c + g.sz < g.nh ? __dadd_rn(psi[c + g.sz], p) : 0.0;
    qd[c] = p >= thr ? __ddiv_rn(half_idh2, p) : 0.0;
  }
}

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
    // psi(i+1)+psi(i), psi(i)+psi(i-1), ... in the reference's term order;
    // psi(i)+psi(i-1) is the stored psi(i-1)+psi(i) (addition commutes)
    const double* fy = a.fs;
    const double* fx = a.fs + g.nh;
    const double* fz = a.fs + 2 * g.nh;
    double s = __dmul_rn(fy[c], __dsub_rn(yp, u));
    s = __dsub_rn(s, __dmul_rn(fy[c - 1], __dsub_rn(u, ym)));
    s = __dadd_rn(s, __dmul_rn(fx[c], __dsub_rn(xp, u)));
    s = __dsub_rn(s, __dmul_rn(fx[c - g.sx], __dsub_rn(u, xm)));
    s = __dadd_rn(s, __dmul_rn(fz[c], __dsub_rn(zp, u)));
    s = __dsub_rn(s, __dmul_rn(fz[c - g.sz], __dsub_rn(u, zm)));
    const double div = __dmul_rn(a.qd[c], s);
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
  // a launch that failed leaves the ping-pong buffer stale: report it before
  // anything is copied back into f
  SBM_CUDA_TRY(cudaGetLastError());
  if (a != f) SBM_CUDA_TRY(cudaMemcpyAsync(f, a, sizeof(double) * g.nh, cudaMemcpyDeviceToDevice, s));
  return SBM_OK;
}

// `iters` Allen-Cahn steps on a device field (ghosts ignored on input,
// zero-gradient on output); tmp scratch of the same size.
int allen_cahn_dev(cudaStream_t s, const Geo& g, double* f, double* tmp, int iters) {
  const dim3 blk(32, 8, 1);
  const dim3 grd((g.ny + 2 + 31) / 32, (g.nx + 2 + 7) / 8, g.nz + 2);
  double* a = f;
  double* b = tmp;
  for (int m = 0; m < (iters > 0 ? iters : 1); ++m) {
    k_allen_cahn<<<grd, blk, 0, s>>>(g, a, b, iters > 0 ? 1 : 0);
    double* t = a;
    a = b;
    b = t;
  }
  SBM_LAUNCHED(iters > 0 ? iters : 1);
  SBM_CUDA_TRY(cudaGetLastError());
  if (a != f) SBM_CUDA_TRY(cudaMemcpyAsync(f, a, sizeof(double) * g.nh, cudaMemcpyDeviceToDevice, s));
  return SBM_OK;
}

namespace {

// The stacked voxel field dsF of LevelSet_3D.f90:80-122 as a gather, one
// thread per cell of the halo-padded (yg+2)(xg+2)(zg+2) array (ghosts take
// the nearest interior value: the NoGrdBc3D call of :122).
//
// The reference builds it in three passes over TmpB(yo,zo,xo):
//   reorient   TmpB(i,kk,jj) = TmpA(i,jj,zo-kk+1)                   (:82-84)
//   tunnels    TmpB(i,j,k) = 0 for j = 1..xg, k = 1..zg where
//              |(i,k)-(1,zg)| < tr or |(i,k)-(yg,1)| < tr             (:87-106)
//   stack      dsF(:,xoff+t*zo+r,:) = TmpB(:, r or zo+1-r, 1:zg) for
//              thickness t (even t straight, odd t mirrored)          (:109-119)
// The tunnel loop runs j up to xg while TmpB's second extent is zo, so with
// Fortran's column-major storage its write to (i,j,k) lands on element
// (i, MOD(j-1+zo*(k-1), zo)+1, (j-1+zo*(k-1))/zo+1): a TmpB element with
// column index J = (b2-1) + zo*(b3-1) is zeroed when some loop point
// (j,k) has j-1 + zo*(k-1) = J and meets the tunnel test for its own k.
// The gather tests exactly those k (at most ceil(xg/zo)+1 of them).
struct StackArgs {
  const double* vox;     // TmpA(yo,xo,zo), Fortran order
  int yo, xo, zo;
  int xoff, xg;          // leading zero columns; xg = xoff + nthick*zo
  double tr;             // tunnel radius
};

__device__ __forceinline__ bool in_tunnel(int i, int k, int yg, int zg, double tr) {
  const double a = __dsub_rn((double)i, 1.0), b = __dsub_rn((double)k, (double)zg);
  if (__dsqrt_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b))) < tr) return true;
  const double c = __dsub_rn((double)i, (double)yg), d = __dsub_rn((double)k, 1.0);
  return __dsqrt_rn(__dadd_rn(__dmul_rn(c, c), __dmul_rn(d, d))) < tr;
}

__global__ void __launch_bounds__(256) k_ls_stack(Geo g, StackArgs a, double* __restrict__ ds) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.ny + 1 || j > g.nx + 1) return;
  const int ci = clampi(i, 1, g.ny), cj = clampi(j, 1, g.nx), ck = clampi(k, 1, g.nz);
  double v = 0.0;
  if (cj > a.xoff) {
    const int t = (cj - a.xoff - 1) / a.zo, r = (cj - a.xoff - 1) - t * a.zo;
    const int b2 = (t & 1) ? a.zo - r : r + 1;  // TmpB second index
    const int b3 = ck;                           // TmpB third index
    const int64_t J = (int64_t)(b2 - 1) + (int64_t)a.zo * (b3 - 1);
    int64_t mlo = J - (a.xg - 1);
    mlo = mlo <= 0 ? 0 : (mlo + a.zo - 1) / a.zo;
    int64_t mhi = J / a.zo;
    if (mhi > g.nz - 1) mhi = g.nz - 1;
    bool zero = false;
    for (int64_t m = mlo; m <= mhi && !zero; ++m) zero = in_tunnel(ci, (int)m + 1, g.ny, g.nz, a.tr);
    if (!zero)
      v = a.vox[(int64_t)(ci - 1) + (int64_t)a.yo * ((int64_t)(b3 - 1) + (int64_t)a.xo * (a.zo - b2))];
  }
  ds[g.ix(i, j, k)] = v;
}

// Sign function of the pre-smoothed field (LevelSet_3D.f90:140-144) over
// every cell, and the zero start of the reinitialisation (:147).
__global__ void k_ls_sign(int64_t n, double* __restrict__ d, double* __restrict__ sg) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    sg[c] = d[c] > 0.5 ? 1.0 : -1.0;
    d[c] = 0.0;
  }
}

}  // namespace

// dsF of LevelSet_3D.f90:80-122 from device voxels; g is the (yg, xg, zg)
// grid, xg = xoff + nthick*zo.
int ls_geometry_dev(cudaStream_t s, const Geo& g, const double* vox, int yo, int xo, int zo,
                    int xoff, double tr, double* ds) {
  StackArgs a;
  a.vox = vox;
  a.yo = yo;
  a.xo = xo;
  a.zo = zo;
  a.xoff = xoff;
  a.xg = g.nx;
  a.tr = tr;
  const dim3 blk(32, 8, 1);
  const dim3 grd((g.ny + 2 + 31) / 32, (g.nx + 2 + 7) / 8, g.nz + 2);
  k_ls_stack<<<grd, blk, 0, s>>>(g, a, ds);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

// One frame of LevelSet_3D.f90:80-150: stacked field, `ac_iters` Allen-Cahn
// steps, sign, `lit` reinitialisation steps from zero.  The distance lands
// in ds; sg and tmp are scratch of the same size.
int ls_frontend_dev(cudaStream_t s, const Geo& g, const double* vox, int yo, int xo, int zo,
                    int xoff, double tr, int ac_iters, int lit, double dt, double* ds, double* sg,
                    double* tmp) {
  int rc = ls_geometry_dev(s, g, vox, yo, xo, zo, xoff, tr, ds);
  if (!rc && ac_iters > 0) rc = allen_cahn_dev(s, g, ds, tmp, ac_iters);
  if (rc) return rc;
  k_ls_sign<<<4 * 152, 256, 0, s>>>(g.nh, ds, sg);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return redist_dev(s, g, sg, ds, tmp, lit, dt);
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
  // per-call constants, stream-ordered scratch released on every return path
  struct Scratch {
    double* p = nullptr;
    cudaStream_t s;
    ~Scratch() {
      if (p) cudaFreeAsync(p, s);
    }
  } scr{nullptr, s};
  SBM_CUDA_TRY(cudaMallocAsync(&scr.p, sizeof(double) * 4 * (size_t)g.nh, s));
  double* fs = scr.p;
  k_acc_pre<<<flat(g.nh), 256, 0, s>>>(g, psi, a.half_idh2, a.thr, fs, fs + 3 * g.nh);
  SBM_LAUNCHED(1);
  a.fs = fs;
  a.qd = fs + 3 * g.nh;
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
// overlaps on the GPU (different streams or host threads) race on it.  A call
// waits for its stream to finish the iterations before it returns.  The
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
  const int64_t cells = ((int64_t)py + 2) * ((int64_t)px + 2) * ((int64_t)pz + 2);
  if (cells > SBM_NOALLOC_REDIST_MAX_CELLS) {
    char msg[160];
    snprintf(msg, sizeof(msg),
             "sbm_redist_noalloc: %lld padded cells exceed the %d-cell built-in scratch",
             (long long)cells, SBM_NOALLOC_REDIST_MAX_CELLS);
    sbm::set_error_msg(msg);
    return SBM_ERR_ARG;
  }
  // one grid plane of CTAs per padded z plane: the grid's z extent is 65535
  if ((int64_t)pz + 2 > 65535) {
    sbm::set_error_msg("sbm_redist_noalloc: pz + 2 exceeds 65535 z planes");
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
