// sbm_internal.cuh -- shared declarations of the GB300 SBM library.
//
// Device layout: every field lives in HBM in the reference's halo-padded
// Fortran layout A(0:ny+1, 0:nx+1, 0:nz+1), y fastest, so host arrays are
// uploaded and downloaded with one contiguous copy and no transpose.  The
// MPI decomposition of the reference (MyDmnCmpn_YZ / BcMpiYZ in
// SBMES_3D_MPI_CH_Gr_CONJG_VD_T05_01_BQ_hx3.f90) collapses into this one
// device-resident domain; physical-boundary ghost rules are applied inside
// the kernels that read the ghosts.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <string>
#include <utility>

#include "../../include/sbm_capi.h"

namespace sbm {

// ------------------------------------------------------------ geometry
struct Geo {
  int ny, nx, nz;
  int64_t sx;  // stride of the x index j   = ny+2
  int64_t sz;  // stride of the z index k   = (ny+2)(nx+2)
  int64_t nh;  // halo-padded element count = (ny+2)(nx+2)(nz+2)
  __host__ __device__ __forceinline__ int64_t ix(int i, int j, int k) const {
    return (int64_t)i + sx * j + sz * k;
  }
  __host__ __device__ __forceinline__ int64_t ninterior() const {
    return (int64_t)ny * nx * nz;
  }
};

inline Geo make_geo(int ny, int nx, int nz) {
  Geo g;
  g.ny = ny;
  g.nx = nx;
  g.nz = nz;
  g.sx = ny + 2;
  g.sz = (int64_t)(ny + 2) * (nx + 2);
  g.nh = g.sz * (nz + 2);
  return g;
}

// Internal FP32 layout of the mixed-precision solver: rows padded to a
// multiple of 4 floats and shifted by kOff32 elements, so the first
// interior element (i = 1) of every row is 16-byte aligned and a row of
// ny (a multiple of 4) interior values is read with float4 loads.  Kernels
// get `buffer + kOff32` as base and index it like the Fortran layout with
// these strides; nh counts the floats to allocate (including the shift).
constexpr int kOff32 = 3;
inline Geo make_geo32(int ny, int nx, int nz) {
  Geo g;
  g.ny = ny;
  g.nx = nx;
  g.nz = nz;
  g.sx = ((int64_t)ny + 2 + kOff32 + 3) / 4 * 4;
  g.sz = g.sx * (nx + 2);
  g.nh = g.sz * (nz + 2) + 4;
  return g;
}

// ------------------------------------------------------- launch shape
// Stencil-family kernels map threadIdx.x to y (the contiguous axis) and
// threadIdx.y to x; each thread marches `zc` planes in z and keeps the
// z-neighbours in registers.
constexpr int BX = 32;
constexpr int BY = 8;
constexpr int kMaxPartials = 1 << 16;  // >= blocks of any reduction launch

struct Shape {
  dim3 grid, block;
  int zc;
  int nblocks() const { return (int)(grid.x * grid.y * grid.z); }
};

inline Shape stencil_shape(const Geo& g, int zc) {
  Shape s;
  s.zc = zc < 1 ? 1 : zc;
  s.block = dim3(BX, BY, 1);
  s.grid = dim3((g.ny + BX - 1) / BX, (g.nx + BY - 1) / BY, (g.nz + s.zc - 1) / s.zc);
  return s;
}

// Picks the z-chunk so that a launch covers the 152 SMs in several full
// waves; `tuned` > 0 overrides (set by the autotuner).
int pick_zc(const Geo& g, int tuned);

// -------------------------------------------------------- CG state
// One per solve, in device memory.  Scalars are produced by the last block
// of each reduction kernel and consumed by the next kernel, so the loop
// needs no host round trip; `done` turns remaining launches of a captured
// chunk into no-ops.
struct CgState {
  double rho;     // CG scalar of the current residual: r.z (r.r without preconditioner)
  double rr;      // r.r of the current residual (stopping test)
  double rr0;     // r.r of the initial residual
  double pq;      // p.Ap
  double alpha, beta;
  double rms;     // value of the stopping norm after the last iteration
  double tol;
  double wsum;    // sum of the stopping weight (tPP / tPE)
  double maxrr;   // mixed: largest FP32 r.r since the last reliable update
  double delta2;  // mixed: reliable update when r.r < delta2 * maxrr
  double aux[4];
  int iter;
  int max_it;
  int done;       // 0 running, 1 converged, 2 iteration cap, 3 non-finite, 4 breakdown
  int stop_rule;
  int reliable;       // mixed: recompute the FP64 residual in this iteration
  int accum_pending;  // mixed: fold the FP32 correction into the FP64 one
  int initial;        // mixed: first residual of the solve (beta = 0)
  int n_reliable;     // mixed: number of FP64 residual replacements
  int pc_off;         // learned preconditioner switched off (no progress): z = D^-1 r
  int stall_iter;     // iteration of the last halving of the FP32 residual norm
  unsigned int counter[8];
};

// ------------------------------------------------------ errors, counters
extern std::atomic<int64_t> g_launches;
void set_error(const char* where, cudaError_t e);
void set_error_msg(const char* msg);
const char* last_error();

#define SBM_CUDA_TRY(call)                                    \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) {                                  \
      ::sbm::set_error(#call, e_);                            \
      return SBM_ERR_CUDA;                                    \
    }                                                         \
  } while (0)

#define SBM_LAUNCHED(n) ::sbm::g_launches.fetch_add((n), std::memory_order_relaxed)

// ------------------------------------- programmatic dependent launch
// Kernels of the captured CG loop start with pdl_begin(): they allow the
// next kernel of the stream to be scheduled as soon as all their CTAs run,
// then wait until the previous kernel has completed and its writes are
// visible (a no-op when launched without the attribute).  Nothing is read
// before the wait, so the overlap covers launch latency and CTA placement
// only, and every wait ends (no kernel waits on a later one).
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// ---------------------------------------------------- device helpers
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of `v` for up to 1024 threads; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double* smem32) {
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthr = blockDim.x * blockDim.y * blockDim.z;
  v = warp_sum(v);
  if ((tid & 31) == 0) smem32[tid >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (tid < 32) {
    r = (tid < (nthr + 31) / 32) ? smem32[tid] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

// Deterministic grid reduction of NV values per thread: block sums go to
// partials[v * nblocks + block]; the last block to finish sums them in a
// fixed order and returns true with the totals in `tot` (valid in every
// thread of that block).  The counter is re-armed for the next launch.
template <int NV>
__device__ __forceinline__ bool grid_reduce(const double (&v)[NV], double* partials,
                                            unsigned int* counter, double (&tot)[NV]) {
  __shared__ double sm[32];
  __shared__ bool is_last;
  __shared__ double res[NV];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthr = blockDim.x * blockDim.y * blockDim.z;
  const int nb = gridDim.x * gridDim.y * gridDim.z;
  const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const double b = block_sum(v[q], sm);
    if (tid == 0) partials[q * nb + bid] = b;
  }
  if (tid == 0) {
    __threadfence();
    const unsigned int t = atomicAdd(counter, 1u);
    is_last = (t == (unsigned int)nb - 1u);
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    double s = 0.0;
    for (int b = tid; b < nb; b += nthr) s += __ldcg(partials + q * nb + b);
    s = block_sum(s, sm);
    if (tid == 0) res[q] = s;
  }
  if (tid == 0) *counter = 0u;
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) tot[q] = res[q];
  return true;
}

// ------------------------------------------------------ operator args
// q = scale*S(p)            (FORM 0: the phP / phE form, SBMES:670-676)
// q = diag*p - scale*S(p)   (FORM 1: the CnE form,       SBMES:515-521)
// with S(p) = sum_f c_f (p_nb - p_c), c_f = hk_nb + hk_c, hk = K/2.
template <typename T>
struct OpArgs {
  Geo g;
  const T* hk;    // half node coefficient, halo-padded
  const T* diag;  // FORM 1 diagonal field (psE), halo-padded, else null
  T scale;
  int form;       // 0 or 1
  int bcx0, bcx1; // SBM_BC_COPY / SBM_BC_ZERO for the search direction
  // optional stored face coefficients (FP64 path): y, x and z faces of every
  // padded cell, fc[c] = hk[c+1] + hk[c], fc[nh + c] = hk[c+sx] + hk[c],
  // fc[2 nh + c] = hk[c+sz] + hk[c] -- the values face_sum forms, read
  // instead of recomputed (the FP64 stencil is bound by GB300's FP64 rate)
  const T* fc = nullptr;
};

// ------------------------------------------- double-float arithmetic
// An unevaluated sum hi + lo of two FP32 values with |lo| <= ulp(hi)/2
// carries about 48 significant bits.  The mixed solver keeps its FP64-grade
// quantities in this form (the correction, the initial residual, the
// coefficients as hi + lo splits of the FP64 values) and forms the
// residual replacement with FP32 instructions, whose rate on GB300 is
// some 64x that of FP64.  Error-free transformations: Knuth's TwoSum,
// Dekker's Fast2Sum (|a| >= |b|) and the FMA product error; the _rn
// intrinsics keep the compiler from contracting or reordering them.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ DF df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_add(DF x, DF y) {
  const DF s = df_two_sum(x.hi, y.hi);
  return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
__device__ __forceinline__ DF df_sub(DF x, DF y) { return df_add(x, DF{-y.hi, -y.lo}); }
__device__ __forceinline__ DF df_add_f(DF x, float y) {
  const DF s = df_two_sum(x.hi, y);
  return df_fast_two_sum(s.hi, __fadd_rn(s.lo, x.lo));
}
__device__ __forceinline__ DF df_mul(DF x, DF y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  return df_fast_two_sum(p, e);
}
// The same operations on pairs of FP32 lanes (paired add / multiply /
// FMA), one double-float value per lane, each lane bit-identical to the
// scalar forms above.
struct DF2 {
  float2 hi, lo;
};
__device__ __forceinline__ float2 f2_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ DF2 df2_two_sum(float2 a, float2 b) {
  const float2 s = __fadd2_rn(a, b);
  const float2 bb = __fadd2_rn(s, f2_neg(a));
  return {s, __fadd2_rn(__fadd2_rn(a, f2_neg(__fadd2_rn(s, f2_neg(bb)))),
                        __fadd2_rn(b, f2_neg(bb)))};
}
__device__ __forceinline__ DF2 df2_fast_two_sum(float2 a, float2 b) {
  const float2 s = __fadd2_rn(a, b);
  return {s, __fadd2_rn(b, f2_neg(__fadd2_rn(s, f2_neg(a))))};
}
__device__ __forceinline__ DF2 df2_add(DF2 x, DF2 y) {
  const DF2 s = df2_two_sum(x.hi, y.hi);
  return df2_fast_two_sum(s.hi, __fadd2_rn(s.lo, __fadd2_rn(x.lo, y.lo)));
}
__device__ __forceinline__ DF2 df2_sub(DF2 x, DF2 y) {
  return df2_add(x, DF2{f2_neg(y.hi), f2_neg(y.lo)});
}
__device__ __forceinline__ DF2 df2_add_f(DF2 x, float2 y) {
  const DF2 s = df2_two_sum(x.hi, y);
  return df2_fast_two_sum(s.hi, __fadd2_rn(s.lo, x.lo));
}
__device__ __forceinline__ DF2 df2_mul(DF2 x, DF2 y) {
  const float2 p = __fmul2_rn(x.hi, y.hi);
  float2 e = __ffma2_rn(x.hi, y.hi, f2_neg(p));
  e = __ffma2_rn(x.hi, y.lo, e);
  e = __ffma2_rn(x.lo, y.hi, e);
  return df2_fast_two_sum(p, e);
}

// hi + lo split of an FP64 value (lo exact to FP32 rounding)
__host__ __device__ __forceinline__ void df_split(double v, float* hi, float* lo) {
  const float h = (float)v;
  *hi = h;
  *lo = (float)(v - (double)h);
}

// (double)f with integer instructions for zero and normal f (exact, as the
// conversion is); subnormal, infinite and NaN f take the conversion.
__device__ __forceinline__ double f2d_int(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  if ((u << 1) == 0) return __longlong_as_double((long long)sign);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0 || e == 0xffu) return (double)f;
  return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 1023 - 127) << 52) |
                                          ((unsigned long long)(u & 0x7fffffu) << 29)));
}

// The same split with integer instructions (GB300's FP64 pipe is some 64x
// slower than its integer and FP32 pipes): hi rounds the 53-bit significand
// to 24 bits (to nearest, ties to even, as the conversion does), the exact
// remainder r (|r| <= 2^28 units of the double's last place) becomes lo by
// one int -> float conversion (round to nearest) and a power-of-two scale,
// so hi and lo are bit-identical to df_split's.  Zero is split as 0 + 0;
// magnitudes outside [2^-70, 2^127) (where lo could be subnormal or hi
// could overflow) take df_split's FP64 path.
__device__ __forceinline__ void df_split_int(double v, float* hi, float* lo) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const int eb = (int)((u >> 52) & 0x7ff);  // biased exponent
  const unsigned sign = (unsigned)(u >> 63) << 31;
  if (eb == 0 && (u << 1) == 0) {  // +-0
    *hi = __uint_as_float(sign);
    *lo = 0.f;
    return;
  }
  const int e = eb - 1023;
  if (e < -70 || e > 126) {
    df_split(v, hi, lo);
    return;
  }
  const unsigned long long m = (u & ((1ull << 52) - 1)) | (1ull << 52);
  unsigned long long mh = m >> 29;
  const unsigned long long drop = m & ((1ull << 29) - 1);
  if (drop > (1ull << 28) || (drop == (1ull << 28) && (mh & 1))) mh += 1;
  const int r = (int)((long long)m - (long long)(mh << 29));
  int eh = e;
  if (mh == (1ull << 24)) {  // rounding carried into the next binade
    mh >>= 1;
    eh += 1;
  }
  *hi = __uint_as_float(sign | ((unsigned)(eh + 127) << 23) | ((unsigned)mh & 0x7fffffu));
  const float scale = __uint_as_float((unsigned)(e - 52 + 127) << 23);  // 2^(e-52), normal
  // an exact split (r = 0) gives lo = +0, as v - (double)hi does
  *lo = r == 0 ? 0.f : __uint_as_float(__float_as_uint(__int2float_rn(r) * scale) ^ sign);
}

// Extra operands of the flexible-CG direction kernel (learned
// preconditioner).  That kernel also applies the previous iteration's
// deferred x32 += alpha p_old (or, after a residual replacement, folds x32
// into the double-float correction first) and restricts q = A p_new to the coarse grid (rq = 4x4x4
// means, strides rcy / rcx of the coarse arrays), so that neither x nor the
// restriction of the residual needs a pass of its own.
struct FcgDirArgs {
  float* x32 = nullptr;       // FP32 correction (g32 layout)
  float* dhi = nullptr;       // double-float correction hi + lo (g32 layout)
  float* dlo = nullptr;
  const float* rc = nullptr;  // R r of the current residual (coarse)
  float* rq = nullptr;        // R q of the new direction (coarse, written)
  float* scal = nullptr;      // s = RMS(R r_next), 1/s (written by the last block)
  int rcy = 0, rcx = 0;       // y and x strides of the coarse arrays
  int64_t ncell = 0;          // valid coarse cells
};

// face_sum with stored faces: the same operands and order, so the same bits.
template <typename T>
__device__ __forceinline__ T face_sum_stored(const Geo& g, const T* __restrict__ fc, int64_t c,
                                             T pc, T pyp, T pym, T pxp, T pxm, T pzp, T pzm) {
  const T* fy = fc;
  const T* fx = fc + g.nh;
  const T* fz = fc + 2 * g.nh;
  T s = fy[c] * (pyp - pc);
  s = s - fy[c - 1] * (pc - pym);
  s = s + fx[c] * (pxp - pc);
  s = s - fx[c - g.sx] * (pc - pxm);
  s = s + fz[c] * (pzp - pc);
  s = s - fz[c - g.sz] * (pc - pzm);
  return s;
}

// Face terms of S(p) = sum_f c_f (p_nb - p_c) in the reference's order
// (y+, y-, x+, x-, z+, z-; SBMES:494-499), c_f = hk_nb + hk_c.
template <typename T>
__device__ __forceinline__ T face_sum(T kc, T pc, T kyp, T pyp, T kym, T pym, T kxp, T pxp,
                                      T kxm, T pxm, T kzp, T pzp, T kzm, T pzm) {
  T s = (kyp + kc) * (pyp - pc);
  s = s - (kym + kc) * (pc - pym);
  s = s + (kxp + kc) * (pxp - pc);
  s = s - (kxm + kc) * (pc - pxm);
  s = s + (kzp + kc) * (pzp - pc);
  s = s - (kzm + kc) * (pc - pzm);
  return s;
}

// ------------------------------------------------------- launchers
// q = A x with x's ghosts read from memory (no reduction), FP64.  Used for
// RHE = (1/dx^2) div(pce grad CnE), SBMES:591-596.
cudaError_t launch_apply_mem64(const OpArgs<double>& op, const double* x, double* q,
                               cudaStream_t s);
// hk = 0.5 * K over the padded array.
cudaError_t launch_half(const Geo& g, const double* k, double* hk, cudaStream_t s);

struct SolveSpec {
  int op;             // SBM_OP_*
  int bcx0, bcx1;
  int form;
  double scale;
  const double* hk64; // FP64 half coefficient
  const double* diag64;
  const double* rhs;  // halo layout, interior used
  double* x;          // halo layout, ghosts hold Dirichlet / flux data
  const double* w;    // stop weight
  double wsum;
  int stop_rule;
  double tol;
  int max_it;
  int precision;
  int precond;
  // FP32 copies for the mixed path (may be null -> built on demand)
  const float* hk32;
  const float* diag32;
};

struct SolveResult {
  int iters;
  int outer;
  double final_res;
  float ms;
  int status;
};

}  // namespace sbm

// ------------------------------------------------------------ context
#include <map>
#include <vector>

struct sbm_ctx {
  sbm::Geo g;
  sbm::Geo g32;  // internal FP32 layout of the mixed-precision solver
  sbm_params p;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evq[2] = {nullptr, nullptr};
  // public fields (halo-padded FP64)
  double* f[SBM_F_COUNT] = {};
  // half node coefficients of the four operators (FP64)
  double *hk_kap = nullptr, *hk_pce = nullptr, *hk_pcc = nullptr, *hk_gen = nullptr;
  // step work fields (halo-padded FP64)
  double *dab = nullptr, *dab1 = nullptr, *mu = nullptr, *mb = nullptr, *pmn = nullptr;
  double *rhs = nullptr, *rhe = nullptr, *rxc = nullptr, *kfw = nullptr, *kbw = nullptr;
  double *ppo = nullptr, *peo = nullptr, *tmp = nullptr;
  // FP64 CG work: residual, direction, A*direction, Jacobi weight
  double *r64 = nullptr, *p64 = nullptr, *q64 = nullptr, *d64 = nullptr;
  // stored y / x / z face coefficients of the current FP64 operator (3 nh)
  double* fc64 = nullptr;
  // FP32 work: half coefficient, diagonal, residual, direction, A*direction, correction, z
  float *hk32 = nullptr, *dg32 = nullptr, *r32 = nullptr, *p32 = nullptr, *q32 = nullptr,
        *x32 = nullptr, *z32 = nullptr, *rold32 = nullptr;
  // double-float work (FP32 layout): low parts of the half coefficient and
  // the diagonal (their high parts are hk32 / dg32), the initial residual
  // and the accumulated correction of the mixed solver
  float *hklo32 = nullptr, *dglo32 = nullptr, *r0hi32 = nullptr, *r0lo32 = nullptr,
        *dhi32 = nullptr, *dlo32 = nullptr;
  // reductions
  double* partials = nullptr;
  sbm::CgState* st = nullptr;      // device: outer / FP64 state
  sbm::CgState* st32 = nullptr;    // device: inner FP32 state
  sbm::CgState* h_st = nullptr;    // pinned host copies [4]
  double* d_scal = nullptr;        // device scalar scratch [64]
  double* h_scal = nullptr;        // pinned host scalar scratch [64]
  // electrochemical scalars (host mirror)
  sbm_scalars sc{};
  // tuning
  int zc64 = 0, zc32 = 0, chunk = 0;
  double inner_tol = 0.0;
  int inner_max = 0;
  // CUDA graphs of captured CG chunks, keyed by solve signature
  struct GraphRec {
    cudaGraphExec_t exec;
    cudaGraph_t graph;
    int nodes;
  };
  std::map<std::string, GraphRec> graphs;
  // device-looped runs of a chunk graph (a WHILE conditional node around
  // it), keyed by the chunk graph, with the round cap they were built for
  struct LoopRec {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int cap = 0;
  };
  std::map<cudaGraph_t, LoopRec> loops;
  // arguments of the last mixed solve, replayed by sbm_bench_kernel
  sbm::OpArgs<float> last_op32{};
  int last_pc = -1;
  int no_tma = 0;  // tuning flag: use the register-tiled FP32 stencil instead of TMA
  int pc_additive = 0;  // tuning flag: additive learned preconditioner (no smoothing step)
  int host_loop = 0;    // tuning flag: mixed-solver chunks driven from the host
  // learned preconditioner plan (opaque; owned by sbm_net.cu) and the
  // preconditioner the last mixed solve actually used
  void* net = nullptr;
  int last_precond = -1;
};

namespace sbm {
int solve(sbm_ctx* ctx, const SolveSpec& spec, SolveResult* out);
// Phases of a mixed-precision solve, shared with the batched driver:
// begin launches the set-up kernels on the context stream and returns the
// captured iteration-chunk graph; end folds the correction into x.
int mixed_begin(sbm_ctx* ctx, const SolveSpec& sp, cudaGraphExec_t* ex, cudaGraph_t* graph,
                int* nodes);
int mixed_end(sbm_ctx* ctx, const SolveSpec& sp, const CgState& fin, SolveResult* out);
int status_of_done(int done);
int generic_spec(sbm_ctx* ctx, int op, int bc_x0, int bc_x1, double scale, double tol, int max_it,
                 int stop_rule, int precision, int precond, SolveSpec* sp);
int bench_kernel(sbm_ctx* ctx, int which, int reps, float* ms_per_launch, double* bytes_per_launch);
int ensure_fp32_work(sbm_ctx* ctx);
int learned_pc_apply(sbm_ctx* ctx, const SolveSpec& sp, const double* r, double* z);
void release_graphs(sbm_ctx* ctx);
// Adds to graph g (after *dep when given) a one-thread kernel node that sets
// the WHILE condition h: another round while st->done is clear and fewer
// than cap rounds ran (init: before the first round, which it counts from
// 0 in *rounds); past the cap the solve is marked as stopped by the
// iteration cap (st->done = 2).
int add_graph_loop_node(cudaGraph_t g, const cudaGraphNode_t* dep, cudaGraphConditionalHandle h,
                        CgState* st, int* rounds, int cap, int init, cudaGraphNode_t* out);
}  // namespace sbm
