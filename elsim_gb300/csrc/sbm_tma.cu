// sbm_tma.cu -- TMA-staged FP32 direction + stencil kernel of the mixed solver.
//
// One CTA owns a 64 (y) x 8 (x) tile of the FP32 layout and marches a
// tunable number of z planes (16 by default).  For every plane it brings in, with cp.async.bulk.tensor (TMA),
// a 72 x 10 box (tile + halo, x-start rounded down to a 16-byte boundary)
// of each input array: r, p_old, hk and, when present, invd (Jacobi) and the
// CnE diagonal.  Planes sit in a 5-stage shared-memory ring, each stage with
// its mbarrier (expect_tx / complete_tx); the single producer thread keeps
// one to two planes in flight ahead of the three being used (5 stages: 5
// CTAs per SM with three arrays; 0.103 ms per flexible-CG launch at 256^3
// against 0.112 ms with 6 stages and 0.113 ms with 4).  p_new = z + beta p_old
// is formed once per staged cell, in place over p_old, and the 7-point SBM
// operator reads p_new and hk from shared memory (y-neighbours by warp
// shuffle).  Each thread produces four y-consecutive voxels (float4 stores
// of p_new and q).  One block barrier per plane.
//
// The flexible-CG variant (FLEX, learned preconditioner) reads the
// preconditioned residual z in place of r and also carries two passes that
// would otherwise stream the grid on their own: the previous iteration's
// x32 += alpha p_old (p_old of the thread's own cells is kept in registers
// from the staged plane before it is overwritten; x32 is read early in the
// plane step so its latency hides behind the barrier) and the 4x4x4 means
// rq = R q of the new q (per-thread sums over the four planes of a coarse
// slab, combined across the tile's rows through shared memory; z planes per
// CTA are then a multiple of 4).  Its last block also sets
// s = RMS(R r - alpha R q), the scale of the next U-Net input, from
// |R r|^2, R r.R q and |R q|^2.
//
// Every mbarrier wait is bounded; on expiry the CTA records done = 5 in the
// solver state (reported as SBM_ERR_TIMEOUT), waits (bounded) for its own
// copies in flight and returns.  Loads use only this CTA's shared memory: no
// cluster multicast.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>

#include "sbm_async.cuh"
#include "sbm_internal.cuh"

namespace sbm {
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();
}

namespace sbm {

namespace {

constexpr int TX = 64;               // tile extent along y (voxels)
constexpr int TY = 8;                // tile extent along x (rows)
constexpr int NTH = TX / 4 * TY;     // 128 threads, one float4 each
constexpr int BOXX = TX + 8;         // 72 floats: x-start rounded down to 4
constexpr int BOXY = TY + 2;         // 10 rows
constexpr int PLANE = BOXX * BOXY;   // 720 floats
constexpr int PLANE_BYTES = PLANE * 4;
constexpr int SLOT = 2944;           // bytes per array-plane, 128-byte multiple
constexpr int NS = 5;                // stages in the ring (5 CTAs per SM fit with 3 arrays)
constexpr int ZCT = 16;              // z planes per CTA
constexpr unsigned kSpin = 1u << 20;  // try_wait attempts before giving up (about a second)

// Attempts of the consumer-side waits (the planes the CTA computes on).  The
// default is kSpin; sbm_set_wait_limit lowers it so that a test can make the
// waits run out without any fault: with 0 every consumer wait gives up at
// once.  The drain of an expired CTA always keeps the full kSpin bound, so
// no copy is still landing in shared memory when the CTA exits.
__device__ unsigned g_wait_tries = kSpin;

struct TmaMaps {
  CUtensorMap r, p, hk, iv, dg;
};

__device__ __forceinline__ float4 lds4(const float* p) {
  return *reinterpret_cast<const float4*>(p);
}

template <int FORM, bool PC, bool FLEX = false>
__global__ void __launch_bounds__(NTH)
    k32t_apply_dir(const __grid_constant__ TmaMaps maps, OpArgs<float> op, int zct,
                   float* __restrict__ pnew, float* __restrict__ q, FcgDirArgs fx,
                   double* partials, CgState* st) {
  pdl_begin();
  constexpr int NA = 3 + (PC ? 1 : 0) + (FORM == 1 ? 1 : 0);
  constexpr int A_IV = 3, A_DG = 3 + (PC ? 1 : 0);
  constexpr int RF4 = BOXX / 4;  // float4s per staged row
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ float red[FLEX ? NTH / 32 : 1][16];  // FLEX: row-pair sums of q per coarse cell
  if (st->done) return;
  const Geo g = op.g;
  const float beta = (float)st->beta;
  // FLEX: the previous iteration's x32 += alpha p_old, applied here; after a
  // residual replacement x32 is first folded into the double-float
  // correction (x32 = alpha p_old)
  const float alpha_x = FLEX ? (float)st->alpha : 0.f;
  const bool fold = FLEX && st->accum_pending != 0;
  const bool xupd = FLEX && (fold || alpha_x != 0.f);
  const unsigned FULL = 0xffffffffu;
  const int tid = threadIdx.x;
  const int ntile_y = (g.ny + TX - 1) / TX;
  const int tyb = blockIdx.x % ntile_y;
  const int txb = blockIdx.x / ntile_y;
  const int k0 = blockIdx.y * zct + 1;
  const int k1 = min(k0 + zct - 1, g.nz);
  const int nplanes = k1 - k0 + 3;  // planes k0-1 .. k1+1
  const int x0 = TX * tyb;          // box start in buffer floats
  const int y0 = TY * txb;          // box start row (= j0 - 1)
  const int q4 = tid % (TX / 4);    // float4 chunk within the row (16 per row)
  const int row = tid / (TX / 4) + 1;
  const int col = 4 + 4 * q4;
  const int i0 = TX * tyb + 4 * q4 + 1;
  const int j = TY * txb + row;
  const bool active = (i0 <= g.ny) && (j <= g.nx);
  // staged float4s each thread turns into p_new: its own cells (row `row`,
  // float4 column 1 + q4) and, for 52 threads, one of the halo float4s
  // (rows 0 and BOXY-1, float4 columns 0 and RF4-1 of the rows between)
  const int vown = row * RF4 + 1 + q4;
  int vhalo = -1;
  if (tid < 2 * RF4) {
    vhalo = tid < RF4 ? tid : (BOXY - 1) * RF4 + (tid - RF4);
  } else if (tid < 2 * RF4 + 2 * TY) {
    const int u = tid - 2 * RF4;
    vhalo = (1 + u % TY) * RF4 + (u < TY ? 0 : RF4 - 1);
  }
  auto stage = [&](int s, int a) -> float* {
    return reinterpret_cast<float*>(smem + (size_t)(s * NA + a) * SLOT);
  };
  uint64_t* const bar = reinterpret_cast<uint64_t*>(smem + (size_t)NS * NA * SLOT);
  if (tid == 0) {
    for (int s = 0; s < NS; ++s) mbar_init(&bar[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  int n_issued = 0;  // planes 0 .. n_issued-1 have been issued (thread 0)
  auto issue = [&](int m) {
    const int s = m % NS;
    n_issued = m + 1;
    const int z = k0 - 1 + m;
    mbar_expect_tx(&bar[s], NA * PLANE_BYTES);
    tma_load_3d(stage(s, 0), &maps.r, x0, y0, z, &bar[s]);
    tma_load_3d(stage(s, 1), &maps.p, x0, y0, z, &bar[s]);
    tma_load_3d(stage(s, 2), &maps.hk, x0, y0, z, &bar[s]);
    if (PC) tma_load_3d(stage(s, A_IV), &maps.iv, x0, y0, z, &bar[s]);
    if (FORM == 1) tma_load_3d(stage(s, A_DG), &maps.dg, x0, y0, z, &bar[s]);
  };
  if (tid == 0) {
    for (int m = 0; m < NS && m < nplanes; ++m) issue(m);
  }
  const unsigned tries = g_wait_tries;
  auto wait_plane = [&](int m) {
    return mbar_wait_bounded(&bar[m % NS], (unsigned)((m / NS) & 1), tries);
  };
  // p_new = z + beta p_old for every staged cell of plane m, written over
  // p_old in place (stage array 1); returns p_old of the thread's own cells
  auto make_pn = [&](int m) -> float4 {
    const float4* R = reinterpret_cast<const float4*>(stage(m % NS, 0));
    float4* P = reinterpret_cast<float4*>(stage(m % NS, 1));
    const float4* IV = reinterpret_cast<const float4*>(stage(m % NS, PC ? A_IV : 0));
    auto one = [&](int v) {
      const float4 rv = R[v], pv = P[v];
      float4 z = rv;
      if (PC) {
        const float4 d = IV[v];
        z = make_float4(d.x * rv.x, d.y * rv.y, d.z * rv.z, d.w * rv.w);
      }
      P[v] = make_float4(z.x + beta * pv.x, z.y + beta * pv.y, z.z + beta * pv.z,
                         z.w + beta * pv.w);
      return pv;
    };
    const float4 pold = one(vown);
    if (vhalo >= 0) one(vhalo);
    return pold;
  };
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 pold_nx = zero4;  // p_old of the thread's cells in the next plane
  bool ok = wait_plane(0);
  if (ok) make_pn(0);
  if (ok) ok = wait_plane(1);
  if (ok) pold_nx = make_pn(1);
  float acc = 0.f;
  // FLEX: R q of the coarse cells whose 4 y x 4 x x 4 z cells lie in this
  // tile (z planes per CTA are a multiple of 4): per-thread sums over the
  // slab's planes, row pairs by shuffle, the two pairs through `red`
  float rq_acc = 0.f;
  int slab_done = -1;  // coarse z index whose row-pair sums wait in red
  double a_cq = 0.0, a_qq = 0.0;
  auto finish_slab = [&](int kc) {  // after a block barrier
    if (tid < 32) {
      const int rg = tid >> 4, qq = tid & 15;
      const int ic = (TX / 4) * tyb + qq, jc = (TY / 4) * txb + rg;
      if (4 * ic < g.ny && 4 * jc < g.nx) {
        const float m = (red[2 * rg][qq] + red[2 * rg + 1][qq]) * (1.f / 64.f);
        const int64_t cc = ic + (int64_t)fx.rcy * (jc + (int64_t)fx.rcx * kc);
        fx.rq[cc] = m;
        a_cq += (double)fx.rc[cc] * (double)m;
        a_qq += (double)m * (double)m;
      }
    }
  };
  const int o = row * BOXX + col;
  for (int mk = 1; mk <= nplanes - 2; ++mk) {
    const int k = k0 - 1 + mk;
    const int64_t c = g.ix(i0, j, k);
    // FLEX: this plane's x32 is read before the barrier (latency hidden)
    float4 xv = zero4;
    if (xupd && active) xv = *reinterpret_cast<const float4*>(fx.x32 + c);
    const float4 pold = pold_nx;
    const bool w = ok && wait_plane(mk + 1);
    if (w) pold_nx = make_pn(mk + 1);
    // one barrier per plane: p_new of mk+1 is complete, and every thread has
    // finished step mk-1, so the stage of plane mk-2 can be refilled.  The
    // barrier also makes the give-up decision of the bounded waits uniform.
    if (!__syncthreads_and(w)) {
      ok = false;
      break;
    }
    if (FLEX && slab_done >= 0) {
      finish_slab(slab_done);
      slab_done = -1;
    }
    if (tid == 0 && mk >= 2 && mk - 2 + NS < nplanes) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(mk - 2 + NS);
    }
    const float* PM = stage((mk - 1) % NS, 1);
    const float* PCc = stage(mk % NS, 1);
    const float* PP = stage((mk + 1) % NS, 1);
    const float* HM = stage((mk - 1) % NS, 2);
    const float* HC = stage(mk % NS, 2);
    const float* HP = stage((mk + 1) % NS, 2);
    const float4 pc = lds4(PCc + o);
    const float4 kc = lds4(HC + o);
    // y-neighbours from the adjacent chunk of the same row (lane +-1 within
    // the 16 lanes of the row), scalar loads only at the row's ends
    float pl = __shfl_up_sync(FULL, pc.w, 1), kl = __shfl_up_sync(FULL, kc.w, 1);
    float pr = __shfl_down_sync(FULL, pc.x, 1), kr = __shfl_down_sync(FULL, kc.x, 1);
    if (q4 == 0) {
      pl = PCc[o - 1];
      kl = HC[o - 1];
    }
    if (q4 == TX / 4 - 1) {
      pr = PCc[o + 4];
      kr = HC[o + 4];
    }
    if (active) {
      float4 pxm = lds4(PCc + o - BOXX), pxp = lds4(PCc + o + BOXX);
      float4 pzm = lds4(PM + o), pzp = lds4(PP + o);
      const float4 kxm = lds4(HC + o - BOXX), kxp = lds4(HC + o + BOXX);
      const float4 kzm = lds4(HM + o), kzp = lds4(HP + o);
      if (i0 == 1) pl = pc.x;
      if (i0 + 3 == g.ny) pr = pc.w;
      if (j == 1) pxm = op.bcx0 ? zero4 : pc;
      if (j == g.nx) pxp = op.bcx1 ? zero4 : pc;
      if (k == 1) pzm = pc;
      if (k == g.nz) pzp = pc;
      const float pa[6] = {pl, pc.x, pc.y, pc.z, pc.w, pr};
      const float ka[6] = {kl, kc.x, kc.y, kc.z, kc.w, kr};
      const float pxa[4] = {pxm.x, pxm.y, pxm.z, pxm.w}, pxb[4] = {pxp.x, pxp.y, pxp.z, pxp.w};
      const float kxa[4] = {kxm.x, kxm.y, kxm.z, kxm.w}, kxb[4] = {kxp.x, kxp.y, kxp.z, kxp.w};
      const float pza[4] = {pzm.x, pzm.y, pzm.z, pzm.w}, pzb[4] = {pzp.x, pzp.y, pzp.z, pzp.w};
      const float kza[4] = {kzm.x, kzm.y, kzm.z, kzm.w}, kzb[4] = {kzp.x, kzp.y, kzp.z, kzp.w};
      float dg[4] = {0.f, 0.f, 0.f, 0.f};
      if (FORM == 1) {
        const float4 d4 = lds4(stage(mk % NS, A_DG) + o);
        dg[0] = d4.x; dg[1] = d4.y; dg[2] = d4.z; dg[3] = d4.w;
      }
      float qa[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float s = face_sum<float>(ka[e + 1], pa[e + 1], ka[e + 2], pa[e + 2], ka[e], pa[e],
                                        kxb[e], pxb[e], kxa[e], pxa[e], kzb[e], pzb[e], kza[e],
                                        pza[e]);
        qa[e] = (FORM == 0) ? op.scale * s : dg[e] * pa[e + 1] - op.scale * s;
      }
      *reinterpret_cast<float4*>(pnew + c) = pc;
      *reinterpret_cast<float4*>(q + c) = make_float4(qa[0], qa[1], qa[2], qa[3]);
      acc += (pa[1] * qa[0] + pa[2] * qa[1]) + (pa[3] * qa[2] + pa[4] * qa[3]);
      if (FLEX) {
        rq_acc += (qa[0] + qa[1]) + (qa[2] + qa[3]);
        if (xupd) {
          if (fold) {
            const float4 dh = *reinterpret_cast<const float4*>(fx.dhi + c);
            const float4 dl = *reinterpret_cast<const float4*>(fx.dlo + c);
            const DF d0 = df_add_f(DF{dh.x, dl.x}, xv.x), d1 = df_add_f(DF{dh.y, dl.y}, xv.y);
            const DF d2 = df_add_f(DF{dh.z, dl.z}, xv.z), d3 = df_add_f(DF{dh.w, dl.w}, xv.w);
            *reinterpret_cast<float4*>(fx.dhi + c) = make_float4(d0.hi, d1.hi, d2.hi, d3.hi);
            *reinterpret_cast<float4*>(fx.dlo + c) = make_float4(d0.lo, d1.lo, d2.lo, d3.lo);
            xv = make_float4(alpha_x * pold.x, alpha_x * pold.y, alpha_x * pold.z,
                             alpha_x * pold.w);
          } else {
            xv.x += alpha_x * pold.x;
            xv.y += alpha_x * pold.y;
            xv.z += alpha_x * pold.z;
            xv.w += alpha_x * pold.w;
          }
          *reinterpret_cast<float4*>(fx.x32 + c) = xv;
        }
      }
    }
    if (FLEX && (k & 3) == 0) {  // k = 4 kc + 4 closes coarse slab kc
      const float v = rq_acc + __shfl_xor_sync(FULL, rq_acc, 16);  // rows 2w+1 and 2w+2
      if ((tid & 31) < 16) red[tid >> 5][tid & 15] = v;
      rq_acc = 0.f;
      slab_done = (k - 1) >> 2;
    }
  }
  // Every thread must agree before the reduction: a CTA whose wait expired
  // records the error and drains its own copies in flight.
  const int failed = __syncthreads_or(ok ? 0 : 1);
  if (failed) {
    if (tid == 0) {
      st->done = 5;
      // Planes land in issue order per stage, and a stage is refilled only
      // after every thread waited for its previous plane, so each stage has
      // at most its last issued plane outstanding: wait for that phase.
      for (int s = 0; s < NS && s < n_issued; ++s) {
        const int last = s + ((n_issued - 1 - s) / NS) * NS;
        mbar_wait_bounded(&bar[s], (unsigned)((last / NS) & 1), kSpin);
      }
    }
    __syncthreads();
    acc = 0.f;
    a_cq = a_qq = 0.0;
  } else if (FLEX && slab_done >= 0) {
    finish_slab(slab_done);
  }
  if (FLEX) {
    double v[3] = {(double)acc, a_cq, a_qq}, tot[3];
    if (grid_reduce<3>(v, partials, &st->counter[0], tot)) {
      if (threadIdx.x == 0) {
        const double pq = tot[0];
        const double alpha = st->rho / pq;
        st->pq = pq;
        st->alpha = alpha;
        st->accum_pending = 0;
        // s = RMS(R r - alpha R q) over the valid coarse cells, |R r|^2 in
        // aux[2]: the scale of the next U-Net input; |R r - alpha R q|^2
        // becomes the next |R r|^2
        const double ss2 = st->aux[2] - 2.0 * alpha * tot[1] + alpha * alpha * tot[2];
        const double sc = ss2 > 0.0 ? sqrt(ss2 / (double)fx.ncell) : 0.0;
        st->aux[2] = ss2 > 0.0 ? ss2 : 0.0;  // |R r|^2 after the pack applies alpha R q
        fx.scal[0] = (float)sc;
        fx.scal[1] = sc > 0.0 ? (float)(1.0 / sc) : 0.f;
        if (st->done == 0) {
          if (pq == 0.0) st->done = 4;
          else if (!isfinite(pq)) st->done = 3;
        }
      }
    }
    return;
  }
  double v[1] = {(double)acc}, tot[1];
  if (grid_reduce<1>(v, partials, &st->counter[0], tot)) {
    if (threadIdx.x == 0) {
      const double pq = tot[0];
      st->pq = pq;
      st->alpha = st->rho / pq;
      if (st->done == 0) {
        if (pq == 0.0) st->done = 4;
        else if (!isfinite(pq)) st->done = 3;
      }
    }
  }
}

size_t smem_bytes(int pc, int form) {
  const int na = 3 + pc + form;
  return (size_t)NS * na * SLOT + NS * sizeof(uint64_t);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() { return tensor_map_encoder(); }

// 3-D map over an FP32-layout buffer (base = allocation start, 16-byte aligned).
bool make_map(CUtensorMap* m, const float* base, const Geo& g32) {
  auto fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[3] = {(cuuint64_t)g32.sx, (cuuint64_t)(g32.nx + 2), (cuuint64_t)(g32.nz + 2)};
  cuuint64_t strides[2] = {(cuuint64_t)g32.sx * 4, (cuuint64_t)g32.sz * 4};
  cuuint32_t box[3] = {BOXX, BOXY, 1};
  cuuint32_t es[3] = {1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims,
                        strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace

bool make_map_box(CUtensorMap* m, const float* base, const Geo& g32, int bx, int by, int bz) {
  auto fn = tensor_map_encoder();
  if (!fn) return false;
  cuuint64_t dims[3] = {(cuuint64_t)g32.sx, (cuuint64_t)(g32.nx + 2), (cuuint64_t)(g32.nz + 2)};
  cuuint64_t strides[2] = {(cuuint64_t)g32.sx * 4, (cuuint64_t)g32.sz * 4};
  cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
  cuuint32_t es[3] = {1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims,
                        strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// The CUDA driver API's tensor-map encoder (runtime entry-point query, once).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// Occupancy of one instantiation of the direction kernel.
int dir_blocks_per_sm(int pc, int form, bool flex, size_t smem) {
  int per_sm = 0;
  cudaError_t e;
  if (flex)
    e = form ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k32t_apply_dir<1, false, true>, NTH, smem)
             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k32t_apply_dir<0, false, true>, NTH, smem);
  else if (form == 0)
    e = pc ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k32t_apply_dir<0, true>, NTH, smem)
           : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k32t_apply_dir<0, false>, NTH, smem);
  else
    e = pc ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k32t_apply_dir<1, true>, NTH, smem)
           : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k32t_apply_dir<1, false>, NTH, smem);
  return e == cudaSuccess ? per_sm : 0;
}

// z planes per CTA when not tuned: the launch should fill whole waves of
// resident CTAs (a last, partly filled wave leaves SMs idle), and each CTA
// also streams 2 halo planes, so minimise waves x (planes + 2) over 8..32
// (multiples of 4 for the flexible-CG variant, whose CTAs own whole coarse
// slabs).
int auto_zct(int ntile, int nz, int pc, int form, bool flex) {
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int per_sm = dir_blocks_per_sm(pc, form, flex, smem_bytes(pc, form));
  if (per_sm < 1) return ZCT;
  const int64_t cap = (int64_t)nsm * per_sm;
  // One wave when the columns allow it: the most z chunks whose CTAs are all
  // resident at once (a partly filled last wave runs at a fraction of the
  // bandwidth; 256^3 flexible-CG direction kernel: 0.0978 ms with 5 chunks
  // of 52 planes, one wave of 640 CTAs, against 0.1047 ms with 11 chunks of
  // 24 in 1.85 waves, 0.111 / 0.115 ms with 16 / 32 planes).  At least 8
  // planes per CTA, so that the two halo planes stay a small part of it.
  const int64_t chunks = cap / ntile;
  if (chunks >= 1) {
    int z = (int)((nz + chunks - 1) / chunks);
    if (flex) z = (z + 3) / 4 * 4;
    return z >= 8 ? z : 8;
  }
  int best = ZCT;
  int64_t best_cost = -1;
  for (int z = 8; z <= 32; z += flex ? 4 : 1) {
    const int64_t ctas = (int64_t)ntile * ((nz + z - 1) / z);
    const int64_t cost = ((ctas + cap - 1) / cap) * (int64_t)(std::min(z, nz) + 2);
    if (best_cost < 0 || cost < best_cost || (cost == best_cost && z > best)) {
      best = z;
      best_cost = cost;
    }
  }
  return best;
}

// The TMA path needs rows of a multiple of 4 voxels (float4 output) and
// 16-byte row strides (always true of the FP32 layout).
bool tma_supported(const Geo& g32) { return (g32.ny % 4) == 0 && (g32.sx % 4) == 0 && encode_fn(); }

struct TmaPlan {
  TmaMaps fwd, bwd;  // fwd reads p buffer a, bwd reads buffer b
  dim3 grid;
  size_t smem;
  int pc, form, zct, flex;
};

// Builds the tensor maps of one mixed solve.  Buffers are allocation bases
// (the FP32 layout's element (i,j,k) sits at base + kOff32 + g32.ix(i,j,k)).
// flex: the flexible-CG variant (no Jacobi array; zct a multiple of 4, and
// every extent a multiple of 4).
int tma_plan(const Geo& g32, const float* r, const float* pa, const float* pb, const float* hk,
             const float* iv, const float* dg, int pc, int form, int zct, int flex,
             TmaPlan* plan) {
  memset(plan, 0, sizeof(*plan));
  if (flex && (pc || g32.nx % 4 || g32.nz % 4)) return SBM_ERR_STATE;
  if (!make_map(&plan->fwd.r, r, g32) || !make_map(&plan->fwd.p, pa, g32) ||
      !make_map(&plan->fwd.hk, hk, g32) || (pc && !make_map(&plan->fwd.iv, iv, g32)) ||
      (form && !make_map(&plan->fwd.dg, dg, g32)))
    return SBM_ERR_STATE;
  plan->bwd = plan->fwd;
  if (!make_map(&plan->bwd.p, pb, g32)) return SBM_ERR_STATE;
  const int ntile = ((g32.ny + TX - 1) / TX) * ((g32.nx + TY - 1) / TY);
  if (zct < 1) zct = auto_zct(ntile, g32.nz, pc, form, flex != 0);
  if (flex) zct = (zct + 3) / 4 * 4;
  plan->zct = zct;
  plan->grid = dim3((unsigned)ntile, (unsigned)((g32.nz + zct - 1) / zct));
  plan->pc = pc;
  plan->form = form;
  plan->flex = flex;
  plan->smem = smem_bytes(pc, form);
  return SBM_OK;
}

int tma_plan_size(void) { return (int)sizeof(TmaPlan); }

// Sets the dynamic shared-memory limit of the six instantiations (once).
int tma_init() {
  static bool done = false;
  if (done) return SBM_OK;
  SBM_CUDA_TRY(cudaFuncSetAttribute(k32t_apply_dir<0, false>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes(0, 0)));
  SBM_CUDA_TRY(cudaFuncSetAttribute(k32t_apply_dir<0, true>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes(1, 0)));
  SBM_CUDA_TRY(cudaFuncSetAttribute(k32t_apply_dir<1, false>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes(0, 1)));
  SBM_CUDA_TRY(cudaFuncSetAttribute(k32t_apply_dir<1, true>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes(1, 1)));
  SBM_CUDA_TRY(cudaFuncSetAttribute(k32t_apply_dir<0, false, true>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes(0, 0)));
  SBM_CUDA_TRY(cudaFuncSetAttribute(k32t_apply_dir<1, false, true>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes(0, 1)));
  done = true;
  return SBM_OK;
}

// One launch: reads p from buffer a (fwd) or b (!fwd), writes p_new to pnew.
void tma_launch(const TmaPlan& plan, bool fwd, const OpArgs<float>& op, float* pnew, float* q,
                double* partials, CgState* st, cudaStream_t s) {
  const TmaMaps& m = fwd ? plan.fwd : plan.bwd;
  const FcgDirArgs none{};
  if (plan.form == 0) {
    if (plan.pc) k32t_apply_dir<0, true><<<plan.grid, NTH, plan.smem, s>>>(m, op, plan.zct, pnew, q, none, partials, st);
    else k32t_apply_dir<0, false><<<plan.grid, NTH, plan.smem, s>>>(m, op, plan.zct, pnew, q, none, partials, st);
  } else {
    if (plan.pc) k32t_apply_dir<1, true><<<plan.grid, NTH, plan.smem, s>>>(m, op, plan.zct, pnew, q, none, partials, st);
    else k32t_apply_dir<1, false><<<plan.grid, NTH, plan.smem, s>>>(m, op, plan.zct, pnew, q, none, partials, st);
  }
}

// One launch of the flexible-CG variant (plan built with flex), with
// programmatic dependent launch inside the captured loop.
void tma_launch_fcg(const TmaPlan& plan, bool fwd, const OpArgs<float>& op, float* pnew, float* q,
                    const FcgDirArgs& fx, double* partials, CgState* st, cudaStream_t s) {
  const TmaMaps& m = fwd ? plan.fwd : plan.bwd;
  if (plan.form == 0)
    launch_pdl(k32t_apply_dir<0, false, true>, plan.grid, dim3(NTH), plan.smem, s, m, op,
               plan.zct, pnew, q, fx, partials, st);
  else
    launch_pdl(k32t_apply_dir<1, false, true>, plan.grid, dim3(NTH), plan.smem, s, m, op,
               plan.zct, pnew, q, fx, partials, st);
}

}  // namespace sbm

// Test hook of the bounded waits (no counterpart in the reference): sets how
// many times the consumer-side mbarrier waits of the TMA-staged stencil
// kernel try before giving up, on the current device; tries < 0 restores the
// built-in bound.  With 0 every launch of the kernel records SBM_ERR_TIMEOUT
// without touching its outputs; its CTAs still wait out their own copies.
extern "C" int sbm_set_wait_limit(int tries) {
  const unsigned v = tries < 0 ? sbm::kSpin : (unsigned)tries;
  SBM_CUDA_TRY(cudaMemcpyToSymbol(sbm::g_wait_tries, &v, sizeof(v)));
  return SBM_OK;
}
