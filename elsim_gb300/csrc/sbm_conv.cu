// sbm_conv.cu -- BF16 3x3x3 convolution on the 5th-generation tensor cores.
//
// Forward / data-gradient kernel (k_conv3_tc): implicit GEMM with rows
// (M) = 128 voxels of a grid stored channels-last (x[v*C + c],
// v = i + ny*(j + nx*k)), columns (N) = up to 64 output channels per CTA,
// reduction (K) = 27 taps x input channels.  The input tile with its halo is
// staged once per 16-channel chunk and the 27 tap MMAs read it through
// shifted UMMA descriptors (see the kernel).  One elected thread issues the
// MMAs with FP32 accumulation in tensor memory and commits them to the
// stage's mbarrier; the epilogue reads the accumulator with tcgen05.ld (each
// warp its 32 lanes), adds the bias, optionally applies ReLU and stores BF16
// or FP32 into a channel slice of the output.
//
// Weight-gradient kernel (k_wgrad_tc): GEMM with rows = (tap, input
// channel) pairs, columns = output channels, reduction = voxels.
//
// Operands are BF16 x BF16 -> FP32 only.  Every mbarrier wait is bounded;
// on expiry the CTA sets an error flag, frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <vector>

#include "sbm_conv.cuh"

namespace sbm {

namespace {

constexpr int TM = 128;          // voxels per CTA (MMA M)
constexpr int NTHR = 128;        // 4 warps
constexpr int KS = 16;           // K per MMA (BF16)
constexpr int NSTG = 4;          // stages
constexpr int A_BYTES = TM * KS * 2;   // 4096
constexpr unsigned kSpinTc = 1u << 20;
// halo-tiled forward kernel
constexpr int TY = 8, TX = 16;                  // voxel tile (y, x), one z plane
constexpr int HY = TY + 2, HX = TX + 2;        // halo tile in y, x (P + 2 planes in z)
// slot of one 8-channel half of the halo tile of P planes, 128-byte aligned
__host__ __device__ constexpr int a_half_bytes(int P) {
  return (HY * HX * (P + 2) * 16 + 127) / 128 * 128;
}
constexpr int NT_MAX = 64;                      // output channels per CTA (wide tiles)
constexpr int NST = 8;                          // most pipeline stages (<= 7 chunks used)
constexpr int kSmemBudget = 200 * 1024;         // stage memory of a lone CTA
#ifndef SBM_CONV_WAVE_STAGES
#define SBM_CONV_WAVE_STAGES 1
#endif
constexpr int kWaveStages = SBM_CONV_WAVE_STAGES;  // stages per CTA when the grid has several waves

__device__ __forceinline__ uint32_t sa(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// UMMA shared-memory descriptor: start address, leading (K) and stride (M/N)
// byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // version
  // base offset 0, lbo mode 0, layout type 0 (no swizzle)
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = 128, N = n.
__host__ __device__ __forceinline__ uint32_t idesc_bf16(int n) {
  uint32_t d = 0;
  d |= 1u << 4;                       // D format: F32
  d |= 1u << 7;                       // A format: BF16
  d |= 1u << 10;                      // B format: BF16
  d |= (uint32_t)(n >> 3) << 17;      // N >> 3
  d |= (uint32_t)(TM >> 4) << 24;     // M >> 4
  return d;
}

__device__ __forceinline__ void mb_init(uint64_t* b) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sa(b)) : "memory");
}

__device__ __forceinline__ bool mb_try(uint64_t* b, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(sa(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mb_wait(uint64_t* b, unsigned parity) {
  for (unsigned n = 0; n < kSpinTc; ++n)
    if (mb_try(b, parity)) return true;
  return false;
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t id,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(id), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(sa(bar))
      : "memory");
}

// 16 consecutive FP32 accumulator columns of this thread's lane.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

}  // namespace

namespace {

// Halo-tiled implicit GEMM fed by TMA.  A CTA owns a tile of TY x TX voxels
// in P = 1 or 2 z planes (per plane M = 128 rows, row m = voxel
// (y0 + m%8, x0 + m/8), its own TMEM accumulator) and NT <= 64 output
// channels.  For each 16-channel input chunk two tensor-map loads bring the
// (TY+2) x (TX+2) x (P+2) halo tile into shared memory (one
// 8-channel half each, zero outside the grid and the sample), which is
// exactly the canonical K-major operand layout: 8 consecutive y voxels x 16
// bytes form a core matrix, x lines are HY*16 bytes apart, the halves
// A_HALF bytes apart.  A bulk copy brings the chunk's weights for all 27
// taps (pre-arranged image).  The 27 tap MMAs read the tile through
// shifted descriptor start addresses: tap (dy, dx, dz) starts
// (dy + HY*(dx + HX*dz)) * 16 bytes further, with the same strides, so the
// input is read ~4x (halo) instead of 27x; the second plane's MMAs start
// one plane (HX*HY*16 bytes) further.  Thread 0 is producer and MMA issuer
// over an NST-stage ring (full / consumed mbarriers).  The epilogue can
// also write the 2x2x2-pooled output (planes in registers, y / x pairs by
// warp shuffle), the output copied to the 8 children of a 2x finer grid
// (nearest upsampling into a decoder's concat buffer), and a fused 1x1
// output layer.
__device__ __forceinline__ void tma_load5(void* dst, const CUtensorMap* map, uint64_t* bar, int c0,
                                          int c1, int c2, int c3, int c4) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(sa(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4),
      "r"(sa(bar))
      : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes,
                                          uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(sa(dst)),
      "l"(src), "r"(bytes), "r"(sa(bar))
      : "memory");
}

__device__ __forceinline__ void expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(bar)), "r"(bytes)
               : "memory");
}

// Adds to the transaction count of the current phase without arriving (the
// arrival follows with the stage's remaining copies).
__device__ __forceinline__ void expect_tx_only(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(sa(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mb_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(sa(bar)) : "memory");
}

// The tap MMAs of one chunk.  A descriptor = halo plane 0 at offset
// (0, 0); B descriptor = the chunk's weight image.  Descriptors advance by
// constant start-address offsets (the 14-bit start field holds address /
// 16): halo plane h, in-plane offset (dy, dx) at ((h*HX + 1+dx)*HY + 1+dy)
// units, B block q at 6 nt units and B row r at 2 r units.  One plane: 27
// MMAs of N = nt.  Two planes (accumulators at columns 0 and nt): per
// (dy, dx) four MMAs, halo planes 1 and 2 with N = 2 nt feeding both
// accumulators (rows [W0 | W-1] and [W+1 | W0]), planes 0 and 3 with N = nt.
// Four planes (accumulators at 0, nt, 2nt, 3nt): halo plane h feeds the
// outputs h-2 .. h with dz = +1, 0, -1, so planes 2 and 3 are one MMA of
// N = 3 nt over rows [W+1 | W0 | W-1] each; planes 1 and 4 (N = 2 nt) come
// first, as each of them starts two accumulators that no earlier MMA of the
// chunk touched.
__device__ __forceinline__ void issue_taps(uint32_t tmem, uint64_t ad, uint64_t bd, int nt, int P,
                                           uint32_t id1, uint32_t id2, uint32_t id3, bool acc) {
#pragma unroll
  for (int qq = 0; qq < 9; ++qq) {
    const int dy = qq % 3 - 1, dx = qq / 3 - 1;
    const uint64_t a0 = ad + (uint64_t)((1 + dx) * HY + (1 + dy));
    const uint64_t b = bd + (uint64_t)(qq * 6 * nt);
    const uint32_t first = (acc || qq > 0) ? 1u : 0u;
    if (P == 1) {
      // plane z0 + dz is halo plane 1 + dz; its weights are rows (1 - dz) nt
      tc_mma(tmem, a0 + (uint64_t)(1 * HX * HY), b + (uint64_t)(2 * nt), id1, first);  // dz = 0
      tc_mma(tmem, a0, b + (uint64_t)(4 * nt), id1, 1u);                               // dz = -1
      tc_mma(tmem, a0 + (uint64_t)(2 * HX * HY), b, id1, 1u);                          // dz = +1
    } else if (P == 2) {
      tc_mma(tmem, a0 + (uint64_t)(1 * HX * HY), b + (uint64_t)(2 * nt), id2, first);  // h = 1
      tc_mma(tmem, a0, b + (uint64_t)(4 * nt), id1, 1u);                               // h = 0
      tc_mma(tmem, a0 + (uint64_t)(2 * HX * HY), b, id2, 1u);                          // h = 2
      tc_mma(tmem + (uint32_t)nt, a0 + (uint64_t)(3 * HX * HY), b, id1, 1u);           // h = 3
    } else {
      const uint32_t hs = (uint32_t)(HX * HY);
      tc_mma(tmem, a0 + 1 * hs, b + (uint64_t)(2 * nt), id2, first);           // h = 1: o0, o1
      tc_mma(tmem + (uint32_t)(2 * nt), a0 + 4 * hs, b, id2, first);           // h = 4: o2, o3
      tc_mma(tmem, a0, b + (uint64_t)(4 * nt), id1, 1u);                       // h = 0: o0
      tc_mma(tmem, a0 + 2 * hs, b, id3, 1u);                                   // h = 2: o0..o2
      tc_mma(tmem + (uint32_t)nt, a0 + 3 * hs, b, id3, 1u);                    // h = 3: o1..o3
      tc_mma(tmem + (uint32_t)(3 * nt), a0 + 5 * hs, b, id1, 1u);              // h = 5: o3
    }
  }
}

// Epilogue of one output tile: thread m (0..127) of the four warps that
// read TMEM lanes 32 (m / 32) .. + 31 owns voxel row m (y = y0 + m % 8,
// x = x0 + m / 8) of every plane; accumulator columns of plane pl start at
// tacc + pl nt.  Bias, ReLU, BF16 / FP32 stores, the fused 2x2x2 pooling
// (y and x pairs by warp shuffle), nearest upsampling into the finer
// concat buffer and the fused 1x1 output layer.  Warp shuffles only: no
// block barrier, so a subset of warps can run it.
__device__ __forceinline__ void conv_epilogue(const ConvArgs& a, uint32_t tacc, int m, int y0,
                                              int x0, int z0, int zl, int n0, int nt, int P) {
  const int tid = m;
  const int warp = m >> 5;
  const uint32_t tmem = tacc;
  const unsigned FULL = 0xffffffffu;
  const int64_t V = (int64_t)a.ny * a.nx * a.nz;
  const int y = y0 + (tid & 7), x = x0 + (tid >> 3);
  const bool valid = y < a.ny && x < a.nx;
  const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
  float head[4] = {0.f, 0.f, 0.f, 0.f};  // fused 1x1 output layer, per plane
  for (int c0 = 0; c0 < nt; c0 += 16) {
    __align__(16) __nv_bfloat16 o[4][16];
    for (int pl = 0; pl < P; ++pl) {
      float acc[16];
      tc_ld16(lane_base + (uint32_t)(pl * nt + c0), acc);
      const int64_t v = (int64_t)y + (int64_t)a.ny * (x + (int64_t)a.nx * (z0 + pl));
      // voxels in the zero padding of a padded grid keep zero outputs, as
      // the zero fill beyond a grid face would present them
      const bool live =
          a.vny == 0 || (y < a.vny && x < a.vnx && (zl + pl) < a.vnz);
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        float val = acc[q] + (a.bias ? a.bias[n0 + c0 + q] : 0.f);
        if (a.relu) val = fmaxf(val, 0.f);
        if (!live) val = 0.f;
        o[pl][q] = __float2bfloat16_rn(val);
        acc[q] = val;
        if (a.w1x1) head[pl] += a.w1x1[n0 + c0 + q] * __bfloat162float(o[pl][q]);
      }
      if (!valid) continue;
      const int ch = a.offy + n0 + c0;
      if (a.y16) {
        *reinterpret_cast<uint4*>(a.y16 + act_index(v, ch, V)) =
            *reinterpret_cast<const uint4*>(&o[pl][0]);
        *reinterpret_cast<uint4*>(a.y16 + act_index(v, ch + 8, V)) =
            *reinterpret_cast<const uint4*>(&o[pl][8]);
      }
      if (a.y32) {
        float4* d0 = reinterpret_cast<float4*>(a.y32 + act_index(v, ch, V));
        float4* d1 = reinterpret_cast<float4*>(a.y32 + act_index(v, ch + 8, V));
        d0[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
        d0[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
        d1[0] = make_float4(acc[8], acc[9], acc[10], acc[11]);
        d1[1] = make_float4(acc[12], acc[13], acc[14], acc[15]);
      }
      if (a.up) {
        // nearest upsampling: the 8 children in the finer grid
        const int fy = 2 * a.ny, fx = 2 * a.nx;
        for (int ch = 0; ch < 8; ++ch) {
          const int cy = 2 * y + (ch & 1), cxx = 2 * x + ((ch >> 1) & 1);
          const int czl = 2 * (zl + pl) + (ch >> 2);
          const int64_t u = (int64_t)cy +
                            (int64_t)fy * (cxx + (int64_t)fx * (2 * (z0 + pl) + (ch >> 2)));
          const int cu = a.offu + n0 + c0;
          const bool ulive = a.uvny == 0 || (cy < a.uvny && cxx < a.uvnx && czl < a.uvnz);
          const uint4 zero4 = make_uint4(0u, 0u, 0u, 0u);
          *reinterpret_cast<uint4*>(a.up + act_index(u, cu, 8 * V)) =
              ulive ? *reinterpret_cast<const uint4*>(&o[pl][0]) : zero4;
          *reinterpret_cast<uint4*>(a.up + act_index(u, cu + 8, 8 * V)) =
              ulive ? *reinterpret_cast<const uint4*>(&o[pl][8]) : zero4;
        }
      }
    }
    // 2x2x2 average: plane pairs in registers, y pairs lane^1, x pairs lane^8
    for (int pp = 0; a.pool && pp < P; pp += 2) {
      __align__(16) __nv_bfloat16 pv[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        float sum = __bfloat162float(o[pp][q]) + __bfloat162float(o[pp + 1][q]);
        sum += __shfl_xor_sync(FULL, sum, 1);
        sum += __shfl_xor_sync(FULL, sum, 8);
        pv[q] = __float2bfloat16_rn(sum * 0.125f);
      }
      if (valid && (tid & 1) == 0 && ((tid >> 3) & 1) == 0) {
        const int cy = a.ny / 2, cx = a.nx / 2;
        const int64_t vc =
            (int64_t)(y / 2) + (int64_t)cy * ((x / 2) + (int64_t)cx * ((z0 + pp) / 2));
        *reinterpret_cast<uint4*>(a.pool + act_index(vc, n0 + c0, V / 8)) =
            *reinterpret_cast<const uint4*>(&pv[0]);
        *reinterpret_cast<uint4*>(a.pool + act_index(vc, n0 + c0 + 8, V / 8)) =
            *reinterpret_cast<const uint4*>(&pv[8]);
      }
    }
  }
  if (a.w1x1 && valid) {
    for (int pl = 0; pl < P; ++pl) {
      const int64_t v = (int64_t)y + (int64_t)a.ny * (x + (int64_t)a.nx * (z0 + pl));
      a.out1x1[v] = head[pl] + a.b1x1[0];
    }
  }
}

__global__ void __launch_bounds__(NTHR) k_conv3_tc(const __grid_constant__ ConvMap m, ConvArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int P = a.planes;  // z planes per CTA (1, 2 or 4), one accumulator each
  const int ahalf = a_half_bytes(P);
  const int n0 = blockIdx.y * a.tw;
  const int nt = min(a.tw, a.cout - n0);
  const int bbytes = 27 * nt * 32;
  const int stage_bytes = 2 * ahalf + bbytes;
  const int nchunk = a.cin / KS;
  const int nst = a.nst;
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + nst * stage_bytes);
  uint64_t* used = full + NST;
  uint64_t* done = used + NST;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int nty = (a.ny + TY - 1) / TY, ntx = (a.nx + TX - 1) / TX;
  const int ty = blockIdx.x % nty;
  const int tx = (blockIdx.x / nty) % ntx;
  const int z0 = (blockIdx.x / (nty * ntx)) * P;
  const int y0 = ty * TY, x0 = tx * TX;
  const int zl = z0 % a.nzs, sample = z0 / a.nzs;
  const int ncols = P * nt <= 32 ? 32 : (P * nt <= 64 ? 64 : (P * nt <= 128 ? 128 : 256));
  // Set-up that reads nothing the preceding kernels write runs before
  // griddepcontrol.wait, overlapping their tail: the barriers, the
  // tensor-map prefetch and, when the weights are frozen (a.wpre), the
  // weight copies of the first stages.  Tensor memory is allocated only
  // after the wait: a CTA waiting on an earlier grid holds none, so it can
  // never keep a CTA of that grid from allocating.
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const __nv_bfloat16* wsrc =
      (a.tw == 16 ? a.wimg16 : a.wimg) + (int64_t)a.tw * blockIdx.y * 27 * a.cin;
  const int npre = a.wpre ? min(nchunk, nst) : 0;  // chunks whose weights are already on the way
  if (tid == 0) {
    for (int s = 0; s < 2 * NST + 1; ++s) mb_init(&full[s]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&m.x)) : "memory");
    for (int c = 0; c < npre; ++c) {
      expect_tx_only(&full[c], bbytes);
      bulk_load(sm + c * stage_bytes + 2 * ahalf, wsrc + (int64_t)c * 27 * nt * 16, bbytes,
                &full[c]);
    }
  }
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if ((a.skip && *a.skip) || (a.skip2 && *a.skip2)) {
    // the flag is the same for every thread; the copies in flight land
    // before the CTA exits
    if (tid == 0) {
      for (int c = 0; c < npre; ++c) {
        mb_arrive(&full[c]);
        mb_wait(&full[c], 0);
      }
    }
    return;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     sa(tslot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  bool ok = true;
  if (tid == 0) {
    const uint32_t id = idesc_bf16(nt), id2 = idesc_bf16(2 * nt), id3 = idesc_bf16(3 * nt);
    const unsigned abox = (unsigned)(HY * HX * (P + 2) * 16);
    int issued[NST] = {}, landed[NST] = {}, committed[NST] = {}, freed[NST] = {};
    auto load = [&](int c, int s) {
      unsigned char* A = sm + s * stage_bytes;
      const bool pre = c < npre;  // weights issued before the wait
      expect_tx(&full[s], 2 * abox + (pre ? 0u : (unsigned)bbytes));
      const int grp = (a.offx + c * KS) >> 3;
      tma_load5(A, &m.x, &full[s], 8 * (y0 - 1), x0 - 1, zl - 1, sample, grp);
      tma_load5(A + ahalf, &m.x, &full[s], 8 * (y0 - 1), x0 - 1, zl - 1, sample, grp + 1);
      if (!pre) bulk_load(A + 2 * ahalf, wsrc + (int64_t)c * 27 * nt * 16, bbytes, &full[s]);
      ++issued[s];
    };
    for (int c = 0; c < nchunk && c < nst; ++c) load(c, c);
    for (int c = 0; c < nchunk; ++c) {
      const int s = c % nst;
      if (!mb_wait(&full[s], (unsigned)(landed[s] & 1))) {
        ok = false;
        break;
      }
      ++landed[s];
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t A = sa(sm + s * stage_bytes);
      const uint64_t ad = umma_desc(A, ahalf, HY * 16);
      const uint64_t bd = umma_desc(A + 2 * ahalf, 128, 256);
      issue_taps(tmem, ad, bd, nt, P, id, id2, id3, c > 0);
      tc_commit(&used[s]);
      ++committed[s];
      if (c + nst < nchunk) {
        // the stage is reloaded once its MMAs have read it
        if (!mb_wait(&used[s], (unsigned)(freed[s] & 1))) {
          ok = false;
          break;
        }
        ++freed[s];
        load(c + nst, s);
      }
    }
    if (ok) {
      tc_commit(done);
    } else {
      // bounded drain of the copies and MMAs still in flight
      for (int s = 0; s < nst; ++s) {
        for (; landed[s] < issued[s]; ++landed[s]) mb_wait(&full[s], (unsigned)(landed[s] & 1));
        for (; freed[s] < committed[s]; ++freed[s]) mb_wait(&used[s], (unsigned)(freed[s] & 1));
      }
    }
  }
  ok = __syncthreads_and(ok);
  ok = ok && mb_wait(done, 0);
  ok = __syncthreads_and(ok);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    conv_epilogue(a, tmem, tid, y0, x0, z0, zl, n0, nt, P);
  } else if (tid == 0) {
    atomicExch(a.err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols)
                 : "memory");
}

// Weight image: destination element (co, t, ci) of the (possibly
// transposed) convolution from the source layout.
__global__ void k_wimage(const __nv_bfloat16* __restrict__ w, int cout, int cin, int transpose,
                         int reverse, int tw, __nv_bfloat16* __restrict__ img) {
  const int64_t n = (int64_t)cout * 27 * cin;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int ci = (int)(q % cin);
    const int t = (int)((q / cin) % 27);
    const int co = (int)(q / ((int64_t)27 * cin));
    const int64_t src = transpose ? ((int64_t)ci * 27 + t) * cout + co : q;
    img[wimage_index(co, reverse ? 26 - t : t, ci, cout, cin, tw)] = w[src];
  }
}

// Reference 3x3x3 convolution on the CUDA cores (same data layout), FP32
// accumulation of BF16 products: the check of the tensor-core kernel.
__global__ void k_conv3_ref(ConvArgs a) {
  if (a.skip && *a.skip) return;
  const int64_t nvox = (int64_t)a.ny * a.nx * a.nz;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nvox * a.cout) return;
  const int co = (int)(idx % a.cout);
  const int64_t v = idx / a.cout;
  const int vi = (int)(v % a.ny);
  const int64_t r = v / a.ny;
  const int vj = (int)(r % a.nx), vk = (int)(r / a.nx);
  float acc = a.bias ? a.bias[co] : 0.f;
  for (int t = 0; t < 27; ++t) {
    int di = t % 3 - 1, dj = (t / 3) % 3 - 1, dk = t / 9 - 1;
    if (a.flip) {
      di = -di;
      dj = -dj;
      dk = -dk;
    }
    const int ii = vi + di, jj = vj + dj, kk = vk + dk, kl = vk % a.nzs + dk;
    if (ii < 0 || ii >= a.ny || jj < 0 || jj >= a.nx || kl < 0 || kl >= a.nzs) continue;
    const int64_t nv = (int64_t)ii + (int64_t)a.ny * (jj + (int64_t)a.nx * kk);
    for (int ci = 0; ci < a.cin; ++ci)
      acc += __bfloat162float(a.x[act_index(nv, a.offx + ci, nvox)]) *
             __bfloat162float(a.w[((int64_t)co * 27 + t) * a.cin + ci]);
  }
  if (a.relu) acc = fmaxf(acc, 0.f);
  if (a.y16) a.y16[act_index(v, a.offy + co, nvox)] = __float2bfloat16_rn(acc);
  if (a.y32) a.y32[act_index(v, a.offy + co, nvox)] = acc;
}

// Weight gradient dW[co][t][ci] = sum_v dy[v][co] * x[nb(v,t)][ci] as a
// tensor-core GEMM: rows (M) = 128 of the 27*cin (tap, channel) pairs,
// columns (N) = cout, reduction (K) = the voxels of this CTA's slice, 16 per
// MMA; both operands gathered into the same K-major core-matrix layout as
// the forward kernel.  Each CTA adds its slice's partial sums atomically.
__global__ void __launch_bounds__(NTHR) k_wgrad_tc(WgradArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* As = sm;
  unsigned char* Bs = sm + NSTG * A_BYTES;
  const int bstride = a.cout * KS * 2;
  uint64_t* bar = reinterpret_cast<uint64_t*>(Bs + NSTG * bstride);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + NSTG + 1);
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int64_t nvox = (int64_t)a.ny * a.nx * a.nz;
  const int rows = 27 * a.cin;
  const int m = blockIdx.x * TM + tid;  // (tap, channel) row of this thread
  const int t = m / a.cin, ci = m % a.cin;
  const int di = t % 3 - 1, dj = (t / 3) % 3 - 1, dk = t / 9 - 1;
  const int64_t v0 = (int64_t)blockIdx.y * a.kv;
  const int64_t v1 = min(v0 + a.kv, nvox);
  const int ncols = a.cout <= 32 ? 32 : (a.cout <= 64 ? 64 : (a.cout <= 128 ? 128 : 256));
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     sa(tslot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s <= NSTG; ++s) mb_init(&bar[s]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t id = idesc_bf16(a.cout);
  const int nsteps = (int)((v1 - v0 + KS - 1) / KS);
  const int g = tid >> 3, rr = tid & 7;
  bool ok = true;
  int ncommitted = 0;      // steps whose MMAs thread 0 committed to bar[step % NSTG]
  bool done_commit = false;  // the final commit to bar[NSTG] was issued
  for (int step = 0; step < nsteps; ++step) {
    const int s = step % NSTG;
    if (step >= NSTG) ok = ok && mb_wait(&bar[s], (unsigned)(((step - NSTG) / NSTG) & 1));
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    const int64_t vb = v0 + (int64_t)step * KS;
    // A row m: x[nb(v, t)][ci] for the 16 voxels of this step
    __align__(16) __nv_bfloat16 av[16];
#pragma unroll
    for (int e = 0; e < 16; ++e) {
      __nv_bfloat16 val = __float2bfloat16_rn(0.f);
      const int64_t vv = vb + e;
      if (m < rows && vv < v1) {
        const int vi = (int)(vv % a.ny);
        const int64_t r2 = vv / a.ny;
        const int vj = (int)(r2 % a.nx), vk = (int)(r2 / a.nx);
        const int ii = vi + di, jj = vj + dj, kk = vk + dk, kl = vk % a.nzs + dk;
        if (ii >= 0 && ii < a.ny && jj >= 0 && jj < a.nx && kl >= 0 && kl < a.nzs)
          val = a.x[act_index((int64_t)ii + (int64_t)a.ny * (jj + (int64_t)a.nx * kk),
                              a.offx + ci, nvox)];
      }
      av[e] = val;
    }
    unsigned char* A = As + s * A_BYTES;
    *reinterpret_cast<uint4*>(A + g * 256 + rr * 16) = *reinterpret_cast<const uint4*>(&av[0]);
    *reinterpret_cast<uint4*>(A + g * 256 + 128 + rr * 16) = *reinterpret_cast<const uint4*>(&av[8]);
    // B row n: dy[v][n] for the 16 voxels
    unsigned char* B = Bs + s * bstride;
    for (int q = tid; q < a.cout * 2; q += NTHR) {
      const int n = q >> 1, kh = q & 1;
      __align__(16) __nv_bfloat16 bv[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int64_t vv = vb + kh * 8 + e;
        bv[e] = (vv < v1) ? a.dy[act_index(vv, n, nvox)] : __float2bfloat16_rn(0.f);
      }
      *reinterpret_cast<uint4*>(B + (n >> 3) * 256 + kh * 128 + (n & 7) * 16) =
          *reinterpret_cast<const uint4*>(bv);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      tc_mma(tmem, umma_desc(sa(A), 128, 256), umma_desc(sa(B), 128, 256), id, step > 0 ? 1u : 0u);
      tc_commit(&bar[s]);
      ncommitted = step + 1;
    }
  }
  if (ok && tid == 0 && nsteps > 0) {
    tc_commit(&bar[NSTG]);
    done_commit = true;
  }
  ok = __syncthreads_and(ok) && (nsteps == 0 || mb_wait(&bar[NSTG], 0));
  ok = __syncthreads_and(ok);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok && nsteps > 0) {
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c0 = 0; c0 < a.cout; c0 += 16) {
      float acc[16];
      tc_ld16(lane_base + (uint32_t)c0, acc);
      if (m < rows) {
#pragma unroll
        for (int q = 0; q < 16; ++q)
          atomicAdd(&a.dw[((int64_t)(c0 + q) * 27 + t) * a.cin + ci], acc[q]);
      }
    }
  } else if (!ok && tid == 0) {
    atomicExch(a.err, 1);
    // Bounded drain before the tensor memory is freed: a stage's commits
    // complete in order, and the loop waited for every commit but the last
    // of each stage, so wait for that last phase of each stage, then for the
    // final commit if it was issued.
    for (int s = 0; s < NSTG && s < ncommitted; ++s) {
      const int last = s + ((ncommitted - 1 - s) / NSTG) * NSTG;
      mb_wait(&bar[s], (unsigned)((last / NSTG) & 1));
    }
    if (done_commit) mb_wait(&bar[NSTG], 0);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols)
                 : "memory");
}

size_t conv_smem(int cout) {
  return (size_t)NSTG * A_BYTES + (size_t)NSTG * cout * KS * 2 + (NSTG + 1) * 8 + 16;
}

size_t conv_tile_smem(int nt, int nst, int planes) {
  return (size_t)nst * (2 * a_half_bytes(planes) + 27 * nt * 32) + (2 * NST + 1) * 8 + 16;
}

}  // namespace

bool conv_shape_ok(int cin, int cout) {
  return cin >= 16 && cin % 16 == 0 && cout >= 16 && cout % 16 == 0 && cout <= 256;
}

int conv3_init() {
  static bool done = false;
  if (done) return SBM_OK;
  SBM_CUDA_TRY(cudaFuncSetAttribute(k_conv3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(kSmemBudget + 1024)));
  SBM_CUDA_TRY(cudaFuncSetAttribute(k_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)conv_smem(256)));
  done = true;
  return SBM_OK;
}

}  // namespace sbm

using namespace sbm;

// Host-array entry point of one convolution (no counterpart in the
// reference): x[(ny*nx*nz) x cin] and w[cout x 27 x cin] as BF16 bit
// patterns, bias[cout], y[(ny*nx*nz) x cout] FP32 out.  use_tc = 1 runs the
// tcgen05 kernel, 0 the CUDA-core reference kernel.
extern "C" int sbm_conv3d_bf16(int ny, int nx, int nz, int cin, int cout, const uint16_t* x,
                               const uint16_t* w, const float* bias, int relu, int flip,
                               int use_tc, float* y) {
  if (ny < 1 || nx < 1 || nz < 1 || !conv_shape_ok(cin, cout) || !x || !w || !y) return SBM_ERR_ARG;
  int rc = conv3_init();
  if (rc) return rc;
  const int64_t nv = (int64_t)ny * nx * nz;
  cudaStream_t s;
  SBM_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  void *dx = nullptr, *dw = nullptr, *db = nullptr, *dy = nullptr, *de = nullptr;
  auto fail = [&](int code) {
    cudaFree(dx);
    cudaFree(dw);
    cudaFree(db);
    cudaFree(dy);
    cudaFree(de);
    cudaStreamDestroy(s);
    return code;
  };
  void* dimg = nullptr;
  if (cudaMalloc(&dx, nv * cin * 2) || cudaMalloc(&dw, (size_t)cout * 27 * cin * 2) ||
      cudaMalloc(&db, cout * 4) || cudaMalloc(&dy, nv * cout * 4) || cudaMalloc(&de, 4) ||
      cudaMalloc(&dimg, (size_t)cout * 27 * cin * 2)) {
    cudaFree(dimg);
    return fail(SBM_ERR_NOMEM);
  }
  // channels-last host arrays <-> channel-group planes on the device
  std::vector<uint16_t> xp((size_t)(nv * cin));
  for (int64_t v = 0; v < nv; ++v)
    for (int c = 0; c < cin; ++c) xp[(size_t)act_index(v, c, nv)] = x[v * cin + c];
  cudaMemcpyAsync(dx, xp.data(), nv * cin * 2, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dw, w, (size_t)cout * 27 * cin * 2, cudaMemcpyHostToDevice, s);
  if (bias) cudaMemcpyAsync(db, bias, cout * 4, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(de, 0, 4, s);
  ConvArgs a{};
  a.ny = ny; a.nx = nx; a.nz = nz; a.nzs = nz; a.cin = cin; a.cout = cout;
  a.planes = (nz % 4 == 0 && cout <= 32) ? 4 : ((nz % 2 == 0) ? 2 : 1);
  a.ldx = cin; a.offx = 0; a.offy = 0;
  a.x = (const __nv_bfloat16*)dx; a.w = (const __nv_bfloat16*)dw;
  a.bias = bias ? (const float*)db : nullptr;
  a.y16 = nullptr; a.y32 = (float*)dy; a.relu = relu; a.flip = flip; a.err = (int*)de;
  conv3_wimage(a.w, cout, cin, 0, flip, 64, (__nv_bfloat16*)dimg, s);
  a.wimg = (const __nv_bfloat16*)dimg;
  // the uploads and the weight image are complete before the launch, so
  // the kernel may copy the weights before its dependency wait
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    cudaFree(dimg);
    return fail(SBM_ERR_CUDA);
  }
  a.wpre = 1;
  rc = conv3_launch(&a, nullptr, use_tc, s);
  if (rc) {
    cudaStreamSynchronize(s);
    cudaFree(dimg);
    return fail(rc);
  }
  int herr = 0;
  std::vector<float> yp((size_t)(nv * cout));
  cudaMemcpyAsync(yp.data(), dy, nv * cout * 4, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(&herr, de, 4, cudaMemcpyDeviceToHost, s);
  const cudaError_t e = cudaStreamSynchronize(s);
  cudaFree(dimg);
  if (e != cudaSuccess) return fail(SBM_ERR_CUDA);
  for (int64_t v = 0; v < nv; ++v)
    for (int c = 0; c < cout; ++c) y[v * cout + c] = yp[(size_t)act_index(v, c, nv)];
  fail(0);
  return herr ? SBM_ERR_TIMEOUT : SBM_OK;
}

namespace sbm {
int wgrad_launch(const WgradArgs* pa, cudaStream_t s) {
  const WgradArgs& a = *pa;
  const int64_t nv = (int64_t)a.ny * a.nx * a.nz;
  const dim3 grid((unsigned)((27 * a.cin + TM - 1) / TM), (unsigned)((nv + a.kv - 1) / a.kv));
  k_wgrad_tc<<<grid, NTHR, conv_smem(a.cout), s>>>(a);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

int conv3_map(const ConvArgs* pa, ConvMap* m) {
  const ConvArgs& a = *pa;
  auto fn = tensor_map_encoder();
  if (!fn) {
    set_error_msg("cuTensorMapEncodeTiled unavailable");
    return SBM_ERR_STATE;
  }
  const cuuint64_t row = (cuuint64_t)8 * a.ny;  // 8 channels x y
  const cuuint64_t V = (cuuint64_t)a.ny * a.nx * a.nz;
  cuuint64_t dims[5] = {row, (cuuint64_t)a.nx, (cuuint64_t)a.nzs, (cuuint64_t)(a.nz / a.nzs),
                        (cuuint64_t)(a.ldx / 8)};
  cuuint64_t strides[4] = {row * 2, row * 2 * a.nx, row * 2 * a.nx * a.nzs, V * 8 * 2};
  cuuint32_t box[5] = {8 * HY, HX, (cuuint32_t)(a.planes + 2), 1, 1};
  cuuint32_t es[5] = {1, 1, 1, 1, 1};
  const CUresult r = fn(&m->x, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5,
                        const_cast<__nv_bfloat16*>(a.x), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error_msg("cuTensorMapEncodeTiled rejected a convolution input");
    return SBM_ERR_STATE;
  }
  return SBM_OK;
}

void conv3_wimage(const __nv_bfloat16* w, int cout, int cin, int transpose, int reverse, int tw,
                  __nv_bfloat16* img, cudaStream_t s) {
  const int64_t n = (int64_t)cout * 27 * cin;
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  k_wimage<<<(unsigned)b, 256, 0, s>>>(w, cout, cin, transpose, reverse, tw, img);
  SBM_LAUNCHED(1);
}

int conv3_launch(const ConvArgs* pa, const ConvMap* map, int use_tc, cudaStream_t s) {
  ConvArgs a = *pa;
  const int64_t nv = (int64_t)a.ny * a.nx * a.nz;
  if (use_tc) {
    if ((a.ldx % 8) || (a.offx % 8) || (a.nz % a.nzs) || !a.wimg) return SBM_ERR_ARG;
    if ((a.planes != 1 && a.planes != 2 && a.planes != 4) || (a.nzs % a.planes) ||
        (a.pool && (a.planes == 1 || a.ny % 2 || a.nx % 2)) || (a.w1x1 && a.cout != 16) ||
        (a.offu % 8) || (a.offy % 8))
      return SBM_ERR_ARG;
    ConvMap local;
    if (!map) {
      const int rc = conv3_map(pa, &local);
      if (rc) return rc;
      map = &local;
    }
    const int64_t tiles =
        (int64_t)((a.ny + TY - 1) / TY) * ((a.nx + TX - 1) / TX) * (a.nz / a.planes);
    // narrow output tiles when the wide ones leave most SMs idle
    a.tw = (a.wimg16 && tiles * ((a.cout + NT_MAX - 1) / NT_MAX) < 152) ? 16 : NT_MAX;
    const int ntn = (a.cout + a.tw - 1) / a.tw;
    const int nt = std::min(a.cout, a.tw);
    const int nchunk = a.cin / KS;
    // a lone wave keeps every chunk in flight; several waves keep one stage
    // per CTA so that more CTAs share an SM (at 256^3: 115 us for the nine
    // layers against 118 us with two stages and 132 us with three)
    const size_t stage = conv_tile_smem(nt, 1, a.planes) - conv_tile_smem(nt, 0, a.planes);
    int nst = std::min(kWaveStages, nchunk);
    if (tiles * ntn <= 152)
      nst = std::max(nst, (int)std::min<size_t>(nchunk, kSmemBudget / stage));
    a.nst = std::min(nst, NST);
    const cudaError_t e = launch_pdl(k_conv3_tc, dim3((unsigned)tiles, (unsigned)ntn), dim3(NTHR),
                                     conv_tile_smem(nt, a.nst, a.planes), s, *map, a);
    if (e != cudaSuccess) {
      set_error("k_conv3_tc launch", e);
      return SBM_ERR_CUDA;
    }
  } else {
    const int64_t n = nv * a.cout;
    k_conv3_ref<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
  }
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}
}  // namespace sbm
