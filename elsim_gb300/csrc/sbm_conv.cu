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
constexpr int HY = TY + 2, HX = TX + 2, HZ = 3;  // halo tile
constexpr int HVOX = HY * HX * HZ;              // 540 voxels
constexpr int A_HALF = HVOX * 16;               // one 8-channel half, bytes
constexpr int A_STAGE = 2 * A_HALF;             // 17280
constexpr int NT_MAX = 64;                      // output channels per CTA
constexpr int NST = 2;                          // stages

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

// Halo-tiled implicit GEMM.  A CTA owns a tile of TY x TX voxels in one z
// plane (M = 128 rows, row m = voxel (y0 + m%8, x0 + m/8)) and NT output
// channels.  For each 16-channel input chunk it stages the (TY+2) x (TX+2)
// x 3 halo tile once in shared memory, in the canonical K-major layout
// (8 consecutive y voxels x 16 bytes = one core matrix; x lines HY*16
// bytes apart; the two 8-channel halves A_HALF bytes apart), together with
// the chunk's weights for all 27 taps, and issues the 27 tap MMAs from
// shifted descriptor start addresses: the tap offset (dy, dx, dz) moves the
// start by (dy + HY*(dx + HX*dz)) * 16 bytes and the core-matrix strides stay
// the same, so the input is read about 4x (halo) instead of 27x.  Two
// stages let the gather of the next chunk overlap the MMAs in flight.
__global__ void __launch_bounds__(NTHR) k_conv3_tc(ConvArgs a) {
  if (a.skip && *a.skip) return;
  extern __shared__ __align__(1024) unsigned char sm[];
  const int n0 = blockIdx.y * NT_MAX;
  const int nt = min(NT_MAX, a.cout - n0);
  const int bbytes = 27 * nt * 32;
  const int stage_bytes = A_STAGE + bbytes;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + NST * stage_bytes);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + NST + 1);
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int nty = (a.ny + TY - 1) / TY, ntx = (a.nx + TX - 1) / TX;
  const int ty = blockIdx.x % nty;
  const int tx = (blockIdx.x / nty) % ntx;
  const int z0 = blockIdx.x / (nty * ntx);
  const int y0 = ty * TY, x0 = tx * TX;
  const int zl = z0 % a.nzs;  // plane index within its sample
  const int ncols = nt <= 32 ? 32 : 64;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     sa(tslot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s <= NST; ++s) mb_init(&bar[s]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t id = idesc_bf16(nt);
  const int nchunk = a.cin / KS;
  const uint4 zero4 = make_uint4(0, 0, 0, 0);
  bool ok = true;
  for (int c = 0; c < nchunk; ++c) {
    const int s = c % NST;
    // the stage was last read by the MMAs of chunk c - NST
    if (c >= NST) ok = ok && mb_wait(&bar[s], (unsigned)(((c - NST) / NST) & 1));
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    unsigned char* A = sm + s * stage_bytes;
    unsigned char* B = A + A_STAGE;
    // halo tile: item q -> voxel hv = q / 2 (hy fastest), channel half q % 2
    for (int q0 = 0; q0 < HVOX * 2; q0 += NTHR * 4) {
      uint4 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int q = q0 + u * NTHR + tid;
        v[u] = zero4;
        if (q < HVOX * 2) {
          const int hv = q >> 1, kh = q & 1;
          const int hy = hv % HY, hx = (hv / HY) % HX, hz = hv / (HY * HX);
          const int y = y0 + hy - 1, x = x0 + hx - 1, dz = hz - 1;
          if (y >= 0 && y < a.ny && x >= 0 && x < a.nx && zl + dz >= 0 && zl + dz < a.nzs) {
            const int64_t vox = (int64_t)y + (int64_t)a.ny * (x + (int64_t)a.nx * (z0 + dz));
            v[u] = *reinterpret_cast<const uint4*>(a.x + vox * a.ldx + a.offx + c * KS + kh * 8);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int q = q0 + u * NTHR + tid;
        if (q < HVOX * 2)
          *reinterpret_cast<uint4*>(A + (q & 1) * A_HALF + (q >> 1) * 16) = v[u];
      }
    }
    // weights of the chunk for all taps: item q -> tap, row n, half kh
    const int nb2 = nt * 2;
    for (int q0 = 0; q0 < 27 * nb2; q0 += NTHR * 4) {
      uint4 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int q = q0 + u * NTHR + tid;
        v[u] = zero4;
        if (q < 27 * nb2) {
          const int t = q / nb2, n = (q % nb2) >> 1, kh = q & 1;
          v[u] = *reinterpret_cast<const uint4*>(a.w + ((int64_t)(n0 + n) * 27 + t) * a.cin +
                                                 c * KS + kh * 8);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int q = q0 + u * NTHR + tid;
        if (q < 27 * nb2) {
          const int t = q / nb2, n = (q % nb2) >> 1, kh = q & 1;
          *reinterpret_cast<uint4*>(B + t * (nt * 32) + (n >> 3) * 256 + kh * 128 + (n & 7) * 16) =
              v[u];
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int t = 0; t < 27; ++t) {
        int dy = t % 3 - 1, dx = (t / 3) % 3 - 1, dz = t / 9 - 1;
        if (a.flip) {
          dy = -dy;
          dx = -dx;
          dz = -dz;
        }
        const uint32_t aoff = (uint32_t)(((1 + dz) * HX + (1 + dx)) * HY + (1 + dy)) * 16u;
        const uint64_t ad = umma_desc(sa(A) + aoff, A_HALF, HY * 16);
        const uint64_t bd = umma_desc(sa(B) + (uint32_t)(t * nt * 32), 128, 256);
        tc_mma(tmem, ad, bd, id, (c > 0 || t > 0) ? 1u : 0u);
      }
      tc_commit(&bar[s]);
    }
  }
  // all MMAs complete -> accumulator ready
  if (ok && tid == 0) tc_commit(&bar[NST]);
  ok = __syncthreads_and(ok) && mb_wait(&bar[NST], 0);
  ok = __syncthreads_and(ok);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    const int y = y0 + (tid & 7), x = x0 + (tid >> 3);
    const bool valid = y < a.ny && x < a.nx;
    const int64_t v = (int64_t)y + (int64_t)a.ny * (x + (int64_t)a.nx * z0);
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c0 = 0; c0 < nt; c0 += 16) {
      float acc[16];
      tc_ld16(lane_base + (uint32_t)c0, acc);
      if (valid) {
        if (a.y16) {
          __align__(16) __nv_bfloat16 o[16];
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            float val = acc[q] + (a.bias ? a.bias[n0 + c0 + q] : 0.f);
            if (a.relu) val = fmaxf(val, 0.f);
            o[q] = __float2bfloat16_rn(val);
          }
          uint4* dst = reinterpret_cast<uint4*>(a.y16 + v * a.ldy + a.offy + n0 + c0);
          dst[0] = *reinterpret_cast<const uint4*>(&o[0]);
          dst[1] = *reinterpret_cast<const uint4*>(&o[8]);
        }
        if (a.y32) {
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            float val = acc[q] + (a.bias ? a.bias[n0 + c0 + q] : 0.f);
            if (a.relu) val = fmaxf(val, 0.f);
            a.y32[v * a.ldy + a.offy + n0 + c0 + q] = val;
          }
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(a.err, 1);
    // bounded drain of MMAs still in flight before the memory is released
    for (int s = 0; s < NST; ++s) {
      for (unsigned n = 0; n < kSpinTc && !mb_try(&bar[s], 0) && !mb_try(&bar[s], 1); ++n) {
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols)
                 : "memory");
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
      acc += __bfloat162float(a.x[nv * a.ldx + a.offx + ci]) *
             __bfloat162float(a.w[((int64_t)co * 27 + t) * a.cin + ci]);
  }
  if (a.relu) acc = fmaxf(acc, 0.f);
  if (a.y16) a.y16[v * a.ldy + a.offy + co] = __float2bfloat16_rn(acc);
  if (a.y32) a.y32[v * a.ldy + a.offy + co] = acc;
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
          val = a.x[((int64_t)ii + (int64_t)a.ny * (jj + (int64_t)a.nx * kk)) * a.ldx + a.offx + ci];
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
        bv[e] = (vv < v1) ? a.dy[vv * a.cout + n] : __float2bfloat16_rn(0.f);
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
    }
  }
  if (ok && tid == 0 && nsteps > 0) tc_commit(&bar[NSTG]);
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
    for (int s = 0; s < NSTG; ++s) {
      for (unsigned n = 0; n < kSpinTc && !mb_try(&bar[s], 0) && !mb_try(&bar[s], 1); ++n) {
      }
    }
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

size_t conv_tile_smem(int nt) {
  return (size_t)NST * (A_STAGE + 27 * nt * 32) + (NST + 1) * 8 + 16;
}

}  // namespace

bool conv_shape_ok(int cin, int cout) {
  return cin >= 16 && cin % 16 == 0 && cout >= 16 && cout % 16 == 0 && cout <= 256;
}

int conv3_init() {
  static bool done = false;
  if (done) return SBM_OK;
  SBM_CUDA_TRY(cudaFuncSetAttribute(k_conv3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)conv_tile_smem(NT_MAX)));
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
  if (cudaMalloc(&dx, nv * cin * 2) || cudaMalloc(&dw, (size_t)cout * 27 * cin * 2) ||
      cudaMalloc(&db, cout * 4) || cudaMalloc(&dy, nv * cout * 4) || cudaMalloc(&de, 4))
    return fail(SBM_ERR_NOMEM);
  cudaMemcpyAsync(dx, x, nv * cin * 2, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dw, w, (size_t)cout * 27 * cin * 2, cudaMemcpyHostToDevice, s);
  if (bias) cudaMemcpyAsync(db, bias, cout * 4, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(de, 0, 4, s);
  ConvArgs a{};
  a.ny = ny; a.nx = nx; a.nz = nz; a.nzs = nz; a.cin = cin; a.cout = cout;
  a.ldx = cin; a.offx = 0; a.ldy = cout; a.offy = 0;
  a.x = (const __nv_bfloat16*)dx; a.w = (const __nv_bfloat16*)dw;
  a.bias = bias ? (const float*)db : nullptr;
  a.y16 = nullptr; a.y32 = (float*)dy; a.relu = relu; a.flip = flip; a.err = (int*)de;
  rc = conv3_launch(&a, use_tc, s);
  if (rc) return fail(rc);
  int herr = 0;
  cudaMemcpyAsync(y, dy, nv * cout * 4, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(&herr, de, 4, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return fail(SBM_ERR_CUDA);
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

int conv3_launch(const ConvArgs* pa, int use_tc, cudaStream_t s) {
  const ConvArgs& a = *pa;
  const int64_t nv = (int64_t)a.ny * a.nx * a.nz;
  if (use_tc) {
    const int64_t tiles = (int64_t)((a.ny + TY - 1) / TY) * ((a.nx + TX - 1) / TX) * a.nz;
    const int ntn = (a.cout + NT_MAX - 1) / NT_MAX;
    k_conv3_tc<<<dim3((unsigned)tiles, (unsigned)ntn), NTHR,
                 conv_tile_smem(std::min(a.cout, NT_MAX)), s>>>(a);
  } else {
    const int64_t n = nv * a.cout;
    k_conv3_ref<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
  }
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}
}  // namespace sbm
