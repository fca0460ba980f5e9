// sbm_conv.cu -- BF16 3x3x3 convolution on the 5th-generation tensor cores.
//
// Implicit GEMM: rows (M) = 128 consecutive voxels of a grid stored
// channels-last (x[v*C + c], v = i + ny*(j + nx*k)), columns (N) = output
// channels, reduction (K) = 27 taps x input channels, walked one tap and 16
// input channels at a time (one tcgen05.mma of K = 16 per step).  For each
// step the 128 threads gather the 128 x 16 activation slice (zero outside
// the grid) and the N x 16 weight slice into shared memory in the canonical
// no-swizzle K-major layout (8-row x 16-byte core matrices; K-adjacent core
// matrices 128 bytes apart, row groups 256 bytes apart), one elected thread
// issues the MMA with FP32 accumulation into tensor memory and commits it to
// the stage's mbarrier, and a 4-stage ring lets the gather of the next steps
// overlap the MMAs in flight.  The epilogue reads the accumulator with
// tcgen05.ld (each warp its 32 lanes), adds the bias, optionally applies
// ReLU and stores BF16 or FP32 into a channel slice of the output.
//
// Operands are BF16 x BF16 -> FP32 only.  Every mbarrier wait is bounded;
// on expiry the CTA sets an error flag, frees its tensor memory and returns.
#include <cuda_bf16.h>

#include "sbm_internal.cuh"

namespace sbm {

namespace {

constexpr int TM = 128;          // voxels per CTA (MMA M)
constexpr int NTHR = 128;        // 4 warps
constexpr int KS = 16;           // K per MMA (BF16)
constexpr int NSTG = 4;          // stages
constexpr int A_BYTES = TM * KS * 2;   // 4096
constexpr unsigned kSpinTc = 1u << 20;

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

struct ConvArgs {
  int ny, nx, nz;        // grid
  int cin, cout;         // channels (multiples of 16)
  int ldx, offx;         // input channel stride and offset (channel slices of concat buffers)
  int ldy, offy;         // output channel stride and offset
  const __nv_bfloat16* x;
  const __nv_bfloat16* w;  // [cout][27][cin]
  const float* bias;       // [cout] or null
  __nv_bfloat16* y16;      // BF16 output or null
  float* y32;              // FP32 output or null
  int relu;
  int flip;                // 1: tap t reads neighbour -offset (transposed convolution)
  int* err;                // set to 1 if a wait expired
};

__global__ void __launch_bounds__(NTHR) k_conv3_tc(ConvArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* As = sm;                               // NSTG x 4096
  unsigned char* Bs = sm + NSTG * A_BYTES;              // NSTG x N*32
  const int bstride = a.cout * KS * 2;
  uint64_t* bar = reinterpret_cast<uint64_t*>(Bs + NSTG * bstride);  // NSTG barriers + 1
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + NSTG + 1);
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int64_t nvox = (int64_t)a.ny * a.nx * a.nz;
  const int64_t v = (int64_t)blockIdx.x * TM + tid;
  int vi = 0, vj = 0, vk = 0;
  if (v < nvox) {
    vi = (int)(v % a.ny);
    const int64_t r = v / a.ny;
    vj = (int)(r % a.nx);
    vk = (int)(r / a.nx);
  }
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
  const int csteps = a.cin / KS;
  const int nsteps = 27 * csteps;
  // A row of this thread: core matrix (group m/8, k-half) at g*256 + kk*128, row r at +r*16
  const int g = tid >> 3, rr = tid & 7;
  bool ok = true;
  for (int step = 0; step < nsteps; ++step) {
    const int s = step % NSTG;
    // the stage was last used by step - NSTG: wait until its MMA has read it
    if (step >= NSTG) ok = ok && mb_wait(&bar[s], (unsigned)(((step - NSTG) / NSTG) & 1));
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    const int t = step / csteps, cs = step % csteps;
    const int di = t % 3 - 1, dj = (t / 3) % 3 - 1, dk = t / 9 - 1;
    // gather 16 input channels of the tap's neighbour (zero outside the grid)
    uint4 lo = make_uint4(0, 0, 0, 0), hi = lo;
    if (v < nvox) {
      const int si = a.flip ? -di : di, sj = a.flip ? -dj : dj, sk = a.flip ? -dk : dk;
      const int ii = vi + si, jj = vj + sj, kk = vk + sk;
      if (ii >= 0 && ii < a.ny && jj >= 0 && jj < a.nx && kk >= 0 && kk < a.nz) {
        const int64_t nv = (int64_t)ii + (int64_t)a.ny * (jj + (int64_t)a.nx * kk);
        const uint4* src =
            reinterpret_cast<const uint4*>(a.x + nv * a.ldx + a.offx + cs * KS);
        lo = src[0];
        hi = src[1];
      }
    }
    unsigned char* A = As + s * A_BYTES;
    *reinterpret_cast<uint4*>(A + g * 256 + rr * 16) = lo;
    *reinterpret_cast<uint4*>(A + g * 256 + 128 + rr * 16) = hi;
    // weights: row n = output channel, 16 input channels of this tap
    unsigned char* B = Bs + s * bstride;
    for (int q = tid; q < a.cout * 2; q += NTHR) {
      const int n = q >> 1, kh = q & 1;
      const uint4 wv = *reinterpret_cast<const uint4*>(a.w + ((int64_t)n * 27 + t) * a.cin +
                                                       cs * KS + kh * 8);
      *reinterpret_cast<uint4*>(B + (n >> 3) * 256 + kh * 128 + (n & 7) * 16) = wv;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint64_t ad = umma_desc(sa(A), 128, 256);
      const uint64_t bd = umma_desc(sa(B), 128, 256);
      tc_mma(tmem, ad, bd, id, step > 0 ? 1u : 0u);
      tc_commit(&bar[s]);
    }
  }
  // all MMAs complete -> accumulator ready
  if (ok && tid == 0) tc_commit(&bar[NSTG]);
  ok = __syncthreads_and(ok) && mb_wait(&bar[NSTG], 0);
  ok = __syncthreads_and(ok);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c0 = 0; c0 < a.cout; c0 += 16) {
      float acc[16];
      tc_ld16(lane_base + (uint32_t)c0, acc);
      if (v < nvox) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          float val = acc[q] + (a.bias ? a.bias[c0 + q] : 0.f);
          if (a.relu) val = fmaxf(val, 0.f);
          if (a.y16) a.y16[v * a.ldy + a.offy + c0 + q] = __float2bfloat16_rn(val);
          if (a.y32) a.y32[v * a.ldy + a.offy + c0 + q] = val;
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(a.err, 1);
    // bounded drain of MMAs still in flight before the memory is released
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

// Reference 3x3x3 convolution on the CUDA cores (same data layout), FP32
// accumulation of BF16 products: the check of the tensor-core kernel.
__global__ void k_conv3_ref(ConvArgs a) {
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
    const int ii = vi + di, jj = vj + dj, kk = vk + dk;
    if (ii < 0 || ii >= a.ny || jj < 0 || jj >= a.nx || kk < 0 || kk >= a.nz) continue;
    const int64_t nv = (int64_t)ii + (int64_t)a.ny * (jj + (int64_t)a.nx * kk);
    for (int ci = 0; ci < a.cin; ++ci)
      acc += __bfloat162float(a.x[nv * a.ldx + a.offx + ci]) *
             __bfloat162float(a.w[((int64_t)co * 27 + t) * a.cin + ci]);
  }
  if (a.relu) acc = fmaxf(acc, 0.f);
  if (a.y16) a.y16[v * a.ldy + a.offy + co] = __float2bfloat16_rn(acc);
  if (a.y32) a.y32[v * a.ldy + a.offy + co] = acc;
}

size_t conv_smem(int cout) {
  return (size_t)NSTG * A_BYTES + (size_t)NSTG * cout * KS * 2 + (NSTG + 1) * 8 + 16;
}

}  // namespace

bool conv_shape_ok(int cin, int cout) {
  return cin >= 16 && cin % 16 == 0 && cout >= 16 && cout % 16 == 0 && cout <= 256;
}

int conv3_launch(const ConvArgs* pa, int use_tc, cudaStream_t s);

int conv3_init() {
  static bool done = false;
  if (done) return SBM_OK;
  SBM_CUDA_TRY(cudaFuncSetAttribute(k_conv3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
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
  a.ny = ny; a.nx = nx; a.nz = nz; a.cin = cin; a.cout = cout;
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
int conv3_launch(const ConvArgs* pa, int use_tc, cudaStream_t s) {
  const ConvArgs& a = *pa;
  const int64_t nv = (int64_t)a.ny * a.nx * a.nz;
  if (use_tc) {
    const unsigned blocks = (unsigned)((nv + TM - 1) / TM);
    k_conv3_tc<<<blocks, NTHR, conv_smem(a.cout), s>>>(a);
  } else {
    const int64_t n = nv * a.cout;
    k_conv3_ref<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
  }
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}
}  // namespace sbm
