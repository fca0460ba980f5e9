// sbm_net.cu -- learned coarse-grid preconditioner for the flexible CG of
// the mixed-precision solver (no counterpart in the reference, whose CG
// loops are unpreconditioned).
//
//   z = D^-1 r + P e_c,     e_c = (s k_out / (scale c_ref)) N(f),
//
// R = average over 4x4x4 fine cells, P = cell-centred trilinear
// interpolation (clamped at the faces), s = RMS of R r, c_ref = mean of
// R K, N a 3D U-Net on the coarse grid whose input channels f are
// [R r / s, R K / c_ref, 1, Dirichlet x0 face, Dirichlet x1 face, 0 ...].
// N is trained (below, on the tensor cores) to map f to
// R(A^-1 r) scale c_ref / (s k_out), so e_c approximates the restricted
// error.  The result is not linear in r, hence the flexible CG.
//
// U-Net (channels, BF16 activations channels-last, FP32 accumulation):
//   level 0 (coarse grid)   E0 16->16  ...........................  D0 48->16 -> 1x1 16->1
//   level 1 (avg pool 2)    E1 16->32  .....................  D1 64->32
//   level 2                 E2 32->32  ...............  D2 80->32
//   level 3                 E3 32->48  .........  D3 112->48
//   level 4                 E4 48->64 --(nearest upsampling)--^
// 3x3x3 convolutions with bias and ReLU; each decoder level reads the
// concatenation [upsampled lower output | encoder output] from one buffer.
//
// Training: loss = mean (N(f) - t)^2.  Backward uses the same tcgen05
// convolution kernel with flipped taps and transposed weights for the data
// gradient, a tcgen05 GEMM over voxels for the weight gradient, and Adam on
// FP32 master weights that rebuilds the BF16 weight images of both passes.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "sbm_async.cuh"
#include "sbm_conv.cuh"
#include "sbm_net.cuh"

namespace sbm {
namespace netd {

typedef __nv_bfloat16 bf16;

enum { E0, E1, E2, E3, E4, D3, D2, D1, D0, OUT, NLAYER };
constexpr int kCi[NLAYER] = {16, 16, 32, 32, 48, 112, 80, 64, 48, 16};
constexpr int kCo[NLAYER] = {16, 32, 32, 48, 64, 48, 32, 32, 16, 1};
constexpr int kLev = 5;
constexpr int kFeat = 16;
constexpr int kCatW[4] = {48, 64, 80, 112};  // concat buffer width per level
constexpr int kUpW[4] = {32, 32, 48, 64};    // [0, kUpW): upsampled; [kUpW, kCatW): encoder
constexpr int kEnc[4] = {E0, E1, E2, E3};
constexpr int kDec[4] = {D0, D1, D2, D3};

struct Layout {
  int64_t off[NLAYER];   // weights [co][taps][ci]
  int64_t boff[NLAYER];  // biases [co]
  int64_t total;
};

Layout make_layout() {
  Layout L{};
  int64_t o = 0;
  for (int l = 0; l < NLAYER; ++l) {
    const int taps = (l == OUT) ? 1 : 27;
    L.off[l] = o;
    o += (int64_t)kCo[l] * taps * kCi[l];
    L.boff[l] = o;
    o += kCo[l];
  }
  L.total = o;
  return L;
}
const Layout kL = make_layout();

struct Dims {
  int ny, nx, nz, nzs;  // nz = stacked depth of all samples, nzs = one sample
  __host__ __device__ int64_t v() const { return (int64_t)ny * nx * nz; }
};

inline Dims half(const Dims& d) { return Dims{d.ny / 2, d.nx / 2, d.nz / 2, d.nzs / 2}; }

struct Work {
  Dims d[kLev];
  // a zero-padded grid: the valid extents per level (voxels beyond them
  // keep zero activations); vd == d when not padded
  Dims vd[kLev];
  bool padded = false;
  bool train = false;
  bf16* in0 = nullptr;
  bf16* cat[4] = {};
  bf16* pin[kLev] = {};  // pooled encoder outputs, levels 1..4
  bf16* a4 = nullptr;
  bf16* dec[4] = {};
  float* out = nullptr;
  float* tgt = nullptr;
  // backward
  bf16* gdec[4] = {};  // gradients of the pre-activations
  bf16* genc[4] = {};
  bf16* ga4 = nullptr;
  float* gcat[4] = {};  // data gradients of the decoder inputs
  float* gpin[kLev] = {};
  std::vector<void*> mem;
  std::map<std::pair<const void*, int>, ConvMap> maps;  // per convolution input and planes
  ~Work() {
    for (void* p : mem) cudaFree(p);
  }
  template <typename T>
  bool alloc(T** p, int64_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, sizeof(T) * (size_t)(n > 0 ? n : 1)) != cudaSuccess) return false;
    mem.push_back(q);
    *p = static_cast<T*>(q);
    return true;
  }
};

// ------------------------------------------------------------- kernels

__device__ __forceinline__ void vox(const Dims& d, int64_t v, int* i, int* j, int* k) {
  *i = (int)(v % d.ny);
  const int64_t r = v / d.ny;
  *j = (int)(r % d.nx);
  *k = (int)(r / d.nx);
}

__device__ __forceinline__ int64_t vid(const Dims& d, int i, int j, int k) {
  return (int64_t)i + (int64_t)d.ny * (j + (int64_t)d.nx * k);
}

__device__ __forceinline__ int64_t child(const Dims& f, int i, int j, int k, int q) {
  return vid(f, 2 * i + (q & 1), 2 * j + ((q >> 1) & 1), 2 * k + (q >> 2));
}

#define NET_LOOP(n)                                                                 \
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (n);         \
       t += (int64_t)gridDim.x * blockDim.x)

// Loads / stores of one 8-channel group of a voxel (channel-group planes).
__device__ __forceinline__ void ld8(const bf16* p, float (&v)[8]) {
  const uint4 u = *reinterpret_cast<const uint4*>(p);
  const bf16* h = reinterpret_cast<const bf16*>(&u);
#pragma unroll
  for (int e = 0; e < 8; ++e) v[e] = __bfloat162float(h[e]);
}
__device__ __forceinline__ void ld8(const float* p, float (&v)[8]) {
  const float4 a = reinterpret_cast<const float4*>(p)[0], b = reinterpret_cast<const float4*>(p)[1];
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void st8(bf16* p, const float (&v)[8]) {
  __align__(16) bf16 h[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) h[e] = __float2bfloat16_rn(v[e]);
  *reinterpret_cast<uint4*>(p) = *reinterpret_cast<const uint4*>(h);
}

// Backward of upsampling + ReLU: out(vc, c) = (act(vc, c) > 0) * sum over
// the children of g(vf, offg + c).  One thread per coarse voxel and group.
__global__ void k_bwd_up(Dims f, int C, const float* __restrict__ g, int offg,
                         const bf16* __restrict__ act, bf16* __restrict__ out) {
  const Dims c = Dims{f.ny / 2, f.nx / 2, f.nz / 2, f.nzs / 2};
  const int64_t Vc = c.v(), Vf = f.v();
  NET_LOOP(Vc * (C / 8)) {
    const int64_t vc = t % Vc;
    const int grp = (int)(t / Vc) * 8;
    int i, j, k;
    vox(c, vc, &i, &j, &k);
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, a[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      float v[8];
      ld8(g + act_index(child(f, i, j, k, q), offg + grp, Vf), v);
#pragma unroll
      for (int e = 0; e < 8; ++e) s[e] += v[e];
    }
    ld8(act + act_index(vc, grp, Vc), a);
#pragma unroll
    for (int e = 0; e < 8; ++e) s[e] = a[e] > 0.f ? s[e] : 0.f;
    st8(out + act_index(vc, grp, Vc), s);
  }
}

// Backward of an encoder output read by the skip connection and by the
// pooling: out(vf, c) = (act(vf, offa + c) > 0) * (g(vf, offg + c) +
// gp(parent, c) / 8).  One thread per fine voxel and group.
__global__ void k_bwd_skip(Dims f, int C, const float* __restrict__ g, int offg,
                           const float* __restrict__ gp, const bf16* __restrict__ act, int offa,
                           bf16* __restrict__ out) {
  const Dims c = Dims{f.ny / 2, f.nx / 2, f.nz / 2, f.nzs / 2};
  const int64_t Vc = c.v(), Vf = f.v();
  NET_LOOP(Vf * (C / 8)) {
    const int64_t vf = t % Vf;
    const int grp = (int)(t / Vf) * 8;
    float s[8], a[8];
    ld8(g + act_index(vf, offg + grp, Vf), s);
    if (gp) {
      int i, j, k;
      vox(f, vf, &i, &j, &k);
      float p[8];
      ld8(gp + act_index(vid(c, i / 2, j / 2, k / 2), grp, Vc), p);
#pragma unroll
      for (int e = 0; e < 8; ++e) s[e] += 0.125f * p[e];
    }
    ld8(act + act_index(vf, offa + grp, Vf), a);
#pragma unroll
    for (int e = 0; e < 8; ++e) s[e] = a[e] > 0.f ? s[e] : 0.f;
    st8(out + act_index(vf, grp, Vf), s);
  }
}

// *loss += sum_v (out[v] - tgt[v])^2
__global__ void k_loss(int64_t V, const float* __restrict__ out, const float* __restrict__ tgt,
                       double* loss) {
  __shared__ double sm[32];
  double acc = 0.0;
  NET_LOOP(V) {
    const double e = (double)out[t] - (double)tgt[t];
    acc += e * e;
  }
  const double tot = block_sum(acc, sm);
  if (threadIdx.x == 0) atomicAdd(loss, tot);
}

// Backward of the output layer and of D0's ReLU:
// dout = 2 (out - tgt) / V_total; gd0[v][c] = (d0 > 0) dout w[c];
// gw[c] += sum_v dout d0[v][c]; gb += sum_v dout.
__global__ void k_out_bwd(int64_t V, float inv_v, const bf16* __restrict__ d0,
                          const float* __restrict__ w, const float* __restrict__ out,
                          const float* __restrict__ tgt, bf16* __restrict__ gd0,
                          float* __restrict__ gw, float* __restrict__ gb) {
  __shared__ float sm[17];
  if (threadIdx.x < 17) sm[threadIdx.x] = 0.f;
  __syncthreads();
  float acc[17];
#pragma unroll
  for (int c = 0; c < 17; ++c) acc[c] = 0.f;
  NET_LOOP(V) {
    const float dout = 2.f * (out[t] - tgt[t]) * inv_v;
    acc[16] += dout;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float a[8], gv[8];
      ld8(d0 + act_index(t, 8 * h, V), a);
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        acc[8 * h + e] += dout * a[e];
        gv[e] = a[e] > 0.f ? dout * w[8 * h + e] : 0.f;
      }
      st8(gd0 + act_index(t, 8 * h, V), gv);
    }
  }
#pragma unroll
  for (int c = 0; c < 17; ++c) {
    float v = acc[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&sm[c], v);
  }
  __syncthreads();
  if (threadIdx.x < 16) atomicAdd(&gw[threadIdx.x], sm[threadIdx.x]);
  if (threadIdx.x == 16) atomicAdd(gb, sm[16]);
}

// gb[c] += sum_v dy[v][c]   (C <= 64)
__global__ void k_bias_grad(int64_t V, int C, const bf16* __restrict__ dy, float* __restrict__ gb) {
  __shared__ float sm[64];
  if (threadIdx.x < C) sm[threadIdx.x] = 0.f;
  __syncthreads();
  const int groups = blockDim.x / C;
  const int c = threadIdx.x % C, grp = threadIdx.x / C;
  float s = 0.f;
  if (grp < groups)
    for (int64_t v = (int64_t)blockIdx.x * groups + grp; v < V; v += (int64_t)gridDim.x * groups)
      s += __bfloat162float(dy[act_index(v, c, V)]);
  if (grp < groups) atomicAdd(&sm[c], s);
  __syncthreads();
  if (threadIdx.x < C) atomicAdd(&gb[threadIdx.x], sm[threadIdx.x]);
}

struct LayerTab {
  int64_t off[NLAYER];
  int ci[NLAYER], co[NLAYER];
};

// Adam step on the FP32 master parameters (when `update`), then the BF16
// weight images of the tensor-core kernel: wimg for the forward pass and
// wtimg for the data gradient (transposed convolution), at the layer's
// parameter offset.
__global__ void k_adam(int64_t P, int update, float* __restrict__ w, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2,
                       float eps, float c1, float c2, LayerTab tab, bf16* __restrict__ wimg,
                       bf16* __restrict__ wtimg, bf16* __restrict__ wimg16,
                       bf16* __restrict__ wtimg16) {
  NET_LOOP(P) {
    float wv = w[t];
    if (update) {
      const float gv = g[t];
      const float mv = b1 * m[t] + (1.f - b1) * gv;
      const float vv = b2 * v[t] + (1.f - b2) * gv * gv;
      m[t] = mv;
      v[t] = vv;
      wv -= lr * (mv * c1) / (sqrtf(vv * c2) + eps);
      w[t] = wv;
    }
    for (int l = 0; l < OUT; ++l) {
      const int64_t n = (int64_t)tab.co[l] * 27 * tab.ci[l];
      const int64_t rel = t - tab.off[l];
      if (rel >= 0 && rel < n) {
        const bf16 b = __float2bfloat16_rn(wv);
        const int ci = (int)(rel % tab.ci[l]);
        const int tap = (int)((rel / tab.ci[l]) % 27);
        const int co = (int)(rel / ((int64_t)27 * tab.ci[l]));
        // data gradient: transposed channels and reversed taps
        wimg[tab.off[l] + wimage_index(co, tap, ci, tab.co[l], tab.ci[l], 64)] = b;
        wtimg[tab.off[l] + wimage_index(ci, 26 - tap, co, tab.ci[l], tab.co[l], 64)] = b;
        wimg16[tab.off[l] + wimage_index(co, tap, ci, tab.co[l], tab.ci[l], 16)] = b;
        wtimg16[tab.off[l] + wimage_index(ci, 26 - tap, co, tab.ci[l], tab.co[l], 16)] = b;
      }
    }
  }
}

__global__ void k_loss_rec(double* loss, float inv_v, float* hist) {
  *hist = (float)(*loss * (double)inv_v);
  *loss = 0.0;
}

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace netd
}  // namespace sbm

using namespace sbm;
using namespace sbm::netd;

struct sbm_net {
  float* w32 = nullptr;  // master parameters
  float* m = nullptr;
  float* v = nullptr;
  float* grad = nullptr;
  bf16* wimg = nullptr;   // forward weight images (64-wide output tiles)
  bf16* wtimg = nullptr;  // data-gradient weight images
  bf16* wimg16 = nullptr;   // the same for 16-wide output tiles
  bf16* wtimg16 = nullptr;
  int* err = nullptr;
  double* loss = nullptr;
  int64_t step = 0;
  int mass = 0;  // trained with input channel 5 (the CnE form's mass term)
  cudaStream_t stream = nullptr;
  // resident training set (sbm_net_set_data)
  bf16* din = nullptr;     // per-sample channel-group planes
  float* dt = nullptr;
  int dny = 0, dnx = 0, dnz = 0, dns = 0;
  std::map<std::tuple<int, int, int, int, int>, Work*> works;
};

namespace sbm {
namespace netd {

LayerTab layer_tab() {
  LayerTab t{};
  for (int l = 0; l < NLAYER; ++l) {
    t.off[l] = kL.off[l];
    t.ci[l] = kCi[l];
    t.co[l] = kCo[l];
  }
  return t;
}

int cast_weights(sbm_net* n, cudaStream_t s) {
  k_adam<<<grid_for(kL.total), 256, 0, s>>>(kL.total, 0, n->w32, nullptr, nullptr, nullptr, 0.f,
                                            0.f, 0.f, 0.f, 0.f, 0.f, layer_tab(), n->wimg,
                                            n->wtimg, n->wimg16, n->wtimg16);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

bool dims_ok(int ny, int nx, int nz) {
  return ny >= 16 && nx >= 16 && nz >= 16 && ny % 16 == 0 && nx % 16 == 0 && nz % 16 == 0;
}

Work* make_work(const Dims& d0, bool train, const Dims* valid = nullptr) {
  Work* w = new Work();
  w->train = train;
  w->d[0] = d0;
  for (int l = 1; l < kLev; ++l) w->d[l] = half(w->d[l - 1]);
  w->padded = valid != nullptr;
  w->vd[0] = valid ? *valid : d0;
  for (int l = 1; l < kLev; ++l) {
    const Dims& u = w->vd[l - 1];
    w->vd[l] = Dims{(u.ny + 1) / 2, (u.nx + 1) / 2, (u.nz + 1) / 2, (u.nzs + 1) / 2};
  }
  bool ok = w->alloc(&w->in0, w->d[0].v() * kFeat) && w->alloc(&w->out, w->d[0].v()) &&
            w->alloc(&w->tgt, w->d[0].v()) && w->alloc(&w->a4, w->d[4].v() * kCo[E4]);
  for (int l = 0; l < 4 && ok; ++l)
    ok = w->alloc(&w->cat[l], w->d[l].v() * kCatW[l]) &&
         w->alloc(&w->dec[l], w->d[l].v() * kCo[kDec[l]]) &&
         w->alloc(&w->pin[l + 1], w->d[l + 1].v() * kCi[kEnc[0] + l + 1]);
  if (ok && train) {
    ok = w->alloc(&w->ga4, w->d[4].v() * kCo[E4]);
    for (int l = 0; l < 4 && ok; ++l)
      ok = w->alloc(&w->gdec[l], w->d[l].v() * kCo[kDec[l]]) &&
           w->alloc(&w->genc[l], w->d[l].v() * kCo[kEnc[l]]) &&
           w->alloc(&w->gcat[l], w->d[l].v() * kCatW[l]) &&
           w->alloc(&w->gpin[l + 1], w->d[l + 1].v() * kCi[kEnc[0] + l + 1]);
  }
  if (!ok) {
    delete w;
    return nullptr;
  }
  // channels 1.. of the input stay zero unless a caller fills them
  cudaMemset(w->in0, 0, sizeof(bf16) * w->d[0].v() * kFeat);
  return w;
}

Work* work_for(sbm_net* n, int ny, int nx, int nzs, int nb, bool train) {
  const auto key = std::make_tuple(ny, nx, nzs, nb, train ? 1 : 0);
  auto it = n->works.find(key);
  if (it != n->works.end()) return it->second;
  Work* w = make_work(Dims{ny, nx, nzs * nb, nzs}, train);
  if (!w) return nullptr;
  n->works[key] = w;
  return w;
}

// Tensor map of a convolution input (encoded once per buffer and plane count).
const ConvMap* map_for(Work& w, const ConvArgs& a) {
  const auto key = std::make_pair((const void*)a.x, a.planes);
  auto it = w.maps.find(key);
  if (it != w.maps.end()) return &it->second;
  ConvMap m;
  if (conv3_map(&a, &m)) return nullptr;
  return &(w.maps[key] = m);
}

// Arguments of layer l at level lev reading x (a buffer of ldx channels),
// with ReLU; outputs are filled in by the caller.
// Two z planes per CTA where the epilogue pools (it needs both planes of a
// 2x2x2 block) or the grid is large; one plane keeps more CTAs busy on the
// small levels.
// z planes per CTA of a convolution at level d: four on the large levels
// with at most 32 output channels (half the CTAs of two planes, so the 64^3
// layers of a 256^3 solve fit in one wave), two when pooling or on other
// large levels, else one.
int planes_for(const Dims& d, bool pool, int cout) {
  if (d.nzs % 2) return 1;
  if (d.nzs % 4 == 0 && cout <= 32 && d.v() >= (int64_t)1 << 17) return 4;
  return (pool || d.v() >= (int64_t)1 << 17) ? 2 : 1;
}

ConvArgs layer_args(sbm_net* n, const Work& w, int l, int lev, const bf16* x, int ldx,
                    bool pool, const int* skip, const int* skip2) {
  ConvArgs a{};
  const Dims& d = w.d[lev];
  a.ny = d.ny; a.nx = d.nx; a.nz = d.nz; a.nzs = d.nzs;
  a.planes = planes_for(d, pool, kCo[l]);
  a.cin = kCi[l]; a.cout = kCo[l];
  a.ldx = ldx; a.offx = 0;
  a.x = x; a.wimg = n->wimg + kL.off[l]; a.wimg16 = n->wimg16 + kL.off[l];
  a.bias = n->w32 + kL.boff[l];
  a.relu = 1; a.flip = 0; a.err = n->err; a.skip = skip; a.skip2 = skip2;
  // the preconditioner's passes (the only ones with skip flags) run on
  // frozen weights; training rewrites them between passes
  a.wpre = skip != nullptr;
  if (w.padded) {
    a.vny = w.vd[lev].ny; a.vnx = w.vd[lev].nx; a.vnz = w.vd[lev].nzs;
    if (lev > 0) {
      a.uvny = w.vd[lev - 1].ny; a.uvnx = w.vd[lev - 1].nx; a.uvnz = w.vd[lev - 1].nzs;
    }
  }
  return a;
}

int launch(Work& w, const ConvArgs& a, cudaStream_t s) {
  const ConvMap* m = map_for(w, a);
  if (!m) return SBM_ERR_STATE;
  return conv3_launch(&a, m, 1, s);
}

// Forward pass of the U-Net on w.in0 -> w.out (and the squared error
// against w.tgt into n->loss when tgt).  Pooling, upsampling and the 1x1
// output layer run in the convolution epilogues; activations that only the
// backward pass reads (bottleneck and decoder outputs) are stored only
// when training.
int forward(sbm_net* n, Work& w, bool tgt, const int* skip, const int* skip2, cudaStream_t s) {
  int rc;
  for (int lev = 0; lev < 4; ++lev) {
    const int l = kEnc[lev];
    ConvArgs a =
        layer_args(n, w, l, lev, lev == 0 ? w.in0 : w.pin[lev], kCi[l], true, skip, skip2);
    a.y16 = w.cat[lev];
    a.offy = kUpW[lev];
    a.pool = w.pin[lev + 1];
    if ((rc = launch(w, a, s))) return rc;
  }
  {
    ConvArgs a = layer_args(n, w, E4, 4, w.pin[4], kCi[E4], false, skip, skip2);
    a.y16 = w.train ? w.a4 : nullptr;
    a.up = w.cat[3];
    if ((rc = launch(w, a, s))) return rc;
  }
  for (int lev = 3; lev >= 0; --lev) {
    const int l = kDec[lev];
    ConvArgs a = layer_args(n, w, l, lev, w.cat[lev], kCatW[lev], false, skip, skip2);
    a.y16 = w.train ? w.dec[lev] : nullptr;
    if (lev > 0) {
      a.up = w.cat[lev - 1];
    } else {
      a.w1x1 = n->w32 + kL.off[OUT];
      a.b1x1 = n->w32 + kL.boff[OUT];
      a.out1x1 = w.out;
    }
    if ((rc = launch(w, a, s))) return rc;
  }
  if (tgt) {
    const int64_t V = w.d[0].v();
    k_loss<<<grid_for(V), 256, 0, s>>>(V, w.out, w.tgt, n->loss);
    SBM_LAUNCHED(1);
  }
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

int wgrad(sbm_net* n, const Work& w, int l, int lev, const bf16* x, int ldx, const bf16* gy,
          cudaStream_t s) {
  const Dims& d = w.d[lev];
  WgradArgs a{};
  a.ny = d.ny; a.nx = d.nx; a.nz = d.nz; a.nzs = d.nzs;
  a.cin = kCi[l]; a.cout = kCo[l]; a.offx = 0;
  a.x = x; a.dy = gy; a.dw = n->grad + kL.off[l]; a.err = n->err;
  const int64_t V = d.v();
  const int64_t gx = (27 * kCi[l] + 127) / 128;
  int64_t kv = (V * gx + 1215) / 1216;
  kv = (kv + 15) / 16 * 16;
  if (kv < 64) kv = 64;
  if (kv > 4096) kv = 4096;
  a.kv = (int)kv;
  int rc = wgrad_launch(&a, s);
  if (rc) return rc;
  const int C = kCo[l];
  const int groups = 256 / C;
  int64_t b = (V + groups * 8 - 1) / (groups * 8);
  if (b > 152 * 8) b = 152 * 8;
  if (b < 1) b = 1;
  k_bias_grad<<<(unsigned)b, 256, 0, s>>>(V, C, gy, n->grad + kL.boff[l]);
  SBM_LAUNCHED(1);
  return SBM_OK;
}

int dgrad(sbm_net* n, Work& w, int l, int lev, const bf16* gy, float* gx, cudaStream_t s) {
  ConvArgs a{};
  const Dims& d = w.d[lev];
  a.ny = d.ny; a.nx = d.nx; a.nz = d.nz; a.nzs = d.nzs;
  a.planes = planes_for(d, false, kCi[l]);
  a.cin = kCo[l]; a.cout = kCi[l];
  a.ldx = kCo[l]; a.offx = 0; a.offy = 0;
  a.x = gy; a.wimg = n->wtimg + kL.off[l]; a.wimg16 = n->wtimg16 + kL.off[l];
  a.bias = nullptr;
  a.y16 = nullptr; a.y32 = gx; a.relu = 0; a.flip = 1; a.err = n->err; a.skip = nullptr;
  return launch(w, a, s);
}

// Gradient of mean (out - tgt)^2 over all voxels of w into n->grad
// (forward with the target must have run).
int backward(sbm_net* n, Work& w, cudaStream_t s) {
  int rc;
  SBM_CUDA_TRY(cudaMemsetAsync(n->grad, 0, sizeof(float) * kL.total, s));
  const int64_t V = w.d[0].v();
  k_out_bwd<<<grid_for(V), 256, 0, s>>>(V, 1.0f / (float)V, w.dec[0], n->w32 + kL.off[OUT], w.out,
                                        w.tgt, w.gdec[0], n->grad + kL.off[OUT],
                                        n->grad + kL.boff[OUT]);
  SBM_LAUNCHED(1);
  for (int lev = 0; lev < 4; ++lev) {
    const int l = kDec[lev];
    if ((rc = wgrad(n, w, l, lev, w.cat[lev], kCatW[lev], w.gdec[lev], s))) return rc;
    if ((rc = dgrad(n, w, l, lev, w.gdec[lev], w.gcat[lev], s))) return rc;
    const Dims& f = w.d[lev];
    const bf16* act = lev == 3 ? w.a4 : w.dec[lev + 1];
    bf16* out = lev == 3 ? w.ga4 : w.gdec[lev + 1];
    k_bwd_up<<<grid_for(f.v() / 8 * kUpW[lev] / 8), 256, 0, s>>>(f, kUpW[lev], w.gcat[lev], 0,
                                                                 act, out);
    SBM_LAUNCHED(1);
  }
  if ((rc = wgrad(n, w, E4, 4, w.pin[4], kCi[E4], w.ga4, s))) return rc;
  if ((rc = dgrad(n, w, E4, 4, w.ga4, w.gpin[4], s))) return rc;
  for (int lev = 3; lev >= 0; --lev) {
    const int l = kEnc[lev];
    const Dims& f = w.d[lev];
    const int C = kCo[l];
    k_bwd_skip<<<grid_for(f.v() * C / 8), 256, 0, s>>>(f, C, w.gcat[lev], kUpW[lev],
                                                       w.gpin[lev + 1], w.cat[lev], kUpW[lev],
                                                       w.genc[lev]);
    SBM_LAUNCHED(1);
    const bf16* x = lev == 0 ? w.in0 : w.pin[lev];
    if ((rc = wgrad(n, w, l, lev, x, kCi[l], w.genc[lev], s))) return rc;
    if (lev > 0 && (rc = dgrad(n, w, l, lev, w.genc[lev], w.gpin[lev], s))) return rc;
  }
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

int adam(sbm_net* n, float lr, cudaStream_t s) {
  n->step += 1;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f / (1.f - powf(b1, (float)n->step));
  const float c2 = 1.f / (1.f - powf(b2, (float)n->step));
  k_adam<<<grid_for(kL.total), 256, 0, s>>>(kL.total, 1, n->w32, n->grad, n->m, n->v, lr, b1, b2,
                                            eps, c1, c2, layer_tab(), n->wimg, n->wtimg,
                                            n->wimg16, n->wtimg16);
  SBM_LAUNCHED(1);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

uint16_t to_bf16_bits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

// Channels-last FP32 input features (nblk blocks of V voxels x 16) ->
// BF16 channel-group planes, each block planar over its own V.
int upload_features(bf16* dst, const float* src, int64_t V, int64_t nblk, cudaStream_t s) {
  const int64_t n = V * kFeat * nblk;
  std::vector<uint16_t> h((size_t)n);
  for (int64_t b = 0; b < nblk; ++b)
    for (int64_t v = 0; v < V; ++v)
      for (int c = 0; c < kFeat; ++c)
        h[(size_t)(b * V * kFeat + act_index(v, c, V))] =
            to_bf16_bits(src[(b * V + v) * kFeat + c]);
  SBM_CUDA_TRY(cudaMemcpyAsync(dst, h.data(), sizeof(uint16_t) * n, cudaMemcpyHostToDevice, s));
  SBM_CUDA_TRY(cudaStreamSynchronize(s));
  return SBM_OK;
}

uint64_t splitmix(uint64_t* x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

double unit(uint64_t* x) { return ((splitmix(x) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

int check_err(sbm_net* n) {
  int h = 0;
  SBM_CUDA_TRY(cudaMemcpyAsync(&h, n->err, sizeof(int), cudaMemcpyDeviceToHost, n->stream));
  SBM_CUDA_TRY(cudaStreamSynchronize(n->stream));
  if (h) {
    set_error_msg("tensor-core convolution wait expired");
    cudaMemsetAsync(n->err, 0, sizeof(int), n->stream);
    return SBM_ERR_TIMEOUT;
  }
  return SBM_OK;
}

// ------------------------------------------------ solver-side plan

// The coarse grid of a solve: cv = the fine interior / 4 per axis (the
// valid cells), c = cv rounded up to a multiple of 16 per axis (the grid the
// U-Net runs on; its extra cells are zero padding).  Coarse arrays use c's
// strides.

// Coarse-cell means of the coefficient (2 hk) and, for the CnE form, of the
// diagonal; the last block stores c_ref = mean of the former over the valid
// cells and the output factor sgn k_out / (scale c_ref).  sgn = -1 for the
// CnE form, whose operator diag - scale S has the opposite sign of the
// potential form's scale S, so that the network sees both in one convention.
__global__ void k_pc_coef(Geo g, Dims c, Dims cv, const float* __restrict__ hk,
                          const float* __restrict__ dg, float* __restrict__ coefc,
                          float* __restrict__ massc, double* partials, unsigned* counter,
                          float* scal, double kout, double scale, double sgn) {
  double acc = 0.0, accm = 0.0;
  NET_LOOP(cv.v()) {
    int i, j, k;
    vox(cv, t, &i, &j, &k);
    float s = 0.f, sm = 0.f;
    for (int kk = 0; kk < 4; ++kk)
      for (int jj = 0; jj < 4; ++jj) {
        const int64_t o = g.ix(4 * i + 1, 4 * j + jj + 1, 4 * k + kk + 1);
        const float4 v = *reinterpret_cast<const float4*>(hk + o);
        s += (v.x + v.y) + (v.z + v.w);
        if (dg) {
          const float4 d = *reinterpret_cast<const float4*>(dg + o);
          sm += (d.x + d.y) + (d.z + d.w);
        }
      }
    const float m = s * (2.f / 64.f);
    const int64_t tp = vid(c, i, j, k);
    coefc[tp] = m;
    acc += m;
    if (dg) {
      massc[tp] = sm * (1.f / 64.f);
      accm += sm * (1.f / 64.f);
    }
  }
  double v[2] = {acc, accm}, tot[2];
  if (grid_reduce<2>(v, partials, counter, tot)) {
    if (threadIdx.x == 0) {
      const double cref = tot[0] / (double)cv.v();
      scal[3] = (float)cref;
      scal[2] = (float)(sgn * kout / (scale * cref));
      scal[4] = (float)(scale * cref);
      scal[5] = (float)(tot[1] / (double)cv.v());
    }
  }
}

// Static input channels 1..15 of the coarse grid: R K / c_ref, 1, the two
// Dirichlet x-face masks and, for the CnE form (mass), x / (1 + x) with
// x = R diag / (scale c_ref), the weight of the mass term against the
// diffusion; zero in the padding.
__global__ void k_pc_feat(Dims c, Dims cv, const float* __restrict__ coefc,
                          const float* __restrict__ massc, const float* scal, int bcx0,
                          int bcx1, int mass, bf16* __restrict__ in0) {
  NET_LOOP(c.v()) {
    int i, j, k;
    vox(c, t, &i, &j, &k);
    const bool live = i < cv.ny && j < cv.nx && k < cv.nz;
    float f[kFeat];
#pragma unroll
    for (int q = 0; q < kFeat; ++q) f[q] = 0.f;
    if (live) {
      f[1] = coefc[t] / scal[3];
      f[2] = 1.f;
      f[3] = (bcx0 == SBM_BC_ZERO && j == 0) ? 1.f : 0.f;
      f[4] = (bcx1 == SBM_BC_ZERO && j == cv.nx - 1) ? 1.f : 0.f;
      if (mass) {
        const float x = massc[t] / scal[4];
        f[5] = x / (1.f + x);
      }
    }
#pragma unroll
    for (int q = 1; q < kFeat; ++q) in0[act_index(t, q, c.v())] = __float2bfloat16_rn(f[q]);
  }
}

// rc = R r (4x4x4 means of the FP32 residual) when it is stale (first use,
// residual replacement); s = RMS(rc - alpha rq), the scale of the next U-Net
// input (the pack kernel that follows applies the pending alpha rq).
__global__ void k_pc_restrict(Geo g, Dims c, Dims cv, const float* __restrict__ r,
                              float* __restrict__ rc, const float* __restrict__ rq,
                              double* partials, float* scal, CgState* st) {
  pdl_begin();
  if (st->done || st->pc_off || st->aux[1] != 0.0) return;
  const float alpha = (float)st->alpha;
  double acc = 0.0;
  NET_LOOP(cv.v()) {
    int i, j, k;
    vox(cv, t, &i, &j, &k);
    float s = 0.f;
    for (int kk = 0; kk < 4; ++kk)
      for (int jj = 0; jj < 4; ++jj) {
        const float4 v =
            *reinterpret_cast<const float4*>(r + g.ix(4 * i + 1, 4 * j + jj + 1, 4 * k + kk + 1));
        s += (v.x + v.y) + (v.z + v.w);
      }
    const float m = s * (1.f / 64.f);
    const int64_t tc = vid(c, i, j, k);
    rc[tc] = m;
    const float mn = m - alpha * rq[tc];
    acc += (double)mn * (double)mn;
  }
  double v[1] = {acc}, tot[1];
  if (grid_reduce<1>(v, partials, &st->counter[4], tot)) {
    if (threadIdx.x == 0) {
      const double s = sqrt(tot[0] / (double)cv.v());
      scal[0] = (float)s;
      scal[1] = s > 0.0 ? (float)(1.0 / s) : 0.f;
      st->aux[1] = 1.0;     // rc holds R r of the current residual
      st->aux[2] = tot[0];  // |rc - alpha rq|^2: |rc|^2 once the pack has applied alpha
    }
  }
}

// rc -= alpha rq (R r of the updated residual, alpha the step the
// preconditioner kernel that follows applies to r) and the U-Net's residual
// channel rc / s.  |rc|^2 of the updated rc is already in aux[2] (set with
// s by the direction kernel or the restriction).
__global__ void k_pc_pack(int64_t V, float* __restrict__ rc, const float* __restrict__ rq,
                          const float* scal, bf16* __restrict__ in0, const CgState* st) {
  pdl_begin();
  if (st->done || st->pc_off) return;
  const float inv = scal[1];
  const float alpha = (float)st->alpha;
  NET_LOOP(V) {
    const float m = rc[t] - alpha * rq[t];
    rc[t] = m;
    in0[act_index(t, 0, V)] = __float2bfloat16_rn(m * inv);
  }
}

// Last block of the flexible CG's preconditioner kernel, which also applies
// the pending r -= alpha q (rupd; not on the first residual): rho = z.r,
// beta = -z.q_old / p.q_old (0 on the first residual), and what an update
// of r decides -- the iteration count, the learned preconditioner's
// progress check (the FP32 residual norm must halve within 50 iterations,
// else the solve continues as Jacobi-PCG, so a network that does not fit
// the problem cannot stall it) and the reliable-update trigger.
__device__ void fcg_close(CgState* st, double zr, double zq, double rr, bool rupd, int err) {
  const double beta = st->initial ? 0.0 : -zq / st->pq;
  st->initial = 0;
  st->rho = zr;
  st->beta = beta;
  if (err) {
    st->done = 5;
    return;
  }
  if (!isfinite(zr) || !isfinite(beta)) {
    st->done = 3;
    return;
  }
  if (!rupd) return;
  const int it = st->iter + 1;
  st->iter = it;
  if (!st->pc_off) {
    if (st->aux[3] <= 0.0 || rr < 0.25 * st->aux[3]) {
      st->aux[3] = rr;
      st->stall_iter = it;
    } else if (it - st->stall_iter > 50) {
      st->pc_off = 1;
    }
  }
  if (!isfinite(rr) || !isfinite(st->alpha)) {
    st->done = 3;
    return;
  }
  const double maxrr = fmax(st->maxrr, rr);
  if ((rr < st->delta2 * maxrr) || (rr <= st->tol * st->tol * st->aux[0]) || (it >= st->max_it))
    st->reliable = 1;
  st->rr = rr;
  st->maxrr = maxrr;
}

// Interpolation weights of the 4 fine cells of one coarse cell along an
// axis: fine cell e of coarse cell m lies at m - 3/8 + e/4 in coarse units.
__device__ __forceinline__ void interp1(int fi, int n, int* lo, int* hi, float* wlo) {
  const int m = fi >> 2, e = fi & 3;
  *lo = (e < 2) ? max(m - 1, 0) : m;
  *hi = (e < 2) ? m : min(m + 1, n - 1);
  *wlo = 0.375f - 0.25f * (float)(e & 1) + 0.5f * (float)(e >> 1);  // 3/8, 1/8, 7/8, 5/8
}

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// The additive form: r -= alpha q (the pending update of the flexible CG,
// not on the first residual), then z = invd*r + f * P(out) over the fine
// interior, f = s k_out / (scale c_ref); z.r, z.q_old and r.r reduced; the
// last block runs fcg_close.  One item = 4 y-consecutive fine cells (one
// coarse cell in y) on one x row, marched over the 4 fine planes of one
// coarse z cell, so the coarse values (3 y x 2 x x 3 z) are loaded once for
// 16 cells.  With the coarse part switched off (pc_off): z = invd*r.
__global__ void __launch_bounds__(256)
    k_pc_prolong(Geo g, Dims c, Dims cv, const float* __restrict__ out, const float* scal,
                 float* __restrict__ r, const float* __restrict__ iv,
                 const float* __restrict__ q, float* __restrict__ z, const int* err,
                 double* partials, CgState* st) {
  pdl_begin();
  if (st->done) return;
  const bool coarse = st->pc_off == 0;  // off: z = D^-1 r (Jacobi-PCG)
  const float f = coarse ? scal[0] * scal[2] : 0.f;
  const bool rupd = st->initial == 0;
  const float alpha = (float)st->alpha;
  float a_zr = 0.f, a_zq = 0.f, a_rr = 0.f;
  {
    const int nchunk = g.ny / 4;
    const int64_t n = (int64_t)nchunk * g.nx * (g.nz / 4);
    const float wl[4] = {0.375f, 0.125f, 0.875f, 0.625f};
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n;
         u += (int64_t)gridDim.x * blockDim.x) {
      const int m = (int)(u % nchunk);
      const int64_t rr = u / nchunk;
      const int j = (int)(rr % g.nx) + 1;
      const int kc = (int)(rr / g.nx);
      int x0, x1;
      float wx;
      interp1(j - 1, cv.nx, &x0, &x1, &wx);
      const int ys[3] = {max(m - 1, 0), m, min(m + 1, cv.ny - 1)};
      const int zs[3] = {max(kc - 1, 0), kc, min(kc + 1, cv.nz - 1)};
      float cx[3][3] = {};  // [y neighbour][z plane], interpolated in x
      if (coarse) {
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          const int64_t r0 = (int64_t)c.ny * (x0 + (int64_t)c.nx * zs[b]);
          const int64_t r1 = (int64_t)c.ny * (x1 + (int64_t)c.nx * zs[b]);
#pragma unroll
          for (int a = 0; a < 3; ++a) cx[a][b] = wx * out[r0 + ys[a]] + (1.f - wx) * out[r1 + ys[a]];
        }
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int lo = e < 2 ? 0 : 1;  // coarse planes (lo, lo + 1) of fine plane e
        const float wz = wl[e];
        float col[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) col[a] = wz * cx[a][lo] + (1.f - wz) * cx[a][lo + 1];
        const float e4[4] = {0.375f * col[0] + 0.625f * col[1], 0.125f * col[0] + 0.875f * col[1],
                             0.875f * col[1] + 0.125f * col[2], 0.625f * col[1] + 0.375f * col[2]};
        const int64_t idx = g.ix(4 * m + 1, j, 4 * kc + 1 + e);
        float4 rv = *reinterpret_cast<const float4*>(r + idx);
        const float4 dv = *reinterpret_cast<const float4*>(iv + idx);
        const float4 qv = *reinterpret_cast<const float4*>(q + idx);
        if (rupd) {
          rv.x -= alpha * qv.x; rv.y -= alpha * qv.y; rv.z -= alpha * qv.z; rv.w -= alpha * qv.w;
          *reinterpret_cast<float4*>(r + idx) = rv;
        }
        float4 zv;
        zv.x = dv.x * rv.x + f * e4[0];
        zv.y = dv.y * rv.y + f * e4[1];
        zv.z = dv.z * rv.z + f * e4[2];
        zv.w = dv.w * rv.w + f * e4[3];
        *reinterpret_cast<float4*>(z + idx) = zv;
        a_zr += (zv.x * rv.x + zv.y * rv.y) + (zv.z * rv.z + zv.w * rv.w);
        a_zq += (zv.x * qv.x + zv.y * qv.y) + (zv.z * qv.z + zv.w * qv.w);
        a_rr += (rv.x * rv.x + rv.y * rv.y) + (rv.z * rv.z + rv.w * rv.w);
      }
    }
  }
  double v[3] = {(double)a_zr, (double)a_zq, (double)a_rr}, tot[3];
  if (grid_reduce<3>(v, partials, &st->counter[5], tot))
    if (threadIdx.x == 0) fcg_close(st, tot[0], tot[1], tot[2], rupd, *err);
}

// The multiplicative form z = z1 + omega*invd*(r - A z1), z1 = f P(out), by
// tiles of 64 (y) x 8 (x) x 4 (z) fine cells, after the pending update
// r -= alpha q of the flexible CG (not on the first residual).  A tile's r
// and q boxes and its hk box with the one-cell halo arrive by TMA, and its
// coarse window (18 y x 4 x x 3 z cells, clamped) by per-thread cp.async,
// into the other half of a double buffer while the block computes the tile
// before it.  The block interpolates the window in x and then in z onto the
// tile's fine x / z positions with their one-cell halo (the order of
// k_pc_prolong); each thread then takes 4 y-consecutive cells (one coarse y
// cell), interpolates z1 in y for them and their 6 neighbours from three
// coarse values per row, and applies the FP32 operator with the
// search-direction ghost rules.  The Jacobi weight invd is formed from the
// same half coefficients (k_invdiag's face sums; the reciprocal within
// 1 ulp), so it is not read.  The cells' arithmetic runs on pairs of FP32
// lanes, and a thread's two items (planes zl and zl + 2) are unrolled.
// Global traffic per cell: r, q_old and hk read, r and z written (20 B).
// z.r, z.q_old and r.r are reduced and the last block runs fcg_close.
// Tiles are walked grid-stride (every block the same count: the barriers
// are uniform); two barriers per tile.
// Weight of the Jacobi step of the multiplicative form.  Flexible-CG
// iterations on the GPU (256^3 headline / 128^3 and 256^3 held-out / 64^3 /
// 128^3 structures): omega 1.5: 86/56/82/54/67, 1.9: 72/47/71/51/53,
// 2.1: 63/46/66/52/50, 2.3: 61/49/63/55/50, 2.6: 61/55/63/60/56; small
// grids hardly depend on it, large ones gain most near 2.1-2.3.
#ifndef SBM_PC_OMEGA
#define SBM_PC_OMEGA 2.3f
#endif
constexpr float kPcOmega = SBM_PC_OMEGA;
constexpr int kMTY = 64, kMTX = 8, kMTZ = 4;
constexpr int kWY = kMTY / 4 + 2;  // coarse y window
// Tensor maps of the multiplicative step: r and q (64 x 8 x 4 boxes, the
// tile) and hk (72 x 10 x 6 boxes, the tile with its one-cell halo, x-start
// rounded down to a 16-byte boundary), over the FP32 layout.
struct MultMaps {
  CUtensorMap r, q, hk;
};
constexpr int kMRB = kMTY * kMTX * kMTZ * 4;                    // r (and q) box bytes (8192)
constexpr int kMHB = (kMTY + 8) * (kMTX + 2) * (kMTZ + 2) * 4;  // hk box bytes (17280)
constexpr int kMBuf = (2 * kMRB + kMHB + 127) / 128 * 128;      // one staging buffer: r, q, hk
constexpr int kMWin = 3 * (kMTX / 4 + 2) * kWY;                 // coarse window (216 values)
constexpr size_t kMultSmem = 2 * (size_t)kMBuf + 2 * sizeof(uint64_t);

// A tile of the walk as (y, x, z) tile coordinates, y fastest.
struct MultTile {
  int by, bx, bz;
};

// 1 / d by the hardware reciprocal approximation (PTX rcp.approx.f32,
// within 1 ulp): the weight of a smoothing step needs no correct rounding.
__device__ __forceinline__ float rcp_approx(float d) {
  float y;
  asm("rcp.approx.f32 %0, %1;" : "=f"(y) : "f"(d));
  return y;
}

__global__ void __launch_bounds__(256, 3)
    k_pc_mult_tiled(const __grid_constant__ MultMaps maps, Geo g, Dims c, Dims cv,
                    const float* __restrict__ out, const float* scal, float* __restrict__ r,
                    const float* __restrict__ dg, float scale,
                    int bcx0, int bcx1, float omega, float* __restrict__ z, const int* err,
                    double* partials, CgState* st) {
  __shared__ float sA[2][3][kMTX / 4 + 2][kWY];  // coarse windows, double-buffered
  __shared__ float sC[kMTZ + 2][kMTX + 2][kWY];   // f z1 interpolated in x and z
  extern __shared__ __align__(128) unsigned char dsm[];
  uint64_t* const bar = reinterpret_cast<uint64_t*>(dsm + 2 * kMBuf);
  pdl_begin();
  if (st->done) return;
  const bool coarse = st->pc_off == 0;  // off: z = D^-1 r (Jacobi-PCG)
  const float f = coarse ? scal[0] * scal[2] : 0.f;
  const bool rupd = st->initial == 0;
  const float alpha = (float)st->alpha;
  const int tid = threadIdx.x;
  const int nty = (g.ny + kMTY - 1) / kMTY, ntx = g.nx / kMTX;  // the last y tile may be partial
  const int ntiles = nty * ntx * (g.nz / kMTZ);
  // the walk: tile blockIdx.x, then steps of gridDim.x tiles, advanced in
  // tile coordinates (no division per tile)
  auto decomp = [&](int t) {
    MultTile m;
    m.bz = t / (nty * ntx);
    const int rem = t - m.bz * nty * ntx;
    m.bx = rem / nty;
    m.by = rem - m.bx * nty;
    return m;
  };
  const MultTile step = decomp(gridDim.x);
  auto advance = [&](MultTile m) {
    m.by += step.by;
    int carry = m.by >= nty;
    if (carry) m.by -= nty;
    m.bx += step.bx + carry;
    carry = m.bx >= ntx;
    if (carry) m.bx -= ntx;
    m.bz += step.bz + carry;
    return m;
  };
  // thread 0 stages the r, q and hk boxes of a tile into buffer b
  auto stage = [&](MultTile m, int b) {
    unsigned char* B = dsm + (size_t)b * kMBuf;
    const int ry = kMTY * m.by + 1 + kOff32, rx = kMTX * m.bx + 1, rz = kMTZ * m.bz + 1;
    mbar_expect_tx(&bar[b], (unsigned)(2 * kMRB + kMHB));
    tma_load_3d(B, &maps.r, ry, rx, rz, &bar[b]);
    tma_load_3d(B + kMRB, &maps.q, ry, rx, rz, &bar[b]);
    tma_load_3d(B + 2 * kMRB, &maps.hk, kMTY * m.by, kMTX * m.bx, kMTZ * m.bz, &bar[b]);
  };
  // threads 0..215 fetch one value each of a tile's coarse window into sA[b]
  // (y fastest, then x, then z; coarse indexes clamped to the grid, so the
  // interpolation below needs no clamping of its own)
  auto fetch_window = [&](MultTile m, int b) {
    if (coarse && tid < kMWin) {
      const int wy = tid % kWY, wx = (tid / kWY) % (kMTX / 4 + 2);
      const int wz = tid / (kWY * (kMTX / 4 + 2));
      const int cy = min(max((kMTY / 4) * m.by - 1 + wy, 0), cv.ny - 1);
      const int cx = min(max((kMTX / 4) * m.bx - 1 + wx, 0), cv.nx - 1);
      const int cz = min(max(m.bz - 1 + wz, 0), cv.nz - 1);
      cp_async4(&sA[b][wz][wx][wy], out + cy + (int64_t)c.ny * (cx + (int64_t)c.nx * cz));
    }
    cp_async_commit();
  };
  MultTile cur = decomp(blockIdx.x);
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if ((int)blockIdx.x < ntiles) stage(cur, 0);
  }
  if ((int)blockIdx.x < ntiles) fetch_window(cur, 0);
  __syncthreads();  // the barriers' initialisation is seen by every thread
  int n_issued = (int)blockIdx.x < ntiles ? 1 : 0;  // tiles staged (thread 0's count)
  // Cell roles: item h of a thread is 4 y-consecutive cells (coarse y cell
  // mq) on x row xl of plane zl + 2h; offsets of item 0 in the r / q box,
  // the hk box and sC (item 1: + 2 planes)
  const int mq = tid % (kMTY / 4), xl = (tid / (kMTY / 4)) % kMTX, zl = tid / ((kMTY / 4) * kMTX);
  const int so = 4 * tid;
  constexpr int hxs = kMTY + 8, hzs = (kMTY + 8) * (kMTX + 2), cxs = kWY, czs = kWY * (kMTX + 2);
  const int ho = ((zl + 1) * (kMTX + 2) + xl + 1) * hxs + 4 * mq + 4;
  const int co = ((zl + 1) * (kMTX + 2) + xl + 1) * cxs + mq;
  // the cells' arithmetic runs on pairs of FP32 lanes (paired FMA / add /
  // multiply), one pair per two y-consecutive cells
  const float2 nal = make_float2(-alpha, -alpha), om2 = make_float2(omega, omega);
  const float2 sc2 = make_float2(scale, scale), nsc2 = make_float2(-scale, -scale);
  const float2 zero2 = make_float2(0.f, 0.f);
  float2 acc_zr = zero2, acc_zq = zero2, acc_rr = zero2;
  bool ok = true;
  int n = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, cur = advance(cur), ++n) {
    const int y0 = kMTY * cur.by + 1, x0 = kMTX * cur.bx + 1, z0 = kMTZ * cur.bz + 1;
    // the tile's boxes and window have landed (the wait decision is made
    // uniform), and every thread is done with the previous tile: its
    // buffer and window take the next tile's
    cp_async_wait_all();
    const bool w_ok = mbar_wait_bounded(&bar[n & 1], (unsigned)((n >> 1) & 1), 1u << 20);
    if (!__syncthreads_and(w_ok)) {
      ok = false;
      break;
    }
    if (tile + (int)gridDim.x < ntiles) {
      const MultTile nxt = advance(cur);
      if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        stage(nxt, (n + 1) & 1);
        ++n_issued;
      }
      fetch_window(nxt, (n + 1) & 1);
    }
    if (coarse) {
      // x interpolation of the window's 3 z planes, then z interpolation to
      // the fine planes z0-1 .. z0+kMTZ (fine plane zf at coarse window
      // cells (zlo, zlo + 1) with weight wz on zlo), scaled by f
      // (the roles are the same in every tile: tiles start at multiples of 4
      // fine cells, so the weights repeat).  Threads 0..179 own the column
      // (x position xf, y entry cy) of the fine x positions x0-1 ..
      // x0+kMTX; fine x position xf lies in the window's coarse cells
      // (xlo, xlo + 1) with weight wxl on xlo.
      if (tid < (kMTX + 2) * kWY) {
        const int cy = tid % kWY, xf = tid / kWY;
        const int xe = (xf - 1) & 3, xm = (xf - 1) >> 2;  // interp1 of fine index 8 bx - 1 + xf
        const int xlo = xe < 2 ? xm : xm + 1;
        const float wxl = 0.375f - 0.25f * (float)(xe & 1) + 0.5f * (float)(xe >> 1);
        const float* W = &sA[n & 1][0][0][0] + xlo * kWY + cy;
        constexpr int wzs = (kMTX / 4 + 2) * kWY;
        float bz3[3];
#pragma unroll
        for (int zz = 0; zz < 3; ++zz)
          bz3[zz] = wxl * W[zz * wzs] + (1.f - wxl) * W[zz * wzs + kWY];
        float* C = &sC[0][0][0] + xf * kWY + cy;
#pragma unroll
        for (int zf = 0; zf < kMTZ + 2; ++zf) {
          const int ze = (zf - 1) & 3, zm = (zf - 1) >> 2;
          const int zlo = ze < 2 ? zm : zm + 1;
          const float wz = 0.375f - 0.25f * (float)(ze & 1) + 0.5f * (float)(ze >> 1);
          C[zf * czs] = f * (wz * bz3[zlo] + (1.f - wz) * bz3[zlo + 1]);
        }
      }
      __syncthreads();
    }
    const float* R = reinterpret_cast<const float*>(dsm + (size_t)(n & 1) * kMBuf);
    const float* Q = R + kMRB / 4;
    const float* H = R + 2 * kMRB / 4;
    const int i0 = y0 + 4 * mq, j = x0 + xl;
    const int64_t gbase = g.ix(i0, j, z0 + zl);
    // both items unrolled: their independent chains interleave, and the
    // register allocation has no spills (0.088 -> 0.072 ms at 256^3)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = z0 + zl + 2 * h;
      if (i0 > g.ny) break;  // beyond a partial tile (ny is a multiple of 4)
      const int64_t idx = gbase + 2 * h * g.sz;
      // the thread's 4 cells as two pairs, (i0, i0+1) and (i0+2, i0+3)
      const int sh = so + h * (2 * kMTX * kMTY);
      const float4 qv = *reinterpret_cast<const float4*>(Q + sh);
      const float4 rv = *reinterpret_cast<const float4*>(R + sh);
      const float2 q0 = make_float2(qv.x, qv.y), q1 = make_float2(qv.z, qv.w);
      float2 r0 = make_float2(rv.x, rv.y), r1 = make_float2(rv.z, rv.w);
      if (rupd) {
        r0 = __ffma2_rn(nal, q0, r0);
        r1 = __ffma2_rn(nal, q1, r1);
        *reinterpret_cast<float4*>(r + idx) = make_float4(r0.x, r0.y, r1.x, r1.y);
      }
      // hk box: (zl + 2h + 1, xl + 1, column 4 mq + 4) is the first cell
      const float* hk = H + ho + h * (2 * hzs);
      const float4 k4 = *reinterpret_cast<const float4*>(hk);
      const float4 kx0 = *reinterpret_cast<const float4*>(hk - hxs);
      const float4 kx1 = *reinterpret_cast<const float4*>(hk + hxs);
      const float4 kz0 = *reinterpret_cast<const float4*>(hk - hzs);
      const float4 kz1 = *reinterpret_cast<const float4*>(hk + hzs);
      const float kyl = hk[-1], kyh = hk[4];
      const float2 kc0 = make_float2(k4.x, k4.y), kc1 = make_float2(k4.z, k4.w);
      // face coefficients c_f = hk_nb + hk_c; the y faces of the four cells
      // are F_t = hk(i0-1+t) + hk(i0+t), t = 0..4 (cell y: F_y below, F_y+1
      // above).  A face outside the operator (a Neumann or copied ghost)
      // gets c_f = 0: it then drops out of the diagonal and of S(z1), as the
      // ghost rules make its difference vanish.
      float2 fym0 = __fadd2_rn(make_float2(kyl, k4.x), kc0);         // F0, F1
      const float2 fym1 = __fadd2_rn(make_float2(k4.y, k4.z), kc1);  // F2, F3
      float f4 = kyh + k4.w;
      if (i0 == 1) fym0.x = 0.f;
      if (i0 + 3 == g.ny) f4 = 0.f;
      const float2 fyp0 = make_float2(fym0.y, fym1.x), fyp1 = make_float2(fym1.y, f4);
      float2 fxm0 = __fadd2_rn(make_float2(kx0.x, kx0.y), kc0);
      float2 fxm1 = __fadd2_rn(make_float2(kx0.z, kx0.w), kc1);
      float2 fxp0 = __fadd2_rn(make_float2(kx1.x, kx1.y), kc0);
      float2 fxp1 = __fadd2_rn(make_float2(kx1.z, kx1.w), kc1);
      float2 fzm0 = __fadd2_rn(make_float2(kz0.x, kz0.y), kc0);
      float2 fzm1 = __fadd2_rn(make_float2(kz0.z, kz0.w), kc1);
      float2 fzp0 = __fadd2_rn(make_float2(kz1.x, kz1.y), kc0);
      float2 fzp1 = __fadd2_rn(make_float2(kz1.z, kz1.w), kc1);
      if (j == 1 && !bcx0) fxm0 = fxm1 = zero2;
      if (j == g.nx && !bcx1) fxp0 = fxp1 = zero2;
      if (k == 1) fzm0 = fzm1 = zero2;
      if (k == g.nz) fzp0 = fzp1 = zero2;
      // the Jacobi weight 1 / A_cc, faces summed in k_invdiag's order
      const float2 s0 = __fadd2_rn(
          __fadd2_rn(__fadd2_rn(__fadd2_rn(__fadd2_rn(fym0, fyp0), fxm0), fxp0), fzm0), fzp0);
      const float2 s1 = __fadd2_rn(
          __fadd2_rn(__fadd2_rn(__fadd2_rn(__fadd2_rn(fym1, fyp1), fxm1), fxp1), fzm1), fzp1);
      float2 dg0 = zero2, dg1 = zero2, d0, d1;
      if (dg) {  // the CnE form: A p = diag p - scale S(p)
        const float4 d4 = *reinterpret_cast<const float4*>(dg + idx);
        dg0 = make_float2(d4.x, d4.y);
        dg1 = make_float2(d4.z, d4.w);
        d0 = __ffma2_rn(sc2, s0, dg0);
        d1 = __ffma2_rn(sc2, s1, dg1);
      } else {
        d0 = __fmul2_rn(nsc2, s0);
        d1 = __fmul2_rn(nsc2, s1);
      }
      const float2 da0 = make_float2(d0.x != 0.f ? rcp_approx(d0.x) : 0.f,
                                     d0.y != 0.f ? rcp_approx(d0.y) : 0.f);
      const float2 da1 = make_float2(d1.x != 0.f ? rcp_approx(d1.x) : 0.f,
                                     d1.y != 0.f ? rcp_approx(d1.y) : 0.f);
      float2 z0v, z1v;
      if (coarse) {
        // y interpolation: coarse cells (m-1, m, m+1) are window entries mq,
        // mq+1, mq+2; z1 at the fine offsets -1..4 of this coarse cell as
        // the pairs (-1, 0), (1, 2), (3, 4)
        const float* cc0 = &sC[0][0][0] + co + h * (2 * czs);
        const float a0 = cc0[0], a1 = cc0[1], a2 = cc0[2];
        const float2 A1 = make_float2(a1, a1);
        const float2 cm = __ffma2_rn(make_float2(0.625f, 0.375f), make_float2(a0, a0),
                                     __fmul2_rn(make_float2(0.375f, 0.625f), A1));
        const float2 cc = __ffma2_rn(make_float2(0.125f, 0.125f), make_float2(a0, a2),
                                     __fmul2_rn(make_float2(0.875f, 0.875f), A1));
        const float2 cp = __ffma2_rn(make_float2(0.375f, 0.625f), make_float2(a2, a2),
                                     __fmul2_rn(make_float2(0.625f, 0.375f), A1));
        const float2 pc0 = make_float2(cm.y, cc.x), pc1 = make_float2(cc.y, cp.x);
        // the four neighbour rows (x-1, x+1, z-1, z+1), offsets 0..3
        auto row = [&](const float* rp, float2& lo, float2& hi) {
          const float b0 = rp[0], b1 = rp[1], b2 = rp[2];
          const float2 B1 = make_float2(b1, b1);
          lo = __ffma2_rn(make_float2(0.375f, 0.125f), make_float2(b0, b0),
                          __fmul2_rn(make_float2(0.625f, 0.875f), B1));
          hi = __ffma2_rn(make_float2(0.125f, 0.375f), make_float2(b2, b2),
                          __fmul2_rn(make_float2(0.875f, 0.625f), B1));
        };
        float2 xm0, xm1, xp0, xp1, zm0, zm1, zp0, zp1;
        row(cc0 - cxs, xm0, xm1);
        row(cc0 + cxs, xp0, xp1);
        row(cc0 - czs, zm0, zm1);
        row(cc0 + czs, zp0, zp1);
        // a Dirichlet x face reads a zero ghost (a Neumann one has c_f = 0)
        if (j == 1) xm0 = xm1 = zero2;
        if (j == g.nx) xp0 = xp1 = zero2;
        // S(z1) = sum_f c_f (z1_nb - z1_c), faces in the order of face_sum
        auto fsum = [&](float2 pc, float2 pyp, float2 pym, float2 pxp, float2 pxm, float2 pzp,
                        float2 pzm, float2 cyp, float2 cym, float2 cxp, float2 cxm, float2 czp,
                        float2 czm) {
          float2 sv = __fmul2_rn(cyp, __fadd2_rn(pyp, neg2(pc)));
          sv = __ffma2_rn(cym, __fadd2_rn(pym, neg2(pc)), sv);
          sv = __ffma2_rn(cxp, __fadd2_rn(pxp, neg2(pc)), sv);
          sv = __ffma2_rn(cxm, __fadd2_rn(pxm, neg2(pc)), sv);
          sv = __ffma2_rn(czp, __fadd2_rn(pzp, neg2(pc)), sv);
          return __ffma2_rn(czm, __fadd2_rn(pzm, neg2(pc)), sv);
        };
        const float2 sv0 = fsum(pc0, cc, cm, xp0, xm0, zp0, zm0, fyp0, fym0, fxp0, fxm0, fzp0,
                                fzm0);
        const float2 sv1 = fsum(pc1, cp, cc, xp1, xm1, zp1, zm1, fyp1, fym1, fxp1, fxm1, fzp1,
                                fzm1);
        // -A z1 = scale S(z1) - diag z1 (potential form: -scale S(z1))
        float2 naz0, naz1;
        if (dg) {
          naz0 = __ffma2_rn(neg2(dg0), pc0, __fmul2_rn(sc2, sv0));
          naz1 = __ffma2_rn(neg2(dg1), pc1, __fmul2_rn(sc2, sv1));
        } else {
          naz0 = __fmul2_rn(nsc2, sv0);
          naz1 = __fmul2_rn(nsc2, sv1);
        }
        z0v = __ffma2_rn(om2, __fmul2_rn(da0, __fadd2_rn(r0, naz0)), pc0);
        z1v = __ffma2_rn(om2, __fmul2_rn(da1, __fadd2_rn(r1, naz1)), pc1);
      } else {
        z0v = __fmul2_rn(da0, r0);
        z1v = __fmul2_rn(da1, r1);
      }
      acc_zr = __ffma2_rn(z0v, r0, __ffma2_rn(z1v, r1, acc_zr));
      acc_zq = __ffma2_rn(z0v, q0, __ffma2_rn(z1v, q1, acc_zq));
      acc_rr = __ffma2_rn(r0, r0, __ffma2_rn(r1, r1, acc_rr));
      *reinterpret_cast<float4*>(z + idx) = make_float4(z0v.x, z0v.y, z1v.x, z1v.y);
    }
  }
  if (!ok) {
    // a staging wait expired: the copies still landing are waited out
    // (only the last staged tile of each buffer can be) and the solve stops
    if (tid == 0) {
      st->done = 5;
      for (int b = 0; b < 2; ++b) {
        const int cnt = (n_issued + 1 - b) / 2;  // tiles staged into buffer b
        if (cnt > 0) mbar_wait_bounded(&bar[b], (unsigned)((cnt - 1) & 1), 1u << 20);
      }
    }
    cp_async_wait_all();
    acc_zr = acc_zq = acc_rr = zero2;
  }
  double v[3] = {(double)acc_zr.x + acc_zr.y, (double)acc_zq.x + acc_zq.y,
                 (double)acc_rr.x + acc_rr.y},
         tot[3];
  if (grid_reduce<3>(v, partials, &st->counter[5], tot))
    if (threadIdx.x == 0) fcg_close(st, tot[0], tot[1], tot[2], rupd, *err);
}

struct NetPc {
  sbm_net* net = nullptr;
  double kout = 1.0;
  Dims c{};   // the U-Net's grid: cv rounded up to multiples of 16 (zero padding)
  Dims cv{};  // the coarse cells of the solve's grid (fine interior / 4)
  Work* w = nullptr;
  float* rc = nullptr;   // R r of the current residual
  float* rq = nullptr;   // R q of the current direction (flexible-CG direction kernel)
  float* coefc = nullptr;
  float* massc = nullptr;  // coarse means of the CnE diagonal
  float* zf = nullptr;   // FP32 z (g32 layout)
  float* scal = nullptr; // s, 1/s, k_out/(scale c_ref), c_ref
  double* parts = nullptr;
  unsigned* cnt = nullptr;
  // operator of the current solve, for the multiplicative smoothing step
  const float* hk32 = nullptr;
  const float* dg32 = nullptr;  // the CnE form's diagonal (null: potential form)
  MultMaps mmaps{};             // tensor maps of the multiplicative step (r, q, hk)
  float scale = 1.f;
  int bcx0 = 0, bcx1 = 0;
  void release() {
    delete w;
    w = nullptr;
    cudaFree(rc);
    cudaFree(rq);
    cudaFree(coefc);
    cudaFree(massc);
    cudaFree(zf);
    cudaFree(scal);
    cudaFree(parts);
    cudaFree(cnt);
    rc = rq = coefc = massc = zf = scal = nullptr;
    parts = nullptr;
    cnt = nullptr;
  }
};

}  // namespace netd

// The learned preconditioner applies to grids whose extents are multiples
// of 16 (coarse grids of whole 4^3 blocks, zero-padded to multiples of 16
// for the U-Net's four poolings), to the potential form, and to the CnE
// form (diag - scale S) when the network was trained with the mass channel.
bool net_pc_usable(const sbm_ctx* ctx, int form) {
  const netd::NetPc* pc = static_cast<const netd::NetPc*>(ctx->net);
  const Geo& g = ctx->g;
  return pc && pc->net && (form == 0 || pc->net->mass) && g.ny % 16 == 0 && g.nx % 16 == 0 &&
         g.nz % 16 == 0;
}

int net_pc_begin(sbm_ctx* ctx, const float* hk32, const float* dg32, const float* r32,
                 const float* q32, double scale, int bcx0, int bcx1, cudaStream_t s) {
  netd::NetPc* pc = static_cast<netd::NetPc*>(ctx->net);
  int rc = conv3_init();
  if (rc) return rc;
  static bool mult_attr = false;
  if (!mult_attr) {
    SBM_CUDA_TRY(cudaFuncSetAttribute(netd::k_pc_mult_tiled,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)netd::kMultSmem));
    // three blocks of ~72 KB per SM: the largest shared-memory carveout
    SBM_CUDA_TRY(cudaFuncSetAttribute(netd::k_pc_mult_tiled,
                                      cudaFuncAttributePreferredSharedMemoryCarveout,
                                      (int)cudaSharedmemCarveoutMaxShared));
    mult_attr = true;
  }
  const Geo& g = ctx->g32;
  const netd::Dims cv{g.ny / 4, g.nx / 4, g.nz / 4, g.nz / 4};
  auto r16 = [](int n) { return (n + 15) / 16 * 16; };
  const netd::Dims c{r16(cv.ny), r16(cv.nx), r16(cv.nz), r16(cv.nz)};
  if (!pc->w || pc->cv.ny != cv.ny || pc->cv.nx != cv.nx || pc->cv.nz != cv.nz) {
    pc->release();
    pc->c = c;
    pc->cv = cv;
    pc->w = netd::make_work(c, false, &cv);
    if (!pc->w || cudaMalloc(&pc->rc, sizeof(float) * c.v()) ||
        cudaMalloc(&pc->rq, sizeof(float) * c.v()) ||
        cudaMalloc(&pc->coefc, sizeof(float) * c.v()) ||
        cudaMalloc(&pc->massc, sizeof(float) * c.v()) ||
        cudaMalloc(&pc->zf, sizeof(float) * g.nh) || cudaMalloc(&pc->scal, sizeof(float) * 8) ||
        cudaMalloc(&pc->parts, sizeof(double) * 152 * 16 * 2) ||
        cudaMalloc(&pc->cnt, sizeof(unsigned) * 4)) {
      pc->release();
      return SBM_ERR_NOMEM;
    }
    // the padding cells of the coarse arrays stay zero
    SBM_CUDA_TRY(cudaMemsetAsync(pc->rc, 0, sizeof(float) * c.v(), s));
    SBM_CUDA_TRY(cudaMemsetAsync(pc->coefc, 0, sizeof(float) * c.v(), s));
    SBM_CUDA_TRY(cudaMemsetAsync(pc->massc, 0, sizeof(float) * c.v(), s));
    SBM_CUDA_TRY(cudaMemsetAsync(pc->zf, 0, sizeof(float) * g.nh, s));
    SBM_CUDA_TRY(cudaMemsetAsync(pc->cnt, 0, sizeof(unsigned) * 4, s));
    SBM_CUDA_TRY(cudaMemsetAsync(pc->scal, 0, sizeof(float) * 8, s));
  }
  // no direction yet: the first pack applies alpha = 0 to a zero R q
  SBM_CUDA_TRY(cudaMemsetAsync(pc->rq, 0, sizeof(float) * c.v(), s));
  pc->hk32 = hk32;
  pc->dg32 = dg32;
  if (!make_map_box(&pc->mmaps.r, r32 - kOff32, g, netd::kMTY, netd::kMTX, netd::kMTZ) ||
      !make_map_box(&pc->mmaps.q, q32 - kOff32, g, netd::kMTY, netd::kMTX, netd::kMTZ) ||
      !make_map_box(&pc->mmaps.hk, hk32 - kOff32, g, netd::kMTY + 8, netd::kMTX + 2,
                    netd::kMTZ + 2))
    return SBM_ERR_STATE;
  pc->scale = (float)scale;
  pc->bcx0 = bcx0;
  pc->bcx1 = bcx1;
  netd::k_pc_coef<<<netd::grid_for(cv.v()), 256, 0, s>>>(g, c, cv, hk32, dg32, pc->coefc,
                                                          pc->massc, pc->parts, pc->cnt, pc->scal,
                                                          pc->kout, scale, dg32 ? -1.0 : 1.0);
  netd::k_pc_feat<<<netd::grid_for(c.v()), 256, 0, s>>>(c, cv, pc->coefc, pc->massc, pc->scal,
                                                         bcx0, bcx1, dg32 ? 1 : 0, pc->w->in0);
  SBM_LAUNCHED(2);
  SBM_CUDA_TRY(cudaGetLastError());
  return SBM_OK;
}

float* net_pc_zbuf(sbm_ctx* ctx) {
  netd::NetPc* pc = static_cast<netd::NetPc*>(ctx->net);
  return pc->zf + kOff32;
}

float* net_pc_rc(sbm_ctx* ctx) { return static_cast<netd::NetPc*>(ctx->net)->rc; }
float* net_pc_rq(sbm_ctx* ctx) { return static_cast<netd::NetPc*>(ctx->net)->rq; }
int64_t net_pc_ncell(sbm_ctx* ctx) { return static_cast<netd::NetPc*>(ctx->net)->cv.v(); }
// y and x strides of the coarse arrays (the padded grid's extents)
void net_pc_rc_strides(sbm_ctx* ctx, int* sy, int* sx) {
  const netd::NetPc* pc = static_cast<const netd::NetPc*>(ctx->net);
  *sy = pc->c.ny;
  *sx = pc->c.nx;
}
float* net_pc_scal(sbm_ctx* ctx) { return static_cast<netd::NetPc*>(ctx->net)->scal; }

int net_pc_nodes() { return 3 + 9; }

// The multiplicative step: tiles of 64 x 8 x 4 fine cells (the last y tile
// may be partial), one wave of resident blocks (3 per SM at 80 registers)
// walking them grid-stride.
static void launch_mult(netd::NetPc* pc, const Geo& g, float* r32, double* partials, CgState* st,
                        cudaStream_t s) {
  const int64_t tiles = (int64_t)((g.ny + netd::kMTY - 1) / netd::kMTY) * (g.nx / netd::kMTX) *
                        (g.nz / netd::kMTZ);
  const unsigned bt = (unsigned)(tiles < 152 * 3 ? tiles : 152 * 3);
  launch_pdl(netd::k_pc_mult_tiled, dim3(bt), dim3(256), netd::kMultSmem, s, pc->mmaps, g, pc->c,
             pc->cv, (const float*)pc->w->out, (const float*)pc->scal, r32, pc->dg32,
             pc->scale, pc->bcx0, pc->bcx1, netd::kPcOmega, pc->zf + kOff32,
             (const int*)pc->net->err, partials, st);
}

void net_pc_launch(sbm_ctx* ctx, float* r32, const float* iv32, const float* q32,
                   double* partials, CgState* st, cudaStream_t s) {
  netd::NetPc* pc = static_cast<netd::NetPc*>(ctx->net);
  const Geo& g = ctx->g32;
  const netd::Dims& c = pc->c;
  // the restriction (a grid reduction): two blocks per SM at most, so the
  // last block sums few partials
  const int rgrid = std::min(netd::grid_for(pc->cv.v()), 2 * 152);
  launch_pdl(netd::k_pc_restrict, dim3(rgrid), dim3(256), 0, s, g, c, pc->cv, (const float*)r32,
             pc->rc, (const float*)pc->rq, partials, (float*)pc->scal, st);
  launch_pdl(netd::k_pc_pack, dim3(netd::grid_for(c.v())), dim3(256), 0, s, c.v(), pc->rc,
             (const float*)pc->rq, (const float*)pc->scal, pc->w->in0, (const CgState*)st);
  SBM_LAUNCHED(2);
  netd::forward(pc->net, *pc->w, false, &st->done, &st->pc_off, s);
  const int64_t items = (int64_t)(g.ny / 4) * g.nx * (g.nz / 4);
  int64_t b = (items + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  if (b < 1) b = 1;
  // the multiplicative form with an over-relaxed Jacobi step (kPcOmega;
  // flexible-CG iterations of the 256^3 headline solve fall from 123-128
  // with the additive form to 61)
  if (ctx->pc_additive) {
    launch_pdl(netd::k_pc_prolong, dim3((unsigned)b), dim3(256), 0, s, g, c, pc->cv,
               (const float*)pc->w->out, (const float*)pc->scal, r32, iv32, q32, pc->zf + kOff32,
               (const int*)pc->net->err, partials, st);
  } else {
    launch_mult(pc, g, r32, partials, st, s);
  }
  SBM_LAUNCHED(1);
}

void net_pc_launch_part(sbm_ctx* ctx, int part, float* r32, const float* q32,
                        double* partials, CgState* st, cudaStream_t s) {
  netd::NetPc* pc = static_cast<netd::NetPc*>(ctx->net);
  if (part == 0) {
    netd::forward(pc->net, *pc->w, false, &st->done, &st->pc_off, s);
    return;
  }
  launch_mult(pc, ctx->g32, r32, partials, st, s);
  SBM_LAUNCHED(1);
}

void net_pc_release(sbm_ctx* ctx) {
  netd::NetPc* pc = static_cast<netd::NetPc*>(ctx->net);
  if (!pc) return;
  pc->release();
  delete pc;
  ctx->net = nullptr;
}

}  // namespace sbm

// ------------------------------------------------------------- C-ABI

extern "C" {

int64_t sbm_net_param_count(void) { return kL.total; }

int sbm_net_create(uint64_t seed, sbm_net** out) {
  if (!out) return SBM_ERR_ARG;
  *out = nullptr;
  int rc = conv3_init();
  if (rc) return rc;
  sbm_net* n = new sbm_net();
  const int64_t P = kL.total;
  if (cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) ||
      cudaMalloc(&n->w32, sizeof(float) * P) || cudaMalloc(&n->m, sizeof(float) * P) ||
      cudaMalloc(&n->v, sizeof(float) * P) || cudaMalloc(&n->grad, sizeof(float) * P) ||
      cudaMalloc(&n->wimg, sizeof(bf16) * P) || cudaMalloc(&n->wtimg, sizeof(bf16) * P) ||
      cudaMalloc(&n->wimg16, sizeof(bf16) * P) || cudaMalloc(&n->wtimg16, sizeof(bf16) * P) ||
      cudaMalloc(&n->err, sizeof(int)) || cudaMalloc(&n->loss, sizeof(double))) {
    sbm_net_destroy(n);
    return SBM_ERR_NOMEM;
  }
  // He-normal initialisation of the convolutions, zero biases, small output layer
  std::vector<float> h((size_t)P, 0.f);
  uint64_t st = seed * 0x2545F4914F6CDD1Dull + 1;
  for (int l = 0; l < NLAYER; ++l) {
    const int taps = (l == OUT) ? 1 : 27;
    const int64_t nw = (int64_t)kCo[l] * taps * kCi[l];
    const double sd = (l == OUT) ? 0.1 : sqrt(2.0 / (taps * kCi[l]));
    for (int64_t i = 0; i < nw; ++i) {
      const double u1 = unit(&st), u2 = unit(&st);
      h[(size_t)(kL.off[l] + i)] = (float)(sd * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
    }
  }
  rc = sbm_net_set_params(n, h.data(), P);
  if (rc) {
    sbm_net_destroy(n);
    return rc;
  }
  *out = n;
  return SBM_OK;
}

int sbm_net_destroy(sbm_net* n) {
  if (!n) return SBM_ERR_ARG;
  if (n->stream) cudaStreamSynchronize(n->stream);
  for (auto& kv : n->works) delete kv.second;
  void* p[] = {n->w32, n->m, n->v, n->grad, n->wimg, n->wtimg, n->wimg16, n->wtimg16,
               n->err, n->loss, n->din, n->dt};
  for (void* q : p) cudaFree(q);
  if (n->stream) cudaStreamDestroy(n->stream);
  delete n;
  return SBM_OK;
}

int sbm_net_get_params(const sbm_net* n, float* host, int64_t count) {
  if (!n || !host || count != kL.total) return SBM_ERR_ARG;
  SBM_CUDA_TRY(cudaMemcpyAsync(host, n->w32, sizeof(float) * count, cudaMemcpyDeviceToHost,
                               n->stream));
  SBM_CUDA_TRY(cudaStreamSynchronize(n->stream));
  return SBM_OK;
}

int sbm_net_set_params(sbm_net* n, const float* host, int64_t count) {
  if (!n || !host || count != kL.total) return SBM_ERR_ARG;
  cudaStream_t s = n->stream;
  SBM_CUDA_TRY(cudaMemcpyAsync(n->w32, host, sizeof(float) * count, cudaMemcpyHostToDevice, s));
  SBM_CUDA_TRY(cudaMemsetAsync(n->m, 0, sizeof(float) * count, s));
  SBM_CUDA_TRY(cudaMemsetAsync(n->v, 0, sizeof(float) * count, s));
  SBM_CUDA_TRY(cudaMemsetAsync(n->err, 0, sizeof(int), s));
  SBM_CUDA_TRY(cudaMemsetAsync(n->loss, 0, sizeof(double), s));
  n->step = 0;
  int rc = cast_weights(n, s);
  if (rc) return rc;
  SBM_CUDA_TRY(cudaStreamSynchronize(s));
  return SBM_OK;
}

int sbm_net_forward(sbm_net* n, int ny, int nx, int nz, int nb, const float* in, float* out) {
  if (!n || !in || !out || nb < 1 || !dims_ok(ny, nx, nz)) return SBM_ERR_ARG;
  Work* w = work_for(n, ny, nx, nz, nb, false);
  if (!w) return SBM_ERR_NOMEM;
  const int64_t V = w->d[0].v();
  int rc = upload_features(w->in0, in, V, 1, n->stream);
  if (rc) return rc;
  if ((rc = forward(n, *w, false, nullptr, nullptr, n->stream))) return rc;
  SBM_CUDA_TRY(cudaMemcpyAsync(out, w->out, sizeof(float) * V, cudaMemcpyDeviceToHost, n->stream));
  return check_err(n);
}

int sbm_net_loss_grad(sbm_net* n, int ny, int nx, int nz, int nb, const float* in,
                      const float* target, double* loss, float* grad) {
  if (!n || !in || !target || nb < 1 || !dims_ok(ny, nx, nz)) return SBM_ERR_ARG;
  Work* w = work_for(n, ny, nx, nz, nb, true);
  if (!w) return SBM_ERR_NOMEM;
  cudaStream_t s = n->stream;
  const int64_t V = w->d[0].v();
  int rc = upload_features(w->in0, in, V, 1, s);
  if (rc) return rc;
  SBM_CUDA_TRY(cudaMemcpyAsync(w->tgt, target, sizeof(float) * V, cudaMemcpyHostToDevice, s));
  SBM_CUDA_TRY(cudaMemsetAsync(n->loss, 0, sizeof(double), s));
  if ((rc = forward(n, *w, true, nullptr, nullptr, s))) return rc;
  if ((rc = backward(n, *w, s))) return rc;
  double h = 0.0;
  SBM_CUDA_TRY(cudaMemcpyAsync(&h, n->loss, sizeof(double), cudaMemcpyDeviceToHost, s));
  if (grad)
    SBM_CUDA_TRY(cudaMemcpyAsync(grad, n->grad, sizeof(float) * kL.total, cudaMemcpyDeviceToHost, s));
  if ((rc = check_err(n))) return rc;
  if (loss) *loss = h / (double)V;
  return SBM_OK;
}

int sbm_net_set_data(sbm_net* n, int ny, int nx, int nz, int nsamples, const float* in,
                     const float* target) {
  if (!n || !in || !target || nsamples < 1 || !dims_ok(ny, nx, nz)) return SBM_ERR_ARG;
  cudaStream_t s = n->stream;
  cudaStreamSynchronize(s);
  cudaFree(n->din);
  cudaFree(n->dt);
  n->din = nullptr;
  n->dt = nullptr;
  n->dns = 0;
  const int64_t Vs = (int64_t)ny * nx * nz;
  if (cudaMalloc(&n->din, sizeof(bf16) * Vs * kFeat * nsamples) ||
      cudaMalloc(&n->dt, sizeof(float) * Vs * nsamples))
    return SBM_ERR_NOMEM;
  int rc = upload_features(n->din, in, Vs, nsamples, s);
  if (rc) return rc;
  SBM_CUDA_TRY(cudaMemcpyAsync(n->dt, target, sizeof(float) * Vs * nsamples,
                               cudaMemcpyHostToDevice, s));
  SBM_CUDA_TRY(cudaStreamSynchronize(s));
  n->dny = ny;
  n->dnx = nx;
  n->dnz = nz;
  n->dns = nsamples;
  return SBM_OK;
}

int sbm_net_train_steps(sbm_net* n, int steps, int batch, float lr, uint64_t seed,
                        float* loss_hist) {
  if (!n || steps < 1 || batch < 1 || !(lr > 0.f)) return SBM_ERR_ARG;
  if (!n->dns) return SBM_ERR_STATE;
  const int ny = n->dny, nx = n->dnx, nz = n->dnz, nsamples = n->dns;
  Work* w = work_for(n, ny, nx, nz, batch, true);
  if (!w) return SBM_ERR_NOMEM;
  cudaStream_t s = n->stream;
  const int64_t Vs = (int64_t)ny * nx * nz;
  float* hist = nullptr;
  if (cudaMalloc(&hist, sizeof(float) * steps)) return SBM_ERR_NOMEM;
  auto fail = [&](int code) {
    cudaStreamSynchronize(s);
    cudaFree(hist);
    return code;
  };
  if (cudaMemsetAsync(n->loss, 0, sizeof(double), s)) return fail(SBM_ERR_CUDA);
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 7;
  const int64_t V = Vs * batch;
  const float inv_v = 1.0f / (float)V;
  int rc;
  for (int it = 0; it < steps; ++it) {
    for (int b = 0; b < batch; ++b) {
      const int64_t q = (int64_t)(splitmix(&st) % (uint64_t)nsamples);
      if (cudaMemcpyAsync(w->in0 + act_index(b * Vs, 0, V), n->din + q * Vs * kFeat,
                          sizeof(bf16) * Vs * 8, cudaMemcpyDeviceToDevice, s) ||
          cudaMemcpyAsync(w->in0 + act_index(b * Vs, 8, V), n->din + q * Vs * kFeat + Vs * 8,
                          sizeof(bf16) * Vs * 8, cudaMemcpyDeviceToDevice, s) ||
          cudaMemcpyAsync(w->tgt + b * Vs, n->dt + q * Vs, sizeof(float) * Vs,
                          cudaMemcpyDeviceToDevice, s))
        return fail(SBM_ERR_CUDA);
    }
    if ((rc = forward(n, *w, true, nullptr, nullptr, s))) return fail(rc);
    if ((rc = backward(n, *w, s))) return fail(rc);
    if ((rc = adam(n, lr, s))) return fail(rc);
    k_loss_rec<<<1, 1, 0, s>>>(n->loss, inv_v, hist + it);
    SBM_LAUNCHED(1);
  }
  if (loss_hist &&
      cudaMemcpyAsync(loss_hist, hist, sizeof(float) * steps, cudaMemcpyDeviceToHost, s))
    return fail(SBM_ERR_CUDA);
  if ((rc = check_err(n))) return fail(rc);
  return fail(SBM_OK);
}

int sbm_net_train(sbm_net* n, int ny, int nx, int nz, int nsamples, const float* in,
                  const float* target, int steps, int batch, float lr, uint64_t seed,
                  float* loss_hist) {
  if (!n || steps < 1 || batch < 1 || !(lr > 0.f)) return SBM_ERR_ARG;
  int rc = sbm_net_set_data(n, ny, nx, nz, nsamples, in, target);
  if (rc) return rc;
  return sbm_net_train_steps(n, steps, batch, lr, seed, loss_hist);
}

// Weights file: 8-byte magic "SBMNET01" (a network trained on the potential
// form only) or "SBMNET02" (also trained on the CnE form, reading input
// channel 5), int64 parameter count, float64 output scale k_out, then the
// FP32 parameters (little-endian).
int sbm_net_load(const char* path, sbm_net** out, double* out_scale) {
  if (!path || !out || !out_scale) return SBM_ERR_ARG;
  *out = nullptr;
  FILE* f = fopen(path, "rb");
  if (!f) {
    set_error_msg("cannot open the weights file");
    return SBM_ERR_ARG;
  }
  char magic[8];
  int64_t count = 0;
  double scale = 0.0;
  std::vector<float> h;
  bool ok = fread(magic, 1, 8, f) == 8 &&
            (memcmp(magic, "SBMNET01", 8) == 0 || memcmp(magic, "SBMNET02", 8) == 0) &&
            fread(&count, sizeof(count), 1, f) == 1 && count == kL.total &&
            fread(&scale, sizeof(scale), 1, f) == 1 && scale > 0.0;
  if (ok) {
    h.resize((size_t)count);
    ok = fread(h.data(), sizeof(float), (size_t)count, f) == (size_t)count;
  }
  fclose(f);
  if (!ok) {
    set_error_msg("not a weights file of this network");
    return SBM_ERR_ARG;
  }
  int rc = sbm_net_create(0, out);
  if (rc) return rc;
  if ((rc = sbm_net_set_params(*out, h.data(), count))) {
    sbm_net_destroy(*out);
    *out = nullptr;
    return rc;
  }
  (*out)->mass = memcmp(magic, "SBMNET02", 8) == 0 ? 1 : 0;
  *out_scale = scale;
  return SBM_OK;
}

int sbm_net_set_mass_channel(sbm_net* n, int on) {
  if (!n || (on != 0 && on != 1)) return SBM_ERR_ARG;
  n->mass = on;
  return SBM_OK;
}

int sbm_net_get_mass_channel(const sbm_net* n) { return n ? n->mass : SBM_ERR_ARG; }

int sbm_ctx_set_net(sbm_ctx* ctx, sbm_net* n, double out_scale) {
  if (!ctx || !(out_scale > 0.0)) return SBM_ERR_ARG;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  release_graphs(ctx);
  if (!n) {
    net_pc_release(ctx);
    return SBM_OK;
  }
  NetPc* pc = static_cast<NetPc*>(ctx->net);
  if (!pc) {
    pc = new NetPc();
    ctx->net = pc;
  }
  pc->net = n;
  pc->kout = out_scale;
  return SBM_OK;
}

}  // extern "C"
