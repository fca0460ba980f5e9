// sbm_conv.cuh -- argument blocks and launchers of the BF16 tensor-core
// convolution kernels (sbm_conv.cu), shared with the learned
// preconditioner (sbm_net.cu).
//
// Grids are channels-last, voxel v = i + ny*(j + nx*k).  A batch of
// samples is stacked along z: nz = samples * nzs, and no tap reaches across
// a sample boundary (zero padding at every sample's faces).
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "sbm_internal.cuh"

namespace sbm {

struct ConvArgs {
  int ny, nx, nz;          // grid (nz = stacked depth)
  int nzs;                 // depth of one sample
  int cin, cout;           // channels (multiples of 16)
  int ldx, offx;           // input channel stride and offset (channel slices of concat buffers)
  int ldy, offy;           // output channel stride and offset
  const __nv_bfloat16* x;
  const __nv_bfloat16* w;  // [cout][27][cin] (CUDA-core kernel)
  const __nv_bfloat16* wimg;  // weight image of the tensor-core kernel (conv3_wimage)
  const float* bias;       // [cout] or null
  __nv_bfloat16* y16;      // BF16 output or null
  float* y32;              // FP32 output or null
  int relu;
  int flip;                // 1: tap t reads neighbour -offset (transposed convolution)
  int* err;                // set to 1 if a wait expired
  const int* skip;         // launch is a no-op while *skip != 0 (may be null)
};

struct WgradArgs {
  int ny, nx, nz, nzs;
  int cin, cout;
  int ldx, offx;                 // input activation channel stride / offset
  const __nv_bfloat16* x;        // forward input of the layer
  const __nv_bfloat16* dy;       // gradient of the pre-activation [V][cout]
  float* dw;                     // [cout][27][cin], accumulated (atomic adds)
  int kv;                        // voxels per CTA (multiple of 16)
  int* err;
};

// Tensor map of a convolution input: 5-D (channel, y, x, z within the
// sample, sample) over x with channel stride ldx; box = one 8-channel half
// of the halo tile.
struct ConvMap {
  CUtensorMap x;
};

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();

bool conv_shape_ok(int cin, int cout);
int conv3_init();
int conv3_map(const ConvArgs* a, ConvMap* m);
// Weight image of the tensor-core kernel from w [cout][27][cin] (transpose
// = 0), or of the transposed convolution (data gradient) from the layer's
// weights [cin][27][cout] (transpose = 1, cout/cin are those of the
// transposed convolution).  img has cout*27*cin elements.
void conv3_wimage(const __nv_bfloat16* w, int cout, int cin, int transpose, __nv_bfloat16* img,
                  cudaStream_t s);
// Index in the weight image of element (co, tap, ci) of a convolution with
// cout x cin channels.
__host__ __device__ inline int64_t wimage_index(int co, int t, int ci, int cout, int cin) {
  const int j = co >> 6, n = co & 63;
  const int nt = min(64, cout - 64 * j);
  const int c = ci >> 4, kh = (ci >> 3) & 1, e = ci & 7;
  const int64_t byte = (int64_t)64 * j * 27 * cin * 2 + (int64_t)c * 27 * nt * 32 +
                       (int64_t)t * nt * 32 + (n >> 3) * 256 + kh * 128 + (n & 7) * 16 + e * 2;
  return byte / 2;
}
// use_tc = 1: tcgen05 kernel (needs a.wimg and a map, encoded here when m
// is null); 0: CUDA-core reference kernel (a.w).
int conv3_launch(const ConvArgs* a, const ConvMap* m, int use_tc, cudaStream_t s);
int wgrad_launch(const WgradArgs* a, cudaStream_t s);

}  // namespace sbm
