// sbm_conv.cuh -- argument blocks and launchers of the BF16 tensor-core
// convolution kernels (sbm_conv.cu), shared with the learned
// preconditioner (sbm_net.cu).
//
// Activations are stored in channel-group planes: element (voxel v,
// channel c) of a buffer of V voxels sits at act_index(v, c, V) =
// ((c / 8) * V + v) * 8 + c % 8, voxel v = i + ny*(j + nx*k).  A run of 8
// channels of consecutive y voxels is contiguous, so one tensor-map row of
// the halo tile is 10 voxels x 16 bytes, and a channel slice starting at a
// multiple of 8 is a set of whole planes (concatenation buffers).  A batch
// of samples is stacked along z: nz = samples * nzs, and no tap reaches
// across a sample boundary (zero padding at every sample's faces).
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "sbm_internal.cuh"

namespace sbm {

__host__ __device__ __forceinline__ int64_t act_index(int64_t v, int c, int64_t V) {
  return (((int64_t)(c >> 3) * V + v) << 3) + (c & 7);
}

struct ConvArgs {
  int ny, nx, nz;          // grid (nz = stacked depth)
  int nzs;                 // depth of one sample
  int cin, cout;           // channels (multiples of 16)
  int ldx, offx;           // channels of the input buffer and the slice's first channel
  int offy;                // first output channel in the output buffer
  const __nv_bfloat16* x;
  const __nv_bfloat16* w;  // [cout][27][cin] (CUDA-core kernel)
  const __nv_bfloat16* wimg;    // weight images of the tensor-core kernel (conv3_wimage)
  const __nv_bfloat16* wimg16;  //   for 64- and 16-channel output tiles (wimg16 may be null)
  const float* bias;       // [cout] or null
  __nv_bfloat16* y16;      // BF16 output or null
  float* y32;              // FP32 output or null
  int relu;
  int flip;                // 1: tap t reads neighbour -offset (CUDA-core kernel; the
                           //    tensor-core kernel takes it from a reversed weight image)
  int* err;                // set to 1 if a wait expired
  const int* skip;         // launch is a no-op while *skip != 0 (may be null)
  const int* skip2;        //   or while *skip2 != 0 (may be null)
  int wpre;                // 1: no kernel of the launch's dependency chain writes the
                           //    weight images, so the tensor-core kernel copies them
                           //    before waiting on the preceding kernel
  // tensor-core kernel only:
  int planes;              // z planes per CTA: 1, or 2 (nzs even)
  int vny, vnx, vnz;       // valid extents of a zero-padded grid (vnz per sample): outputs
                           //   of voxels beyond them are stored as 0; vny = 0: all valid
  int uvny, uvnx, uvnz;    // the same of the 2x finer grid `up` writes (children beyond
                           //   them receive 0)
  __nv_bfloat16* pool;     // 2x2x2-averaged BF16 output [V/8][cout] (planes 2) or null
  __nv_bfloat16* up;       // BF16 output copied to the 8 children in the 2x finer grid
  int offu;                //   (first channel there) or null
  const float* w1x1;       // fused 1x1 output layer (cout 16): out1x1[v] = b1x1 +
  const float* b1x1;       //   sum_c w1x1[c] bf16(y[v][c]), or null
  float* out1x1;
  // set by conv3_launch
  int tw;                  // output channels per CTA tile (64 or 16)
  int nst;                 // pipeline stages
};

struct WgradArgs {
  int ny, nx, nz, nzs;
  int cin, cout;
  int offx;                      // first channel of the layer input in its buffer
  const __nv_bfloat16* x;        // forward input of the layer
  const __nv_bfloat16* dy;       // gradient of the pre-activation [V][cout]
  float* dw;                     // [cout][27][cin], accumulated (atomic adds)
  int kv;                        // voxels per CTA (multiple of 16)
  int* err;
};

// Tensor map of a convolution input: 5-D (8 channels x y merged, x, z
// within the sample, sample, channel group); box = one 8-channel half of
// the halo tile.
struct ConvMap {
  CUtensorMap x;
};

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();

bool conv_shape_ok(int cin, int cout);
int conv3_init();
int conv3_map(const ConvArgs* a, ConvMap* m);
// Weight image (output-channel tiles of width tw = 64 or 16) of the
// tensor-core kernel from w [cout][27][cin] (transpose = 0), or of the
// transposed convolution (data gradient) from the layer's weights
// [cin][27][cout] (transpose = 1, cout/cin are those of the transposed
// convolution); reverse = 1 stores tap t at 26 - t (the flipped taps of
// the data gradient; the tensor-core kernel itself never flips).  img has
// cout*27*cin elements.
void conv3_wimage(const __nv_bfloat16* w, int cout, int cin, int transpose, int reverse, int tw,
                  __nv_bfloat16* img, cudaStream_t s);
// Index in the weight image of element (co, tap, ci) of a convolution with
// cout x cin channels.  Per output tile, per 16-channel input chunk, per
// in-plane offset (dy, dx): one B operand of 3 nt rows in the canonical
// K-major layout, rows [W(dz=+1) | W(dz=0) | W(dz=-1)], so that the two
// middle halo planes of a two-plane tile each feed both accumulators with
// one MMA of 2 nt columns.
__host__ __device__ inline int64_t wimage_index(int co, int t, int ci, int cout, int cin, int tw) {
  const int j = co / tw, n = co % tw;
  const int nt = min(tw, cout - tw * j);
  const int c = ci >> 4, kh = (ci >> 3) & 1, e = ci & 7;
  const int q = t % 9, dz = t / 9 - 1;  // (dy, dx) pair and z offset of tap t
  const int r = (1 - dz) * nt + n;
  const int64_t byte = (int64_t)tw * j * 27 * cin * 2 + (int64_t)c * 27 * nt * 32 +
                       (int64_t)q * 3 * nt * 32 + (r >> 3) * 256 + kh * 128 + (r & 7) * 16 +
                       e * 2;
  return byte / 2;
}
// use_tc = 1: tcgen05 kernel (needs a.wimg and a map, encoded here when m
// is null); 0: CUDA-core reference kernel (a.w).
int conv3_launch(const ConvArgs* a, const ConvMap* m, int use_tc, cudaStream_t s);
int wgrad_launch(const WgradArgs* a, cudaStream_t s);

}  // namespace sbm
