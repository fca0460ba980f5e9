// sbm_conv.cuh -- argument blocks and launchers of the BF16 tensor-core
// convolution kernels (sbm_conv.cu), shared with the learned
// preconditioner (sbm_net.cu).
//
// Grids are channels-last, voxel v = i + ny*(j + nx*k).  A batch of
// samples is stacked along z: nz = samples * nzs, and no tap reaches across
// a sample boundary (zero padding at every sample's faces).
#pragma once

#include <cuda_bf16.h>

#include "sbm_internal.cuh"

namespace sbm {

struct ConvArgs {
  int ny, nx, nz;          // grid (nz = stacked depth)
  int nzs;                 // depth of one sample
  int cin, cout;           // channels (multiples of 16)
  int ldx, offx;           // input channel stride and offset (channel slices of concat buffers)
  int ldy, offy;           // output channel stride and offset
  const __nv_bfloat16* x;
  const __nv_bfloat16* w;  // [cout][27][cin]
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

bool conv_shape_ok(int cin, int cout);
int conv3_init();
// use_tc = 1: tcgen05 kernel; 0: CUDA-core reference kernel.
int conv3_launch(const ConvArgs* a, int use_tc, cudaStream_t s);
int wgrad_launch(const WgradArgs* a, cudaStream_t s);

}  // namespace sbm
