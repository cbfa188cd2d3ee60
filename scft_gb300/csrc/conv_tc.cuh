// conv_tc.cuh -- the warm-start network's 64 -> 64 convolutions on the 5th
// generation tensor cores (tcgen05.mma, accumulators in tensor memory).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace scft {

// Bytes of the BF16 weight image of one 64 -> 64 layer (5 taps x 64 x 64).
constexpr int CONV_TC_IMAGE_BYTES = 5 * 64 * 64 * 2;

// Packs the FP32 weights W[co][ci][k] of a 64 -> 64 layer into the BF16 operand
// image the tensor-core kernel copies into shared memory (one launch).
cudaError_t conv_tc_pack(const float *W, __nv_bfloat16 *img, cudaStream_t st);

// y[b][co][p] = act(bias[co] + sum_ci sum_k W[co][ci][k] x[b][ci][p + (k-2) dil]) for
// B instances of 256 points, x and y BF16 [B][64][256], dil in {2, 4, 8}, act = tanh
// or identity.  Accumulation in FP32.  *err (device) receives a nonzero code if
// a wait of the kernel ran out (the outputs of that instance are then not
// written).
cudaError_t conv_tc_forward(const __nv_bfloat16 *x, const __nv_bfloat16 *img, const float *bias, int dil,
                            int act, __nv_bfloat16 *y, int B, int *err, cudaStream_t st);

}  // namespace scft
