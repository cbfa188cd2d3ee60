// solve_f32_a.cu -- instantiations of the fused FP32 solve (NW in {1 2 4}).
#include "propagate.cuh"
#include "propagate_dispatch.cuh"
namespace scft {
cudaError_t solve_launch_f32_a(int C, int NW, const BatchDev &b, const ClassDev &cls, const MixDev &m, int grid,
                                   cudaStream_t st, int *ctas_per_sm) {
  switch (C * 64 + NW) {
    case 1 * 64 + 1: return dispatch_solve<float, 1, 1, true>(b, cls, m, grid, st, ctas_per_sm);
    case 1 * 64 + 2: return dispatch_solve<float, 1, 2, true>(b, cls, m, grid, st, ctas_per_sm);
    case 1 * 64 + 4: return dispatch_solve<float, 1, 4, true>(b, cls, m, grid, st, ctas_per_sm);
    case 2 * 64 + 1: return dispatch_solve<float, 2, 1, true>(b, cls, m, grid, st, ctas_per_sm);
    case 2 * 64 + 2: return dispatch_solve<float, 2, 2, true>(b, cls, m, grid, st, ctas_per_sm);
    case 2 * 64 + 4: return dispatch_solve<float, 2, 4, true>(b, cls, m, grid, st, ctas_per_sm);
    case 4 * 64 + 1: return dispatch_solve<float, 4, 1, true>(b, cls, m, grid, st, ctas_per_sm);
    case 4 * 64 + 2: return dispatch_solve<float, 4, 2, true>(b, cls, m, grid, st, ctas_per_sm);
    case 4 * 64 + 4: return dispatch_solve<float, 4, 4, true>(b, cls, m, grid, st, ctas_per_sm);
    case 8 * 64 + 1: return dispatch_solve<float, 8, 1, true>(b, cls, m, grid, st, ctas_per_sm);
    case 8 * 64 + 2: return dispatch_solve<float, 8, 2, true>(b, cls, m, grid, st, ctas_per_sm);
    case 8 * 64 + 4: return dispatch_solve<float, 8, 4, true>(b, cls, m, grid, st, ctas_per_sm);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace scft
