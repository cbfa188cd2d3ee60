// solve_f32_b.cu -- instantiations of the fused FP32 solve (NW in {8 16 32}).
#include "propagate.cuh"
#include "propagate_dispatch.cuh"
namespace scft {
cudaError_t solve_launch_f32_b(int C, int NW, const BatchDev &b, const ClassDev &cls, const MixDev &m, int grid,
                                   cudaStream_t st, int *ctas_per_sm) {
  switch (C * 64 + NW) {
    case 1 * 64 + 8: return dispatch_solve<float, 1, 8, true>(b, cls, m, grid, st, ctas_per_sm);
    case 1 * 64 + 16: return dispatch_solve<float, 1, 16, true>(b, cls, m, grid, st, ctas_per_sm);
    case 1 * 64 + 32: return dispatch_solve<float, 1, 32, true>(b, cls, m, grid, st, ctas_per_sm);
    case 2 * 64 + 8: return dispatch_solve<float, 2, 8, true>(b, cls, m, grid, st, ctas_per_sm);
    case 2 * 64 + 16: return dispatch_solve<float, 2, 16, true>(b, cls, m, grid, st, ctas_per_sm);
    case 2 * 64 + 32: return dispatch_solve<float, 2, 32, true>(b, cls, m, grid, st, ctas_per_sm);
    case 4 * 64 + 8: return dispatch_solve<float, 4, 8, true>(b, cls, m, grid, st, ctas_per_sm);
    case 4 * 64 + 16: return dispatch_solve<float, 4, 16, true>(b, cls, m, grid, st, ctas_per_sm);
    case 4 * 64 + 32: return dispatch_solve<float, 4, 32, true>(b, cls, m, grid, st, ctas_per_sm);
    case 8 * 64 + 8: return dispatch_solve<float, 8, 8, true>(b, cls, m, grid, st, ctas_per_sm);
    case 8 * 64 + 16: return dispatch_solve<float, 8, 16, true>(b, cls, m, grid, st, ctas_per_sm);
    case 8 * 64 + 32: return dispatch_solve<float, 8, 32, true>(b, cls, m, grid, st, ctas_per_sm);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace scft
