// propagate_f32_a.cu -- instantiations of the f32 propagator (NW in {1 2 4}).
#include "propagate.cuh"
#include "propagate_dispatch.cuh"
namespace scft {
cudaError_t propagate_launch_f32_a(int C, int NW, const BatchDev &b, const ClassDev &cls, int grid, cudaStream_t st, int *ctas_per_sm, bool *exists) {
  switch (C * 64 + NW) {
    case 1 * 64 + 1: return dispatch_class<float, 1, 1, true>(b, cls, grid, st, ctas_per_sm, exists);
    case 1 * 64 + 2: return dispatch_class<float, 1, 2, true>(b, cls, grid, st, ctas_per_sm, exists);
    case 1 * 64 + 4: return dispatch_class<float, 1, 4, true>(b, cls, grid, st, ctas_per_sm, exists);
    case 2 * 64 + 1: return dispatch_class<float, 2, 1, true>(b, cls, grid, st, ctas_per_sm, exists);
    case 2 * 64 + 2: return dispatch_class<float, 2, 2, true>(b, cls, grid, st, ctas_per_sm, exists);
    case 2 * 64 + 4: return dispatch_class<float, 2, 4, true>(b, cls, grid, st, ctas_per_sm, exists);
    case 4 * 64 + 1: return dispatch_class<float, 4, 1, true>(b, cls, grid, st, ctas_per_sm, exists);
    case 4 * 64 + 2: return dispatch_class<float, 4, 2, true>(b, cls, grid, st, ctas_per_sm, exists);
    case 4 * 64 + 4: return dispatch_class<float, 4, 4, true>(b, cls, grid, st, ctas_per_sm, exists);
    case 8 * 64 + 1: return dispatch_class<float, 8, 1, true>(b, cls, grid, st, ctas_per_sm, exists);
    case 8 * 64 + 2: return dispatch_class<float, 8, 2, true>(b, cls, grid, st, ctas_per_sm, exists);
    case 8 * 64 + 4: return dispatch_class<float, 8, 4, true>(b, cls, grid, st, ctas_per_sm, exists);
    default: if (exists) *exists = false; return cudaErrorInvalidValue;
  }
}
}  // namespace scft
