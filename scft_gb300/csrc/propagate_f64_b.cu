// propagate_f64_b.cu -- instantiations of the f64 propagator (NW in {8 16 32}).
#include "propagate.cuh"
#include "propagate_dispatch.cuh"
namespace scft {
cudaError_t propagate_launch_f64_b(int C, int NW, const BatchDev &b, const ClassDev &cls, int grid, cudaStream_t st, int *ctas_per_sm, bool *exists) {
  switch (C * 64 + NW) {
    case 1 * 64 + 8: return dispatch_class<double, 1, 8, false>(b, cls, grid, st, ctas_per_sm, exists);
    case 1 * 64 + 16: return dispatch_class<double, 1, 16, false>(b, cls, grid, st, ctas_per_sm, exists);
    case 1 * 64 + 32: return dispatch_class<double, 1, 32, false>(b, cls, grid, st, ctas_per_sm, exists);
    case 2 * 64 + 8: return dispatch_class<double, 2, 8, false>(b, cls, grid, st, ctas_per_sm, exists);
    case 2 * 64 + 16: return dispatch_class<double, 2, 16, false>(b, cls, grid, st, ctas_per_sm, exists);
    case 2 * 64 + 32: return dispatch_class<double, 2, 32, false>(b, cls, grid, st, ctas_per_sm, exists);
    case 4 * 64 + 8: return dispatch_class<double, 4, 8, false>(b, cls, grid, st, ctas_per_sm, exists);
    case 4 * 64 + 16: return dispatch_class<double, 4, 16, false>(b, cls, grid, st, ctas_per_sm, exists);
    case 4 * 64 + 32: return dispatch_class<double, 4, 32, false>(b, cls, grid, st, ctas_per_sm, exists);
    case 8 * 64 + 8: return dispatch_class<double, 8, 8, false>(b, cls, grid, st, ctas_per_sm, exists);
    case 8 * 64 + 16: return dispatch_class<double, 8, 16, false>(b, cls, grid, st, ctas_per_sm, exists);
    case 8 * 64 + 32: return dispatch_class<double, 8, 32, false>(b, cls, grid, st, ctas_per_sm, exists);
    default: if (exists) *exists = false; return cudaErrorInvalidValue;
  }
}
}  // namespace scft
