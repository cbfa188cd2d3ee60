// propagate_dispatch.cuh -- one shape class: occupancy query or persistent launch.
#pragma once
#include "propagate.cuh"

namespace scft {

// ctas_per_sm != nullptr: report occupancy only.  exists != nullptr: report presence only.
template <typename R, int C, int NW, bool DELTA>
cudaError_t dispatch_class(const BatchDev &b, const ClassDev &cls, int grid, cudaStream_t st,
                           int *ctas_per_sm, bool *exists) {
  using Pp = Propagator<R, C, NW, DELTA>;
  if (exists) { *exists = true; return cudaSuccess; }
  if (ctas_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, propagate_kernel<R, C, NW, DELTA>,
                                                         Pp::CTA, 0);
  }
  if (grid <= 0) return cudaSuccess;
  propagate_kernel<R, C, NW, DELTA><<<grid, Pp::CTA, 0, st>>>(b, cls);
  return cudaGetLastError();
}

// Fused solve of one shape class: occupancy query or persistent launch.
template <typename R, int C, int NW, bool DELTA>
cudaError_t dispatch_solve(const BatchDev &b, const ClassDev &cls, const MixDev &m, int grid, cudaStream_t st,
                           int *ctas_per_sm) {
  using Pp = Propagator<R, C, NW, DELTA>;
  if (ctas_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, solve_kernel<R, C, NW, DELTA>, Pp::CTA, 0);
  }
  if (grid <= 0) return cudaSuccess;
  solve_kernel<R, C, NW, DELTA><<<grid, Pp::CTA, 0, st>>>(b, cls, m);
  return cudaGetLastError();
}

}  // namespace scft
