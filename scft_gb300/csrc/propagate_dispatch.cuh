// propagate_dispatch.cuh -- one shape class: occupancy query or persistent launch.
#pragma once
#include "propagate.cuh"

namespace scft {

// Cluster form of a class: grid counts CTAs (a multiple of CL is launched, at
// most one cluster per worker).
template <typename R, int C, int NW, bool DELTA, int CL>
cudaError_t dispatch_cluster(const BatchDev &b, const ClassDev &cls, int grid, cudaStream_t st, int *ctas_per_sm) {
  using Pp = Propagator<R, C, NW, DELTA, CL>;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3(Pp::CTA);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (ctas_per_sm) {
    int dev = 0, sms = 0, ncl = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cfg.gridDim = dim3(CL);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(&ncl, propagate_cluster_kernel<R, C, NW, DELTA, CL>, &cfg);
    if (e != cudaSuccess) return e;
    *ctas_per_sm = (sms > 0 && ncl > 0) ? (ncl * CL + sms - 1) / sms : 0;
    return cudaSuccess;
  }
  if (grid <= 0) return cudaSuccess;
  const int clusters = grid / CL < cls.workers ? (grid / CL > 0 ? grid / CL : 1) : cls.workers;
  cfg.gridDim = dim3(clusters * CL);
  return cudaLaunchKernelEx(&cfg, propagate_cluster_kernel<R, C, NW, DELTA, CL>, b, cls);
}

// ctas_per_sm != nullptr: report occupancy only.  exists != nullptr: report presence only.
template <typename R, int C, int NW, bool DELTA>
cudaError_t dispatch_class(const BatchDev &b, const ClassDev &cls, int grid, cudaStream_t st,
                           int *ctas_per_sm, bool *exists) {
  using Pp = Propagator<R, C, NW, DELTA>;
  if (exists) { *exists = true; return cudaSuccess; }
  constexpr int CL = cluster_ctas(std::is_same<R, double>::value, C, NW);
  if constexpr (CL > 1) {
    return dispatch_cluster<R, C, NW, DELTA, CL>(b, cls, grid, st, ctas_per_sm);
  } else {  // the one-CTA kernel is instantiated only for the shapes that use it
    if (ctas_per_sm) {
      return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, propagate_kernel<R, C, NW, DELTA>,
                                                           Pp::CTA, 0);
    }
    if (grid <= 0) return cudaSuccess;
    propagate_kernel<R, C, NW, DELTA><<<grid, Pp::CTA, 0, st>>>(b, cls);
    return cudaGetLastError();
  }
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
