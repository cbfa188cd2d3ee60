// propagate_launch.cuh -- host-side dispatch over the propagator's shape classes.
#pragma once
#include "common.cuh"

namespace scft {

enum Precision : int { PREC_F32 = 0, PREC_F64 = 1 };

// Threads per CTA of the (C, NW) class (groups of 32*NW threads, 256 threads per CTA
// for small groups).
int propagate_cta_threads(int C, int NW);
// Groups (workers) per CTA.
int propagate_groups_per_cta(int C, int NW);
// Resident CTAs per SM for the class (occupancy API), 0 if the class does not exist.
int propagate_ctas_per_sm(int prec, int C, int NW);
// Launch the persistent propagator of one shape class.
cudaError_t propagate_launch(int prec, int C, int NW, const BatchDev &b, const ClassDev &cls,
                             int grid, cudaStream_t stream);
// Whether a (prec, C, NW) class is compiled.
bool propagate_has_class(int prec, int C, int NW);

}  // namespace scft
