// common.cuh -- shared device/host definitions of the scft_gb300 runtime.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace scft {

// Per-instance batch arrays (struct of arrays, device pointers).  Node arrays of
// instance i start at node_off[i] in the x / w / phi / f0 pools.
struct BatchDev {
  int count;
  const int *n;            // nodes (elements + 1)
  const int *nsteps;       // contour steps
  const double *ds;        // contour step length
  const long long *node_off;
  const double *x;         // node coordinates
  const double *w;         // field (full nodal vector, wall values unused)
  double *phi;             // density out
  double *Q;               // (1/L) int q(x,1) dx out
  const double *qw;        // 16 quadrature weights per instance: [v] for 2-adic class v of the
                           // sample index (v = min(ctz(k), 14)), [15] for k = 0 and k = nsteps
  const int *active;       // nonzero: evaluate this instance
  int *status;             // per-instance status bits (SCFT_ST_*)
  // Forked solve paths: id v = r * base + i is path r of instance i (r = 0 the
  // instance itself).  Static data (n, nsteps, ds, x, qw, node_off) is read at
  // i, the field, density and Q of path r at node_off[i] + r * rep_nodes, and
  // active / status / Q at v.  base = 0: no forks, v = i.
  int base = 0;
  long long rep_nodes = 0;
};

// CTAs per thread-block cluster of the (precision, C, NW) propagator class: the
// shapes that would spill registers at 32*NW threads in one CTA run as clusters
// of 256-thread CTAs (see Propagator); 1 = one CTA per group.
__host__ __device__ constexpr int cluster_ctas(bool f64, int C, int NW) {
  return NW == 32 ? 4 : (NW == 16 && (C == 8 || (f64 && C == 4))) ? 2 : 1;
}

// Path and instance of id v (see BatchDev::base).
__host__ __device__ __forceinline__ int path_of(int v, int base) { return base ? v / base : 0; }

// One shape class (C nodes per thread, NW warps per instance) of a batch.
struct ClassDev {
  const int *items;        // instance ids, most expensive first
  int count;
  int *head;               // work-queue counter (reset to 0 before each launch)
  void *scratch;           // worker slots for the half-contour store
  long long slot_elems;    // elements per worker slot
  int workers;             // number of slots
  int want;                // evaluate instances whose active flag equals this value
  unsigned long long *work = nullptr;  // if set: += n (nsteps/2 + 1) per instance evaluated
  // Forked paths of the fused solve (MixDev::forks > 0): fork_ctl = {published
  // forks, claimed path jobs, instances that may still fork}; fork_list[k] =
  // 1 + the instance of the k-th published fork (0: not yet written).
  int *fork_ctl = nullptr;
  int *fork_list = nullptr;
};

// Status bits written by the kernels.
enum : int {
  ST_NOT_DOMINANT = 1,     // system matrix lost diagonal dominance (1 + ds w < 0 somewhere)
  ST_NONFINITE = 2,        // non-finite density
  ST_CONVERGED = 4,
  ST_MAXIT = 8,
  ST_RESTARTED = 16,
  ST_WATCHDOG = 32,
  ST_FP64 = 64,
  ST_FORKED = 128,         // the result comes from a forked path of the mixing
};

}  // namespace scft
