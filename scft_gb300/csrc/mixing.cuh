// mixing.cuh -- field-update kernels (FP64): batched Anderson mixing and the
// single-instance reference-form solvers used by the drop-in entry points.
#pragma once
#include "common.cuh"

namespace scft {

// Batched Anderson state.  Interior unknowns of instance i start at int_off[i];
// history slot s of instance i starts at depth*int_off[i] + s*N_i.
struct MixDev {
  int count;
  const int *n;
  const long long *node_off;
  const long long *int_off;
  const double *x, *f0, *phi;
  double *w;
  int *active;     // 1: evaluate in FP32, 2: evaluate in FP64, 0: finished
  int *status;
  int *iters;
  double *err;     // ||phi - f0||_inf of the last evaluation
  double *best;    // best error since the last restart
  double *lk;      // per instance: 1 - mixing parameter (ADM_chen_C.c:42, 122)
  double *graw, *gcur, *gprev, *wprev;  // interior vectors: residual, mixed residual, previous residual / field
  double *hdx, *hdg;                    // history of field / residual differences
  double *gram;                         // depth*depth per instance
  int *hcount, *hhead;
  int depth;
  int maxit;
  int mode;        // 0: mixing residual phi - f0; 1: ln phi - ln f0
  int verify64;    // FP32-converged instances are re-evaluated once in FP64
  int lk_schedule; // ADM_chen_C.c:125-129: lk *= lmd once err < 0.03 after 100 iterations, reset below 1e-5
  double tol, tol32, lmd, clip, grow, precond, reg;
  const double *ds;   // contour step per instance
  int weighted;       // least squares and clip weighted by f0 / max f0
  double step_cap;    // |step_i| <= step_cap / ds (0: off)
  double field_floor; // w_i >= -field_floor / ds (0: off)
  // FP32 stall hand-off: ref_err / ref_it = error and iteration of the last
  // halving of the error; ref_it < 0 marks a history that starts afresh (the
  // first evaluation after a hand-off pushes no difference pair)
  int finish_stall;   // 0: off
  double finish_tol;
  double *ref_err;
  int *ref_it;
  // time budget: globaltimer (ns) after which a group stops its instance with
  // ST_WATCHDOG at the next iteration boundary; null: no budget
  const unsigned long long *deadline;
  // graded meshes (spacing[i] = largest / smallest element > graded_ratio): the
  // preconditioner's spacings are floored at sqrt(hfloor * ds) and each node's
  // move is clamped to step_cap / ds instead of scaling the whole step
  const double *spacing = nullptr;
  double graded_ratio = 0.0, hfloor = 0.0;
  // Forked paths (BatchDev::base): static data at instance i, the node arrays
  // of path r at node_off[i] + r * rep_nodes, the interior arrays at
  // int_off[i] + r * rep_int (history: depth times that), scalars and the Gram
  // matrix at id v.  forks > 0: an instance (r = 0) copies its state into paths
  // 1..forks when it forks, path r stepping with fork_scale[r - 1] times the
  // mixing parameter of the instance.
  // An instance forks at its first update number >= fork_at taken at an error
  // <= fork_err; fork_it[i] records that update number (0: not forked).
  // win[i] = min over converged paths of their key, iterations * 16 + r, or 0
  // for the instance's own path converging within fork_grace updates of its
  // fork; a path stops once its earliest possible key exceeds win[i].
  int base = 0;
  long long rep_nodes = 0, rep_int = 0;
  int forks = 0, fork_at = 0, fork_grace = 0;
  double fork_err = 0.0;
  int fork_first = 0;  // groups take published path jobs before new instances
  int *fork_it = nullptr;
  double fork_scale[4] = {1.0, 1.0, 1.0, 1.0};
  int *win = nullptr;
};

cudaError_t mix_launch(const MixDev &m, cudaStream_t st);

// Single-instance Anderson in the residual form of ADM_chen_C.c:18-147.
struct AdmChenDev {
  int n, nm, depth;
  double *X, *Y;     // depth rows of n (ring by iteration index)
  double tol, lmd;
  int final_;
  // state (device)
  int *k, *krestart;
  double *lk, *err;
  int *flag;         // 0 continue, 1 converged, 2 NaN
};
cudaError_t admchen_step_launch(const AdmChenDev &a, cudaStream_t st);

// Single-instance Anderson in the fixed-point ring form of adm.c:24-313.
struct AdmDev {
  int n;
  double *x, *xnew;  // current iterate and g(x)
  double *xh, *dh;   // 11 slots of n
  double tol;
  int *its, *nc;
  double *err;
  int *flag;         // 0 continue, 1 converged
};
cudaError_t adm_first_launch(const AdmDev &a, cudaStream_t st);
cudaError_t adm_step_launch(const AdmDev &a, cudaStream_t st);

// residual helpers for the drop-in path
cudaError_t residual_launch(int n, const double *phi, const double *f0, int sign, double *out_int,
                            double *w_int_in, int fixed_point, cudaStream_t st);

}  // namespace scft
