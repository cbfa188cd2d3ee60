/*
 * scft.h -- C ABI of libscft (scft_gb300): the SCFT inner loop of giantsda/SCFT
 * (field w -> FEM propagator q -> density phi -> residual -> Anderson/Broyden
 * update of w) on one GB300 GPU.
 *
 * All entry points return int status codes (SCFT_OK = 0, negative = error) and
 * never throw.  Host buffers are owned by the caller; device memory is owned by
 * the library.  The drop-in entry points keep the reference's argument meaning
 * and indexing; each cites the reference function it replaces.
 */
#ifndef SCFT_H
#define SCFT_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define SCFT_OK 0
#define SCFT_EINVAL (-1)    /* invalid argument */
#define SCFT_ECUDA (-2)     /* CUDA runtime error */
#define SCFT_ENOMEM (-3)    /* device or host allocation failed */
#define SCFT_ENOCONFIG (-4) /* scft_set_config was not called */
#define SCFT_ENODEV (-5)    /* no CUDA device */
#define SCFT_ESINGULAR (-6) /* singular Jacobian (Broyden) */
#define SCFT_EIO (-7)       /* a file could not be opened, read or written */

/* ---- per-instance result status bits ---- */
#define SCFT_ST_NOT_DOMINANT 1 /* 1 + ds*w < 0 somewhere: system lost diagonal dominance */
#define SCFT_ST_NONFINITE 2    /* non-finite density: instance stopped */
#define SCFT_ST_CONVERGED 4
#define SCFT_ST_MAXIT 8
#define SCFT_ST_RESTARTED 16   /* the Anderson history was restarted at least once */
#define SCFT_ST_WATCHDOG 32    /* stopped by a bound: the host loop's launch cap, the solve's time
                                  budget (budget_ms), or (shapes on thread-block clusters) a
                                  per-step exchange wait between the cluster's CTAs that ran out,
                                  which voids that pass's density */
#define SCFT_ST_FP64 64        /* the FP32 iteration stalled and the FP64 propagator finished the solve */
#define SCFT_ST_FORKED 128     /* the result comes from a forked path of the mixing (scft_solve_opts.forks) */
#define SCFT_MAX_FORKS 4

enum { SCFT_RULE_ROMBERG = 0, SCFT_RULE_TRAPEZOID = 1 };
enum { SCFT_F32 = 0, SCFT_F64 = 1 };
enum { SCFT_MIX_LINEAR = 0, SCFT_MIX_LOG = 1 };
enum { SCFT_SCHEME_IE = 0, SCFT_SCHEME_IRK2 = 1 };   /* implicit Euler (1D_FEM.c) | Gauss-Legendre IRK2 (drivescft.cc) */
enum { SCFT_W_ROWSCALED = 0, SCFT_W_CONSISTENT = 1 }; /* W_ij = w_i M_ij (1D_FEM.c:104) | int w_h phi_i phi_j (scft.cc:653) */

/* =========================================================================
 * Drop-in single-instance path (the reference's process globals become one
 * configuration set by scft_set_config).
 * ========================================================================= */

typedef struct scft_config {
  int n_nodes;       /* total nodes N+2 (1D_FEM.c:50 adds the two walls) */
  const double *x;   /* n_nodes coordinates, or NULL for uniform on [0, L] (1D_FEM.c:61) */
  double L;          /* film width (1D_FEM.c:61: 3.72374) */
  const double *f0;  /* n_nodes target density (the global f0_given, 1D_FEM.c:14) */
  int nsteps;        /* contour steps (1D_FEM.c:60 runs 2049 steps of ds = 1/2048) */
  double ds;         /* contour step */
  int rule;          /* SCFT_RULE_ROMBERG (romint.c:21) or SCFT_RULE_TRAPEZOID (.m:119-124) */
  int sign;          /* +1: out = phi - f0 (1D_FEM.c:276); -1: out = f0 - phi (drivescft.cc:212) */
  int precision;     /* SCFT_F64 (default) or SCFT_F32 */
  int scheme;        /* SCFT_SCHEME_IE (default, 1D_FEM.c:208-228) or SCFT_SCHEME_IRK2 (the 2-stage
                        Gauss-Legendre method of drivescft.cc:130-165; FP64 only) */
  int wmode;         /* SCFT_W_ROWSCALED (default, 1D_FEM.c:104-105) or SCFT_W_CONSISTENT
                        (scft.cc:653-655; FP64 only) */
  double w_wall[2];  /* field at nodes 0 and n-1, used by the consistent field term (the deal.II
                        field files carry wall values); 0 by default */
} scft_config;

/* Defaults of the drop-in: 2049 steps of ds = 1/2048 with the trapezoid rule
   (the MATLAB prototype's reading of 1D_FEM.c:60-61,208), sign +1, FP64. */
void scft_config_init(scft_config *c);

/* Sets the problem the drop-in residual evaluates (replaces the globals
   f0_given / L / total_time_step of 1D_FEM.c:13-14,60-61).  Copies the arrays. */
int scft_set_config(const scft_config *c);

/* Replaces simple_FEM_1D_transient (1D_FEM.c:47-287): n_interior = N-2 interior
   nodes, w and out are 1-based NR vectors (w[1..n_interior] read,
   out[1..n_interior] written).  Returns SCFT_OK or an error code. */
int scft_fem_residual(int n_interior, double *w, double *out);

/* The same evaluation with the void(int, double*, double*) callback type the
   reference's solvers take: 1-based (broydn.c:44, adm.c with flag=1) ... */
void scft_fem_residual_vf(int n_interior, double *w, double *out);
/* ... and 0-based (ADM_chen_C.c:18 / SCFT_wrapper without BROYDN, drivescft.cc:218-234). */
void scft_fem_residual0_vf(int n_interior, double *w, double *out);
/* Fixed-point form for adm (adm.c:16-21 solves x = f(x)): out = w + (phi - f0), 1-based. */
void scft_fem_fixedpoint_vf(int n_interior, double *w, double *out);

/* Density and partition function of the configured problem for a full nodal
   field w_nodes[0..n_nodes-1] (walls ignored).  phi: n_nodes, Q: optional. */
int scft_density(const double *w_nodes, double *phi, double *Q);

/* Last error message of the calling thread (never NULL). */
const char *scft_last_error(void);
const char *scft_strerror(int code);

/* ---- the reference's solvers, mixing on the GPU ---- */

typedef void (*scft_vecfunc)(int n, double *in, double *out);

/* Replaces adm (adm.c:24-313): Anderson mixing for x = f(x); flag 0: x[0..n-1],
   flag 1: x[1..n].  *check = 0 converged (|f(x)-x|_inf < 1e-10), 1 not.
   f == scft_fem_fixedpoint_vf keeps every evaluation on the device.
   Returns SCFT_OK or an error code. */
int scft_adm(double *x, int n, int *check, scft_vecfunc f, int flag);
/* Iteration cap of scft_adm (the reference's MAXITS, adm.c:5: 1000000). */
void scft_adm_set_maxit(int maxit);

/* Replaces adm_chen (DEALII_SCFT/src/ADM_chen_C.c:18-147): Anderson mixing for
   F(x) = 0, 0-based.  Returns 0 solved, 1 not solved, 2 NaN residual, <0 error.
   The history depth min(nn, n) may be up to 63 (the deal.II driver uses up to
   50, drivescft.cc:296).  f == scft_fem_residual0_vf keeps every evaluation on
   the device. */
int scft_adm_chen(scft_vecfunc f, double *x, double tol, int maxit, int n, double lmd, int nn,
                  int final_);

/* Replaces broydn (broydn.c:44-292; fdjac/lnsrch/qrdcmp/qrupdt/rsolv/rotate of
   DEALII_SCFT/src): x 1-based, *check as broydn sets it.  The tolerance is the
   reference's global err (set with scft_broydn_set_tol, read back the reached
   error with scft_broydn_get_err).  With f == scft_fem_residual_vf the
   finite-difference Jacobian's n evaluations run as one batched launch. */
int scft_broydn(double *x, int n, int *check, scft_vecfunc f);
void scft_broydn_set_tol(double tol);
double scft_broydn_get_err(void);

/* The two solvers with the reference's exact signatures, for code that uses
   their return values unchanged.
   scft_nr_adm has the signature of adm (adm.c:24-27) and, like it, returns the
   last map value g(x) (the vector adm calls xnew) in a heap vector laid out as
   nrutil's vector(flag, n + flag - 1) (nrutil.c:25-33, one element below index
   flag): free it with the reference's free_vector(v, flag, n + flag - 1) or with
   scft_nr_free_vector(v, flag).  On an error it returns NULL with *check = 1
   (scft_last_error tells why).
   scft_nr_broydn has the signature of broydn (broydn.c:44-46, with NR's float
   defined as double, nrutil.h:8): void, *check = 1 on failure or error. */
double *scft_nr_adm(double *x, int n, int *check, scft_vecfunc f, int flag);
void scft_nr_free_vector(double *v, int flag);
void scft_nr_broydn(double x[], int n, int *check, scft_vecfunc f);

/* =========================================================================
 * Batched path: thousands of independent instances per launch.
 * ========================================================================= */

typedef struct scft_instance {
  int n_nodes;        /* elements + 1 */
  const double *x;    /* n_nodes coordinates or NULL (uniform on [0, L]) */
  double L;
  const double *f0;   /* n_nodes target density */
  const double *w0;   /* n_nodes initial field or NULL (zero); wall values are kept but never
                         enter the propagator (1D_FEM.c:65-66) */
  int nsteps;
  double ds;
  int rule;           /* SCFT_RULE_* */
} scft_instance;

typedef struct scft_solve_opts {
  int precision;      /* SCFT_F32 (propagator in FP32, mixing/residual FP64) or SCFT_F64 */
  double tol;         /* ||phi - f0||_inf target */
  double tol32_factor;/* FP32 iterations stop at tol * tol32_factor (default 0.65: the FP32 density's
                         bias, about 1.3e-7, keeps the field within tol under FP64) */
  int verify64;       /* FP32-converged instances are re-evaluated once in FP64 */
  int maxit;
  int depth;          /* Anderson history depth (<= 16) */
  double beta;        /* mixing parameter (initial 1 - lk of ADM_chen_C.c) */
  double clip;        /* max-norm bound on one field update */
  double grow;        /* restart the history when the error grows by this factor */
  double reg;         /* relative Tikhonov term of the least-squares solve */
  int residual_mode;  /* SCFT_MIX_LINEAR (phi - f0) or SCFT_MIX_LOG (ln phi - ln f0) */
  double precond;     /* a in (1 - a d2/dx2) applied to the mixing residual */
  int iters_per_graph;/* iterations captured in one CUDA graph */
  int beta_schedule;  /* 1: the mixing parameter follows ADM_chen_C.c:125-129 (lk = 1 - beta is
                         multiplied by 1 - beta once ||phi - f0|| < 0.03 after 100 iterations and
                         reset below 1e-5); 0: fixed */
  int weighted;       /* 1: the least squares and the clip weight node i by f0_i / max f0, the
                         scale on which ||phi - f0||_inf is judged; 0: unweighted */
  double step_cap;    /* one update moves no node by more than step_cap / ds (0: no cap) */
  double field_floor; /* the field stays >= -field_floor / ds, so 1 + ds w >= 1 - field_floor
                         (0: no floor) */
  int fused;          /* 1: each instance iterates on its own inside one persistent launch per shape
                         class (contour pass and Anderson step by the same thread group, no barrier
                         across the batch; FP32 without verify64); 0: every iteration is a batch-wide
                         step (propagator launches, then the mixing kernel) replayed from CUDA graphs.
                         Batches with instances whose shape runs as a thread-block cluster (the default
                         shapes above 2048 interior unknowns) take the batch-wide form */
  int finish_stall;   /* FP32 solves: an instance whose error is below finish_tol and has not halved
                         for this many iterations continues with the FP64 propagator (fresh Anderson
                         history, tolerance tol, status bit SCFT_ST_FP64); 0: off.  FP32 rounding
                         in the density, amplified by the least squares, lengthens the tail */
  double finish_tol;
  double budget_ms;   /* > 0: device-side time budget of the solve; a thread group that finds it
                         spent at an iteration boundary stops its instance with SCFT_ST_WATCHDOG
                         (the solve returns normally); 0: none */
  int forks;          /* fused FP32 solves: an instance still running after fork_at updates, at its
                         first update taken with ||phi - f0||_inf <= fork_err, is copied into `forks`
                         (<= SCFT_MAX_FORKS) further paths whose mixing parameter is beta times
                         fork_scale[r]; idle thread groups take these paths.  The instance's own path
                         wins if it converges within fork_grace updates of its fork; otherwise the
                         path that converges in the fewest iterations wins (ties: the lowest path,
                         the instance itself first).
                         The outcome does not depend on timing; paths stop once they cannot win.
                         The iteration count is the winner's, SCFT_ST_FORKED marks a forked winner.
                         0: off.  Not used with finish_stall > 0 */
  int fork_at;
  int fork_grace;
  int fork_first;     /* 1: thread groups take published forked paths before new instances; 0: only
                         once the class's instances have all been taken */
  double fork_err;
  double fork_scale[4];
  double graded_ratio;   /* instances whose mesh has largest / smallest element above this ratio (0:
                            none) take the graded-mesh step: preconditioner spacings floored at
                            sqrt(precond_hfloor * ds), the contour diffusion scale below which the
                            preconditioner's curvature means nothing, and each node's move clamped
                            to step_cap / ds instead of the whole step scaled (one wall node of a
                            mesh graded to 1e-6 would otherwise throttle every other node) */
  double precond_hfloor;
  int transfer_stride;/* > 1: instances that share a mesh shape (node count, contour steps, rule and
                         spacing ratio) are solved in rounds.  Sorted by film width L, every
                         transfer_stride-th of them (and the widest) is solved first from its own
                         field with the cap maxit/2; then every instance not converged starts from
                         the field interpolated in L, node by node, between its two nearest
                         converged neighbours, and is solved with the cap maxit/4, and once more
                         with the full cap for those still not converged.  Iteration counts add up
                         over an instance's rounds.  On meshes graded toward the walls, where the
                         field's wall layer makes any smooth start slower than the cold one, a
                         neighbour's converged field is a start within a few iterations of the
                         answer.  0 or 1: off */
} scft_solve_opts;

typedef struct scft_result {
  int status;         /* SCFT_ST_* bits */
  int iterations;
  double err;         /* ||phi - f0||_inf at the last evaluation */
  double Q;
} scft_result;

typedef struct scft_batch scft_batch;

void scft_solve_opts_init(scft_solve_opts *o);

/* Copies the instances to the device.  Returns SCFT_OK and *out, or an error
   (the lowest invalid instance is named).  Large batches are checked and packed
   into one pinned upload buffer by up to 8 host threads that end before the
   call returns; the caller's arrays are only read, and may be reused at once. */
int scft_batch_create(const scft_instance *inst, int count, scft_batch **out);
/* Overwrite all fields (concatenated n_nodes values per instance; wall values
   are kept for the free energy, the propagator ignores them). */
int scft_batch_set_fields(scft_batch *b, const double *w_nodes);
/* One propagator pass at the current fields (density and Q for every instance). */
int scft_batch_evaluate(scft_batch *b, int precision);
/* Solve every instance to opts->tol; res (count entries) may be NULL. */
int scft_batch_solve(scft_batch *b, const scft_solve_opts *opts, scft_result *res);
/* Enqueues the fused FP32 solve of b (opts as scft_batch_solve; fused = 1,
   verify64 = 0) on b's own streams and returns without waiting; scft_batch_wait
   completes it (results as scft_batch_solve).  Solves of different batches in
   flight at the same time share the GPU: while one batch's slowest instances run
   their last iterations, the next batch's instances take the SMs that have
   emptied.  One solve per batch may be in flight. */
int scft_batch_solve_async(scft_batch *b, const scft_solve_opts *opts);
int scft_batch_wait(scft_batch *b, scft_result *res);
/* Copy fields / densities (concatenated n_nodes per instance) and Q out; any may be NULL. */
int scft_batch_get(scft_batch *b, double *w_nodes, double *phi_nodes, double *Q);
/* Restore every field to the w0 given at creation (device copy, no host traffic). */
int scft_batch_reset(scft_batch *b);
/* Device time of the last scft_batch_evaluate / scft_batch_solve / scft_batch_reset,
   measured with CUDA events on the batch's stream (ms). */
double scft_batch_last_ms(scft_batch *b);
/* Progress of the last scft_batch_solve: after each CUDA-graph launch
   (iters_per_graph iterations) the number of unfinished instances and the host
   time since the solve started (ms).  Writes at most max entries and returns
   the number of graph launches. */
int scft_batch_trace(scft_batch *b, int max, int *active, double *ms);
/* Per shape class of precision p: nodes per thread, warps per instance, instance
   count, algorithmic half-contour bytes of one pass (write + read of slices
   0..nsteps/2 of every node, 4 or 8 bytes each) and the event-timed duration (ms)
   of one pass of that class alone.  Writes at most max_classes entries and
   returns the number of classes (or an error code). */
int scft_batch_profile(scft_batch *b, int precision, int max_classes, int *C, int *NW, int *items,
                       double *bytes, double *ms);
/* Propagator launches of the last scft_batch_solve, per shape class of the
   given precision: launches that evaluated at least one instance, their
   algorithmic bytes (write and read of every half-contour slice) and their
   summed durations from CUDA events recorded around each launch inside the
   solve graphs.  Returns the number of classes (entries written <= max_classes).
   No reference counterpart (measurement). */
int scft_batch_live_stats(scft_batch *b, int precision, int max_classes, int *C, int *NW, long long *launches,
                          double *bytes, double *ms);
/* Mean-field free energy of every instance at its current field, as
   DEALII_SCFT/src/scft.cc:404-450 reports it:
     F = ( int w_h f0 dx / f0bar / L + ln f0bar ) / (-1000),  f0bar = (1/L) int f0 dx,
   with both integrals by Romberg (romint.c:21) over m+1 uniform samples of the
   target on [0, L] (m a power of two >= 16; scft.cc uses 2^18) and w_h the
   piecewise-linear field.  f0_samples: count x (m+1) doubles; F: count doubles. */
int scft_batch_free_energy(scft_batch *b, int m, const double *f0_samples, double *F);
/* Per-instance status bits of the last evaluate/solve (count ints). */
int scft_batch_status(scft_batch *b, int *status);
/* Choose the propagator shape of one instance: C nodes per thread (1,2,4,8) and
   NW warps per instance (1..32); C = 0 restores the default. */
int scft_batch_set_shape(scft_batch *b, int precision, int index, int C, int NW);
/* Time the candidate shapes of each (size, precision) bucket on this batch and
   keep the fastest (the autotuner). */
int scft_batch_autotune(scft_batch *b, int precision);
int scft_batch_destroy(scft_batch *b);

/* =========================================================================
 * Learned warm start.  No counterpart in the reference, which reads its
 * initial fields from files (1D_FEM.c:321-342, DEALII_SCFT/src/scft_util.cc:14-41).
 * A 1D-conv network (4 dilated layers, 64 channels, kernel 5, FP32 weights,
 * BF16 activations) maps the film width L, the contour step count and the
 * target profile on a 256-point grid of the mesh coordinate to w0(x).  The
 * plain mixing loop still converges every instance to the same tolerance.
 * ========================================================================= */

typedef struct scft_ws scft_ws;

/* act_bf16 = 1 stores hidden activations in BF16 (0: FP32, for gradient checks). */
int scft_ws_create(int act_bf16, unsigned long long seed, scft_ws **out);
int scft_ws_destroy(scft_ws *ws);
/* Number of FP32 parameters (weights then bias of each layer), or an error code. */
int scft_ws_param_count(scft_ws *ws);
int scft_ws_get_params(scft_ws *ws, float *out);
int scft_ws_set_params(scft_ws *ws, const float *in);
/* Host buffers: features B x 4 x 256, out B x 256 (w / 5 on the grid). */
int scft_ws_forward(scft_ws *ws, const float *features, int B, float *out);
/* Mean-squared error of the forward pass against targets (B x 256) and its
   gradient with respect to every parameter (param_count floats). */
int scft_ws_loss_grad(scft_ws *ws, const float *features, const float *targets, int B, double *loss,
                      float *grad);
/* The network inputs of every instance of a batch (count x 4 x 256) and, when
   targets != NULL, its current fields resampled to the grid (count x 256, / 5). */
int scft_ws_batch_features(scft_batch *b, float *features, float *targets);
/* Append the instances of b selected by mask (NULL: all) with their current
   fields as training samples.  Returns the dataset size or an error code. */
int scft_ws_dataset_from_batch(scft_ws *ws, scft_batch *b, const int *mask);
/* Adam on the dataset: steps minibatches of `batch` samples, learning rate
   decaying from lr to lr/50 on a cosine; losses (steps floats, may be NULL)
   receives the minibatch losses. */
int scft_ws_train(scft_ws *ws, int steps, int batch, float lr, unsigned long long seed, float *losses);
/* Overwrite the fields of b with the network's prediction (on b's stream;
   scft_batch_last_ms reports its device time).  Instances whose mesh has
   largest / smallest element above 16 (outside the network's training set of
   uniform meshes) keep their field. */
int scft_ws_predict(scft_ws *ws, scft_batch *b);
const char *scft_ws_last_error(void);
/* With BF16 activations the two 64 -> 64 layers run on the tensor cores
   (tcgen05.mma, BF16 operands from a BF16 copy of the FP32 weights, FP32
   accumulators in tensor memory); on = 0 selects the CUDA-core convolution
   (FP32 weights) instead.  Returns the previous setting. */
int scft_ws_set_tensor_cores(scft_ws *ws, int on);
/* 0, or the nonzero code a bounded wait of the tensor-core layers recorded
   since the network was created (that layer's outputs were then not written). */
int scft_ws_tensor_core_status(scft_ws *ws);

/* =========================================================================
 * Density without any device allocation.  No counterpart in the reference.
 *
 * For callers that may not allocate GPU memory: applications whose device
 * memory belongs to another allocator (a framework's pool with a fixed budget)
 * and per-iteration loops that cannot afford cudaMalloc/cudaFree, which can
 * block on or synchronize the whole device.  The caller passes device buffers:
 * x and w (n_nodes doubles: mesh and field, wall values of w ignored), phi
 * (n_nodes doubles, out), Q (one double, out, may be NULL) and status (one int,
 * out, may be NULL: the SCFT_ST_NOT_DOMINANT / SCFT_ST_NONFINITE bits of the
 * instance, as scft_batch_status reports them; 0 when the density is sound).
 * Each must be device (or managed) memory; anything else is refused with
 * SCFT_EINVAL before any launch.  The work is enqueued on `stream` (a
 * cudaStream_t, NULL for the default stream) and the results are ready when
 * that stream has completed; nothing is copied to or from the host.
 *
 * The propagator's half-contour store lives in one fixed 32 MiB device array
 * of the library (every GPU that loads the library holds it until the process
 * exits): an instance needs (nsteps/2 + 1) x padded nodes x 4 bytes (FP32) or
 * 8 bytes (FP64); larger instances are rejected with SCFT_EINVAL and a message
 * from scft_last_error().  All calls of one process share that array, so calls
 * whose GPU work overlaps in time (different streams or threads of the process)
 * race and must be serialised by the caller.  Every call looks up the array's
 * device address (cudaGetSymbolAddress); the first call on a device may load the
 * library's device code, so make it before any stream capture.  Same density,
 * Q and status as scft_batch_evaluate.
 * ========================================================================= */
int scft_density_noalloc(int n_nodes, const double *x, const double *w, int nsteps, double ds, int rule,
                         int precision, double *phi, double *Q, int *status, void *stream);

/* =========================================================================
 * The reference's field files (host only; no device is needed).
 * ========================================================================= */

/* Reads a field file in the form DEALII_SCFT/src/scft.cc:317-333 writes and
   DEALII_SCFT/src/scft_util.cc:14-41 (read_yita_middle_1D) reads:
     "N= <nodes>, ERROR= <e>", "mean_field_free_energy, <F>", then "i,x_i,w_i"
   per node.  The MATLAB inputs (Matlab_files/inputFiles/solution_yita_1D_N=*.txt,
   first line "N= <nodes>" only, no energy line) are read too.  *n_nodes receives
   N (also when N > max_nodes, which returns SCFT_EINVAL); x and w (max_nodes
   doubles, either may be NULL) receive the nodes; *err and *free_energy (may be
   NULL) receive the header values or NAN when the file has none.  Every node
   0..N-1 must be present.  SCFT_EIO when the file cannot be opened. */
int scft_field_read(const char *path, int max_nodes, int *n_nodes, double *x, double *w, double *err,
                    double *free_energy);
/* Writes the form above with the reference's formats ("%e" error, "%2.15f"
   energy and values), so read_yita_middle_1D reads it back. */
int scft_field_write(const char *path, int n_nodes, const double *x, const double *w, double err,
                     double free_energy);
/* Reads a .res table of the external implicit-Euler code (the file
   1D_FEM.c:321-342 takes its starting field from): every row of five numbers
   (x/l, phi, eta, phie, phij; walls included) into table (row-major, max_rows x
   5), *rows = rows found (SCFT_EINVAL when above max_rows), *m and *nsteps from
   "m = <m>   n = <steps>" (-1 when absent), header[6] = l, mphi, t, Z, f,
   |f|max (NAN when absent; may be NULL). */
int scft_res_read(const char *path, int max_rows, int *rows, double *table, int *m, int *nsteps, double *header);

/* =========================================================================
 * Mesh refinement and field transfer of the deal.II driver (refine_mesh,
 * DEALII_SCFT/src/scft.cc:132-166).
 * ========================================================================= */

/* Bisects every element of the mesh x (n_nodes points) into x_new (2 n_nodes - 1
   points), the refinement refine_mesh applies (every cell is cut in x). */
int scft_refine_bisect(int n_nodes, const double *x, double *x_new);
/* Cubic splines of `count` tables, evaluated on the GPU (FP64): table t has
   nx[t] points (x, y; concatenated over the tables, x strictly increasing) and
   is evaluated at nxp[t] points (xp, concatenated) into yp.  The spline of
   spline_chen (spline_chen.c:13-106): m == NULL gives not-a-knot ends (nx >= 4),
   otherwise the second derivative *m at both ends; points outside a table take
   its end cubic.  refine_mesh transfers the interior field with
   spline_chen(&x[1], &w[1], &x_new[1], &w_new[1], n - 2, n_new - 2, NULL). */
int scft_spline(int count, const int *nx, const double *x, const double *y, const int *nxp, const double *xp,
                double *yp, const double *m);

/* The library keeps the device and pinned host blocks it releases (batches,
   scratch, warm-start buffers) for reuse, so creating a batch per request does
   not call cudaMalloc/cudaFree again; a failed allocation releases the cache and
   retries.  This returns the cached blocks of the current device and the cached
   pinned blocks to CUDA and reports the bytes released. */
long long scft_mem_trim(void);
/* Allocation counters of the library since load: *requests = device and pinned
   host blocks requested from the cache above (served from it or new), *cuda_allocs
   = the cudaMalloc / cudaMallocHost calls among them.  Either may be NULL. */
void scft_mem_counters(long long *requests, long long *cuda_allocs);

/* Density and Q of every instance of b (FP64) with the given contour scheme and
   field term: SCFT_SCHEME_IRK2 with SCFT_W_CONSISTENT is the propagator of the
   reference's deal.II driver (drivescft.cc:130-207, scft.cc:589-696);
   SCFT_SCHEME_IE with SCFT_W_ROWSCALED is the one of 1D_FEM.c.  Results via
   scft_batch_get; one thread per instance (complex Thomas sweeps of the
   decoupled stage system).  No counterpart of its own in the reference. */
int scft_batch_evaluate_scheme(scft_batch *b, int scheme, int wmode);

/* Kernels launched by this library since load (graph replays count each node). */
long long scft_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif
