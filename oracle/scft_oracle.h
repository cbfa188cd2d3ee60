/*
 * scft_oracle.h -- CPU FP64 oracle for the SCFT inner loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker, not the product: only the
 * tests, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs
 * may load it.  The product path (libscft.so) never links or calls it.
 *
 * It restates, in plain C, the reference's method for the hot path:
 *   - FEM assembly and implicit Euler contour loop   1D_FEM.c:95-228,
 *                                                     Matlab_files/simple_FEM_1D_transient.m:34-114
 *   - density quadrature (Romberg / trapezoid)        DEALII_SCFT/src/romint.c:21-57, polint.c:5-43,
 *                                                     simple_FEM_1D_transient.m:119-124
 *   - residual                                        1D_FEM.c:274-277 (phi-f0), drivescft.cc:210-215 (f0-phi)
 *   - deal.II variant (consistent W, Gauss-Legendre 2-stage IRK)
 *                                                     drivescft.cc:130-207, scft.cc:589-696
 *   - Gauss-Jordan, Anderson (adm, adm_chen)          gaussj.c:7-60, adm.c:24-313,
 *                                                     DEALII_SCFT/src/ADM_chen_C.c:18-147
 *   - Broyden (QR-updated, line search)               broydn.c:44-292 and DEALII_SCFT/src/{fdjac,lnsrch,
 *                                                     qrdcmp,qrupdt,rsolv,rotate}.c
 *
 * Parity of this restatement is pinned against the reference's golden fields
 * (Matlab_files/inputFiles/solution_matlab_N=33, DEALII_SCFT/inputFiles/N=33_for_read.txt),
 * the known answer f0bar (scft.cc:368) and the reference's own NR routines compiled from
 * source into oracle/_ref by oracle/Makefile.
 *
 * All arrays are 0-based; interior unknowns of an n-node mesh are nodes 1..n-2.
 */
#ifndef SCFT_ORACLE_H
#define SCFT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* density quadrature rule over the contour samples 0..nsteps */
enum { OR_RULE_ROMBERG = 0, OR_RULE_TRAPEZOID = 1 };
/* field term of the FEM system */
enum { OR_W_ROWSCALED = 0, OR_W_CONSISTENT = 1 };
/* contour time stepping */
enum { OR_SCHEME_IE = 0, OR_SCHEME_IRK2 = 1 };

typedef struct or_problem {
  int n;               /* nodes (elements + 1) */
  const double *x;     /* node coordinates, n, x[0]=0, x[n-1]=L */
  const double *f0;    /* target density at the nodes, n */
  double ds;           /* contour step */
  int nsteps;          /* number of contour steps (samples 0..nsteps) */
  int rule;            /* OR_RULE_* */
  int wmode;           /* OR_W_* */
  int scheme;          /* OR_SCHEME_* */
  int sign;            /* +1: out = phi - f0 (1D_FEM.c:276); -1: out = f0 - phi (drivescft.cc:212) */
  const double *wall_w;/* optional: w at nodes 0 and n-1 (consistent W only), else 0 */
} or_problem;

/* ---- meshes and targets ---- */
void or_mesh_uniform(int n, double L, double *x);
int  or_mesh_graded(int m_elem, double ratio, double L, double *x);
void or_f0_tanh2_ceil(int n, const double *x, double tau, double L, double *f0);
void or_f0_tanh2_le(int n, const double *x, double tau, double *f0);
void or_f0_gauss_wall(int n, const double *x, double L, double width, double *f0);

/* ---- quadrature ---- */
double or_romint(const double *f, int m, double hh);
int    or_quad_weights(int nsteps, double ds, int rule, double *W);

/* ---- propagator ---- */
/* w: full nodal field (n values; w[0], w[n-1] only used by consistent W).
   phi: n values out. Q: optional, (1/L) * int q(x,1) dx.  q_store: optional
   (nsteps+1)*n values, slice-major.  Returns 0, or <0 on bad input. */
int or_propagate(const or_problem *p, const double *w, double *phi, double *Q, double *q_store);
/* residual on interior nodes: w_int has n-2 values, out has n-2 values */
int or_residual(const or_problem *p, const double *w_int, double *out, double *phi_out);

/* ---- dense algebra + solvers ---- */
/* a: n*n row-major, b: n*m row-major; singular_mode 0: perturb zero pivot by 1e-18
   (gaussj.c:38), 1: return 1 (DEALII_SCFT/src/gaussj.c:45-50). Returns 0 / 1. */
int or_gaussj(double *a, int n, double *b, int m, int singular_mode);

typedef void (*or_vecfunc)(int n, const double *x, double *out, void *ctx);
void or_problem_vecfunc(int n, const double *x, double *out, void *ctx);

/* Anderson mixing for F(x)=0 in the form of ADM_chen_C.c:18-147.
   x: in/out (n).  trace (optional, maxit+2 doubles) receives ||F||_inf per
   iteration.  *iters receives the iteration count.  Returns 0 converged,
   1 not converged, 2 NaN residual. */
int or_adm_chen(or_vecfunc f, void *ctx, double *x, double tol, int maxit, int n,
                double lmd, int nn, int final_, int *iters, double *trace);

/* Anderson mixing for x = g(x) in the ring-buffer form of adm.c:24-313.
   Returns 0 converged (err < tol), 1 otherwise; *iters receives its. */
int or_adm(or_vecfunc g, void *ctx, double *x, int n, double tol, int maxit, int *iters);

/* Globally convergent Broyden (broydn.c:44-292) for F(x)=0; tol on ||F||_inf.
   Returns 0 converged, 1 failed, 2 singular Jacobian, 3 line-search roundoff. */
int or_broydn(or_vecfunc f, void *ctx, double *x, int n, double tol, int *iters, int *nfev);

/* Safeguarded Anderson solve of one instance, the CPU restatement of the GPU
   batched solver's mixing (scft_gb300/csrc/mixing.cu, mix_kernel): mixing
   residual g = P(ln phi - ln f0) (mode 1) or P(phi - f0) (mode 0) with
   P = 1 + a (-d2/dx2) (lumped FEM Laplacian, no curvature term at the first and
   last interior nodes), difference-form history of depth <= 16,
   Tikhonov-regularised least squares (inner products weighted by
   (f0 / max f0)^2 when `weighted`), a step clip in the (f0 / max f0)-weighted
   max norm, a cap of cap/ds on any node's change, a floor -floor/ds on the
   field and a history restart when the error grows by `grow`.  w: full nodal
   field in/out.
   Returns 0 converged (||phi - f0||_inf <= tol), 1 max iterations, 2 non-finite. */
typedef struct or_mix_opts {
  double tol, beta, clip, grow, reg, precond;
  int maxit, depth, mode, schedule; /* schedule: beta = 1 - lk with lk of ADM_chen_C.c:125-129 */
  double cap, floor;                /* 0 disables either */
  int weighted;
  /* meshes whose largest / smallest element exceeds graded_ratio (0: never)
     take the graded-mesh step: preconditioner spacings floored at
     sqrt(hfloor * ds), and each node's move clamped to cap / ds instead of the
     whole step scaled */
  double graded_ratio, hfloor;
} or_mix_opts;
int or_anderson_solve(const or_problem *p, double *w, const or_mix_opts *o, int *iters, double *err);

/* The CPU baseline's batch driver: or_anderson_solve of `count` independent
   instances on `threads` POSIX threads (each thread takes the next unsolved
   instance from a shared counter).  w: the instances' full nodal fields one
   after another (node counts p[i].n), solved in place.  rc, iters, err:
   per-instance outputs.  Returns 0, or -1 when a thread cannot be started. */
int or_anderson_solve_batch(const or_problem *p, int count, double *w, const or_mix_opts *o, int threads,
                            int *rc, int *iters, double *err);

/* Cubic spline of the table (x, y) (nx points, x increasing) evaluated at the
   nxp points xp into yp: spline_chen.c:13-106.  m == NULL: not-a-knot end
   conditions (the third derivative is continuous at the second and second-last
   points; nx > 3); otherwise the second derivative is *m at both ends.  The
   second derivatives solve the same equations as the reference's dense system,
   here with the end values eliminated into the inner rows and a Thomas sweep.
   Points outside [x0, x_{nx-1}] take the end cubic (extrapolation), as the
   reference's bisection does.  Returns 0, -1 for nx too small, -2 for x not
   strictly increasing. */
int or_spline(const double *x, const double *y, int nx, const double *xp, double *yp, int nxp, const double *m);

#ifdef __cplusplus
}
#endif
#endif
