/* A C program that uses libscft the way the reference's 1D_FEM.c main
   (1D_FEM.c:289-370) uses its own solvers: it sets the problem once, then hands
   the drop-in residual (the replacement of simple_FEM_1D_transient, 1D_FEM.c:47)
   to Broyden (broydn(x_nr, N - 2, &check, simple_FEM_1D_transient), 1D_FEM.c:356)
   and to Anderson mixing (adm(in, n, &check, f, flag), 1D_FEM.c:366), with
   1-based NR vectors throughout.

   Input on stdin: N, tol, then N node coordinates, N target values and N-2
   initial interior field values.  Output: the residual of the initial field,
   then one line per solver run -- "<name> check=<c> rc=<rc> maxres=<|F|inf>"
   followed by the interior field. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "scft.h"

static int N;

static double max_residual(const double *x_nr) {
  double *out = (double *)calloc((size_t)N, sizeof(double));
  double m = -1.0;
  if (out && scft_fem_residual(N - 2, (double *)x_nr, out) == SCFT_OK) {
    m = 0.0;
    for (int i = 1; i <= N - 2; i++) m = fmax(m, fabs(out[i]));
  }
  free(out);
  return m;
}

static void report(const char *name, int check, int rc, const double *x_nr) {
  printf("%s check=%d rc=%d maxres=%.17g", name, check, rc, max_residual(x_nr));
  for (int i = 1; i <= N - 2; i++) printf(" %.17g", x_nr[i]);
  printf("\n");
}

int main(void) {
  double tol;
  if (scanf("%d %lf", &N, &tol) != 2 || N < 4) return 2;
  double *x = (double *)malloc(sizeof(double) * N), *f0 = (double *)malloc(sizeof(double) * N);
  double *w0 = (double *)malloc(sizeof(double) * N), *x_nr = (double *)malloc(sizeof(double) * N);
  if (!x || !f0 || !w0 || !x_nr) return 2;
  for (int i = 0; i < N; i++) if (scanf("%lf", &x[i]) != 1) return 2;
  for (int i = 0; i < N; i++) if (scanf("%lf", &f0[i]) != 1) return 2;
  for (int i = 1; i <= N - 2; i++) if (scanf("%lf", &w0[i]) != 1) return 2;

  /* the reference's globals: 2049 implicit-Euler steps of 1/2048, trapezoid,
     out = f0 - phi (the MATLAB driver's residual) */
  scft_config c;
  scft_config_init(&c);
  c.n_nodes = N;
  c.x = x;
  c.L = x[N - 1] - x[0];
  c.f0 = f0;
  c.nsteps = 2049;
  c.ds = 1.0 / 2048;
  c.rule = SCFT_RULE_TRAPEZOID;
  c.sign = -1;
  if (scft_set_config(&c) != SCFT_OK) {
    fprintf(stderr, "scft_set_config: %s\n", scft_last_error());
    return 1;
  }

  printf("initial maxres=%.17g\n", max_residual(w0));

  /* Broyden through the library's int-returning entry point */
  int check = 1;
  for (int i = 1; i <= N - 2; i++) x_nr[i] = w0[i];
  scft_broydn_set_tol(tol);
  int rc = scft_broydn(x_nr, N - 2, &check, scft_fem_residual_vf);
  report("scft_broydn", check, rc, x_nr);

  /* Broyden with broydn's own signature (void) */
  check = 1;
  for (int i = 1; i <= N - 2; i++) x_nr[i] = w0[i];
  scft_nr_broydn(x_nr, N - 2, &check, scft_fem_residual_vf);
  report("scft_nr_broydn", check, 0, x_nr);

  /* Anderson mixing with adm's own signature: the returned vector is the last
     map value, freed as the reference frees its NR vectors */
  check = 1;
  for (int i = 1; i <= N - 2; i++) x_nr[i] = w0[i];
  scft_adm_set_maxit(30);
  double *xnew = scft_nr_adm(x_nr, N - 2, &check, scft_fem_fixedpoint_vf, 1);
  report("scft_nr_adm", check, xnew ? 0 : -1, x_nr);
  if (xnew) {
    /* xnew[1..N-2] = x + (phi - f0) at the last evaluated field: finite values */
    int finite = 1;
    for (int i = 1; i <= N - 2; i++) finite &= isfinite(xnew[i]) != 0;
    printf("scft_nr_adm_xnew finite=%d\n", finite);
    scft_nr_free_vector(xnew, 1);
  }
  free(x); free(f0); free(w0); free(x_nr);
  return 0;
}
