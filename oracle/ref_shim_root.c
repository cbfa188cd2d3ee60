/* ref_shim_root.c -- TEST INFRASTRUCTURE ONLY (checker bridge).
 *
 * Links the reference's root-level adm.c (adm.c:24-313), gaussj.c (gaussj.c:7-60)
 * and nrutil.c, compiled from source as C, and exposes them to the tests.  exit()
 * in the reference objects is redirected to __wrap_exit at link time so that an
 * error unwinds back here instead of ending the test process. */
#include <setjmp.h>
#include <stdlib.h>

double *adm(double *x, int n, int *check, void (*funcvmix)(int, double *, double *), int flag);
void gaussj(double **a, int n, double **b, int m);
double **dmatrix(long, long, long, long);
void free_dmatrix(double **, long, long, long, long);

static jmp_buf g_jb;
static int g_armed = 0;
static void (*g_user)(int, double *, double *) = 0;
static int g_calls = 0, g_max_calls = 0;

void __wrap_exit(int code) {
  if (g_armed) longjmp(g_jb, 100 + (code & 0xff));
  _Exit(code);
}

static void trampoline(int n, double *in, double *out) {
  if (g_max_calls > 0 && g_calls >= g_max_calls) longjmp(g_jb, 1);
  g_calls++;
  g_user(n, in, out);
}

/* x indexed from flag (0 or 1) as adm.c expects.  Returns 0 when adm returned
   (its status in *check), -1 when the call budget ran out, -(100+code) on exit. */
int ref_adm(void (*g)(int, double *, double *), double *x, int n, int flag, int max_calls,
            int *ncalls, int *check) {
  g_user = g; g_calls = 0; g_max_calls = max_calls;
  int rc = 0;
  int j = setjmp(g_jb);
  if (j == 0) {
    g_armed = 1;
    adm(x, n, check, trampoline, flag);
  } else {
    rc = (j == 1) ? -1 : -j;
  }
  g_armed = 0;
  if (ncalls) *ncalls = g_calls;
  return rc;
}

void ref_gaussj_root(double *a, int n, double *b, int m) {
  double **A = dmatrix(1, n, 1, n), **B = dmatrix(1, n, 1, m);
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < n; k++) A[i + 1][k + 1] = a[i * n + k];
    for (int k = 0; k < m; k++) B[i + 1][k + 1] = b[i * m + k];
  }
  gaussj(A, n, B, m);
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < n; k++) a[i * n + k] = A[i + 1][k + 1];
    for (int k = 0; k < m; k++) b[i * m + k] = B[i + 1][k + 1];
  }
  free_dmatrix(A, 1, n, 1, n);
  free_dmatrix(B, 1, m, 1, m);
}
