// ref_shim_dealii.cc -- TEST INFRASTRUCTURE ONLY (checker bridge).
//
// Links the reference's own DEALII_SCFT/src NR routines, compiled from source
// as C++ the way DEALII_SCFT/CMakeLists.txt:36 compiles them, and exposes them
// with C linkage for the tests: adm_chen (ADM_chen_C.c:18), broydn
// (DEALII_SCFT/src/broydn.c:44), romint (romint.c:21), gaussj
// (DEALII_SCFT/src/gaussj.c:7) and spline_chen (spline_chen.c:13).  The reference calls exit() on errors
// (nrutil.c:16-23, romint.c:31, ADM_chen_C.c:65); the recipe redirects exit to
// __wrap_exit at link time so that an error unwinds back here.
#include <csetjmp>
#include <cstdio>
#include <cstdlib>

#include "NR_chen.h"

// Globals the reference's broydn.c expects from its caller (drivescft.cc:250-256).
double *f0_given;
double **qt, **r, *d, err;
int funcerr, jc, PRINT;

double **dmatrix(long, long, long, long);
double *dvector(long, long);
void free_dmatrix(double **, long, long, long, long);
void free_dvector(double *, long, long);
void broydn(double x[], int n, int *check, void (*vecfunc)(int, double[], double[]));
int gaussj(double **a, int n, double **b, int m);
double romint(double *, int, double);

static std::jmp_buf g_jb;
static int g_armed = 0;
static void (*g_user)(int, double *, double *) = nullptr;
static int g_calls = 0, g_max_calls = 0;

extern "C" void __wrap_exit(int code) {
  if (g_armed) std::longjmp(g_jb, 100 + (code & 0xff));
  std::_Exit(code);
}

static void trampoline(int n, double *in, double *out) {
  if (g_max_calls > 0 && g_calls >= g_max_calls) std::longjmp(g_jb, 1);
  g_calls++;
  g_user(n, in, out);
}

extern "C" {

// Returns adm_chen's status (0 solved, 1 not), -1 when the call budget ran
// out, or -(100+code) when the reference called exit(code).
int ref_adm_chen(void (*f)(int, double *, double *), double *x, double tol, int maxit, int n,
                 double lmd, int nn, int final_, int max_calls, int *ncalls) {
  g_user = f; g_calls = 0; g_max_calls = max_calls;
  int rc;
  int j = setjmp(g_jb);
  if (j == 0) {
    g_armed = 1;
    rc = adm_chen(trampoline, x, tol, maxit, n, lmd, nn, final_ != 0);
  } else {
    rc = (j == 1) ? -1 : -j;
  }
  g_armed = 0;
  if (ncalls) *ncalls = g_calls;
  return rc;
}

// x1 is 1-based (x1[1..n]) as broydn.c expects.  *check as broydn sets it.
int ref_broydn(void (*f)(int, double *, double *), double *x1, int n, double tol, int max_calls,
               int *ncalls, int *check) {
  g_user = f; g_calls = 0; g_max_calls = max_calls;
  qt = dmatrix(1, n, 1, n);
  r = dmatrix(1, n, 1, n);
  d = dvector(1, n);
  jc = 0; funcerr = 0; PRINT = 0;
  err = tol;
  int rc = 0;
  int j = setjmp(g_jb);
  if (j == 0) {
    g_armed = 1;
    broydn(x1, n, check, trampoline);
  } else {
    rc = (j == 1) ? -1 : -j;
  }
  g_armed = 0;
  free_dmatrix(qt, 1, n, 1, n);
  free_dmatrix(r, 1, n, 1, n);
  free_dvector(d, 1, n);
  if (ncalls) *ncalls = g_calls;
  return rc;
}

double ref_romint(double *f, int m, double hh) {
  double v = 0.0;
  int j = setjmp(g_jb);
  if (j == 0) {
    g_armed = 1;
    v = romint(f, m, hh);
  } else {
    v = 0.0 / 0.0;
  }
  g_armed = 0;
  return v;
}

// a: n*n row-major, b: n*m row-major, solved in place. Returns gaussj's status.
int ref_gaussj_dealii(double *a, int n, double *b, int m) {
  double **A = dmatrix(1, n, 1, n), **B = dmatrix(1, n, 1, m);
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < n; k++) A[i + 1][k + 1] = a[i * n + k];
    for (int k = 0; k < m; k++) B[i + 1][k + 1] = b[i * m + k];
  }
  int rc = gaussj(A, n, B, m);
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < n; k++) a[i * n + k] = A[i + 1][k + 1];
    for (int k = 0; k < m; k++) b[i * m + k] = B[i + 1][k + 1];
  }
  free_dmatrix(A, 1, n, 1, n);
  free_dmatrix(B, 1, n, 1, m);
  return rc;
}


// spline_chen (spline_chen.c:13-106): m == NULL selects the not-a-knot end
// condition.  Returns 0, or -(100+code) when the reference called exit(code).
int ref_spline_chen(double *x, double *y, double *xp, double *yp, int nx, int nxp, double *m) {
  int rc = 0;
  int j = setjmp(g_jb);
  if (j == 0) {
    g_armed = 1;
    spline_chen(x, y, xp, yp, nx, nxp, m);
  } else {
    rc = -j;
  }
  g_armed = 0;
  return rc;
}

}  // extern "C"
