/*
 * scft_oracle.c -- CPU FP64 oracle for the SCFT inner loop (test infrastructure).
 *
 * TEST INFRASTRUCTURE ONLY: the checker used by tests/, __graft_entry__.smoke()
 * and bench.py's CPU legs.  It is never linked into the product library.
 *
 * Each function cites the reference lines whose behaviour it restates.  The
 * reference's own PETSc/deal.II executables cannot be built (PETSc and deal.II
 * are absent), so the propagator is restated here; the MATLAB prototype's exact
 * dense solve (simple_FEM_1D_transient.m:80) defines the discrete answer, which
 * a tridiagonal (Thomas) solve reproduces to rounding.
 */
#include "scft_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* meshes and wall targets                                                   */
/* ------------------------------------------------------------------------- */

/* Uniform mesh x_i = i L/(n-1)  (1D_FEM.c:61,310; drivescft.cc:94-98). */
void or_mesh_uniform(int n, double L, double *x) {
  for (int i = 0; i < n; i++) x[i] = L * (double)i / (double)(n - 1);
  x[n - 1] = L;
}

/* Mesh of m_elem elements graded geometrically toward both walls: element k
   (counted from the nearer wall) has length h0*ratio^k; the two halves mirror.
   The reference refines adaptively (scft.cc:132-169); this is the fixed graded
   mesh of the large-mesh workload.  Returns -1 if m_elem is odd. */
int or_mesh_graded(int m_elem, double ratio, double L, double *x) {
  if (m_elem < 2 || (m_elem & 1)) return -1;
  int half = m_elem / 2;
  double geo = (fabs(ratio - 1.0) < 1e-15) ? (double)half
                                          : (pow(ratio, half) - 1.0) / (ratio - 1.0);
  double h0 = 0.5 * L / geo, acc = 0.0, hk = h0;
  x[0] = 0.0;
  for (int k = 0; k < half; k++) {
    acc += hk;
    x[k + 1] = acc;
    hk *= ratio;
  }
  x[half] = 0.5 * L;
  for (int k = 0; k < half; k++) x[m_elem - k] = L - x[k];
  return 0;
}

/* tanh^2-type wall profile, f0 = ((e^a-1)/(e^a+1))^2 with a = 4 tau x/(tau^2-x^2),
   applied to the first ceil(n tau/L) nodes and mirrored; 1 elsewhere
   (1D_FEM.c:303-319, Matlab_files/set_f0_given.m:1-14; NaN -> 1 as in the .m). */
void or_f0_tanh2_ceil(int n, const double *x, double tau, double L, double *f0) {
  for (int i = 0; i < n; i++) f0[i] = 1.0;
  int left = (int)ceil((double)n * tau / L);
  for (int i = 0; i < left && i < n; i++) {
    double a = 4.0 * tau * x[i] / (tau * tau - x[i] * x[i]);
    double e = exp(a);
    double v = ((e - 1.0) * (e - 1.0)) / ((e + 1.0) * (e + 1.0));
    if (isnan(v)) v = 1.0;
    f0[i] = v;
    f0[n - 1 - i] = v;
  }
}

/* Same profile applied while x <= tau, NaN -> 1 (DEALII_SCFT/src/scft.cc:188-215). */
void or_f0_tanh2_le(int n, const double *x, double tau, double *f0) {
  for (int i = 0; i < n; i++) f0[i] = 1.0;
  for (int i = 0; i < n; i++) {
    if (!(x[i] <= tau)) break;
    double a = 4.0 * tau * x[i] / (tau * tau - x[i] * x[i]);
    double e = exp(a);
    double v = ((e - 1.0) * (e - 1.0)) / ((e + 1.0) * (e + 1.0));
    if (isnan(v)) v = 1.0;
    f0[i] = v;
    f0[n - 1 - i] = v;
  }
}

/* Gaussian wall profile f0 = (1-exp(-(x/w)^2)) (1-exp(-((L-x)/w)^2)) of the
   synthetic workloads (the reference's tanh^2 profile replaced, width w). */
void or_f0_gauss_wall(int n, const double *x, double L, double width, double *f0) {
  for (int i = 0; i < n; i++) {
    double a = x[i] / width, b = (L - x[i]) / width;
    f0[i] = (1.0 - exp(-a * a)) * (1.0 - exp(-b * b));
  }
}

/* ------------------------------------------------------------------------- */
/* quadrature                                                                */
/* ------------------------------------------------------------------------- */

/* Extrapolate the points (h[k], s[k]), k=0..K-1 to h=0 with Neville's tableau
   (the role polint.c:5-43 plays inside romint.c:50). */
static double neville_at_zero(const double *h, const double *s, int K) {
  double t[16];
  for (int k = 0; k < K; k++) t[k] = s[k];
  for (int m = 1; m < K; m++)
    for (int k = 0; k + m < K; k++)
      t[k] = (h[k + m] * t[k] - h[k] * t[k + 1]) / (h[k + m] - h[k]);
  return t[0];
}

/* Romberg integral of f[0..m] with spacing hh (DEALII_SCFT/src/romint.c:21-57):
   trapezoid sums on 1,2,4,..,m intervals, the last K=5 extrapolated to h->0 in
   the variable h_j = 4^-(j-1).  m must be a power of two >= 16; returns NaN
   otherwise (the reference exits, romint.c:29-33). */
double or_romint(const double *f, int m, double hh) {
  int levels = 1;
  while ((1 << (levels - 1)) < m) levels++;
  if ((1 << (levels - 1)) != m || levels < 5 || levels > 30) return NAN;
  double s[32], h[32];
  h[0] = 1.0;
  s[0] = m * hh * (f[0] + f[m]) / 2.0;
  int np = 1;
  for (int j = 1; j < levels; j++) {
    int ii = m / np;
    double sum = 0.0;
    for (int i = ii / 2; i < m; i += ii) sum += f[i];
    s[j] = (s[j - 1] + ii * hh * sum) / 2.0;
    np += np;
    h[j] = h[j - 1] / 4.0;
  }
  return neville_at_zero(&h[levels - 5], &s[levels - 5], 5);
}

/* Quadrature weights W[0..nsteps] such that rule(v) = sum_k W_k v_k.
   Romberg is linear in the samples, so its weights follow from the trapezoid
   level weights and the Lagrange coefficients at h=0 of the 5-point Neville
   extrapolation.  Trapezoid: simple_FEM_1D_transient.m:119-124. */
int or_quad_weights(int nsteps, double ds, int rule, double *W) {
  if (rule == OR_RULE_TRAPEZOID) {
    for (int k = 0; k <= nsteps; k++) W[k] = ds;
    W[0] = W[nsteps] = 0.5 * ds;
    return 0;
  }
  int levels = 1;
  while ((1 << (levels - 1)) < nsteps) levels++;
  if ((1 << (levels - 1)) != nsteps || levels < 5) return -1;
  for (int k = 0; k <= nsteps; k++) W[k] = 0.0;
  double h[5];
  for (int a = 0; a < 5; a++) h[a] = pow(0.25, (double)(levels - 5 + a));
  for (int a = 0; a < 5; a++) {
    double c = 1.0;
    for (int b = 0; b < 5; b++)
      if (b != a) c *= (0.0 - h[b]) / (h[a] - h[b]);
    int j = levels - 5 + a;             /* 0-based level: 2^j intervals */
    int stride = nsteps >> j;
    double H = stride * ds;
    for (int k = 0; k <= nsteps; k += stride)
      W[k] += c * H * ((k == 0 || k == nsteps) ? 0.5 : 1.0);
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* FEM system                                                                */
/* ------------------------------------------------------------------------- */

/* Tridiagonal bands on the N = n-2 interior unknowns (unknown j = node j+1).
   Mass / stiffness on a nonuniform mesh: simple_FEM_1D_transient.m:34-63
   (uniform case 1D_FEM.c:95-98).  Field term:
     row-scaled  W_ij = w_i M_ij             1D_FEM.c:104-105, .m:66-70
     consistent  W_ij = int w_h phi_i phi_j  scft.cc:653-655 (exact for P1 w_h)  */
typedef struct {
  int N;
  double *ml, *md, *mu; /* mass */
  double *al, *ad, *au; /* stiffness + field (K + W) */
} bands;

static int bands_build(const or_problem *p, const double *w, bands *B) {
  int n = p->n, N = n - 2;
  if (N < 1) return -1;
  B->N = N;
  double *mem = (double *)malloc(sizeof(double) * 6 * (size_t)N);
  if (!mem) return -2;
  B->ml = mem; B->md = mem + N; B->mu = mem + 2 * N;
  B->al = mem + 3 * N; B->ad = mem + 4 * N; B->au = mem + 5 * N;
  for (int j = 0; j < N; j++) {
    int i = j + 1;
    double a1 = p->x[i] - p->x[i - 1], a2 = p->x[i + 1] - p->x[i];
    B->ml[j] = a1 / 6.0;
    B->md[j] = a1 / 3.0 + a2 / 3.0;
    B->mu[j] = a2 / 6.0;
    double kl = -1.0 / a1, kd = 1.0 / a1 + 1.0 / a2, ku = -1.0 / a2;
    if (p->wmode == OR_W_CONSISTENT) {
      double wl = w[i - 1], wc = w[i], wr = w[i + 1];
      B->al[j] = kl + a1 * (wl + wc) / 12.0;
      B->ad[j] = kd + a1 * (wl + 3.0 * wc) / 12.0 + a2 * (3.0 * wc + wr) / 12.0;
      B->au[j] = ku + a2 * (wc + wr) / 12.0;
    } else {
      B->al[j] = kl + w[i] * B->ml[j];
      B->ad[j] = kd + w[i] * B->md[j];
      B->au[j] = ku + w[i] * B->mu[j];
    }
  }
  return 0;
}

static void bands_free(bands *B) { free(B->ml); }

/* y = T x for a tridiagonal T (zero Dirichlet values outside 0..N-1). */
static void tri_mul(int N, const double *l, const double *d, const double *u,
                    const double *x, double *y) {
  for (int j = 0; j < N; j++) {
    double v = d[j] * x[j];
    if (j > 0) v += l[j] * x[j - 1];
    if (j < N - 1) v += u[j] * x[j + 1];
    y[j] = v;
  }
}

/* ------------------------------------------------------------------------- */
/* contour stepping                                                          */
/* ------------------------------------------------------------------------- */

/* Implicit Euler: (M + ds(K+W)) q_{k+1} = M q_k, Dirichlet rows removed
   (1D_FEM.c:177-186, 212-215; .m:74-91).  Factored once by Thomas. */
typedef struct {
  int N;
  double *ml, *md, *mu; /* rhs bands (mass) */
  double *dl, *cp, *inv; /* factored D: sub-band, modified super, 1/pivot */
  double *rhs;
} ie_solver;

static int ie_init(ie_solver *S, const bands *B, double ds) {
  int N = B->N;
  S->N = N;
  S->ml = B->ml; S->md = B->md; S->mu = B->mu;
  double *mem = (double *)malloc(sizeof(double) * 4 * (size_t)N);
  if (!mem) return -2;
  S->dl = mem; S->cp = mem + N; S->inv = mem + 2 * N; S->rhs = mem + 3 * N;
  for (int j = 0; j < N; j++) {
    double l = B->ml[j] + ds * B->al[j];
    double d = B->md[j] + ds * B->ad[j];
    double u = B->mu[j] + ds * B->au[j];
    double piv = d - (j > 0 ? l * S->cp[j - 1] : 0.0);
    S->dl[j] = l;
    S->inv[j] = 1.0 / piv;
    S->cp[j] = u * S->inv[j];
  }
  return 0;
}

static void ie_step(ie_solver *S, const double *q, double *qn) {
  int N = S->N;
  tri_mul(N, S->ml, S->md, S->mu, q, S->rhs);
  double prev = 0.0;
  for (int j = 0; j < N; j++) {
    prev = (S->rhs[j] - (j > 0 ? S->dl[j] * prev : 0.0)) * S->inv[j];
    qn[j] = prev;
  }
  for (int j = N - 2; j >= 0; j--) qn[j] -= S->cp[j] * qn[j + 1];
}

static void ie_free(ie_solver *S) { free(S->dl); }

/* Gauss-Legendre 2-stage implicit Runge-Kutta on M dq/ds = -(K+W) q
   (drivescft.cc:130-146, block system scft.cc:668-695):
     [M + ds/4 D, c01 D; c10 D, M + ds/4 D] [k1;k2] = [-D q; -D q],
     q' = q + ds/2 (k1 + k2),  c01 = (1/4 - sqrt3/6) ds, c10 = (1/4 + sqrt3/6) ds.
   Solved as a block-tridiagonal system with 2x2 blocks (block Thomas). */
typedef struct {
  int N;
  double ds;
  const bands *B;
  double *G;    /* 4 per unknown: S_j^{-1} B_{j,j+1} */
  double *Sinv; /* 4 per unknown */
  double *L;    /* 4 per unknown: sub-diagonal block */
  double *r, *y, *k;
} irk_solver;

static void blk(const bands *B, double ds, int j, int which, double out[4]) {
  double c01 = (0.25 - sqrt(3.0) / 6.0) * ds, c10 = (0.25 + sqrt(3.0) / 6.0) * ds;
  double m, a;
  if (which < 0) { m = B->ml[j]; a = B->al[j]; }
  else if (which == 0) { m = B->md[j]; a = B->ad[j]; }
  else { m = B->mu[j]; a = B->au[j]; }
  out[0] = m + 0.25 * ds * a; out[1] = c01 * a;
  out[2] = c10 * a;           out[3] = m + 0.25 * ds * a;
}
static void m2_mul(const double a[4], const double b[4], double c[4]) {
  double t0 = a[0] * b[0] + a[1] * b[2], t1 = a[0] * b[1] + a[1] * b[3];
  double t2 = a[2] * b[0] + a[3] * b[2], t3 = a[2] * b[1] + a[3] * b[3];
  c[0] = t0; c[1] = t1; c[2] = t2; c[3] = t3;
}
static void m2_inv(const double a[4], double c[4]) {
  double det = a[0] * a[3] - a[1] * a[2];
  c[0] = a[3] / det; c[1] = -a[1] / det; c[2] = -a[2] / det; c[3] = a[0] / det;
}

static int irk_init(irk_solver *S, const bands *B, double ds) {
  int N = B->N;
  S->N = N; S->ds = ds; S->B = B;
  double *mem = (double *)malloc(sizeof(double) * (12 * (size_t)N + 6 * (size_t)N));
  if (!mem) return -2;
  S->G = mem; S->Sinv = mem + 4 * N; S->L = mem + 8 * N;
  S->r = mem + 12 * N; S->y = mem + 14 * N; S->k = mem + 16 * N;
  double prevG[4] = {0, 0, 0, 0};
  for (int j = 0; j < N; j++) {
    double Dd[4], Lb[4], Ub[4], t[4], Sj[4];
    blk(B, ds, j, 0, Dd);
    blk(B, ds, j, -1, Lb);
    blk(B, ds, j, +1, Ub);
    if (j > 0) {
      m2_mul(Lb, prevG, t);
      for (int a = 0; a < 4; a++) Sj[a] = Dd[a] - t[a];
    } else {
      for (int a = 0; a < 4; a++) Sj[a] = Dd[a];
    }
    m2_inv(Sj, &S->Sinv[4 * j]);
    m2_mul(&S->Sinv[4 * j], Ub, &S->G[4 * j]);
    for (int a = 0; a < 4; a++) { S->L[4 * j + a] = Lb[a]; prevG[a] = S->G[4 * j + a]; }
  }
  return 0;
}


static void irk_step(irk_solver *S, const double *q, double *qn) {
  int N = S->N;
  const bands *B = S->B;
  /* r_j = -(K+W) q, identical for both stages */
  for (int j = 0; j < N; j++) {
    double v = B->ad[j] * q[j];
    if (j > 0) v += B->al[j] * q[j - 1];
    if (j < N - 1) v += B->au[j] * q[j + 1];
    S->r[2 * j] = -v;
    S->r[2 * j + 1] = -v;
  }
  /* forward: y_j = S_j^{-1} (r_j - L_j y_{j-1}) */
  for (int j = 0; j < N; j++) {
    double t0 = S->r[2 * j], t1 = S->r[2 * j + 1];
    if (j > 0) {
      const double *L = &S->L[4 * j];
      t0 -= L[0] * S->y[2 * j - 2] + L[1] * S->y[2 * j - 1];
      t1 -= L[2] * S->y[2 * j - 2] + L[3] * S->y[2 * j - 1];
    }
    const double *Si = &S->Sinv[4 * j];
    S->y[2 * j] = Si[0] * t0 + Si[1] * t1;
    S->y[2 * j + 1] = Si[2] * t0 + Si[3] * t1;
  }
  /* backward: k_j = y_j - G_j k_{j+1} */
  for (int j = N - 1; j >= 0; j--) {
    double k0 = S->y[2 * j], k1 = S->y[2 * j + 1];
    if (j < N - 1) {
      const double *G = &S->G[4 * j];
      k0 -= G[0] * S->k[2 * j + 2] + G[1] * S->k[2 * j + 3];
      k1 -= G[2] * S->k[2 * j + 2] + G[3] * S->k[2 * j + 3];
    }
    S->k[2 * j] = k0;
    S->k[2 * j + 1] = k1;
  }
  for (int j = 0; j < N; j++) qn[j] = q[j] + 0.5 * S->ds * (S->k[2 * j] + S->k[2 * j + 1]);
}

static void irk_free(irk_solver *S) { free(S->G); }

/* ------------------------------------------------------------------------- */
/* propagator: q(x,s), phi(x) = int_0^1 q(x,s) q(x,1-s) ds, Q                 */
/* ------------------------------------------------------------------------- */

#define OR_FULL_STORE_LIMIT ((size_t)1 << 25) /* doubles kept when all slices are stored */

/* Propagator and density of one field (1D_FEM.c:47-272; .m:1-124;
   drivescft.cc:81-207).  q(.,0) = 1 on interior nodes, 0 on the walls
   (1D_FEM.c:114-128).  phi_i applies the quadrature rule to
   v_k = q_k,i q_{nsteps-k},i (1D_FEM.c:262-272 pairs k with nsteps-k; the .m
   with time_step-k, i.e. the same pairing over nsteps=2049).  When all slices
   fit (nsteps+1)*N <= 2^25 the rule is applied per node exactly as the
   reference does (romint over the v array); otherwise the linear weights of
   or_quad_weights are accumulated from a half store. */
int or_propagate(const or_problem *p, const double *w, double *phi, double *Q, double *q_store) {
  int n = p->n, N = n - 2, ns = p->nsteps;
  if (N < 1 || ns < 1) return -1;
  if (p->rule == OR_RULE_ROMBERG) {
    int lv = 1;
    while ((1 << (lv - 1)) < ns) lv++;
    if ((1 << (lv - 1)) != ns || lv < 5) return -3;
  }
  bands B;
  if (bands_build(p, w, &B)) return -2;
  ie_solver ie;
  irk_solver irk;
  memset(&ie, 0, sizeof ie);
  memset(&irk, 0, sizeof irk);
  int rc = (p->scheme == OR_SCHEME_IRK2) ? irk_init(&irk, &B, p->ds) : ie_init(&ie, &B, p->ds);
  if (rc) { bands_free(&B); return rc; }

  size_t full = (size_t)(ns + 1) * (size_t)N;
  int exact = full <= OR_FULL_STORE_LIMIT;
  int half = ns / 2;
  size_t kept = exact ? full : (size_t)(half + 1) * (size_t)N;
  double *store = (double *)malloc(sizeof(double) * kept);
  double *W = (double *)malloc(sizeof(double) * (size_t)(ns + 1));
  double *acc = (double *)calloc((size_t)N, sizeof(double));
  double *qa = (double *)malloc(sizeof(double) * (size_t)N);
  double *qb = (double *)malloc(sizeof(double) * (size_t)N);
  if (!store || !W || !acc || !qa || !qb) { rc = -2; goto done; }
  or_quad_weights(ns, p->ds, p->rule, W);

  for (int j = 0; j < N; j++) qa[j] = 1.0;
  memcpy(store, qa, sizeof(double) * N);
  for (int k = 1; k <= ns; k++) {
    if (p->scheme == OR_SCHEME_IRK2) irk_step(&irk, qa, qb);
    else ie_step(&ie, qa, qb);
    double *t = qa; qa = qb; qb = t;
    if (exact || k <= half) memcpy(store + (size_t)k * N, qa, sizeof(double) * N);
    if (!exact && k >= ns - half) {
      /* pair (k, ns-k): both members carry weight W_k = W_{ns-k} */
      const double *qo = store + (size_t)(ns - k) * N;
      double wk = (k == ns - k) ? W[k] : 2.0 * W[k];
      for (int j = 0; j < N; j++) acc[j] += wk * qa[j] * qo[j];
    }
  }
  if (q_store && exact) {
    for (int k = 0; k <= ns; k++) {
      q_store[(size_t)k * n] = 0.0;
      memcpy(q_store + (size_t)k * n + 1, store + (size_t)k * N, sizeof(double) * N);
      q_store[(size_t)k * n + n - 1] = 0.0;
    }
  }
  phi[0] = phi[n - 1] = 0.0;
  if (exact) {
    double *v = (double *)malloc(sizeof(double) * (size_t)(ns + 1));
    if (!v) { rc = -2; goto done; }
    for (int j = 0; j < N; j++) {
      for (int k = 0; k <= ns; k++) v[k] = store[(size_t)k * N + j] * store[(size_t)(ns - k) * N + j];
      double s;
      if (p->rule == OR_RULE_ROMBERG) {
        s = or_romint(v, ns, p->ds);
      } else {
        s = 0.0;
        for (int k = 0; k < ns; k++) s += 0.5 * (v[k] + v[k + 1]) * p->ds;
      }
      phi[j + 1] = s;
    }
    free(v);
  } else {
    for (int j = 0; j < N; j++) phi[j + 1] = acc[j];
  }
  if (Q) {
    /* Q = (1/L) int q(x,1) dx = (1/L) 1^T M q  (mass row sums (a1+a2)/2) */
    double s = 0.0;
    for (int j = 0; j < N; j++) s += 0.5 * (p->x[j + 2] - p->x[j]) * qa[j];
    *Q = s / (p->x[n - 1] - p->x[0]);
  }
  rc = 0;
done:
  free(store); free(W); free(acc); free(qa); free(qb);
  if (p->scheme == OR_SCHEME_IRK2) irk_free(&irk); else ie_free(&ie);
  bands_free(&B);
  return rc;
}

/* Residual on interior nodes (1D_FEM.c:274-277: out = phi - f0;
   drivescft.cc:210-215: out = f0 - phi).  w_int holds the n-2 interior values;
   wall values are 0 (1D_FEM.c:65-66) unless p->wall_w supplies them. */
int or_residual(const or_problem *p, const double *w_int, double *out, double *phi_out) {
  int n = p->n;
  double *w = (double *)malloc(sizeof(double) * (size_t)n);
  double *phi = phi_out ? phi_out : (double *)malloc(sizeof(double) * (size_t)n);
  if (!w || !phi) { free(w); if (!phi_out) free(phi); return -2; }
  w[0] = p->wall_w ? p->wall_w[0] : 0.0;
  w[n - 1] = p->wall_w ? p->wall_w[1] : 0.0;
  memcpy(w + 1, w_int, sizeof(double) * (size_t)(n - 2));
  int rc = or_propagate(p, w, phi, NULL, NULL);
  if (rc == 0) {
    double sg = p->sign >= 0 ? 1.0 : -1.0;
    for (int i = 1; i < n - 1; i++) out[i - 1] = sg * (phi[i] - p->f0[i]);
  }
  free(w);
  if (!phi_out) free(phi);
  return rc;
}

void or_problem_vecfunc(int n, const double *x, double *out, void *ctx) {
  (void)n;
  or_residual((const or_problem *)ctx, x, out, NULL);
}

/* ------------------------------------------------------------------------- */
/* Gauss-Jordan elimination with full pivoting                               */
/* ------------------------------------------------------------------------- */

/* Solves a X = b in place (a -> a^{-1}, b -> X) with full pivoting, choosing
   the last largest |a_jk| in row-major scan order among unpivoted rows and
   columns, as gaussj.c:7-60 does.  Zero pivot: mode 0 adds 1e-18
   (gaussj.c:38), mode 1 returns 1 (DEALII_SCFT/src/gaussj.c:45-50). */
int or_gaussj(double *a, int n, double *b, int m, int singular_mode) {
  if (n <= 0) return 0;
  int *ipiv = (int *)calloc((size_t)n * 3, sizeof(int));
  if (!ipiv) return 2;
  int *indxr = ipiv + n, *indxc = ipiv + 2 * n;
  for (int i = 0; i < n; i++) {
    double big = 0.0;
    int irow = 0, icol = 0;
    for (int j = 0; j < n; j++) {
      if (ipiv[j] == 1) continue;
      for (int k = 0; k < n; k++) {
        if (ipiv[k] != 0) continue;
        double v = fabs(a[j * n + k]);
        if (v >= big) { big = v; irow = j; icol = k; }
      }
    }
    ipiv[icol]++;
    if (irow != icol) {
      for (int l = 0; l < n; l++) { double t = a[irow * n + l]; a[irow * n + l] = a[icol * n + l]; a[icol * n + l] = t; }
      for (int l = 0; l < m; l++) { double t = b[irow * m + l]; b[irow * m + l] = b[icol * m + l]; b[icol * m + l] = t; }
    }
    indxr[i] = irow;
    indxc[i] = icol;
    if (a[icol * n + icol] == 0.0) {
      if (singular_mode == 1) { free(ipiv); return 1; }
      a[icol * n + icol] += 1e-18;
    }
    double pinv = 1.0 / a[icol * n + icol];
    a[icol * n + icol] = 1.0;
    for (int l = 0; l < n; l++) a[icol * n + l] *= pinv;
    for (int l = 0; l < m; l++) b[icol * m + l] *= pinv;
    for (int r = 0; r < n; r++) {
      if (r == icol) continue;
      double f = a[r * n + icol];
      a[r * n + icol] = 0.0;
      for (int l = 0; l < n; l++) a[r * n + l] -= a[icol * n + l] * f;
      for (int l = 0; l < m; l++) b[r * m + l] -= b[icol * m + l] * f;
    }
  }
  for (int l = n - 1; l >= 0; l--) {
    if (indxr[l] == indxc[l]) continue;
    for (int k = 0; k < n; k++) {
      double t = a[k * n + indxr[l]]; a[k * n + indxr[l]] = a[k * n + indxc[l]]; a[k * n + indxc[l]] = t;
    }
  }
  free(ipiv);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Anderson mixing, residual form (ADM_chen_C.c:18-147)                      */
/* ------------------------------------------------------------------------- */

/* History is a ring of depth min(nn,n)+1 (the reference keeps every iterate;
   only the last nm+1 are ever read).  Sums run in the reference's order so the
   iterates agree with it to rounding. */
int or_adm_chen(or_vecfunc f, void *ctx, double *x, double tol, int maxit, int n,
                double lmd, int nn, int final_, int *iters, double *trace) {
  int nm = nn < n ? nn : n;
  int depth = nm + 1;
  double *X = (double *)malloc(sizeof(double) * (size_t)depth * n);
  double *Y = (double *)malloc(sizeof(double) * (size_t)depth * n);
  double *U = (double *)malloc(sizeof(double) * (size_t)(nm * nm + nm + 1));
  double *xn = (double *)malloc(sizeof(double) * (size_t)n);
  if (!X || !Y || !U || !xn) { free(X); free(Y); free(U); free(xn); return 3; }
  double *V = U + nm * nm;
  double lk = lmd;
  int k = 0, krestart = 0, rc = 1;
  memcpy(X, x, sizeof(double) * n);
#define XR(kk) (X + (size_t)((kk) % depth) * n)
#define YR(kk) (Y + (size_t)((kk) % depth) * n)
  while (k <= maxit) {
    double *Xk = XR(k), *Yk = YR(k);
    f(n, Xk, Yk, ctx);
    double err = 0.0;
    int bad = 0;
    for (int i = 0; i < n; i++) {
      if (isnan(Yk[i])) { bad = 1; break; }
      if (fabs(Yk[i]) >= err) err = fabs(Yk[i]);
    }
    if (bad) { memcpy(x, Xk, sizeof(double) * n); rc = 2; goto out; }
    if (trace) trace[k] = err;
    if (err < tol) { memcpy(x, Xk, sizeof(double) * n); rc = 0; goto out; }
    int m;
    for (;;) {
      m = nm < (k - krestart) ? nm : (k - krestart);
      for (int i = 0; i < m; i++) {
        const double *Yi = YR(k - i - 1);
        for (int j = 0; j < m; j++) {
          const double *Yj = YR(k - j - 1);
          double s = 0.0;
          for (int t = 0; t < n; t++) s += (Yk[t] - Yi[t]) * (Yk[t] - Yj[t]);
          U[i * m + j] = s;
        }
        double s = 0.0;
        for (int t = 0; t < n; t++) s += (Yk[t] - Yi[t]) * Yk[t];
        V[i] = s;
      }
      if (or_gaussj(U, m, V, 1, 1) == 1) { krestart = k; lk = lmd; continue; }
      break;
    }
    for (int i = 0; i < n; i++) {
      double cx = 0.0, cd = 0.0;
      for (int j = 0; j < m; j++) {
        cx += V[j] * (XR(k - j - 1)[i] - Xk[i]);
        cd += V[j] * (YR(k - j - 1)[i] - Yk[i]);
      }
      xn[i] = Xk[i] + cx + (1.0 - lk) * (Yk[i] + cd);
    }
    memcpy(XR(k + 1), xn, sizeof(double) * n);
    if (err < 0.03 && k > 100) lk *= lmd;
    if (!final_ && lk < 1e-5) lk = lmd;
    if (final_ && lk < 1e-15) lk = lmd;
    k++;
  }
  memcpy(x, XR(k), sizeof(double) * n);
  rc = 1;
out:
#undef XR
#undef YR
  if (iters) *iters = k;
  free(X); free(Y); free(U); free(xn);
  return rc;
}

/* ------------------------------------------------------------------------- */
/* Anderson mixing, fixed-point ring form (adm.c:24-313)                      */
/* ------------------------------------------------------------------------- */

#define OR_ADM_NRMAX 10

/* x = g(x).  First step x <- x + 0.05 (g(x)-x) (adm.c:103-146); then with
   lambda = 1 - 0.95^its the Anderson update over the nr = min(its-1, 10)
   other slots of an 11-slot ring (adm.c:148-306).  The unknown ordering of the
   small system follows adm.c:232-276 so full pivoting picks the same pivots. */
int or_adm(or_vecfunc g, void *ctx, double *x, int n, double tol, int maxit, int *iters) {
  const int S = OR_ADM_NRMAX + 1;
  double *xh = (double *)malloc(sizeof(double) * (size_t)S * n);
  double *dh = (double *)malloc(sizeof(double) * (size_t)S * n);
  double *xn = (double *)malloc(sizeof(double) * (size_t)n);
  double u[OR_ADM_NRMAX * OR_ADM_NRMAX], b[OR_ADM_NRMAX];
  int slot_of[OR_ADM_NRMAX];
  int rc = 1, its = 1;
  if (!xh || !dh || !xn) { rc = 3; goto out; }
  g(n, x, xn, ctx);
  double err = 0.0;
  for (int i = 0; i < n; i++) {
    xh[i] = x[i];
    dh[i] = xn[i] - x[i];
    if (fabs(dh[i]) > err) err = fabs(dh[i]);
  }
  if (err < tol) { rc = 0; goto out; }
  int nc = 1;
  for (int i = 0; i < n; i++) x[i] = xh[i] + 0.05 * dh[i];
  for (its = 2; its <= maxit; its++) {
    int nr = its - 1 < OR_ADM_NRMAX ? its - 1 : OR_ADM_NRMAX;
    double lambda = 1.0 - pow(0.95, its);
    g(n, x, xn, ctx);
    if (nc == S) nc = 0;
    int cur = nc;
    double *xc = xh + (size_t)cur * n, *dc = dh + (size_t)cur * n;
    err = 0.0;
    for (int i = 0; i < n; i++) {
      dc[i] = xn[i] - x[i];
      xc[i] = x[i];
      if (fabs(dc[i]) > err) err = fabs(dc[i]);
    }
    nc++;
    if (err < tol) { rc = 0; goto out; }
    /* unknown a -> ring slot: first the slots below cur (ascending), then the
       slots above cur up to nr (descending) */
    int a = 0;
    for (int s = 0; s < cur; s++) slot_of[a++] = s;
    for (int s = nr; s > cur; s--) slot_of[a++] = s;
    for (int p = 0; p < nr; p++) {
      const double *dp = dh + (size_t)slot_of[p] * n;
      for (int q = p; q < nr; q++) {
        const double *dq = dh + (size_t)slot_of[q] * n;
        double s = 0.0;
        for (int i = 0; i < n; i++) s += (dc[i] - dp[i]) * (dc[i] - dq[i]);
        u[p * nr + q] = u[q * nr + p] = s;
      }
      double s = 0.0;
      for (int i = 0; i < n; i++) s += (dc[i] - dp[i]) * dc[i];
      b[p] = s;
    }
    or_gaussj(u, nr, b, 1, 0);
    for (int i = 0; i < n; i++) {
      double t = 0.0, t1 = 0.0;
      for (int p = 0; p < nr; p++) {
        const double *xp = xh + (size_t)slot_of[p] * n, *dp = dh + (size_t)slot_of[p] * n;
        t += b[p] * (xp[i] - xc[i]);
        t1 += b[p] * (dp[i] - dc[i]);
      }
      x[i] = xc[i] + t + lambda * (dc[i] + t1);
    }
  }
  rc = 1;
out:
  if (iters) *iters = its;
  free(xh); free(dh); free(xn);
  return rc;
}

/* ------------------------------------------------------------------------- */
/* Broyden with QR updates and backtracking (broydn.c:44-292 + NR helpers)   */
/* ------------------------------------------------------------------------- */

typedef struct {
  or_vecfunc f;
  void *ctx;
  int n;
  double *fvec;
  int nfev;
} br_state;

/* 0.5 |F|^2 (broydn.c:30-42) */
static double br_fmin(br_state *st, const double *x) {
  st->f(st->n, x, st->fvec, st->ctx);
  st->nfev++;
  double s = 0.0;
  for (int i = 0; i < st->n; i++) s += st->fvec[i] * st->fvec[i];
  return 0.5 * s;
}

/* forward-difference Jacobian, relative step 1e-7 (fdjac.c:10-41); df row-major */
static void br_fdjac(br_state *st, double *x, const double *fv, double *df, double *ftmp) {
  int n = st->n;
  for (int j = 0; j < n; j++) {
    double temp = x[j], h = 1e-7 * temp;
    if (fabs(h) < 1e-7) h = temp >= 0.0 ? 1e-7 : -1e-7;
    x[j] = temp + h;
    h = x[j] - temp;
    st->f(n, x, ftmp, st->ctx);
    st->nfev++;
    x[j] = temp;
    for (int i = 0; i < n; i++) df[i * n + j] = (ftmp[i] - fv[i]) / h;
  }
}

/* Householder QR, R's diagonal in d, reflector norms in c (qrdcmp.c:6-34). */
static int br_qrdcmp(double *a, int n, double *c, double *d) {
  int sing = 0;
  for (int k = 0; k < n - 1; k++) {
    double scale = 0.0;
    for (int i = k; i < n; i++) scale = fmax(scale, fabs(a[i * n + k]));
    if (scale == 0.0) { sing = 1; c[k] = d[k] = 0.0; continue; }
    for (int i = k; i < n; i++) a[i * n + k] /= scale;
    double sum = 0.0;
    for (int i = k; i < n; i++) sum += a[i * n + k] * a[i * n + k];
    double sigma = a[k * n + k] >= 0.0 ? fabs(sqrt(sum)) : -fabs(sqrt(sum));
    a[k * n + k] += sigma;
    c[k] = sigma * a[k * n + k];
    d[k] = -scale * sigma;
    for (int j = k + 1; j < n; j++) {
      double s = 0.0;
      for (int i = k; i < n; i++) s += a[i * n + k] * a[i * n + j];
      double tau = s / c[k];
      for (int i = k; i < n; i++) a[i * n + j] -= tau * a[i * n + k];
    }
  }
  d[n - 1] = a[(n - 1) * n + n - 1];
  if (d[n - 1] == 0.0) sing = 1;
  return sing;
}

/* Givens rotation of rows i,i+1 of r and qt (rotate.c:6-35). */
static void br_rotate(double *r, double *qt, int n, int i, double a, double b) {
  double c, s;
  if (a == 0.0) { c = 0.0; s = b >= 0.0 ? 1.0 : -1.0; }
  else if (fabs(a) > fabs(b)) {
    double fact = b / a;
    c = (a >= 0.0 ? 1.0 : -1.0) * fabs(1.0 / sqrt(1.0 + fact * fact));
    s = fact * c;
  } else {
    double fact = a / b;
    s = (b >= 0.0 ? 1.0 : -1.0) * fabs(1.0 / sqrt(1.0 + fact * fact));
    c = fact * s;
  }
  for (int j = i; j < n; j++) {
    double y = r[i * n + j], w = r[(i + 1) * n + j];
    r[i * n + j] = c * y - s * w;
    r[(i + 1) * n + j] = s * y + c * w;
  }
  for (int j = 0; j < n; j++) {
    double y = qt[i * n + j], w = qt[(i + 1) * n + j];
    qt[i * n + j] = c * y - s * w;
    qt[(i + 1) * n + j] = s * y + c * w;
  }
}

/* rank-1 update R + u v^T re-triangularised by rotations (qrupdt.c:6-24) */
static void br_qrupdt(double *r, double *qt, int n, double *u, const double *v) {
  int k;
  for (k = n - 1; k >= 0; k--) if (u[k] != 0.0) break;
  if (k < 0) k = 0;
  for (int i = k - 1; i >= 0; i--) {
    br_rotate(r, qt, n, i, u[i], -u[i + 1]);
    if (u[i] == 0.0) u[i] = fabs(u[i + 1]);
    else if (fabs(u[i]) > fabs(u[i + 1])) u[i] = fabs(u[i]) * sqrt(1.0 + (u[i + 1] / u[i]) * (u[i + 1] / u[i]));
    else u[i] = fabs(u[i + 1]) * sqrt(1.0 + (u[i] / u[i + 1]) * (u[i] / u[i + 1]));
  }
  for (int j = 0; j < n; j++) r[j] += u[0] * v[j];
  for (int i = 0; i < k; i++) br_rotate(r, qt, n, i, r[i * n + i], -r[(i + 1) * n + i]);
}

/* Backtracking line search along p (lnsrch.c:8-61).  Returns 0 ok, 1 step
   too small (x = xold), 3 roundoff (slope >= 0; the reference exits). */
static int br_lnsrch(br_state *st, const double *xold, double fold, const double *g, double *p,
                     double *x, double *f, double stpmax) {
  int n = st->n;
  double sum = 0.0;
  for (int i = 0; i < n; i++) sum += p[i] * p[i];
  sum = sqrt(sum);
  if (sum > stpmax) for (int i = 0; i < n; i++) p[i] *= stpmax / sum;
  double slope = 0.0;
  for (int i = 0; i < n; i++) slope += g[i] * p[i];
  if (slope >= 0.0) return 3;
  double test = 0.0;
  for (int i = 0; i < n; i++) {
    double t = fabs(p[i]) / fmax(fabs(xold[i]), 1.0);
    if (t > test) test = t;
  }
  double alamin = 1e-7 / test, alam = 1.0, alam2 = 0.0, f2 = 0.0, tmplam;
  for (;;) {
    for (int i = 0; i < n; i++) x[i] = xold[i] + alam * p[i];
    *f = br_fmin(st, x);
    if (alam < alamin) {
      for (int i = 0; i < n; i++) x[i] = xold[i];
      return 1;
    }
    if (*f <= fold + 1e-4 * alam * slope) return 0;
    if (alam == 1.0) {
      tmplam = -slope / (2.0 * (*f - fold - slope));
    } else {
      double rhs1 = *f - fold - alam * slope, rhs2 = f2 - fold - alam2 * slope;
      double a = (rhs1 / (alam * alam) - rhs2 / (alam2 * alam2)) / (alam - alam2);
      double b = (-alam2 * rhs1 / (alam * alam) + alam * rhs2 / (alam2 * alam2)) / (alam - alam2);
      if (a == 0.0) tmplam = -slope / (2.0 * b);
      else {
        double disc = b * b - 3.0 * a * slope;
        if (disc < 0.0) tmplam = 0.5 * alam;
        else if (b <= 0.0) tmplam = (-b + sqrt(disc)) / (3.0 * a);
        else tmplam = -slope / (b + sqrt(disc));
      }
      if (tmplam > 0.5 * alam) tmplam = 0.5 * alam;
    }
    alam2 = alam;
    f2 = *f;
    alam = fmax(tmplam, 0.1 * alam);
  }
}

int or_broydn(or_vecfunc fn, void *ctx, double *x, int n, double tol, int *iters, int *nfev) {
  const int MAXITS = 400;
  const double EPS = 1e-14, TOLX = 1e-14, STPMX = 100.0;
  size_t nn = (size_t)n * n;
  double *mem = (double *)malloc(sizeof(double) * (2 * nn + 13 * (size_t)n));
  if (!mem) return 4;
  double *qt = mem, *r = mem + nn, *c = r + nn, *d = c + n, *fvcold = d + n, *g = fvcold + n,
         *p = g + n, *s = p + n, *t = s + n, *w = t + n, *xold = w + n, *fvec = xold + n,
         *ftmp = fvec + n, *uu = ftmp + n;
  (void)uu;
  br_state st = {fn, ctx, n, fvec, 0};
  int rc = 1, its = 0, restrt = 1;
  double f = br_fmin(&st, x), err = 0.0;
  for (int i = 0; i < n; i++) err = fmax(err, fabs(fvec[i]));
  if (err < tol) { rc = 0; goto out; }
  double sum = 0.0;
  for (int i = 0; i < n; i++) sum += x[i] * x[i];
  double stpmax = STPMX * fmax(sqrt(sum), (double)n);
  for (its = 1; its <= MAXITS; its++) {
    if (restrt) {
      br_fdjac(&st, x, fvec, r, ftmp);
      if (br_qrdcmp(r, n, c, d)) { rc = 2; goto out; }
      for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) qt[i * n + j] = (i == j) ? 1.0 : 0.0;
      for (int k = 0; k < n - 1; k++) {
        if (c[k] == 0.0) continue;
        for (int j = 0; j < n; j++) {
          double sm = 0.0;
          for (int i = k; i < n; i++) sm += r[i * n + k] * qt[i * n + j];
          sm /= c[k];
          for (int i = k; i < n; i++) qt[i * n + j] -= sm * r[i * n + k];
        }
      }
      for (int i = 0; i < n; i++) {
        r[i * n + i] = d[i];
        for (int j = 0; j < i; j++) r[i * n + j] = 0.0;
      }
    } else if (its > 1) {
      for (int i = 0; i < n; i++) s[i] = x[i] - xold[i];
      for (int i = 0; i < n; i++) {
        double sm = 0.0;
        for (int j = i; j < n; j++) sm += r[i * n + j] * s[j];
        t[i] = sm;
      }
      int skip = 1;
      for (int i = 0; i < n; i++) {
        double sm = 0.0;
        for (int j = 0; j < n; j++) sm += qt[j * n + i] * t[j];
        w[i] = fvec[i] - fvcold[i] - sm;
        if (fabs(w[i]) >= EPS * (fabs(fvec[i]) + fabs(fvcold[i]))) skip = 0;
        else w[i] = 0.0;
      }
      if (!skip) {
        for (int i = 0; i < n; i++) {
          double sm = 0.0;
          for (int j = 0; j < n; j++) sm += qt[i * n + j] * w[j];
          t[i] = sm;
        }
        double den = 0.0;
        for (int i = 0; i < n; i++) den += s[i] * s[i];
        for (int i = 0; i < n; i++) s[i] /= den;
        br_qrupdt(r, qt, n, t, s);
        for (int i = 0; i < n; i++) {
          if (r[i * n + i] == 0.0) { rc = 2; goto out; }
          d[i] = r[i * n + i];
        }
      }
    }
    for (int i = 0; i < n; i++) {
      double sm = 0.0;
      for (int j = 0; j < n; j++) sm += qt[i * n + j] * fvec[j];
      p[i] = -sm;
    }
    for (int i = n - 1; i >= 0; i--) {
      double sm = 0.0;
      for (int j = 0; j <= i; j++) sm -= r[j * n + i] * p[j];
      g[i] = sm;
    }
    for (int i = 0; i < n; i++) { xold[i] = x[i]; fvcold[i] = fvec[i]; }
    double fold = f;
    /* R p = -Q^T F by back substitution (rsolv.c:3-12) */
    p[n - 1] /= d[n - 1];
    for (int i = n - 2; i >= 0; i--) {
      double sm = 0.0;
      for (int j = i + 1; j < n; j++) sm += r[i * n + j] * p[j];
      p[i] = (p[i] - sm) / d[i];
    }
    int check = br_lnsrch(&st, xold, fold, g, p, x, &f, stpmax);
    if (check == 3) { rc = 3; goto out; }
    err = 0.0;
    for (int i = 0; i < n; i++) err = fmax(err, fabs(fvec[i]));
    if (err < tol) { rc = 0; goto out; }
    if (check) {
      if (restrt) { rc = 1; goto out; }
      double test = 0.0, den = fmax(f, 0.5 * n);
      for (int i = 0; i < n; i++) {
        double tmp = fabs(g[i]) * fmax(fabs(x[i]), 1.0) / den;
        if (tmp > test) test = tmp;
      }
      if (test < tol) { rc = 0; goto out; }
      restrt = 1;
    } else {
      restrt = 0;
      double test = 0.0;
      for (int i = 0; i < n; i++) {
        double tmp = fabs(x[i] - xold[i]) / fmax(fabs(x[i]), 1.0);
        if (tmp > test) test = tmp;
      }
      if (test < TOLX) { rc = 0; goto out; }
    }
  }
  rc = 1;
out:
  if (iters) *iters = its;
  if (nfev) *nfev = st.nfev;
  free(mem);
  return rc;
}

/* ------------------------------------------------------------------------- */
/* safeguarded Anderson solve (CPU restatement of the batched GPU mixing)     */
/* ------------------------------------------------------------------------- */

static void small_solve_pp(double *A, double *b, int k) {
  for (int c = 0; c < k; c++) {
    int piv = c;
    double big = fabs(A[c * k + c]);
    for (int r = c + 1; r < k; r++)
      if (fabs(A[r * k + c]) > big) { big = fabs(A[r * k + c]); piv = r; }
    if (piv != c) {
      for (int j = 0; j < k; j++) { double t = A[c * k + j]; A[c * k + j] = A[piv * k + j]; A[piv * k + j] = t; }
      double t = b[c]; b[c] = b[piv]; b[piv] = t;
    }
    double pv = A[c * k + c];
    if (pv == 0.0) pv = 1e-300;
    for (int r = c + 1; r < k; r++) {
      double f = A[r * k + c] / pv;
      for (int j = c; j < k; j++) A[r * k + j] -= f * A[c * k + j];
      b[r] -= f * b[c];
    }
  }
  for (int c = k - 1; c >= 0; c--) {
    double s = b[c];
    for (int j = c + 1; j < k; j++) s -= A[c * k + j] * b[j];
    double pv = A[c * k + c];
    b[c] = s / (pv == 0.0 ? 1e-300 : pv);
  }
}

int or_anderson_solve(const or_problem *p, double *w, const or_mix_opts *o, int *iters, double *err) {
  const int n = p->n, N = n - 2, D = o->depth;
  if (N < 1 || D < 1 || D > 16) return -1;
  double *phi = (double *)malloc(sizeof(double) * n);
  double *mem = (double *)malloc(sizeof(double) * ((size_t)N * (4 + 2 * D) + (size_t)D * D));
  if (!phi || !mem) { free(phi); free(mem); return -2; }
  double *graw = mem, *g = graw + N, *gprev = g + N, *wprev = gprev + N;
  double *hdx = wprev + N, *hdg = hdx + (size_t)D * N, *G = hdg + (size_t)D * N;
  int cnt = 0, head = 0, rc = 1, it;
  double best = INFINITY, e = INFINITY;
  const double lmd = 1.0 - o->beta;
  double lk = lmd;
  double fmx = 0.0;
  for (int j = 0; j < N; j++) fmx = fmax(fmx, p->f0[j + 1]);
  const double winv = (o->weighted && fmx > 0.0) ? 1.0 / fmx : 0.0;
  const double wfloor = o->floor > 0.0 ? -o->floor / p->ds : -INFINITY;
  double hmin = INFINITY, hmax = 0.0;
  for (int k = 1; k < n; k++) {
    hmin = fmin(hmin, p->x[k] - p->x[k - 1]);
    hmax = fmax(hmax, p->x[k] - p->x[k - 1]);
  }
  const int graded = o->graded_ratio > 0.0 && hmax / hmin > o->graded_ratio;
  const double hf = graded ? sqrt(o->hfloor * p->ds) : 0.0;
  w[0] = w[n - 1] = 0.0;
  for (it = 0;; it++) {
    if (or_propagate(p, w, phi, NULL, NULL)) { rc = -3; break; }
    e = 0.0;
    int bad = 0;
    for (int j = 0; j < N; j++) {
      double pj = phi[j + 1], fj = p->f0[j + 1], r = pj - fj;
      if (!isfinite(r)) bad = 1;
      e = fmax(e, fabs(r));
      graw[j] = o->mode ? log(fmax(pj, 1e-300)) - log(fj) : r;
    }
    if (bad) { rc = 2; break; }
    if (e <= o->tol) { rc = 0; break; }
    if (it >= o->maxit) { rc = 1; break; }
    int restart = (it > 0) && (e > o->grow * best);
    if (restart) { cnt = 0; best = e; }
    else best = (it == 0) ? e : fmin(best, e);
    int push = (it > 0) && !restart, h = head;
    if (push) {
      for (int j = 0; j < N; j++) {
        hdg[(size_t)h * N + j] = graw[j] - gprev[j];
        hdx[(size_t)h * N + j] = w[j + 1] - wprev[j];
      }
      head = (head + 1) % D;
      cnt = cnt + 1 < D ? cnt + 1 : D;
    }
    int slot[16];
    double gam[16], A[256];
    for (int t = 0; t < cnt; t++) slot[t] = ((head - 1 - t) % D + D) % D;
    if (cnt > 0) {
      for (int t = 0; t < cnt; t++) {
        const double *ds_ = hdg + (size_t)slot[t] * N;
        double sb = 0.0, sg = 0.0;
        for (int j = 0; j < N; j++) {
          const double wj = o->weighted ? p->f0[j + 1] * winv : 1.0, w2 = wj * wj;
          sb += ds_[j] * (graw[j] * w2);
          if (push) sg += (hdg[(size_t)h * N + j] * w2) * ds_[j];
        }
        gam[t] = sb;
        if (push) { G[h * D + slot[t]] = sg; G[slot[t] * D + h] = sg; }
      }
      double dmax = 0.0;
      for (int t = 0; t < cnt; t++)
        for (int u = 0; u < cnt; u++) {
          A[t * cnt + u] = G[slot[t] * D + slot[u]];
          if (t == u) dmax = fmax(dmax, A[t * cnt + u]);
        }
      for (int t = 0; t < cnt; t++) A[t * cnt + t] += o->reg * dmax + 1e-300;
      small_solve_pp(A, gam, cnt);
    }
    /* mixed residual, then the preconditioned step */
    for (int j = 0; j < N; j++) {
      double rb = graw[j];
      for (int t = 0; t < cnt; t++) rb -= gam[t] * hdg[(size_t)slot[t] * N + j];
      g[j] = rb;
    }
    double dm = 0.0, da = 0.0;
    for (int j = 0; j < N; j++) {
      double gc = g[j], lap = 0.0;
      if (j > 0 && j < N - 1) {
        double a1 = fmax(p->x[j + 1] - p->x[j], hf), a2 = fmax(p->x[j + 2] - p->x[j + 1], hf);
        lap = ((gc - g[j - 1]) / a1 + (gc - g[j + 1]) / a2) / (0.5 * (a1 + a2));
      }
      double step = (1.0 - lk) * (gc + o->precond * lap);
      for (int t = 0; t < cnt; t++) step -= gam[t] * hdx[(size_t)slot[t] * N + j];
      wprev[j] = step;
      dm = fmax(dm, fabs(step) * (o->weighted ? p->f0[j + 1] * winv : 1.0));
      da = fmax(da, fabs(step));
    }
    double scale = dm > o->clip ? o->clip / dm : 1.0;
    if (!graded && o->cap > 0.0 && da * scale * p->ds > o->cap) scale = o->cap / (da * p->ds);
    const double lim = o->cap / p->ds;
    for (int j = 0; j < N; j++) {
      double dw = scale * wprev[j];
      if (graded && o->cap > 0.0) dw = fmin(fmax(dw, -lim), lim);
      wprev[j] = w[j + 1];
      gprev[j] = graw[j];
      w[j + 1] = fmax(w[j + 1] + dw, wfloor);
    }
    if (o->schedule) {
      if (e < 0.03 && it > 100) lk *= lmd;
      if (lk < 1e-5) lk = lmd;
    }
  }
  if (iters) *iters = it;
  if (err) *err = e;
  free(phi);
  free(mem);
  return rc;
}

/* ------------------------------------------------------------------------- */
/* cubic spline transfer (spline_chen.c:13-106)                               */
/* ------------------------------------------------------------------------- */
int or_spline(const double *x, const double *y, int nx, const double *xp, double *yp, int nxp, const double *m) {
  if (nx < 2 || (!m && nx <= 3)) return -1;
  for (int i = 1; i < nx; i++)
    if (!(x[i] > x[i - 1])) return -2;
  double *lo = (double *)calloc((size_t)nx, sizeof(double)), *di = (double *)calloc((size_t)nx, sizeof(double));
  double *up = (double *)calloc((size_t)nx, sizeof(double)), *rh = (double *)calloc((size_t)nx, sizeof(double));
  if (!lo || !di || !up || !rh) { free(lo); free(di); free(up); free(rh); return -3; }
  /* interior rows i = 1..nx-2 (0-based): h_{i-1}/6 M_{i-1} + (h_{i-1}+h_i)/3 M_i + h_i/6 M_{i+1} = slope jump */
  for (int i = 1; i < nx - 1; i++) {
    double a = x[i] - x[i - 1], b = x[i + 1] - x[i];
    lo[i] = a / 6.0;
    di[i] = (x[i + 1] - x[i - 1]) / 3.0;
    up[i] = b / 6.0;
    rh[i] = (y[i + 1] - y[i]) / b - (y[i] - y[i - 1]) / a;
  }
  /* The end values M0, M_{nx-1} are eliminated from the inner rows 1 and nx-2:
     M = m at both ends, or the not-a-knot conditions
     M0 = (1 + h0/h1) M1 - (h0/h1) M2  and its mirror at the right end; the
     inner system for M1..M_{nx-2} is then swept by Thomas. */
  double *M = (double *)calloc((size_t)nx, sizeof(double));
  if (!M) { free(lo); free(di); free(up); free(rh); return -3; }
  const int a = 1, b = nx - 2; /* inner rows */
  double rl = 0.0, rr = 0.0;   /* not-a-knot ratios h0/h1 and g1/g0 */
  if (m) {
    M[0] = M[nx - 1] = *m;
    if (b >= a) { rh[a] -= lo[a] * *m; rh[b] -= up[b] * *m; }
  } else {
    rl = (x[1] - x[0]) / (x[2] - x[1]);
    rr = (x[nx - 1] - x[nx - 2]) / (x[nx - 2] - x[nx - 3]);
    di[a] += lo[a] * (1.0 + rl);
    up[a] -= lo[a] * rl;
    di[b] += up[b] * (1.0 + rr);
    lo[b] -= up[b] * rr;
  }
  for (int i = a + 1; i <= b; i++) {
    double w = lo[i] / di[i - 1];
    di[i] -= w * up[i - 1];
    rh[i] -= w * rh[i - 1];
  }
  if (b >= a) {
    M[b] = rh[b] / di[b];
    for (int i = b - 1; i >= a; i--) M[i] = (rh[i] - up[i] * M[i + 1]) / di[i];
  }
  if (!m) {
    M[0] = (1.0 + rl) * M[1] - rl * M[2];
    M[nx - 1] = (1.0 + rr) * M[nx - 2] - rr * M[nx - 3];
  }
  for (int k = 0; k < nxp; k++) {
    int klo = 0, khi = nx - 1;
    while (khi - klo > 1) {
      int c = (khi + klo) >> 1;
      if (x[c] > xp[k]) khi = c; else klo = c;
    }
    double h = x[khi] - x[klo], a = (x[khi] - xp[k]) / h, b = (xp[k] - x[klo]) / h;
    yp[k] = a * y[klo] + b * y[khi] + ((a * a * a - a) * M[klo] + (b * b * b - b) * M[khi]) * (h * h) / 6.0;
  }
  free(lo); free(di); free(up); free(rh); free(M);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* CPU baseline batch driver (threads over independent instances)            */
/* ------------------------------------------------------------------------- */

typedef struct {
  const or_problem *p;
  int count;
  double *w;
  const long long *off;
  const or_mix_opts *o;
  int *rc, *iters;
  double *err;
  int next; /* next unsolved instance, taken with an atomic add */
} or_batch_job;

static void *or_batch_worker(void *arg) {
  or_batch_job *J = (or_batch_job *)arg;
  for (;;) {
    const int i = __atomic_fetch_add(&J->next, 1, __ATOMIC_RELAXED);
    if (i >= J->count) break;
    J->rc[i] = or_anderson_solve(&J->p[i], J->w + J->off[i], J->o, &J->iters[i], &J->err[i]);
  }
  return NULL;
}

int or_anderson_solve_batch(const or_problem *p, int count, double *w, const or_mix_opts *o, int threads,
                            int *rc, int *iters, double *err) {
  if (count <= 0) return 0;
  if (threads < 1) threads = 1;
  if (threads > count) threads = count;
  long long *off = (long long *)malloc(sizeof(long long) * (size_t)count);
  pthread_t *tid = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)threads);
  if (!off || !tid) { free(off); free(tid); return -1; }
  long long acc = 0;
  for (int i = 0; i < count; i++) { off[i] = acc; acc += p[i].n; }
  or_batch_job J = {p, count, w, off, o, rc, iters, err, 0};
  int started = 0, ret = 0;
  for (int t = 1; t < threads; t++) {
    if (pthread_create(&tid[t], NULL, or_batch_worker, &J) != 0) { ret = -1; break; }
    started = t;
  }
  or_batch_worker(&J); /* the calling thread works too */
  for (int t = 1; t <= started; t++) pthread_join(tid[t], NULL);
  free(off);
  free(tid);
  return ret;
}
