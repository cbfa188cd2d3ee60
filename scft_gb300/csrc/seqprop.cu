// seqprop.cu -- the deal.II form of the propagator on the GPU (FP64).
//
// DEALII_SCFT's HeatEquation (drivescft.cc:130-165, scft.cc:589-696) steps
// M dq/ds = -(K + W) q with the consistent field term W_ij = int w_h phi_i
// phi_j (scft.cc:653-655, exact for the piecewise-linear w_h) and the 2-stage
// Gauss-Legendre implicit Runge-Kutta method, whose stage system is the 2n x 2n
// block system [M + ds a11 S, ds a12 S; ds a21 S, M + ds a22 S] k = -[S q; S q]
// (S = K + W, scft.cc:668-695).  The Butcher matrix of the method has the
// complex pair of eigenvalues lambda = 1/4 +- i/(4 sqrt 3); in its eigenbasis the
// stage system decouples into one complex tridiagonal system per step:
//
//   (M + ds lambda S) u = S q,      q <- q + 2 ds Re(gamma u),
//   lambda = 1/4 + i/(4 sqrt 3),    gamma = -1/2 + i sqrt(3)/2,
//
// which reproduces the method's stability function (1 + z/2 + z^2/12) /
// (1 - z/2 + z^2/12) exactly.  Implicit Euler (1D_FEM.c:208-228) is the same
// update with lambda = 1, gamma = -1/2, so one kernel serves both schemes and
// both field terms (row-scaled W_ij = w_i M_ij of 1D_FEM.c:104-105, or
// consistent).  One thread per instance: complex Thomas factorisation once per
// field, then a forward and a backward sweep per contour step; the density is
// accumulated from a half-contour store exactly as the batched propagator
// does (slice k paired with slice ns - k, quadrature weights per 2-adic class).
#include <cuComplex.h>

#include "batch.cuh"
#include "common.cuh"
#include "scft.h"

namespace scft {
namespace {

struct SeqDev {
  int scheme;             // SCFT_SCHEME_IE or SCFT_SCHEME_IRK2
  int wmode;              // SCFT_W_ROWSCALED or SCFT_W_CONSISTENT
  double *scratch;        // per instance: 4 N complex, 5 N real, (half + 1) N store
  const long long *off;   // scratch offset of each instance
};

__device__ __forceinline__ cuDoubleComplex cmul(cuDoubleComplex a, cuDoubleComplex b) { return cuCmul(a, b); }
__device__ __forceinline__ cuDoubleComplex csub(cuDoubleComplex a, cuDoubleComplex b) { return cuCsub(a, b); }

__global__ void seq_propagate_kernel(BatchDev b, SeqDev s) {
  const int inst = blockIdx.x * blockDim.x + threadIdx.x;
  if (inst >= b.count || b.active[inst] == 0) return;
  const int n = b.n[inst], N = n - 2, ns = b.nsteps[inst], half = ns / 2;
  const double ds = b.ds[inst];
  const long long no = b.node_off[inst];
  const double *x = b.x + no, *w = b.w + no, *qw = b.qw + 16LL * inst;
  // complex arrays first: the scratch base and every instance offset are
  // multiples of 16 bytes
  double *base = s.scratch + s.off[inst];
  cuDoubleComplex *Dl = reinterpret_cast<cuDoubleComplex *>(base);  // sub-band of M + ds lambda S
  cuDoubleComplex *inv = Dl + N, *cp = inv + N, *u = cp + N;        // 1/pivot, modified super-band, sweep
  double *sl = reinterpret_cast<double *>(u + N), *sd = sl + N, *su = sd + N;  // S = K + W
  double *q = su + N, *acc = q + N, *store = acc + N;

  const bool irk = (s.scheme == SCFT_SCHEME_IRK2);
  const cuDoubleComplex lam = irk ? make_cuDoubleComplex(0.25, 0.25 / sqrt(3.0)) : make_cuDoubleComplex(1.0, 0.0);
  const cuDoubleComplex gam = irk ? make_cuDoubleComplex(-0.5, 0.5 * sqrt(3.0)) : make_cuDoubleComplex(-0.5, 0.0);
  const cuDoubleComplex dl = make_cuDoubleComplex(ds * lam.x, ds * lam.y);
  int bad = 0;

  // bands and the complex Thomas factorisation of M + ds lambda S
  cuDoubleComplex cprev = make_cuDoubleComplex(0.0, 0.0);
  for (int j = 0; j < N; j++) {
    const int i = j + 1;
    const double a1 = x[i] - x[i - 1], a2 = x[i + 1] - x[i];
    const double ml = a1 / 6.0, md = a1 / 3.0 + a2 / 3.0, mu = a2 / 6.0;
    const double kl = -1.0 / a1, kd = 1.0 / a1 + 1.0 / a2, ku = -1.0 / a2;
    double al, ad, au;
    if (s.wmode == SCFT_W_CONSISTENT) {
      const double wl = w[i - 1], wc = w[i], wr = w[i + 1];
      al = kl + a1 * (wl + wc) / 12.0;
      ad = kd + a1 * (wl + 3.0 * wc) / 12.0 + a2 * (3.0 * wc + wr) / 12.0;
      au = ku + a2 * (wc + wr) / 12.0;
    } else {
      al = kl + w[i] * ml;
      ad = kd + w[i] * md;
      au = ku + w[i] * mu;
    }
    sl[j] = al; sd[j] = ad; su[j] = au;
    const cuDoubleComplex L = make_cuDoubleComplex(ml + dl.x * al, dl.y * al);
    const cuDoubleComplex Dd = make_cuDoubleComplex(md + dl.x * ad, dl.y * ad);
    const cuDoubleComplex U = make_cuDoubleComplex(mu + dl.x * au, dl.y * au);
    const cuDoubleComplex piv = (j > 0) ? csub(Dd, cmul(L, cprev)) : Dd;
    const cuDoubleComplex iv = cuCdiv(make_cuDoubleComplex(1.0, 0.0), piv);
    Dl[j] = L;
    inv[j] = iv;
    cprev = (j < N - 1) ? cmul(U, iv) : make_cuDoubleComplex(0.0, 0.0);
    cp[j] = cprev;
  }
  for (int j = 0; j < N; j++) {
    q[j] = 1.0;
    acc[j] = 0.0;
    store[j] = 1.0;
  }
  const double wend = qw[15];
  for (int k = 1; k <= ns; k++) {
    // forward sweep on r = S q (walls zero)
    cuDoubleComplex y = make_cuDoubleComplex(0.0, 0.0);
    for (int j = 0; j < N; j++) {
      double r = sd[j] * q[j];
      if (j > 0) r += sl[j] * q[j - 1];
      if (j < N - 1) r += su[j] * q[j + 1];
      const cuDoubleComplex t = (j > 0) ? csub(make_cuDoubleComplex(r, 0.0), cmul(Dl[j], y)) : make_cuDoubleComplex(r, 0.0);
      y = cmul(t, inv[j]);
      u[j] = y;
    }
    // backward sweep and the update q += 2 ds Re(gamma u)
    cuDoubleComplex nx = make_cuDoubleComplex(0.0, 0.0);
    for (int j = N - 1; j >= 0; j--) {
      const cuDoubleComplex v = (j < N - 1) ? csub(u[j], cmul(cp[j], nx)) : u[j];
      nx = v;
      q[j] += 2.0 * ds * (gam.x * v.x - gam.y * v.y);
    }
    if (k <= half) {
      double *dst = store + (long long)k * N;
      for (int j = 0; j < N; j++) dst[j] = q[j];
    }
    if (k >= ns - half) {
      const double *o = store + (long long)(ns - k) * N;
      double wk = (k == ns) ? wend : qw[min(__ffs(k) - 1, 14)];
      if (k != ns - k) wk += wk;
      for (int j = 0; j < N; j++) acc[j] += wk * q[j] * o[j];
    }
  }
  double *phi = b.phi + no;
  double qs = 0.0;
  for (int j = 0; j < N; j++) {
    if (!isfinite(acc[j])) bad |= ST_NONFINITE;
    phi[j + 1] = acc[j];
    qs += 0.5 * (x[j + 2] - x[j]) * q[j];
  }
  phi[0] = 0.0;
  phi[n - 1] = 0.0;
  b.Q[inst] = qs / (x[n - 1] - x[0]);
  if (bad) atomicOr(&b.status[inst], bad);
}

}  // namespace

// Scratch doubles of one instance (even, so the next instance starts 16-byte aligned).
long long seq_scratch_doubles(int n, int nsteps) {
  const long long N = n - 2;
  const long long d = N * (8 + 5) + N * (nsteps / 2 + 1);
  return d + (d & 1);
}

// Evaluate the instances whose active flag is nonzero with the given scheme and
// field term, on `st`; scratch and offsets are device arrays the caller owns.
cudaError_t seq_propagate_launch(const BatchDev &b, int scheme, int wmode, double *scratch, const long long *off,
                                 cudaStream_t st) {
  SeqDev s{scheme, wmode, scratch, off};
  const int threads = 64;
  seq_propagate_kernel<<<(b.count + threads - 1) / threads, threads, 0, st>>>(b, s);
  return cudaGetLastError();
}

}  // namespace scft
