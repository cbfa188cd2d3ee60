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

#include <algorithm>

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

// ---------------------------------------------------------------------------
// Block-parallel form: one CTA of SB_T threads per instance, the instance's
// coefficients and state in shared memory.  The two sweeps of the complex
// Thomas solve are first-order linear recurrences, y_j = alpha_j y_{j-1} + beta_j
// (forward) and u_j = -cp_j u_{j+1} + y_j (backward); each thread composes the
// affine maps of its contiguous segment of nodes, a block-wide scan of those
// maps gives every segment its input value, and each thread replays its
// segment.  Per step: two scans of log2(32) shuffle levels plus one pass over
// the warp aggregates, instead of 2 N dependent complex operations.
// ---------------------------------------------------------------------------
constexpr int SB_T = 256;                 // most threads per instance (fewer for small batches)
constexpr int SB_W = SB_T / 32;
constexpr int SB_DOUBLES_PER_NODE = 13;   // al(2) iv(2) mc(2) sl sd su q acc y(2)

struct Map { cuDoubleComplex A, B; };     // y_out = A y_in + B

__device__ __forceinline__ Map compose(const Map &later, const Map &earlier) {
  // later o earlier
  return {cmul(later.A, earlier.A), cuCadd(cmul(later.A, earlier.B), later.B)};
}
__device__ __forceinline__ Map shfl_map(const Map &m, int src_delta, bool up) {
  Map r;
  const unsigned F = 0xffffffffu;
  if (up) {
    r.A.x = __shfl_up_sync(F, m.A.x, src_delta); r.A.y = __shfl_up_sync(F, m.A.y, src_delta);
    r.B.x = __shfl_up_sync(F, m.B.x, src_delta); r.B.y = __shfl_up_sync(F, m.B.y, src_delta);
  } else {
    r.A.x = __shfl_down_sync(F, m.A.x, src_delta); r.A.y = __shfl_down_sync(F, m.A.y, src_delta);
    r.B.x = __shfl_down_sync(F, m.B.x, src_delta); r.B.y = __shfl_down_sync(F, m.B.y, src_delta);
  }
  return r;
}

// Exclusive scan of the threads' maps in thread order (fwd) or reverse thread
// order (!fwd); returns the composite map of all earlier segments.
__device__ Map block_exclusive_scan(Map m, bool fwd, Map *agg) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const Map I = {make_cuDoubleComplex(1.0, 0.0), make_cuDoubleComplex(0.0, 0.0)};
  Map inc = m;
#pragma unroll
  for (int s = 1; s < 32; s <<= 1) {
    const Map o = shfl_map(inc, s, fwd);
    const bool ok = fwd ? (lane >= s) : (lane + s < 32);
    if (ok) inc = compose(inc, o);
  }
  Map exc = shfl_map(inc, 1, fwd);
  if (fwd ? (lane == 0) : (lane == 31)) exc = I;
  if (fwd ? (lane == 31) : (lane == 0)) agg[wid] = inc;
  __syncthreads();
  Map wp = I;  // composite of the earlier warps
  if (fwd) {
    for (int v = 0; v < wid; v++) wp = compose(agg[v], wp);
  } else {
    for (int v = (int)(blockDim.x >> 5) - 1; v > wid; v--) wp = compose(agg[v], wp);
  }
  __syncthreads();  // agg is reused by the next scan
  return compose(exc, wp);
}

__global__ void __launch_bounds__(SB_T) block_propagate_kernel(BatchDev b, SeqDev s) {
  const int inst = blockIdx.x;
  if (b.active[inst] == 0) return;
  extern __shared__ double smem[];
  __shared__ Map agg[SB_W];
  const int tid = threadIdx.x, T = blockDim.x;
  const int n = b.n[inst], N = n - 2, ns = b.nsteps[inst], half = ns / 2;
  const double ds = b.ds[inst];
  const long long no = b.node_off[inst];
  const double *x = b.x + no, *w = b.w + no, *qw = b.qw + 16LL * inst;
  cuDoubleComplex *al = reinterpret_cast<cuDoubleComplex *>(smem), *iv = al + N, *mc = iv + N, *yv = mc + N;
  double *sl = reinterpret_cast<double *>(yv + N), *sd = sl + N, *su = sd + N, *q = su + N, *acc = q + N;
  double *store = s.scratch + s.off[inst];  // (half + 1) x N slices

  const bool irk = (s.scheme == SCFT_SCHEME_IRK2);
  const cuDoubleComplex lam = irk ? make_cuDoubleComplex(0.25, 0.25 / sqrt(3.0)) : make_cuDoubleComplex(1.0, 0.0);
  const cuDoubleComplex gam = irk ? make_cuDoubleComplex(-0.5, 0.5 * sqrt(3.0)) : make_cuDoubleComplex(-0.5, 0.0);
  const cuDoubleComplex dl = make_cuDoubleComplex(ds * lam.x, ds * lam.y);

  // bands (every thread, interleaved), then the Thomas factors (thread 0: the
  // pivots are a sequential recurrence, once per field)
  for (int j = tid; j < N; j += T) {
    const int i = j + 1;
    const double a1 = x[i] - x[i - 1], a2 = x[i + 1] - x[i];
    const double ml = a1 / 6.0, md = a1 / 3.0 + a2 / 3.0, mu = a2 / 6.0;
    const double kl = -1.0 / a1, kd = 1.0 / a1 + 1.0 / a2, ku = -1.0 / a2;
    double a_l, a_d, a_u;
    if (s.wmode == SCFT_W_CONSISTENT) {
      const double wl = w[i - 1], wc = w[i], wr = w[i + 1];
      a_l = kl + a1 * (wl + wc) / 12.0;
      a_d = kd + a1 * (wl + 3.0 * wc) / 12.0 + a2 * (3.0 * wc + wr) / 12.0;
      a_u = ku + a2 * (wc + wr) / 12.0;
    } else {
      a_l = kl + w[i] * ml;
      a_d = kd + w[i] * md;
      a_u = ku + w[i] * mu;
    }
    sl[j] = a_l; sd[j] = a_d; su[j] = a_u;
    q[j] = 1.0;
    acc[j] = 0.0;
    store[j] = 1.0;
  }
  __syncthreads();
  if (tid == 0) {
    cuDoubleComplex cprev = make_cuDoubleComplex(0.0, 0.0);
    for (int j = 0; j < N; j++) {
      const int i = j + 1;
      const double a1 = x[i] - x[i - 1], a2 = x[i + 1] - x[i];
      const double ml = a1 / 6.0, md = a1 / 3.0 + a2 / 3.0, mu = a2 / 6.0;
      const cuDoubleComplex L = make_cuDoubleComplex(ml + dl.x * sl[j], dl.y * sl[j]);
      const cuDoubleComplex Dd = make_cuDoubleComplex(md + dl.x * sd[j], dl.y * sd[j]);
      const cuDoubleComplex U = make_cuDoubleComplex(mu + dl.x * su[j], dl.y * su[j]);
      const cuDoubleComplex piv = (j > 0) ? csub(Dd, cmul(L, cprev)) : Dd;
      const cuDoubleComplex ivj = cuCdiv(make_cuDoubleComplex(1.0, 0.0), piv);
      iv[j] = ivj;
      al[j] = (j > 0) ? make_cuDoubleComplex(-(L.x * ivj.x - L.y * ivj.y), -(L.x * ivj.y + L.y * ivj.x))
                      : make_cuDoubleComplex(0.0, 0.0);
      cprev = (j < N - 1) ? cmul(U, ivj) : make_cuDoubleComplex(0.0, 0.0);
      mc[j] = make_cuDoubleComplex(-cprev.x, -cprev.y);
    }
  }
  __syncthreads();

  // contiguous segment of this thread
  const int C = (N + T - 1) / T;
  const int j0 = min(tid * C, N), j1 = min(j0 + C, N);
  const Map I = {make_cuDoubleComplex(1.0, 0.0), make_cuDoubleComplex(0.0, 0.0)};
  const double wend = qw[15];
  for (int k = 1; k <= ns; k++) {
    // forward: y_j = al_j y_{j-1} + iv_j r_j, r = S q
    Map m = I;
    for (int j = j0; j < j1; j++) {
      double r = sd[j] * q[j];
      if (j > 0) r += sl[j] * q[j - 1];
      if (j < N - 1) r += su[j] * q[j + 1];
      const cuDoubleComplex be = make_cuDoubleComplex(iv[j].x * r, iv[j].y * r);
      yv[j] = be;
      m = compose(Map{al[j], be}, m);
    }
    Map p = block_exclusive_scan(m, true, agg);
    cuDoubleComplex y = p.B;  // y before the segment (y_{-1} = 0)
    for (int j = j0; j < j1; j++) {
      y = cuCadd(cmul(al[j], y), yv[j]);
      yv[j] = y;
    }
    // backward: u_j = mc_j u_{j+1} + y_j (reverse thread order)
    m = I;
    for (int j = j1 - 1; j >= j0; j--) m = compose(Map{mc[j], yv[j]}, m);
    p = block_exclusive_scan(m, false, agg);
    cuDoubleComplex u = p.B;
    for (int j = j1 - 1; j >= j0; j--) {
      u = cuCadd(cmul(mc[j], u), yv[j]);
      q[j] += 2.0 * ds * (gam.x * u.x - gam.y * u.y);
    }
    __syncthreads();
    // half-contour store and density (interleaved, coalesced)
    if (k <= half) {
      double *dst = store + (long long)k * N;
      for (int j = tid; j < N; j += T) dst[j] = q[j];
    }
    if (k >= ns - half) {
      const double *o = store + (long long)(ns - k) * N;
      double wk = (k == ns) ? wend : qw[min(__ffs(k) - 1, 14)];
      if (k != ns - k) wk += wk;
      for (int j = tid; j < N; j += T) acc[j] += wk * q[j] * o[j];
    }
    __syncthreads();
  }
  double *phi = b.phi + no;
  double qs = 0.0;
  int bad = 0;
  for (int j = tid; j < N; j += T) {
    if (!isfinite(acc[j])) bad |= ST_NONFINITE;
    phi[j + 1] = acc[j];
    qs += 0.5 * (x[j + 2] - x[j]) * q[j];
  }
  for (int o = 16; o > 0; o >>= 1) {
    qs += __shfl_down_sync(0xffffffffu, qs, o);
    bad |= __shfl_down_sync(0xffffffffu, bad, o);
  }
  __shared__ double red[SB_W];
  __shared__ int ired[SB_W];
  if ((tid & 31) == 0) { red[tid >> 5] = qs; ired[tid >> 5] = bad; }
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    int bb = 0;
    for (int v = 0; v < (T >> 5); v++) { t += red[v]; bb |= ired[v]; }
    phi[0] = 0.0;
    phi[n - 1] = 0.0;
    b.Q[inst] = t / (x[n - 1] - x[0]);
    if (bb) atomicOr(&b.status[inst], bb);
  }
}

}  // namespace

// Largest instance (nodes) of the block-parallel form, and its shared memory.
int seq_block_max_nodes() {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return (int)((optin - 4096) / (SB_DOUBLES_PER_NODE * sizeof(double))) + 2;
}

// Half-store doubles of one instance in the block-parallel form.
long long seq_block_store_doubles(int n, int nsteps) {
  const long long N = n - 2;
  return N * (nsteps / 2 + 1);
}

// Block-parallel evaluation of the active instances (every one must fit).
cudaError_t seq_block_launch(const BatchDev &b, int max_nodes, int scheme, int wmode, double *scratch,
                             const long long *off, cudaStream_t st) {
  const size_t smem = (size_t)(max_nodes - 2) * SB_DOUBLES_PER_NODE * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(block_propagate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  SeqDev s{scheme, wmode, scratch, off};
  // threads: the largest instance's interior nodes rounded up to warps, at most SB_T
  const int threads = std::min(SB_T, 32 * ((max_nodes - 2 + 31) / 32));
  block_propagate_kernel<<<b.count, threads, smem, st>>>(b, s);
  return cudaGetLastError();
}

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
