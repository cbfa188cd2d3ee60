// mixing.cu -- FP64 field-update kernels.
//
// mix_kernel        batched Anderson mixing (one CTA per instance) used by the
//                   batched solver: residual check, difference-form history of
//                   the mixing residual, regularised least squares, a
//                   preconditioned and clipped step, restart safeguard.
// admchen_step_*    one iteration of ADM_chen_C.c:55-135 for the drop-in solver.
// adm_*             one iteration of adm.c:103-306 for the drop-in solver.
#include "mixing.cuh"

namespace scft {

constexpr int MIX_THREADS = 256;
constexpr int MAXD = 16;

__device__ __forceinline__ double warp_max(double v) {
  for (int s = 16; s > 0; s >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, s));
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
  for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
  return v;
}

// block-wide max of v (all threads receive it)
__device__ double block_max(double v, double *sm) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) sm[wid] = v;
  __syncthreads();
  double r = (lane < nw) ? sm[lane] : 0.0;
  r = warp_max(r);
  return r;
}

// Solve the k x k system A g = b (row-major, A overwritten) by Gaussian
// elimination with partial pivoting; single thread.
__device__ void small_solve(double *A, double *b, int k) {
  for (int c = 0; c < k; c++) {
    int p = c;
    double big = fabs(A[c * k + c]);
    for (int r = c + 1; r < k; r++)
      if (fabs(A[r * k + c]) > big) { big = fabs(A[r * k + c]); p = r; }
    if (p != c) {
      for (int j = 0; j < k; j++) { double t = A[c * k + j]; A[c * k + j] = A[p * k + j]; A[p * k + j] = t; }
      double t = b[c]; b[c] = b[p]; b[p] = t;
    }
    double piv = A[c * k + c];
    if (piv == 0.0) piv = 1e-300;
    for (int r = c + 1; r < k; r++) {
      double f = A[r * k + c] / piv;
      for (int j = c; j < k; j++) A[r * k + j] -= f * A[c * k + j];
      b[r] -= f * b[c];
    }
  }
  for (int c = k - 1; c >= 0; c--) {
    double s = b[c];
    for (int j = c + 1; j < k; j++) s -= A[c * k + j] * b[j];
    double piv = A[c * k + c];
    b[c] = s / (piv == 0.0 ? 1e-300 : piv);
  }
}

__global__ void __launch_bounds__(MIX_THREADS) mix_kernel(MixDev m) {
  const int inst = blockIdx.x;
  const int act = m.active[inst];
  if (act == 0) return;
  __shared__ double sm[32];
  __shared__ double red[2 * MAXD][MIX_THREADS / 32];
  __shared__ double gam[MAXD];
  __shared__ int sh_slot[MAXD];
  __shared__ int sh_ctl[4];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int n = m.n[inst], N = n - 2;
  const long long no = m.node_off[inst], io = m.int_off[inst];
  const double *x = m.x + no, *f0 = m.f0 + no, *phi = m.phi + no;
  double *w = m.w + no;
  double *graw = m.graw + io, *gcur = m.gcur + io, *gprev = m.gprev + io, *wprev = m.wprev + io;
  const int D = m.depth;
  double *hdx = m.hdx + io * D, *hdg = m.hdg + io * D;
  double *G = m.gram + (long long)inst * D * D;

  // 1. residual, its norm, raw mixing residual
  double e = 0.0, badv = 0.0;
  for (int j = tid; j < N; j += MIX_THREADS) {
    const double p = phi[j + 1], f = f0[j + 1], r = p - f;
    if (!isfinite(r)) badv = 1.0;
    e = fmax(e, fabs(r));
    graw[j] = m.mode ? (log(fmax(p, 1e-300)) - log(f)) : r;
  }
  e = block_max(e, sm);
  badv = block_max(badv, sm);
  // weights f0_j / max f0: the scale on which ||phi - f0||_inf is judged
  double fmx = 0.0;
  if (m.weighted) {
    for (int j = tid; j < N; j += MIX_THREADS) fmx = fmax(fmx, f0[j + 1]);
    fmx = block_max(fmx, sm);
  }
  const double winv = (m.weighted && fmx > 0.0) ? 1.0 / fmx : 0.0;
  const int it = m.iters[inst];
  if (badv != 0.0) {
    if (tid == 0) { m.status[inst] |= ST_NONFINITE; m.active[inst] = 0; m.err[inst] = e; }
    return;
  }
  const double tol_here = (act == 1) ? m.tol32 : m.tol;
  if (e <= tol_here) {
    if (tid == 0) {
      m.err[inst] = e;
      if (act == 1 && m.verify64) m.active[inst] = 2;
      else { m.status[inst] |= ST_CONVERGED; m.active[inst] = 0; }
    }
    return;
  }
  if (it >= m.maxit) {
    if (tid == 0) { m.status[inst] |= ST_MAXIT; m.active[inst] = 0; m.err[inst] = e; }
    return;
  }
  // 2. history bookkeeping (restart when the error grew by more than `grow`)
  if (tid == 0) {
    int cnt = m.hcount[inst], head = m.hhead[inst];
    double best = m.best[inst];
    const bool restart = (it > 0) && (e > m.grow * best);
    if (restart) { cnt = 0; best = e; m.status[inst] |= ST_RESTARTED; }
    else best = (it == 0) ? e : fmin(best, e);
    const int push = (it > 0) && !restart;
    const int h = head;
    if (push) { head = (head + 1) % D; cnt = cnt + 1 < D ? cnt + 1 : D; }
    for (int t = 0; t < cnt; t++) sh_slot[t] = ((head - 1 - t) % D + D) % D;
    sh_ctl[0] = cnt; sh_ctl[1] = head; sh_ctl[2] = push; sh_ctl[3] = h;
    m.best[inst] = best;
  }
  __syncthreads();
  const int cnt = sh_ctl[0], push = sh_ctl[2], h = sh_ctl[3];
  if (push) {
    for (int j = tid; j < N; j += MIX_THREADS) {
      hdg[(long long)h * N + j] = graw[j] - gprev[j];
      hdx[(long long)h * N + j] = w[j + 1] - wprev[j];
    }
  }
  __syncthreads();
  // 3. least squares on the raw mixing residual r: new Gram row <dr_h, dr_s>
  //    and right-hand side <dr_s, r>, inner products weighted by (f0_j / max f0)^2
  //    so that nodes whose ||phi - f0|| is far below any tolerance (the walls)
  //    do not steer the extrapolation
  if (cnt > 0) {
    double pb[MAXD], pg[MAXD];
#pragma unroll
    for (int t = 0; t < MAXD; t++) { pb[t] = 0.0; pg[t] = 0.0; }
    for (int j = tid; j < N; j += MIX_THREADS) {
      const double wj = m.weighted ? f0[j + 1] * winv : 1.0;
      const double gv = graw[j] * wj * wj;
      const double dh = push ? hdg[(long long)h * N + j] * wj * wj : 0.0;
#pragma unroll
      for (int t = 0; t < MAXD; t++) {
        if (t < cnt) {
          const double d = hdg[(long long)sh_slot[t] * N + j];
          pb[t] += d * gv;
          pg[t] += dh * d;
        }
      }
    }
#pragma unroll
    for (int t = 0; t < MAXD; t++) {
      if (t < cnt) {
        const double a = warp_sum(pb[t]), b = warp_sum(pg[t]);
        if (lane == 0) { red[t][wid] = a; red[MAXD + t][wid] = b; }
      }
    }
    __syncthreads();
    if (tid == 0) {
      double A[MAXD * MAXD], rhs[MAXD];
      for (int t = 0; t < cnt; t++) {
        double sb = 0.0, sg = 0.0;
        for (int q = 0; q < MIX_THREADS / 32; q++) { sb += red[t][q]; sg += red[MAXD + t][q]; }
        rhs[t] = sb;
        if (push) { G[h * D + sh_slot[t]] = sg; G[sh_slot[t] * D + h] = sg; }
      }
      double dmax = 0.0;
      for (int t = 0; t < cnt; t++)
        for (int u = 0; u < cnt; u++) {
          A[t * cnt + u] = G[sh_slot[t] * D + sh_slot[u]];
          if (t == u) dmax = fmax(dmax, A[t * cnt + u]);
        }
      for (int t = 0; t < cnt; t++) A[t * cnt + t] += m.reg * dmax + 1e-300;
      small_solve(A, rhs, cnt);
      for (int t = 0; t < cnt; t++) gam[t] = rhs[t];
    }
    __syncthreads();
  }
  // 4. mixed residual rbar = r - sum_s gam_s dr_s (into gcur)
  for (int j = tid; j < N; j += MIX_THREADS) {
    double rb = graw[j];
    for (int t = 0; t < cnt; t++) rb -= gam[t] * hdg[(long long)sh_slot[t] * N + j];
    gcur[j] = rb;
  }
  __syncthreads();
  // 5. update w <- w - sum_s gam_s dx_s + beta (1 + a (-d2/dx2)) rbar
  //    (the preconditioner acts on the step only, so FP32 rounding noise it
  //    amplifies never enters the least squares; the mixed residual is
  //    extended linearly past the first and last interior nodes, i.e. no
  //    curvature term there); beta = 1 - lk.  The step is scaled so that its
  //    f0-weighted max norm is <= clip and no node moves by more than
  //    step_cap / ds; the field is kept >= -field_floor / ds.
  const double beta = 1.0 - m.lk[inst];
  const double dsi = m.ds[inst];
  double dm = 0.0, da = 0.0;
  for (int j = tid; j < N; j += MIX_THREADS) {
    const double gc = gcur[j];
    double lap = 0.0;
    if (j > 0 && j < N - 1) {
      const double a1 = x[j + 1] - x[j], a2 = x[j + 2] - x[j + 1];
      lap = ((gc - gcur[j - 1]) / a1 + (gc - gcur[j + 1]) / a2) / (0.5 * (a1 + a2));
    }
    double d = beta * (gc + m.precond * lap);
    for (int t = 0; t < cnt; t++) d -= gam[t] * hdx[(long long)sh_slot[t] * N + j];
    wprev[j] = d;  // staged; wprev receives the old field below
    const double wj = m.weighted ? f0[j + 1] * winv : 1.0;
    dm = fmax(dm, fabs(d) * wj);
    da = fmax(da, fabs(d));
  }
  dm = block_max(dm, sm);
  da = block_max(da, sm);
  double scale = (dm > m.clip) ? m.clip / dm : 1.0;
  if (m.step_cap > 0.0 && da * scale * dsi > m.step_cap) scale = m.step_cap / (da * dsi);
  const double wfloor = (m.field_floor > 0.0) ? -m.field_floor / dsi : -INFINITY;
  for (int j = tid; j < N; j += MIX_THREADS) {
    const double wo = w[j + 1];
    const double d = wprev[j];
    wprev[j] = wo;
    gprev[j] = graw[j];
    w[j + 1] = fmax(wo + scale * d, wfloor);
  }
  if (tid == 0) {
    m.iters[inst] = it + 1;
    m.hcount[inst] = cnt;
    m.hhead[inst] = sh_ctl[1];
    m.err[inst] = e;
    if (m.lk_schedule) {
      double l = m.lk[inst];
      if (e < 0.03 && it > 100) l *= m.lmd;
      if (l < 1e-5) l = m.lmd;
      m.lk[inst] = l;
    }
  }
}

cudaError_t mix_launch(const MixDev &m, cudaStream_t st) {
  if (m.count <= 0) return cudaSuccess;
  if (m.depth > MAXD || m.depth < 1) return cudaErrorInvalidValue;
  mix_kernel<<<m.count, MIX_THREADS, 0, st>>>(m);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Gauss-Jordan with full pivoting, single thread (gaussj.c:7-60): the last
// largest |a| in row-major scan among unpivoted rows/columns is the pivot.
// mode 0: zero pivot += 1e-18 (gaussj.c:38); mode 1: return 1
// (DEALII_SCFT/src/gaussj.c:45-50).  a: n x n, b: n x 1, row-major.
__device__ int dev_gaussj(double *a, int n, double *b, int mode) {
  int ipiv[MAXD], indxr[MAXD], indxc[MAXD];
  for (int j = 0; j < n; j++) ipiv[j] = 0;
  for (int i = 0; i < n; i++) {
    double big = 0.0;
    int irow = 0, icol = 0;
    for (int j = 0; j < n; j++) {
      if (ipiv[j] == 1) continue;
      for (int k = 0; k < n; k++) {
        if (ipiv[k] != 0) continue;
        const double v = fabs(a[j * n + k]);
        if (v >= big) { big = v; irow = j; icol = k; }
      }
    }
    ipiv[icol]++;
    if (irow != icol) {
      for (int l = 0; l < n; l++) { double t = a[irow * n + l]; a[irow * n + l] = a[icol * n + l]; a[icol * n + l] = t; }
      double t = b[irow]; b[irow] = b[icol]; b[icol] = t;
    }
    indxr[i] = irow;
    indxc[i] = icol;
    if (a[icol * n + icol] == 0.0) {
      if (mode == 1) return 1;
      a[icol * n + icol] += 1e-18;
    }
    const double pinv = 1.0 / a[icol * n + icol];
    a[icol * n + icol] = 1.0;
    for (int l = 0; l < n; l++) a[icol * n + l] *= pinv;
    b[icol] *= pinv;
    for (int r = 0; r < n; r++) {
      if (r == icol) continue;
      const double f = a[r * n + icol];
      a[r * n + icol] = 0.0;
      for (int l = 0; l < n; l++) a[r * n + l] -= a[icol * n + l] * f;
      b[r] -= b[icol] * f;
    }
  }
  for (int l = n - 1; l >= 0; l--) {
    if (indxr[l] == indxc[l]) continue;
    for (int k = 0; k < n; k++) {
      double t = a[k * n + indxr[l]]; a[k * n + indxr[l]] = a[k * n + indxc[l]]; a[k * n + indxc[l]] = t;
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// ADM_chen_C.c:55-135, one iteration k: Y_k = f(X_k) is already in Y.
__global__ void __launch_bounds__(MIX_THREADS) admchen_step_kernel(AdmChenDev a) {
  __shared__ double sm[32];
  __shared__ double U[MAXD * MAXD], V[MAXD];
  __shared__ int sh_m, sh_fail;
  const int tid = threadIdx.x, n = a.n, D = a.depth;
  const int k = *a.k;
  const double *Xk = a.X + (long long)(k % D) * n, *Yk = a.Y + (long long)(k % D) * n;
  double e = 0.0, nanv = 0.0;
  for (int i = tid; i < n; i += MIX_THREADS) {
    const double y = Yk[i];
    if (isnan(y)) nanv = 1.0;
    e = fmax(e, fabs(y));
  }
  e = block_max(e, sm);
  nanv = block_max(nanv, sm);
  if (tid == 0) *a.err = e;
  if (nanv != 0.0) { if (tid == 0) *a.flag = 2; return; }
  if (e < a.tol) { if (tid == 0) *a.flag = 1; return; }
  for (;;) {
    if (tid == 0) {
      const int kr = *a.krestart;
      sh_m = (a.nm < k - kr) ? a.nm : k - kr;
    }
    __syncthreads();
    const int m = sh_m;
    // U_ij and V_i, each summed over t in the reference's order by one thread
    const int npairs = m * m + m;
    for (int q = tid; q < npairs; q += MIX_THREADS) {
      double s = 0.0;
      if (q < m * m) {
        const int i = q / m, j = q % m;
        const double *Yi = a.Y + (long long)(((k - i - 1) % D + D) % D) * n;
        const double *Yj = a.Y + (long long)(((k - j - 1) % D + D) % D) * n;
        for (int t = 0; t < n; t++) s += (Yk[t] - Yi[t]) * (Yk[t] - Yj[t]);
        U[i * m + j] = s;
      } else {
        const int i = q - m * m;
        const double *Yi = a.Y + (long long)(((k - i - 1) % D + D) % D) * n;
        for (int t = 0; t < n; t++) s += (Yk[t] - Yi[t]) * Yk[t];
        V[i] = s;
      }
    }
    __syncthreads();
    if (tid == 0) {
      sh_fail = (m > 0) ? dev_gaussj(U, m, V, 1) : 0;
      if (sh_fail) { *a.krestart = k; *a.lk = a.lmd; }
    }
    __syncthreads();
    if (!sh_fail) break;
  }
  const int m = sh_m;
  const double lk = *a.lk;
  double *Xn = a.X + (long long)((k + 1) % D) * n;
  for (int i = tid; i < n; i += MIX_THREADS) {
    double cx = 0.0, cd = 0.0;
    for (int j = 0; j < m; j++) {
      const long long r = (long long)(((k - j - 1) % D + D) % D) * n;
      cx += V[j] * (a.X[r + i] - Xk[i]);
      cd += V[j] * (a.Y[r + i] - Yk[i]);
    }
    Xn[i] = Xk[i] + cx + (1.0 - lk) * (Yk[i] + cd);
  }
  __syncthreads();
  if (tid == 0) {
    double l = lk;
    if (e < 0.03 && k > 100) l *= a.lmd;
    if (!a.final_ && l < 1e-5) l = a.lmd;
    if (a.final_ && l < 1e-15) l = a.lmd;
    *a.lk = l;
    *a.k = k + 1;
    *a.flag = 0;
  }
}

cudaError_t admchen_step_launch(const AdmChenDev &a, cudaStream_t st) {
  if (a.nm > MAXD - 1) return cudaErrorInvalidValue;
  admchen_step_kernel<<<1, MIX_THREADS, 0, st>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// adm.c:103-146: first Anderson step, x <- x + 0.05 (g(x) - x).
__global__ void __launch_bounds__(MIX_THREADS) adm_first_kernel(AdmDev a) {
  __shared__ double sm[32];
  const int tid = threadIdx.x, n = a.n;
  double e = 0.0;
  for (int i = tid; i < n; i += MIX_THREADS) {
    a.xh[i] = a.x[i];
    a.dh[i] = a.xnew[i] - a.x[i];
    e = fmax(e, fabs(a.dh[i]));
  }
  e = block_max(e, sm);
  if (tid == 0) { *a.err = e; *a.its = 1; *a.nc = 1; *a.flag = (e < a.tol) ? 1 : 0; }
  if (e < a.tol) return;
  for (int i = tid; i < n; i += MIX_THREADS) a.x[i] = a.xh[i] + 0.05 * a.dh[i];
}

// adm.c:148-306, iteration its >= 2 (xnew = g(x) already evaluated).
__global__ void __launch_bounds__(MIX_THREADS) adm_step_kernel(AdmDev a) {
  constexpr int S = 11;
  __shared__ double sm[32];
  __shared__ double U[10 * 10], B[10];
  __shared__ int slot_of[10];
  __shared__ int sh_cur, sh_nr;
  const int tid = threadIdx.x, n = a.n;
  const int its = *a.its + 1;
  if (tid == 0) {
    int nc = *a.nc;
    if (nc == S) nc = 0;
    sh_cur = nc;
    sh_nr = (its - 1 < 10) ? its - 1 : 10;
  }
  __syncthreads();
  const int cur = sh_cur, nr = sh_nr;
  double *xc = a.xh + (long long)cur * n, *dc = a.dh + (long long)cur * n;
  double e = 0.0;
  for (int i = tid; i < n; i += MIX_THREADS) {
    dc[i] = a.xnew[i] - a.x[i];
    xc[i] = a.x[i];
    e = fmax(e, fabs(dc[i]));
  }
  e = block_max(e, sm);
  if (tid == 0) { *a.err = e; *a.its = its; *a.nc = cur + 1; *a.flag = (e < a.tol) ? 1 : 0; }
  if (e < a.tol) return;
  if (tid == 0) {
    int q = 0;
    for (int s = 0; s < cur; s++) slot_of[q++] = s;
    for (int s = nr; s > cur; s--) slot_of[q++] = s;
  }
  __syncthreads();
  const int npairs = nr * nr + nr;
  for (int q = tid; q < npairs; q += MIX_THREADS) {
    double s = 0.0;
    if (q < nr * nr) {
      const int p = q / nr, r = q % nr;
      const double *dp = a.dh + (long long)slot_of[p] * n, *dr = a.dh + (long long)slot_of[r] * n;
      for (int i = 0; i < n; i++) s += (dc[i] - dp[i]) * (dc[i] - dr[i]);
      U[p * nr + r] = s;
    } else {
      const int p = q - nr * nr;
      const double *dp = a.dh + (long long)slot_of[p] * n;
      for (int i = 0; i < n; i++) s += (dc[i] - dp[i]) * dc[i];
      B[p] = s;
    }
  }
  __syncthreads();
  if (tid == 0) dev_gaussj(U, nr, B, 0);
  __syncthreads();
  const double lambda = 1.0 - pow(0.95, (double)its);
  for (int i = tid; i < n; i += MIX_THREADS) {
    double t = 0.0, t1 = 0.0;
    for (int p = 0; p < nr; p++) {
      const long long o = (long long)slot_of[p] * n + i;
      t += B[p] * (a.xh[o] - xc[i]);
      t1 += B[p] * (a.dh[o] - dc[i]);
    }
    a.x[i] = xc[i] + t + lambda * (dc[i] + t1);
  }
}

cudaError_t adm_first_launch(const AdmDev &a, cudaStream_t st) {
  adm_first_kernel<<<1, MIX_THREADS, 0, st>>>(a);
  return cudaGetLastError();
}
cudaError_t adm_step_launch(const AdmDev &a, cudaStream_t st) {
  adm_step_kernel<<<1, MIX_THREADS, 0, st>>>(a);
  return cudaGetLastError();
}

// out_j = sign (phi_{j+1} - f0_{j+1}) [+ w_j when fixed_point], j = 0..n-3
__global__ void residual_kernel(int n, const double *phi, const double *f0, int sign, double *out,
                                const double *w_int, int fixed_point) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n - 2) return;
  double r = phi[j + 1] - f0[j + 1];
  if (sign < 0) r = -r;
  out[j] = fixed_point ? w_int[j] + r : r;
}

cudaError_t residual_launch(int n, const double *phi, const double *f0, int sign, double *out_int,
                            double *w_int_in, int fixed_point, cudaStream_t st) {
  const int N = n - 2;
  if (N <= 0) return cudaSuccess;
  residual_kernel<<<(N + 255) / 256, 256, 0, st>>>(n, phi, f0, sign, out_int, w_int_in, fixed_point);
  return cudaGetLastError();
}

}  // namespace scft
