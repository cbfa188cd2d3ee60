// mixing.cu -- FP64 field-update kernels.
//
// mix_kernel        batched Anderson mixing (one CTA per instance) used by the
//                   batched solver: residual check, difference-form history of
//                   the mixing residual, regularised least squares, a
//                   preconditioned and clipped step, restart safeguard.
// admchen_step_*    one iteration of ADM_chen_C.c:55-135 for the drop-in solver.
// adm_*             one iteration of adm.c:103-306 for the drop-in solver.
#include "mix_group.cuh"

namespace scft {

constexpr int MIX_THREADS = 256;
constexpr int MAXD = MIX_MAXD;
// history limit of the drop-in adm_chen (the deal.II driver asks for up to 50,
// drivescft.cc:296): U (m x m) and V live in shared memory
constexpr int ADM_MAXD = 64;

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

// One batched Anderson iteration per unfinished instance, one CTA each.
__global__ void __launch_bounds__(MIX_THREADS) mix_kernel(MixDev m) {
  const int inst = blockIdx.x;
  if (m.active[inst] == 0) return;
  __shared__ MixSmem<MIX_THREADS / 32> S;
  auto sync = []() { __syncthreads(); };
  mix_step<MIX_THREADS / 32>(m, inst, threadIdx.x, S, sync);
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
  int ipiv[ADM_MAXD], indxr[ADM_MAXD], indxc[ADM_MAXD];
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
  __shared__ double U[ADM_MAXD * ADM_MAXD], V[ADM_MAXD];
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
  if (a.nm > ADM_MAXD - 1) return cudaErrorInvalidValue;
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
