// spline.cu -- mesh refinement and the field transfer that goes with it.
//
// The deal.II driver refines by bisecting every cell (refine_mesh,
// DEALII_SCFT/src/scft.cc:132-166: the Kelly estimate is computed, then every
// cell is flagged for refinement in x) and carries the interior field over to the
// new mesh with a cubic spline, spline_chen (DEALII_SCFT/src/spline_chen.c:13-106).
// The spline's second derivatives M satisfy, at the inner points,
//   h_{i-1}/6 M_{i-1} + (h_{i-1}+h_i)/3 M_i + h_i/6 M_{i+1} = slope jump at i,
// closed either by not-a-knot conditions (continuous third derivative at the
// second and second-last points) or by M = m at both ends.  The reference solves
// the system densely (gaussj); here the end values are expressed through the
// closing conditions, substituted into the first and last inner rows, and the
// inner tridiagonal system is swept by Thomas, one thread per table, FP64.  Evaluation follows the reference:
// bisection for the bracketing interval, the end cubics outside the table.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "memory.cuh"
#include "scft.h"

int scft_internal_set_error(int code, const char *msg);  // runtime.cu: records the message for scft_last_error

namespace {

struct SplineDev {
  int count;
  const int *nx, *np;
  const long long *xoff, *poff;   // table / evaluation point offsets
  const double *x, *y, *xp;
  double *yp;
  double *work;                   // 4 nx per table: lower, diagonal, upper, right-hand side
  int have_m;
  double m;
};

__global__ void spline_kernel(SplineDev s) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= s.count) return;
  const int n = s.nx[t];
  const double *x = s.x + s.xoff[t], *y = s.y + s.xoff[t];
  double *lo = s.work + 4 * s.xoff[t], *di = lo + n, *up = di + n, *rh = up + n;
  for (int i = 0; i < n; i++) { lo[i] = 0.0; di[i] = 0.0; up[i] = 0.0; rh[i] = 0.0; }
  for (int i = 1; i < n - 1; i++) {
    const double a = x[i] - x[i - 1], b = x[i + 1] - x[i];
    lo[i] = a / 6.0;
    di[i] = (x[i + 1] - x[i - 1]) / 3.0;
    up[i] = b / 6.0;
    rh[i] = (y[i + 1] - y[i]) / b - (y[i] - y[i - 1]) / a;
  }
  // The end values M0, M_{n-1} are eliminated from the inner rows 1 and n-2
  // (M = m at both ends, or the not-a-knot conditions
  // M0 = (1 + h0/h1) M1 - (h0/h1) M2 and its mirror), then Thomas on M1..M_{n-2}.
  double *M = rh;  // solved in place; rh[0] and rh[n-1] are unused by the sweep
  const int a = 1, b = n - 2;
  double rl = 0.0, rr = 0.0;
  if (s.have_m) {
    if (b >= a) { rh[a] -= lo[a] * s.m; rh[b] -= up[b] * s.m; }
  } else {
    rl = (x[1] - x[0]) / (x[2] - x[1]);
    rr = (x[n - 1] - x[n - 2]) / (x[n - 2] - x[n - 3]);
    di[a] += lo[a] * (1.0 + rl);
    up[a] -= lo[a] * rl;
    di[b] += up[b] * (1.0 + rr);
    lo[b] -= up[b] * rr;
  }
  for (int i = a + 1; i <= b; i++) {
    const double w = lo[i] / di[i - 1];
    di[i] -= w * up[i - 1];
    rh[i] -= w * rh[i - 1];
  }
  if (b >= a) {
    M[b] = rh[b] / di[b];
    for (int i = b - 1; i >= a; i--) M[i] = (rh[i] - up[i] * M[i + 1]) / di[i];
  }
  if (s.have_m) {
    M[0] = s.m;
    M[n - 1] = s.m;
  } else {
    M[0] = (1.0 + rl) * M[1] - rl * M[2];
    M[n - 1] = (1.0 + rr) * M[n - 2] - rr * M[n - 3];
  }
  const double *xp = s.xp + s.poff[t];
  double *yp = s.yp + s.poff[t];
  for (int k = 0; k < s.np[t]; k++) {
    int klo = 0, khi = n - 1;
    while (khi - klo > 1) {
      const int c = (khi + klo) >> 1;
      if (x[c] > xp[k]) khi = c; else klo = c;
    }
    const double h = x[khi] - x[klo], a = (x[khi] - xp[k]) / h, b = (xp[k] - x[klo]) / h;
    yp[k] = a * y[klo] + b * y[khi] + ((a * a * a - a) * M[klo] + (b * b * b - b) * M[khi]) * (h * h) / 6.0;
  }
}

int fail(int code, const std::string &msg) { return scft_internal_set_error(code, msg.c_str()); }

}  // namespace

extern "C" {

int scft_refine_bisect(int n_nodes, const double *x, double *x_new) {
  if (n_nodes < 2 || !x || !x_new) return fail(SCFT_EINVAL, "scft_refine_bisect: bad argument");
  for (int i = 0; i + 1 < n_nodes; i++) {
    if (!(x[i + 1] > x[i])) return fail(SCFT_EINVAL, "scft_refine_bisect: mesh not strictly increasing");
    x_new[2 * i] = x[i];
    x_new[2 * i + 1] = 0.5 * (x[i] + x[i + 1]);
  }
  x_new[2 * (n_nodes - 1)] = x[n_nodes - 1];
  return SCFT_OK;
}

int scft_spline(int count, const int *nx, const double *x, const double *y, const int *nxp, const double *xp,
                double *yp, const double *m) {
  if (count < 1 || !nx || !x || !y || !nxp || (!xp && count > 0) || !yp)
    return fail(SCFT_EINVAL, "scft_spline: bad argument");
  std::vector<long long> xoff(count), poff(count);
  long long tx = 0, tp = 0;
  for (int t = 0; t < count; t++) {
    if (nx[t] < 2 || (!m && nx[t] <= 3) || nxp[t] < 0)
      return fail(SCFT_EINVAL, "scft_spline: table " + std::to_string(t) +
                                   (m ? " needs 2 points" : " needs 4 points for not-a-knot ends"));
    for (int i = 1; i < nx[t]; i++)
      if (!(x[tx + i] > x[tx + i - 1]))
        return fail(SCFT_EINVAL, "scft_spline: table " + std::to_string(t) + ": x not strictly increasing");
    xoff[t] = tx;
    poff[t] = tp;
    tx += nx[t];
    tp += nxp[t];
  }
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(SCFT_ECUDA, std::string("scft_spline: ") + cudaGetErrorString(e));
  // device: x, y, xp, yp, work (4 tx) | nx, np | xoff, poff
  const size_t nd = (size_t)(2 * tx + 2 * tp + 4 * tx), ni = (size_t)(2 * count), nl = (size_t)(2 * count);
  const size_t bytes = nd * sizeof(double) + nl * sizeof(long long) + ni * sizeof(int);
  void *dbuf = nullptr, *hbuf = nullptr;
  e = scft::mem_alloc(&dbuf, bytes);
  if (e == cudaSuccess) e = scft::host_alloc(&hbuf, bytes);
  int rc = SCFT_OK;
  if (e != cudaSuccess) {
    rc = fail(SCFT_ENOMEM, "scft_spline: allocation");
  } else {
    double *hd = static_cast<double *>(hbuf), *dd = static_cast<double *>(dbuf);
    long long *hl = reinterpret_cast<long long *>(hd + nd), *dl = reinterpret_cast<long long *>(dd + nd);
    int *hi = reinterpret_cast<int *>(hl + nl), *di = reinterpret_cast<int *>(dl + nl);
    std::copy(x, x + tx, hd);
    std::copy(y, y + tx, hd + tx);
    std::copy(xp, xp + tp, hd + 2 * tx);
    std::copy(nx, nx + count, hi);
    std::copy(nxp, nxp + count, hi + count);
    std::copy(xoff.begin(), xoff.end(), hl);
    std::copy(poff.begin(), poff.end(), hl + count);
    SplineDev s{count, di, di + count, dl, dl + count, dd, dd + tx, dd + 2 * tx, dd + 2 * tx + tp,
                dd + 2 * tx + 2 * tp, m ? 1 : 0, m ? *m : 0.0};
    const size_t head = (size_t)(2 * tx + tp) * sizeof(double);
    e = cudaMemcpyAsync(dd, hd, head, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dl, hl, nl * sizeof(long long) + ni * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
      spline_kernel<<<(count + 63) / 64, 64, 0, st>>>(s);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hd + 2 * tx + tp, dd + 2 * tx + tp, tp * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) std::copy(hd + 2 * tx + tp, hd + 2 * tx + 2 * tp, yp);
    else rc = fail(SCFT_ECUDA, std::string("scft_spline: ") + cudaGetErrorString(e));
  }
  cudaStreamSynchronize(st);
  if (dbuf) scft::mem_free(dbuf);
  if (hbuf) scft::host_free(hbuf);
  cudaStreamDestroy(st);
  return rc;
}

}  // extern "C"
