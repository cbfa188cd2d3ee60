// free_energy.cu -- mean-field free energy of every instance of a batch, the
// quantity DEALII_SCFT/src/scft.cc:404-450 reports:
//   F = ( int_0^L w_h(x) f0(x) dx / f0bar / L + ln f0bar ) / (-1000),
//   f0bar = (1/L) int_0^L f0(x) dx,
// both integrals by Romberg (romint.c:21-57) over m+1 uniform samples of the
// target on [0, L] (scft.cc samples the analytic profile at 2^18 + 1 points);
// w_h is the piecewise-linear field on the instance's mesh.  One CTA per
// instance, FP64 with per-thread partial sums reduced in a fixed order.
#include <vector>

#include "batch.cuh"
#include "common.cuh"
#include "memory.cuh"
#include "scft.h"

namespace {

// Romberg weight of sample j of m+1 (the table of scft_internal_quad_table)
__device__ double romberg_weight(long long j, long long m, const double *qw) {
  if (j == 0 || j == m) return qw[15];
  const int v = __ffsll(j) - 1;
  return qw[v < 14 ? v : 14];
}

__global__ void free_energy_kernel(const int *n, const long long *node_off, const double *x, const double *w,
                                   int count, long long m, const double *f0s, const double *qw, double *F) {
  const int i = blockIdx.x;
  if (i >= count) return;
  const int nn = n[i];
  const double *xi = x + node_off[i];
  const double *wi = w + node_off[i];
  const double *fs = f0s + (long long)i * (m + 1);
  const double L = xi[nn - 1] - xi[0];
  double s_wf = 0.0, s_f = 0.0;
  for (long long j = threadIdx.x; j <= m; j += blockDim.x) {
    const double xq = xi[0] + L * (double)j / (double)m;
    int lo = 0, hi = nn - 1;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (xi[mid] <= xq) lo = mid;
      else hi = mid;
    }
    const double t = (xq - xi[lo]) / (xi[hi] - xi[lo]);
    const double wq = wi[lo] + t * (wi[hi] - wi[lo]);
    const double W = romberg_weight(j, m, qw);
    s_wf += W * wq * fs[j];
    s_f += W * fs[j];
  }
  __shared__ double red[2][32];
  for (int o = 16; o > 0; o >>= 1) {
    s_wf += __shfl_xor_sync(0xffffffffu, s_wf, o);
    s_f += __shfl_xor_sync(0xffffffffu, s_f, o);
  }
  if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = s_wf; red[1][threadIdx.x >> 5] = s_f; }
  __syncthreads();
  if (threadIdx.x == 0) {
    // a, b are the averages over [0, L] (weights of the unit interval), so
    // int w f0 dx / f0bar / L = a / b and f0bar = b
    double a = 0.0, b = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) { a += red[0][k]; b += red[1][k]; }
    F[i] = (a / b + log(b)) / (-1000.0);
  }
}

}  // namespace

int scft_internal_quad_table(int nsteps, double ds, int rule, double *qw);
int scft_internal_set_error(int code, const char *msg);
void scft_count_launches(long long n);

extern "C" int scft_batch_free_energy(scft_batch *b, int m, const double *f0_samples, double *F) {
  if (!b || !f0_samples || !F || m < 16) return scft_internal_set_error(SCFT_EINVAL, "scft_batch_free_energy");
  double qw[16];  // Romberg weights of m intervals of the unit interval
  if (scft_internal_quad_table(m, 1.0 / m, SCFT_RULE_ROMBERG, qw) != SCFT_OK)
    return scft_internal_set_error(SCFT_EINVAL, "scft_batch_free_energy: m must be a power of two >= 16");
  const size_t ns = (size_t)b->count * (m + 1);
  double *d_f = nullptr, *d_F = nullptr, *d_qw = nullptr;
  cudaError_t e = scft::mem_alloc((void **)&d_f, ns * sizeof(double));
  if (e == cudaSuccess) e = scft::mem_alloc((void **)&d_F, b->count * sizeof(double));
  if (e == cudaSuccess) e = scft::mem_alloc((void **)&d_qw, 16 * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_f, f0_samples, ns * sizeof(double), cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_qw, qw, 16 * sizeof(double), cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess) {
    free_energy_kernel<<<b->count, 256, 0, b->st>>>(b->d_n, b->d_node_off, b->d_x, b->d_w, b->count, m, d_f,
                                                    d_qw, d_F);
    scft_count_launches(1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(F, d_F, b->count * sizeof(double), cudaMemcpyDeviceToHost, b->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
  scft::mem_free(d_f);
  scft::mem_free(d_F);
  scft::mem_free(d_qw);
  if (e != cudaSuccess) return scft_internal_set_error(SCFT_ECUDA, cudaGetErrorString(e));
  return SCFT_OK;
}
