// runtime.cu -- host runtime and C ABI of libscft.
//
// * batches: per-instance device arrays, shape-class planning of the persistent
//   propagator (one work queue per class, cost-sorted), worker-slot scratch for
//   the half-contour store, Anderson state, and a CUDA graph that captures
//   several solver iterations (all class launches on forked streams, then the
//   mixing kernel) so the host only polls the count of unfinished instances;
// * the drop-in single-instance path replacing simple_FEM_1D_transient
//   (1D_FEM.c:47) and the reference solvers adm (adm.c:24), adm_chen
//   (ADM_chen_C.c:18) and broydn (broydn.c:44).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "mixing.cuh"
#include "batch.cuh"
#include "propagate_launch.cuh"
#include "memory.cuh"
#include "scft.h"

namespace scft {
cudaError_t propagate_launch_f32_a(int, int, const BatchDev &, const ClassDev &, int, cudaStream_t, int *, bool *);
cudaError_t propagate_launch_f32_b(int, int, const BatchDev &, const ClassDev &, int, cudaStream_t, int *, bool *);
cudaError_t propagate_launch_f64_a(int, int, const BatchDev &, const ClassDev &, int, cudaStream_t, int *, bool *);
cudaError_t propagate_launch_f64_b(int, int, const BatchDev &, const ClassDev &, int, cudaStream_t, int *, bool *);
cudaError_t solve_launch_f32_a(int, int, const BatchDev &, const ClassDev &, const MixDev &, int, cudaStream_t, int *);
cudaError_t solve_launch_f32_b(int, int, const BatchDev &, const ClassDev &, const MixDev &, int, cudaStream_t, int *);

// Fused FP32 solve of one shape class: launch (ctas == nullptr) or occupancy query.
static cudaError_t solve_dispatch(int C, int NW, const BatchDev &b, const ClassDev &cls, const MixDev &m, int grid,
                                  cudaStream_t st, int *ctas) {
  return NW <= 4 ? solve_launch_f32_a(C, NW, b, cls, m, grid, st, ctas)
                 : solve_launch_f32_b(C, NW, b, cls, m, grid, st, ctas);
}
long long seq_scratch_doubles(int n, int nsteps);
cudaError_t seq_propagate_launch(const BatchDev &b, int scheme, int wmode, double *scratch, const long long *off,
                                 cudaStream_t st);
int seq_block_max_nodes();
cudaError_t seq_block_launch(const BatchDev &b, int max_nodes, int scheme, int wmode, double *scratch,
                             const long long *off, cudaStream_t st);

static int solve_ctas_per_sm(int C, int NW) {
  int n = 0;
  BatchDev b{};
  ClassDev c{};
  MixDev m{};
  if (solve_dispatch(C, NW, b, c, m, 0, 0, &n) != cudaSuccess) return 0;
  return n;
}

static cudaError_t dispatch(int prec, int C, int NW, const BatchDev &b, const ClassDev &cls, int grid,
                            cudaStream_t st, int *ctas, bool *exists) {
  const bool small = NW <= 4;
  if (prec == PREC_F32)
    return small ? propagate_launch_f32_a(C, NW, b, cls, grid, st, ctas, exists)
                 : propagate_launch_f32_b(C, NW, b, cls, grid, st, ctas, exists);
  return small ? propagate_launch_f64_a(C, NW, b, cls, grid, st, ctas, exists)
               : propagate_launch_f64_b(C, NW, b, cls, grid, st, ctas, exists);
}

int propagate_cta_threads(int C, int NW) {
  (void)C;
  const int T = 32 * NW;
  return T >= 64 ? T : 64;
}
int propagate_groups_per_cta(int C, int NW) {
  (void)C;
  const int T = 32 * NW;
  return T >= 64 ? 1 : 64 / T;
}
bool propagate_has_class(int prec, int C, int NW) {
  bool ex = false;
  BatchDev b{};
  ClassDev c{};
  dispatch(prec, C, NW, b, c, 0, 0, nullptr, &ex);
  return ex;
}
int propagate_ctas_per_sm(int prec, int C, int NW) {
  int n = 0;
  BatchDev b{};
  ClassDev c{};
  if (dispatch(prec, C, NW, b, c, 0, 0, &n, nullptr) != cudaSuccess) return 0;
  return n;
}
cudaError_t propagate_launch(int prec, int C, int NW, const BatchDev &b, const ClassDev &cls, int grid,
                             cudaStream_t st) {
  return dispatch(prec, C, NW, b, cls, grid, st, nullptr, nullptr);
}

}  // namespace scft

using namespace scft;

// ---------------------------------------------------------------------------
// errors and counters
// ---------------------------------------------------------------------------
static thread_local std::string g_err = "";
static std::atomic<long long> g_launches{0};
void scft_count_launches(long long n) { g_launches += n; }

static int set_err(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return set_err(SCFT_ECUDA, "%s: %s", #call, cudaGetErrorString(e_));   \
  } while (0)

template <typename T>
static int dalloc(T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = mem_alloc((void **)p, n * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    return set_err(SCFT_ENOMEM, "device allocation of %zu bytes: %s", n * sizeof(T), cudaGetErrorString(e));
  }
  return SCFT_OK;
}
template <typename T>
static void dfree(T *&p) {
  if (p) mem_free((void *)p);
  p = nullptr;
}

static int device_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  return sms;
}

static int next_pow2(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

// Default propagator shape: C nodes per thread up to 8 (FP32) / 4 (FP64), then
// as few warps as cover the interior unknowns.
static void default_shape(int N, int prec, int *C, int *NW) {
  int cmax = (prec == PREC_F32) ? 8 : 4;
  int c = std::min(cmax, next_pow2((N + 31) / 32));
  int nw = next_pow2((N + 32 * c - 1) / (32 * c));
  if (nw > 32 && c < 8) {
    c = 8;
    nw = next_pow2((N + 32 * c - 1) / (32 * c));
  }
  *C = c;
  *NW = nw;
}

// Quadrature weight table: [v] = weight of sample k with 2-adic valuation v (v <
// 15), [15] = weight of k = 0 and k = nsteps.  Romberg (romint.c:21-57) is linear
// in the samples: the last five trapezoid levels combined with the Lagrange
// coefficients at h = 0 of the Neville extrapolation in h_j = 4^-j.
static int quad_table(int nsteps, double ds, int rule, double *qw) {
  if (rule == SCFT_RULE_TRAPEZOID) {
    for (int v = 0; v < 15; v++) qw[v] = ds;
    qw[15] = 0.5 * ds;
    return SCFT_OK;
  }
  int lv = 0;
  while ((1 << lv) < nsteps) lv++;
  if ((1 << lv) != nsteps || lv < 4) return SCFT_EINVAL;
  double h[5], cf[5];
  for (int a = 0; a < 5; a++) h[a] = std::pow(0.25, (double)(lv - 4 + a));
  for (int a = 0; a < 5; a++) {
    double c = 1.0;
    for (int b2 = 0; b2 < 5; b2++)
      if (b2 != a) c *= (0.0 - h[b2]) / (h[a] - h[b2]);
    cf[a] = c;
  }
  auto weight = [&](int k) {
    double W = 0.0;
    for (int a = 0; a < 5; a++) {
      const int j = lv - 4 + a;  // level with 2^j intervals
      const int stride = nsteps >> j;
      if (k % stride) continue;
      W += cf[a] * stride * ds * ((k == 0 || k == nsteps) ? 0.5 : 1.0);
    }
    return W;
  };
  for (int v = 0; v < 15; v++) qw[v] = (v < lv) ? weight(1 << v) : weight(0) * 2.0;
  qw[15] = weight(0);
  return SCFT_OK;
}

// Internal helpers shared with the no-allocation entry point (noalloc.cu).
int scft_internal_default_shape(int n_interior, int precision, int *C, int *NW) {
  if (precision != PREC_F32 && precision != PREC_F64) return SCFT_EINVAL;
  default_shape(n_interior, precision, C, NW);
  return (*NW <= 32 && 32 * *NW * *C >= n_interior && propagate_has_class(precision, *C, *NW)) ? SCFT_OK
                                                                                                 : SCFT_EINVAL;
}
int scft_internal_quad_table(int nsteps, double ds, int rule, double *qw) {
  return quad_table(nsteps, ds, rule, qw);
}
int scft_internal_set_error(int code, const char *msg) { return set_err(code, "%s", msg); }

// ---------------------------------------------------------------------------
// batch
// ---------------------------------------------------------------------------
BatchDev batch_dev(const scft_batch *B) {
  BatchDev b;
  b.count = B->count;
  b.n = B->d_n;
  b.nsteps = B->d_nsteps;
  b.ds = B->d_ds;
  b.node_off = B->d_node_off;
  b.x = B->d_x;
  b.w = B->d_w;
  b.phi = B->d_phi;
  b.Q = B->d_Q;
  b.qw = B->d_qw;
  b.active = B->d_active;
  b.status = B->d_status;
  return b;
}

static void free_plans(scft_batch *B, int p) {
  for (auto &c : B->plans[p]) {
    dfree(c.d_items);
    if (c.scratch) mem_free(c.scratch);
    c.scratch = nullptr;
  }
  B->plans[p].clear();
  B->planned[p] = false;
}

static int ensure_streams(scft_batch *B, int nside) {
  if (!B->st) {
    CK(cudaStreamCreateWithFlags(&B->st, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&B->ev_fork, cudaEventDisableTiming));
  }
  while ((int)B->side.size() < nside) {
    cudaStream_t s;
    cudaEvent_t e;
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    B->side.push_back(s);
    B->ev_join.push_back(e);
  }
  return SCFT_OK;
}

// Plan the shape classes of precision p with `frac` of the GPU's resident CTAs;
// `paths` forked paths per instance may add thread groups to a class beyond one
// per instance (a class of few instances then runs its forks side by side).
static int plan(scft_batch *B, int p, double frac, int paths = 0) {
  if (B->planned[p] && B->plan_frac[p] == frac && B->plan_paths[p] == paths) return SCFT_OK;
  free_plans(B, p);
  const int sms = device_sms();
  if (sms <= 0) return set_err(SCFT_ENODEV, "no CUDA device");
  std::map<std::pair<int, int>, std::vector<int>> groups;
  double total = 0.0;
  for (int i = 0; i < B->count; i++) {
    int C = B->shapeC[p][i], NW = B->shapeNW[p][i];
    if (C == 0) default_shape(B->n[i] - 2, p, &C, &NW);
    if (NW > 32 || !propagate_has_class(p, C, NW) || 32 * NW * C < B->n[i] - 2)
      return set_err(SCFT_EINVAL, "instance %d: %d interior nodes exceed the largest propagator shape", i,
                     B->n[i] - 2);
    groups[{C, NW}].push_back(i);
    total += (double)B->n[i] * B->nsteps[i];
  }
  for (auto &kv : groups) {
    ClassPlan c;
    c.prec = p;
    c.C = kv.first.first;
    c.NW = kv.first.second;
    c.items = kv.second;
    std::stable_sort(c.items.begin(), c.items.end(), [&](int a, int b) {
      return (double)B->n[a] * B->nsteps[a] > (double)B->n[b] * B->nsteps[b];
    });
    double cost = 0.0;
    int maxhalf = 0;
    for (int i : c.items) {
      cost += (double)B->n[i] * B->nsteps[i];
      maxhalf = std::max(maxhalf, B->nsteps[i] / 2);
    }
    // resident CTAs per SM: FP32 classes may also run as the fused solve kernel,
    // whose register budget can allow more; size the workers for the larger
    int cps = std::max(1, propagate_ctas_per_sm(p, c.C, c.NW));
    if (p == PREC_F32) cps = std::max(cps, solve_ctas_per_sm(c.C, c.NW));
    c.gpc = propagate_groups_per_cta(c.C, c.NW);
    int budget = (int)std::floor(cost / total * frac * cps * sms + 0.5);
    budget = std::max(1, budget);
    // cluster classes: one group per cluster of CL CTAs
    const int CL = cluster_ctas(p == PREC_F64, c.C, c.NW);
    c.workers = (int)std::min((long long)c.items.size() * (1 + paths),
                              std::max(1LL, (long long)budget * c.gpc / CL));
    // A class with a small share of the cost would otherwise get a handful of
    // groups that run its instances one after another, a chain as long as the
    // large classes' whole solve: one-CTA classes get at least one group per
    // instance up to 64 (a few CTAs, nothing next to the large classes).
    if (CL == 1) c.workers = std::max(c.workers, (int)std::min<size_t>(c.items.size(), 64));
    c.grid = (c.workers + c.gpc - 1) / c.gpc * CL;
    c.slot_elems = (long long)(maxhalf + 1) * 32 * c.NW * c.C;
    const size_t esz = (p == PREC_F32) ? 4 : 8;
    for (;;) {
      cudaError_t e = mem_alloc(&c.scratch, (size_t)c.workers * c.slot_elems * esz);
      if (e == cudaSuccess) break;
      cudaGetLastError();
      c.scratch = nullptr;
      if (c.workers <= 1) return set_err(SCFT_ENOMEM, "propagator scratch: %s", cudaGetErrorString(e));
      c.workers = (c.workers + 1) / 2;
      c.grid = (c.workers + c.gpc - 1) / c.gpc * CL;
    }
    int rc = dalloc(&c.d_items, c.items.size());
    if (rc) return rc;
    CK(cudaMemcpy(c.d_items, c.items.data(), c.items.size() * sizeof(int), cudaMemcpyHostToDevice));
    B->plans[p].push_back(c);
  }
  // queue heads: precision 0 classes first, then precision 1
  int nh = 0;
  for (int q = 0; q < 2; q++)
    for (auto &c : B->plans[q]) c.head = nh++;
  if (nh > B->nheads) {
    dfree(B->d_heads);
    int rc = dalloc(&B->d_heads, (size_t)nh);
    if (rc) return rc;
    B->nheads = nh;
  }
  B->planned[p] = true;
  B->plan_frac[p] = frac;
  B->plan_paths[p] = paths;
  return ensure_streams(B, (int)std::max(B->plans[0].size(), B->plans[1].size()));
}

static void class_dev(const scft_batch *B, const ClassPlan &c, ClassDev *d) {
  d->items = c.d_items;
  d->count = (int)c.items.size();
  d->head = B->d_heads + c.head;
  d->scratch = c.scratch;
  d->slot_elems = c.slot_elems;
  d->workers = c.workers;
  d->want = c.prec == PREC_F32 ? 1 : 2;
}

// Index of the live-statistics slot of (iteration k of a graph, precision p, class i).
static int live_index(const scft_batch *B, int k, int p, int i) { return (k * 2 + p) * B->live_maxc + i; }

// Enqueue one propagator pass of precision p on B->st (forked over class streams).
// live_k >= 0 (inside a solve graph): each class launch is bracketed by external
// event records on its stream and counts its work into the live slot.
static int enqueue_propagate(scft_batch *B, int p, int live_k = -1) {
  auto &plans = B->plans[p];
  if (plans.empty()) return SCFT_OK;
  const BatchDev b = batch_dev(B);
  for (auto &c : plans) CK(cudaMemsetAsync(B->d_heads + c.head, 0, sizeof(int), B->st));
  auto launch = [&](size_t i, cudaStream_t s) -> int {
    ClassDev d;
    class_dev(B, plans[i], &d);
    int li = -1;
    if (live_k >= 0) {
      li = live_index(B, live_k, p, (int)i);
      d.work = B->d_work + li;
      CK(cudaEventRecordWithFlags(B->ev_live[2 * li], s, cudaEventRecordExternal));
    }
    CK(propagate_launch(p, plans[i].C, plans[i].NW, b, d, plans[i].grid, s));
    g_launches++;
    if (li >= 0) CK(cudaEventRecordWithFlags(B->ev_live[2 * li + 1], s, cudaEventRecordExternal));
    return SCFT_OK;
  };
  if (plans.size() == 1) return launch(0, B->st);
  CK(cudaEventRecord(B->ev_fork, B->st));
  for (size_t i = 0; i < plans.size(); i++) {
    CK(cudaStreamWaitEvent(B->side[i], B->ev_fork, 0));
    int rc = launch(i, B->side[i]);
    if (rc) return rc;
    CK(cudaEventRecord(B->ev_join[i], B->side[i]));
  }
  for (size_t i = 0; i < plans.size(); i++) CK(cudaStreamWaitEvent(B->st, B->ev_join[i], 0));
  return SCFT_OK;
}

// Make room for the live statistics of K iterations per graph.
static int live_prepare(scft_batch *B, int K) {
  const int maxc = (int)std::max<size_t>(1, std::max(B->plans[0].size(), B->plans[1].size()));
  const int need = K * 2 * maxc;
  if (need > B->live_cap) {
    if (B->d_work) mem_free(B->d_work);
    if (B->h_work) host_free(B->h_work);
    B->d_work = nullptr;
    B->h_work = nullptr;
    CK(mem_alloc((void **)&B->d_work, need * sizeof(unsigned long long)));
    CK(host_alloc((void **)&B->h_work, need * sizeof(unsigned long long)));
    while ((int)B->ev_live.size() < 2 * need) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      B->ev_live.push_back(e);
    }
    B->live_cap = need;
  }
  B->live_maxc = maxc;
  for (int p = 0; p < 2; p++) {
    B->live_ms[p].assign(B->plans[p].size(), 0.0);
    B->live_units[p].assign(B->plans[p].size(), 0.0);
    B->live_launches[p].assign(B->plans[p].size(), 0);
  }
  return SCFT_OK;
}

// After a replay: accumulate the launches of that replay that evaluated anything.
static int live_collect(scft_batch *B, int K, bool f32, bool f64) {
  for (int k = 0; k < K; k++)
    for (int p = 0; p < 2; p++) {
      if ((p == PREC_F32 && !f32) || (p == PREC_F64 && !f64)) continue;
      for (size_t i = 0; i < B->plans[p].size(); i++) {
        const int li = live_index(B, k, p, (int)i);
        const unsigned long long u = B->h_work[li];
        if (u == 0) continue;
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, B->ev_live[2 * li], B->ev_live[2 * li + 1]));
        B->live_ms[p][i] += ms;
        B->live_units[p][i] += (double)u;
        B->live_launches[p][i]++;
      }
    }
  return SCFT_OK;
}

__global__ void fill_int_kernel(int *a, int n, int v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}
__global__ void fill_double_kernel(double *a, long long n, double v) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}
// The solve's deadline on the device clock: now + budget.
// instances outside the selection take no part in the solve
__global__ void select_kernel(int *active, const int *select, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !select[i]) active[i] = 0;
}

// Start of a second-stage instance of a staged solve: its interior field is
// interpolated in the film width between two solved neighbours of the same
// mesh shape, node by node: w_i = (1 - t) w_a + t w_b.  One CTA per instance;
// plan[4k .. 4k+2] = (i, a, b), tt[k] = t.
__global__ void transfer_kernel(const int *plan, const double *tt, int m, const int *n, const long long *node_off,
                                double *w) {
  const int k = blockIdx.x;
  if (k >= m) return;
  const int i = plan[4 * k], a = plan[4 * k + 1], bb = plan[4 * k + 2];
  const double t = tt[k];
  const int ni = n[i];
  if (n[a] != ni || n[bb] != ni) return;
  double *wi = w + node_off[i];
  const double *wa = w + node_off[a], *wb = w + node_off[bb];
  // each product and the sum rounded on its own (no fused multiply-add), as
  // the same formula evaluates on the host
  const double s = __dadd_rn(1.0, -t);
  for (int j = 1 + threadIdx.x; j < ni - 1; j += blockDim.x) wi[j] = __dadd_rn(__dmul_rn(s, wa[j]), __dmul_rn(t, wb[j]));
}

__global__ void set_deadline_kernel(unsigned long long *deadline, unsigned long long budget_ns) {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  *deadline = t + budget_ns;
}

__global__ void count_active_kernel(const int *a, int n, int *out) {
  __shared__ int s;
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  int c = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) c += (a[i] != 0);
  atomicAdd(&s, c);
  __syncthreads();
  if (threadIdx.x == 0) *out = s;
}

static int fill_int(int *a, int n, int v, cudaStream_t st) {
  if (n <= 0) return SCFT_OK;
  fill_int_kernel<<<(n + 255) / 256, 256, 0, st>>>(a, n, v);
  g_launches++;
  CK(cudaGetLastError());
  return SCFT_OK;
}
static int fill_double(double *a, long long n, double v, cudaStream_t st) {
  if (n <= 0) return SCFT_OK;
  fill_double_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a, n, v);
  g_launches++;
  CK(cudaGetLastError());
  return SCFT_OK;
}

static void free_mix(scft_batch *B) {
  dfree(B->d_graw); dfree(B->d_gcur); dfree(B->d_gprev); dfree(B->d_wprev);
  dfree(B->d_hdx); dfree(B->d_hdg); dfree(B->d_gram); dfree(B->d_err); dfree(B->d_best); dfree(B->d_lk);
  dfree(B->d_ref_err); dfree(B->d_ref_it); dfree(B->d_deadline);
  dfree(B->d_iters); dfree(B->d_hcount); dfree(B->d_hhead); dfree(B->d_nactive);
  if (B->h_nactive) host_free(B->h_nactive);
  B->h_nactive = nullptr;
  B->depth = 0;
}

// Replace a device array of n_old elements by one of n_new, keeping the first n_old.
template <typename T>
static int grow_array(T *&p, size_t n_old, size_t n_new) {
  T *q = nullptr;
  int rc = dalloc(&q, n_new);
  if (rc) return rc;
  if (p && n_old) CK(cudaMemcpy(q, p, n_old * sizeof(T), cudaMemcpyDeviceToDevice));
  dfree(p);
  p = q;
  return SCFT_OK;
}

// Anderson state for history depth `depth` and room for `paths` forked paths
// per instance (the capacity only grows).
static int ensure_mix(scft_batch *B, int depth, int paths = 0) {
  paths = std::max(paths, B->paths);
  if (B->depth == depth && B->paths == paths) return SCFT_OK;
  int rc;
  if (paths > B->paths) {
    const size_t no = (size_t)B->total_nodes, c = (size_t)B->count, f0 = 1 + B->paths, f1 = 1 + paths;
    if ((rc = grow_array(B->d_w, no * f0, no * f1)) || (rc = grow_array(B->d_phi, no * f0, no * f1)) ||
        (rc = grow_array(B->d_Q, c * f0, c * f1)) || (rc = grow_array(B->d_status, c * f0, c * f1)) ||
        (rc = grow_array(B->d_active, c * f0, c * f1)))
      return rc;
    dfree(B->d_win);
    dfree(B->d_fork_it);
    if ((rc = dalloc(&B->d_win, c)) || (rc = dalloc(&B->d_fork_it, c))) return rc;
  }
  free_mix(B);
  B->paths = paths;
  const size_t f = 1 + (size_t)paths;
  const size_t ni = (size_t)B->total_int * f, c = (size_t)B->count * f;
  if ((rc = dalloc(&B->d_graw, ni)) || (rc = dalloc(&B->d_gcur, ni)) || (rc = dalloc(&B->d_gprev, ni)) ||
      (rc = dalloc(&B->d_wprev, ni)) || (rc = dalloc(&B->d_hdx, ni * depth)) ||
      (rc = dalloc(&B->d_hdg, ni * depth)) || (rc = dalloc(&B->d_gram, c * depth * depth)) ||
      (rc = dalloc(&B->d_err, c)) || (rc = dalloc(&B->d_best, c)) || (rc = dalloc(&B->d_lk, c)) || (rc = dalloc(&B->d_iters, c)) ||
      (rc = dalloc(&B->d_hcount, c)) || (rc = dalloc(&B->d_hhead, c)) || (rc = dalloc(&B->d_nactive, 1)) ||
      (rc = dalloc(&B->d_ref_err, c)) || (rc = dalloc(&B->d_ref_it, c)) || (rc = dalloc(&B->d_deadline, 1)))
    return rc;
  CK(host_alloc((void **)&B->h_nactive, sizeof(int)));
  B->depth = depth;
  return SCFT_OK;
}

// Copies the winning forked path of every instance into the instance's own
// slots (field, density, Q, error, iterations, status); win[i] = iterations * 16
// + path of the winner, INT_MAX when no path converged.
__global__ void resolve_forks_kernel(int count, const int *n, const long long *node_off, long long rep_nodes,
                                     const int *win, double *w, double *phi, double *Q, double *err, int *iters,
                                     int *status, int *active) {
  const int i = blockIdx.x;
  const int key = win[i];
  if (key == 0x7fffffff) return;
  const int r = key & 15;
  if (r == 0) return;
  const int v = r * count + i;
  const long long o = node_off[i], ro = o + r * rep_nodes;
  for (int j = threadIdx.x; j < n[i]; j += blockDim.x) {
    w[o + j] = w[ro + j];
    phi[o + j] = phi[ro + j];
  }
  if (threadIdx.x == 0) {
    Q[i] = Q[v];
    err[i] = err[v];
    iters[i] = iters[v];
    status[i] = status[v] | ST_FORKED;
    active[i] = 0;
  }
}

static void destroy_batch(scft_batch *B) {
  dfree(B->d_seq);
  dfree(B->d_seq_off);
  if (!B) return;
  if (B->st) cudaStreamSynchronize(B->st);
  free_plans(B, 0);
  free_plans(B, 1);
  free_mix(B);
  dfree(B->d_n); dfree(B->d_nsteps); dfree(B->d_active); dfree(B->d_status);
  dfree(B->d_ds); dfree(B->d_x); dfree(B->d_f0); dfree(B->d_w); dfree(B->d_phi);
  dfree(B->d_Q); dfree(B->d_qw); dfree(B->d_node_off); dfree(B->d_int_off); dfree(B->d_heads);
  dfree(B->d_w0);
  dfree(B->d_spacing);
  dfree(B->d_select);
  dfree(B->d_win);
  dfree(B->d_fork_it);
  dfree(B->d_fork);
  if (B->h_fork) host_free(B->h_fork);
  B->h_fork = nullptr;
  if (B->t0) cudaEventDestroy(B->t0);
  if (B->t1) cudaEventDestroy(B->t1);
  for (auto s : B->side) cudaStreamDestroy(s);
  for (auto e : B->ev_join) cudaEventDestroy(e);
  for (auto e : B->ev_live) cudaEventDestroy(e);
  if (B->d_work) mem_free(B->d_work);
  if (B->h_work) host_free(B->h_work);
  if (B->ev_fork) cudaEventDestroy(B->ev_fork);
  if (B->st) cudaStreamDestroy(B->st);
  delete B;
}

// Host work over [0, n) split across up to 8 threads when there is enough of
// it (packing and unpacking the batch arrays): f(begin, end) on each share.
template <typename F>
static void host_parallel(long long n, long long grain, F f) {
  const long long hw = std::max(1u, std::thread::hardware_concurrency());
  const int T = (int)std::min<long long>(std::min<long long>(8, hw), std::max(1LL, n / std::max(1LL, grain)));
  if (T <= 1) {
    f(0LL, n);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 1; t < T; t++) th.emplace_back(f, n * t / T, n * (t + 1) / T);
  f(0LL, n / T);
  for (auto &x : th) x.join();
}

static int create_batch(const scft_instance *inst, int count, scft_batch **out) {
  if (!inst || count <= 0 || !out) return set_err(SCFT_EINVAL, "batch: no instances");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_err(SCFT_ENODEV, "no CUDA device");
  }
  scft_batch *B = new scft_batch();
  B->count = count;
  B->n.resize(count); B->nsteps.resize(count); B->rule.resize(count); B->ds.resize(count);
  B->node_off.resize(count); B->int_off.resize(count); B->spacing_ratio.resize(count); B->width.resize(count);
  for (int p = 0; p < 2; p++) { B->shapeC[p].assign(count, 0); B->shapeNW[p].assign(count, 0); }
  // per instance (in parallel): validity, spacing ratio, width; 0 or the
  // error (1 description, 2 Romberg step count, 3 mesh order)
  std::vector<int> bad(count, 0);
  host_parallel(count, 256, [&](long long i0, long long i1) {
    for (long long i = i0; i < i1; i++) {
      const scft_instance &s = inst[i];
      if (s.n_nodes < 3 || s.nsteps < 1 || !(s.ds > 0.0) || !s.f0 ||
          (s.rule != SCFT_RULE_ROMBERG && s.rule != SCFT_RULE_TRAPEZOID) || (!s.x && !(s.L > 0.0))) {
        bad[i] = 1;
        continue;
      }
      double qw[16];
      if (quad_table(s.nsteps, s.ds, s.rule, qw)) {
        bad[i] = 2;
        continue;
      }
      double hmin = 1.0, hmax = 1.0;  // uniform when x is not given
      if (s.x) {
        hmin = INFINITY;
        hmax = 0.0;
        for (int k = 1; k < s.n_nodes; k++) {
          const double h = s.x[k] - s.x[k - 1];
          if (!(h > 0.0)) {
            bad[i] = 3;
            break;
          }
          hmin = std::min(hmin, h);
          hmax = std::max(hmax, h);
        }
        if (bad[i]) continue;
      }
      B->spacing_ratio[i] = hmax / hmin;
      B->width[i] = s.x ? s.x[s.n_nodes - 1] - s.x[0] : s.L;
    }
  });
  long long no = 0, io = 0;
  for (int i = 0; i < count; i++) {
    if (bad[i]) {
      destroy_batch(B);
      if (bad[i] == 1) return set_err(SCFT_EINVAL, "instance %d: invalid description", i);
      if (bad[i] == 2) return set_err(SCFT_EINVAL, "instance %d: Romberg needs a power-of-two step count >= 16", i);
      return set_err(SCFT_EINVAL, "instance %d: mesh not strictly increasing", i);
    }
    const scft_instance &s = inst[i];
    B->n[i] = s.n_nodes; B->nsteps[i] = s.nsteps; B->rule[i] = s.rule; B->ds[i] = s.ds;
    B->node_off[i] = no; B->int_off[i] = io;
    no += s.n_nodes; io += s.n_nodes - 2;
  }
  B->total_nodes = no; B->total_int = io;
  int rc;
  if ((rc = dalloc(&B->d_n, count)) || (rc = dalloc(&B->d_nsteps, count)) || (rc = dalloc(&B->d_active, count)) ||
      (rc = dalloc(&B->d_status, count)) || (rc = dalloc(&B->d_ds, count)) || (rc = dalloc(&B->d_x, no)) ||
      (rc = dalloc(&B->d_f0, no)) || (rc = dalloc(&B->d_w, no)) || (rc = dalloc(&B->d_phi, no)) ||
      (rc = dalloc(&B->d_Q, count)) || (rc = dalloc(&B->d_qw, 16 * (size_t)count)) ||
      (rc = dalloc(&B->d_node_off, count)) || (rc = dalloc(&B->d_int_off, count)) ||
      (rc = dalloc(&B->d_w0, no)) || (rc = dalloc(&B->d_spacing, count))) {
    destroy_batch(B);
    return rc;
  }
  rc = ensure_streams(B, 1);
  if (rc) { destroy_batch(B); return rc; }
  if (cudaEventCreate(&B->t0) != cudaSuccess || cudaEventCreate(&B->t1) != cudaSuccess) {
    destroy_batch(B);
    return set_err(SCFT_ECUDA, "event creation failed");
  }
  // one pinned staging buffer (from the library's cache) for every upload
  const size_t nd = (size_t)no, nc = (size_t)count;
  const size_t stage_doubles = 3 * nd + 16 * nc + 2 * nc + 2 * nc + nc;  // x, f0, w | qw | ds, spacing | offsets | n+nsteps
  double *stage = nullptr;
  if (host_alloc((void **)&stage, stage_doubles * sizeof(double)) != cudaSuccess) {
    destroy_batch(B);
    return set_err(SCFT_ENOMEM, "pinned staging buffer of %zu bytes", stage_doubles * sizeof(double));
  }
  double *hx = stage, *hf = hx + nd, *hw = hf + nd, *hqw = hw + nd, *hds = hqw + 16 * nc, *hsp = hds + nc;
  long long *hno = reinterpret_cast<long long *>(hsp + nc), *hio = hno + nc;
  int *hn = reinterpret_cast<int *>(hio + nc), *hns = hn + nc;
  host_parallel(count, 256, [&](long long i0, long long i1) {
    for (long long i = i0; i < i1; i++) {
      const scft_instance &s = inst[i];
      const long long o = B->node_off[i];
      if (s.x) std::memcpy(hx + o, s.x, s.n_nodes * sizeof(double));
      else
        for (int k = 0; k < s.n_nodes; k++) hx[o + k] = s.L * (double)k / (double)(s.n_nodes - 1);
      std::memcpy(hf + o, s.f0, s.n_nodes * sizeof(double));
      if (s.w0) std::memcpy(hw + o, s.w0, s.n_nodes * sizeof(double));
      else std::memset(hw + o, 0, s.n_nodes * sizeof(double));
      if (!s.x) hx[o + s.n_nodes - 1] = s.L;
      quad_table(s.nsteps, s.ds, s.rule, hqw + 16 * (size_t)i);
      hds[i] = s.ds;
      hsp[i] = B->spacing_ratio[i];
      hno[i] = o;
      hio[i] = B->int_off[i];
      hn[i] = s.n_nodes;
      hns[i] = s.nsteps;
    }
  });
  cudaStream_t st = B->st;
  struct Cp { void *d; const void *h; size_t bytes; } cps[] = {
      {B->d_n, hn, nc * sizeof(int)},
      {B->d_nsteps, hns, nc * sizeof(int)},
      {B->d_ds, hds, nc * sizeof(double)},
      {B->d_spacing, hsp, nc * sizeof(double)},
      {B->d_node_off, hno, nc * sizeof(long long)},
      {B->d_int_off, hio, nc * sizeof(long long)},
      {B->d_x, hx, nd * sizeof(double)},
      {B->d_f0, hf, nd * sizeof(double)},
      {B->d_w, hw, nd * sizeof(double)},
      {B->d_w0, hw, nd * sizeof(double)},
      {B->d_qw, hqw, 16 * nc * sizeof(double)},
  };
  for (auto &c : cps) {
    cudaError_t e = cudaMemcpyAsync(c.d, c.h, c.bytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
      cudaStreamSynchronize(st);
      host_free(stage);
      destroy_batch(B);
      return set_err(SCFT_ECUDA, "upload: %s", cudaGetErrorString(e));
    }
  }
  cudaMemsetAsync(B->d_status, 0, count * sizeof(int), st);
  cudaMemsetAsync(B->d_phi, 0, no * sizeof(double), st);
  cudaError_t e = cudaStreamSynchronize(st);
  host_free(stage);
  if (e != cudaSuccess) { destroy_batch(B); return set_err(SCFT_ECUDA, "upload: %s", cudaGetErrorString(e)); }
  *out = B;
  return SCFT_OK;
}

static int evaluate(scft_batch *B, int p) {
  if (p != PREC_F32 && p != PREC_F64) return set_err(SCFT_EINVAL, "precision");
  int rc = plan(B, p, 1.0);
  if (rc) return rc;
  rc = fill_int(B->d_active, B->count, p == PREC_F32 ? 1 : 2, B->st);
  if (rc) return rc;
  CK(cudaMemsetAsync(B->d_status, 0, B->count * sizeof(int), B->st));
  CK(cudaEventRecord(B->t0, B->st));
  rc = enqueue_propagate(B, p);
  if (rc) return rc;
  CK(cudaEventRecord(B->t1, B->st));
  CK(cudaStreamSynchronize(B->st));
  CK(cudaEventElapsedTime(&B->last_ms, B->t0, B->t1));
  return SCFT_OK;
}

// Enqueue the scheme-general propagator for the active instances of B on B->st
// (scratch allocated on first use).
static int seq_enqueue(scft_batch *B, int scheme, int wmode) {
  if ((scheme != SCFT_SCHEME_IE && scheme != SCFT_SCHEME_IRK2) ||
      (wmode != SCFT_W_ROWSCALED && wmode != SCFT_W_CONSISTENT))
    return set_err(SCFT_EINVAL, "scheme %d / field term %d", scheme, wmode);
  if (!B->d_seq) {
    std::vector<long long> off(B->count);
    long long tot = 0;
    for (int i = 0; i < B->count; i++) {
      off[i] = tot;
      tot += seq_scratch_doubles(B->n[i], B->nsteps[i]);
    }
    int rc;
    if ((rc = dalloc(&B->d_seq, (size_t)tot)) || (rc = dalloc(&B->d_seq_off, (size_t)B->count))) return rc;
    CK(cudaMemcpyAsync(B->d_seq_off, off.data(), B->count * sizeof(long long), cudaMemcpyHostToDevice, B->st));
  }
  // block-parallel form when every instance's coefficients fit in one CTA's
  // shared memory, the one-thread form otherwise
  const int maxn = *std::max_element(B->n.begin(), B->n.end());
  if (maxn <= seq_block_max_nodes())
    CK(seq_block_launch(batch_dev(B), maxn, scheme, wmode, B->d_seq, B->d_seq_off, B->st));
  else
    CK(seq_propagate_launch(batch_dev(B), scheme, wmode, B->d_seq, B->d_seq_off, B->st));
  g_launches++;
  return SCFT_OK;
}

// Reset the per-instance solver state on B->st and describe it to the mixing step.
static int solve_begin(scft_batch *B, const scft_solve_opts *o, int p, bool verify, MixDev *mp) {
  cudaStream_t st = B->st;
  const int c = B->count;
  int rc;
  if ((rc = fill_int(B->d_active, c, p == PREC_F32 ? 1 : 2, st))) return rc;
  if (B->use_select) {
    select_kernel<<<(c + 255) / 256, 256, 0, st>>>(B->d_active, B->d_select, c);
    g_launches++;
    CK(cudaGetLastError());
  }
  CK(cudaMemsetAsync(B->d_status, 0, c * sizeof(int), st));
  CK(cudaMemsetAsync(B->d_iters, 0, c * sizeof(int), st));
  CK(cudaMemsetAsync(B->d_hcount, 0, c * sizeof(int), st));
  CK(cudaMemsetAsync(B->d_hhead, 0, c * sizeof(int), st));
  CK(cudaMemsetAsync(B->d_gram, 0, (size_t)c * o->depth * o->depth * sizeof(double), st));
  if ((rc = fill_double(B->d_best, c, INFINITY, st))) return rc;
  if ((rc = fill_double(B->d_lk, c, 1.0 - o->beta, st))) return rc;
  if ((rc = fill_double(B->d_err, c, INFINITY, st))) return rc;
  if ((rc = fill_double(B->d_ref_err, c, INFINITY, st))) return rc;
  CK(cudaMemsetAsync(B->d_ref_it, 0, c * sizeof(int), st));

  MixDev &m = *mp;
  m = MixDev();  // no forks unless the fused solve sets them
  m.count = c;
  m.n = B->d_n;
  m.node_off = B->d_node_off;
  m.int_off = B->d_int_off;
  m.x = B->d_x; m.f0 = B->d_f0; m.phi = B->d_phi; m.w = B->d_w;
  m.active = B->d_active; m.status = B->d_status; m.iters = B->d_iters; m.err = B->d_err; m.best = B->d_best;
  m.lk = B->d_lk; m.lk_schedule = o->beta_schedule; m.lmd = 1.0 - o->beta;
  m.graw = B->d_graw; m.gcur = B->d_gcur; m.gprev = B->d_gprev; m.wprev = B->d_wprev;
  m.hdx = B->d_hdx; m.hdg = B->d_hdg; m.gram = B->d_gram;
  m.hcount = B->d_hcount; m.hhead = B->d_hhead;
  m.depth = o->depth; m.maxit = o->maxit; m.mode = o->residual_mode; m.verify64 = verify ? 1 : 0;
  m.tol = o->tol; m.tol32 = o->tol * o->tol32_factor; m.clip = o->clip;
  m.grow = o->grow; m.precond = o->precond; m.reg = o->reg;
  m.ds = B->d_ds; m.weighted = o->weighted; m.step_cap = o->step_cap; m.field_floor = o->field_floor;
  m.finish_stall = (p == PREC_F32) ? o->finish_stall : 0;
  m.finish_tol = o->finish_tol;
  m.ref_err = B->d_ref_err; m.ref_it = B->d_ref_it;
  m.spacing = B->d_spacing; m.graded_ratio = o->graded_ratio; m.hfloor = o->precond_hfloor;
  m.deadline = nullptr;
  if (o->budget_ms > 0.0) {
    set_deadline_kernel<<<1, 1, 0, st>>>(B->d_deadline, (unsigned long long)(o->budget_ms * 1e6));
    g_launches++;
    CK(cudaGetLastError());
    m.deadline = B->d_deadline;
  }
  return SCFT_OK;
}

// Copy the per-instance outcome of the last solve to the caller.
static int solve_results(scft_batch *B, scft_result *res) {
  if (!res) return SCFT_OK;
  const int c = B->count;
  std::vector<int> stt(c), its(c);
  std::vector<double> err(c), Q(c);
  CK(cudaMemcpy(stt.data(), B->d_status, c * sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(its.data(), B->d_iters, c * sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(err.data(), B->d_err, c * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(Q.data(), B->d_Q, c * sizeof(double), cudaMemcpyDeviceToHost));
  for (int i = 0; i < c; i++) { res[i].status = stt[i]; res[i].iterations = its[i]; res[i].err = err[i]; res[i].Q = Q[i]; }
  return SCFT_OK;
}

static int graph_iterate(scft_batch *B, const scft_solve_opts *o, const MixDev &m, bool f32, bool f64);

// Fused FP32 solve: one persistent launch per shape class, all classes on
// forked streams.  Each thread group takes instances from its class queue
// (most expensive first) and iterates each one to the end on its own, the
// contour pass and the Anderson step back to back, so no instance waits for a
// batch-wide iteration.  Every loop is bounded by the iteration limit.
static int solve_fused_enqueue(scft_batch *B, const scft_solve_opts *o) {
  const int p = PREC_F32;
  int rc;
  if ((rc = live_prepare(B, 1))) return rc;
  cudaStream_t st = B->st;
  auto &plans = B->plans[p];
  CK(cudaEventRecord(B->t0, st));
  MixDev &m = B->pending_mix;
  if ((rc = solve_begin(B, o, p, false, &m))) return rc;
  B->pending_opts = *o;
  const size_t live_bytes = (size_t)2 * B->live_maxc * sizeof(unsigned long long);
  CK(cudaMemsetAsync(B->d_work, 0, live_bytes, st));
  for (auto &c : plans) CK(cudaMemsetAsync(B->d_heads + c.head, 0, sizeof(int), st));
  BatchDev b = batch_dev(B);
  const int nf = (o->finish_stall > 0) ? 0 : o->forks;  // forks and the FP64 hand-off exclude each other
  std::vector<size_t> fork_off(plans.size(), 0);
  if (nf > 0) {
    m.base = B->count; m.rep_nodes = B->total_nodes; m.rep_int = B->total_int;
    m.forks = nf; m.fork_at = o->fork_at; m.fork_grace = o->fork_grace; m.fork_first = o->fork_first;
    m.fork_err = o->fork_err; m.win = B->d_win; m.fork_it = B->d_fork_it;
    CK(cudaMemsetAsync(B->d_fork_it, 0, B->count * sizeof(int), st));
    for (int f = 0; f < 4; f++) m.fork_scale[f] = (f < nf) ? o->fork_scale[f] : 1.0;
    b.base = B->count; b.rep_nodes = B->total_nodes;
    if ((rc = fill_int(B->d_win, B->count, 0x7fffffff, st))) return rc;
    // per class: {published, claimed, may still fork, unused} and one entry per instance
    size_t need = 0;
    for (size_t i = 0; i < plans.size(); i++) { fork_off[i] = need; need += 4 + plans[i].items.size(); }
    if (need > B->fork_cap) {
      dfree(B->d_fork);
      if (B->h_fork) host_free(B->h_fork);
      B->h_fork = nullptr;
      B->fork_cap = 0;
      if ((rc = dalloc(&B->d_fork, need))) return rc;
      CK(host_alloc((void **)&B->h_fork, need * sizeof(int)));
      B->fork_cap = need;
    }
    std::fill(B->h_fork, B->h_fork + need, 0);
    for (size_t i = 0; i < plans.size(); i++) B->h_fork[fork_off[i] + 2] = (int)plans[i].items.size();
    CK(cudaMemcpyAsync(B->d_fork, B->h_fork, need * sizeof(int), cudaMemcpyHostToDevice, st));
  }
  B->pending_start = std::chrono::steady_clock::now();
  CK(cudaEventRecord(B->ev_fork, st));
  for (size_t i = 0; i < plans.size(); i++) {
    const ClassPlan &c = plans[i];
    cudaStream_t s = B->side[i];
    CK(cudaStreamWaitEvent(s, B->ev_fork, 0));
    ClassDev d;
    class_dev(B, c, &d);
    const int li = live_index(B, 0, p, (int)i);
    d.work = B->d_work + li;
    if (nf > 0) {
      d.fork_ctl = B->d_fork + fork_off[i];
      d.fork_list = d.fork_ctl + 4;
    }
    // keep the class's share resident if the fused kernel fits fewer CTAs per SM
    // than the plan assumed
    int grid = c.grid;
    const int occ = solve_ctas_per_sm(c.C, c.NW);
    const int pocc = std::max(propagate_ctas_per_sm(p, c.C, c.NW), occ);
    if (occ <= 0) return set_err(SCFT_ECUDA, "fused solve of class (%d, %d) does not fit an SM", c.C, c.NW);
    if (pocc > occ) grid = std::max(1, (int)((long long)c.grid * occ / pocc));
    d.workers = std::min(c.workers, grid * c.gpc);
    grid = std::min(grid, (d.workers + c.gpc - 1) / c.gpc);
    CK(cudaEventRecord(B->ev_live[2 * li], s));
    CK(solve_dispatch(c.C, c.NW, b, d, m, grid, s, nullptr));
    g_launches++;
    CK(cudaEventRecord(B->ev_live[2 * li + 1], s));
    CK(cudaEventRecord(B->ev_join[i], s));
  }
  for (size_t i = 0; i < plans.size(); i++) CK(cudaStreamWaitEvent(st, B->ev_join[i], 0));
  if (nf > 0) {
    resolve_forks_kernel<<<B->count, 128, 0, st>>>(B->count, B->d_n, B->d_node_off, B->total_nodes, B->d_win,
                                                    B->d_w, B->d_phi, B->d_Q, B->d_err, B->d_iters,
                                                    B->d_status, B->d_active);
    g_launches++;
    CK(cudaGetLastError());
  }
  CK(cudaMemcpyAsync(B->h_work, B->d_work, live_bytes, cudaMemcpyDeviceToHost, st));
  count_active_kernel<<<1, 256, 0, st>>>(B->d_active, B->count, B->d_nactive);
  g_launches++;
  CK(cudaMemcpyAsync(B->h_nactive, B->d_nactive, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaEventRecord(B->t1, st));
  B->pending = true;
  return SCFT_OK;
}

// Completes the solve enqueued by solve_fused_enqueue: statistics, the FP64
// continuation of instances whose FP32 iteration stalled, results.
static int solve_fused_finish(scft_batch *B, scft_result *res) {
  if (!B->pending) return set_err(SCFT_EINVAL, "no solve of this batch is in flight");
  B->pending = false;
  cudaStream_t st = B->st;
  int rc;
  cudaError_t e = cudaEventSynchronize(B->t1);
  if (e != cudaSuccess) return set_err(SCFT_ECUDA, "fused solve: %s", cudaGetErrorString(e));
  if ((rc = live_collect(B, 1, true, false))) return rc;
  B->trace_active.assign(1, *B->h_nactive);
  B->trace_ms.assign(1, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() -
                                                                   B->pending_start).count());
  // instances whose FP32 iteration stalled (active == 2) finish with the FP64
  // propagator, batch-wide iterations over those instances only
  if (*B->h_nactive > 0) {
    if ((rc = plan(B, PREC_F64, 1.0))) return rc;
    std::vector<double> ms32 = B->live_ms[PREC_F32], un32 = B->live_units[PREC_F32];
    std::vector<long long> ln32 = B->live_launches[PREC_F32];
    if ((rc = graph_iterate(B, &B->pending_opts, B->pending_mix, false, true))) return rc;
    // keep the fused launch's statistics for the FP32 classes
    B->live_ms[PREC_F32] = ms32; B->live_units[PREC_F32] = un32; B->live_launches[PREC_F32] = ln32;
    CK(cudaEventRecord(B->t1, st));
    CK(cudaEventSynchronize(B->t1));
  }
  CK(cudaEventElapsedTime(&B->last_ms, B->t0, B->t1));
  return solve_results(B, res);
}

static int solve_fused(scft_batch *B, const scft_solve_opts *o, scft_result *res) {
  int rc = solve_fused_enqueue(B, o);
  if (rc) return rc;
  return solve_fused_finish(B, res);
}

// Batch-wide iterations replayed from a CUDA graph until no instance is active:
// each captured iteration launches the propagator classes of the requested
// precisions (each class evaluates the instances whose active flag it serves),
// then the mixing kernel; K iterations per graph, then the host reads the count
// of unfinished instances.
static int graph_iterate(scft_batch *B, const scft_solve_opts *o, const MixDev &m, bool f32, bool f64) {
  cudaStream_t st = B->st;
  const int c = B->count;
  int rc;
  const int K = std::max(1, o->iters_per_graph);
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  long long per_graph = 0;
  if ((rc = live_prepare(B, K))) return rc;
  const size_t live_bytes = (size_t)K * 2 * B->live_maxc * sizeof(unsigned long long);
  CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  long long before = g_launches.load();
  int crc = SCFT_OK;
  if (cudaMemsetAsync(B->d_work, 0, live_bytes, st) != cudaSuccess) crc = set_err(SCFT_ECUDA, "live reset");
  for (int k = 0; k < K && !crc; k++) {
    if (f32) crc = enqueue_propagate(B, PREC_F32, k);
    if (!crc && f64) crc = enqueue_propagate(B, PREC_F64, k);
    if (!crc) {
      cudaError_t e = mix_launch(m, st);
      g_launches++;
      if (e != cudaSuccess) crc = set_err(SCFT_ECUDA, "mix launch: %s", cudaGetErrorString(e));
    }
  }
  if (!crc) {
    count_active_kernel<<<1, 256, 0, st>>>(B->d_active, c, B->d_nactive);
    g_launches++;
    cudaMemcpyAsync(B->h_nactive, B->d_nactive, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(B->h_work, B->d_work, live_bytes, cudaMemcpyDeviceToHost, st);
  }
  per_graph = g_launches.load() - before;
  g_launches -= per_graph;  // counted again per replay below
  cudaError_t ec = cudaStreamEndCapture(st, &graph);
  if (crc) { if (graph) cudaGraphDestroy(graph); return crc; }
  CK(ec);
  ec = cudaGraphInstantiate(&gexec, graph, 0);
  cudaGraphDestroy(graph);
  CK(ec);
  const long long max_launch = (long long)o->maxit / K + 3;
  int result = SCFT_OK;
  const auto t_start = std::chrono::steady_clock::now();
  const double t_base = B->trace_ms.empty() ? 0.0 : B->trace_ms.back();
  for (long long L = 0;; L++) {
    cudaError_t e = cudaGraphLaunch(gexec, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { result = set_err(SCFT_ECUDA, "solver graph: %s", cudaGetErrorString(e)); break; }
    g_launches += per_graph;
    if ((rc = live_collect(B, K, f32, f64))) { result = rc; break; }
    B->trace_active.push_back(*B->h_nactive);
    B->trace_ms.push_back(t_base + std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count());
    if (*B->h_nactive == 0) break;
    if (L + 1 >= max_launch) {
      // watchdog: the mixing kernel stops every instance at maxit, so this is a backstop
      std::vector<int> act(c), stt(c);
      cudaMemcpy(act.data(), B->d_active, c * sizeof(int), cudaMemcpyDeviceToHost);
      cudaMemcpy(stt.data(), B->d_status, c * sizeof(int), cudaMemcpyDeviceToHost);
      for (int i = 0; i < c; i++)
        if (act[i]) { stt[i] |= SCFT_ST_WATCHDOG; act[i] = 0; }
      cudaMemcpy(B->d_status, stt.data(), c * sizeof(int), cudaMemcpyHostToDevice);
      cudaMemcpy(B->d_active, act.data(), c * sizeof(int), cudaMemcpyHostToDevice);
      break;
    }
  }
  cudaGraphExecDestroy(gexec);
  return result;
}

static int check_opts(const scft_solve_opts *o) {
  const int p = o->precision;
  if ((p != PREC_F32 && p != PREC_F64) || o->depth < 1 || o->depth > 16 || o->maxit < 0 || !(o->tol > 0) ||
      !(o->beta > 0.0 && o->beta <= 1.0) || o->finish_stall < 0 || !(o->budget_ms >= 0.0) ||
      !(o->graded_ratio >= 0.0) || !(o->precond_hfloor >= 0.0) || o->transfer_stride < 0)
    return set_err(SCFT_EINVAL, "solve options");
  if (o->forks < 0 || o->forks > SCFT_MAX_FORKS)
    return set_err(SCFT_EINVAL, "solve options: forks must be in [0, %d]", SCFT_MAX_FORKS);
  if (o->forks > 0) {
    if (o->fork_at < 1 || o->fork_grace < 0 || !(o->fork_err > 0.0) || o->maxit > (1 << 26))
      return set_err(SCFT_EINVAL, "solve options: forks need fork_at >= 1, fork_grace >= 0, fork_err > 0");
    for (int f = 0; f < o->forks; f++)
      if (!(o->fork_scale[f] > 0.0 && o->fork_scale[f] * o->beta <= 1.0))
        return set_err(SCFT_EINVAL, "solve options: fork_scale[%d] must give a mixing parameter in (0, 1]", f);
  }
  return SCFT_OK;
}

static int solve(scft_batch *B, const scft_solve_opts *o, scft_result *res) {
  const int p = o->precision;
  if (check_opts(o)) return SCFT_EINVAL;
  if (B->pending) return set_err(SCFT_EINVAL, "a solve of this batch is in flight: call scft_batch_wait");
  const bool verify = (p == PREC_F32) && o->verify64;
  const bool need64 = (p == PREC_F64) || verify || o->finish_stall > 0;
  bool fused = o->fused && p == PREC_F32 && !verify;
  int rc = plan(B, p, 1.0, (fused && o->finish_stall == 0) ? o->forks : 0);
  if (rc) return rc;
  // Classes that run as thread-block clusters (the default shapes above 2048
  // interior unknowns) have no fused form, whose one-CTA group would spill
  // registers: such batches take the batch-wide form.
  for (const auto &c : B->plans[p])
    if (cluster_ctas(p == PREC_F64, c.C, c.NW) > 1) fused = false;
  if (!fused && B->plan_paths[p] != 0 && (rc = plan(B, p, 1.0, 0))) return rc;
  if ((rc = ensure_mix(B, o->depth, fused ? o->forks : 0))) return rc;
  if (fused) return solve_fused(B, o, res);
  if (p == PREC_F32 && need64 && (rc = plan(B, PREC_F64, 0.125))) return rc;
  cudaStream_t st = B->st;
  CK(cudaEventRecord(B->t0, st));
  MixDev m;
  if ((rc = solve_begin(B, o, p, verify, &m))) return rc;
  B->trace_active.clear();
  B->trace_ms.clear();
  if ((rc = graph_iterate(B, o, m, p == PREC_F32, need64))) return rc;
  CK(cudaEventRecord(B->t1, st));
  CK(cudaEventSynchronize(B->t1));
  CK(cudaEventElapsedTime(&B->last_ms, B->t0, B->t1));
  return solve_results(B, res);
}

// Staged solve (transfer_stride > 1).  Instances that share a mesh shape (node
// count, contour steps, rule and spacing ratio to 1 %) are sorted by film width.
// Round 0 solves every stride-th of them and the widest, each from its own
// field, with the iteration cap maxit/2.  Each later round takes every instance
// not converged so far (first-round failures included), starts it from the
// field interpolated in the width, node by node, between its nearest converged
// neighbours below and above (one of them when there is only one; its own field
// when there is none), and solves those: round 1 with the cap maxit/4, round 2
// with the full cap.  A converged neighbour of round 0 is a few tenths of L
// away, one of round 1 a few hundredths, so a straggler of round 1 gets a closer
// start in round 2.  Groups of fewer than three instances are solved in round 0.
static int solve_staged(scft_batch *B, const scft_solve_opts *o, scft_result *res) {
  const int c = B->count, stride = o->transfer_stride;
  std::map<std::tuple<int, int, int, long>, std::vector<int>> groups;
  for (int i = 0; i < c; i++)
    groups[{B->n[i], B->nsteps[i], B->rule[i], std::lround(std::log(B->spacing_ratio[i]) * 100.0)}].push_back(i);
  std::vector<int> sel(c, 1);
  std::vector<const std::vector<int> *> group_of(c, nullptr);
  for (auto &kv : groups) {
    auto &g = kv.second;
    std::stable_sort(g.begin(), g.end(), [&](int a, int b) { return B->width[a] < B->width[b]; });
    for (int i : g) group_of[i] = &g;
    if (g.size() < 3) continue;
    const int m = (int)g.size();
    for (int r = 0; r < m; r++) sel[g[r]] = (r % stride == 0 || r == m - 1) ? 1 : 0;
  }
  if (!B->d_select) {
    int rc = dalloc(&B->d_select, (size_t)c);
    if (rc) return rc;
  }
  std::vector<scft_result> out(c), rr(c);
  std::vector<int> done(c, 0), its(c, 0);
  float total_ms = 0.f;
  const int caps[3] = {std::max(1, o->maxit / 2), std::max(1, o->maxit / 4), o->maxit};
  for (int round = 0; round < 3; round++) {
    if (round > 0) {
      // this round's instances: every one not converged; their starts
      std::vector<int> tplan;
      std::vector<double> tt;
      for (int i = 0; i < c; i++) {
        sel[i] = done[i] ? 0 : 1;
        if (done[i]) continue;
        const std::vector<int> &g = *group_of[i];
        int a = -1, b = -1;  // nearest converged neighbours below and above
        for (int j : g) {
          if (j == i || !done[j]) continue;
          if (B->width[j] <= B->width[i] && (a < 0 || B->width[j] >= B->width[a])) a = j;
          if (B->width[j] >= B->width[i] && (b < 0 || B->width[j] < B->width[b])) b = j;
        }
        if (a < 0 && b < 0) continue;
        if (a < 0) a = b;
        if (b < 0) b = a;
        const double span = B->width[b] - B->width[a];
        double t = span > 0.0 ? (B->width[i] - B->width[a]) / span : 0.0;
        t = std::min(1.0, std::max(0.0, t));
        tplan.insert(tplan.end(), {i, a, b, 0});
        tt.push_back(t);
      }
      if (std::none_of(sel.begin(), sel.end(), [](int v) { return v != 0; })) break;
      if (!tt.empty()) {
        const int m = (int)tt.size();
        int *d_plan = nullptr;
        double *d_t = nullptr;
        int rc;
        if ((rc = dalloc(&d_plan, tplan.size())) || (rc = dalloc(&d_t, tt.size()))) {
          dfree(d_plan);
          return rc;
        }
        float msx = 0.f;
        CK(cudaMemcpyAsync(d_plan, tplan.data(), tplan.size() * sizeof(int), cudaMemcpyHostToDevice, B->st));
        CK(cudaMemcpyAsync(d_t, tt.data(), tt.size() * sizeof(double), cudaMemcpyHostToDevice, B->st));
        CK(cudaEventRecord(B->t0, B->st));
        transfer_kernel<<<m, 256, 0, B->st>>>(d_plan, d_t, m, B->d_n, B->d_node_off, B->d_w);
        g_launches++;
        CK(cudaGetLastError());
        CK(cudaEventRecord(B->t1, B->st));
        CK(cudaEventSynchronize(B->t1));
        CK(cudaEventElapsedTime(&msx, B->t0, B->t1));
        total_ms += msx;
        dfree(d_plan);
        dfree(d_t);
      }
    }
    CK(cudaMemcpy(B->d_select, sel.data(), c * sizeof(int), cudaMemcpyHostToDevice));
    B->use_select = true;
    scft_solve_opts os = *o;
    os.transfer_stride = 0;
    os.maxit = caps[round];
    const int rc = solve(B, &os, rr.data());
    B->use_select = false;
    if (rc) return rc;
    total_ms += B->last_ms;
    for (int i = 0; i < c; i++) {
      if (!sel[i]) continue;
      out[i] = rr[i];
      its[i] += rr[i].iterations;
      out[i].iterations = its[i];  // every round's updates of the instance
      if (rr[i].status & SCFT_ST_CONVERGED) done[i] = 1;
    }
  }
  // the outcome of each instance's last round, with the updates of all its rounds
  std::vector<int> st(c);
  for (int i = 0; i < c; i++) {
    st[i] = out[i].status;
    if (res) res[i] = out[i];
  }
  CK(cudaMemcpy(B->d_status, st.data(), c * sizeof(int), cudaMemcpyHostToDevice));
  B->last_ms = total_ms;
  return SCFT_OK;
}

// ---------------------------------------------------------------------------
// autotuner: per default shape class, time the candidate shapes on a sample
// ---------------------------------------------------------------------------
static int autotune(scft_batch *B, int p) {
  std::map<std::pair<int, int>, std::vector<int>> groups;
  for (int i = 0; i < B->count; i++) {
    int C, NW;
    default_shape(B->n[i] - 2, p, &C, &NW);
    groups[{C, NW}].push_back(i);
  }
  std::vector<int> saveC = B->shapeC[p], saveNW = B->shapeNW[p];
  std::vector<int> act0(B->count, 0);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  for (auto &kv : groups) {
    std::vector<int> sample = kv.second;
    std::sort(sample.begin(), sample.end(),
              [&](int a, int b) { return (double)B->n[a] * B->nsteps[a] > (double)B->n[b] * B->nsteps[b]; });
    if (sample.size() > 256) sample.resize(256);
    int maxN = 0;
    for (int i : sample) maxN = std::max(maxN, B->n[i] - 2);
    std::vector<std::pair<int, int>> cands;
    for (int C : {1, 2, 4, 8})
      for (int NW = 1; NW <= 32; NW *= 2)
        if (32 * NW * C >= maxN && 32 * NW * C < 4 * std::max(maxN, 32) && propagate_has_class(p, C, NW))
          cands.push_back({C, NW});
    float best = 1e30f;
    std::pair<int, int> bestS = kv.first;
    for (auto s : cands) {
      for (int i : kv.second) { B->shapeC[p][i] = s.first; B->shapeNW[p][i] = s.second; }
      B->planned[p] = false;
      int rc = plan(B, p, 1.0);
      if (rc) continue;
      std::vector<int> act(B->count, 0);
      for (int i : sample) act[i] = (p == PREC_F32) ? 1 : 2;
      float ms = 0.f;
      for (int rep = 0; rep < 2; rep++) {
        CK(cudaMemcpy(B->d_active, act.data(), B->count * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaEventRecord(e0, B->st));
        rc = enqueue_propagate(B, p);
        if (rc) return rc;
        CK(cudaEventRecord(e1, B->st));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
      }
      if (ms < best) { best = ms; bestS = s; }
    }
    for (int i : kv.second) { B->shapeC[p][i] = bestS.first; B->shapeNW[p][i] = bestS.second; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  B->planned[p] = false;
  (void)saveC; (void)saveNW;
  return plan(B, p, 1.0);
}

// ---------------------------------------------------------------------------
// drop-in single-instance context
// ---------------------------------------------------------------------------
struct DropIn {
  bool set = false;
  int n = 0, nsteps = 0, rule = 0, sign = 1, prec = PREC_F64, scheme = SCFT_SCHEME_IE, wmode = SCFT_W_ROWSCALED;
  double ds = 0, L = 0;
  std::vector<double> x, f0;
  scft_batch *B = nullptr;
  double *d_out = nullptr, *d_in = nullptr;  // interior vectors
  double *h_stage = nullptr;                  // pinned, 2 * interior
};
static std::recursive_mutex g_mu;
static DropIn g_drop;
static double g_broydn_tol = 1e-8, g_broydn_err = 0.0;
static int g_adm_maxit = 1000000;

static int dropin_eval_device(const double *d_xint, double *d_out, int fixed_point) {
  DropIn &D = g_drop;
  scft_batch *B = D.B;
  const int N = D.n - 2;
  CK(cudaMemcpyAsync(B->d_w + 1, d_xint, N * sizeof(double), cudaMemcpyDeviceToDevice, B->st));
  int rc = fill_int(B->d_active, 1, D.prec == PREC_F32 ? 1 : 2, B->st);
  if (rc) return rc;
  if (D.scheme != SCFT_SCHEME_IE || D.wmode != SCFT_W_ROWSCALED) rc = seq_enqueue(B, D.scheme, D.wmode);
  else rc = enqueue_propagate(B, D.prec);
  if (rc) return rc;
  CK(residual_launch(D.n, B->d_phi, B->d_f0, D.sign, d_out, B->d_w + 1, fixed_point, B->st));
  g_launches++;
  return SCFT_OK;
}

static int dropin_eval_host(const double *w_int, double *out_int, int fixed_point) {
  DropIn &D = g_drop;
  if (!D.set) return set_err(SCFT_ENOCONFIG, "scft_set_config was not called");
  const int N = D.n - 2;
  memcpy(D.h_stage, w_int, N * sizeof(double));
  CK(cudaMemcpyAsync(D.d_in, D.h_stage, N * sizeof(double), cudaMemcpyHostToDevice, D.B->st));
  int rc = dropin_eval_device(D.d_in, D.d_out, fixed_point);
  if (rc) return rc;
  CK(cudaMemcpyAsync(D.h_stage + N, D.d_out, N * sizeof(double), cudaMemcpyDeviceToHost, D.B->st));
  CK(cudaStreamSynchronize(D.B->st));
  memcpy(out_int, D.h_stage + N, N * sizeof(double));
  return SCFT_OK;
}

// ---------------------------------------------------------------------------
// Broyden (broydn.c:44-292 with fdjac.c, qrdcmp.c, qrupdt.c, rotate.c, rsolv.c,
// lnsrch.c): the O(n^2) quasi-Newton algebra runs on the host, every function
// evaluation on the GPU; the internal propagator evaluates the n columns of the
// finite-difference Jacobian as one batch.
// ---------------------------------------------------------------------------
namespace {
struct Evaluator {
  scft_vecfunc f = nullptr;
  int n = 0;
  bool internal = false;
  std::vector<double> buf_in, buf_out;  // 1-based staging for host callbacks
  int rc = SCFT_OK;
  void operator()(const double *x, double *out) {  // 0-based x, out
    if (internal) {
      int r = dropin_eval_host(x, out, 0);
      if (r && !rc) rc = r;
      return;
    }
    buf_in.assign(n + 1, 0.0);
    buf_out.assign(n + 1, 0.0);
    memcpy(buf_in.data() + 1, x, n * sizeof(double));
    f(n, buf_in.data(), buf_out.data());
    memcpy(out, buf_out.data() + 1, n * sizeof(double));
  }
};

// finite-difference Jacobian, relative step 1e-7 (fdjac.c:10-41); df row-major
int fdjac(Evaluator &E, std::vector<double> &x, const std::vector<double> &fv, std::vector<double> &df) {
  const int n = E.n;
  std::vector<double> h(n);
  for (int j = 0; j < n; j++) {
    const double temp = x[j];
    double hh = 1e-7 * temp;
    if (std::fabs(hh) < 1e-7) hh = temp >= 0.0 ? 1e-7 : -1e-7;
    h[j] = (temp + hh) - temp;
  }
  if (E.internal) {
    // one batch of n perturbed fields
    DropIn &D = g_drop;
    std::vector<scft_instance> inst(n);
    std::vector<double> wall((size_t)n * D.n, 0.0);
    for (int j = 0; j < n; j++) {
      double *w = wall.data() + (size_t)j * D.n;
      for (int i = 0; i < n; i++) w[i + 1] = x[i];
      w[j + 1] = x[j] + h[j];
      inst[j].n_nodes = D.n; inst[j].x = D.x.data(); inst[j].L = D.L; inst[j].f0 = D.f0.data();
      inst[j].w0 = w; inst[j].nsteps = D.nsteps; inst[j].ds = D.ds; inst[j].rule = D.rule;
    }
    scft_batch *J = nullptr;
    int rc = create_batch(inst.data(), n, &J);
    if (rc) return rc;
    rc = evaluate(J, D.prec);
    std::vector<double> phi((size_t)n * D.n);
    if (!rc && cudaMemcpy(phi.data(), J->d_phi, phi.size() * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = set_err(SCFT_ECUDA, "jacobian download");
    destroy_batch(J);
    if (rc) return rc;
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        double r = phi[(size_t)j * D.n + i + 1] - D.f0[i + 1];
        if (D.sign < 0) r = -r;
        df[(size_t)i * n + j] = (r - fv[i]) / h[j];
      }
    return SCFT_OK;
  }
  std::vector<double> ft(n);
  for (int j = 0; j < n; j++) {
    const double temp = x[j];
    x[j] = temp + h[j];
    E(x.data(), ft.data());
    x[j] = temp;
    for (int i = 0; i < n; i++) df[(size_t)i * n + j] = (ft[i] - fv[i]) / h[j];
  }
  return E.rc;
}

void rotate(std::vector<double> &r, std::vector<double> &qt, int n, int i, double a, double b) {
  double c, s;
  if (a == 0.0) { c = 0.0; s = b >= 0.0 ? 1.0 : -1.0; }
  else if (std::fabs(a) > std::fabs(b)) {
    const double f = b / a;
    c = std::copysign(1.0 / std::sqrt(1.0 + f * f), a);
    s = f * c;
  } else {
    const double f = a / b;
    s = std::copysign(1.0 / std::sqrt(1.0 + f * f), b);
    c = f * s;
  }
  for (int j = i; j < n; j++) {
    const double y = r[i * n + j], w = r[(i + 1) * n + j];
    r[i * n + j] = c * y - s * w;
    r[(i + 1) * n + j] = s * y + c * w;
  }
  for (int j = 0; j < n; j++) {
    const double y = qt[i * n + j], w = qt[(i + 1) * n + j];
    qt[i * n + j] = c * y - s * w;
    qt[(i + 1) * n + j] = s * y + c * w;
  }
}
}  // namespace

static int broydn_impl(Evaluator &E, std::vector<double> &x, double tol, int *check) {
  const int n = E.n, MAXITS = 400;
  const double EPS = 1e-14, TOLX = 1e-14, STPMX = 100.0;
  std::vector<double> qt((size_t)n * n), r((size_t)n * n), c(n), d(n), fvec(n), fvcold(n), g(n), p(n), s(n),
      t(n), w(n), xold(n);
  auto fmin = [&](const double *xx) {
    E(xx, fvec.data());
    double sm = 0.0;
    for (int i = 0; i < n; i++) sm += fvec[i] * fvec[i];
    return 0.5 * sm;
  };
  *check = 1;
  double f = fmin(x.data());
  if (E.rc) return E.rc;
  double err = 0.0;
  for (int i = 0; i < n; i++) err = std::max(err, std::fabs(fvec[i]));
  g_broydn_err = err;
  if (err < tol) { *check = 0; return SCFT_OK; }
  double sum = 0.0;
  for (int i = 0; i < n; i++) sum += x[i] * x[i];
  const double stpmax = STPMX * std::max(std::sqrt(sum), (double)n);
  bool restrt = true;
  for (int its = 1; its <= MAXITS; its++) {
    if (restrt) {
      int rc = fdjac(E, x, fvec, r);
      if (rc) return rc;
      // Householder QR (qrdcmp.c:6-34)
      bool sing = false;
      for (int k = 0; k < n - 1; k++) {
        double scale = 0.0;
        for (int i = k; i < n; i++) scale = std::max(scale, std::fabs(r[i * n + k]));
        if (scale == 0.0) { sing = true; c[k] = d[k] = 0.0; continue; }
        for (int i = k; i < n; i++) r[i * n + k] /= scale;
        double sm = 0.0;
        for (int i = k; i < n; i++) sm += r[i * n + k] * r[i * n + k];
        const double sigma = std::copysign(std::sqrt(sm), r[k * n + k]);
        r[k * n + k] += sigma;
        c[k] = sigma * r[k * n + k];
        d[k] = -scale * sigma;
        for (int j = k + 1; j < n; j++) {
          double sj = 0.0;
          for (int i = k; i < n; i++) sj += r[i * n + k] * r[i * n + j];
          const double tau = sj / c[k];
          for (int i = k; i < n; i++) r[i * n + j] -= tau * r[i * n + k];
        }
      }
      d[n - 1] = r[(n - 1) * n + n - 1];
      if (d[n - 1] == 0.0) sing = true;
      if (sing) return set_err(SCFT_ESINGULAR, "singular Jacobian in broydn");
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
      bool skip = true;
      for (int i = 0; i < n; i++) {
        double sm = 0.0;
        for (int j = 0; j < n; j++) sm += qt[j * n + i] * t[j];
        w[i] = fvec[i] - fvcold[i] - sm;
        if (std::fabs(w[i]) >= EPS * (std::fabs(fvec[i]) + std::fabs(fvcold[i]))) skip = false;
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
        // rank-1 update re-triangularised by Givens rotations (qrupdt.c:6-24)
        int k;
        for (k = n - 1; k >= 0; k--) if (t[k] != 0.0) break;
        if (k < 0) k = 0;
        for (int i = k - 1; i >= 0; i--) {
          rotate(r, qt, n, i, t[i], -t[i + 1]);
          if (t[i] == 0.0) t[i] = std::fabs(t[i + 1]);
          else if (std::fabs(t[i]) > std::fabs(t[i + 1])) t[i] = std::fabs(t[i]) * std::sqrt(1.0 + (t[i + 1] / t[i]) * (t[i + 1] / t[i]));
          else t[i] = std::fabs(t[i + 1]) * std::sqrt(1.0 + (t[i] / t[i + 1]) * (t[i] / t[i + 1]));
        }
        for (int j = 0; j < n; j++) r[j] += t[0] * s[j];
        for (int i = 0; i < k; i++) rotate(r, qt, n, i, r[i * n + i], -r[(i + 1) * n + i]);
        for (int i = 0; i < n; i++) {
          if (r[i * n + i] == 0.0) return set_err(SCFT_ESINGULAR, "r singular in broydn");
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
    const double fold = f;
    // back substitution R p = -Q^T F (rsolv.c:3-12)
    p[n - 1] /= d[n - 1];
    for (int i = n - 2; i >= 0; i--) {
      double sm = 0.0;
      for (int j = i + 1; j < n; j++) sm += r[i * n + j] * p[j];
      p[i] = (p[i] - sm) / d[i];
    }
    // backtracking line search (lnsrch.c:8-61)
    int lcheck = 0;
    {
      double sm = 0.0;
      for (int i = 0; i < n; i++) sm += p[i] * p[i];
      sm = std::sqrt(sm);
      if (sm > stpmax) for (int i = 0; i < n; i++) p[i] *= stpmax / sm;
      double slope = 0.0;
      for (int i = 0; i < n; i++) slope += g[i] * p[i];
      if (slope >= 0.0) return set_err(SCFT_EINVAL, "roundoff problem in lnsrch");
      double test = 0.0;
      for (int i = 0; i < n; i++) test = std::max(test, std::fabs(p[i]) / std::max(std::fabs(xold[i]), 1.0));
      const double alamin = 1e-7 / test;
      double alam = 1.0, alam2 = 0.0, f2 = 0.0, tmplam;
      for (;;) {
        for (int i = 0; i < n; i++) x[i] = xold[i] + alam * p[i];
        f = fmin(x.data());
        if (E.rc) return E.rc;
        if (alam < alamin) {
          for (int i = 0; i < n; i++) x[i] = xold[i];
          lcheck = 1;
          break;
        }
        if (f <= fold + 1e-4 * alam * slope) break;
        if (alam == 1.0) {
          tmplam = -slope / (2.0 * (f - fold - slope));
        } else {
          const double rhs1 = f - fold - alam * slope, rhs2 = f2 - fold - alam2 * slope;
          const double a = (rhs1 / (alam * alam) - rhs2 / (alam2 * alam2)) / (alam - alam2);
          const double b = (-alam2 * rhs1 / (alam * alam) + alam * rhs2 / (alam2 * alam2)) / (alam - alam2);
          if (a == 0.0) tmplam = -slope / (2.0 * b);
          else {
            const double disc = b * b - 3.0 * a * slope;
            if (disc < 0.0) tmplam = 0.5 * alam;
            else if (b <= 0.0) tmplam = (-b + std::sqrt(disc)) / (3.0 * a);
            else tmplam = -slope / (b + std::sqrt(disc));
          }
          if (tmplam > 0.5 * alam) tmplam = 0.5 * alam;
        }
        alam2 = alam;
        f2 = f;
        alam = std::max(tmplam, 0.1 * alam);
      }
    }
    err = 0.0;
    for (int i = 0; i < n; i++) err = std::max(err, std::fabs(fvec[i]));
    g_broydn_err = err;
    if (err < tol) { *check = 0; return SCFT_OK; }
    if (lcheck) {
      if (restrt) { *check = 1; return SCFT_OK; }
      double test = 0.0;
      const double den = std::max(f, 0.5 * n);
      for (int i = 0; i < n; i++) test = std::max(test, std::fabs(g[i]) * std::max(std::fabs(x[i]), 1.0) / den);
      if (test < tol) { *check = 0; return SCFT_OK; }
      restrt = true;
    } else {
      restrt = false;
      double test = 0.0;
      for (int i = 0; i < n; i++) test = std::max(test, std::fabs(x[i] - xold[i]) / std::max(std::fabs(x[i]), 1.0));
      if (test < TOLX) { *check = 0; return SCFT_OK; }
    }
  }
  *check = 1;
  return SCFT_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char *scft_last_error(void) { return g_err.c_str(); }

const char *scft_strerror(int code) {
  switch (code) {
    case SCFT_OK: return "ok";
    case SCFT_EINVAL: return "invalid argument";
    case SCFT_ECUDA: return "CUDA error";
    case SCFT_ENOMEM: return "out of memory";
    case SCFT_ENOCONFIG: return "scft_set_config was not called";
    case SCFT_ENODEV: return "no CUDA device";
    case SCFT_ESINGULAR: return "singular Jacobian";
    case SCFT_EIO: return "file error";
    default: return "unknown error";
  }
}

long long scft_kernel_launches(void) { return g_launches.load(); }

void scft_config_init(scft_config *c) {
  if (!c) return;
  memset(c, 0, sizeof *c);
  c->n_nodes = 33;
  c->L = 3.72374;
  c->nsteps = 2049;
  c->ds = 1.0 / 2048.0;
  c->rule = SCFT_RULE_TRAPEZOID;
  c->sign = 1;
  c->precision = SCFT_F64;
}

int scft_set_config(const scft_config *c) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  if (!c || c->n_nodes < 3 || !c->f0 || c->nsteps < 1 || !(c->ds > 0.0) ||
      (c->precision != SCFT_F32 && c->precision != SCFT_F64) ||
      (c->scheme != SCFT_SCHEME_IE && c->scheme != SCFT_SCHEME_IRK2) ||
      (c->wmode != SCFT_W_ROWSCALED && c->wmode != SCFT_W_CONSISTENT))
    return set_err(SCFT_EINVAL, "scft_set_config: invalid configuration");
  if ((c->scheme != SCFT_SCHEME_IE || c->wmode != SCFT_W_ROWSCALED) && c->precision != SCFT_F64)
    return set_err(SCFT_EINVAL, "scft_set_config: the IRK2 scheme and the consistent field term run in FP64");
  DropIn &D = g_drop;
  if (D.B) { destroy_batch(D.B); D.B = nullptr; }
  dfree(D.d_in); dfree(D.d_out);
  if (D.h_stage) host_free(D.h_stage);
  D.h_stage = nullptr;
  D.set = false;
  D.n = c->n_nodes; D.nsteps = c->nsteps; D.ds = c->ds; D.rule = c->rule;
  D.sign = c->sign >= 0 ? 1 : -1; D.prec = c->precision;
  D.scheme = c->scheme; D.wmode = c->wmode;
  D.x.resize(D.n);
  D.f0.assign(c->f0, c->f0 + D.n);
  D.L = c->x ? c->x[D.n - 1] - c->x[0] : c->L;
  for (int i = 0; i < D.n; i++) D.x[i] = c->x ? c->x[i] : c->L * (double)i / (double)(D.n - 1);
  if (!c->x) D.x[D.n - 1] = c->L;
  scft_instance inst;
  inst.n_nodes = D.n; inst.x = D.x.data(); inst.L = D.L; inst.f0 = D.f0.data(); inst.w0 = nullptr;
  inst.nsteps = D.nsteps; inst.ds = D.ds; inst.rule = D.rule;
  std::vector<double> w0(D.n, 0.0);
  w0[0] = c->w_wall[0];
  w0[D.n - 1] = c->w_wall[1];
  inst.w0 = w0.data();  // interior values come with every evaluation; wall values stay
  int rc = create_batch(&inst, 1, &D.B);
  if (rc) return rc;
  if ((rc = plan(D.B, D.prec, 1.0))) return rc;
  if ((rc = dalloc(&D.d_in, D.n)) || (rc = dalloc(&D.d_out, D.n))) return rc;
  CK(host_alloc((void **)&D.h_stage, 2 * D.n * sizeof(double)));
  D.set = true;
  return SCFT_OK;
}

int scft_fem_residual(int n_interior, double *w, double *out) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  if (!g_drop.set) return set_err(SCFT_ENOCONFIG, "scft_set_config was not called");
  if (n_interior != g_drop.n - 2 || !w || !out)
    return set_err(SCFT_EINVAL, "scft_fem_residual: %d interior nodes, configured %d", n_interior, g_drop.n - 2);
  return dropin_eval_host(w + 1, out + 1, 0);
}

void scft_fem_residual_vf(int n_interior, double *w, double *out) {
  if (scft_fem_residual(n_interior, w, out) != SCFT_OK)
    for (int i = 1; i <= n_interior; i++) out[i] = NAN;
}

void scft_fem_residual0_vf(int n_interior, double *w, double *out) {
  if (scft_fem_residual(n_interior, w - 1, out - 1) != SCFT_OK)
    for (int i = 0; i < n_interior; i++) out[i] = NAN;
}

void scft_fem_fixedpoint_vf(int n_interior, double *w, double *out) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  if (!g_drop.set || n_interior != g_drop.n - 2 || dropin_eval_host(w + 1, out + 1, 1) != SCFT_OK)
    for (int i = 1; i <= n_interior; i++) out[i] = NAN;
}

int scft_density(const double *w_nodes, double *phi, double *Q) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  DropIn &D = g_drop;
  if (!D.set) return set_err(SCFT_ENOCONFIG, "scft_set_config was not called");
  if (!w_nodes || !phi) return set_err(SCFT_EINVAL, "scft_density: null buffer");
  std::vector<double> w(w_nodes, w_nodes + D.n);
  if (D.wmode == SCFT_W_ROWSCALED) w[0] = w[D.n - 1] = 0.0;  // the consistent term uses the wall values
  CK(cudaMemcpy(D.B->d_w, w.data(), D.n * sizeof(double), cudaMemcpyHostToDevice));
  int rc = (D.scheme != SCFT_SCHEME_IE || D.wmode != SCFT_W_ROWSCALED)
               ? scft_batch_evaluate_scheme(D.B, D.scheme, D.wmode)
               : evaluate(D.B, D.prec);
  if (rc) return rc;
  CK(cudaMemcpy(phi, D.B->d_phi, D.n * sizeof(double), cudaMemcpyDeviceToHost));
  if (Q) CK(cudaMemcpy(Q, D.B->d_Q, sizeof(double), cudaMemcpyDeviceToHost));
  return SCFT_OK;
}

void scft_adm_set_maxit(int maxit) { g_adm_maxit = maxit > 0 ? maxit : 1; }

// adm of adm.c:24-313; xnew_out (n doubles, may be NULL) receives the last map
// value g(x), the vector adm.c returns.
static int adm_impl(double *x, int n, int *check, scft_vecfunc f, int flag, double *xnew_out) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  if (!x || n <= 0 || !check || !f || (flag != 0 && flag != 1)) return set_err(SCFT_EINVAL, "scft_adm");
  const bool internal = (f == scft_fem_fixedpoint_vf) && g_drop.set && n == g_drop.n - 2;
  cudaStream_t st;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  double *d_x = nullptr, *d_xn = nullptr, *d_xh = nullptr, *d_dh = nullptr, *d_err = nullptr;
  int *d_ctl = nullptr;
  int rc;
  if ((rc = dalloc(&d_x, n)) || (rc = dalloc(&d_xn, n)) || (rc = dalloc(&d_xh, 11 * (size_t)n)) ||
      (rc = dalloc(&d_dh, 11 * (size_t)n)) || (rc = dalloc(&d_err, 1)) || (rc = dalloc(&d_ctl, 3))) {
    cudaStreamDestroy(st);
    return rc;
  }
  AdmDev a;
  a.n = n; a.x = d_x; a.xnew = d_xn; a.xh = d_xh; a.dh = d_dh; a.tol = 1e-10;
  a.its = d_ctl; a.nc = d_ctl + 1; a.flag = d_ctl + 2; a.err = d_err;
  std::vector<double> hx(n + 1), hy(n + 1);
  auto evaluate_map = [&]() -> int {
    if (internal) {
      int r2;
      if ((r2 = dropin_eval_device(d_x, d_xn, 1))) return r2;
      CK(cudaStreamSynchronize(g_drop.B->st));
      return SCFT_OK;
    }
    CK(cudaMemcpy(hx.data() + flag, d_x, n * sizeof(double), cudaMemcpyDeviceToHost));
    f(n, hx.data(), hy.data());
    CK(cudaMemcpy(d_xn, hy.data() + flag, n * sizeof(double), cudaMemcpyHostToDevice));
    return SCFT_OK;
  };
  int hctl[3];
  CK(cudaMemcpy(d_x, x + flag, n * sizeof(double), cudaMemcpyHostToDevice));
  *check = 1;
  rc = evaluate_map();
  if (!rc) {
    CK(adm_first_launch(a, st));
    g_launches++;
    CK(cudaMemcpyAsync(hctl, d_ctl, 3 * sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (hctl[2] == 1) *check = 0;
    for (int its = 2; its <= g_adm_maxit && *check && !rc; its++) {
      rc = evaluate_map();
      if (rc) break;
      CK(adm_step_launch(a, st));
      g_launches++;
      CK(cudaMemcpyAsync(hctl, d_ctl, 3 * sizeof(int), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      if (hctl[2] == 1) *check = 0;
    }
  }
  if (!rc) CK(cudaMemcpy(x + flag, d_x, n * sizeof(double), cudaMemcpyDeviceToHost));
  if (!rc && xnew_out) CK(cudaMemcpy(xnew_out, d_xn, n * sizeof(double), cudaMemcpyDeviceToHost));
  dfree(d_x); dfree(d_xn); dfree(d_xh); dfree(d_dh); dfree(d_err); dfree(d_ctl);
  cudaStreamDestroy(st);
  return rc;
}

int scft_adm(double *x, int n, int *check, scft_vecfunc f, int flag) {
  return adm_impl(x, n, check, f, flag, nullptr);
}

double *scft_nr_adm(double *x, int n, int *check, scft_vecfunc f, int flag) {
  if (check) *check = 1;
  if (n <= 0 || (flag != 0 && flag != 1)) {
    set_err(SCFT_EINVAL, "scft_nr_adm");
    return nullptr;
  }
  // laid out like nrutil's vector(flag, n + flag - 1): one spare element below
  // index flag, so that the reference's free_vector(v, flag, n + flag - 1) frees it
  double *base = static_cast<double *>(malloc(sizeof(double) * ((size_t)n + 1)));
  if (!base) {
    set_err(SCFT_ENOMEM, "scft_nr_adm: host allocation");
    return nullptr;
  }
  double *v = base - flag + 1;
  if (adm_impl(x, n, check, f, flag, v + flag) != SCFT_OK) {
    if (check) *check = 1;
    free(base);
    return nullptr;
  }
  return v;
}

void scft_nr_free_vector(double *v, int flag) {
  if (v) free(v + flag - 1);
}

int scft_adm_chen(scft_vecfunc f, double *x, double tol, int maxit, int n, double lmd, int nn, int final_) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  if (!f || !x || n <= 0 || maxit < 0 || nn < 0) return set_err(SCFT_EINVAL, "scft_adm_chen");
  const int nm = std::min(nn, n);
  if (nm > 63) return set_err(SCFT_EINVAL, "scft_adm_chen: history depth %d exceeds 63", nm);
  const bool internal = (f == scft_fem_residual0_vf) && g_drop.set && n == g_drop.n - 2;
  const int depth = nm + 1;
  cudaStream_t st;
  CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  double *d_X = nullptr, *d_Y = nullptr, *d_s = nullptr;
  int *d_i = nullptr;
  int rc;
  if ((rc = dalloc(&d_X, (size_t)depth * n)) || (rc = dalloc(&d_Y, (size_t)depth * n)) ||
      (rc = dalloc(&d_s, 2)) || (rc = dalloc(&d_i, 3))) {
    cudaStreamDestroy(st);
    return rc;
  }
  AdmChenDev a;
  a.n = n; a.nm = nm; a.depth = depth; a.X = d_X; a.Y = d_Y; a.tol = tol; a.lmd = lmd; a.final_ = final_ ? 1 : 0;
  a.k = d_i; a.krestart = d_i + 1; a.flag = d_i + 2; a.lk = d_s; a.err = d_s + 1;
  CK(cudaMemset(d_i, 0, 3 * sizeof(int)));
  CK(cudaMemcpy(d_s, &lmd, sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_X, x, n * sizeof(double), cudaMemcpyHostToDevice));
  std::vector<double> hx(n), hy(n);
  int result = 1, k = 0;
  for (k = 0; k <= maxit; k++) {
    double *Xk = d_X + (size_t)(k % depth) * n, *Yk = d_Y + (size_t)(k % depth) * n;
    if (internal) {
      if ((rc = dropin_eval_device(Xk, Yk, 0))) break;
      CK(cudaStreamSynchronize(g_drop.B->st));
    } else {
      CK(cudaMemcpy(hx.data(), Xk, n * sizeof(double), cudaMemcpyDeviceToHost));
      f(n, hx.data(), hy.data());
      CK(cudaMemcpy(Yk, hy.data(), n * sizeof(double), cudaMemcpyHostToDevice));
    }
    CK(admchen_step_launch(a, st));
    g_launches++;
    int flag = 0;
    CK(cudaMemcpyAsync(&flag, d_i + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (flag == 1 || flag == 2) {
      CK(cudaMemcpy(x, Xk, n * sizeof(double), cudaMemcpyDeviceToHost));
      result = (flag == 1) ? 0 : 2;
      break;
    }
  }
  if (!rc && result == 1) CK(cudaMemcpy(x, d_X + (size_t)(k % depth) * n, n * sizeof(double), cudaMemcpyDeviceToHost));
  dfree(d_X); dfree(d_Y); dfree(d_s); dfree(d_i);
  cudaStreamDestroy(st);
  return rc ? rc : result;
}

void scft_broydn_set_tol(double tol) { g_broydn_tol = tol; }
double scft_broydn_get_err(void) { return g_broydn_err; }

int scft_broydn(double *x, int n, int *check, scft_vecfunc f) {
  std::lock_guard<std::recursive_mutex> lk(g_mu);
  if (!x || n <= 0 || !check || !f) return set_err(SCFT_EINVAL, "scft_broydn");
  Evaluator E;
  E.f = f;
  E.n = n;
  E.internal = (f == scft_fem_residual_vf) && g_drop.set && n == g_drop.n - 2;
  std::vector<double> xv(x + 1, x + 1 + n);
  int rc = broydn_impl(E, xv, g_broydn_tol, check);
  memcpy(x + 1, xv.data(), n * sizeof(double));
  return rc;
}

void scft_nr_broydn(double x[], int n, int *check, scft_vecfunc f) {
  if (scft_broydn(x, n, check, f) != SCFT_OK && check) *check = 1;
}

void scft_solve_opts_init(scft_solve_opts *o) {
  if (!o) return;
  memset(o, 0, sizeof *o);
  o->precision = SCFT_F32;
  o->tol = 1e-6;
  o->tol32_factor = 0.65;
  o->verify64 = 0;
  o->maxit = 2000;
  o->depth = 10;
  o->beta = 1.0;
  o->clip = 1.0;
  o->grow = 10.0;
  o->reg = 1e-12;
  o->residual_mode = SCFT_MIX_LOG;
  o->precond = 0.6;
  o->iters_per_graph = 8;
  o->beta_schedule = 0;
  o->weighted = 1;
  o->step_cap = 0.25;
  o->field_floor = 0.5;
  o->fused = 1;
  o->finish_stall = 0;
  o->finish_tol = 1e-4;
  o->budget_ms = 0.0;
  o->forks = 0;
  o->fork_at = 42;
  o->fork_grace = 6;
  o->fork_first = 1;
  o->fork_err = 1e-5;
  o->fork_scale[0] = 0.9;
  o->fork_scale[1] = 0.8;
  o->fork_scale[2] = 0.6;
  o->fork_scale[3] = 0.95;
  o->graded_ratio = 16.0;
  o->precond_hfloor = 0.1;
}

int scft_batch_create(const scft_instance *inst, int count, scft_batch **out) {
  return create_batch(inst, count, out);
}

int scft_batch_set_fields(scft_batch *b, const double *w_nodes) {
  if (!b || !w_nodes) return set_err(SCFT_EINVAL, "scft_batch_set_fields");
  CK(cudaMemcpy(b->d_w, w_nodes, b->total_nodes * sizeof(double), cudaMemcpyHostToDevice));
  return SCFT_OK;
}

int scft_batch_evaluate(scft_batch *b, int precision) {
  if (!b) return set_err(SCFT_EINVAL, "scft_batch_evaluate");
  return evaluate(b, precision);
}

int scft_batch_evaluate_scheme(scft_batch *b, int scheme, int wmode) {
  if (!b) return set_err(SCFT_EINVAL, "scft_batch_evaluate_scheme");
  int rc = fill_int(b->d_active, b->count, 2, b->st);
  if (rc) return rc;
  CK(cudaMemsetAsync(b->d_status, 0, b->count * sizeof(int), b->st));
  CK(cudaEventRecord(b->t0, b->st));
  if ((rc = seq_enqueue(b, scheme, wmode))) return rc;
  CK(cudaEventRecord(b->t1, b->st));
  CK(cudaStreamSynchronize(b->st));
  CK(cudaEventElapsedTime(&b->last_ms, b->t0, b->t1));
  return SCFT_OK;
}

int scft_batch_solve(scft_batch *b, const scft_solve_opts *opts, scft_result *res) {
  if (!b) return set_err(SCFT_EINVAL, "scft_batch_solve");
  scft_solve_opts o;
  scft_solve_opts_init(&o);
  const scft_solve_opts *op = opts ? opts : &o;
  if (op->transfer_stride > 1) {
    if (check_opts(op)) return SCFT_EINVAL;
    if (b->pending) return set_err(SCFT_EINVAL, "a solve of this batch is in flight: call scft_batch_wait");
    return solve_staged(b, op, res);
  }
  return solve(b, op, res);
}

int scft_batch_solve_async(scft_batch *b, const scft_solve_opts *opts) {
  if (!b) return set_err(SCFT_EINVAL, "scft_batch_solve_async");
  scft_solve_opts d;
  scft_solve_opts_init(&d);
  const scft_solve_opts *o = opts ? opts : &d;
  if (check_opts(o)) return SCFT_EINVAL;
  if (o->precision != PREC_F32 || !o->fused || o->verify64 || o->transfer_stride > 1)
    return set_err(SCFT_EINVAL,
                   "asynchronous solves run the fused FP32 form (fused = 1, verify64 = 0, transfer_stride <= 1)");
  if (b->pending) return set_err(SCFT_EINVAL, "a solve of this batch is in flight: call scft_batch_wait");
  int rc;
  if ((rc = plan(b, PREC_F32, 1.0, o->finish_stall == 0 ? o->forks : 0)) || (rc = ensure_mix(b, o->depth, o->forks)))
    return rc;
  return solve_fused_enqueue(b, o);
}

int scft_batch_wait(scft_batch *b, scft_result *res) {
  if (!b) return set_err(SCFT_EINVAL, "scft_batch_wait");
  return solve_fused_finish(b, res);
}

int scft_batch_get(scft_batch *b, double *w_nodes, double *phi_nodes, double *Q) {
  if (!b) return set_err(SCFT_EINVAL, "scft_batch_get");
  CK(cudaStreamSynchronize(b->st));
  if (w_nodes) CK(cudaMemcpy(w_nodes, b->d_w, b->total_nodes * sizeof(double), cudaMemcpyDeviceToHost));
  if (phi_nodes) CK(cudaMemcpy(phi_nodes, b->d_phi, b->total_nodes * sizeof(double), cudaMemcpyDeviceToHost));
  if (Q) CK(cudaMemcpy(Q, b->d_Q, b->count * sizeof(double), cudaMemcpyDeviceToHost));
  return SCFT_OK;
}

int scft_batch_status(scft_batch *b, int *status) {
  if (!b || !status) return set_err(SCFT_EINVAL, "scft_batch_status");
  CK(cudaMemcpy(status, b->d_status, b->count * sizeof(int), cudaMemcpyDeviceToHost));
  return SCFT_OK;
}

int scft_batch_set_shape(scft_batch *b, int precision, int index, int C, int NW) {
  if (!b || (precision != 0 && precision != 1) || index < 0 || index >= b->count)
    return set_err(SCFT_EINVAL, "scft_batch_set_shape");
  if (C != 0 && (!propagate_has_class(precision, C, NW) || 32 * NW * C < b->n[index] - 2))
    return set_err(SCFT_EINVAL, "scft_batch_set_shape: shape (%d,%d) unavailable", C, NW);
  b->shapeC[precision][index] = C;
  b->shapeNW[precision][index] = C ? NW : 0;
  b->planned[precision] = false;
  return SCFT_OK;
}

int scft_batch_autotune(scft_batch *b, int precision) {
  if (!b || (precision != 0 && precision != 1)) return set_err(SCFT_EINVAL, "scft_batch_autotune");
  return autotune(b, precision);
}

int scft_batch_reset(scft_batch *b) {
  if (!b) return set_err(SCFT_EINVAL, "scft_batch_reset");
  CK(cudaEventRecord(b->t0, b->st));
  CK(cudaMemcpyAsync(b->d_w, b->d_w0, b->total_nodes * sizeof(double), cudaMemcpyDeviceToDevice, b->st));
  CK(cudaEventRecord(b->t1, b->st));
  CK(cudaEventSynchronize(b->t1));
  CK(cudaEventElapsedTime(&b->last_ms, b->t0, b->t1));
  return SCFT_OK;
}

double scft_batch_last_ms(scft_batch *b) { return b ? (double)b->last_ms : -1.0; }

int scft_batch_trace(scft_batch *b, int max, int *active, double *ms) {
  if (!b || max < 0) return set_err(SCFT_EINVAL, "scft_batch_trace");
  const int n = (int)b->trace_active.size();
  for (int i = 0; i < n && i < max; i++) {
    if (active) active[i] = b->trace_active[i];
    if (ms) ms[i] = b->trace_ms[i];
  }
  return n;
}

int scft_batch_profile(scft_batch *b, int precision, int max_classes, int *C, int *NW, int *items,
                       double *bytes, double *ms) {
  if (!b || (precision != 0 && precision != 1) || max_classes < 0) return set_err(SCFT_EINVAL, "scft_batch_profile");
  int rc = plan(b, precision, 1.0);
  if (rc) return rc;
  auto &plans = b->plans[precision];
  const BatchDev bd = batch_dev(b);
  const double esz = precision == PREC_F32 ? 4.0 : 8.0;
  for (size_t k = 0; k < plans.size() && (int)k < max_classes; k++) {
    ClassPlan &cp = plans[k];
    double by = 0.0;
    for (int i : cp.items) by += 2.0 * esz * b->n[i] * (double)(b->nsteps[i] / 2 + 1);
    if ((rc = fill_int(b->d_active, b->count, precision == PREC_F32 ? 1 : 2, b->st))) return rc;
    ClassDev d;
    class_dev(b, cp, &d);
    CK(cudaMemsetAsync(b->d_heads + cp.head, 0, sizeof(int), b->st));
    CK(cudaEventRecord(b->t0, b->st));
    CK(propagate_launch(precision, cp.C, cp.NW, bd, d, cp.grid, b->st));
    g_launches++;
    CK(cudaEventRecord(b->t1, b->st));
    CK(cudaEventSynchronize(b->t1));
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, b->t0, b->t1));
    if (C) C[k] = cp.C;
    if (NW) NW[k] = cp.NW;
    if (items) items[k] = (int)cp.items.size();
    if (bytes) bytes[k] = by;
    if (ms) ms[k] = t;
  }
  return (int)plans.size();
}

int scft_batch_live_stats(scft_batch *b, int precision, int max_classes, int *C, int *NW, long long *launches,
                          double *bytes, double *ms) {
  if (!b || (precision != 0 && precision != 1) || max_classes < 0) return set_err(SCFT_EINVAL, "scft_batch_live_stats");
  const auto &plans = b->plans[precision];
  const double esz = precision == PREC_F32 ? 4.0 : 8.0;
  const size_t nc = std::min(plans.size(), b->live_ms[precision].size());
  for (size_t k = 0; k < nc && (int)k < max_classes; k++) {
    if (C) C[k] = plans[k].C;
    if (NW) NW[k] = plans[k].NW;
    if (launches) launches[k] = b->live_launches[precision][k];
    if (bytes) bytes[k] = 2.0 * esz * b->live_units[precision][k];
    if (ms) ms[k] = b->live_ms[precision][k];
  }
  return (int)nc;
}

int scft_batch_destroy(scft_batch *b) {
  destroy_batch(b);
  return SCFT_OK;
}

}  // extern "C"
