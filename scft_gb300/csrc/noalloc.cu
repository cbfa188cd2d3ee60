// noalloc.cu -- density of one instance without any device allocation.
//
// Some callers of this library may not allocate GPU memory: applications whose
// device memory is handed out entirely by another allocator (a framework's
// caching pool with a fixed budget) and may not grow it behind that
// allocator's back, and per-iteration loops -- such as the reference's solvers,
// which call the residual thousands of times -- that cannot afford
// cudaMalloc/cudaFree, which can block on or synchronize the whole device.
// scft_density_noalloc serves them: the caller passes device buffers for the
// inputs and outputs, and the propagator's half-contour store lives in a
// fixed, file-scope device array instead of memory the library allocates.
#include <cstdio>
#include <string>

#include "common.cuh"
#include "propagate_launch.cuh"
#include "scft.h"

namespace {

// Capacity of the shared scratch: 32 MiB.  Every GPU that loads the library
// holds it until the process exits.
constexpr size_t kScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Per-call description of the single instance, written by noalloc_setup_kernel.
struct NoAllocMeta {
  int n, nsteps, active, status, item, head;
  long long node_off;
  double ds, Q;
  double qw[16];
};
static __device__ __align__(256) NoAllocMeta g_meta;

__global__ void noalloc_setup_kernel(NoAllocMeta m, int *status) {
  // Every call reuses g_meta: the work-queue counter and the status must start
  // at zero, the rest is overwritten with this call's instance.
  m.head = 0;
  m.status = 0;
  m.item = 0;
  g_meta = m;
  if (status) *status = 0;
}

}  // namespace

// shape, quadrature and error helpers of the runtime (runtime.cu)
int scft_internal_default_shape(int n_interior, int precision, int *C, int *NW);
int scft_internal_quad_table(int nsteps, double ds, int rule, double *qw);
int scft_internal_set_error(int code, const char *msg);

namespace {
int fail(int code, const std::string &m) { return scft_internal_set_error(code, m.c_str()); }

// Whether p is memory the current device can address as device memory (device
// or managed allocations); host pointers, freed or unknown addresses are not.
bool device_pointer(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}
}  // namespace

extern "C" {

int scft_density_noalloc(int n_nodes, const double *x, const double *w, int nsteps, double ds, int rule,
                         int precision, double *phi, double *Q, int *status, void *stream) {
  if (n_nodes < 3 || nsteps < 1 || !(ds > 0.0) || !x || !w || !phi ||
      (precision != SCFT_F32 && precision != SCFT_F64) ||
      (rule != SCFT_RULE_ROMBERG && rule != SCFT_RULE_TRAPEZOID))
    return fail(SCFT_EINVAL, "scft_density_noalloc: invalid argument");
  NoAllocMeta m = {};
  if (scft_internal_quad_table(nsteps, ds, rule, m.qw) != SCFT_OK)
    return fail(SCFT_EINVAL, "scft_density_noalloc: Romberg needs a power-of-two step count >= 16");
  int C = 0, NW = 0;
  if (scft_internal_default_shape(n_nodes - 2, precision, &C, &NW) != SCFT_OK)
    return fail(SCFT_EINVAL, "scft_density_noalloc: mesh too large for the propagator");
  const long long slot_elems = (long long)(nsteps / 2 + 1) * 32 * NW * C;
  const size_t need = (size_t)slot_elems * (precision == SCFT_F32 ? 4 : 8);
  if (need > kScratchBytes) {
    char buf[256];
    snprintf(buf, sizeof buf,
             "scft_density_noalloc: this instance needs %zu bytes of scratch; the fixed scratch holds %zu "
             "bytes (use scft_batch_evaluate, which allocates)", need, kScratchBytes);
    return fail(SCFT_EINVAL, buf);
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(SCFT_ENODEV, "scft_density_noalloc: no usable CUDA device");
  }
  // the kernels dereference these: only device (or managed) memory is accepted
  if (!device_pointer(x) || !device_pointer(w) || !device_pointer(phi) || (Q && !device_pointer(Q)) ||
      (status && !device_pointer(status)))
    return fail(SCFT_EINVAL, "scft_density_noalloc: x, w, phi, Q and status must be device memory");
  // Host code names the device arrays by host-side stand-ins, not device
  // addresses: ask the runtime for their addresses on the current device.  This
  // is done on every call (it allocates nothing), so a reset or recreated
  // context never leaves a stale address behind.  The first call on a device may
  // load the library's device code, which is why it belongs before any stream
  // capture.
  void *scratch = nullptr, *mp = nullptr;
  e = cudaGetSymbolAddress(&scratch, g_scratch);
  if (e == cudaSuccess) e = cudaGetSymbolAddress(&mp, g_meta);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(SCFT_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  }
  NoAllocMeta *meta = static_cast<NoAllocMeta *>(mp);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int want = precision == SCFT_F32 ? 1 : 2;
  m.n = n_nodes;
  m.nsteps = nsteps;
  m.ds = ds;
  m.node_off = 0;
  m.active = want;
  noalloc_setup_kernel<<<1, 1, 0, st>>>(m, status);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(SCFT_ECUDA, std::string("setup launch: ") + cudaGetErrorString(e));

  scft::BatchDev b;
  b.count = 1;
  b.n = &meta->n;
  b.nsteps = &meta->nsteps;
  b.ds = &meta->ds;
  b.node_off = &meta->node_off;
  b.x = x;
  b.w = w;
  b.phi = phi;
  b.Q = Q ? Q : &meta->Q;
  b.qw = meta->qw;
  b.active = &meta->active;
  b.status = status ? status : &meta->status;
  scft::ClassDev c;
  c.items = &meta->item;
  c.count = 1;
  c.head = &meta->head;
  c.scratch = scratch;
  c.slot_elems = slot_elems;
  c.workers = 1;
  c.want = want;
  e = scft::propagate_launch(precision, C, NW, b, c, 1, st);
  if (e != cudaSuccess) return fail(SCFT_ECUDA, std::string("propagator launch: ") + cudaGetErrorString(e));
  return SCFT_OK;
}

}  // extern "C"
