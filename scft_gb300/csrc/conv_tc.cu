// conv_tc.cu -- the warm-start network's 64 -> 64 dilated convolutions as
// tcgen05 tensor-core GEMMs (no counterpart in the reference, whose initial
// fields come from files: 1D_FEM.c:321-342, scft_util.cc:14-41).
//
// One CTA of 128 threads per instance.  For each tap k the layer is the GEMM
//   D[p][co] += A_k[p][ci] * B_k[co][ci],   A_k[p][ci] = x[ci][p + (k-2) dil],
// M = 256 points (two 128-row tiles), N = 64 output channels, K = 5 taps x 64
// input channels.  The threads build the five shifted copies A_k (BF16) in
// shared memory in the canonical K-major layout without swizzle (8-row x
// 16-byte core matrices: K chunks 128 B apart, row groups 1024 B apart); the
// BF16 weight image B (same layout) arrives by one bulk asynchronous copy
// (cp.async.bulk, completion on an mbarrier).  One thread issues the 2 x 20
// tcgen05.mma (kind::f16, BF16 x BF16 -> FP32) into two 64-column accumulators
// in tensor memory and commits them to a second mbarrier; each warp then reads
// its 32 rows of both accumulators (tcgen05.ld 32x32b), adds the bias, applies
// tanh and stores BF16.  Every wait is bounded (one second of %globaltimer);
// a wait that runs out sets *err, skips what depended on it and still frees the
// tensor memory.
#include <cstdint>

#include "conv_tc.cuh"

namespace scft {
namespace {

constexpr int P = 256, CH = 64, KT = 5, THREADS = 128;
constexpr int A_TAP = P * CH * 2;       // bytes of one shifted copy A_k (both row tiles)
constexpr int A_TILE = 128 * CH * 2;    // bytes of one 128-row tile of A_k
constexpr int A_BYTES = KT * A_TAP;
constexpr int B_TAP = CH * CH * 2;
constexpr int B_BYTES = KT * B_TAP;
static_assert(B_BYTES == CONV_TC_IMAGE_BYTES, "weight image size");
constexpr int SMEM_BYTES = A_BYTES + B_BYTES + 64;  // + two mbarriers, the TMEM address, a flag
constexpr unsigned TMEM_COLS = 128;                // two 128 x 64 FP32 accumulators
constexpr unsigned long long WAIT_NS = 1000000000ull;

// Byte offset of element (row r, K element e) in a canonical K-major tile
// without swizzle.
__host__ __device__ constexpr unsigned canon(int r, int e) {
  return (unsigned)((r >> 3) * 1024 + (e >> 3) * 128 + (r & 7) * 16 + (e & 7) * 2);
}

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of a tcgen05.mma operand: start address,
// leading byte offset 128 (next K chunk), stride byte offset 1024 (next 8 rows),
// descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t mdesc(unsigned addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
         (1ull << 46);
}

// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator, BF16 A and
// B, both K-major, N = 64, M = 128.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for phase `parity` of the mbarrier at `bar`; false after WAIT_NS.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  const unsigned long long t0 = now_ns();
  for (unsigned it = 0;; it++) {
    unsigned done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if ((it & 255u) == 255u && now_ns() - t0 > WAIT_NS) return false;
  }
}

__device__ __forceinline__ void tmem_ld16(unsigned taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__global__ void conv_tc_pack_kernel(const float *__restrict__ W, __nv_bfloat16 *__restrict__ img) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // over co, ci, k of W[co][ci][k]
  if (i >= CH * CH * KT) return;
  const int k = i % KT, ci = (i / KT) % CH, co = i / (KT * CH);
  img[(k * B_TAP + canon(co, ci)) / 2] = __float2bfloat16_rn(W[i]);
}

template <int DIL, bool ACT>
__global__ void __launch_bounds__(THREADS, 1)
    conv_tc_kernel(const __nv_bfloat16 *__restrict__ x, const __nv_bfloat16 *__restrict__ img,
                   const float *__restrict__ bias, __nv_bfloat16 *__restrict__ y, int *err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char *A = sm;
  unsigned char *Bs = sm + A_BYTES;
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm + A_BYTES + B_BYTES);  // [0] weights, [1] products
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(bar + 2);
  int *go = reinterpret_cast<int *>(tmem_slot + 1);
  const int b = blockIdx.x, t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const unsigned bar_w = smem_addr(&bar[0]), bar_d = smem_addr(&bar[1]);

  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_w) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_d) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  if (t == 0) {
    // the weight image: one bulk copy, completion counted on bar_w
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_w), "r"(B_BYTES) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(Bs)),
        "l"(img), "r"(B_BYTES), "r"(bar_w)
        : "memory");
  }

  // the five shifted copies A_k (zero outside the 256 points)
  const unsigned short *xb = reinterpret_cast<const unsigned short *>(x) + (size_t)b * CH * P;
#pragma unroll 1
  for (int half = 0; half < 2; half++) {
    const int p = half * 128 + t;
#pragma unroll 1
    for (int k = 0; k < KT; k++) {
      const int q = p + (k - 2) * DIL;
      const bool in = q >= 0 && q < P;
      unsigned char *At = A + k * A_TAP;
#pragma unroll
      for (int c = 0; c < CH / 8; c++) {
        uint32_t v[4];
#pragma unroll
        for (int h = 0; h < 4; h++) {
          const uint32_t lo = in ? __ldg(xb + (8 * c + 2 * h) * P + q) : 0u;
          const uint32_t hi = in ? __ldg(xb + (8 * c + 2 * h + 1) * P + q) : 0u;
          v[h] = lo | (hi << 16);
        }
        *reinterpret_cast<uint4 *>(At + canon(p, 8 * c)) = make_uint4(v[0], v[1], v[2], v[3]);
      }
    }
  }
  // generic-proxy stores -> visible to the tensor core's reads
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  const unsigned tmem = *tmem_slot;

  if (t == 0) {
    int ok = mbar_wait(bar_w, 0) ? 1 : 0;
    if (ok) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
      for (int m = 0; m < 2; m++) {
#pragma unroll 1
        for (int k = 0; k < KT; k++) {
#pragma unroll
          for (int j = 0; j < CH / 16; j++) {
            const uint64_t ad = mdesc(smem_addr(A + k * A_TAP + m * A_TILE + j * 256));
            const uint64_t bd = mdesc(smem_addr(Bs + k * B_TAP + j * 256));
            const uint32_t acc = (k | j) ? 1u : 0u;
            asm volatile(
                "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem + m * 64),
                "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                : "memory");
          }
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_d)
                   : "memory");
    } else {
      atomicExch(err, 1);
    }
    *go = ok;
  }
  __syncthreads();

  if (*go) {
    // one waiter per warp, so that the warp stays converged for tcgen05.ld
    int done = 0;
    if (lane == 0) done = mbar_wait(bar_d, 0) ? 1 : 0;
    done = __shfl_sync(0xffffffffu, done, 0);
    if (done) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
      for (int m = 0; m < 2; m++) {
        const int p = m * 128 + warp * 32 + lane;
        __nv_bfloat16 *yp = y + (size_t)b * CH * P + p;
#pragma unroll 1
        for (int c0 = 0; c0 < CH; c0 += 16) {
          uint32_t r[16];
          tmem_ld16(tmem + ((unsigned)(warp * 32) << 16) + m * 64 + c0, r);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int i = 0; i < 16; i++) {
            float v = __uint_as_float(r[i]) + __ldg(bias + c0 + i);
            if (ACT) v = tanhf(v);
            yp[(size_t)(c0 + i) * P] = __float2bfloat16_rn(v);
          }
        }
      }
    } else if (lane == 0) {
      atomicExch(err, 2);
      mbar_wait(bar_d, 0);  // give products still in flight a second chance before the memory goes
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

template <int DIL, bool ACT>
cudaError_t launch(const __nv_bfloat16 *x, const __nv_bfloat16 *img, const float *bias, __nv_bfloat16 *y, int B,
                   int *err, cudaStream_t st) {
  auto kern = conv_tc_kernel<DIL, ACT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
  if (e != cudaSuccess) return e;
  kern<<<B, THREADS, SMEM_BYTES, st>>>(x, img, bias, y, err);
  return cudaGetLastError();
}

}  // namespace

cudaError_t conv_tc_pack(const float *W, __nv_bfloat16 *img, cudaStream_t st) {
  conv_tc_pack_kernel<<<(CH * CH * KT + 255) / 256, 256, 0, st>>>(W, img);
  return cudaGetLastError();
}

cudaError_t conv_tc_forward(const __nv_bfloat16 *x, const __nv_bfloat16 *img, const float *bias, int dil, int act,
                            __nv_bfloat16 *y, int B, int *err, cudaStream_t st) {
  if (B <= 0) return cudaSuccess;
  switch (dil * 2 + (act ? 1 : 0)) {
    case 2: return launch<1, false>(x, img, bias, y, B, err, st);
    case 3: return launch<1, true>(x, img, bias, y, B, err, st);
    case 4: return launch<2, false>(x, img, bias, y, B, err, st);
    case 5: return launch<2, true>(x, img, bias, y, B, err, st);
    case 8: return launch<4, false>(x, img, bias, y, B, err, st);
    case 9: return launch<4, true>(x, img, bias, y, B, err, st);
    case 16: return launch<8, false>(x, img, bias, y, B, err, st);
    case 17: return launch<8, true>(x, img, bias, y, B, err, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace scft
