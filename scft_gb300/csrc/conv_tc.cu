// conv_tc.cu -- the warm-start network's 64 -> 64 dilated convolutions as
// tcgen05 tensor-core GEMMs (no counterpart in the reference, whose initial
// fields come from files: 1D_FEM.c:321-342, scft_util.cc:14-41).
//
// One CTA of 128 threads per instance.  For each tap k the layer is the GEMM
//   D[p][co] += A_k[p][ci] * B_k[co][ci],   A_k[p][ci] = x[ci][p + s_k], s_k = (k-2) dil,
// M = 256 points (two 128-row tiles), N = 64 output channels, K = 5 taps x 64
// input channels.  A tensor-map copy (cp.async.bulk.tensor, TMA) brings the
// instance's input x[64][256] (BF16, 32 KB) into shared memory, and one bulk
// copy brings the BF16 weight image; both complete on mbarriers.  The threads
// then transpose x into the canonical K-major operand layout without swizzle
// (8-row x 16-byte core matrices: K chunks 128 B apart, row groups 1024 B
// apart).  An operand's start must fall on a row group, so the shifts s_k are
// served by 8/dil copies of the transposed input, copy i shifted by i*dil rows:
// tap k reads copy (s_k mod 8)/dil from the row group that puts row p at
// p + s_k.  One thread issues the 2 x 20 tcgen05.mma (kind::f16, BF16 x BF16
// -> FP32) into two 64-column accumulators in tensor memory and commits them
// to a third mbarrier; each warp then reads its 32 rows of both accumulators
// (tcgen05.ld 32x32b), adds the bias, applies tanh and stores BF16.  Every wait
// is bounded (one second of %globaltimer); a wait that runs out sets *err,
// skips what depended on it and still frees the tensor memory.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdint>

#include "conv_tc.cuh"

namespace scft {
namespace {

constexpr int P = 256, CH = 64, KT = 5, THREADS = 128;
constexpr int X_BYTES = CH * P * 2;     // the instance's input, [ci][p] BF16
constexpr int B_TAP = CH * CH * 2;
constexpr int B_BYTES = KT * B_TAP;
static_assert(B_BYTES == CONV_TC_IMAGE_BYTES, "weight image size");
constexpr unsigned TMEM_COLS = 128;                // two 128 x 64 FP32 accumulators
constexpr unsigned long long WAIT_NS = 1000000000ull;

// Shifted copies of the transposed input for dilation DIL (2, 4 or 8): NR
// copies of R rows; copy i holds row j = x^T[j + i*DIL - H] (zero outside the
// 256 points), H the halo rounded up to a row group.
template <int DIL>
struct Copies {
  static_assert(DIL == 2 || DIL == 4 || DIL == 8, "dilation 2, 4 or 8");
  static constexpr int NR = 8 / DIL;
  static constexpr int H = (2 * DIL + 7) / 8 * 8;
  static constexpr int R = P + 2 * H;
  static constexpr int BYTES = NR * R * CH * 2;
  static constexpr int SMEM = X_BYTES + BYTES + B_BYTES + 64;  // + three mbarriers, the TMEM address, a flag
};

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
    conv_tc_kernel(const __grid_constant__ CUtensorMap xmap, const __nv_bfloat16 *__restrict__ img,
                   const float *__restrict__ bias, __nv_bfloat16 *__restrict__ y, int *err) {
  using Cp = Copies<DIL>;
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char *X = sm;                       // [ci][p], 512 B per channel
  unsigned char *A = sm + X_BYTES;             // the shifted copies
  unsigned char *Bs = A + Cp::BYTES;
  uint64_t *bar = reinterpret_cast<uint64_t *>(Bs + B_BYTES);  // [0] input, [1] weights, [2] products
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(bar + 3);
  int *go = reinterpret_cast<int *>(tmem_slot + 1);
  const int b = blockIdx.x, t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const unsigned bar_x = smem_addr(&bar[0]), bar_w = smem_addr(&bar[1]), bar_d = smem_addr(&bar[2]);

  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_x) : "memory");
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
    // the input tile (rows b*64 .. b*64+63 of the [B*64][256] tensor) by TMA,
    // the weight image by one bulk copy
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_x), "r"(X_BYTES) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_addr(X)),
        "l"(reinterpret_cast<uint64_t>(&xmap)), "r"(0), "r"(b * CH), "r"(bar_x)
        : "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_w), "r"(B_BYTES) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(Bs)),
        "l"(img), "r"(B_BYTES), "r"(bar_w)
        : "memory");
    const int ok = mbar_wait(bar_x, 0) ? 1 : 0;
    if (!ok) atomicExch(err, 3);
    *go = ok;
  }
  __syncthreads();

  if (*go) {
    // the shifted copies, transposed into the operand layout; consecutive
    // threads take consecutive rows (conflict-free reads and writes)
    const unsigned short *xs = reinterpret_cast<const unsigned short *>(X);
#pragma unroll 1
    for (int i = 0; i < Cp::NR; i++) {
      unsigned char *Ci = A + i * (Cp::R * CH * 2);
#pragma unroll 1
      for (int j = t; j < Cp::R; j += THREADS) {
        const int q = j + i * DIL - Cp::H;
        const bool in = q >= 0 && q < P;
#pragma unroll
        for (int c = 0; c < CH / 8; c++) {
          uint32_t v[4] = {0u, 0u, 0u, 0u};
          if (in) {
#pragma unroll
            for (int h = 0; h < 4; h++)
              v[h] = (uint32_t)xs[(8 * c + 2 * h) * P + q] | ((uint32_t)xs[(8 * c + 2 * h + 1) * P + q] << 16);
          }
          *reinterpret_cast<uint4 *>(Ci + canon(j, 8 * c)) = make_uint4(v[0], v[1], v[2], v[3]);
        }
      }
    }
    // generic-proxy stores -> visible to the tensor core's reads
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  const unsigned tmem = *tmem_slot;

  if (t == 0 && *go) {
    int ok = mbar_wait(bar_w, 0) ? 1 : 0;
    if (ok) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
      for (int m = 0; m < 2; m++) {
#pragma unroll 1
        for (int k = 0; k < KT; k++) {
          const int sft = (k - 2) * DIL, r = ((sft % 8) + 8) % 8, i = r / DIL;
          const int row0 = m * 128 + sft - r + Cp::H;  // a multiple of 8
          const unsigned char *Ak = A + i * (Cp::R * CH * 2) + (row0 / 8) * 1024;
#pragma unroll
          for (int jj = 0; jj < CH / 16; jj++) {
            const uint64_t ad = mdesc(smem_addr(Ak + jj * 256));
            const uint64_t bd = mdesc(smem_addr(Bs + k * B_TAP + jj * 256));
            const uint32_t acc = (k | jj) ? 1u : 0u;
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
          uint32_t rr[16];
          tmem_ld16(tmem + ((unsigned)(warp * 32) << 16) + m * 64 + c0, rr);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int i = 0; i < 16; i++) {
            float v = __uint_as_float(rr[i]) + __ldg(bias + c0 + i);
            if (ACT) v = tanhf(v);
            yp[(size_t)(c0 + i) * P] = __float2bfloat16_rn(v);
          }
        }
      }
    } else if (lane == 0) {
      atomicExch(err, 2);
      mbar_wait(bar_d, 0);  // give products still in flight a second chance before the memory goes
    }
  } else if (t == 0) {
    // copies issued but not waited for must land before the CTA's memory goes
    mbar_wait(bar_x, 0);
    mbar_wait(bar_w, 0);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

// cuTensorMapEncodeTiled, from the driver through the runtime (no link to the driver library)
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    cudaGetLastError();
  }
  return fn;
}

template <int DIL, bool ACT>
cudaError_t launch(const __nv_bfloat16 *x, const __nv_bfloat16 *img, const float *bias, __nv_bfloat16 *y, int B,
                   int *err, cudaStream_t st) {
  // x as a [B*64][256] BF16 tensor, one 64 x 256 box per instance
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return cudaErrorNotSupported;
  CUtensorMap map;
  const cuuint64_t dims[2] = {(cuuint64_t)P, (cuuint64_t)B * CH};
  const cuuint64_t strides[1] = {(cuuint64_t)P * 2};
  const cuuint32_t box[2] = {(cuuint32_t)P, (cuuint32_t)CH};
  const cuuint32_t estr[2] = {1, 1};
  if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16 *>(x), dims, strides, box, estr,
          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  auto kern = conv_tc_kernel<DIL, ACT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Copies<DIL>::SMEM);
  if (e != cudaSuccess) return e;
  kern<<<B, THREADS, Copies<DIL>::SMEM, st>>>(map, img, bias, y, err);
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
