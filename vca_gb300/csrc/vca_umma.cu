// vca_umma.cu -- BF16 x BF16 -> FP32 GEMM on the tcgen05 tensor cores.
//
// One CTA of 128 threads per 128-row tile of C; N = 128.  Thread 0 streams
// the K dimension in 64-column chunks: one cp.async.bulk per operand chunk
// (16 KB each, tiled as in vca_umma.cuh) into a two-stage shared-memory ring,
// completion counted on an mbarrier (complete_tx), then four
// tcgen05.mma.cta_group::1.kind::f16 (M=128, N=128, K=16) into a 128-column
// FP32 accumulator in tensor memory, and tcgen05.commit onto the stage's
// second mbarrier, which frees the stage for the chunk after next.  The four
// warps then read the accumulator back with tcgen05.ld (warp w owns TMEM
// lanes 32w..32w+31 = rows of the tile) and write FP32 rows of C.
//
// Every wait is bounded (1 s on the global timer): a wait that runs out
// records a status code, the CTA skips the rest, frees its tensor memory and
// returns, so a fault in the pipeline shows up as an error the host reads
// instead of a hung GPU.
#include "vca_umma.cuh"

#include <vector>

namespace vca {

void count_launch_external();

namespace {

constexpr uint32_t kStageBytes = 32768;  // A chunk + B chunk
constexpr uint32_t kChunkBytes = 16384;
constexpr uint64_t kWaitNs = 1000000000ull;
// kind::f16 instruction descriptor: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
// The descriptors' reach: with LBO = 2048 and SBO = 128 one instruction
// reads 4 KB from its start; the 32 KB of padding past the ring keeps any
// reading of the two offsets (16 core matrices x 2048 + 2 x 128) inside the
// allocation, so a layout error shows up as wrong numbers, not a fault.
constexpr size_t kSmemBytes = 2 * kStageBytes + 1024 + 64 + 32768;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  const uint64_t t0 = gtimer();
  while (!mbar_try_wait(bar, parity))
    if (gtimer() - t0 > kWaitNs) return false;
  return true;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
// shared-memory matrix descriptor, no swizzle: start address, LBO, SBO (all
// >> 4), descriptor version 1 at bits 46-47
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
        "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
        "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__global__ void __launch_bounds__(128, 1)
    k_umma_gemm(const __nv_bfloat16* __restrict__ A, const __nv_bfloat16* __restrict__ B, float* __restrict__ C,
                int K, int accumulate, int* status, uint32_t extra_tx) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ int s_ok;
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  const uint32_t bars = sbase + 2 * kStageBytes;  // load[0], load[1], mma[0], mma[1]
  const uint32_t slot = bars + 32;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nch = K >> 6;
  if (tid == 0) {
    for (int i = 0; i < 4; i++) mbar_init(bars + 8 * i, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_ok = 1;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(128)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  uint32_t tmem;
  asm volatile("ld.shared.u32 %0, [%1];" : "=r"(tmem) : "r"(slot) : "memory");

  if (tid == 0) {
    for (int c = 0; c < nch; c++) {
      const int s = c & 1;
      const uint32_t lb = bars + 8 * s, mb = bars + 16 + 8 * s;
      if (c >= 2 && !mbar_wait_bounded(mb, ((c - 2) >> 1) & 1)) {  // the stage's previous MMAs are done
        atomicExch(status, UMMA_ST_TIMEOUT_MMA);
        s_ok = 0;
        break;
      }
      const uint32_t sa = sbase + s * kStageBytes, sb = sa + kChunkBytes;
      mbar_expect_tx(lb, kStageBytes + extra_tx);  // extra_tx > 0 only in the timeout test
      bulk_g2s(sa, A + ((size_t)blockIdx.x * nch + c) * UMMA_CHUNK_ELEMS, kChunkBytes, lb);
      bulk_g2s(sb, B + (size_t)c * UMMA_CHUNK_ELEMS, kChunkBytes, lb);
      if (!mbar_wait_bounded(lb, (c >> 1) & 1)) {
        atomicExch(status, UMMA_ST_TIMEOUT_LOAD);
        s_ok = 0;
        break;
      }
      tc_fence_after();
#pragma unroll
      for (int j = 0; j < 4; j++)  // K = 16 per instruction: two core matrices along K
        umma_bf16(tmem, sdesc(sa + j * 4096, 2048, 128), sdesc(sb + j * 4096, 2048, 128), (c | j) ? 1u : 0u);
      umma_commit(mb);
    }
  }
  __syncthreads();
  bool have = s_ok != 0;
  if (have) {
    const int c = nch - 1;
    if (!mbar_wait_bounded(bars + 16 + 8 * (c & 1), (c >> 1) & 1)) {
      atomicExch(status, UMMA_ST_TIMEOUT_MMA);
      have = false;
    }
  }
  // the epilogue's tcgen05.ld is warp-collective: every warp agrees on `have`
  have = __syncthreads_and(have ? 1 : 0) != 0;
  tc_fence_after();
  if (have) {
    const int row = blockIdx.x * 128 + warp * 32 + lane;
    float* crow = C + (size_t)row * 128;
#pragma unroll 1
    for (int cb = 0; cb < 128; cb += 32) {
      uint32_t r[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cb, r);
      float4* dst = reinterpret_cast<float4*>(crow + cb);
#pragma unroll
      for (int q = 0; q < 8; q++) {
        float4 v = make_float4(__uint_as_float(r[4 * q]), __uint_as_float(r[4 * q + 1]),
                               __uint_as_float(r[4 * q + 2]), __uint_as_float(r[4 * q + 3]));
        if (accumulate) {
          const float4 o = dst[q];
          v.x += o.x;
          v.y += o.y;
          v.z += o.z;
          v.w += o.w;
        }
        dst[q] = v;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128) : "memory");
}

}  // namespace

cudaError_t umma_prepare() {
  return cudaFuncSetAttribute(k_umma_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
}

void launch_umma_gemm(const __nv_bfloat16* A, const __nv_bfloat16* B, float* C, int M, int K, int accumulate,
                      int* status, cudaStream_t st, uint32_t extra_tx) {
  if (M <= 0 || (M & 127) || K <= 0 || (K & 63)) return;
  count_launch_external();
  k_umma_gemm<<<M / 128, 128, kSmemBytes, st>>>(A, B, C, K, accumulate, status, extra_tx);
}

}  // namespace vca
