// vca_umma.cuh -- BF16 GEMM on the sm_103a tensor cores (tcgen05), used by
// the Omega surrogate network.
//
// C[M x 128] (fp32, row-major) = A[M x K] * B[128 x K]^T, optionally added to
// C.  A and B are bf16 in the tiled K-major layout below, so that each
// 128-row x 64-column chunk is one contiguous 16 KB block that one
// cp.async.bulk moves to shared memory, already in the tensor core's
// no-swizzle canonical form:
//   * a chunk holds 16 x 8 core matrices of 8 rows x 8 columns (128 bytes,
//     row-major inside);
//   * core matrix (rb, kb) of a chunk sits at (kb * 16 + rb) * 128 bytes, so
//     the K-direction core stride (LBO) is 2048 bytes and the row-direction
//     one (SBO) 128 bytes;
//   * chunk (rt, kt) of an R x K matrix is block rt * (K / 64) + kt.
// R must be a multiple of 128 and K of 64.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace vca {

#define UMMA_CHUNK_ELEMS 8192  // 128 x 64 bf16

__host__ __device__ __forceinline__ size_t umma_off(int r, int k, int K) {
  const int rt = r >> 7, kt = k >> 6, rr = r & 127, kk = k & 63;
  return ((size_t)rt * (size_t)(K >> 6) + (size_t)kt) * UMMA_CHUNK_ELEMS +
         (size_t)((((kk >> 3) << 4) + (rr >> 3)) << 6) + (size_t)((rr & 7) << 3) + (size_t)(kk & 7);
}

// status codes written by the kernel (0 = fine)
#define UMMA_ST_TIMEOUT_LOAD 1
#define UMMA_ST_TIMEOUT_MMA 2
#define UMMA_ST_BAD_SHAPE 3

// opt the kernel into its 98 KB of dynamic shared memory; call once before
// the first launch (outside any stream capture)
cudaError_t umma_prepare();

// C = A B^T (+ C if accumulate) for M/128 row tiles; status: device int,
// set to a nonzero code when a bounded wait runs out (the kernel then frees
// its tensor memory and returns).  extra_tx > 0 makes every chunk's load
// barrier expect bytes that never arrive, so that its bounded wait runs out:
// the timeout test's switch, 0 otherwise.
void launch_umma_gemm(const __nv_bfloat16* A, const __nv_bfloat16* B, float* C, int M, int K, int accumulate,
                      int* status, cudaStream_t st, uint32_t extra_tx = 0);

}  // namespace vca
