// 128 x 128 x 128 tile products on the CUDA cores (FP32 FMA), used by the
// blocked factorisation and the B^-1 = Z Z^T product.
//   acc(r, c) += sum_k A[r, k] * B[c, k]
// A and B are 128 x 128 tiles of row-major matrices (k contiguous).  256
// threads; thread (tx, ty) = (tid % 16, tid / 16) owns rows
// {ty*4 + 0..3, 64 + ty*4 + 0..3} x cols {tx*4 + 0..3, 64 + tx*4 + 0..3}.
#pragma once

#include "common.cuh"

namespace pgb {

constexpr int KC = 32;           // k-chunk staged in shared memory
constexpr int SROW = T + 4;      // padded row of the staged (transposed) chunk

__device__ __forceinline__ int acc_row(int ty, int e) { return e < 4 ? ty * 4 + e : 64 + ty * 4 + (e - 4); }

__device__ __forceinline__ void acc_zero(float (&acc)[8][8]) {
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int b = 0; b < 8; ++b) acc[a][b] = 0.0f;
}

// Stage a 128 x KC chunk (columns kc .. kc+KC) of tile `src` (ld floats per
// row) into s[k][row] (transposed).  Reads bypass L1 (the data may have been
// written by another block of the same launch).
__device__ __forceinline__ void stage_chunk(const float* __restrict__ src, long long ld, int kc,
                                            float* __restrict__ s) {
  const int t = threadIdx.x;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int row = (t >> 3) + 32 * q;
    const int k4 = (t & 7) * 4;
    const float4 v = __ldcg(reinterpret_cast<const float4*>(src + (size_t)row * ld + kc + k4));
    s[(k4 + 0) * SROW + row] = v.x;
    s[(k4 + 1) * SROW + row] = v.y;
    s[(k4 + 2) * SROW + row] = v.z;
    s[(k4 + 3) * SROW + row] = v.w;
  }
}

__device__ __forceinline__ void acc_gemm_tile(float (&acc)[8][8], const float* __restrict__ A, long long lda,
                                              const float* __restrict__ B, long long ldb, float* __restrict__ sA,
                                              float* __restrict__ sB) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int kc = 0; kc < T; kc += KC) {
    __syncthreads();
    stage_chunk(A, lda, kc, sA);
    stage_chunk(B, ldb, kc, sB);
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < KC; ++k) {
      const float4 a0 = *reinterpret_cast<const float4*>(sA + k * SROW + ty * 4);
      const float4 a1 = *reinterpret_cast<const float4*>(sA + k * SROW + 64 + ty * 4);
      const float4 b0 = *reinterpret_cast<const float4*>(sB + k * SROW + tx * 4);
      const float4 b1 = *reinterpret_cast<const float4*>(sB + k * SROW + 64 + tx * 4);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int r = 0; r < 8; ++r)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[r][c] = fmaf(av[r], bv[c], acc[r][c]);
    }
  }
  __syncthreads();
}

}  // namespace pgb
