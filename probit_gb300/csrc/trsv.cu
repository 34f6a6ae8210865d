// Blocked triangular solve with one factor L (row-major lower tiles):
//   lower: L x = b        trans: L^T x = b
// Wavefront over 128-row blocks: blocks are claimed in solve order through an
// atomic counter, each block accumulates the contributions of already-solved
// blocks as their flags are released, then applies the inverse of its
// diagonal tile (kept by the factorisation).  A block only waits on blocks
// claimed before it, so the launch cannot deadlock.
// Replaces the triangular part of the reference's LU solve
// (implicit/solvers.py:24) in the B form L L^T = B.
#include "kernels.cuh"

namespace pgb {

constexpr int TS_THREADS = 256;

__global__ void __launch_bounds__(TS_THREADS, 1) trsv_kernel(int n, int nt, long long ld, const float* __restrict__ L,
                                                             const float* __restrict__ Linv,
                                                             const float* __restrict__ b, float* __restrict__ x,
                                                             int trans, int* __restrict__ flags,
                                                             int* __restrict__ counter, int* __restrict__ status,
                                                             const int* __restrict__ run_if, int run_when) {
  if (run_if && *run_if != run_when) return;
  __shared__ float sacc[T];
  __shared__ float sx[T];
  __shared__ float spart[2][T];
  __shared__ int s_q, s_ok;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  while (true) {
    __syncthreads();
    if (tid == 0) {
      int q = atomicAdd(counter, 1);
      if (q < nt && ld_relaxed(status + ST_ABORT)) q = nt;
      s_q = q;
    }
    __syncthreads();
    const int q = s_q;
    if (q >= nt) break;
    const int i = trans ? nt - 1 - q : q;
    if (tid < T) {
      const int gi = i * T + tid;
      sacc[tid] = gi < n ? __ldcg(b + gi) : 0.0f;
    }
    const int k_begin = trans ? i + 1 : 0;
    const int k_end = trans ? nt : i;
    bool ok = true;
    for (int k = k_begin; k < k_end; ++k) {
      if (tid == 0) {
        s_ok = wait_flag_geq(flags + k, 1, status) ? 1 : 0;
        __threadfence();
      }
      __syncthreads();
      if (!s_ok) {
        ok = false;
        break;
      }
      if (tid < T) sx[tid] = __ldcg(x + (size_t)k * T + tid);
      __syncthreads();
      if (!trans) {
        // sacc[r] -= sum_c L[iT + r, kT + c] x_k[c]; warp w owns rows 16w..16w+15
        for (int rr = 0; rr < 16; ++rr) {
          const int r = warp * 16 + rr;
          const float4 lv = __ldcg(reinterpret_cast<const float4*>(L + (size_t)(i * T + r) * ld + k * T + lane * 4));
          float s = lv.x * sx[lane * 4] + lv.y * sx[lane * 4 + 1] + lv.z * sx[lane * 4 + 2] + lv.w * sx[lane * 4 + 3];
          s = warp_sum(s);
          if (lane == 0) sacc[r] -= s;
        }
      } else {
        // sacc[r] -= sum_c L[kT + c, iT + r] x_k[c]
        const int r = tid & (T - 1), half = tid >> 7;
        float s = 0.0f;
        for (int c = half * 64; c < half * 64 + 64; ++c)
          s = fmaf(__ldcg(L + (size_t)(k * T + c) * ld + i * T + r), sx[c], s);
        spart[half][r] = s;
        __syncthreads();
        if (tid < T) sacc[tid] -= spart[0][tid] + spart[1][tid];
      }
      __syncthreads();
    }
    if (!ok) continue;
    // diagonal tile: x_i = Linv_ii acc (lower) or Linv_ii^T acc (trans)
    const float* Li = Linv + (size_t)i * T * T;
    if (tid < T) sx[tid] = sacc[tid];
    __syncthreads();
    if (!trans) {
      for (int rr = 0; rr < 16; ++rr) {
        const int r = warp * 16 + rr;
        const float4 lv = __ldcg(reinterpret_cast<const float4*>(Li + (size_t)r * T + lane * 4));
        float s = lv.x * sx[lane * 4] + lv.y * sx[lane * 4 + 1] + lv.z * sx[lane * 4 + 2] + lv.w * sx[lane * 4 + 3];
        s = warp_sum(s);
        if (lane == 0) sacc[r] = s;
      }
    } else {
      const int c = tid & (T - 1), half = tid >> 7;
      float s = 0.0f;
      for (int r = half * 64; r < half * 64 + 64; ++r) s = fmaf(__ldcg(Li + (size_t)r * T + c), sx[r], s);
      spart[half][c] = s;
      __syncthreads();
      if (tid < T) sacc[tid] = spart[0][tid] + spart[1][tid];
    }
    __syncthreads();
    if (tid < T) x[(size_t)i * T + tid] = sacc[tid];
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      st_release(flags + i, 1);
    }
  }
}

void trsv_set_attributes() {}

void launch_trsv(int n, int nt, long long ld, const float* L, const float* Linv, const float* b, float* x, int trans,
                 int* flags, int* counter, int* status, int grid, const int* run_if, int run_when, cudaStream_t st) {
  trsv_kernel<<<grid, TS_THREADS, 0, st>>>(n, nt, ld, L, Linv, b, x, trans, flags, counter, status, run_if, run_when);
}

}  // namespace pgb
