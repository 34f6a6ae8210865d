// Blocked triangular solve with one factor L (row-major lower tiles):
//   lower: L x = b        trans: L^T x = b
// Wavefront over 128-row blocks of every problem of a batch: blocks are
// claimed in solve order through an atomic counter, each block accumulates
// the contributions of already-solved blocks as their flags are released,
// then applies the inverse of its diagonal tile (kept by the factorisation).
// A block only waits on blocks claimed before it, so the launch cannot
// deadlock.
// Replaces the triangular part of the reference's LU solve
// (implicit/solvers.py:24) in the B form L L^T = B.
#include "kernels.cuh"

namespace pgb {

constexpr int TS_THREADS = 256;

// A 128 x 128 tile A (row stride lda) in registers: thread t holds rows
// 16 (t >> 5) .. +15, columns 4 (t & 31) .. +3, so every load instruction
// of a warp reads one 512-byte row segment.  The loads are issued before the
// block waits for the vector they multiply.
__device__ __forceinline__ void tile_load(const float* __restrict__ A, long long lda, float4 (&v)[16]) {
  const int t = threadIdx.x;
  const int cq = t & 31, g = t >> 5;
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __ldcg(reinterpret_cast<const float4*>(A + (size_t)(g * 16 + q) * lda + 4 * cq));
}

// acc[r] (+)= sign * sum_c A[r, c] x[c], A in registers (tile_load layout):
// each thread's 16 row partials are summed over the warp's 32 lanes by a
// halving butterfly (16 shuffles), after which lanes 2m and 2m + 1 hold row m.
__device__ __forceinline__ void tile_mv_rows(const float4 (&v)[16], const float* sv, float* sacc, bool assign) {
  const int t = threadIdx.x;
  const int lane = t & 31, g = t >> 5;
  const float4 x = reinterpret_cast<const float4*>(sv)[lane];
  float p[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) p[q] = fmaf(v[q].x, x.x, fmaf(v[q].y, x.y, fmaf(v[q].z, x.z, v[q].w * x.w)));
#pragma unroll
  for (int w = 8; w >= 1; w >>= 1) {   // keep w values: the upper or lower half by lane bit
    const bool up = (lane & (2 * w)) != 0;
#pragma unroll
    for (int q = 0; q < w; ++q) {
      const float send = up ? p[q] : p[q + w];
      const float keep = up ? p[q + w] : p[q];
      p[q] = keep + __shfl_xor_sync(0xffffffffu, send, 2 * w);
    }
  }
  const float s = p[0] + __shfl_xor_sync(0xffffffffu, p[0], 1);
  if ((lane & 1) == 0) {
    const int r = g * 16 + (lane >> 1);
    sacc[r] = assign ? s : sacc[r] - s;
  }
}

// acc[c] (+)= sign * sum_r A[r, c] x[r], A in registers (tile_load layout);
// the 8 warps' partial column sums are combined in spart.
__device__ __forceinline__ void tile_mv_cols(const float4 (&v)[16], const float* sv, float* sacc, float (*spart)[T],
                                             bool assign) {
  const int t = threadIdx.x;
  const int cq = t & 31, g = t >> 5;
  float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const float x = sv[g * 16 + q];
    s.x = fmaf(v[q].x, x, s.x);
    s.y = fmaf(v[q].y, x, s.y);
    s.z = fmaf(v[q].z, x, s.z);
    s.w = fmaf(v[q].w, x, s.w);
  }
  spart[g][4 * cq + 0] = s.x;
  spart[g][4 * cq + 1] = s.y;
  spart[g][4 * cq + 2] = s.z;
  spart[g][4 * cq + 3] = s.w;
  __syncthreads();
  if (t < T) {
    float tot = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) tot += spart[k][t];
    sacc[t] = assign ? tot : sacc[t] - tot;
  }
}

// Claims (problem, position) are taken in list order; each problem's claims
// appear in solve order, so a claim only waits on claims taken before it.
//   trans = 1: L^T x = w   (w = row 0 of Rv, x = x)
//   trans = 0: L w = t     (t, w = row 0 of Rv)
// A claim is skipped when its problem has stopped (only_active), when the
// problem does not reuse its factor this step (run_on_reuse) or when the
// problem has aborted; every claim of such a problem is skipped alike.
__global__ void __launch_bounds__(TS_THREADS, 1) trsv_kernel(const Prob* __restrict__ probs,
                                                             const int2* __restrict__ claims, int nclaims, int trans,
                                                             int* __restrict__ counter, int run_on_reuse,
                                                             int only_active) {
  __shared__ float sacc[T];
  __shared__ __align__(16) float sx[T];
  __shared__ float spart[8][T];
  __shared__ int s_q, s_ok;
  const int tid = threadIdx.x;
  while (true) {
    __syncthreads();
    if (tid == 0) {
      int q = atomicAdd(counter, 1);
      if (q < nclaims) {
        const Prob& P = probs[claims[q].x];
        if ((only_active && *P.active == 0) || (run_on_reuse && P.reuse[2] != 1) || ld_relaxed(P.status + ST_ABORT))
          q = -1;
      }
      s_q = q;
    }
    __syncthreads();
    const int q = s_q;
    if (q >= nclaims) break;
    if (q < 0) continue;
    const int2 cl = claims[q];
    const Prob& P = probs[cl.x];
    const int n = P.sh.n, nt = P.nt;
    const long long ld = P.ld;
    const float* __restrict__ L = P.L;
    const float* __restrict__ b = trans ? P.Rv : P.t;
    float* __restrict__ x = trans ? P.x : P.Rv;
    int* flags = P.tflags + (trans ? 0 : nt);
    int* status = P.status;
    const int i = trans ? nt - 1 - cl.y : cl.y;
    // the inverse of the diagonal tile, needed last, is loaded first
    float4 dv[16];
    tile_load(P.Linv + (size_t)i * T * T, T, dv);
    if (tid < T) {
      const int gi = i * T + tid;
      sacc[tid] = gi < n ? __ldcg(b + gi) : 0.0f;
    }
    // dependencies oldest first (the order they were solved in), so a block
    // accumulates everything already available while the newest is pending;
    // each tile of L is loaded before its vector is waited for
    const int ndep = trans ? nt - 1 - i : i;
    bool ok = true;
    for (int kk = 0; kk < ndep; ++kk) {
      const int k = trans ? nt - 1 - kk : kk;
      float4 v[16];
      tile_load(trans ? L + (size_t)(k * T) * ld + i * T : L + (size_t)(i * T) * ld + k * T, ld, v);
      // thread 0's acquire load, then the barrier, order the block's reads of x_k
      if (tid == 0) s_ok = wait_flag_geq(flags + k, 1, status) ? 1 : 0;
      __syncthreads();
      if (!s_ok) {
        ok = false;
        break;
      }
      if (tid < T) sx[tid] = __ldcg(x + (size_t)k * T + tid);
      __syncthreads();
      if (!trans)
        tile_mv_rows(v, sx, sacc, false);          // sacc -= L_ik x_k
      else
        tile_mv_cols(v, sx, sacc, spart, false);   // sacc -= L_ki^T x_k
      __syncthreads();
    }
    if (!ok) continue;
    // diagonal tile: x_i = Linv_ii acc (lower) or Linv_ii^T acc (trans)
    if (tid < T) sx[tid] = sacc[tid];
    __syncthreads();
    if (!trans)
      tile_mv_rows(dv, sx, sacc, true);
    else
      tile_mv_cols(dv, sx, sacc, spart, true);
    __syncthreads();
    if (tid < T) x[(size_t)i * T + tid] = sacc[tid];
    __syncthreads();
    if (tid == 0) st_release(flags + i, 1);   // orders the block's stores of x_i (barrier above)
  }
}

void trsv_set_attributes() {}

void launch_trsv(const Prob* probs, const int2* claims, int nclaims, int trans, int* counter, int run_on_reuse,
                 int only_active, int grid, cudaStream_t st) {
  if (nclaims <= 0) return;
  trsv_kernel<<<grid, TS_THREADS, 0, st>>>(probs, claims, nclaims, trans, counter, run_on_reuse, only_active);
}

}  // namespace pgb
