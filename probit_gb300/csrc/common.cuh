// Shared device helpers for the probit_gb300 CUDA library (sm_103a).
//
// Hyperparameter block layout (float32, device memory), the same layout the
// C-ABI documents in include/probit_gb300.h:
//   theta = [ l_0 .. l_{nl-1}, s, sigma_n, b_0 .. b_J ]
// nl = 1 (isotropic) or D (ARD); s = signal variance; sigma_n = noise std;
// b = ordinal cutpoints (probit only; b_0 = -inf, b_J = +inf).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "../../include/probit_gb300.h"

namespace pgb {

constexpr int T = 128;           // tile edge of every blocked matrix
// k-columns of one tensor-core pipeline chunk: one tensor-map box of 128
// rows, stored with a 64-byte swizzle (16 fp32 a row) or a 128-byte one (32)
constexpr int CHUNK_COLS = 32;
constexpr int MAX_D = 16;        // input dimensions handled by the kernels
constexpr int MAX_THETA = 64;    // entries of one hyperparameter block

// Device status word layout (int32[8]) shared by every kernel of one GP.
enum StatusSlot {
  ST_CODE = 0,        // first error code (PGB_E*), 0 = ok
  ST_ITERS = 1,       // Newton iterations done
  ST_NOTPD_COL = 2,   // first column whose pivot was not positive (or -1)
  ST_ABORT = 3,       // set by any kernel that gave up waiting
  ST_CONVERGED = 4,   // 1 once the fixed point test passed
  ST_WAIT_US = 5,     // limit of this problem's flag waits in microseconds (0: WAIT_LIMIT_NS);
                      // written only by a test hook, kept across operations
  ST_STALL = 6,       // consecutive Newton steps that did not halve ||delta||
  ST_PREV_ERR = 7,    // float bits of the previous step's ||delta||
};
// A Newton loop that has stopped contracting (kStallSteps steps in a row
// without halving ||delta||, at ||delta|| <= max(kStallTol * tol,
// kStallAbs)) is at the float32 floor of its fixed point; its remaining
// steps reuse the resident factor.
constexpr int kStallSteps = 2;
constexpr float kStallTol = 16.0f;
constexpr float kStallAbs = 1e-2f;

// ---------------------------------------------------------------- memory order
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait for *flag >= target.  Gives up after WAIT_LIMIT_NS of wall
// time (or the problem's ST_WAIT_US override) or as soon as another block has
// raised the abort word; a give-up raises the abort word itself (with
// PGB_ETIMEOUT as the status code when none is set) so every other waiter of
// this launch returns promptly.  Returns true when the flag was seen.
constexpr uint64_t WAIT_LIMIT_NS = 4000000000ull;   // 4 s
// wait_flag_value: the same wait for a target >= 1, returning the value
// seen (>= target), or 0 when it gave up.
__device__ __forceinline__ int wait_flag_value(const int* flag, int target, int* status) {
  int v = ld_acquire(flag);
  if (v >= target) return v;
  const uint64_t t0 = global_ns();
  const int limit_us = ld_relaxed(status + ST_WAIT_US);
  const uint64_t limit_ns = limit_us > 0 ? (uint64_t)limit_us * 1000ull : WAIT_LIMIT_NS;
  unsigned ns = 32;
  while (true) {
    v = ld_acquire(flag);
    if (v >= target) return v;
    if (ld_relaxed(status + ST_ABORT)) return 0;
    if (global_ns() - t0 > limit_ns) {
      atomicCAS(status + ST_CODE, 0, PGB_ETIMEOUT);
      atomicExch(status + ST_ABORT, 1);
      return 0;
    }
    __nanosleep(ns);
    if (ns < 256) ns <<= 1;
  }
}

__device__ __forceinline__ bool wait_flag_geq(const int* flag, int target, int* status) {
  return target <= 0 || wait_flag_value(flag, target, status) >= target;
}

__device__ __forceinline__ void raise_status(int* status, int code) {
  atomicCAS(status + ST_CODE, 0, code);
}

// ---------------------------------------------------------------- kernels
// Kernel functions restated from mlkernels' EQ / Matern12 / EQ.periodic(p)
// with ``stretch`` (the inputs are divided by the lengthscale before the
// distance).  Every kernel is evaluated on prepared features:
//   eq, matern12 : f_d = x_d / l_d                         (F = D features)
//   eq_periodic  : f_2d = sin(2 pi x_d / p) / l_d,
//                  f_2d+1 = cos(2 pi x_d / p) / l_d          (F = 2D features)
// (mlkernels' periodic composition maps each input to (sin, cos) and the
// stretch divides them by l; (sin a - sin b)^2 + (cos a - cos b)^2 =
// 4 sin^2((a - b) / 2), so the feature distance is the periodic one).
// Feature rows are zero padded to Dp = 4 ceil(F / 4), so a kernel value is
// d2 = sum over all Dp features of (f_i - f_j)^2, then
//   eq, eq_periodic: s exp(-d2 / 2),   matern12: s exp(-sqrt(d2)).
__device__ __forceinline__ float kernel_of_d2(int matern, float s, float d2) {
  return s * expf(matern ? -sqrtf(d2) : -0.5f * d2);
}

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of one float per thread into a double (deterministic order).
template <int NT>
__device__ __forceinline__ double block_sum_d(float v, double* smem_red) {
  double w = warp_sum_d((double)v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smem_red[warp] = w;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < NT / 32; ++i) r += smem_red[i];
    smem_red[0] = r;
  }
  __syncthreads();
  r = smem_red[0];
  __syncthreads();
  return r;
}

__host__ __device__ inline int ceil_div(int a, int b) { return (a + b - 1) / b; }

// Tiles (i, j) with j < i <= j + near of an nt-tile factor are solved by
// substitution with the panels of L_jj as they are published (the next
// columns' critical path); the tiles further down wait for L_jj^-1 and use
// the tensor cores.  A deeper band keeps the inverse off the critical path of
// long factorisations; short ones save the substitution work.  near >= 1:
// the tile just below the diagonal publishes its panels for the next
// diagonal tile.  This is the built-in rule; a handle's tuning may set
// another depth per problem (DagJob::near).
__host__ __device__ inline int near_depth(int nt) { return nt >= 16 ? 3 : 2; }
constexpr int kMaxNearDepth = 16;

// Problems of at most this many tile rows are factored whole by one block
// (their tiles run in order on that block, which waits for no other block).
// Off by default (0): PGB_WHOLE_TILES=k turns it on for N <= 128 k.
constexpr int kWholeMaxTiles = 0;

}  // namespace pgb

namespace pgb {

// Static shape of one GP problem (kernel arguments by value).
struct Shape {
  int n;          // training points
  int D;          // input dims
  int F;          // kernel features (D, or 2D for eq_periodic)
  int Dp;         // feature row stride (floats, multiple of 4, <= MAX_D)
  int kind;       // PGB_KERNEL_*
  int nl;         // lengthscales (1 or D)
  int lik;        // PGB_LIK_*
  int J;          // ordinal classes
  float inv_p;    // 1 / period
};

// Shape of a validated descriptor.
inline Shape shape_from_desc(const pgb_desc* d) {
  Shape s;
  s.n = d->n;
  s.D = d->d;
  s.F = d->kernel == PGB_KERNEL_EQ_PERIODIC ? 2 * d->d : d->d;
  s.Dp = (s.F + 3) / 4 * 4;
  s.kind = d->kernel;
  s.nl = d->n_lengthscales;
  s.lik = d->likelihood;
  s.J = d->likelihood == PGB_LIK_GAUSSIAN ? 0 : d->j;
  s.inv_p = d->kernel == PGB_KERNEL_EQ_PERIODIC ? (float)(1.0 / (double)d->period) : 0.0f;
  return s;
}

// Kernel features of a descriptor (F above); the kernels handle F <= MAX_D.
inline int feature_count(const pgb_desc* d) { return d->kernel == PGB_KERNEL_EQ_PERIODIC ? 2 * d->d : d->d; }

__device__ __forceinline__ float theta_signal(const Shape& sh, const float* theta) { return __ldg(theta + sh.nl); }

__device__ __forceinline__ float theta_sigma(const Shape& sh, const float* theta) {
  return __ldg(theta + sh.nl + 1);
}
__device__ __forceinline__ const float* theta_cutpoints(const Shape& sh, const float* theta) {
  return theta + sh.nl + 2;
}
__host__ __device__ inline int theta_len(int nl, int lik, int J) {
  return nl + 2 + (lik == PGB_LIK_GAUSSIAN ? 0 : J + 1);
}

}  // namespace pgb
