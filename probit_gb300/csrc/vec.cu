// Per-point kernels of the Newton step, the evidence and the gradient, and
// their deterministic two-phase reductions (block partials in double, then
// one warp per problem summing them in a fixed order).
//
// Batched kernels take the device problem table and vmap, a map from thread
// block to (problem, local block of VT points over the padded length).
#include <climits>

#include "kernels.cuh"
#include "lik.cuh"

namespace pgb {

constexpr int MAX_LIK_SLOTS = 1 + 41;   // sigma_n + cutpoints b_0 .. b_J for J <= 40

__device__ __forceinline__ float load_y(const Shape& sh, const void* y, int i, int* yi) {
  if (sh.lik == PGB_LIK_GAUSSIAN) {
    *yi = 0;
    return static_cast<const float*>(y)[i];
  }
  *yi = static_cast<const int*>(y)[i];
  return 0.0f;
}

// ---------------------------------------------------------------- likelihood
// Stand-alone per-point evaluation (pgb_log_likelihood).
__global__ void lik_eval_kernel(Shape sh, const float* __restrict__ theta, const float* __restrict__ f,
                                const void* __restrict__ y, int n, float* logp, float* d1, float* d2, float* d3) {
  const int i = blockIdx.x * VT + threadIdx.x;
  if (i >= n) return;
  int yi;
  const float yv = load_y(sh, y, i, &yi);
  LikOut o;
  lik_point<false>(sh.lik, f[i], yv, yi, theta_sigma(sh, theta), theta_cutpoints(sh, theta), o);
  if (logp) logp[i] = o.logp;
  if (d1) d1[i] = o.d1;
  if (d2) d2[i] = o.d2;
  if (d3) d3[i] = o.d3;
}

void launch_lik_eval(const Shape& sh, const float* theta, const float* f, const void* y, int n, float* logp,
                     float* d1, float* d2, float* d3, cudaStream_t st) {
  if (n > 0) lik_eval_kernel<<<ceil_div(n, VT), VT, 0, st>>>(sh, theta, f, y, n, logp, d1, d2, d3);
}

// ---------------------------------------------------------------- reset
// Per problem: status words (no error, no iterations, no bad column), reuse
// flags cleared (new theta: no resident factor), active = 1; when zero_a,
// a = 0 over the padded length and with it f = K a = 0 and the last update
// da = 0 (the Newton loop keeps f by f += K da).
__global__ void reset_problems_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap, int zero_a) {
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.enabled == 0) {
    if (m.y == 0 && threadIdx.x == 0) *P.active = 0;
    return;
  }
  const int i = m.y * VT + threadIdx.x;
  if (zero_a && i < P.n_pad) {   // a = 0, f = K a = 0, no update yet
    P.a[i] = 0.0f;
    P.f[i] = 0.0f;
    P.da[i] = 0.0f;
  }
  if (m.y == 0) {
    if (threadIdx.x < 8 && threadIdx.x != ST_WAIT_US)
      P.status[threadIdx.x] = threadIdx.x == ST_NOTPD_COL ? INT_MAX : 0;
    if (threadIdx.x < 4) P.reuse[threadIdx.x] = 0;
    if (threadIdx.x == 0) *P.active = 1;
    if (threadIdx.x == 0) *P.zvalid = 0;
  }
}

void launch_reset_problems(const Prob* probs, const int2* vmap, int nblocks, int zero_a, cudaStream_t st) {
  if (nblocks > 0) reset_problems_kernel<<<nblocks, VT, 0, st>>>(probs, vmap, zero_a);
}

// active = enabled for every problem (the phases after the Newton loop act on
// every enabled problem)
__global__ void activate_enabled_kernel(const Prob* __restrict__ probs, int nprob) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < nprob && *probs[p].enabled != 0) {
    *probs[p].active = 1;
    probs[p].status[ST_STALL] = 0;   // the factor of the final W is compared bitwise again
  } else if (p < nprob) {
    *probs[p].active = 0;
  }
}

void launch_activate_enabled(const Prob* probs, int nprob, cudaStream_t st) {
  activate_enabled_kernel<<<ceil_div(nprob, 128), 128, 0, st>>>(probs, nprob);
}

// ---------------------------------------------------------------- Newton step
// The reference's update is a correction, z <- z - J^-1 (F(z) - z) with
// J = diag(d2) K - I (implicit/solvers.py:18-25).  With W = -d2 and
// B = I + W^1/2 K W^1/2, -J^-1 = (I + W K)^-1 = W^1/2 B^-1 W^-1/2, so
//   r = d1 - a,   delta = W^1/2 B^-1 (W^-1/2 r),   a <- a + delta.
// This form has no subtraction of nearly equal vectors (the GPML form
// r - W^1/2 B^-1 W^1/2 K r cancels where K W is large), so its float32 error
// is that of the reference's LU solve.  W^1/2 is floored at 1e-18 so a W
// that underflows to 0 keeps every quantity finite.
// From f = K a this kernel writes d1, W, W^1/2, r and the right-hand side
// t = r / W^1/2.  Padding entries (i >= n, up to n_pad) are zeroed.
constexpr float kSwFloor = 1e-18f;

__global__ void newton_lik_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const int i = m.y * VT + threadIdx.x;
  if (i >= P.n_pad) return;
  if (i >= P.sh.n) {
    P.d1[i] = 0.0f; P.W[i] = 0.0f; P.sw[i] = 0.0f; P.r[i] = 0.0f; P.t[i] = 0.0f;
    return;
  }
  const Shape sh = P.sh;
  int yi;
  const float yv = load_y(sh, P.y, i, &yi);
  LikOut o;
  lik_point<false>(sh.lik, P.f[i], yv, yi, theta_sigma(sh, P.theta), theta_cutpoints(sh, P.theta), o);
  const float w = -o.d2;
  const float s = fmaxf(sqrtf(w), kSwFloor);
  const float ri = o.d1 - P.a[i];
  P.d1[i] = o.d1;
  P.W[i] = w;
  P.sw[i] = s;
  P.r[i] = ri;
  P.t[i] = ri / s;
}

void launch_newton_lik(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) newton_lik_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

// a_new = a + sw * x; block partial of ||a_new - a||^2 (as jaxopt measures
// it, on the rounded new iterate); a <- a_new
__global__ void newton_update_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  __shared__ double sred[VT / 32];
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;   // uniform per block
  const int i = m.y * VT + threadIdx.x;
  float e = 0.0f;
  if (i < P.sh.n) {
    const float ai = P.a[i];
    const float an = ai + P.sw[i] * P.x[i];
    const float dlt = an - ai;
    e = dlt * dlt;
    P.a[i] = an;
    P.da[i] = dlt;
  } else if (i < P.n_pad) {
    P.da[i] = 0.0f;
  }
  const double s = block_sum_d<VT>(e, sred);
  if (threadIdx.x == 0) P.part[m.y] = s;
}

void launch_newton_update(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) newton_update_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

// One warp per active problem: err = sqrt(sum part); iterations += 1; decide
// whether this problem goes on.  jaxopt FixedPointIteration semantics
// (solvers.py:7-15): keep going while err > tol and fewer than maxiter
// updates were made; a NaN error stops.
__global__ void newton_finalize_kernel(const Prob* __restrict__ probs, int nprob, int* __restrict__ any_active) {
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= nprob) return;
  const Prob& P = probs[w];
  if (*P.active == 0) return;
  const int nparts = ceil_div(P.n_pad, VT);
  double s = 0.0;
  for (int k = lane; k < nparts; k += 32) s += P.part[k];
  s = warp_sum_d(s);
  if (lane == 0) {
    int* status = P.status;
    const float err = (float)sqrt(s);
    const int it = status[ST_ITERS] + 1;
    status[ST_ITERS] = it;
    *P.err = err;
    const float prev = __int_as_float(status[ST_PREV_ERR]);
    const bool flat = it > 1 && err > 0.5f * prev && err <= fmaxf(kStallTol * P.tol, kStallAbs);
    status[ST_STALL] = flat ? status[ST_STALL] + 1 : 0;
    status[ST_PREV_ERR] = __float_as_int(err);
    if (!(err > P.tol)) status[ST_CONVERGED] = 1;
    if (err != err) atomicCAS(status + ST_CODE, 0, PGB_ENAN);
    const bool again = (err > P.tol) && (it < P.maxiter) && (status[ST_ABORT] == 0);
    *P.active = again ? 1 : 0;
    if (again) atomicOr(any_active, 1);
  }
}

// any_active[0] -> loop condition; copied to any_active[1] for a host-driven
// loop; any_active[0] cleared for the next step.
__global__ void newton_cond_kernel(int* any_active, cudaGraphConditionalHandle cond, int use_cond) {
  const int v = any_active[0];
  any_active[1] = v;
  any_active[0] = 0;
  if (use_cond) cudaGraphSetConditional(cond, v ? 1u : 0u);
}

void launch_newton_finalize(const Prob* probs, int nprob, int* any_active, cudaGraphConditionalHandle cond,
                            int use_cond, cudaStream_t st) {
  newton_finalize_kernel<<<ceil_div(nprob, 8), 256, 0, st>>>(probs, nprob, any_active);
  newton_cond_kernel<<<1, 1, 0, st>>>(any_active, cond, use_cond);
}

// ---------------------------------------------------------------- precision
// Full per-point terms at the final f: logp, d1, d3, W, sw (padding 0).
__global__ void lik_full_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const int i = m.y * VT + threadIdx.x;
  if (i >= P.n_pad) return;
  if (i >= P.sh.n) {
    P.logp[i] = 0.0f; P.d1[i] = 0.0f; P.d3[i] = 0.0f; P.W[i] = 0.0f; P.sw[i] = 0.0f;
    return;
  }
  const Shape sh = P.sh;
  int yi;
  const float yv = load_y(sh, P.y, i, &yi);
  LikOut o;
  lik_point<false>(sh.lik, P.f[i], yv, yi, theta_sigma(sh, P.theta), theta_cutpoints(sh, P.theta), o);
  P.logp[i] = o.logp;
  P.d1[i] = o.d1;
  P.d3[i] = o.d3;
  P.W[i] = -o.d2;
  P.sw[i] = fmaxf(sqrtf(-o.d2), kSwFloor);
}

void launch_lik_full(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) lik_full_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

// ---------------------------------------------------------------- evidence
// -log Z = -sum log p(f) + 1/2 f^T a + sum log diag L_B   (objective_LA,
// Laplace.py:25-30, with sum log diag chol(K + W^-1) + 1/2 sum log W
// = sum log diag chol(B)).  Block partials, then one warp per problem.
__global__ void evidence_partial_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  __shared__ double sred[VT / 32];
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const int i = m.y * VT + threadIdx.x;
  float v = 0.0f;
  if (i < P.sh.n) v = -P.logp[i] + 0.5f * P.f[i] * P.a[i] + logf(__ldcg(P.L + (size_t)i * P.ld + i));
  const double s = block_sum_d<VT>(v, sred);
  if (threadIdx.x == 0) P.part[m.y] = s;
}

__global__ void evidence_sum_kernel(const Prob* __restrict__ probs, int nprob) {
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= nprob) return;
  const Prob& P = probs[w];
  if (*P.active == 0) return;
  const int nparts = ceil_div(P.n_pad, VT);
  double s = 0.0;
  for (int k = lane; k < nparts; k += 32) s += P.part[k];
  s = warp_sum_d(s);
  if (lane == 0) *P.value = (float)s;
}

void launch_evidence(const Prob* probs, const int2* vmap, int nblocks, int nprob, cudaStream_t st) {
  if (nblocks <= 0) return;
  evidence_partial_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
  evidence_sum_kernel<<<ceil_div(nprob, 8), 256, 0, st>>>(probs, nprob);
}

// ---------------------------------------------------------------- gradient
// s = 1/2 diag(Sigma) d3 with diag(Sigma)_i = rowdot_i / sw_i
// (rowdot_i = sum_j B^-1_ij sw_j K_ji, i.e. Sigma = W^-1/2 B^-1 W^1/2 K),
// rv = a - d1 - s.
__global__ void grad_vec1_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const int i = m.y * VT + threadIdx.x;
  if (i >= P.n_pad) return;
  if (i >= P.sh.n) {
    P.dsig[i] = 0.0f; P.svec[i] = 0.0f; P.rv[i] = 0.0f;
    return;
  }
  const float ds = P.rowdot[i] / P.sw[i];
  const float s = 0.5f * ds * P.d3[i];
  P.dsig[i] = ds;
  P.svec[i] = s;
  P.rv[i] = P.a[i] - P.d1[i] - s;
}

void launch_grad_vec1(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) grad_vec1_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

// tz = sw * zbar (padding zero)
__global__ void scale_tz_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const int i = m.y * VT + threadIdx.x;
  if (i >= P.n_pad) return;
  P.tz[i] = i < P.sh.n ? P.sw[i] * P.zbar[i] : 0.0f;
}

void launch_scale_tz(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) scale_tz_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

// u = (I + K W)^-1 zbar = W^-1/2 B^-1 (W^1/2 zbar) = y2 / sw (no cancellation);
// c = a/2 - d1 - s - W u
__global__ void grad_vec3_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const int i = m.y * VT + threadIdx.x;
  if (i >= P.n_pad) return;
  if (i >= P.sh.n) {
    P.u[i] = 0.0f; P.c[i] = 0.0f;
    return;
  }
  const float ui = P.y2[i] / P.sw[i];
  P.u[i] = ui;
  P.c[i] = 0.5f * P.a[i] - P.d1[i] - P.svec[i] - P.W[i] * ui;
}

void launch_grad_vec3(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) grad_vec3_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

// Likelihood-parameter gradient, per block: slot 0 = sigma_n, slots
// 1 .. J+1 = cutpoints b_0 .. b_J.  Per point:
//   -dlogp/dt - 1/2 Sigma_ii dd2/dt + u_i dd1/dt
__global__ void grad_lik_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  __shared__ double sacc[VT / 32][MAX_LIK_SLOTS];
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const Shape sh = P.sh;
  const int nslots = 1 + (sh.lik == PGB_LIK_GAUSSIAN ? 0 : sh.J + 1);
  const int i = m.y * VT + threadIdx.x;
  float gs = 0.0f, glo = 0.0f, ghi = 0.0f;
  int ylo = -1;
  if (i < sh.n) {
    int yi;
    const float yv = load_y(sh, P.y, i, &yi);
    LikOut o;
    lik_point<true>(sh.lik, P.f[i], yv, yi, theta_sigma(sh, P.theta), theta_cutpoints(sh, P.theta), o);
    const float ds = P.dsig[i], ui = P.u[i];
    gs = -o.lp_s - 0.5f * ds * o.d2_s + ui * o.d1_s;
    if (sh.lik != PGB_LIK_GAUSSIAN) {
      glo = -o.lp_lo - 0.5f * ds * o.d2_lo + ui * o.d1_lo;
      ghi = -o.lp_hi - 0.5f * ds * o.d2_hi + ui * o.d1_hi;
      ylo = o.ylo;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double s = warp_sum_d((double)gs);
  if (lane == 0) sacc[warp][0] = s;
  if (sh.lik != PGB_LIK_GAUSSIAN) {
    // per-class sums within the warp, in lane order (deterministic)
    for (int cls = 0; cls <= sh.J; ++cls) {
      double v = 0.0;
      if (ylo == cls) v += glo;
      if (ylo >= 0 && ylo + 1 == cls) v += ghi;
      v = warp_sum_d(v);
      if (lane == 0) sacc[warp][1 + cls] = v;
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nslots; k += VT) {
    double t = 0.0;
    for (int w = 0; w < VT / 32; ++w) t += sacc[w][k];
    P.lpart[(size_t)m.y * nslots + k] = t;
  }
}

// One block per problem: the theta gradient from the trace partials (nl + 1
// prior slots, one row per lower tile) and the likelihood partials (1 + J+1
// slots, one row per vmap block), each slot reduced by the whole block in a
// fixed order.  Infinite cutpoints get 0.
constexpr int FINAL_THREADS = 256;
__global__ void __launch_bounds__(FINAL_THREADS) grad_final_kernel(const Prob* __restrict__ probs) {
  __shared__ double sred[FINAL_THREADS / 32];
  const Prob& P = probs[blockIdx.x];
  if (*P.active == 0) return;
  const Shape sh = P.sh;
  const int NP = sh.nl + 1;
  const int nslots = 1 + (sh.lik == PGB_LIK_GAUSSIAN ? 0 : sh.J + 1);
  const int ntp = P.nt * (P.nt + 1) / 2;
  const int nlp = ceil_div(P.n_pad, VT);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < NP + nslots; ++k) {
    double s = 0.0;
    if (k < NP) {
      for (int b = threadIdx.x; b < ntp; b += FINAL_THREADS) s += P.tpart[(size_t)b * NP + k];
    } else {
      for (int b = threadIdx.x; b < nlp; b += FINAL_THREADS) s += P.lpart[(size_t)b * nslots + (k - NP)];
    }
    s = warp_sum_d(s);
    if (lane == 0) sred[warp] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < FINAL_THREADS / 32; ++w) t += sred[w];
      if (k >= NP && k - NP >= 1 && !isfinite(P.theta[sh.nl + 2 + (k - NP) - 1])) t = 0.0;
      P.grad[k] = (float)t;
    }
    __syncthreads();
  }
}

void launch_grad_lik_final(const Prob* probs, const int2* vmap, int nblocks, int nprob, cudaStream_t st) {
  if (nblocks <= 0) return;
  grad_lik_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
  grad_final_kernel<<<nprob, FINAL_THREADS, 0, st>>>(probs);
}

// ---------------------------------------------------------------- Variational Bayes
// VBGP (approximators.py:280-339) with the maps of implicit/VB.py:
//   f_VB(w) = (sigma^2 I + K)^-1 (K w + sigma d log p(K w))        (VB.py:4-17)
// iterated by fwd_solver from w = 0 (approximators.py:332-334), and
//   objective_VB = 1/2 sum(K o cov) + 1/2 sigma^2 tr(cov) + 1/2 (K w)^T w
//                  - N log sigma - 1/2 log det cov - N/2 - sum log p(K w)
// with cov = (sigma^2 I + K)^-1 (VB.py:20-40).  With B = I + K / sigma^2
// (the B of this library at W = 1 / sigma^2) and L L^T = B:
//   (sigma^2 I + K)^-1 v = B^-1 v / sigma^2,  log det cov = -2 (N log sigma + sum log L_ii),
// so objective_VB = sum_i [1/2 rowdot_i / sigma + 1/2 (B^-1)_ii + 1/2 f_i w_i
//                          + log L_ii - 1/2 - log p_i]
// where rowdot_i = sum_j (B^-1)_ij K_ij sw_j, sw = 1 / sigma.

// sw = 1 / sigma, W = 1 / sigma^2 on the data points (0 on the padding)
__global__ void vb_setup_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const int i = m.y * VT + threadIdx.x;
  if (i >= P.n_pad) return;
  const float sig = theta_sigma(P.sh, P.theta);
  const bool in = i < P.sh.n;
  P.sw[i] = in ? 1.0f / sig : 0.0f;
  P.W[i] = in ? 1.0f / (sig * sig) : 0.0f;
  P.sw_prev[i] = P.sw[i];
}

void launch_vb_setup(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) vb_setup_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

// After the factorisation of B: the resident factor serves every step.
__global__ void vb_mark_kernel(const Prob* __restrict__ probs, int nprob) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nprob) return;
  const Prob& P = probs[p];
  if (*P.active == 0) return;
  const int ok = P.status[ST_CODE] == 0 ? 1 : 0;
  P.reuse[0] = ok;
  P.reuse[2] = ok;
}

void launch_vb_mark(const Prob* probs, int nprob, cudaStream_t st) {
  vb_mark_kernel<<<ceil_div(nprob, 128), 128, 0, st>>>(probs, nprob);
}

// t = f + sigma d log p(f) (padding 0): the right-hand side of one step
__global__ void vb_rhs_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const int i = m.y * VT + threadIdx.x;
  if (i >= P.n_pad) return;
  if (i >= P.sh.n) {
    P.d1[i] = 0.0f;
    P.t[i] = 0.0f;
    return;
  }
  const Shape sh = P.sh;
  int yi;
  const float yv = load_y(sh, P.y, i, &yi);
  const float sig = theta_sigma(sh, P.theta);
  LikOut o;
  lik_point<false>(sh.lik, P.f[i], yv, yi, sig, theta_cutpoints(sh, P.theta), o);
  P.d1[i] = o.d1;
  P.t[i] = P.f[i] + sig * o.d1;
}

void launch_vb_rhs(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) vb_rhs_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

// w_new = (B^-1 t) / sigma^2 (x holds B^-1 t); block partial of ||w_new - w||^2;
// da = w_new - w (f follows w by f += K da)
__global__ void vb_update_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  __shared__ double sred[VT / 32];
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;   // uniform per block
  const int i = m.y * VT + threadIdx.x;
  float e = 0.0f;
  if (i < P.sh.n) {
    const float sig = theta_sigma(P.sh, P.theta);
    const float ai = P.a[i];
    const float an = P.x[i] / (sig * sig);
    const float dlt = an - ai;
    e = dlt * dlt;
    P.a[i] = an;
    P.da[i] = dlt;
  } else if (i < P.n_pad) {
    P.da[i] = 0.0f;
  }
  const double s = block_sum_d<VT>(e, sred);
  if (threadIdx.x == 0) P.part[m.y] = s;
}

void launch_vb_update(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) vb_update_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

// After the fixed point, at f = K w: log p, d1 and d2 (kept in dsig), rv =
// w - d1 (zbar = K rv is d objective / d w), and u = t = 0 for the adjoint.
// The objective is then the Laplace-form sum over -log p + f w / 2 + log L_ii
// (launch_evidence): the two trace terms of objective_VB add up to
// tr((K + sigma^2 I) cov) / 2 = N / 2, which cancels its -N / 2.
__global__ void vb_post_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const int i = m.y * VT + threadIdx.x;
  if (i >= P.n_pad) return;
  P.u[i] = 0.0f;
  P.t[i] = 0.0f;
  if (i >= P.sh.n) {
    P.logp[i] = 0.0f; P.d1[i] = 0.0f; P.dsig[i] = 0.0f; P.rv[i] = 0.0f;
    return;
  }
  const Shape sh = P.sh;
  int yi;
  const float yv = load_y(sh, P.y, i, &yi);
  LikOut o;
  lik_point<false>(sh.lik, P.f[i], yv, yi, theta_sigma(sh, P.theta), theta_cutpoints(sh, P.theta), o);
  P.logp[i] = o.logp;
  P.d1[i] = o.d1;
  P.dsig[i] = o.d2;
  P.rv[i] = P.a[i] - o.d1;
}

void launch_vb_post(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) vb_post_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

// ---- the adjoint of fixed_point_layer_bwd (implicit/solvers.py:52-64) for f_VB:
// u <- K (I + sigma D2) A^-1 u + zbar, A = sigma^2 I + K, from u = 0, with
// fwd_solver's stopping rule; reuse[3] counts its steps.
__global__ void vb_adj_reset_kernel(const Prob* __restrict__ probs, int nprob) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nprob) return;
  const Prob& P = probs[p];
  *P.active = *P.enabled != 0 ? 1 : 0;
  P.reuse[3] = 0;
}

void launch_vb_adj_reset(const Prob* probs, int nprob, cudaStream_t st) {
  vb_adj_reset_kernel<<<ceil_div(nprob, 128), 128, 0, st>>>(probs, nprob);
}

// tz = (1 + sigma d2) x / sigma^2, x = B^-1 u (so tz = (I + sigma D2) A^-1 u)
__global__ void vb_adj_scale_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const int i = m.y * VT + threadIdx.x;
  if (i >= P.n_pad) return;
  const float sig = theta_sigma(P.sh, P.theta);
  P.tz[i] = i < P.sh.n ? (1.0f + sig * P.dsig[i]) * P.x[i] / (sig * sig) : 0.0f;
}

void launch_vb_adj_scale(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) vb_adj_scale_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

// u_new = K tz + zbar (y2 = K tz); block partial of ||u_new - u||^2; u = t = u_new
__global__ void vb_adj_update_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  __shared__ double sred[VT / 32];
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;   // uniform per block
  const int i = m.y * VT + threadIdx.x;
  float e = 0.0f;
  if (i < P.sh.n) {
    const float un = P.y2[i] + P.zbar[i];
    const float dlt = un - P.u[i];
    e = dlt * dlt;
    P.u[i] = un;
    P.t[i] = un;
  }
  const double s = block_sum_d<VT>(e, sred);
  if (threadIdx.x == 0) P.part[m.y] = s;
}

void launch_vb_adj_update(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) vb_adj_update_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

__global__ void vb_adj_finalize_kernel(const Prob* __restrict__ probs, int nprob, int* __restrict__ any_active) {
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= nprob) return;
  const Prob& P = probs[w];
  if (*P.active == 0) return;
  const int nparts = ceil_div(P.n_pad, VT);
  double s = 0.0;
  for (int k = lane; k < nparts; k += 32) s += P.part[k];
  s = warp_sum_d(s);
  if (lane == 0) {
    const float err = (float)sqrt(s);
    const int it = P.reuse[3] + 1;
    P.reuse[3] = it;
    if (err != err) atomicCAS(P.status + ST_CODE, 0, PGB_ENAN);
    const bool again = (err > P.tol) && (it < P.maxiter) && (P.status[ST_ABORT] == 0);
    *P.active = again ? 1 : 0;
    if (again) atomicOr(any_active, 1);
  }
}

void launch_vb_adj_finalize(const Prob* probs, int nprob, int* any_active, cudaGraphConditionalHandle cond,
                            int use_cond, cudaStream_t st) {
  vb_adj_finalize_kernel<<<ceil_div(nprob, 8), 256, 0, st>>>(probs, nprob, any_active);
  newton_cond_kernel<<<1, 1, 0, st>>>(any_active, cond, use_cond);
}

// v = A^-1 u = x / sigma^2 (x = B^-1 u), kept in y2; c = w/2 - d1 + sigma v d2,
// the vector of the prior trace sum_ij (A^-1 / 2 + c w^T)_ij dK_ij
__global__ void vb_grad_vec_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const int i = m.y * VT + threadIdx.x;
  if (i >= P.n_pad) return;
  if (i >= P.sh.n) {
    P.y2[i] = 0.0f;
    P.c[i] = 0.0f;
    return;
  }
  const float sig = theta_sigma(P.sh, P.theta);
  const float v = P.x[i] / (sig * sig);
  P.y2[i] = v;
  P.c[i] = 0.5f * P.a[i] - P.d1[i] + sig * v * P.dsig[i];
}

void launch_vb_grad_vec(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) vb_grad_vec_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

// Per point, the likelihood-parameter part of the VB gradient (slots as in
// grad_lik_kernel):
//   sigma : ((B^-1)_ii - 1) / sigma - dlogp/dsigma + v (d1 + sigma dd1/dsigma - 2 sigma w)
//   b     : -dlogp/db + sigma v dd1/db
__global__ void vb_grad_lik_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  __shared__ double sacc[VT / 32][MAX_LIK_SLOTS];
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const Shape sh = P.sh;
  const int nslots = 1 + (sh.lik == PGB_LIK_GAUSSIAN ? 0 : sh.J + 1);
  const int i = m.y * VT + threadIdx.x;
  float gs = 0.0f, glo = 0.0f, ghi = 0.0f;
  int ylo = -1;
  if (i < sh.n) {
    int yi;
    const float yv = load_y(sh, P.y, i, &yi);
    const float sig = theta_sigma(sh, P.theta);
    LikOut o;
    lik_point<true>(sh.lik, P.f[i], yv, yi, sig, theta_cutpoints(sh, P.theta), o);
    const float v = P.y2[i];
    const float bii = __ldcg(P.Binv + (size_t)i * P.ld + i);
    gs = (bii - 1.0f) / sig - o.lp_s + v * (o.d1 + sig * o.d1_s - 2.0f * sig * P.a[i]);
    if (sh.lik != PGB_LIK_GAUSSIAN) {
      glo = -o.lp_lo + sig * v * o.d1_lo;
      ghi = -o.lp_hi + sig * v * o.d1_hi;
      ylo = o.ylo;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double s = warp_sum_d((double)gs);
  if (lane == 0) sacc[warp][0] = s;
  if (sh.lik != PGB_LIK_GAUSSIAN) {
    for (int cls = 0; cls <= sh.J; ++cls) {
      double v = 0.0;
      if (ylo == cls) v += glo;
      if (ylo >= 0 && ylo + 1 == cls) v += ghi;
      v = warp_sum_d(v);
      if (lane == 0) sacc[warp][1 + cls] = v;
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nslots; k += VT) {
    double t = 0.0;
    for (int w = 0; w < VT / 32; ++w) t += sacc[w][k];
    P.lpart[(size_t)m.y * nslots + k] = t;
  }
}

void launch_vb_grad_lik_final(const Prob* probs, const int2* vmap, int nblocks, int nprob, cudaStream_t st) {
  if (nblocks <= 0) return;
  vb_grad_lik_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
  grad_final_kernel<<<nprob, FINAL_THREADS, 0, st>>>(probs);
}

// ---------------------------------------------------------------- predict
// var[m] = s - sum_j rowsq[m, j]   (rowsq from the cross-kernel solve)
__global__ void predict_var_kernel(Shape sh, const float* __restrict__ theta, const float* __restrict__ rowsq,
                                   int nt, int m, float* __restrict__ var) {
  const int i = blockIdx.x * VT + threadIdx.x;
  if (i >= m) return;
  double s = 0.0;
  for (int j = 0; j < nt; ++j) s += rowsq[(size_t)i * nt + j];
  var[i] = __ldg(theta + sh.nl) - (float)s;
}

void launch_predict_var(const Shape& sh, const float* theta, const float* rowsq, int nt, int m, float* var,
                        cudaStream_t st) {
  if (m > 0) predict_var_kernel<<<ceil_div(m, VT), VT, 0, st>>>(sh, theta, rowsq, nt, m, var);
}

// Ordinal predictive distribution (probit_predictive_distributions,
// utilities.py:232-249, through the guarded probit of utilities.py:195-229):
// dist[i, j] = Phi((b_{j+1} - mean_i) / s_i) - Phi((b_j - mean_i) / s_i),
// s_i = sqrt(var_i + sigma^2); an infinite cutpoint gives Phi = 0 or 1.
__global__ void predictive_dist_kernel(Shape sh, const float* __restrict__ theta, const float* __restrict__ mean,
                                       const float* __restrict__ var, int m, float* __restrict__ dist) {
  const int i = blockIdx.x * VT + threadIdx.x;
  if (i >= m) return;
  const float sig = theta_sigma(sh, theta);
  const float* b = theta_cutpoints(sh, theta);
  const float mu = mean[i];
  const float sd = sqrtf(var[i] + sig * sig);
  float lo = 0.0f;   // b_0 = -inf
  for (int j = 0; j < sh.J; ++j) {
    const float bh = __ldg(b + j + 1);
    const float hi = isinf(bh) ? (bh > 0.0f ? 1.0f : 0.0f) : ndtr_ref((bh - mu) / sd);
    dist[(size_t)i * sh.J + j] = hi - lo;
    lo = hi;
  }
}

void launch_predictive_dist(const Shape& sh, const float* theta, const float* mean, const float* var, int m,
                            float* dist, cudaStream_t st) {
  if (m > 0) predictive_dist_kernel<<<ceil_div(m, VT), VT, 0, st>>>(sh, theta, mean, var, m, dist);
}

// sw = sqrt(W) for a caller-supplied precision (padding 0)
__global__ void sqrt_w_kernel(int n, int n_pad, const float* __restrict__ W, float* __restrict__ sw) {
  const int i = blockIdx.x * VT + threadIdx.x;
  if (i >= n_pad) return;
  sw[i] = i < n ? sqrtf(W[i]) : 0.0f;
}

void launch_sqrt_w(int n, int n_pad, const float* W, float* sw, cudaStream_t st) {
  if (n_pad > 0) sqrt_w_kernel<<<ceil_div(n_pad, VT), VT, 0, st>>>(n, n_pad, W, sw);
}

// ---------------------------------------------------------------- factor reuse
// Per active problem: reuse[1] |= any(sw != sw_prev) (bitwise; NaN always
// differs); sw_prev <- sw.  Then per problem: reuse[2] = valid && !differs,
// differs <- 0.  A Newton loop at its float32 floor (ST_STALL) skips the
// comparison and keeps the resident factor of sw_prev: its steps are then
// Newton steps with a Jacobian a few rounding errors old.
__global__ void reuse_check_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;   // uniform per block
  if (P.status[ST_STALL] >= kStallSteps) return;
  const int i = m.y * VT + threadIdx.x;
  bool diff = false;
  if (i < P.sh.n) {
    const float a = P.sw[i];
    diff = __float_as_uint(a) != __float_as_uint(P.sw_prev[i]) || a != a;
    P.sw_prev[i] = a;
  }
  if (__syncthreads_or(diff) && threadIdx.x == 0) atomicOr(P.reuse + 1, 1);
}

__global__ void reuse_decide_kernel(const Prob* __restrict__ probs, int nprob) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nprob) return;
  const Prob& P = probs[p];
  if (*P.active == 0) return;
  int* f = P.reuse;
  f[2] = (f[0] != 0 && f[1] == 0) ? 1 : 0;
  f[1] = 0;
}

void launch_reuse_check(const Prob* probs, const int2* vmap, int nblocks, int nprob, cudaStream_t st) {
  if (nblocks <= 0) return;
  reuse_check_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
  reuse_decide_kernel<<<ceil_div(nprob, 128), 128, 0, st>>>(probs, nprob);
}

// After a factorisation that computed L: the resident L matches sw_prev.
__global__ void reuse_mark_valid_kernel(const Prob* __restrict__ probs, int nprob) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nprob) return;
  const Prob& P = probs[p];
  if (*P.active == 0) return;
  P.reuse[0] = P.status[ST_CODE] == 0 ? 1 : 0;
}

void launch_reuse_mark_valid(const Prob* probs, int nprob, cudaStream_t st) {
  reuse_mark_valid_kernel<<<ceil_div(nprob, 128), 128, 0, st>>>(probs, nprob);
}

__global__ void mark_z_kernel(const Prob* __restrict__ probs, int nprob) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nprob) return;
  const Prob& P = probs[p];
  if (*P.active == 0 || P.sh.lik != PGB_LIK_GAUSSIAN) return;
  if (P.reuse[2] == 0) *P.zvalid = P.status[ST_CODE] == 0 ? 1 : 0;   // factored (with L^-T) in this step
}

void launch_mark_z(const Prob* probs, int nprob, cudaStream_t st) {
  mark_z_kernel<<<ceil_div(nprob, 128), 128, 0, st>>>(probs, nprob);
}

__global__ void need_factor_kernel(const Prob* __restrict__ probs, int nprob, cudaGraphConditionalHandle cond) {
  bool need = false;
  for (int p = threadIdx.x; p < nprob; p += blockDim.x) {
    const Prob& P = probs[p];
    if (*P.active != 0 && P.reuse[2] == 0) need = true;
  }
  need = __syncthreads_or(need) != 0;
  if (threadIdx.x == 0) cudaGraphSetConditional(cond, need ? 1u : 0u);
}

void launch_need_factor(const Prob* probs, int nprob, cudaGraphConditionalHandle cond, cudaStream_t st) {
  need_factor_kernel<<<1, 256, 0, st>>>(probs, nprob, cond);
}

}  // namespace pgb
