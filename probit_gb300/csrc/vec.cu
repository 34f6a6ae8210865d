// Per-point kernels of the Newton step, the evidence and the gradient, and
// their deterministic two-phase reductions (block partials in double, then
// one block summing them in a fixed order).
#include "kernels.cuh"
#include "lik.cuh"

namespace pgb {

constexpr int VT = 256;   // threads per block for vector kernels

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
  lik_eval_kernel<<<ceil_div(n, VT), VT, 0, st>>>(sh, theta, f, y, n, logp, d1, d2, d3);
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
// y = r / W^1/2.  Padding entries (i >= n, up to n_pad) are zeroed.
constexpr float kSwFloor = 1e-18f;

__global__ void newton_lik_kernel(Shape sh, const float* __restrict__ theta, const float* __restrict__ f,
                                  const void* __restrict__ y, const float* __restrict__ a, int n_pad,
                                  float* __restrict__ d1, float* __restrict__ W, float* __restrict__ sw,
                                  float* __restrict__ r, float* __restrict__ rhs) {
  const int i = blockIdx.x * VT + threadIdx.x;
  if (i >= n_pad) return;
  if (i >= sh.n) {
    d1[i] = 0.0f; W[i] = 0.0f; sw[i] = 0.0f; r[i] = 0.0f; rhs[i] = 0.0f;
    return;
  }
  int yi;
  const float yv = load_y(sh, y, i, &yi);
  LikOut o;
  lik_point<false>(sh.lik, f[i], yv, yi, theta_sigma(sh, theta), theta_cutpoints(sh, theta), o);
  const float w = -o.d2;
  const float s = fmaxf(sqrtf(w), kSwFloor);
  const float ri = o.d1 - a[i];
  d1[i] = o.d1;
  W[i] = w;
  sw[i] = s;
  r[i] = ri;
  rhs[i] = ri / s;
}

void launch_newton_lik(const Shape& sh, const float* theta, const float* f, const void* y, const float* a,
                       int n_pad, float* d1, float* W, float* sw, float* r, float* rhs, cudaStream_t st) {
  newton_lik_kernel<<<ceil_div(n_pad, VT), VT, 0, st>>>(sh, theta, f, y, a, n_pad, d1, W, sw, r, rhs);
}

// a_new = a + sw * x; block partial of ||a_new - a||^2 (as jaxopt measures
// it, on the rounded new iterate); a <- a_new
__global__ void newton_update_kernel(int n, const float* __restrict__ sw, const float* __restrict__ x,
                                     float* __restrict__ a, double* __restrict__ part) {
  __shared__ double sred[VT / 32];
  const int i = blockIdx.x * VT + threadIdx.x;
  float e = 0.0f;
  if (i < n) {
    const float ai = a[i];
    const float an = ai + sw[i] * x[i];
    const float dlt = an - ai;
    e = dlt * dlt;
    a[i] = an;
  }
  const double s = block_sum_d<VT>(e, sred);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// One block: err = sqrt(sum part); iterations += 1; decide whether to loop.
// jaxopt FixedPointIteration semantics (solvers.py:7-15): keep going while
// err > tol and fewer than maxiter updates were made; a NaN error stops.
__global__ void newton_finalize_kernel(const double* __restrict__ part, int nparts, float tol, int maxiter,
                                       int* __restrict__ status, float* __restrict__ err_out,
                                       cudaGraphConditionalHandle cond, int use_cond) {
  double s = 0.0;
  for (int k = threadIdx.x; k < nparts; k += 32) s += part[k];
  s = warp_sum_d(s);
  if (threadIdx.x == 0) {
    const float err = (float)sqrt(s);
    const int it = status[ST_ITERS] + 1;
    status[ST_ITERS] = it;
    *err_out = err;
    const bool conv = !(err > tol);
    if (conv) status[ST_CONVERGED] = 1;
    if (err != err) atomicCAS(status + ST_CODE, 0, PGB_ENAN);
    const bool again = (err > tol) && (it < maxiter) && (status[ST_ABORT] == 0);
    status[ST_SPARE0] = again ? 1 : 0;   // read by the host-driven (eager) loop
    if (use_cond) cudaGraphSetConditional(cond, again ? 1u : 0u);
  }
}

void launch_newton_update(int n, const float* sw, const float* x, float* a, double* part, cudaStream_t st) {
  newton_update_kernel<<<ceil_div(n, VT), VT, 0, st>>>(n, sw, x, a, part);
}

void launch_newton_finalize(const double* part, int nparts, float tol, int maxiter, int* status, float* err_out,
                            cudaGraphConditionalHandle cond, int use_cond, cudaStream_t st) {
  newton_finalize_kernel<<<1, 32, 0, st>>>(part, nparts, tol, maxiter, status, err_out, cond, use_cond);
}

// ---------------------------------------------------------------- precision
// Full per-point terms at the final f: logp, d1, d2, d3, W, sw (padding 0).
__global__ void lik_full_kernel(Shape sh, const float* __restrict__ theta, const float* __restrict__ f,
                                const void* __restrict__ y, int n_pad, float* __restrict__ logp,
                                float* __restrict__ d1, float* __restrict__ d3, float* __restrict__ W,
                                float* __restrict__ sw) {
  const int i = blockIdx.x * VT + threadIdx.x;
  if (i >= n_pad) return;
  if (i >= sh.n) {
    logp[i] = 0.0f; d1[i] = 0.0f; d3[i] = 0.0f; W[i] = 0.0f; sw[i] = 0.0f;
    return;
  }
  int yi;
  const float yv = load_y(sh, y, i, &yi);
  LikOut o;
  lik_point<false>(sh.lik, f[i], yv, yi, theta_sigma(sh, theta), theta_cutpoints(sh, theta), o);
  logp[i] = o.logp;
  d1[i] = o.d1;
  d3[i] = o.d3;
  W[i] = -o.d2;
  sw[i] = fmaxf(sqrtf(-o.d2), kSwFloor);
}

void launch_lik_full(const Shape& sh, const float* theta, const float* f, const void* y, int n_pad, float* logp,
                     float* d1, float* d3, float* W, float* sw, cudaStream_t st) {
  lik_full_kernel<<<ceil_div(n_pad, VT), VT, 0, st>>>(sh, theta, f, y, n_pad, logp, d1, d3, W, sw);
}

// ---------------------------------------------------------------- evidence
// -log Z = -sum log p(f) + 1/2 f^T a + sum log diag L_B   (objective_LA,
// Laplace.py:25-30, with sum log diag chol(K + W^-1) + 1/2 sum log W
// = sum log diag chol(B)).  Block partials, then evidence_finalize.
__global__ void evidence_partial_kernel(int n, const float* __restrict__ logp, const float* __restrict__ f,
                                        const float* __restrict__ a, const float* __restrict__ L, long long ld,
                                        double* __restrict__ part) {
  __shared__ double sred[VT / 32];
  const int i = blockIdx.x * VT + threadIdx.x;
  float v = 0.0f;
  if (i < n) v = -logp[i] + 0.5f * f[i] * a[i] + logf(__ldcg(L + (size_t)i * ld + i));
  const double s = block_sum_d<VT>(v, sred);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void sum_parts_kernel(const double* __restrict__ part, int nparts, float* __restrict__ out) {
  double s = 0.0;
  for (int k = threadIdx.x; k < nparts; k += 32) s += part[k];
  s = warp_sum_d(s);
  if (threadIdx.x == 0) *out = (float)s;
}

void launch_evidence(int n, const float* logp, const float* f, const float* a, const float* L, long long ld,
                     double* part, float* value, cudaStream_t st) {
  const int nb = ceil_div(n, VT);
  evidence_partial_kernel<<<nb, VT, 0, st>>>(n, logp, f, a, L, ld, part);
  sum_parts_kernel<<<1, 32, 0, st>>>(part, nb, value);
}

// ---------------------------------------------------------------- gradient
// s = 1/2 diag(Sigma) d3 with diag(Sigma)_i = rowdot_i / sw_i
// (rowdot_i = sum_j B^-1_ij sw_j K_ji, i.e. Sigma = W^-1/2 B^-1 W^1/2 K),
// r = a - d1 - s.
__global__ void grad_vec1_kernel(int n, int n_pad, const float* __restrict__ rowdot, const float* __restrict__ sw,
                                 const float* __restrict__ d3, const float* __restrict__ a,
                                 const float* __restrict__ d1, float* __restrict__ dsig, float* __restrict__ svec,
                                 float* __restrict__ r) {
  const int i = blockIdx.x * VT + threadIdx.x;
  if (i >= n_pad) return;
  if (i >= n) {
    dsig[i] = 0.0f; svec[i] = 0.0f; r[i] = 0.0f;
    return;
  }
  const float ds = rowdot[i] / sw[i];
  const float s = 0.5f * ds * d3[i];
  dsig[i] = ds;
  svec[i] = s;
  r[i] = a[i] - d1[i] - s;
}

void launch_grad_vec1(int n, int n_pad, const float* rowdot, const float* sw, const float* d3, const float* a,
                      const float* d1, float* dsig, float* svec, float* r, cudaStream_t st) {
  grad_vec1_kernel<<<ceil_div(n_pad, VT), VT, 0, st>>>(n, n_pad, rowdot, sw, d3, a, d1, dsig, svec, r);
}

// out = sw * in (padding zero)
__global__ void scale_vec_kernel(int n, int n_pad, const float* __restrict__ sw, const float* __restrict__ in,
                                 float* __restrict__ out) {
  const int i = blockIdx.x * VT + threadIdx.x;
  if (i >= n_pad) return;
  out[i] = i < n ? sw[i] * in[i] : 0.0f;
}

void launch_scale_vec(int n, int n_pad, const float* sw, const float* in, float* out, cudaStream_t st) {
  scale_vec_kernel<<<ceil_div(n_pad, VT), VT, 0, st>>>(n, n_pad, sw, in, out);
}

// u = (I + K W)^-1 zbar = W^-1/2 B^-1 (W^1/2 zbar) = y1 / sw (no cancellation);
// c = a/2 - d1 - s - W u
__global__ void grad_vec3_kernel(int n, int n_pad, const float* __restrict__ y1, const float* __restrict__ sw,
                                 const float* __restrict__ a, const float* __restrict__ d1,
                                 const float* __restrict__ svec, const float* __restrict__ W, float* __restrict__ u,
                                 float* __restrict__ c) {
  const int i = blockIdx.x * VT + threadIdx.x;
  if (i >= n_pad) return;
  if (i >= n) {
    u[i] = 0.0f; c[i] = 0.0f;
    return;
  }
  const float ui = y1[i] / sw[i];
  u[i] = ui;
  c[i] = 0.5f * a[i] - d1[i] - svec[i] - W[i] * ui;
}

void launch_grad_vec3(int n, int n_pad, const float* y1, const float* sw, const float* a, const float* d1,
                      const float* svec, const float* W, float* u, float* c, cudaStream_t st) {
  grad_vec3_kernel<<<ceil_div(n_pad, VT), VT, 0, st>>>(n, n_pad, y1, sw, a, d1, svec, W, u, c);
}

// Likelihood-parameter gradient, per block: slot 0 = sigma_n, slots
// 1 .. J+1 = cutpoints b_0 .. b_J.  Per point:
//   -dlogp/dt - 1/2 Sigma_ii dd2/dt + u_i dd1/dt
__global__ void grad_lik_kernel(Shape sh, const float* __restrict__ theta, const float* __restrict__ f,
                                const void* __restrict__ y, const float* __restrict__ dsig,
                                const float* __restrict__ u, double* __restrict__ part) {
  const int nslots = 1 + (sh.lik == PGB_LIK_GAUSSIAN ? 0 : sh.J + 1);
  extern __shared__ float sacc[];   // [VT/32 warps][nslots] as double below
  double* sw_acc = reinterpret_cast<double*>(sacc);
  for (int e = threadIdx.x; e < nslots * (VT / 32); e += VT) sw_acc[e] = 0.0;
  __syncthreads();
  const int i = blockIdx.x * VT + threadIdx.x;
  float gs = 0.0f, glo = 0.0f, ghi = 0.0f;
  int ylo = -1;
  if (i < sh.n) {
    int yi;
    const float yv = load_y(sh, y, i, &yi);
    LikOut o;
    lik_point<true>(sh.lik, f[i], yv, yi, theta_sigma(sh, theta), theta_cutpoints(sh, theta), o);
    const float ds = dsig[i], ui = u[i];
    gs = -o.lp_s - 0.5f * ds * o.d2_s + ui * o.d1_s;
    if (sh.lik != PGB_LIK_GAUSSIAN) {
      glo = -o.lp_lo - 0.5f * ds * o.d2_lo + ui * o.d1_lo;
      ghi = -o.lp_hi - 0.5f * ds * o.d2_hi + ui * o.d1_hi;
      ylo = o.ylo;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // sigma slot: warp sum
  const double s = warp_sum_d((double)gs);
  if (lane == 0) sw_acc[warp * nslots + 0] = s;
  if (sh.lik != PGB_LIK_GAUSSIAN) {
    // per-class sums within the warp, in lane order (deterministic)
    for (int cls = 0; cls <= sh.J; ++cls) {
      double v = 0.0;
      if (ylo == cls) v += glo;
      if (ylo >= 0 && ylo + 1 == cls) v += ghi;
      v = warp_sum_d(v);
      if (lane == 0) sw_acc[warp * nslots + 1 + cls] = v;
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nslots; k += VT) {
    double t = 0.0;
    for (int w = 0; w < VT / 32; ++w) t += sw_acc[w * nslots + k];
    part[(size_t)blockIdx.x * nslots + k] = t;
  }
}

// Assemble the theta gradient from the trace partials (nl+1 prior slots)
// and the likelihood partials (1 + J+1 slots).  Infinite cutpoints get 0.
__global__ void grad_final_kernel(Shape sh, const float* __restrict__ theta, const double* __restrict__ tpart,
                                  int ntp, const double* __restrict__ lpart, int nlp, float* __restrict__ grad) {
  const int P = sh.nl + 1;
  const int nslots = 1 + (sh.lik == PGB_LIK_GAUSSIAN ? 0 : sh.J + 1);
  const int k = threadIdx.x;
  if (k < P) {
    double s = 0.0;
    for (int b = 0; b < ntp; ++b) s += tpart[(size_t)b * P + k];
    grad[k] = (float)s;
  } else if (k < P + nslots) {
    const int slot = k - P;
    double s = 0.0;
    for (int b = 0; b < nlp; ++b) s += lpart[(size_t)b * nslots + slot];
    if (slot >= 1) {
      const float bv = theta[sh.nl + 2 + slot - 1];
      if (!isfinite(bv)) s = 0.0;
    }
    grad[P + slot] = (float)s;
  }
}

void launch_grad_lik_final(const Shape& sh, const float* theta, const float* f, const void* y, const float* dsig,
                           const float* u, const double* tpart, int ntp, double* lpart, float* grad,
                           cudaStream_t st) {
  const int nslots = 1 + (sh.lik == PGB_LIK_GAUSSIAN ? 0 : sh.J + 1);
  const int nb = ceil_div(sh.n, VT);
  grad_lik_kernel<<<nb, VT, sizeof(double) * nslots * (VT / 32), st>>>(sh, theta, f, y, dsig, u, lpart);
  grad_final_kernel<<<1, 64, 0, st>>>(sh, theta, tpart, ntp, lpart, nb, grad);
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
  predict_var_kernel<<<ceil_div(m, VT), VT, 0, st>>>(sh, theta, rowsq, nt, m, var);
}

// sw = sqrt(W) for a caller-supplied precision (padding 0)
__global__ void sqrt_w_kernel(int n, int n_pad, const float* __restrict__ W, float* __restrict__ sw) {
  const int i = blockIdx.x * VT + threadIdx.x;
  if (i >= n_pad) return;
  sw[i] = i < n ? sqrtf(W[i]) : 0.0f;
}

void launch_sqrt_w(int n, int n_pad, const float* W, float* sw, cudaStream_t st) {
  sqrt_w_kernel<<<ceil_div(n_pad, VT), VT, 0, st>>>(n, n_pad, W, sw);
}

// ---------------------------------------------------------------- factor reuse
// flags[1] |= any(sw != sw_prev) (bitwise; NaN always differs); sw_prev <- sw.
__global__ void reuse_check_kernel(int n, const float* __restrict__ sw, float* __restrict__ sw_prev,
                                   int* __restrict__ flags) {
  const int i = blockIdx.x * VT + threadIdx.x;
  bool diff = false;
  if (i < n) {
    const float a = sw[i];
    diff = __float_as_uint(a) != __float_as_uint(sw_prev[i]) || a != a;
    sw_prev[i] = a;
  }
  if (__syncthreads_or(diff) && threadIdx.x == 0) atomicOr(flags + 1, 1);
}

// flags[2] = valid && !differs; differs <- 0
__global__ void reuse_decide_kernel(int* flags) {
  flags[2] = (flags[0] != 0 && flags[1] == 0) ? 1 : 0;
  flags[1] = 0;
}

void launch_reuse_check(int n, const float* sw, float* sw_prev, int* flags, cudaStream_t st) {
  reuse_check_kernel<<<ceil_div(n, VT), VT, 0, st>>>(n, sw, sw_prev, flags);
  reuse_decide_kernel<<<1, 1, 0, st>>>(flags);
}

// After a factorisation that computed L: the resident L matches sw_prev.
__global__ void reuse_mark_valid_kernel(int* flags, const int* status) {
  flags[0] = status[ST_CODE] == 0 ? 1 : 0;
}

void launch_reuse_mark_valid(int* flags, const int* status, cudaStream_t st) {
  reuse_mark_valid_kernel<<<1, 1, 0, st>>>(flags, status);
}

}  // namespace pgb
