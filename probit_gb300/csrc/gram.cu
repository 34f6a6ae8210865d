// Gram-matrix kernels.  K is never stored on the hot path: every consumer
// recomputes its entries from the prepared features (a few FMAs and one exp
// per entry), which costs less than streaming an N x N matrix from HBM.
//
// Kernel algebra restated from mlkernels as used by the reference
// (Laplace.py:7,21,24; approximators.py:172-174,192-194,272).
#include "kernels.cuh"

namespace pgb {

// ---------------------------------------------------------------- features
// eq / matern12: x_d / l_d (mlkernels' stretch divides the inputs);
// eq_periodic: the raw inputs (the lengthscale is applied after the sine).
__global__ void prep_features_kernel(Shape sh, const float* __restrict__ X, const float* __restrict__ theta,
                                     float* __restrict__ Xf, int n, int n_pad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  for (int d = 0; d < sh.Dp; ++d) {
    float v = 0.0f;
    if (i < n && d < sh.D) {
      v = X[(size_t)i * sh.D + d];
      if (sh.kind != PGB_KERNEL_EQ_PERIODIC) v = v / __ldg(theta + (sh.nl == 1 ? 0 : d));
    }
    Xf[(size_t)i * sh.Dp + d] = v;
  }
}

void launch_prep_features(const Shape& sh, const float* X, const float* theta, float* Xf, int n, int n_pad,
                          cudaStream_t st) {
  prep_features_kernel<<<ceil_div(n_pad, 256), 256, 0, st>>>(sh, X, theta, Xf, n, n_pad);
}

// Summed scaled squared distance with the feature loop unrolled to DM.
template <int DM>
__device__ __forceinline__ float d2_t(const KernelParams& kp, const float* xi, const float* xj) {
  float d2 = 0.0f;
#pragma unroll
  for (int d = 0; d < DM; ++d) {
    if (d < kp.D) {
      if (kp.kind == PGB_KERNEL_EQ_PERIODIC) {
        const float v = (2.0f * sinpif((xi[d] - xj[d]) * kp.inv_p)) / kp.l[kp.nl == 1 ? 0 : d];
        d2 += v * v;
      } else {
        const float v = xi[d] - xj[d];
        d2 += v * v;
      }
    }
  }
  return d2;
}

// ---------------------------------------------------------------- full Gram
template <int DM>
__global__ void gram_full_kernel(Shape sh, const float* __restrict__ theta, const float* __restrict__ X1, int n1,
                                 const float* __restrict__ X2, int n2, float* __restrict__ K, long long ldk) {
  const KernelParams kp = make_kp(sh, theta);
  const int j = blockIdx.x * 32 + (threadIdx.x & 31);
  const int i0 = blockIdx.y * 32 + (threadIdx.x >> 5);
  if (j >= n2) return;
  float xj[DM];
#pragma unroll
  for (int d = 0; d < DM; ++d) xj[d] = d < sh.Dp ? X2[(size_t)j * sh.Dp + d] : 0.0f;
  for (int i = i0; i < min(n1, blockIdx.y * 32 + 32); i += 8) {
    float xi[DM];
#pragma unroll
    for (int d = 0; d < DM; ++d) xi[d] = d < sh.Dp ? X1[(size_t)i * sh.Dp + d] : 0.0f;
    K[(size_t)i * ldk + j] = kernel_from_d2(kp, d2_t<DM>(kp, xi, xj));
  }
}

void launch_gram_full(const Shape& sh, const float* theta, const float* X1f, int n1, const float* X2f, int n2,
                      float* K, long long ldk, cudaStream_t st) {
  dim3 grid(ceil_div(n2, 32), ceil_div(n1, 32));
  if (sh.Dp <= 4)
    gram_full_kernel<4><<<grid, 256, 0, st>>>(sh, theta, X1f, n1, X2f, n2, K, ldk);
  else if (sh.Dp <= 8)
    gram_full_kernel<8><<<grid, 256, 0, st>>>(sh, theta, X1f, n1, X2f, n2, K, ldk);
  else
    gram_full_kernel<16><<<grid, 256, 0, st>>>(sh, theta, X1f, n1, X2f, n2, K, ldk);
}

// ---------------------------------------------------------------- Gram matvec
// y[r] = row_scale[r] * sum_c K(xr_r, xc_c) * (M ? M[r, c] : 1) * v[c]
// One block owns MV_ROWS rows and sweeps all columns; the per-row sums are
// reduced in a fixed order, so results are bitwise reproducible.  The kernel
// family is a template parameter and every per-entry quantity lives in
// registers or shared memory.
constexpr int MV_THREADS = 256;
// rows per block: 32 for D <= 4, 16 for D <= 8, 8 for D <= 16 (constant
// unrolled work per column)
template <int DM>
constexpr int mv_rows() { return 128 / DM; }

template <int KIND, int DM>
__device__ __forceinline__ float kval(const float* xi, const float* xj, int D, float s, float inv_p,
                                      const float* sl) {
  float d2 = 0.0f;
#pragma unroll
  for (int d = 0; d < DM; ++d) {
    if (d < D) {
      float q;
      if (KIND == PGB_KERNEL_EQ_PERIODIC) {
        q = (2.0f * sinpif((xi[d] - xj[d]) * inv_p)) / sl[d];
      } else {
        q = xi[d] - xj[d];
      }
      d2 += q * q;
    }
  }
  if (KIND == PGB_KERNEL_MATERN12) return s * expf(-sqrtf(d2));
  return s * expf(-0.5f * d2);
}

template <int KIND, int DM, bool HAS_M>
__global__ void __launch_bounds__(MV_THREADS) gram_matvec_kernel(
    Shape sh, const float* __restrict__ theta, const float* __restrict__ Xr, int nr, const float* __restrict__ Xc,
    int nc, const float* __restrict__ M, long long ldm, const float* __restrict__ v,
    const float* __restrict__ row_scale, float* __restrict__ y) {
  constexpr int MV_ROWS = mv_rows<DM>();
  __shared__ float sx[MV_ROWS][DM];
  __shared__ float sred[MV_THREADS / 32][MV_ROWS];
  __shared__ float sl[MAX_D];
  const int D = sh.D, Dp = sh.Dp;
  const float sv = __ldg(theta + sh.nl);
  const float inv_p = sh.inv_p;
  if (threadIdx.x < MAX_D) sl[threadIdx.x] = threadIdx.x < D ? __ldg(theta + (sh.nl == 1 ? 0 : threadIdx.x)) : 1.0f;
  const int r0 = blockIdx.x * MV_ROWS;
  for (int e = threadIdx.x; e < MV_ROWS * DM; e += MV_THREADS) {
    const int r = e / DM, d = e % DM;
    sx[r][d] = (r0 + r < nr && d < Dp) ? Xr[(size_t)(r0 + r) * Dp + d] : 0.0f;
  }
  __syncthreads();
  float acc[MV_ROWS];
#pragma unroll
  for (int r = 0; r < MV_ROWS; ++r) acc[r] = 0.0f;
  const int rmax = min(MV_ROWS, nr - r0);
  for (int c = threadIdx.x; c < nc; c += MV_THREADS) {
    float xc[DM];
#pragma unroll
    for (int d = 0; d < DM; ++d) xc[d] = d < Dp ? __ldg(Xc + (size_t)c * Dp + d) : 0.0f;
    const float vc = __ldg(v + c);
    if (rmax == MV_ROWS) {
#pragma unroll
      for (int r = 0; r < MV_ROWS; ++r) {
        float k = kval<KIND, DM>(sx[r], xc, D, sv, inv_p, sl);
        if (HAS_M) k *= __ldg(M + (size_t)(r0 + r) * ldm + c);
        acc[r] = fmaf(k, vc, acc[r]);
      }
    } else {
#pragma unroll
      for (int r = 0; r < MV_ROWS; ++r) {
        if (r < rmax) {
          float k = kval<KIND, DM>(sx[r], xc, D, sv, inv_p, sl);
          if (HAS_M) k *= __ldg(M + (size_t)(r0 + r) * ldm + c);
          acc[r] = fmaf(k, vc, acc[r]);
        }
      }
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < MV_ROWS; ++r) {
    const float t = warp_sum(acc[r]);
    if (lane == 0) sred[warp][r] = t;
  }
  __syncthreads();
  if (threadIdx.x < MV_ROWS && threadIdx.x < rmax) {
    float t = 0.0f;
#pragma unroll
    for (int w = 0; w < MV_THREADS / 32; ++w) t += sred[w][threadIdx.x];
    if (row_scale) t *= row_scale[r0 + threadIdx.x];
    y[r0 + threadIdx.x] = t;
  }
}

template <int KIND, int DM>
static void mv_dispatch_m(const Shape& sh, const float* theta, const float* Xr, int nr, const float* Xc, int nc,
                          const float* M, long long ldm, const float* v, const float* row_scale, float* y,
                          cudaStream_t st) {
  const int grid = ceil_div(nr, mv_rows<DM>());
  if (M)
    gram_matvec_kernel<KIND, DM, true><<<grid, MV_THREADS, 0, st>>>(sh, theta, Xr, nr, Xc, nc, M, ldm, v, row_scale, y);
  else
    gram_matvec_kernel<KIND, DM, false><<<grid, MV_THREADS, 0, st>>>(sh, theta, Xr, nr, Xc, nc, M, ldm, v, row_scale, y);
}

template <int KIND>
static void mv_dispatch_d(const Shape& sh, const float* theta, const float* Xr, int nr, const float* Xc, int nc,
                          const float* M, long long ldm, const float* v, const float* row_scale, float* y,
                          cudaStream_t st) {
  if (sh.Dp <= 4)
    mv_dispatch_m<KIND, 4>(sh, theta, Xr, nr, Xc, nc, M, ldm, v, row_scale, y, st);
  else if (sh.Dp <= 8)
    mv_dispatch_m<KIND, 8>(sh, theta, Xr, nr, Xc, nc, M, ldm, v, row_scale, y, st);
  else
    mv_dispatch_m<KIND, 16>(sh, theta, Xr, nr, Xc, nc, M, ldm, v, row_scale, y, st);
}

void launch_gram_matvec(const Shape& sh, const float* theta, const float* Xr, int nr, const float* Xc, int nc,
                        const float* M, long long ldm, const float* v, const float* row_scale, float* y,
                        cudaStream_t st) {
  if (sh.kind == PGB_KERNEL_MATERN12)
    mv_dispatch_d<PGB_KERNEL_MATERN12>(sh, theta, Xr, nr, Xc, nc, M, ldm, v, row_scale, y, st);
  else if (sh.kind == PGB_KERNEL_EQ_PERIODIC)
    mv_dispatch_d<PGB_KERNEL_EQ_PERIODIC>(sh, theta, Xr, nr, Xc, nc, M, ldm, v, row_scale, y, st);
  else
    mv_dispatch_d<PGB_KERNEL_EQ>(sh, theta, Xr, nr, Xc, nc, M, ldm, v, row_scale, y, st);
}

// ---------------------------------------------------------------- dense matvec
// y[r] = row_scale[r] * sum_c A[r, c] v[c]   (A row-major, lda)
__global__ void __launch_bounds__(256) dense_matvec_kernel(const float* __restrict__ A, long long lda, int nr, int nc,
                                                           const float* __restrict__ v, const float* __restrict__ row_scale,
                                                           float* __restrict__ y) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * 8 + warp;
  if (r >= nr) return;
  const float* a = A + (size_t)r * lda;
  float s = 0.0f;
  for (int c = lane * 4; c < nc; c += 128) {
    if (c + 3 < nc) {
      const float4 x = __ldg(reinterpret_cast<const float4*>(a + c));
      const float4 w = __ldg(reinterpret_cast<const float4*>(v + c));
      s = fmaf(x.x, w.x, s);
      s = fmaf(x.y, w.y, s);
      s = fmaf(x.z, w.z, s);
      s = fmaf(x.w, w.w, s);
    } else {
      for (int e = c; e < nc; ++e) s = fmaf(a[e], v[e], s);
    }
  }
  s = warp_sum(s);
  if (lane == 0) y[r] = row_scale ? s * row_scale[r] : s;
}

void launch_dense_matvec(const float* A, long long lda, int nr, int nc, const float* v, const float* row_scale,
                         float* y, cudaStream_t st) {
  dense_matvec_kernel<<<ceil_div(nr, 8), 256, 0, st>>>(A, lda, nr, nc, v, row_scale, y);
}

// ---------------------------------------------------------------- gradient trace
// Over the lower 128x128 tiles (I >= J) of B^-1 (stored full, row-major, ld):
//   g_k += sum_{i,j} M_ij dK_k(x_i, x_j),  M = 1/2 R + c a^T,  R = sw B^-1 sw
// folded to the lower triangle: off-diagonal pairs carry R_ij + c_i a_j +
// c_j a_i, the diagonal 1/2 R_ii + c_i a_i (only dK/ds is nonzero there).
// dK/dl_d = K q_d / l_d (Matern12: times 1/r, 0 at r = 0), dK/ds = K / s.
// Each block writes its partial sums (double) to part[block * P + k].
template <int DM>
__global__ void __launch_bounds__(256) grad_trace_kernel(Shape sh, const float* __restrict__ theta,
                                                         const float* __restrict__ Xf, const float* __restrict__ Binv,
                                                         long long ld, const float* __restrict__ sw,
                                                         const float* __restrict__ cvec, const float* __restrict__ avec,
                                                         const int2* __restrict__ tiles, double* __restrict__ part) {
  const KernelParams kp = make_kp(sh, theta);
  const int P = sh.nl + 1;
  const int2 tl = tiles[blockIdx.x];
  const int I = tl.x, J = tl.y;
  const int n = sh.n;
  __shared__ float sxc[T][DM];
  __shared__ float ssw[T], sc[T], sa[T];
  __shared__ double sred[8][MAX_D + 1];
  for (int e = threadIdx.x; e < T * DM; e += 256) {
    const int c = e / DM, d = e % DM;
    const int gc = J * T + c;
    sxc[c][d] = (gc < n && d < sh.Dp) ? Xf[(size_t)gc * sh.Dp + d] : 0.0f;
  }
  for (int c = threadIdx.x; c < T; c += 256) {
    const int gc = J * T + c;
    ssw[c] = gc < n ? sw[gc] : 0.0f;
    sc[c] = gc < n ? cvec[gc] : 0.0f;
    sa[c] = gc < n ? avec[gc] : 0.0f;
  }
  __syncthreads();
  float acc[DM];
  float acc_s = 0.0f;
#pragma unroll
  for (int k = 0; k < DM; ++k) acc[k] = 0.0f;
  const int c = threadIdx.x & (T - 1);
  const int rh = threadIdx.x >> 7;  // 0 or 1
  const int gc = J * T + c;
  for (int r = rh; r < T; r += 2) {
    const int gr = I * T + r;
    if (gr >= n || gc >= n || gc > gr) continue;
    float xr[DM];
#pragma unroll
    for (int d = 0; d < DM; ++d) xr[d] = d < sh.Dp ? __ldg(Xf + (size_t)gr * sh.Dp + d) : 0.0f;
    const float swr = __ldg(sw + gr), cr = __ldg(cvec + gr), ar = __ldg(avec + gr);
    const float bij = __ldcg(Binv + (size_t)gr * ld + gc);
    float m;
    if (gr == gc)
      m = 0.5f * swr * bij * swr + cr * ar;
    else
      m = swr * bij * ssw[c] + cr * sa[c] + sc[c] * ar;
    // distances
    float q[DM];
    float d2 = 0.0f;
#pragma unroll
    for (int d = 0; d < DM; ++d) {
      q[d] = 0.0f;
      if (d < sh.D) {
        float v;
        if (kp.kind == PGB_KERNEL_EQ_PERIODIC) {
          v = (2.0f * sinpif((xr[d] - sxc[c][d]) * kp.inv_p)) / kp.l[kp.nl == 1 ? 0 : d];
        } else {
          v = xr[d] - sxc[c][d];
        }
        q[d] = v * v;
        d2 += q[d];
      }
    }
    const float K = kernel_from_d2(kp, d2);
    float scale = K * m;
    if (kp.kind == PGB_KERNEL_MATERN12) {
      const float rr = sqrtf(d2);
      scale = rr > 0.0f ? scale / rr : 0.0f;
    }
    if (kp.nl == 1) {
      acc[0] += scale * d2 * kp.inv_l[0];
    } else {
#pragma unroll
      for (int d = 0; d < DM; ++d)
        if (d < sh.D) acc[d] += scale * q[d] * kp.inv_l[d];
    }
    acc_s += K * m / kp.s;
  }
  // block reduction of P partials
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < DM + 1; ++k) {
    if (k < P) {
      const float v = (k == P - 1) ? acc_s : acc[k < DM ? k : 0];
      const double s = warp_sum_d((double)v);
      if (lane == 0) sred[warp][k] = s;
    }
  }
  __syncthreads();
  if (threadIdx.x < P) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += sred[w][threadIdx.x];
    part[(size_t)blockIdx.x * P + threadIdx.x] = s;
  }
}

void launch_grad_trace(const Shape& sh, const float* theta, const float* Xf, const float* Binv, long long ld,
                       const float* sw, const float* c, const float* a, const int2* tiles, int ntiles, double* part,
                       cudaStream_t st) {
  if (sh.Dp <= 4)
    grad_trace_kernel<4><<<ntiles, 256, 0, st>>>(sh, theta, Xf, Binv, ld, sw, c, a, tiles, part);
  else if (sh.Dp <= 8)
    grad_trace_kernel<8><<<ntiles, 256, 0, st>>>(sh, theta, Xf, Binv, ld, sw, c, a, tiles, part);
  else
    grad_trace_kernel<16><<<ntiles, 256, 0, st>>>(sh, theta, Xf, Binv, ld, sw, c, a, tiles, part);
}

}  // namespace pgb
