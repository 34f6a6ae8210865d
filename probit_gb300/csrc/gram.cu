// Gram-matrix kernels.  K is never stored on the hot path: every consumer
// recomputes its entries from the prepared features (a few FMAs and one exp
// per entry), which costs less than streaming an N x N matrix from HBM.
//
// Kernel algebra restated from mlkernels as used by the reference
// (Laplace.py:7,21,24; approximators.py:172-174,192-194,272).
//
// The batched kernels take a device table of problems and a map from thread
// block to (problem, local block), so one launch covers every problem of a
// batch whatever their sizes.
#include "kernels.cuh"

namespace pgb {

// ---------------------------------------------------------------- features
// Row i of the features (zero padded to Dp; rows n .. n_pad all zero):
//   eq / matern12: x_d / l_d
//   eq_periodic:   sin(2 pi x_d / p) / l_d, cos(2 pi x_d / p) / l_d at 2d, 2d+1
__device__ __forceinline__ void prep_point(const Shape& sh, const float* __restrict__ X,
                                           const float* __restrict__ theta, float* __restrict__ Xf, int n, int i) {
  float* out = Xf + (size_t)i * sh.Dp;
  for (int f = 0; f < sh.Dp; ++f) out[f] = 0.0f;
  if (i >= n) return;
  for (int d = 0; d < sh.D; ++d) {
    const float x = X[(size_t)i * sh.D + d];
    const float l = __ldg(theta + (sh.nl == 1 ? 0 : d));
    if (sh.kind == PGB_KERNEL_EQ_PERIODIC) {
      const float u = 2.0f * x * sh.inv_p;
      out[2 * d] = sinpif(u) / l;
      out[2 * d + 1] = cospif(u) / l;
    } else {
      out[d] = x / l;
    }
  }
}

__global__ void prep_features_kernel(const Prob* __restrict__ probs, const int2* __restrict__ vmap) {
  const int2 m = vmap[blockIdx.x];
  const Prob& P = probs[m.x];
  if (*P.enabled == 0) return;
  const int i = m.y * VT + threadIdx.x;
  if (i >= P.n_pad) return;
  prep_point(P.sh, P.X, P.theta, P.Xf, P.sh.n, i);
}

void launch_prep_features(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st) {
  if (nblocks > 0) prep_features_kernel<<<nblocks, VT, 0, st>>>(probs, vmap);
}

__global__ void prep_features_raw_kernel(Shape sh, const float* __restrict__ X, const float* __restrict__ theta,
                                         float* __restrict__ Xf, int n, int n_pad) {
  const int i = blockIdx.x * VT + threadIdx.x;
  if (i >= n_pad) return;
  prep_point(sh, X, theta, Xf, n, i);
}

void launch_prep_features_raw(const Shape& sh, const float* X, const float* theta, float* Xf, int n, int n_pad,
                              cudaStream_t st) {
  if (n_pad > 0) prep_features_raw_kernel<<<ceil_div(n_pad, VT), VT, 0, st>>>(sh, X, theta, Xf, n, n_pad);
}

// Squared feature distance with the feature loop unrolled to DM (>= Dp;
// features beyond Dp are zero on both sides).
template <int DM>
__device__ __forceinline__ float d2_t(const float* xi, const float* xj) {
  float d2 = 0.0f;
#pragma unroll
  for (int f = 0; f < DM; ++f) {
    const float v = xi[f] - xj[f];
    d2 = fmaf(v, v, d2);
  }
  return d2;
}

// ---------------------------------------------------------------- full Gram
template <int DM>
__global__ void gram_full_kernel(Shape sh, const float* __restrict__ theta, const float* __restrict__ X1, int n1,
                                 const float* __restrict__ X2, int n2, float* __restrict__ K, long long ldk) {
  const float s = theta_signal(sh, theta);
  const int matern = sh.kind == PGB_KERNEL_MATERN12;
  const int j = blockIdx.x * 32 + (threadIdx.x & 31);
  const int i0 = blockIdx.y * 32 + (threadIdx.x >> 5);
  if (j >= n2) return;
  float xj[DM];
#pragma unroll
  for (int f = 0; f < DM; ++f) xj[f] = f < sh.Dp ? X2[(size_t)j * sh.Dp + f] : 0.0f;
  for (int i = i0; i < min(n1, blockIdx.y * 32 + 32); i += 8) {
    float xi[DM];
#pragma unroll
    for (int f = 0; f < DM; ++f) xi[f] = f < sh.Dp ? X1[(size_t)i * sh.Dp + f] : 0.0f;
    K[(size_t)i * ldk + j] = kernel_of_d2(matern, s, d2_t<DM>(xi, xj));
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
// One block owns mv_block_rows(DM) rows and sweeps all columns; the per-row sums are
// reduced in a fixed order, so results are bitwise reproducible.  The kernel
// family is a template parameter and every per-entry quantity lives in
// registers or shared memory.
constexpr int MV_THREADS = 256;
template <int DM>
constexpr int mv_rows() { return mv_block_rows(DM); }

template <int MATERN, int DM>
__device__ __forceinline__ float kval(const float* xi, const float* xj, float s) {
  const float d2 = d2_t<DM>(xi, xj);
  if (MATERN) return s * expf(-sqrtf(d2));
  return s * expf(-0.5f * d2);
}

template <int MATERN, int DM, bool HAS_M>
__device__ __forceinline__ void mv_core(const Shape& sh, const float* __restrict__ theta,
                                        const float* __restrict__ Xr, int nr, const float* __restrict__ Xc, int nc,
                                        const float* __restrict__ M, long long ldm, const float* __restrict__ v,
                                        const float* __restrict__ row_scale, float* __restrict__ y, int r0,
                                        bool accumulate = false) {
  constexpr int MV_ROWS = mv_rows<DM>();
  __shared__ float sx[MV_ROWS][DM];
  __shared__ float sred[MV_THREADS / 32][MV_ROWS];
  const int Dp = sh.Dp;
  const float sv = theta_signal(sh, theta);
  for (int e = threadIdx.x; e < MV_ROWS * DM; e += MV_THREADS) {
    const int r = e / DM, f = e % DM;
    sx[r][f] = (r0 + r < nr && f < Dp) ? Xr[(size_t)(r0 + r) * Dp + f] : 0.0f;
  }
  __syncthreads();
  float acc[MV_ROWS];
#pragma unroll
  for (int r = 0; r < MV_ROWS; ++r) acc[r] = 0.0f;
  const int rmax = min(MV_ROWS, nr - r0);
  // HAS_M: the column's entries of M (one per row, from HBM) are loaded one
  // column step ahead, so their latency overlaps the kernel evaluations of
  // the current step instead of stalling each row's product
  float mr[HAS_M ? MV_ROWS : 1], mn[HAS_M ? MV_ROWS : 1];
  auto load_m = [&](float (&dst)[HAS_M ? MV_ROWS : 1], int c) {
#pragma unroll
    for (int r = 0; r < (HAS_M ? MV_ROWS : 1); ++r)
      dst[r] = (HAS_M && r < rmax && c < nc) ? __ldg(M + (size_t)(r0 + r) * ldm + c) : 0.0f;
  };
  if constexpr (HAS_M) load_m(mr, threadIdx.x);
  for (int c = threadIdx.x; c < nc; c += MV_THREADS) {
    if constexpr (HAS_M) load_m(mn, c + MV_THREADS);
    float xc[DM];
#pragma unroll
    for (int f = 0; f < DM; ++f) xc[f] = f < Dp ? __ldg(Xc + (size_t)c * Dp + f) : 0.0f;
    const float vc = __ldg(v + c);
    if (rmax == MV_ROWS) {
#pragma unroll
      for (int r = 0; r < MV_ROWS; ++r) {
        float k = kval<MATERN, DM>(sx[r], xc, sv);
        if constexpr (HAS_M) k *= mr[r];
        acc[r] = fmaf(k, vc, acc[r]);
      }
    } else {
#pragma unroll
      for (int r = 0; r < MV_ROWS; ++r) {
        if (r < rmax) {
          float k = kval<MATERN, DM>(sx[r], xc, sv);
          if constexpr (HAS_M) k *= mr[r];
          acc[r] = fmaf(k, vc, acc[r]);
        }
      }
    }
    if constexpr (HAS_M) {
#pragma unroll
      for (int r = 0; r < MV_ROWS; ++r) mr[r] = mn[r];
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
    y[r0 + threadIdx.x] = accumulate ? y[r0 + threadIdx.x] + t : t;
  }
}

__device__ __forceinline__ float* prob_field(const Prob& P, int f) {
  switch (f) {
    case F_A: return P.a;
    case F_F: return P.f;
    case F_D1: return P.d1;
    case F_W: return P.W;
    case F_SW: return P.sw;
    case F_R: return P.r;
    case F_T: return P.t;
    case F_X: return P.x;
    case F_LOGP: return P.logp;
    case F_D3: return P.d3;
    case F_DSIG: return P.dsig;
    case F_SVEC: return P.svec;
    case F_RV: return P.rv;
    case F_ZBAR: return P.zbar;
    case F_TZ: return P.tz;
    case F_Y2: return P.y2;
    case F_U: return P.u;
    case F_C: return P.c;
    case F_ROWDOT: return P.rowdot;
    case F_DA: return P.da;
    default: return nullptr;
  }
}

template <int MATERN, int DM, bool HAS_M>
__device__ __forceinline__ void gram_matvec_item(const Prob* __restrict__ probs, int2 m, const MatvecOp& op) {
  const Prob& P = probs[m.x];
  if (op.only_active && *P.active == 0) return;
  const int n = P.sh.n;
  mv_core<MATERN, DM, HAS_M>(P.sh, P.theta, P.Xf, n, P.Xf, n, P.Binv, P.ld, prob_field(P, op.v),
                           prob_field(P, op.row_scale), prob_field(P, op.y), m.y * mv_rows<DM>(), op.accumulate != 0);
}

// One map item (problem, row block) per block.  STRIDE: the grid is smaller
// than the map (a handle whose launches are capped to a share of the SMs)
// and the blocks stride over it; a separate instantiation, so the one-item
// kernel keeps its own register allocation.
template <int MATERN, int DM, bool HAS_M, bool STRIDE>
__global__ void __launch_bounds__(MV_THREADS) gram_matvec_kernel(const Prob* __restrict__ probs,
                                                                 const int2* __restrict__ mvmap, int nitems,
                                                                 MatvecOp op) {
  if constexpr (!STRIDE) {
    gram_matvec_item<MATERN, DM, HAS_M>(probs, mvmap[blockIdx.x], op);
  } else {
    for (int b = blockIdx.x; b < nitems; b += gridDim.x) {
      gram_matvec_item<MATERN, DM, HAS_M>(probs, mvmap[b], op);
      __syncthreads();   // the next item's staging overwrites the shared rows
    }
  }
}

template <int MATERN, int DM>
__global__ void __launch_bounds__(MV_THREADS) gram_matvec_raw_kernel(Shape sh, const float* __restrict__ theta,
                                                                     const float* __restrict__ Xr, int nr,
                                                                     const float* __restrict__ Xc, int nc,
                                                                     const float* __restrict__ v,
                                                                     float* __restrict__ y) {
  mv_core<MATERN, DM, false>(sh, theta, Xr, nr, Xc, nc, nullptr, 0, v, nullptr, y, blockIdx.x * mv_rows<DM>());
}

template <int MATERN, int DM>
static void mv_launch(const Prob* probs, const int2* mvmap, int nitems, int grid, MatvecOp op, cudaStream_t st) {
  const bool stride = grid < nitems;
  if (op.use_binv) {
    if (stride)
      gram_matvec_kernel<MATERN, DM, true, true><<<grid, MV_THREADS, 0, st>>>(probs, mvmap, nitems, op);
    else
      gram_matvec_kernel<MATERN, DM, true, false><<<grid, MV_THREADS, 0, st>>>(probs, mvmap, nitems, op);
  } else {
    if (stride)
      gram_matvec_kernel<MATERN, DM, false, true><<<grid, MV_THREADS, 0, st>>>(probs, mvmap, nitems, op);
    else
      gram_matvec_kernel<MATERN, DM, false, false><<<grid, MV_THREADS, 0, st>>>(probs, mvmap, nitems, op);
  }
}

template <int MATERN>
static void mv_launch_d(int DM, const Prob* probs, const int2* mvmap, int nitems, int grid, MatvecOp op,
                        cudaStream_t st) {
  if (DM <= 4)
    mv_launch<MATERN, 4>(probs, mvmap, nitems, grid, op, st);
  else if (DM <= 8)
    mv_launch<MATERN, 8>(probs, mvmap, nitems, grid, op, st);
  else
    mv_launch<MATERN, 16>(probs, mvmap, nitems, grid, op, st);
}

void launch_gram_matvec(int kind, int DM, const Prob* probs, const int2* mvmap, int nitems, int grid, MatvecOp op,
                        cudaStream_t st) {
  if (nitems <= 0) return;
  grid = grid > 0 && grid < nitems ? grid : nitems;
  if (kind == PGB_KERNEL_MATERN12)
    mv_launch_d<1>(DM, probs, mvmap, nitems, grid, op, st);
  else
    mv_launch_d<0>(DM, probs, mvmap, nitems, grid, op, st);
}

template <int MATERN>
static void mv_raw_d(const Shape& sh, const float* theta, const float* Xr, int nr, const float* Xc, int nc,
                     const float* v, float* y, cudaStream_t st) {
  if (sh.Dp <= 4)
    gram_matvec_raw_kernel<MATERN, 4>
        <<<ceil_div(nr, mv_rows<4>()), MV_THREADS, 0, st>>>(sh, theta, Xr, nr, Xc, nc, v, y);
  else if (sh.Dp <= 8)
    gram_matvec_raw_kernel<MATERN, 8>
        <<<ceil_div(nr, mv_rows<8>()), MV_THREADS, 0, st>>>(sh, theta, Xr, nr, Xc, nc, v, y);
  else
    gram_matvec_raw_kernel<MATERN, 16>
        <<<ceil_div(nr, mv_rows<16>()), MV_THREADS, 0, st>>>(sh, theta, Xr, nr, Xc, nc, v, y);
}

void launch_gram_matvec_raw(const Shape& sh, const float* theta, const float* Xr, int nr, const float* Xc, int nc,
                            const float* v, float* y, cudaStream_t st) {
  if (nr <= 0) return;
  if (sh.kind == PGB_KERNEL_MATERN12)
    mv_raw_d<1>(sh, theta, Xr, nr, Xc, nc, v, y, st);
  else
    mv_raw_d<0>(sh, theta, Xr, nr, Xc, nc, v, y, st);
}

// ---------------------------------------------------------------- B^-1 matvec
// One map item of binv_matvec_kernel (no shared memory, no barrier: a warp
// whose row is past n returns on its own).
__device__ __forceinline__ void binv_matvec_item(const Prob* __restrict__ probs, int2 m) {
  const Prob& P = probs[m.x];
  if (*P.active == 0) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = m.y * 8 + warp;
  const int n = P.sh.n;
  if (r >= n) return;
  const float* a = P.Binv + (size_t)r * P.ld;
  const float* v = P.tz;
  float s = 0.0f;
  for (int c = lane * 4; c < n; c += 128) {
    if (c + 3 < n) {
      const float4 x = __ldg(reinterpret_cast<const float4*>(a + c));
      const float4 w = __ldg(reinterpret_cast<const float4*>(v + c));
      s = fmaf(x.x, w.x, s);
      s = fmaf(x.y, w.y, s);
      s = fmaf(x.z, w.z, s);
      s = fmaf(x.w, w.w, s);
    } else {
      for (int e = c; e < n; ++e) s = fmaf(a[e], v[e], s);
    }
  }
  s = warp_sum(s);
  if (lane == 0) P.y2[r] = s;
}

// y2[r] = sum_c B^-1[r, c] tz[c]: one warp per row, 8 rows per map item
// (bmap: item -> (problem, row block)); a grid smaller than the map strides
// over it.
__global__ void __launch_bounds__(256) binv_matvec_kernel(const Prob* __restrict__ probs,
                                                          const int2* __restrict__ bmap, int nitems) {
  for (int b = blockIdx.x; b < nitems; b += gridDim.x) binv_matvec_item(probs, bmap[b]);
}

void launch_binv_matvec(const Prob* probs, const int2* bmap, int nitems, int grid, cudaStream_t st) {
  if (nitems <= 0) return;
  grid = grid > 0 && grid < nitems ? grid : nitems;
  binv_matvec_kernel<<<grid, 256, 0, st>>>(probs, bmap, nitems);
}

// ---------------------------------------------------------------- gradient trace
// Over the lower 128x128 tiles (I >= J) of B^-1 (stored full, row-major, ld):
//   g_k += sum_{i,j} M_ij dK_k(x_i, x_j),  M = 1/2 R + c a^T,  R = sw B^-1 sw
// folded to the lower triangle: off-diagonal pairs carry R_ij + c_i a_j +
// c_j a_i, the diagonal 1/2 R_ii + c_i a_i (only dK/ds is nonzero there).
// With q_d the squared feature distance of input dimension d (feature d, or
// features 2d and 2d+1 for eq_periodic): dK/dl_d = K q_d / l_d (Matern12:
// times 1/r, 0 at r = 0), dK/ds = K / s.
// tiles: (problem, I, J, ordinal of the tile within its problem); each block
// writes its partial sums (double) to tpart[ordinal * (nl + 1) + k].
template <int DM, bool PER>
__device__ __forceinline__ void grad_trace_tile(const Prob* __restrict__ probs, const int4 tl) {
  constexpr int ND = PER ? DM / 2 : DM;   // input dimensions covered
  const Prob& P = probs[tl.x];
  if (*P.active == 0) return;
  const int I = tl.y, J = tl.z, ord = tl.w;
  const Shape sh = P.sh;
  const float sv = theta_signal(sh, P.theta);
  const int matern = sh.kind == PGB_KERNEL_MATERN12;
  const int NP = sh.nl + 1;
  const int n = sh.n;
  const float* __restrict__ Xf = P.Xf;
  const float* __restrict__ Binv = P.Binv;
  const long long ld = P.ld;
  const float* __restrict__ sw = P.sw;
  const float* __restrict__ cvec = P.c;
  const float* __restrict__ avec = P.a;
  // features and per-point vectors of the tile's columns (J) and rows (I)
  __shared__ float sxc[T][DM], sxr[T][DM];
  __shared__ float ssw[T], sc[T], sa[T], sswr[T], scr[T], sar[T];
  __shared__ float sinvl[MAX_D];
  __shared__ double sred[8][MAX_D + 1];
  for (int e = threadIdx.x; e < T * DM; e += 256) {
    const int c = e / DM, f = e % DM;
    const int gc = J * T + c, gr = I * T + c;
    sxc[c][f] = (gc < n && f < sh.Dp) ? Xf[(size_t)gc * sh.Dp + f] : 0.0f;
    sxr[c][f] = (gr < n && f < sh.Dp) ? Xf[(size_t)gr * sh.Dp + f] : 0.0f;
  }
  for (int c = threadIdx.x; c < T; c += 256) {
    const int gc = J * T + c, gr = I * T + c;
    ssw[c] = gc < n ? sw[gc] : 0.0f;
    sc[c] = gc < n ? cvec[gc] : 0.0f;
    sa[c] = gc < n ? avec[gc] : 0.0f;
    sswr[c] = gr < n ? sw[gr] : 0.0f;
    scr[c] = gr < n ? cvec[gr] : 0.0f;
    sar[c] = gr < n ? avec[gr] : 0.0f;
  }
  if (threadIdx.x < MAX_D) sinvl[threadIdx.x] = threadIdx.x < sh.nl ? 1.0f / __ldg(P.theta + threadIdx.x) : 0.0f;
  __syncthreads();
  float acc[ND];
  float acc_s = 0.0f;
#pragma unroll
  for (int k = 0; k < ND; ++k) acc[k] = 0.0f;
  const int c = threadIdx.x & (T - 1);
  const int rh = threadIdx.x >> 7;  // 0 or 1
  const int gc = J * T + c;
  // this thread's entries of B^-1 are loaded two of its rows ahead, so their
  // latency overlaps the kernel evaluations of the rows before them
  auto load_b = [&](int r) {
    const int gr = I * T + r;
    return (r < T && gr < n && gc < n && gc <= gr) ? __ldcg(Binv + (size_t)gr * ld + gc) : 0.0f;
  };
  float b0 = load_b(rh), b1 = load_b(rh + 2);
  for (int r = rh; r < T; r += 2) {
    const int gr = I * T + r;
    const float bij = b0;
    b0 = b1;
    b1 = load_b(r + 4);
    if (gr >= n || gc >= n || gc > gr) continue;
    float xr[DM];
#pragma unroll
    for (int f = 0; f < DM; ++f) xr[f] = sxr[r][f];
    const float swr = sswr[r], cr = scr[r], ar = sar[r];
    float m;
    if (gr == gc)
      m = 0.5f * swr * bij * swr + cr * ar;
    else
      m = swr * bij * ssw[c] + cr * sa[c] + sc[c] * ar;
    float q[ND];
    float d2 = 0.0f;
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      if (PER) {
        const float u = xr[2 * d] - sxc[c][2 * d], w = xr[2 * d + 1] - sxc[c][2 * d + 1];
        q[d] = fmaf(u, u, w * w);
      } else {
        const float u = xr[d] - sxc[c][d];
        q[d] = u * u;
      }
      d2 += q[d];
    }
    const float K = kernel_of_d2(matern, sv, d2);
    float scale = K * m;
    if (matern) {
      const float rr = sqrtf(d2);
      scale = rr > 0.0f ? scale / rr : 0.0f;
    }
    if (sh.nl == 1) {
      acc[0] += scale * d2 * sinvl[0];
    } else {
#pragma unroll
      for (int d = 0; d < ND; ++d) acc[d] += scale * q[d] * sinvl[d];
    }
    acc_s += K * m / sv;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < ND + 1; ++k) {
    if (k < NP) {
      const float v = (k == NP - 1) ? acc_s : acc[k < ND ? k : 0];
      const double s = warp_sum_d((double)v);
      if (lane == 0) sred[warp][k] = s;
    }
  }
  __syncthreads();
  if (threadIdx.x < NP) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += sred[w][threadIdx.x];
    P.tpart[(size_t)ord * NP + threadIdx.x] = s;
  }
}

// One tile per block.  STRIDE: the grid is smaller than the tile list (a
// handle whose launches are capped to a share of the SMs) and the blocks
// stride over it (a separate instantiation, as for the Gram matvec).
template <int DM, bool PER, bool STRIDE>
__global__ void __launch_bounds__(256) grad_trace_kernel(const Prob* __restrict__ probs,
                                                         const int4* __restrict__ tiles, int ntiles) {
  if constexpr (!STRIDE) {
    grad_trace_tile<DM, PER>(probs, tiles[blockIdx.x]);
  } else {
    for (int b = blockIdx.x; b < ntiles; b += gridDim.x) {
      grad_trace_tile<DM, PER>(probs, tiles[b]);
      __syncthreads();   // the next tile's staging overwrites the shared rows and sums
    }
  }
}

template <int DM, bool PER>
static void trace_launch(const Prob* probs, const int4* tiles, int ntiles, int grid, cudaStream_t st) {
  if (grid < ntiles)
    grad_trace_kernel<DM, PER, true><<<grid, 256, 0, st>>>(probs, tiles, ntiles);
  else
    grad_trace_kernel<DM, PER, false><<<grid, 256, 0, st>>>(probs, tiles, ntiles);
}

void launch_grad_trace(int DM, int periodic, const Prob* probs, const int4* tiles, int ntiles, int grid,
                       cudaStream_t st) {
  if (ntiles <= 0) return;
  grid = grid > 0 && grid < ntiles ? grid : ntiles;
  if (periodic) {
    if (DM <= 4)
      trace_launch<4, true>(probs, tiles, ntiles, grid, st);
    else if (DM <= 8)
      trace_launch<8, true>(probs, tiles, ntiles, grid, st);
    else
      trace_launch<16, true>(probs, tiles, ntiles, grid, st);
  } else {
    if (DM <= 4)
      trace_launch<4, false>(probs, tiles, ntiles, grid, st);
    else if (DM <= 8)
      trace_launch<8, false>(probs, tiles, ntiles, grid, st);
    else
      trace_launch<16, false>(probs, tiles, ntiles, grid, st);
  }
}

}  // namespace pgb
