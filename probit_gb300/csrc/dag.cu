// Persistent tile-DAG Cholesky of B = I + W^1/2 K W^1/2 with appended
// right-hand-side rows.
//
// The reference factors the Newton Jacobian with an LU solve
// (implicit/solvers.py:18-25, jnp.linalg.solve) and the evidence matrix with
// cholesky(K + diag(1/W)) (implicit/Laplace.py:24); the B form used here gives
// the same iterates and log-determinant (Woodbury; see the oracle).
//
// Left-looking by tiles: one task per 128 x 128 output tile (i, j), i >= j.
//   C = B_ij - sum_{k<j} L_ik L_jk^T
//   i == j : L_jj = chol(C)                 (in shared memory)
//   i >  j : L_ij = C L_jj^-T               (row-wise substitution)
// B_ij is recomputed from the features (K is never stored).  Tasks are handed
// out in a topological order (column by column) through one atomic counter,
// and a task only waits for tasks earlier in that order, so the launch
// cannot deadlock however many blocks are resident.  Every wait is bounded.
//
// Right-hand-side rows appended below B make the same launch solve
// X L^T = C_rhs, i.e. X = (L^-1 C_rhs^T)^T:
//   RHS_VEC   : one row t^T              -> (L^-1 t)^T        (Newton step)
//   RHS_IDENT : the identity             -> L^-T (upper)      (gradient)
//   RHS_CROSS : rows K(x*_m, X) W^1/2    -> (L^-1 W^1/2 K_*)^T (predict)
#include "kernels.cuh"
#include "tile_gemm.cuh"

namespace pgb {

constexpr int DAG_THREADS = 256;
constexpr int SC_LD = T + 1;
constexpr size_t DAG_SMEM = sizeof(float) * (2 * KC * SROW + 2 * T * SC_LD);

// Initial value of tile (i, j) before the left-looking updates.
template <int DM>
__device__ void fill_init(const DagJob& jb, const KernelParams& kp, int i, int j, float* sC) {
  const int n = jb.n;
  const bool is_rhs = i >= jb.nt;
  const int ri = i - jb.nt;
  for (int e = threadIdx.x; e < T * T; e += DAG_THREADS) {
    const int r = e >> 7, c = e & (T - 1);
    const int gj = j * T + c;
    float v = 0.0f;
    if (!is_rhs) {
      const int gi = i * T + r;
      if (i == j && c > r) {
        v = 0.0f;
      } else if (gi < n && gj < n) {
        float xi[DM], xj[DM];
#pragma unroll
        for (int d = 0; d < DM; ++d) {
          xi[d] = d < kp.Dp ? __ldg(jb.Xf + (size_t)gi * kp.Dp + d) : 0.0f;
          xj[d] = d < kp.Dp ? __ldg(jb.Xf + (size_t)gj * kp.Dp + d) : 0.0f;
        }
        float d2 = 0.0f;
#pragma unroll
        for (int d = 0; d < DM; ++d) {
          if (d < kp.D) {
            float q;
            if (kp.kind == PGB_KERNEL_EQ_PERIODIC) {
              const float t = (xi[d] - xj[d]) * kp.pi_over_p;
              q = (2.0f * sinf(t)) / kp.l[kp.nl == 1 ? 0 : d];
            } else {
              q = xi[d] - xj[d];
            }
            d2 += q * q;
          }
        }
        v = __ldcg(jb.sw + gi) * kernel_from_d2(kp, d2) * __ldcg(jb.sw + gj);
        if (gi == gj) v += 1.0f;
      } else {
        v = (gi == gj) ? 1.0f : 0.0f;
      }
    } else if (jb.rhs_kind == RHS_VEC) {
      const int gi = ri * T + r;
      v = (gi == 0 && gj < n) ? __ldcg(jb.rhs_vec + gj) : 0.0f;
    } else if (jb.rhs_kind == RHS_IDENT) {
      v = (ri == j && r == c) ? 1.0f : 0.0f;
    } else {  // RHS_CROSS
      const int gi = ri * T + r;
      if (gi < jb.nrhs && gj < n) {
        float xi[DM], xj[DM];
#pragma unroll
        for (int d = 0; d < DM; ++d) {
          xi[d] = d < kp.Dp ? __ldg(jb.Xq + (size_t)gi * kp.Dp + d) : 0.0f;
          xj[d] = d < kp.Dp ? __ldg(jb.Xf + (size_t)gj * kp.Dp + d) : 0.0f;
        }
        float d2 = 0.0f;
#pragma unroll
        for (int d = 0; d < DM; ++d) {
          if (d < kp.D) {
            float q;
            if (kp.kind == PGB_KERNEL_EQ_PERIODIC) {
              const float t = (xi[d] - xj[d]) * kp.pi_over_p;
              q = (2.0f * sinf(t)) / kp.l[kp.nl == 1 ? 0 : d];
            } else {
              q = xi[d] - xj[d];
            }
            d2 += q * q;
          }
        }
        v = kernel_from_d2(kp, d2) * __ldcg(jb.sw + gj);
      }
    }
    sC[r * SC_LD + c] = v;
  }
}

// In-place Cholesky of the lower triangle of the 128 x 128 tile in sC.
// 32-wide panels: warp 0 factors the diagonal block, all threads solve the
// rows below and update the trailing lower triangle.
__device__ void potrf_tile(float* sC, int col0, int* status) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int jb = 0; jb < T; jb += 32) {
    if (warp == 0) {
      for (int c = 0; c < 32; ++c) {
        const int cc = jb + c;
        const float piv = sC[cc * SC_LD + cc];
        const float lc = sqrtf(piv);
        if (lane == 0 && !(piv > 0.0f)) {
          atomicMin(status + ST_NOTPD_COL, col0 + cc);
          atomicCAS(status + ST_CODE, 0, PGB_ENOTPD);
        }
        __syncwarp();
        if (lane > c) sC[(jb + lane) * SC_LD + cc] /= lc;
        __syncwarp();
        if (lane == c) sC[cc * SC_LD + cc] = lc;
        if (lane > c) {
          const float lv = sC[(jb + lane) * SC_LD + cc];
          for (int m = c + 1; m <= lane; ++m) sC[(jb + lane) * SC_LD + jb + m] -= lv * sC[(jb + m) * SC_LD + cc];
        }
        __syncwarp();
      }
    }
    __syncthreads();
    const int rem = T - jb - 32;
    if (rem > 0) {
      if (tid < rem) {
        const int r = jb + 32 + tid;
        for (int c = 0; c < 32; ++c) {
          float x = sC[r * SC_LD + jb + c];
          for (int m = 0; m < c; ++m) x -= sC[r * SC_LD + jb + m] * sC[(jb + c) * SC_LD + jb + m];
          sC[r * SC_LD + jb + c] = x / sC[(jb + c) * SC_LD + jb + c];
        }
      }
      __syncthreads();
      for (int e = tid; e < rem * rem; e += DAG_THREADS) {
        const int r = jb + 32 + e / rem, c = jb + 32 + e % rem;
        if (c <= r) {
          float s = sC[r * SC_LD + c];
#pragma unroll 8
          for (int m = 0; m < 32; ++m) s -= sC[r * SC_LD + jb + m] * sC[c * SC_LD + jb + m];
          sC[r * SC_LD + c] = s;
        }
      }
      __syncthreads();
    }
  }
}

// X L^T = C for the rows of sC (in place), L lower in sL.
__device__ void trsm_rows(float* sC, const float* sL) {
  const int tid = threadIdx.x;
  for (int cb = 0; cb < T; cb += 32) {
    if (tid < T) {
      const int r = tid;
      for (int c = cb; c < cb + 32; ++c) {
        float x = sC[r * SC_LD + c];
        for (int m = cb; m < c; ++m) x -= sC[r * SC_LD + m] * sL[c * SC_LD + m];
        sC[r * SC_LD + c] = x / sL[c * SC_LD + c];
      }
    }
    __syncthreads();
    const int rem = T - cb - 32;
    for (int e = tid; e < T * rem; e += DAG_THREADS) {
      const int r = e / rem, c = cb + 32 + e % rem;
      float s = sC[r * SC_LD + c];
#pragma unroll 8
      for (int m = cb; m < cb + 32; ++m) s -= sC[r * SC_LD + m] * sL[c * SC_LD + m];
      sC[r * SC_LD + c] = s;
    }
    __syncthreads();
  }
}

// Thread 0 waits, everyone learns the outcome.
__device__ __forceinline__ bool block_wait(const int* flag, int* status, int* s_ok) {
  if (threadIdx.x == 0) {
    const bool ok = wait_flag_geq(flag, 1, status);
    __threadfence();
    *s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  const bool ok = *s_ok != 0;
  __syncthreads();
  return ok;
}

template <int DM>
__device__ void dag_task(const DagJob& jb, int i, int j, float* smem, int* s_ok) {
  float* sA = smem;
  float* sB = sA + KC * SROW;
  float* sC = sB + KC * SROW;
  float* sL = sC + T * SC_LD;
  const int nt = jb.nt;
  const long long ld = jb.ld;
  const bool is_rhs = i >= nt;
  const int ri = i - nt;
  float* rowbase = is_rhs ? jb.R + (size_t)ri * T * ld : jb.L + (size_t)i * T * ld;
  const int k0 = (is_rhs && jb.rhs_kind == RHS_IDENT) ? ri : 0;
  const KernelParams kp = make_kp(jb.sh, jb.theta);

  float acc[8][8];
  acc_zero(acc);
  for (int k = k0; k < j; ++k) {
    if (!block_wait(jb.ready + (size_t)i * nt + k, jb.status, s_ok)) return;
    if (!block_wait(jb.ready + (size_t)j * nt + k, jb.status, s_ok)) return;
    acc_gemm_tile(acc, rowbase + (size_t)k * T, ld, jb.L + (size_t)j * T * ld + (size_t)k * T, ld, sA, sB);
  }
  fill_init<DM>(jb, kp, i, j, sC);
  __syncthreads();
  {
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
      for (int b = 0; b < 8; ++b) sC[acc_row(ty, a) * SC_LD + acc_row(tx, b)] -= acc[a][b];
  }
  __syncthreads();
  float* dst = rowbase + (size_t)j * T;
  if (!is_rhs && i == j) {
    potrf_tile(sC, j * T, jb.status);
    for (int e = threadIdx.x; e < T * T; e += DAG_THREADS) {
      const int r = e >> 7, c = e & (T - 1);
      dst[(size_t)r * ld + c] = c <= r ? sC[r * SC_LD + c] : 0.0f;
    }
  } else {
    if (!block_wait(jb.ready + (size_t)j * nt + j, jb.status, s_ok)) return;
    const float* Ljj = jb.L + (size_t)j * T * ld + (size_t)j * T;
    for (int e = threadIdx.x; e < T * T; e += DAG_THREADS) {
      const int r = e >> 7, c = e & (T - 1);
      sL[r * SC_LD + c] = c <= r ? __ldcg(Ljj + (size_t)r * ld + c) : 0.0f;
    }
    __syncthreads();
    trsm_rows(sC, sL);
    for (int e = threadIdx.x; e < T * T; e += DAG_THREADS) {
      const int r = e >> 7, c = e & (T - 1);
      dst[(size_t)r * ld + c] = sC[r * SC_LD + c];
    }
    if (is_rhs && jb.rhs_kind == RHS_CROSS && threadIdx.x < T) {
      const int r = threadIdx.x;
      const int gi = ri * T + r;
      if (gi < jb.nrhs) {
        float s = 0.0f;
        for (int c = 0; c < T; ++c) {
          const float x = sC[r * SC_LD + c];
          s = fmaf(x, x, s);
        }
        jb.rowsq[(size_t)gi * nt + j] = s;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    st_release(jb.ready + (size_t)i * nt + j, 1);
  }
}

template <int DM>
__global__ void __launch_bounds__(DAG_THREADS, 1) dag_factor_kernel(const DagJob* __restrict__ jobs,
                                                                    const int4* __restrict__ tasks, int ntasks,
                                                                    int* __restrict__ counter) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int s_task;
  __shared__ int s_ok;
  while (true) {
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = atomicAdd(counter, 1);
      // a raised abort word ends this block's work (uniformly for the block)
      if (t < ntasks && ld_relaxed(jobs[tasks[t].x].status + ST_ABORT)) t = ntasks;
      s_task = t;
    }
    __syncthreads();
    const int t = s_task;
    if (t >= ntasks) break;
    const int4 tk = tasks[t];
    const DagJob jb = jobs[tk.x];
    dag_task<DM>(jb, tk.y, tk.z, smem, &s_ok);
  }
}

void dag_set_attributes() {
  cudaFuncSetAttribute(dag_factor_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DAG_SMEM);
  cudaFuncSetAttribute(dag_factor_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DAG_SMEM);
  cudaFuncSetAttribute(dag_factor_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DAG_SMEM);
}

void launch_dag_factor(const DagJob* jobs_dev, const int4* tasks, int ntasks, int* counter, int Dp, int grid,
                       cudaStream_t st) {
  if (Dp <= 4)
    dag_factor_kernel<4><<<grid, DAG_THREADS, DAG_SMEM, st>>>(jobs_dev, tasks, ntasks, counter);
  else if (Dp <= 8)
    dag_factor_kernel<8><<<grid, DAG_THREADS, DAG_SMEM, st>>>(jobs_dev, tasks, ntasks, counter);
  else
    dag_factor_kernel<16><<<grid, DAG_THREADS, DAG_SMEM, st>>>(jobs_dev, tasks, ntasks, counter);
}

// ---------------------------------------------------------------- B^-1 = Z Z^T
// Z = L^-T (upper, stored in the RHS rows of an RHS_IDENT factorisation).
// Tile (I, J), I >= J: sum over k >= I of Z_Ik Z_Jk^T; written to (I, J) and
// transposed to (J, I) so B^-1 is stored full.
__global__ void __launch_bounds__(256, 1) syrk_zzt_kernel(const float* __restrict__ Z, long long ldz, int nt,
                                                          const int2* __restrict__ tiles, float* __restrict__ Binv,
                                                          long long ldb) {
  extern __shared__ __align__(16) float smem[];
  float* sA = smem;
  float* sB = sA + KC * SROW;
  const int2 tl = tiles[blockIdx.x];
  const int I = tl.x, J = tl.y;
  float acc[8][8];
  acc_zero(acc);
  for (int k = I; k < nt; ++k)
    acc_gemm_tile(acc, Z + (size_t)I * T * ldz + (size_t)k * T, ldz, Z + (size_t)J * T * ldz + (size_t)k * T, ldz, sA,
                  sB);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int r = acc_row(ty, a), c = acc_row(tx, b);
      Binv[(size_t)(I * T + r) * ldb + J * T + c] = acc[a][b];
      if (I != J) Binv[(size_t)(J * T + c) * ldb + I * T + r] = acc[a][b];
    }
}

void launch_syrk_zzt(const float* Z, long long ldz, int nt, const int2* tiles, int ntiles, float* Binv, long long ldb,
                     cudaStream_t st) {
  const size_t smem = sizeof(float) * 2 * KC * SROW;
  syrk_zzt_kernel<<<ntiles, 256, smem, st>>>(Z, ldz, nt, tiles, Binv, ldb);
}

}  // namespace pgb
