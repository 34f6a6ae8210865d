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
#include "umma.cuh"

namespace pgb {

constexpr int DAG_THREADS = 256;
constexpr int SC_LD = T + 1;
// tensor-core pipeline, unioned with the epilogue tiles sC, sL: NST stages,
// each one CHUNK_COLS-column chunk of the A and B operands as their TF32 hi
// and lo parts (four 128 x CHUNK_COLS fp32 boxes), loaded straight from the
// split operand matrices (the epilogue that publishes a tile also writes its
// split).  A stage is reloaded once the MMAs of its chunk completed.
// (16-column chunks, six 32 KB stages with five in flight, measured 8-10%
// slower than 32-column ones in three 64 KB stages.)
constexpr int CHUNK_BYTES = T * CHUNK_COLS * 4;  // 128 rows x CHUNK_COLS fp32
constexpr int STAGE_BYTES = 4 * CHUNK_BYTES;     // A hi, A lo, B hi, B lo
constexpr int NST = 196608 / STAGE_BYTES;        // 192 KB of stages
constexpr int UNION_BYTES = NST * STAGE_BYTES;   // >= 2 * T * SC_LD * 4
constexpr int CHUNKS_PER_KT = T / CHUNK_COLS;    // chunks of one 128-wide k-tile
constexpr int CHUNKS_PER_PART = 64 / CHUNK_COLS; // chunks summed in one partial accumulator (64 k-columns)
constexpr int KSTEPS = CHUNK_COLS / 8;           // MMA k-steps (8 TF32 each) of a chunk
constexpr int DRAIN_WARPS = DAG_THREADS / 32 - 2;   // warps 2..7 fold the partial sums
constexpr int NBARS = 2 * NST + 4;               // full, empty [NST]; part full, part free [2]
// tensor memory: the running 128 x 128 fp32 sum in columns 0..127 and two
// partial accumulators (CHUNKS_PER_PART chunks each) in 128..255, 256..383
constexpr uint32_t RUN_COL = 0;
constexpr uint32_t PART_COL = 128;
constexpr uint32_t TMEM_COLS = 512;
constexpr size_t DAG_SMEM = UNION_BYTES + (2 * T * 17 + 2 * T) * 4 + 1024 + 64;
static_assert(UNION_BYTES >= (T * SC_LD + T * (T + 4)) * 4, "epilogue tiles must fit in the stage buffers");
static_assert(DAG_SMEM <= 232448, "dynamic shared memory above the 227 KB a block may use");
static_assert(CHUNKS_PER_KT % CHUNKS_PER_PART == 0, "a k-tile is a whole number of partials");
constexpr uint32_t IDESC_128x128 = idesc_tf32(128, 128);
constexpr uint64_t MMA_WAIT_NS = 2000000000ull;  // 2 s

// Initial value C_init of tile (i, j) before the left-looking updates.  The
// row and column features (and W^1/2) of the tile are staged in shared
// memory first; each thread then evaluates the entries it owns in the TMEM
// accumulator layout (row = TMEM lane, 64 columns) and stores -C_init there,
// so the MMAs accumulate sum_k L_ik L_jk^T - C_init and the tile costs no
// work after its last dependency arrives.
//   L tile (i, j):  w_r K(x_r, x_c) w_c (+ 1 on the diagonal; the upper half
//                   of a diagonal tile is 0; padding rows/columns have w = 0)
//   RHS_CROSS rows: K(x*_r, x_c) w_c for the query points (row weight 1)
//   RHS_VEC row 0:  t;   RHS_IDENT: the identity block of row tile rrow
// The entry loop is one uniform formula over the zero-padded features, so
// its code stays small whatever the kernel family.
constexpr int SX_STRIDE = 17;   // DM + 1 (<= 16 + 1), breaks bank conflicts

template <int DM>
__device__ void stage_features(const DagJob& jb, int i, int j, float* sX) {
  const int n = jb.n;
  const bool is_rhs = i >= jb.nt;
  const bool cross = is_rhs && jb.rhs_kind == RHS_CROSS;
  const int ri = i - jb.nt;
  const int Dp = jb.sh.Dp;
  float* sXr = sX;
  float* sXc = sX + T * SX_STRIDE;
  float* sWr = sXc + T * SX_STRIDE;
  float* sWc = sWr + T;
  for (int e = threadIdx.x; e < T * DM; e += DAG_THREADS) {
    const int r = e / DM, f = e % DM;
    const int gj = j * T + r;
    sXc[r * SX_STRIDE + f] = (gj < n && f < Dp) ? __ldg(jb.Xf + (size_t)gj * Dp + f) : 0.0f;
    float xr = 0.0f;
    if (f < Dp) {
      if (!is_rhs) {
        const int gi = i * T + r;
        if (gi < n) xr = __ldg(jb.Xf + (size_t)gi * Dp + f);
      } else if (cross) {
        const int gi = ri * T + r;
        if (gi < jb.nrhs) xr = __ldg(jb.Xq + (size_t)gi * Dp + f);
      }
    }
    sXr[r * SX_STRIDE + f] = xr;
  }
  for (int r = threadIdx.x; r < T; r += DAG_THREADS) {
    const int gj = j * T + r, gi = i * T + r;
    sWc[r] = gj < n ? __ldcg(jb.sw + gj) : 0.0f;
    float wr = 0.0f;
    if (!is_rhs)
      wr = gi < n ? __ldcg(jb.sw + gi) : 0.0f;
    else if (cross)
      wr = (ri * T + r < jb.nrhs) ? 1.0f : 0.0f;
    sWr[r] = wr;
  }
}

// -C_init into the TMEM accumulator (all 8 warps; thread: row r, columns
// cb .. cb + 63).
template <int DM>
__device__ void cinit_to_tmem(const DagJob& jb, int i, int j, uint32_t tmem, const float* sX, int rk, int rrow) {
  const float* sXr = sX;
  const float* sXc = sX + T * SX_STRIDE;
  const float* sWr = sXc + T * SX_STRIDE;
  const float* sWc = sWr + T;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = (w & 3) * 32 + lane;
  const int cb = (w >> 2) * 64;
  const uint32_t taddr = tmem + ((uint32_t)((w & 3) * 32) << 16);
  const bool is_rhs = i >= jb.nt;
  if (!is_rhs || rk == RHS_CROSS) {
    const int matern = jb.sh.kind == PGB_KERNEL_MATERN12;
    const float sv = __ldg(jb.theta + jb.sh.nl);
    const bool diag = !is_rhs && i == j;
    float xr[DM];
#pragma unroll
    for (int f = 0; f < DM; ++f) xr[f] = sXr[r * SX_STRIDE + f];
    const float wr = sWr[r];
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
      float v[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const int c = cb + 32 * h + q;
        float d2 = 0.0f;
#pragma unroll
        for (int f = 0; f < DM; ++f) {
          const float u = xr[f] - sXc[c * SX_STRIDE + f];
          d2 = fmaf(u, u, d2);
        }
        float val = wr * kernel_of_d2(matern, sv, d2) * sWc[c];
        if (diag) {
          if (c == r) val += 1.0f;
          if (c > r) val = 0.0f;
        }
        v[q] = -val;
      }
      tmem_st_32x32(taddr + (uint32_t)(cb + 32 * h), v);
    }
  } else {
    const int n = jb.n;
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
      float v[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const int c = cb + 32 * h + q;
        const int gj = j * T + c;
        float val;
        if (rk == RHS_VEC)
          val = (rrow == 0 && r == 0 && gj < n) ? __ldcg(jb.rhs_vec + gj) : 0.0f;
        else
          val = (rrow == j && r == c) ? 1.0f : 0.0f;
        v[q] = -val;
      }
      tmem_st_32x32(taddr + (uint32_t)(cb + 32 * h), v);
    }
  }
  tmem_wait_st();
  tc_fence_before();
}

constexpr unsigned FULL = 0xffffffffu;

// Barrier over the first `count` threads of the block (a multiple of 32),
// named barrier 1 (__syncthreads uses 0).
__device__ __forceinline__ void bar_sync_first(int count) {
  asm volatile("bar.sync 1, %0;" ::"r"(count) : "memory");
}

// Cholesky of one 32-wide panel of the tile in sC (row stride SC_LD): the
// rows jb..127 of columns jb..jb+31, whose trailing updates are applied.
// Thread t < nr = 128 - jb holds row jb + t in registers, and the columns go
// four at a time.  Group C0..C0+3: the warp of the diagonal block (threads
// 0..31) factors its 4 x 4 diagonal block by shuffles (pivot from lane C,
// scale by the pivot's reciprocal square root, update the group's later
// columns with the multiplier shuffled from its row's lane) and puts every
// lane's four entries in four lines of shared memory (line c, entry lane:
// L[jb+lane][C0+c]) and the four reciprocal square roots beside them; one
// barrier over the panel's warps; every row below the diagonal block then
// solves its four entries against the 4 x 4 block from the lines, and every
// row updates its later columns by a rank-4 update with the multipliers
// L[jb+C0+m][C0+c] = line c, entry C0+m (16-byte broadcast loads; entries
// 32..63 of each line are 0, for the register slots past the panel).  So
// one barrier serves four columns.  Entries above the diagonal are computed
// too (no per-entry predicate) and never written back.  The lines are
// double-buffered by group parity: the barrier of group g orders its stores
// before the loads, and every warp passes barrier g + 1 only after its loads
// of group g, before the stores of group g + 2.  Every group the row is
// shifted left by 4 registers, so the loop stays small while every register
// index is a compile-time constant.  sbuf: 576 floats, 16-byte aligned (two
// buffers of four 64-float lines and four reciprocal square roots).
constexpr int PBUF = 4 * 64 + 32;
__device__ __forceinline__ void panel_potrf(float* sC, int jb, float* sbuf, int col0, int* status) {
  const int tid = threadIdx.x, lane = tid & 31;
  const int nr = T - jb;
  if (tid >= nr) return;
  const bool dwarp = tid < 32;
  float* row = sC + (jb + tid) * SC_LD + jb;
  if (dwarp) {
#pragma unroll
    for (int k = 0; k < 8; ++k) sbuf[(k >> 2) * PBUF + (k & 3) * 64 + 32 + lane] = 0.0f;
  }
  float d[32];
#pragma unroll
  for (int m = 0; m < 32; ++m) d[m] = row[m];
  int bad = -1;
#pragma unroll 1
  for (int C0 = 0; C0 < 32; C0 += 4) {
    float* lines = sbuf + PBUF * ((C0 >> 2) & 1);
    float* srl = lines + 4 * 64;
    float l[4];
    if (dwarp) {
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int C = C0 + c;
        const float piv = __shfl_sync(FULL, d[c], C);
        if (!(piv > 0.0f) && bad < 0) bad = C;
        const float rl = rsqrtf(piv);
        l[c] = (lane == C) ? piv * rl : d[c] * rl;
        if (lane == C) srl[c] = rl;
#pragma unroll
        for (int c2 = c + 1; c2 < 4; ++c2) d[c2] = fmaf(-l[c], __shfl_sync(FULL, l[c], C0 + c2), d[c2]);
        lines[c * 64 + lane] = l[c];
      }
      bar_sync_first(nr);
    } else {
      bar_sync_first(nr);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        float v = d[c];
#pragma unroll
        for (int c2 = 0; c2 < c; ++c2) v = fmaf(-l[c2], lines[c2 * 64 + C0 + c], v);
        l[c] = v * srl[c];
      }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c)
      if (!dwarp || lane >= C0 + c) row[C0 + c] = l[c];
#pragma unroll
    for (int q = 1; q < 8; ++q) {
      const float4 v0 = *reinterpret_cast<const float4*>(lines + 0 * 64 + C0 + 4 * q);
      const float4 v1 = *reinterpret_cast<const float4*>(lines + 1 * 64 + C0 + 4 * q);
      const float4 v2 = *reinterpret_cast<const float4*>(lines + 2 * 64 + C0 + 4 * q);
      const float4 v3 = *reinterpret_cast<const float4*>(lines + 3 * 64 + C0 + 4 * q);
      const float a0[4] = {v0.x, v0.y, v0.z, v0.w}, a1[4] = {v1.x, v1.y, v1.z, v1.w};
      const float a2[4] = {v2.x, v2.y, v2.z, v2.w}, a3[4] = {v3.x, v3.y, v3.z, v3.w};
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        float x = d[4 * q + e];
        x = fmaf(-l[0], a0[e], x);
        x = fmaf(-l[1], a1[e], x);
        x = fmaf(-l[2], a2[e], x);
        x = fmaf(-l[3], a3[e], x);
        d[4 * q + e] = x;
      }
    }
#pragma unroll
    for (int m = 0; m < 28; ++m) d[m] = d[m + 4];
  }
  if (tid == 0 && bad >= 0) {
    atomicMin(status + ST_NOTPD_COL, col0 + bad);
    atomicCAS(status + ST_CODE, 0, PGB_ENOTPD);
  }
}

// Row stride of transposed L panels in shared memory (Lt[c * LT_LD + r] =
// L[r][c]): a multiple of 4, so a column of L is read as 16-byte vectors.
constexpr int LT_LD = T + 4;

// Row substitution x L^T = c for a 32-wide block (x[c] = (c[c] - sum_{m<c}
// x[m] L[c][m]) / L[c][c]), column by column: x[C] is final after the
// updates of columns < C, then it updates every later entry with column C of
// L (read from the transposed block, Ltb[C * LT_LD + m] = L[m][C], as 16-byte
// broadcast loads).  The dependency chain is 32 steps long and the updates of
// different entries are independent, where the dot-product order
// (x[C] -= sum over m < C) chains all 496 fused multiply-adds of a row.
// Unrolled by template recursion, so every register index is a constant.
template <int C>
__device__ __forceinline__ void subst32_col(float (&x)[32], const float* Ltb, const float* rdiag) {
  if constexpr (C < 32) {
    x[C] *= rdiag[C];
    const float* col = Ltb + C * LT_LD;
#pragma unroll
    for (int q = (C + 1) / 4; q < 8; ++q) {
      const float4 v = *reinterpret_cast<const float4*>(col + 4 * q);
      const float lv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int m = 4 * q + e;
        if (m > C) x[m] = fmaf(-x[C], lv[e], x[m]);
      }
    }
    subst32_col<C + 1>(x, Ltb, rdiag);
  }
}

__device__ __forceinline__ void subst32_row(float* xs, const float* Ltb, const float* rdiag) {
  float x[32];
#pragma unroll
  for (int m = 0; m < 32; ++m) x[m] = xs[m];
  subst32_col<0>(x, Ltb, rdiag);
#pragma unroll
  for (int m = 0; m < 32; ++m) xs[m] = x[m];
}

// In-place Cholesky of the lower triangle of the 128 x 128 tile in sC:
// 32-wide panels (panel_potrf: all rows of the panel in one column loop),
// 4 x 4 register blocks update the trailing lower triangle.  Panel p of the
// factor (columns 32p .. 32p+31) is final once its column loop is done; it
// is then written to dst (row stride ld; zeros above the diagonal) and
// `progress` is released to p + 1, so the tiles below can start their
// substitution with it while the later panels are factored.  The block's
// writes precede thread 0's release store through the barrier, and the
// release orders them for whoever acquires the count.
//
// Panel jb of the tile goes to dst in fp32 (row stride ld) for the
// substitutions and solves and, when dsts is given, as its TF32 hi/lo split
// (the tile's hi columns in the split matrix, row stride lds) for the
// tensor-core loads; then progress is released to jb / 32 + 1.
__device__ __forceinline__ void publish_panel(const float* sC, float* dst, long long ld, float* dsts, long long lds,
                                              int* progress, int jb) {
  for (int e = threadIdx.x; e < T * 32; e += DAG_THREADS) {
    const int r = e >> 5, c = jb + (e & 31);
    const float x = c <= r ? sC[r * SC_LD + c] : 0.0f;
    dst[(size_t)r * ld + c] = x;
    if (dsts) put_split(dsts + (size_t)r * lds + c, x);
  }
  __syncthreads();
  if (threadIdx.x == 0) st_release(progress, jb / 32 + 1);
}

// Trailing update of the lower triangle of sC by panel jp (columns jp ..
// jp+31 of L, already in sC): C[r][c] -= sum_m L[r][jp+m] L[c][jp+m] for the
// 4 x 4 register blocks with columns c0 in [c_lo, c_hi) and rows r0 >= c0
// (rows up to 127), by `nthr` threads numbered from 0 by `t`.
__device__ __forceinline__ void trail_update(float* sC, int jp, int c_lo, int c_hi, int t, int nthr) {
  const int nbc = (c_hi - c_lo) / 4;                 // column blocks
  const int nbr = (T - c_lo) / 4;                    // row blocks from c_lo
  for (int blk = t; blk < nbr * nbc; blk += nthr) {
    const int br = blk / nbc, bc = blk % nbc;
    const int r0 = c_lo + br * 4, c0 = c_lo + bc * 4;
    if (c0 > r0) continue;
    float acc[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int p = 0; p < 4; ++p) acc[q][p] = 0.0f;
#pragma unroll 8
    for (int m = 0; m < 32; ++m) {
      float a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = sC[(r0 + q) * SC_LD + jp + m];
        b[q] = sC[(c0 + q) * SC_LD + jp + m];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 4; ++p) acc[q][p] = fmaf(a[q], b[p], acc[q][p]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int p = 0; p < 4; ++p) sC[(r0 + q) * SC_LD + c0 + p] -= acc[q][p];
  }
}

// Panel by panel; the trailing update of panel p - 1 is split: its part on
// panel p's columns goes first (all threads), the rest (columns beyond
// panel p) runs on the warps the column loop of panel p leaves idle
// (threads 128 - jb .. 255), at the same time.  Both parts only read
// columns of panel p - 1 and write disjoint entries.
__device__ void potrf_tile(float* sC, float* sbuf, int col0, int* status, float* dst, long long ld, float* dsts,
                           long long lds, int* progress, unsigned long long* pt = nullptr) {
  const int tid = threadIdx.x;
  for (int jb = 0; jb < T; jb += 32) {
    if (pt && tid == 0) pt[(jb / 32) * 3 + 0] = global_ns();
    if (jb > 0) {
      trail_update(sC, jb - 32, jb, jb + 32, tid, DAG_THREADS);
      __syncthreads();
    }
    const int nr = T - jb;
    if (tid < nr)
      panel_potrf(sC, jb, sbuf, col0 + jb, status);
    else if (jb > 0 && jb + 32 < T)
      trail_update(sC, jb - 32, jb + 32, T, tid - nr, DAG_THREADS - nr);
    __syncthreads();
    if (pt && tid == 0) pt[(jb / 32) * 3 + 1] = global_ns();
    publish_panel(sC, dst, ld, dsts, lds, progress, jb);
    if (pt && tid == 0) pt[(jb / 32) * 3 + 2] = global_ns();
  }
}

// X L^T = C in place for the first `rows` rows of sC (a multiple of 4), by
// 32-column blocks: block cb needs panel cb of L (rows cb.., columns
// cb .. cb+31), transposed in sLt (sLt[c * LT_LD + r] = L[r][c]); one thread
// per row solves the block of its row, then 4 x 4 register blocks update the
// remaining columns.  Used on the critical path (the tiles just below the
// diagonal), panel by panel as the diagonal tile publishes them, and for the
// inverse of the diagonal tile.
__device__ void trsm_subst_panel(float* sC, const float* sLt, float* srd, int cb, int rows) {
  const int tid = threadIdx.x;
  if (tid < 32) srd[cb + tid] = __frcp_rn(sLt[(cb + tid) * LT_LD + cb + tid]);
  __syncthreads();
  if (tid < rows) subst32_row(sC + tid * SC_LD + cb, sLt + cb * LT_LD + cb, srd + cb);
  __syncthreads();
}

__device__ void trsm_trail_panel(float* sC, const float* sLt, int cb, int rows) {
  const int tid = threadIdx.x;
  const int rem = T - cb - 32;
  if (rem > 0) {
    const int nbc = rem / 4;   // 4-column groups
    for (int blk = tid; blk < (rows / 4) * nbc; blk += DAG_THREADS) {
      const int r0 = (blk / nbc) * 4, c0 = cb + 32 + (blk % nbc) * 4;
      float acc[4][4];
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 4; ++p) acc[q][p] = 0.0f;
#pragma unroll 8
      for (int m = 0; m < 32; ++m) {
        float a[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) a[q] = sC[(r0 + q) * SC_LD + cb + m];
        const float4 bv = *reinterpret_cast<const float4*>(sLt + (cb + m) * LT_LD + c0);
        const float b[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int p = 0; p < 4; ++p) acc[q][p] = fmaf(a[q], b[p], acc[q][p]);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 4; ++p) sC[(r0 + q) * SC_LD + c0 + p] -= acc[q][p];
    }
    __syncthreads();
  }
}

__device__ void trsm_subst_block(float* sC, const float* sLt, float* srd, int cb, int rows) {
  trsm_subst_panel(sC, sLt, srd, cb, rows);
  trsm_trail_panel(sC, sLt, cb, rows);
}

// Thread 0 waits (an acquire load; the barrier then orders the rest of the
// block after it), everyone learns the value seen (>= target), or 0 when
// the wait gave up.
__device__ __forceinline__ int block_wait_value(const int* flag, int* status, int* s_ok, int target) {
  if (threadIdx.x == 0) *s_ok = wait_flag_value(flag, target, status);
  __syncthreads();
  const int v = *s_ok;
  __syncthreads();
  return v;
}

__device__ __forceinline__ bool block_wait(const int* flag, int* status, int* s_ok, int target = 1) {
  return block_wait_value(flag, status, s_ok, target) >= target;
}

// Per-block tensor-core state, uniform across the block.
struct TcCtx {
  uint32_t tmem;       // running sum in columns RUN_COL.., partial accumulators at PART_COL + 128 pb
  uint32_t g;          // chunks loaded so far by this block (stage g % NST)
  uint32_t kt;         // partials accumulated so far by this block (partial kt % 2)
  uint8_t* stages;     // 1024-aligned stage buffers (unioned with sC, sL)
  uint64_t* full;      // [NST] the stage's tensor loads landed
  uint64_t* empty;     // [NST] the MMAs that read the stage completed
  uint64_t* pfull;     // [2] the MMAs summed in the partial completed
  uint64_t* pfree;     // [2] the partial was added to the running sum (one arrival per drain warp)
};

// Operands of one accumulation acc += sum_{k0 <= k < k1} A_k B_k^T: A_k is
// the 128 x 128 tile of the split matrix behind `amap` at rows arow..,
// logical columns acol + k*T.., B_k likewise.  Chunk c (CHUNK_COLS columns)
// of the loop is k-tile k0 + c / CHUNKS_PER_KT, columns
// (c % CHUNKS_PER_KT) * CHUNK_COLS.
struct TcLoad {
  const void* amap;
  const void* bmap;
  int arow, acol, brow, bcol;
  int k0, nchunks;
  uint32_t base;       // tc.g when the accumulation started
  int issued;          // chunks whose loads were issued (thread 0)
  int ok;              // every dependency wait succeeded (thread 0)
  int kfine;           // k-tile whose dependencies are waited for chunk by chunk (-1: none)
  unsigned long long* kt;   // optional timestamps (thread 0): last k-tile's dependency seen, its 4 chunks landed, drained
};

__device__ __forceinline__ TcLoad tc_load(const void* amap, int arow, int acol, const void* bmap, int brow, int bcol,
                                          int k0, int k1, const TcCtx& tc) {
  TcLoad l;
  l.amap = amap;
  l.bmap = bmap;
  l.arow = arow;
  l.acol = acol;
  l.brow = brow;
  l.bcol = bcol;
  l.k0 = k0;
  l.nchunks = (k1 - k0) * CHUNKS_PER_KT;
  l.base = tc.g;
  l.issued = 0;
  l.ok = 1;
  l.kfine = -1;
  l.kt = nullptr;
  return l;
}

// Thread 0 or 32: issue the loads of chunk `c` (A hi, A lo, B hi, B lo) into
// its stage, after the MMAs of the stage's previous chunk completed and, at
// a k-tile boundary (every chunk of the k-tile l.kfine), after the
// dependencies were published (wait_tile(k-tile, chunk within it)).  A
// dependency wait that gives up still issues the loads (the addresses are
// valid; the result is discarded), so the stage accounting stays
// consistent.  False if a pipeline wait timed out.
template <class WaitTile>
__device__ __forceinline__ bool tc_issue(const TcCtx& tc, TcLoad& l, int c, WaitTile& wait_tile) {
  const uint32_t g = l.base + (uint32_t)c;
  const uint32_t s = g % NST;
  if (g >= NST && !mbar_wait_bounded(tc.empty + s, ((g / NST) - 1u) & 1u, MMA_WAIT_NS)) return false;
  const int kt = l.k0 + c / CHUNKS_PER_KT, q = c % CHUNKS_PER_KT;
  if (q == 0 || kt == l.kfine) {
    if (!wait_tile(kt, q)) l.ok = 0;
    fence_proxy_async_global();
    if (l.kt && c == l.nchunks - CHUNKS_PER_KT) l.kt[0] = global_ns();
  }
  const int col = kt * T + q * CHUNK_COLS;
  const int ax = split_col(l.acol + col), bx = split_col(l.bcol + col);
  uint8_t* stage = tc.stages + s * STAGE_BYTES;
  mbar_arrive_expect_tx(tc.full + s, 4 * CHUNK_BYTES);
  tma_load_2d(stage, l.amap, ax, l.arow, tc.full + s);
  tma_load_2d(stage + CHUNK_BYTES, l.amap, ax + T, l.arow, tc.full + s);
  tma_load_2d(stage + 2 * CHUNK_BYTES, l.bmap, bx, l.brow, tc.full + s);
  tma_load_2d(stage + 3 * CHUNK_BYTES, l.bmap, bx + T, l.brow, tc.full + s);
  l.issued = c + 1;
  return true;
}

// Thread 0: the loads of the first NST - 1 chunks (issued early, e.g.
// before C_init is evaluated, so they land while other work runs).
template <class WaitTile>
__device__ __forceinline__ bool tc_start(const TcCtx& tc, TcLoad& l, WaitTile& wait_tile) {
  for (int c = 0; c < min(NST - 1, l.nchunks); ++c)
    if (!tc_issue(tc, l, c, wait_tile)) return false;
  return true;
}

__device__ __forceinline__ uint64_t sdesc_op(uint32_t saddr) {
  return CHUNK_COLS == 32 ? sdesc_sw128(saddr) : sdesc_sw64(saddr);
}

// Thread 0: the MMAs of one k-chunk into the partial accumulator at
// tensor-memory column `part`, KSTEPS k-steps x (hi lo, lo hi, hi hi), the
// small terms first so they are not lost against the large one (a fourth
// product lo lo changed no measured error).  Both operands come from the
// stage in shared memory.
__device__ __forceinline__ void issue_chunk(const TcCtx& tc, const uint8_t* stage, uint32_t part, bool first) {
  const uint32_t a_hi = smem_u32(stage), a_lo = a_hi + CHUNK_BYTES;
  const uint32_t b_hi = a_hi + 2 * CHUNK_BYTES, b_lo = a_hi + 3 * CHUNK_BYTES;
  const uint32_t d = tc.tmem + part;
#pragma unroll
  for (int ks = 0; ks < KSTEPS; ++ks) {
    const uint32_t o = ks * 32;   // bytes into the swizzled rows
    umma_tf32(d, sdesc_op(a_hi + o), sdesc_op(b_lo + o), IDESC_128x128, (first && ks == 0) ? 0u : 1u);
    umma_tf32(d, sdesc_op(a_lo + o), sdesc_op(b_hi + o), IDESC_128x128, 1u);
    umma_tf32(d, sdesc_op(a_hi + o), sdesc_op(b_hi + o), IDESC_128x128, 1u);
  }
}

// Warps 2..7: add the partial accumulator at tensor-memory column `part`
// to the running sum (or copy it there), each warp its 32-lane quarter of
// the rows (warp w may only reach lanes 32 (w % 4) ..): warps 4 and 5 all
// 128 columns of quarters 0 and 1, warps 2, 6 and 3, 7 half each of
// quarters 2 and 3.  The addition is an ordinary fp32 add (round to
// nearest); the tensor core's own accumulation rounds relative to the
// accumulator's magnitude with a bias, which grows with the number of MMAs
// summed into one accumulator (measured: a relative bias of the diagonal of
// L rising to 2e-5 over 64 tile columns when a whole k-range accumulated in
// place; -1.1e-6 of a 8192-long sum of positive products with one 128-wide
// k-tile per partial), so each partial holds CHUNKS_PER_PART chunks.
__device__ __forceinline__ void fold_partial(const TcCtx& tc, uint32_t part, bool copy) {
  const int warp = threadIdx.x >> 5;
  const uint32_t lanes = (uint32_t)(32 * (warp & 3)) << 16;
  const int c0 = (warp == 4 || warp == 5) ? 0 : (warp >= 6 ? 64 : 0);
  const int nc = (warp == 4 || warp == 5) ? 128 : 64;
  for (int c = c0; c < c0 + nc; c += 32) {
    float pv[32];
    tmem_ld_32x32(tc.tmem + lanes + part + (uint32_t)c, pv);
    if (!copy) {
      float rv[32];
      tmem_ld_32x32(tc.tmem + lanes + RUN_COL + (uint32_t)c, rv);
#pragma unroll
      for (int q = 0; q < 32; ++q) pv[q] += rv[q];
    }
    tmem_st_32x32(tc.tmem + lanes + RUN_COL + (uint32_t)c, pv);
  }
  tmem_wait_st();
}

// The running sum (TMEM columns RUN_COL..) += sum_k A_k B_k^T in 3xTF32; it
// starts from zero unless `preloaded` (e.g. with -C_init).  Thread 0 must
// have called tc_start on `l`, and every thread must have fenced its earlier
// generic writes to the stage buffers (fence_proxy_async_smem) before the
// barrier that preceded it.  Three roles: thread 32 issues the loads of each
// chunk as soon as the MMAs that read its stage have completed (and its
// dependencies are published); thread 0 issues each chunk's MMAs as soon as
// its loads land, into the partial accumulator of its group of
// CHUNKS_PER_PART chunks (alternating between two, each reused once warps
// 2..7 have folded it into the running sum); warps 2..7 fold each partial
// as soon as its MMAs complete.  So loads, MMAs and folds overlap.  Every
// wait is bounded and every loop runs to the end, so each warp takes the
// same number of steps; false when a dependency wait gave up or a pipeline
// wait timed out (the problem is then aborted and the sum is garbage).
template <class WaitTile>
__device__ bool tc_run(TcCtx& tc, TcLoad& l, int* status, WaitTile& wait_tile, bool preloaded) {
  bool bad = false;
  const int n = l.nchunks;   // a multiple of CHUNKS_PER_KT
  const int nparts = n / CHUNKS_PER_PART;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int c = 0; c < n; ++c) {
      const uint32_t g = l.base + (uint32_t)c;
      const uint32_t s = g % NST;
      const int q = c % CHUNKS_PER_PART;
      const uint32_t u = tc.kt + (uint32_t)(c / CHUNKS_PER_PART), pb = u & 1u;
      // partial u's buffer was last used by partial u - 2: wait for its fold
      if (q == 0 && u >= 2 && !mbar_wait_bounded(tc.pfree + pb, ((u - 2u) >> 1) & 1u, MMA_WAIT_NS)) bad = true;
      if (!mbar_wait_bounded(tc.full + s, (g / NST) & 1u, MMA_WAIT_NS)) bad = true;
      if (l.kt && c >= n - 4) l.kt[1 + c - (n - 4)] = global_ns();
      tc_fence_after();
      issue_chunk(tc, tc.stages + s * STAGE_BYTES, PART_COL + 128u * pb, q == 0);
      umma_commit(tc.empty + s);
      if (q == CHUNKS_PER_PART - 1) umma_commit(tc.pfull + pb);
    }
  } else if (threadIdx.x == 32) {
    // the loads of the chunks after the first NST - 1 (issued by tc_start),
    // each as soon as the MMAs that read its stage have completed
    l.issued = min(NST - 1, n);
    for (int c = l.issued; c < n; ++c)
      if (!tc_issue(tc, l, c, wait_tile)) bad = true;
    if (!l.ok) bad = true;
  } else if (warp >= 2) {
    for (int t = 0; t < nparts; ++t) {
      const uint32_t u = tc.kt + (uint32_t)t, pb = u & 1u;
      if (!mbar_wait_bounded(tc.pfull + pb, (u >> 1) & 1u, MMA_WAIT_NS)) bad = true;
      tc_fence_after();
      fold_partial(tc, PART_COL + 128u * pb, !preloaded && t == 0);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(tc.pfree + pb);
    }
  }
  tc.g = l.base + (uint32_t)n;
  tc.kt += (uint32_t)nparts;
  if (threadIdx.x == 0 && !l.ok) bad = true;
  // every MMA has completed once the last partial was folded: the stage
  // buffers are free and the running sum is final
  const bool any_bad = __syncthreads_or(bad) != 0;
  if (any_bad && threadIdx.x == 0) {
    atomicCAS(status + ST_CODE, 0, PGB_ETIMEOUT);
    atomicExch(status + ST_ABORT, 1);
  }
  tc_fence_after();
  if (l.kt && threadIdx.x == 0) l.kt[5] = global_ns();
  return !any_bad;
}

// Store the TMEM accumulator, multiplied by `sign` (+1 or -1), into the
// 128 x 128 shared tile sC (row stride SC_LD); all 8 warps take part.
__device__ __forceinline__ void tmem_to_tile(const TcCtx& tc, float* sC, float sign) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = (w & 3) * 32 + lane;
  const int col0 = (w >> 2) * 64;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float v[32];
    tmem_ld_32x32(tc.tmem + ((uint32_t)((w & 3) * 32) << 16) + (uint32_t)(col0 + 32 * h), v);
#pragma unroll
    for (int q = 0; q < 32; ++q) {
      sC[row * SC_LD + col0 + 32 * h + q] = sign * v[q];
    }
  }
  tc_fence_before();
}

template <int DM>
__device__ void dag_task(const DagJob& jb, int i, int j, TcCtx& tc, int* s_ok, int tidx) {
  unsigned long long* tr = (jb.trace && threadIdx.x == 0) ? jb.trace + (size_t)tidx * 8 : nullptr;
  if (tr) tr[0] = global_ns();
  float* sC = reinterpret_cast<float*>(tc.stages);
  float* sL = sC + T * SC_LD;
  const int nt = jb.nt;
  const long long ld = jb.ld;
  const bool is_rhs = i >= nt;
  const int ri = i - nt;
  // the kind of this right-hand-side row tile and its row tile in its own
  // matrix (RHS_VEC_IDENT: tile 0 is the Newton row, tiles 1.. L^-T rows)
  const bool zrow = is_rhs && jb.rhs_kind == RHS_VEC_IDENT && ri > 0;
  const int rk = !is_rhs ? RHS_NONE : jb.rhs_kind == RHS_VEC_IDENT ? (zrow ? RHS_IDENT : RHS_VEC) : jb.rhs_kind;
  const int rrow = zrow ? ri - 1 : ri;
  const long long lds = 2 * ld;   // row stride of the split matrices
  // fp32 rows (L, and the right-hand-side rows that keep an fp32 copy) and
  // split rows (every tile the tensor cores read later)
  float* rowbase = is_rhs ? ((jb.R && !zrow) ? jb.R + (size_t)rrow * T * ld : nullptr) : jb.L + (size_t)i * T * ld;
  float* rowbase_s = is_rhs ? (zrow ? jb.Zs : jb.Rs) + (size_t)rrow * T * lds : jb.Ls + (size_t)i * T * lds;
  const int k0 = rk == RHS_IDENT ? rrow : 0;
  const bool withheld = jb.withhold == ((i << 16) | j) + 1;
  const bool reused = jb.reuse_mode == 1 && __ldcg(jb.reuse) != 0;
  if (reused && (!is_rhs || (jb.zvalid && __ldcg(jb.zvalid) != 0))) {
    // the resident L tile (and, on the diagonal, its inverse) is already the
    // factor, or the identity rows were solved with it: publish and move on
    __syncthreads();
    if (threadIdx.x == 0 && !withheld) st_release(jb.ready + (size_t)i * nt + j, (!is_rhs && i == j) ? 2 : 1);
    return;
  }

  // operand loads of the first k-chunks go out first (thread 0 waits for
  // their dependencies), then -C_init goes into the accumulator
  const bool have_acc = j > k0;
  const int* ready = jb.ready;
  int* status = jb.status;
  // the diagonal tile takes its last k-tile, the tile just below the
  // previous diagonal, 32 columns at a time as that tile publishes them
  const int kfine = (!is_rhs && i == j && j > 0) ? j - 1 : -1;
  const int* xprog = jb.progress + nt;
  auto wait_tile = [=](int k, int q) {
    if (k == kfine) return wait_flag_geq(xprog + k, (q * CHUNK_COLS) / 32 + 1, status);
    return wait_flag_geq(ready + (size_t)i * nt + k, 1, status) &&
           wait_flag_geq(ready + (size_t)j * nt + k, 1, status);
  };
  const void* rows_map = is_rhs ? (zrow ? jb.tm_Z : jb.tm_R) : jb.tm_L;
  const int row0 = (is_rhs ? rrow : i) * T;
  TcLoad acc_load = tc_load(rows_map, row0, 0, jb.tm_L, j * T, 0, k0, j, tc);
  acc_load.kfine = kfine;
  if (jb.ptrace && (threadIdx.x == 0 || threadIdx.x == 32) && !is_rhs && i <= j + 1) acc_load.kt = jb.ptrace + (size_t)32 * nt + (size_t)(2 * j + (i - j)) * 8;
  if (have_acc && threadIdx.x == 0) {
    fence_tensormap_acquire(rows_map);
    fence_tensormap_acquire(jb.tm_L);
    tc_start(tc, acc_load, wait_tile);
  }
  float* sX = reinterpret_cast<float*>(tc.stages + UNION_BYTES);
  if (!is_rhs || rk == RHS_CROSS) stage_features<DM>(jb, i, j, sX);
  __syncthreads();
  cinit_to_tmem<DM>(jb, i, j, tc.tmem, sX, rk, rrow);
  __syncthreads();
  if (have_acc) {
    if (!tc_run(tc, acc_load, jb.status, wait_tile, true)) return;
  } else {
    tc_fence_after();
  }
  if (tr) tr[1] = global_ns();
  // C = C_init - sum = -(accumulator)
  tmem_to_tile(tc, sC, -1.0f);
  if (tr) tr[6] = global_ns();
  __syncthreads();
  float* dst = rowbase ? rowbase + (size_t)j * T : nullptr;
  float* dsts = rowbase_s + (size_t)split_col(j * T);
  float* Linv_j = jb.Linv + (size_t)j * T * T;
  float* Linvs_j = jb.Linvs + (size_t)j * T * (2 * T);
  if (tr) tr[4] = global_ns();
  if (!is_rhs && i == j) {
    // L_jj = chol(C), published (flag 1) before its inverse (flag 2), so the
    // sub-diagonal tile can start while the inverse is computed
    // (a diagonal tile of L is never a tensor-core operand: no split)
    potrf_tile(sC, sX, j * T, jb.status, dst, ld, nullptr, lds, jb.progress + j,
               jb.ptrace ? jb.ptrace + (size_t)j * 16 : nullptr);
    if (jb.ptrace && threadIdx.x == 0) jb.ptrace[(size_t)j * 16 + 12] = global_ns();
    if (threadIdx.x == 0) {
      if (tr) tr[5] = global_ns();
      __threadfence();
      st_release(jb.ready + (size_t)i * nt + j, 1);
    }
    // L^-1 = X^T with X L^T = I: X = L^-T is upper triangular, so in column
    // block cb only its rows < cb + 32 are nonzero and solved
    for (int e = threadIdx.x; e < T * T; e += DAG_THREADS) {
      const int r = e >> 7, c = e & (T - 1);
      const float l = sC[r * SC_LD + c];
      sL[c * LT_LD + r] = c <= r ? l : 0.0f;   // transposed
      sC[r * SC_LD + c] = r == c ? 1.0f : 0.0f;
    }
    __syncthreads();
    for (int cb = 0; cb < T; cb += 32) trsm_subst_block(sC, sL, sX, cb, cb + 32);
    for (int e = threadIdx.x; e < T * T; e += DAG_THREADS) {
      const int r = e >> 7, c = e & (T - 1);
      const float x = c <= r ? sC[c * SC_LD + r] : 0.0f;
      Linv_j[(size_t)r * T + c] = x;
      put_split(Linvs_j + (size_t)r * (2 * T) + c, x);
    }
  } else if (!is_rhs && i <= j + jb.near) {
    // the tiles just below the diagonal feed the next columns' critical
    // path: substitution with each panel of L_jj as soon as it is
    // published, instead of waiting for L_jj^-1.  The tile just below
    // publishes its own panels as they are solved (progress[nt + j]), for
    // the next diagonal tile's last k-step.
    const float* Ljj = jb.L + (size_t)j * T * ld + (size_t)j * T;
    const bool sub = i == j + 1;
    unsigned long long* sp = (jb.ptrace && threadIdx.x == 0 && sub) ? jb.ptrace + (size_t)(nt + j) * 16 : nullptr;
    int have = 0;   // panels of L_jj known to be published
    for (int cb = 0; cb < T; cb += 32) {
      if (have < cb / 32 + 1) {
        have = block_wait_value(jb.progress + j, jb.status, s_ok + 2, cb / 32 + 1);
        if (have == 0) return;
      }
      if (sp) sp[cb / 8] = global_ns();
      for (int e = threadIdx.x; e < (T - cb) * 32; e += DAG_THREADS) {
        const int r = cb + (e >> 5), c = cb + (e & 31);
        sL[c * LT_LD + r] = __ldcg(Ljj + (size_t)r * ld + c);   // transposed
      }
      __syncthreads();
      if (sp) sp[cb / 8 + 1] = global_ns();
      trsm_subst_panel(sC, sL, sX, cb, T);
      if (sub) {
        for (int e = threadIdx.x; e < T * 32; e += DAG_THREADS) {
          const int r = e >> 5, c = cb + (e & 31);
          const float x = sC[r * SC_LD + c];
          dst[(size_t)r * ld + c] = x;
          put_split(dsts + (size_t)r * lds + c, x);
        }
        __syncthreads();
        if (threadIdx.x == 0) st_release(jb.progress + nt + j, cb / 32 + 1);
      }
      if (sp) sp[cb / 8 + 2] = global_ns();
      trsm_trail_panel(sC, sL, cb, T);
      if (sp) sp[cb / 8 + 3] = global_ns();
    }
    if (!sub) {
      for (int e = threadIdx.x; e < T * T; e += DAG_THREADS) {
        const int r = e >> 7, c = e & (T - 1);
        const float x = sC[r * SC_LD + c];
        dst[(size_t)r * ld + c] = x;
        put_split(dsts + (size_t)r * lds + c, x);
      }
    }
  } else {
    // X = C L_jj^-T = C Linv_jj^T on the tensor cores (C staged through the
    // tile's split, which the result overwrites)
    for (int e = threadIdx.x; e < T * T; e += DAG_THREADS) {
      const int r = e >> 7, c = e & (T - 1);
      put_split(dsts + (size_t)r * lds + c, sC[r * SC_LD + c]);
    }
    fence_proxy_async_global();   // the split is read back by the tensor loads
    fence_proxy_async_smem();     // sC is overwritten by them
    if (!block_wait(jb.ready + (size_t)j * nt + j, jb.status, s_ok + 2, 2)) return;
    if (tr) tr[7] = global_ns();
    auto always = [](int, int) { return true; };
    TcLoad trsm_load = tc_load(rows_map, row0, j * T, jb.tm_Linv, j * T, 0, 0, 1, tc);
    if (threadIdx.x == 0) {
      fence_tensormap_acquire(jb.tm_Linv);
      tc_start(tc, trsm_load, always);
    }
    if (!tc_run(tc, trsm_load, jb.status, always, false)) return;
    if (tr) tr[5] = global_ns();
    tmem_to_tile(tc, sC, 1.0f);
    __syncthreads();
    for (int e = threadIdx.x; e < T * T; e += DAG_THREADS) {
      const int r = e >> 7, c = e & (T - 1);
      const float x = sC[r * SC_LD + c];
      if (dst) dst[(size_t)r * ld + c] = x;
      put_split(dsts + (size_t)r * lds + c, x);
    }
  }
  if (rk == RHS_CROSS && threadIdx.x < T) {
    // predictive variance terms: squared norm of this tile's part of each row
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
  __syncthreads();
  if (threadIdx.x == 0) {
    if (tr) tr[2] = global_ns();
    __threadfence();
    // diagonal tiles: 2 = L_jj and its inverse published; others: 1 = tile ready
    if (!withheld) st_release(jb.ready + (size_t)i * nt + j, (!is_rhs && i == j) ? 2 : 1);
    if (tr) tr[3] = global_ns();
  }
}

// Block set-up of the tensor-core kernels: 1024-aligned stage buffers in the
// dynamic shared memory, NBARS mbarriers, TMEM_COLS tensor-memory columns.
__device__ __forceinline__ TcCtx tc_setup(uint8_t* dsmem, uint64_t* bars, uint32_t* s_tmem) {
  TcCtx tc;
  const uint32_t base = smem_u32(dsmem);
  const uint32_t aligned = (base + 1023u) & ~1023u;
  tc.stages = dsmem + (aligned - base);
  tc.full = bars;
  tc.empty = bars + NST;
  tc.pfull = bars + 2 * NST;
  tc.pfree = bars + 2 * NST + 2;
  tc.g = 0;
  tc.kt = 0;
  if (threadIdx.x < 32) {
    tmem_alloc(s_tmem, TMEM_COLS);
    tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    for (int k = 0; k < NBARS; ++k) mbar_init(bars + k, k >= 2 * NST + 2 ? DRAIN_WARPS : 1);
    fence_mbar_init();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  tc.tmem = *s_tmem;
  return tc;
}

__device__ __forceinline__ void tc_teardown(const TcCtx& tc) {
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) tmem_dealloc(tc.tmem, TMEM_COLS);
}

template <int DM>
__global__ void __launch_bounds__(DAG_THREADS, 1) dag_factor_kernel(const DagJob* __restrict__ jobs,
                                                                    const int4* __restrict__ tasks, int ntasks,
                                                                    int* __restrict__ counter) {
  extern __shared__ uint8_t dsmem[];
  __shared__ int s_task;
  __shared__ int s_ok[4];
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_bars[NBARS];
  TcCtx tc = tc_setup(dsmem, s_bars, &s_tmem);
  while (true) {
    fence_proxy_async_smem();   // this task's shared-memory writes before the next task's tensor loads
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = atomicAdd(counter, 1);
      // tasks of a problem whose abort word is raised are skipped
      if (t < ntasks && ld_relaxed(jobs[tasks[t].x].status + ST_ABORT)) t = -1;
      s_task = t;
    }
    __syncthreads();
    const int t = s_task;
    if (t >= ntasks) break;
    if (t < 0) continue;
    const int4 tk = tasks[t];
    const DagJob jb = jobs[tk.x];
    if (jb.active && __ldcg(jb.active) == 0) continue;           // problem has stopped
    if (jb.reuse_mode == 2 && __ldcg(jb.reuse) != 0) continue;   // solved elsewhere
    if (tk.y >= 0) {
      dag_task<DM>(jb, tk.y, tk.z, tc, s_ok, t);
      continue;
    }
    // a whole small problem: every tile task of the job in column order on
    // this block, so each dependency is already published when it is waited
    // for; stops at the first abort of the problem
    const int nt = jb.nt;
    for (int j = 0; j < nt; ++j) {
      const int nr = jb.rhs_kind == RHS_VEC         ? 1
                     : jb.rhs_kind == RHS_IDENT     ? j + 1
                     : jb.rhs_kind == RHS_VEC_IDENT ? j + 2
                     : jb.rhs_kind == RHS_CROSS     ? jb.nrt
                                                    : 0;
      for (int i = j; i < nt + nr; ++i) {
        __syncthreads();
        if (threadIdx.x == 0) s_task = ld_relaxed(jb.status + ST_ABORT);
        __syncthreads();
        if (s_task) break;
        dag_task<DM>(jb, i, j, tc, s_ok, t);   // i >= nt: right-hand-side row i - nt
        // this task's shared-memory and global writes (its tile of L) before
        // the next task's tensor loads read them
        fence_proxy_async_smem();
        fence_proxy_async_global();
      }
    }
  }
  tc_teardown(tc);
}

// Check kernel: C (128 x 128) = A B^T with A, B 128 x K row-major (K a
// multiple of 128, tensor maps amap / bmap), through the same 3xTF32
// pipeline as the factorisation.
__global__ void __launch_bounds__(DAG_THREADS, 1) tc_tile_check_kernel(const void* amap, const void* bmap, int K,
                                                                       float* __restrict__ C, int* __restrict__ status) {
  extern __shared__ uint8_t dsmem[];
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_bars[NBARS];
  TcCtx tc = tc_setup(dsmem, s_bars, &s_tmem);
  float* sC = reinterpret_cast<float*>(tc.stages);
  auto always = [](int, int) { return true; };
  TcLoad l = tc_load(amap, 0, 0, bmap, 0, 0, 0, K / T, tc);
  if (threadIdx.x == 0) {
    fence_tensormap_acquire(amap);
    fence_tensormap_acquire(bmap);
    tc_start(tc, l, always);
  }
  if (tc_run(tc, l, status, always, false)) {
    tmem_to_tile(tc, sC, 1.0f);
    __syncthreads();
    for (int e = threadIdx.x; e < T * T; e += DAG_THREADS) C[e] = sC[(e >> 7) * SC_LD + (e & (T - 1))];
  }
  tc_teardown(tc);
}

__global__ void syrk_zzt_kernel(const Prob* __restrict__ probs, const int4* __restrict__ tiles, int ntiles,
                                int* __restrict__ counter);
__global__ void sub_rrt_kernel(const void* rmap, int m, int nt, float* __restrict__ C, long long ldc,
                               int* __restrict__ counter, int* __restrict__ status);

void dag_set_attributes() {
  cudaFuncSetAttribute(tc_tile_check_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DAG_SMEM);
  cudaFuncSetAttribute(syrk_zzt_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DAG_SMEM);
  cudaFuncSetAttribute(sub_rrt_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DAG_SMEM);
  cudaFuncSetAttribute(dag_factor_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DAG_SMEM);
  cudaFuncSetAttribute(dag_factor_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DAG_SMEM);
  cudaFuncSetAttribute(dag_factor_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DAG_SMEM);
}

void launch_dag_factor(const DagJob* jobs_dev, const int4* tasks, int ntasks, int* counter, int DM, int grid,
                       cudaStream_t st) {
  if (ntasks <= 0) return;
  if (DM <= 4)
    dag_factor_kernel<4><<<grid, DAG_THREADS, DAG_SMEM, st>>>(jobs_dev, tasks, ntasks, counter);
  else if (DM <= 8)
    dag_factor_kernel<8><<<grid, DAG_THREADS, DAG_SMEM, st>>>(jobs_dev, tasks, ntasks, counter);
  else
    dag_factor_kernel<16><<<grid, DAG_THREADS, DAG_SMEM, st>>>(jobs_dev, tasks, ntasks, counter);
}

// ---------------------------------------------------------------- B^-1 = Z Z^T
// Z = L^-T (upper, stored in the RHS rows of an RHS_IDENT factorisation).
// Tile (I, J), I >= J: sum over k >= I of Z_Ik Z_Jk^T on the tensor cores;
// written to (I, J) and, transposed through shared memory, to (J, I), so
// B^-1 is stored full.  tiles: (problem, I, J, -) of every problem, longest
// k-range first; persistent blocks take them in list order through an
// atomic counter.
__global__ void __launch_bounds__(DAG_THREADS, 1) syrk_zzt_kernel(const Prob* __restrict__ probs,
                                                                  const int4* __restrict__ tiles, int ntiles,
                                                                  int* __restrict__ counter) {
  extern __shared__ uint8_t dsmem[];
  __shared__ int s_task;
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_bars[NBARS];
  TcCtx tc = tc_setup(dsmem, s_bars, &s_tmem);
  float* sC = reinterpret_cast<float*>(tc.stages);
  while (true) {
    fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = atomicAdd(counter, 1);
      // tiles of aborted or inactive problems are skipped (uniformly for the block)
      if (t < ntiles && (ld_relaxed(probs[tiles[t].x].status + ST_ABORT) || *probs[tiles[t].x].active == 0)) t = -1;
      s_task = t;
    }
    __syncthreads();
    const int t = s_task;
    if (t >= ntiles) break;
    if (t < 0) continue;
    const int4 tl = tiles[t];
    const Prob& P = probs[tl.x];
    const int I = tl.y, J = tl.z;
    const long long ld = P.ld;
    float* Binv = P.Binv;
    auto always = [](int, int) { return true; };
    TcLoad l = tc_load(P.tm_Rz, I * T, 0, P.tm_Rz, J * T, 0, I, P.nt, tc);
    if (threadIdx.x == 0) {
      fence_tensormap_acquire(P.tm_Rz);
      tc_start(tc, l, always);
    }
    if (!tc_run(tc, l, P.status, always, false)) continue;   // the problem is aborted
    tmem_to_tile(tc, sC, 1.0f);
    __syncthreads();
    for (int e = threadIdx.x; e < T * T; e += DAG_THREADS) {
      const int r = e >> 7, c = e & (T - 1);
      Binv[(size_t)(I * T + r) * ld + J * T + c] = sC[r * SC_LD + c];
      if (I != J) Binv[(size_t)(J * T + r) * ld + I * T + c] = sC[c * SC_LD + r];
    }
  }
  tc_teardown(tc);
}

// C -= R R^T (predictive covariance: K(Xs, Xs) - V^T V with V^T = R the
// cross-kernel solve rows).  Task t -> lower tile (I, J) of the ceil(m/128)^2
// grid; entries beyond m are not written.
__global__ void __launch_bounds__(DAG_THREADS, 1) sub_rrt_kernel(const void* rmap, int m, int nt,
                                                                 float* __restrict__ C, long long ldc,
                                                                 int* __restrict__ counter, int* __restrict__ status) {
  extern __shared__ uint8_t dsmem[];
  __shared__ int s_task;
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) uint64_t s_bars[NBARS];
  TcCtx tc = tc_setup(dsmem, s_bars, &s_tmem);
  float* sC = reinterpret_cast<float*>(tc.stages);
  const int mt = ceil_div(m, T);
  const int ntiles = mt * (mt + 1) / 2;
  auto always = [](int, int) { return true; };
  while (true) {
    fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) s_task = atomicAdd(counter, 1);
    __syncthreads();
    const int t = s_task;
    if (t >= ntiles) break;
    int I = (int)((sqrtf(8.0f * t + 1.0f) - 1.0f) * 0.5f);
    while (I * (I + 1) / 2 > t) --I;
    while ((I + 1) * (I + 2) / 2 <= t) ++I;
    const int J = t - I * (I + 1) / 2;
    TcLoad l = tc_load(rmap, I * T, 0, rmap, J * T, 0, 0, nt, tc);
    if (threadIdx.x == 0) {
      fence_tensormap_acquire(rmap);
      tc_start(tc, l, always);
    }
    if (!tc_run(tc, l, status, always, false)) continue;
    tmem_to_tile(tc, sC, 1.0f);
    __syncthreads();
    for (int e = threadIdx.x; e < T * T; e += DAG_THREADS) {
      const int r = e >> 7, c = e & (T - 1);
      const int gi = I * T + r, gj = J * T + c;
      if (gi < m && gj < m && (I != J || c <= r)) {
        C[(size_t)gi * ldc + gj] -= sC[r * SC_LD + c];
        if (gi != gj) C[(size_t)gj * ldc + gi] -= sC[r * SC_LD + c];
      }
    }
  }
  tc_teardown(tc);
}

void launch_sub_rrt(const void* rmap, int m, int nt, float* C, long long ldc, int* counter, int* status, int grid,
                    cudaStream_t st) {
  if (m <= 0) return;
  sub_rrt_kernel<<<grid, DAG_THREADS, DAG_SMEM, st>>>(rmap, m, nt, C, ldc, counter, status);
}

void launch_syrk_zzt(const Prob* probs, const int4* tiles, int ntiles, int* counter, int grid, cudaStream_t st) {
  if (ntiles <= 0) return;
  syrk_zzt_kernel<<<grid, DAG_THREADS, DAG_SMEM, st>>>(probs, tiles, ntiles, counter);
}

}  // namespace pgb

namespace pgb {
// The split (TF32 hi/lo per 128-column tile) of a rows x cols fp32 matrix
// (row stride ld; cols a multiple of 128) into dst (row stride 2 cols).
__global__ void split_rows_kernel(const float* __restrict__ src, int rows, int cols, long long ld,
                                  float* __restrict__ dst) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)rows * cols) return;
  const int r = (int)(e / cols), c = (int)(e % cols);
  put_split(dst + (size_t)r * 2 * cols + split_col(c), src[(size_t)r * ld + c]);
}
}  // namespace pgb

// Internal check entry (not part of the public C-ABI): one 128 x 128 tile
// product C = A B^T through the tensor-core pipeline (A, B: 128 x K
// row-major device arrays, split into TF32 hi/lo parts first, as the
// factorisation's epilogues split the tiles they publish).
extern "C" int pgbx_tc_tile_check(const float* A, const float* B, int K, float* C, int* status, void* stream) {
  using namespace pgb;
  if (!A || !B || !C || !status || K <= 0 || K % T) return PGB_EINVAL;
  dag_set_attributes();
  cudaStream_t s = (cudaStream_t)stream;
  float* sp = nullptr;   // split A (T x 2K), then split B
  void* dmaps = nullptr;
  if (cudaMalloc(reinterpret_cast<void**>(&sp), sizeof(float) * 4 * (size_t)T * K) != cudaSuccess) return PGB_ENOMEM;
  if (cudaMalloc(&dmaps, 256) != cudaSuccess) {
    cudaFree(sp);
    return PGB_ENOMEM;
  }
  alignas(64) unsigned char maps[2][128];
  int rc = PGB_OK;
  if (!make_tile_map(maps[0], sp, T, 2LL * K, 2LL * K) ||
      !make_tile_map(maps[1], sp + 2 * (size_t)T * K, T, 2LL * K, 2LL * K))
    rc = PGB_ECUDA;
  if (rc == PGB_OK && cudaMemcpyAsync(dmaps, maps, sizeof(maps), cudaMemcpyHostToDevice, s) != cudaSuccess)
    rc = PGB_ECUDA;
  if (rc == PGB_OK) {
    const int nb = ceil_div(T * K, 256);
    split_rows_kernel<<<nb, 256, 0, s>>>(A, T, K, K, sp);
    split_rows_kernel<<<nb, 256, 0, s>>>(B, T, K, K, sp + 2 * (size_t)T * K);
    tc_tile_check_kernel<<<1, DAG_THREADS, DAG_SMEM, s>>>(dmaps, static_cast<unsigned char*>(dmaps) + 128, K, C,
                                                          status);
    if (cudaGetLastError() != cudaSuccess) rc = PGB_ECUDA;
  }
  cudaStreamSynchronize(s);
  cudaFree(dmaps);
  cudaFree(sp);
  return rc;
}
