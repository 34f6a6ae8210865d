// Device-side problem table and launch wrappers of the kernels (one
// translation unit each) used by the host orchestration in api.cu.
//
// Every kernel works on a batch: a device array of Prob records (one per GP
// problem, each with its own shape and buffers) and a map from thread block
// to (problem, local block).  A single GP is a batch of one.
#pragma once

#include "common.cuh"

namespace pgb {

// RHS_VEC_IDENT: row tile 0 is the Newton right-hand side (RHS_VEC), row
// tiles 1 .. nt the identity rows (RHS_IDENT) of L^-T, solved in the same
// launch as the factor they use.
enum RhsKind { RHS_NONE = 0, RHS_VEC = 1, RHS_IDENT = 2, RHS_CROSS = 3, RHS_VEC_IDENT = 4 };

constexpr int VT = 256;   // points per block of the per-point kernels

// One GP problem: shape, Newton settings and every device buffer it uses.
struct Prob {
  Shape sh;
  int nt;             // tiles per dimension (ceil(n / T))
  int n_pad;          // nt * T
  long long ld;       // floats per row of L, Rz, Binv
  float tol;          // Newton stop: ||a_k - a_{k-1}||_2 <= tol
  int maxiter;
  const float* X;     // inputs (n x D), y (n), theta
  const void* y;
  const float* theta;
  float* Xf;          // features (n_pad x Dp)
  float* L;           // factor of B (n_pad x ld), lower tiles
  float* Linv;        // inverses of the diagonal tiles (nt x T x T)
  float* Rv;          // Newton RHS row tile (T x ld)
  // splits (TF32 hi/lo parts side by side per 128-column tile, row stride
  // 2 ld; see split_col in umma.cuh) of the tiles the tensor cores read
  float* Ls;          // of L (n_pad x 2 ld)
  float* Linvs;       // of Linv (nt T x 2 T)
  float* Rvs;         // of Rv (T x 2 ld)
  float* Rz;          // split of L^-T (n_pad x 2 ld), gradient only
  float* Binv;        // B^-1 (n_pad x ld), gradient only
  // vectors (n_pad each)
  float *a, *f, *d1, *W, *sw, *r, *t, *x, *logp, *d3, *dsig, *svec, *rv, *zbar, *tz, *y2, *u, *c, *rowdot, *sw_prev;
  float* da;             // the last Newton update of a (f follows a by f += K da)
  float* err;         // last ||a_k - a_{k-1}||_2
  float* value;       // negative log evidence
  float* grad;        // theta-sized gradient
  int* status;        // 8 status words
  int* active;        // 1 while this problem takes part in the current phase
                      // (Newton loop: until it stops; later phases: = *enabled)
  const int* enabled; // 0: the problem is skipped by every kernel (outputs kept)
  int* reuse;         // [0] factor valid, [1] W differs, [2] reuse decision
  int* zvalid;        // 1: the split L^-T rows (Rz) were solved with the resident factor
  double* part;       // per-block partial sums (ceil(n_pad / VT))
  double* tpart;      // per-tile trace partials (lower tiles x (MAX_D + 1))
  double* lpart;      // per-block likelihood partials (ceil(n / VT) x (MAX_THETA + 2))
  int* tflags;        // 2 nt flags of the two wavefront solves
  const void* tm_Rz;  // tensor map of the split Rz (128 x 32 fp32 boxes, 128-byte swizzle)
};

// One factorisation job of the tile-DAG kernel (dag.cu).
struct DagJob {
  int n;             // size of B
  int nt;            // tiles per dimension (ceil(n / T))
  long long ld;      // floats per row of L and R
  float* L;          // nt*T rows: lower tiles of the factor
  float* Linv;       // nt tiles of T x T: inverses of the diagonal tiles of L
  float* Ls;         // split of L (row stride 2 ld)
  float* Linvs;      // split of Linv (row stride 2 T)
  int near;          // tiles below each diagonal tile solved by substitution (1 .. kMaxNearDepth)
  int rhs_kind;      // RhsKind
  int nrt;           // RHS tile rows
  int nrhs;          // RHS rows in use
  float* R;          // nrt*T rows: RHS solution in fp32 (NULL: only the split is kept)
  float* Rs;         // split of the RHS solution rows (row stride 2 ld)
  float* Zs;         // RHS_VEC_IDENT: split of the identity rows' solution (L^-T)
  const void* tm_Z;  // RHS_VEC_IDENT: tensor map of Zs
  const int* zvalid; // RHS_IDENT: when 1 (and *reuse), the identity rows are solved already
  const float* rhs_vec;  // RHS_VEC: t (n)
  const float* Xq;       // RHS_CROSS: query features (nrhs x Dp)
  float* rowsq;          // RHS_CROSS: per row, per tile column sum of squares (nrhs x nt)
  const float* Xf;       // training features (nt*T x Dp)
  const float* sw;       // sqrt(W) (nt*T, zero padded)
  const float* theta;
  Shape sh;
  int* ready;            // (nt + nrt) x nt tile flags, zeroed before the launch
  int* progress;         // 2 nt: panels published (0..4) of each diagonal tile, then of the tile
                         // just below it; zeroed with ready
  int* status;
  // factor reuse: when *reuse is 1 the resident L is already the factor of
  // this B (bitwise equal W, same theta).  reuse_mode 1: skip the L tiles and
  // solve only the RHS rows; 2: skip the whole job (the caller solves the
  // RHS with the triangular solve instead).
  const int* reuse;
  int reuse_mode;
  const int* active;     // when non-null and 0 the job is skipped (converged problem)
  // test hook: (i << 16 | j) + 1 of one off-diagonal tile whose ready flag is
  // never released, so the waits for it run out (0: none)
  int withhold;
  // optional per-task timestamps (globaltimer ns): [task][8] = start, k-loop
  // done, tile ready, flag released, epilogue start, L_jj published (diagonal)
  // or tensor-core solve done (other tiles), C assembled (after the
  // accumulator is applied), solve operands staged (tensor-core solves)
  unsigned long long* trace;
  unsigned long long* ptrace;   // optional: [2 nt][16] phase times of the diagonal factorisations, then of the
                                // sub-diagonal substitutions; then [nt][2][8] last k-step times of (j, j), (j+1, j)
  // tensor maps (128 x 32 fp32 boxes, 128-byte swizzle) of the splits of L,
  // of R and of Linv, for the tensor-core operand loads
  const void* tm_L;
  const void* tm_R;
  const void* tm_Linv;
};

// api.cu ----------------------------------------------------------------------
// PGB_OK, or the error code every entry point taking a pgb_desc returns for
// it (PGB_EINVAL for a malformed descriptor, PGB_EUNSUPPORTED for more than
// MAX_D kernel features).
int validate_desc(const pgb_desc* d);

// Tensor map of a row-major fp32 matrix (rows x cols, row stride ld floats)
// with 128-row x CHUNK_COLS-column boxes and the swizzle of that row width,
// the layout the tensor-core operand loads expect.  Host code; false if the
// driver refuses.
bool make_tile_map(void* map128, const float* base, long long rows, long long cols, long long ld);

// gram.cu ---------------------------------------------------------------------
// Features of every problem in the map (vmap: block -> (problem, block)).
void launch_prep_features(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
// Features of one point set (stand-alone use).
void launch_prep_features_raw(const Shape& sh, const float* X, const float* theta, float* Xf, int n, int n_pad,
                              cudaStream_t st);
void launch_gram_full(const Shape& sh, const float* theta, const float* X1f, int n1, const float* X2f, int n2,
                      float* K, long long ldk, cudaStream_t st);

// Vector operands of the batched Gram matvec, named by Prob field.
enum VecField {
  F_A, F_F, F_D1, F_W, F_SW, F_R, F_T, F_X, F_LOGP, F_D3, F_DSIG, F_SVEC, F_RV, F_ZBAR, F_TZ, F_Y2, F_U, F_C,
  F_ROWDOT, F_DA, F_NONE
};
struct MatvecOp {
  int v;            // VecField of the vector
  int row_scale;    // VecField or F_NONE
  int y;            // VecField of the output
  int use_binv;     // multiply K by B^-1 elementwise
  int only_active;  // skip problems whose Newton loop has stopped
  int accumulate;   // y += result instead of y = result
};
// Rows of one Gram-matvec map item (one block): 16 for up to 8 features,
// 8 for 16.  A row's sum does not depend on it (every block sweeps all
// columns in the same order); it sets the grid (n / rows blocks) and the
// feature reloads (each block reads every column's features once).
constexpr int mv_block_rows(int DM) { return DM <= 8 ? 16 : 8; }
// y (+)= row_scale * ((K [o B^-1]) v) for every problem of one (kind, DM)
// group; mvmap: block -> (problem, row block of mv_block_rows(DM) rows).
void launch_gram_matvec(int kind, int DM, const Prob* probs, const int2* mvmap, int nitems, int grid, MatvecOp op,
                        cudaStream_t st);
// Stand-alone Gram matvec over explicit pointers (predict mean).
void launch_gram_matvec_raw(const Shape& sh, const float* theta, const float* Xr, int nr, const float* Xc, int nc,
                            const float* v, float* y, cudaStream_t st);
// y2 = B^-1 tz, 8 rows per block: bmap block -> (problem, row block)
void launch_binv_matvec(const Prob* probs, const int2* bmap, int nitems, int grid, cudaStream_t st);
// trace partials over the lower tiles (problem, I, J, ordinal) of one
// (DM, periodic) group
void launch_grad_trace(int DM, int periodic, const Prob* probs, const int4* tiles, int ntiles, int grid,
                       cudaStream_t st);

// vec.cu ----------------------------------------------------------------------
void launch_lik_eval(const Shape& sh, const float* theta, const float* f, const void* y, int n, float* logp,
                     float* d1, float* d2, float* d3, cudaStream_t st);
void launch_newton_lik(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
void launch_newton_update(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
// per-problem stopping rule; any_active[0] collects whether a problem goes
// on, then becomes the graph condition (use_cond) and is copied to
// any_active[1] for a host-driven loop
void launch_newton_finalize(const Prob* probs, int nprob, int* any_active, cudaGraphConditionalHandle cond,
                            int use_cond, cudaStream_t st);
void launch_lik_full(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
void launch_evidence(const Prob* probs, const int2* vmap, int nblocks, int nprob, cudaStream_t st);
// Variational Bayes (VBGP): B = I + K / sigma^2 (sw = 1 / sigma), so
// sigma^2 I + K = sigma^2 B and the factor of B serves the fixed point and
// the objective.
void launch_vb_setup(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
void launch_vb_mark(const Prob* probs, int nprob, cudaStream_t st);
void launch_vb_rhs(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
void launch_vb_update(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
void launch_vb_post(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
void launch_vb_adj_reset(const Prob* probs, int nprob, cudaStream_t st);
void launch_vb_adj_scale(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
void launch_vb_adj_update(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
void launch_vb_adj_finalize(const Prob* probs, int nprob, int* any_active, cudaGraphConditionalHandle cond,
                            int use_cond, cudaStream_t st);
void launch_vb_grad_vec(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
void launch_vb_grad_lik_final(const Prob* probs, const int2* vmap, int nblocks, int nprob, cudaStream_t st);
void launch_grad_vec1(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
void launch_scale_tz(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
void launch_grad_vec3(const Prob* probs, const int2* vmap, int nblocks, cudaStream_t st);
// likelihood-parameter partials (vmap blocks) and the final theta gradient
// of every problem
void launch_grad_lik_final(const Prob* probs, const int2* vmap, int nblocks, int nprob, cudaStream_t st);
void launch_predict_var(const Shape& sh, const float* theta, const float* rowsq, int nt, int m, float* var,
                        cudaStream_t st);
void launch_sqrt_w(int n, int n_pad, const float* W, float* sw, cudaStream_t st);
// dist (m x J) = ordinal predictive distribution from mean and var
void launch_predictive_dist(const Shape& sh, const float* theta, const float* mean, const float* var, int m,
                            float* dist, cudaStream_t st);
// factor reuse per active problem: differs |= any(sw != sw_prev); decide
void launch_reuse_check(const Prob* probs, const int2* vmap, int nblocks, int nprob, cudaStream_t st);
void launch_reuse_mark_valid(const Prob* probs, int nprob, cudaStream_t st);
// Graph condition = some active problem factors in this Newton step (its
// reuse decision is 0).
void launch_need_factor(const Prob* probs, int nprob, cudaGraphConditionalHandle cond, cudaStream_t st);
// After a Newton-step factorisation whose job solved the identity rows too
// (Gaussian likelihood in an evidence + gradient evaluation): zvalid = 1
// where the factor was computed in this step without error.
void launch_mark_z(const Prob* probs, int nprob, cudaStream_t st);
// enabled problems: status words, reuse flags, active = 1 and (zero_a)
// a = 0; disabled problems: active = 0, nothing else touched
void launch_reset_problems(const Prob* probs, const int2* vmap, int nblocks, int zero_a, cudaStream_t st);
// active = enabled for every problem (the phases after the Newton loop)
void launch_activate_enabled(const Prob* probs, int nprob, cudaStream_t st);

// dag.cu ----------------------------------------------------------------------
void dag_set_attributes();
// DM: feature loop bound (4, 8 or 16), at least every job's Dp
void launch_dag_factor(const DagJob* jobs_dev, const int4* tasks, int ntasks, int* counter, int DM, int grid,
                       cudaStream_t st);
// C (m x m, ldc) -= R R^T for R = rows 0..m of the matrix behind tensor map
// `rmap` (k-range: nt tiles of 128 columns); lower tiles computed, mirrored.
void launch_sub_rrt(const void* rmap, int m, int nt, float* C, long long ldc, int* counter, int* status, int grid,
                    cudaStream_t st);
// B^-1 = Z Z^T over the merged lower-tile list (tiles: problem, I, J, -)
void launch_syrk_zzt(const Prob* probs, const int4* tiles, int ntiles, int* counter, int grid, cudaStream_t st);

// trsv.cu ---------------------------------------------------------------------
void trsv_set_attributes();
// Wavefront solves of every problem in the claim list (problem, position):
// trans = 1: L^T x = w (w = Rv row 0, x = x); trans = 0: L w = t (t, w = Rv
// row 0).  run_on_reuse = 1: only problems whose reuse decision is 1.
void launch_trsv(const Prob* probs, const int2* claims, int nclaims, int trans, int* counter, int run_on_reuse,
                 int only_active, int grid, cudaStream_t st);

}  // namespace pgb
