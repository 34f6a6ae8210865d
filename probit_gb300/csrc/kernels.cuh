// Launch wrappers of the device kernels (one translation unit each) used by
// the host orchestration in api.cu.
#pragma once

#include "common.cuh"

namespace pgb {

enum RhsKind { RHS_NONE = 0, RHS_VEC = 1, RHS_IDENT = 2, RHS_CROSS = 3 };

// One factorisation job of the tile-DAG kernel (dag.cu).
struct DagJob {
  int n;             // size of B
  int nt;            // tiles per dimension (ceil(n / T))
  long long ld;      // floats per row of L and R
  float* L;          // nt*T rows: lower tiles of the factor
  float* Linv;       // nt tiles of T x T: inverses of the diagonal tiles of L
  int rhs_kind;      // RhsKind
  int nrt;           // RHS tile rows
  int nrhs;          // RHS rows in use
  float* R;          // nrt*T rows: RHS rows, overwritten by the solution
  const float* rhs_vec;  // RHS_VEC: t (n)
  const float* Xq;       // RHS_CROSS: query features (nrhs x Dp)
  float* rowsq;          // RHS_CROSS: per row, per tile column sum of squares (nrhs x nt)
  const float* Xf;       // training features (nt*T x Dp)
  const float* sw;       // sqrt(W) (nt*T, zero padded)
  const float* theta;
  Shape sh;
  int* ready;            // (nt + nrt) x nt tile flags, zeroed before the launch
  int* status;
  // factor reuse: when *reuse is 1 the resident L is already the factor of
  // this B (bitwise equal W, same theta).  reuse_mode 1: skip the L tiles and
  // solve only the RHS rows; 2: skip the whole launch (the caller solves the
  // RHS with the triangular solve instead).
  const int* reuse;
  int reuse_mode;
  // optional per-task timestamps (globaltimer ns): [task][8] = start, k-loop
  // done, tile ready, flag released, epilogue start, L_jj published (diagonal),
  // C assembled (after the accumulator is applied)
  unsigned long long* trace;
  unsigned long long* ptrace;   // optional: [nt][16] phase times of the diagonal factorisations
};

// gram.cu
void launch_prep_features(const Shape& sh, const float* X, const float* theta, float* Xf, int n, int n_pad,
                          cudaStream_t st);
void launch_gram_full(const Shape& sh, const float* theta, const float* X1f, int n1, const float* X2f, int n2,
                      float* K, long long ldk, cudaStream_t st);
void launch_gram_matvec(const Shape& sh, const float* theta, const float* Xr, int nr, const float* Xc, int nc,
                        const float* M, long long ldm, const float* v, const float* row_scale, float* y,
                        cudaStream_t st);
void launch_dense_matvec(const float* A, long long lda, int nr, int nc, const float* v, const float* row_scale,
                         float* y, cudaStream_t st);
void launch_grad_trace(const Shape& sh, const float* theta, const float* Xf, const float* Binv, long long ld,
                       const float* sw, const float* c, const float* a, const int2* tiles, int ntiles, double* part,
                       cudaStream_t st);

// vec.cu
void launch_lik_eval(const Shape& sh, const float* theta, const float* f, const void* y, int n, float* logp,
                     float* d1, float* d2, float* d3, cudaStream_t st);
void launch_newton_lik(const Shape& sh, const float* theta, const float* f, const void* y, const float* a,
                       int n_pad, float* d1, float* W, float* sw, float* r, float* rhs, cudaStream_t st);
void launch_newton_update(int n, const float* sw, const float* x, float* a, double* part, cudaStream_t st);
void launch_newton_finalize(const double* part, int nparts, float tol, int maxiter, int* status, float* err_out,
                            cudaGraphConditionalHandle cond, int use_cond, cudaStream_t st);
void launch_lik_full(const Shape& sh, const float* theta, const float* f, const void* y, int n_pad, float* logp,
                     float* d1, float* d3, float* W, float* sw, cudaStream_t st);
void launch_evidence(int n, const float* logp, const float* f, const float* a, const float* L, long long ld,
                     double* part, float* value, cudaStream_t st);
void launch_grad_vec1(int n, int n_pad, const float* rowdot, const float* sw, const float* d3, const float* a,
                      const float* d1, float* dsig, float* svec, float* r, cudaStream_t st);
void launch_scale_vec(int n, int n_pad, const float* sw, const float* in, float* out, cudaStream_t st);
void launch_grad_vec3(int n, int n_pad, const float* y1, const float* sw, const float* a, const float* d1,
                      const float* svec, const float* W, float* u, float* c, cudaStream_t st);
void launch_grad_lik_final(const Shape& sh, const float* theta, const float* f, const void* y, const float* dsig,
                           const float* u, const double* tpart, int ntp, double* lpart, float* grad,
                           cudaStream_t st);
void launch_predict_var(const Shape& sh, const float* theta, const float* rowsq, int nt, int m, float* var,
                        cudaStream_t st);
void launch_sqrt_w(int n, int n_pad, const float* W, float* sw, cudaStream_t st);
// factor reuse: flags[0] = factor valid, flags[1] = W differs, flags[2] = reuse
void launch_reuse_check(int n, const float* sw, float* sw_prev, int* flags, cudaStream_t st);
void launch_reuse_mark_valid(int* flags, const int* status, cudaStream_t st);

// dag.cu
void dag_set_attributes();
void launch_dag_factor(const DagJob* jobs_dev, const int4* tasks, int ntasks, int* counter, int Dp, int grid,
                       cudaStream_t st);
void launch_syrk_zzt(const float* Z, long long ldz, int nt, const int2* tiles, int ntiles, float* Binv, long long ldb,
                     int* counter, int* status, int grid, cudaStream_t st);

// trsv.cu
void trsv_set_attributes();
// run_if: when non-null the launch does nothing unless *run_if == run_when
void launch_trsv(int n, int nt, long long ld, const float* L, const float* Linv, const float* b, float* x, int trans,
                 int* flags, int* counter, int* status, int grid, const int* run_if, int run_when, cudaStream_t st);

}  // namespace pgb
