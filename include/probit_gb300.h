/*
 * probit_gb300 — C-ABI of the GB300 (sm_103a) Laplace approximate-inference
 * library.  Every entry point replaces one call of the reference package's
 * Python API (bb515/probit); the citation beside each names it (path:line
 * inside the reference project).
 *
 * Conventions
 *  - All array arguments are DEVICE pointers (float32 / int32, C order) on the
 *    current CUDA device unless stated otherwise; nothing is copied to or
 *    from the host except where a function says so.
 *  - Every call is ordered on the caller's stream (`stream`, a cudaStream_t
 *    passed as void*; NULL = legacy default stream).  Calls return as soon as
 *    the work is enqueued, except pgb_gp_status, which synchronises.
 *  - The hyperparameter vector `theta` (float32, device) is laid out as
 *        [ l_0 .. l_{nl-1}, s, sigma_n, b_0 .. b_J ]
 *    nl = desc.n_lengthscales (1 or d); s = signal variance of the kernel;
 *    sigma_n = likelihood noise std; b = the J+1 ordinal cutpoints (probit
 *    likelihoods only; b_0 = -inf, b_J = +inf).  pgb_theta_size gives its
 *    length.  Gradients use the same layout.
 *  - Labels `y`: float32 targets for PGB_LIK_GAUSSIAN, int32 class indices
 *    0..J-1 for the probit likelihoods.
 *  - Return value: PGB_OK or a negative PGB_E* code.  Numerical failures
 *    inside a launch (non-positive pivot, NaN) do not fail the call; they are
 *    recorded in the handle's device status word, read by pgb_gp_status, and
 *    the affected outputs are NaN, as in the reference.
 */
#ifndef PROBIT_GB300_H
#define PROBIT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGB_OK 0
#define PGB_EINVAL (-1)        /* bad argument */
#define PGB_ENOMEM (-2)        /* device allocation failed */
#define PGB_ECUDA (-3)         /* CUDA runtime error */
#define PGB_ENOTPD (-4)        /* B = I + W^1/2 K W^1/2 had a non-positive pivot */
#define PGB_ENAN (-5)          /* NaN met in the Newton iteration */
#define PGB_ETIMEOUT (-6)      /* a device-side wait gave up (bounded spin) */
#define PGB_EUNSUPPORTED (-7)  /* shape outside what the kernels handle */
#define PGB_ESTATE (-8)        /* call order (e.g. predict before a fit) */

#define PGB_KERNEL_EQ 0          /* s * EQ().stretch(l)                 */
#define PGB_KERNEL_MATERN12 1    /* s * Matern12().stretch(l)           */
#define PGB_KERNEL_EQ_PERIODIC 2 /* s * EQ().stretch(l).periodic(period) */

#define PGB_LIK_GAUSSIAN 0       /* log_gaussian_likelihood, utilities.py:60-61 */
#define PGB_LIK_PROBIT 1         /* log_probit_likelihood (+1e-10), utilities.py:56-57 */
#define PGB_LIK_PROBIT_STABLE 2  /* same model, log Z evaluated through erfcx */

#define PGB_MAX_D 16

/* Shape of one GP problem; fixed for the life of a handle. */
typedef struct pgb_desc {
  int32_t n;              /* training points N (1 .. 2^20)                   */
  int32_t d;              /* input dimension D (1 .. PGB_MAX_D; eq_periodic:
                             1 .. PGB_MAX_D / 2, else PGB_EUNSUPPORTED)     */
  int32_t kernel;         /* PGB_KERNEL_*                                    */
  int32_t n_lengthscales; /* 1 (isotropic) or d (ARD)                        */
  float period;           /* period of EQ.periodic(period)                   */
  int32_t likelihood;     /* PGB_LIK_*                                       */
  int32_t j;              /* ordinal classes J (probit; 0 for Gaussian)      */
  float tolerance;        /* Newton stop: ||a_k - a_{k-1}||_2 <= tolerance   */
  int32_t maxiter;        /* at most this many Newton updates (jaxopt: 100)  */
  int32_t flags;          /* reserved, must be 0                             */
} pgb_desc;

/* Opaque GP handle: device workspace plus the resident posterior (a, W, f,
 * the Cholesky factor L of B and, after pgb_value_and_grad, L^-T) of the
 * last fit.  Not thread-safe; one stream at a time. */
typedef struct pgb_gp pgb_gp;

/* Device status word of a handle, returned by pgb_gp_status. */
typedef struct pgb_status {
  int32_t code;        /* 0 or PGB_ENOTPD / PGB_ENAN / PGB_ETIMEOUT          */
  int32_t iterations;  /* Newton updates done by the last fit                */
  int32_t notpd_col;   /* first column of B with a non-positive pivot, or -1 */
  int32_t converged;   /* 1 if ||Δa|| <= tolerance was reached               */
} pgb_status;

/* Library version string. */
const char* pgb_version(void);

/* Message for a PGB_* code. */
const char* pgb_strerror(int code);

/* Number of float32 entries of theta for `desc`, or a negative PGB_E* code. */
int pgb_theta_size(const pgb_desc* desc);

/* Create a handle and its device workspace on the current device.
 * Replaces the set-up in Approximator.__init__ (approximators.py:55-112). */
int pgb_gp_create(const pgb_desc* desc, pgb_gp** out);

/* Release a handle and all its device memory (after its work completed). */
int pgb_gp_destroy(pgb_gp* gp);

/* The descriptor the handle was created with (host copy). */
int pgb_gp_desc(const pgb_gp* gp, pgb_desc* out);

/* Cap the persistent blocks of the handle's launches at max_blocks (0: one
 * per SM, the default).  A server gives large problems a share of the SMs so
 * that the launches of small requests on other streams run beside them
 * instead of waiting for them.  This entry point has no counterpart in the
 * reference. */
int pgb_gp_set_max_blocks(pgb_gp* gp, int32_t max_blocks);

/* Launch tuning of the handle's factorisations (the knob the project's
 * autotuner sets per problem-size bucket; no counterpart in the reference):
 * the number of tiles below each 128 x 128 diagonal tile of L that are
 * solved by substitution with the diagonal tile's panels as they are
 * published (the factorisation's critical path), 1 .. 16; the tiles further
 * down wait for the diagonal tile's inverse and use the tensor cores.
 * 0 restores the built-in rule (3 for factors of 16 or more tiles, else 2).
 * Waits for the device when the depth changes; results agree to rounding
 * across depths. */
int pgb_gp_set_near_depth(pgb_gp* gp, int32_t near_depth);

/* Read the handle's device status word; synchronises `stream` first. */
int pgb_gp_status(pgb_gp* gp, pgb_status* out, void* stream);

/* Kernel matrix K[i, j] = k(X1[i], X2[j]) (n1 x n2, leading dimension ldk).
 * Replaces B.dense(prior(theta)(X1, X2)) (Laplace.py:7; approximators.py:172-174). */
int pgb_gram(const pgb_desc* desc, const float* theta, const float* X1, int32_t n1,
             const float* X2, int32_t n2, float* K, int64_t ldk, void* stream);

/* pgb_gram without any device allocation, for callers that must not
 * allocate while they run (XLA FFI custom calls under JAX's preallocating
 * allocator, work recorded by a framework's stream capture, services that
 * reserve memory at start-up).  This entry point has no counterpart in the
 * reference.  Its scratch is a fixed 4 MiB array inside the library, held by
 * every GPU that loads it: (n1 + n2) * ceil4(F) must not exceed 1,048,576
 * floats, else PGB_EUNSUPPORTED, where F is the kernel's feature count (d;
 * 2d for eq_periodic).  Descriptors are checked as pgb_gram checks them.  All calls share that array, so calls whose
 * work overlaps on the GPU race; order them on one stream.  The first call on
 * a device resolves the array's address and may load device code: make it
 * before any stream capture. */
int pgb_gram_noalloc(const pgb_desc* desc, const float* theta, const float* X1, int32_t n1,
                     const float* X2, int32_t n2, float* K, int64_t ldk, void* stream);

/* Per-point log p(y|f) and its first three derivatives in f (any output may
 * be NULL).  Replaces the jit(vmap(...)) likelihood wrappers of
 * Approximator.__init__ (approximators.py:92-104) over log_probit_likelihood /
 * log_gaussian_likelihood (utilities.py:47-70); d1/d2 are what JAX's grad of
 * them gives. */
int pgb_log_likelihood(const pgb_desc* desc, const float* theta, const float* f,
                       const void* y, int32_t n, float* logp, float* d1, float* d2,
                       float* d3, void* stream);

/* Newton fixed point a* from a = 0.  Replaces LaplaceGP.weight
 * (approximators.py:265-269) with newton_solver (implicit/solvers.py:18-25). */
int pgb_weight(pgb_gp* gp, const float* X, const void* y, const float* theta,
               float* a_out, void* stream);

/* W = -d2 log p(K a) and f = K a for a given weight a.  Replaces
 * LaplaceGP.precision (approximators.py:271-277). */
int pgb_precision(pgb_gp* gp, const float* X, const void* y, const float* theta,
                  const float* a, float* W_out, float* f_out, void* stream);

/* (a*, W) in one call.  Replaces Approximator.approximate_posterior
 * (approximators.py:204-210). */
int pgb_approximate_posterior(pgb_gp* gp, const float* X, const void* y,
                              const float* theta, float* a_out, float* W_out,
                              void* stream);

/* Negative log evidence at the Newton fixed point (one float written to
 * value_out).  Replaces LaplaceGP.objective (approximators.py:248-263) ->
 * objective_LA (implicit/Laplace.py:12-30). */
int pgb_objective(pgb_gp* gp, const float* X, const void* y, const float* theta,
                  float* value_out, void* stream);

/* Negative log evidence and its gradient in theta (pgb_theta_size floats;
 * entries for infinite cutpoints are 0) through the implicit-function
 * theorem at the fixed point.  Replaces Approximator.value_and_grad
 * (approximators.py:132-134) with fixed_point_layer_fwd/bwd
 * (implicit/solvers.py:28-64). */
int pgb_value_and_grad(pgb_gp* gp, const float* X, const void* y, const float* theta,
                       float* value_out, float* grad_out, void* stream);

/* Variational-Bayes fixed point w* from w = 0: w <- (sigma^2 I + K)^-1
 * (K w + sigma d log p(K w)), stopped like pgb_weight (the handle's tolerance
 * and maxiter).  Replaces VBGP.weight (approximators.py:332-334) with fwd_solver
 * (implicit/solvers.py:7-15) over f_VB (implicit/VB.py:4-17).  The posterior
 * precision of VBGP.precision (approximators.py:336-339) is 1 / sigma^2 at
 * every point and its mean K w* (pgb_precision's f_out).  Leaves the factor
 * of I + K / sigma^2 resident (not a Laplace posterior for pgb_predict's
 * reuse_factor). */
int pgb_vb_weight(pgb_gp* gp, const float* X, const void* y, const float* theta,
                  float* w_out, void* stream);

/* The VB objective at the fixed point (one float written to value_out).
 * Replaces VBGP.objective (approximators.py:317-330) -> objective_VB
 * (implicit/VB.py:20-40). */
int pgb_vb_objective(pgb_gp* gp, const float* X, const void* y, const float* theta,
                     float* value_out, void* stream);

/* The VB objective and its gradient in theta (pgb_theta_size floats; entries
 * for infinite cutpoints are 0) through the implicit layer: the adjoint
 * fixed point of fixed_point_layer_bwd (implicit/solvers.py:52-64) over f_VB,
 * solved by the same iteration and stopping rule.  Replaces
 * Approximator.value_and_grad (approximators.py:132-134) for VBGP. */
int pgb_vb_value_and_grad(pgb_gp* gp, const float* X, const void* y, const float* theta,
                          float* value_out, float* grad_out, void* stream);

/* Factor B = I + W^1/2 K W^1/2 at the handle's resident precision W (from
 * its last fit) into the resident L, without any right-hand side.  This is
 * the Cholesky of objective_LA (implicit/Laplace.py:24) on its own, for
 * callers that time or reuse the factorisation. */
int pgb_factor(pgb_gp* gp, void* stream);

/* Predictive mean and variance at m test points Xs (m x d).  W must be the
 * precision the weight a was fitted with.  When `reuse_factor` is nonzero,
 * the handle's resident factor of B from its last fit with the same theta is
 * used (the caller asserts W is that fit's precision); otherwise B is
 * refactored from W.  Replaces Approximator.predict (approximators.py:154-180). */
int pgb_predict(pgb_gp* gp, const float* X, const float* theta, const float* a,
                const float* W, const float* Xs, int32_t m, float* mean_out,
                float* var_out, int32_t reuse_factor, void* stream);

/* pgb_predict followed, in the same launch sequence, by the ordinal
 * predictive distribution of every test point: dist_out (m x J, row-major)
 * holds p(y = j) = Phi((b_{j+1} - mean) / s) - Phi((b_j - mean) / s) with
 * s = sqrt(var + sigma_n^2).  Replaces predict followed by
 * probit_predictive_distributions (utilities.py:232-249).  Probit
 * likelihoods only (else PGB_EINVAL); mean_out and var_out may be NULL. */
int pgb_predict_distributions(pgb_gp* gp, const float* X, const float* theta, const float* a,
                              const float* W, const float* Xs, int32_t m, float* dist_out,
                              float* mean_out, float* var_out, int32_t reuse_factor,
                              void* stream);

/* Ordinal predictive distributions from given predictive means and variances
 * (device arrays of m; dist_out m x J).  Replaces
 * probit_predictive_distributions (utilities.py:232-249). */
int pgb_predictive_distributions(const pgb_desc* desc, const float* theta, const float* mean,
                                 const float* var, int32_t m, float* dist_out, void* stream);

/* Full predictive covariance K(Xs, Xs) - K_*^T (K + W^-1)^-1 K_* (m x m,
 * row-major, leading dimension ldc >= m), with the same factor rules as
 * pgb_predict.  Replaces Approximator.predict_covariance
 * (approximators.py:182-197). */
int pgb_predict_covariance(pgb_gp* gp, const float* X, const float* theta, const float* W,
                           const float* Xs, int32_t m, float* cov_out, int64_t ldc,
                           int32_t reuse_factor, void* stream);

/* ---------------------------------------------------------------- batches
 * Many independent GP problems, each with its own pgb_desc (n, d, kernel,
 * likelihood, J, tolerance, maxiter), evaluated together: every kernel of
 * the path covers all problems in one launch and each problem keeps its own
 * Newton stopping rule.  The reference evaluates many problems by
 * vmap(value_and_grad(objective)) (README.md:238-239,
 * examples/classification.py:489-492); a batch replaces that call for
 * problems of different shapes.
 *
 * Packed inputs and outputs (device, problems in creation order):
 *   X      concatenated row-major (n_b x d_b) blocks            float32
 *   y      concatenated n_b labels                                4 bytes each
 *   theta  concatenated pgb_theta_size(desc_b) blocks            float32
 *   values one negative log evidence per problem                 float32
 *   grads  same layout as theta                                  float32
 * pgb_batch_layout gives the element offsets of each problem's block (count
 * + 1 entries each, the last one the total).  Per-problem numerical failures
 * are recorded in per-problem status words (pgb_batch_status) and give NaN
 * outputs for that problem only. */
typedef struct pgb_batch pgb_batch;

/* Create a batch of `count` problems with one device arena on the current
 * device. */
int pgb_batch_create(const pgb_desc* descs, int32_t count, pgb_batch** out);

/* Release a batch and its device memory (after its work completed). */
int pgb_batch_destroy(pgb_batch* b);

/* pgb_gp_set_near_depth for each problem of a batch (host array of count
 * entries, creation order). */
int pgb_batch_set_near_depth(pgb_batch* b, const int32_t* near_depth);

/* Number of problems of the batch. */
int pgb_batch_size(const pgb_batch* b, int32_t* count);

/* Descriptor of problem `index` (creation order) of the batch. */
int pgb_batch_desc(const pgb_batch* b, int32_t index, pgb_desc* out);

/* Element offsets of each problem's block in the packed X, y and theta
 * (host arrays of count + 1 entries; any may be NULL). */
int pgb_batch_layout(const pgb_batch* b, int64_t* x_offsets, int64_t* y_offsets,
                     int64_t* theta_offsets);

/* Negative log evidence of every problem: LaplaceGP.objective
 * (approximators.py:248-263) under vmap. */
int pgb_batch_objective(pgb_batch* b, const float* X, const void* y, const float* theta,
                        float* values, void* stream);

/* Negative log evidence and its theta gradient of every problem:
 * Approximator.value_and_grad (approximators.py:132-134) under vmap. */
int pgb_batch_value_and_grad(pgb_batch* b, const float* X, const void* y,
                             const float* theta, float* values, float* grads,
                             void* stream);

/* Which problems the following evaluations compute (device int32 array of
 * count entries, 0 = skip; all are enabled after pgb_batch_create).  A
 * skipped problem's values, gradients and status words keep what its last
 * evaluation wrote, and it costs (almost) nothing: an optimiser can
 * re-evaluate only the problems whose line search is still running.  This
 * entry point has no counterpart in the reference. */
int pgb_batch_set_enabled(pgb_batch* b, const int32_t* enabled, void* stream);

/* Per-problem status words (host array of count entries); synchronises
 * `stream` first. */
int pgb_batch_status(pgb_batch* b, pgb_status* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PROBIT_GB300_H */
