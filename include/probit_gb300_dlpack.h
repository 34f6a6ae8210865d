/*
 * probit_gb300 — DLPack entry points.
 *
 * The same calls as probit_gb300.h, taking DLPack tensors instead of raw
 * pointers, so that JAX arrays (jax.dlpack / the buffers an XLA FFI handler
 * receives), torch tensors and CuPy arrays cross the boundary zero-copy and
 * with their shapes and dtypes checked.  Each entry point checks every tensor
 * (CUDA or CUDA-managed memory on the current device, dtype, shape against
 * the handle's descriptor, compact row-major strides, 4-byte aligned start)
 * and returns PGB_EINVAL on any mismatch before it enqueues anything; it
 * then makes the pointer call named beside it, with data + byte_offset.
 * Ownership does not move: the caller keeps every tensor (and, for a
 * DLManagedTensor, calls its deleter) after the enqueued work completed.
 *
 * Tensor rules (n, d from the handle's pgb_desc; T = pgb_theta_size):
 *   X      float32 (n, d)        Xs  float32 (m, d), m >= 1
 *   y      float32 (n,) for PGB_LIK_GAUSSIAN, int32 (n,) for the probit likelihoods
 *   theta  float32 (T,)          grad_out float32 (T,)
 *   a, W, a_out, W_out           float32 (n,)
 *   value_out                    float32 () or (1,)
 *   mean_out, var_out            float32 (m,), either may be NULL (not both)
 * Strides may be NULL (compact) or the compact row-major strides; a
 * dimension of extent 1 may carry any stride.
 */
#ifndef PROBIT_GB300_DLPACK_H
#define PROBIT_GB300_DLPACK_H

#include <stdint.h>

#include "probit_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* DLPack's DLTensor (dlpack.h, the struct every DLPack version since 0.2
 * keeps; a DLManagedTensor or DLManagedTensorVersioned starts with or holds
 * one as `dl_tensor`).  When dlpack.h was included first its own type is
 * used; otherwise the same layout under the same field names. */
#if defined(DLPACK_VERSION)
typedef DLTensor pgb_dltensor;
#else
typedef struct pgb_dltensor {
  void* data;
  struct {
    int32_t device_type;   /* kDLCPU 1, kDLCUDA 2, kDLCUDAHost 3, kDLCUDAManaged 13 */
    int32_t device_id;
  } device;
  int32_t ndim;
  struct {
    uint8_t code;          /* kDLInt 0, kDLUInt 1, kDLFloat 2 */
    uint8_t bits;
    uint16_t lanes;
  } dtype;
  int64_t* shape;
  int64_t* strides;        /* in elements; NULL = compact row-major */
  uint64_t byte_offset;
} pgb_dltensor;
#endif

/* pgb_weight: LaplaceGP.weight (approximators.py:265-269). */
int pgb_dl_weight(pgb_gp* gp, const pgb_dltensor* X, const pgb_dltensor* y, const pgb_dltensor* theta,
                  const pgb_dltensor* a_out, void* stream);

/* pgb_approximate_posterior: Approximator.approximate_posterior
 * (approximators.py:204-210). */
int pgb_dl_approximate_posterior(pgb_gp* gp, const pgb_dltensor* X, const pgb_dltensor* y,
                                 const pgb_dltensor* theta, const pgb_dltensor* a_out,
                                 const pgb_dltensor* W_out, void* stream);

/* pgb_objective: LaplaceGP.objective (approximators.py:248-263). */
int pgb_dl_objective(pgb_gp* gp, const pgb_dltensor* X, const pgb_dltensor* y, const pgb_dltensor* theta,
                     const pgb_dltensor* value_out, void* stream);

/* pgb_value_and_grad: Approximator.value_and_grad (approximators.py:132-134)
 * over fixed_point_layer (implicit/solvers.py:28-64). */
int pgb_dl_value_and_grad(pgb_gp* gp, const pgb_dltensor* X, const pgb_dltensor* y, const pgb_dltensor* theta,
                          const pgb_dltensor* value_out, const pgb_dltensor* grad_out, void* stream);

/* pgb_vb_value_and_grad: Approximator.value_and_grad (approximators.py:132-134)
 * of VBGP (approximators.py:280-339). */
int pgb_dl_vb_value_and_grad(pgb_gp* gp, const pgb_dltensor* X, const pgb_dltensor* y,
                             const pgb_dltensor* theta, const pgb_dltensor* value_out,
                             const pgb_dltensor* grad_out, void* stream);

/* pgb_predict (m = Xs.shape[0]): Approximator.predict (approximators.py:154-180). */
int pgb_dl_predict(pgb_gp* gp, const pgb_dltensor* X, const pgb_dltensor* theta, const pgb_dltensor* a,
                   const pgb_dltensor* W, const pgb_dltensor* Xs, const pgb_dltensor* mean_out,
                   const pgb_dltensor* var_out, int32_t reuse_factor, void* stream);

/* pgb_batch_value_and_grad: vmap(value_and_grad(objective))
 * (README.md:238-239).  Packed 1-D tensors as pgb_batch_layout gives:
 * X float32 (x_total,), y (y_total,) float32 when every problem is Gaussian,
 * int32 when every problem is probit, either 4-byte type when mixed; theta
 * and grads float32 (theta_total,); values float32 (count,). */
int pgb_dl_batch_value_and_grad(pgb_batch* b, const pgb_dltensor* X, const pgb_dltensor* y,
                                const pgb_dltensor* theta, const pgb_dltensor* values,
                                const pgb_dltensor* grads, void* stream);

/* The check every entry point applies to one tensor, on its own: 0 when t
 * is a compact row-major array of `ndim` dimensions with the given extents
 * (shape[k] < 0: any extent), of type (code, bits), in CUDA or CUDA-managed
 * memory (with allow_host != 0 also host or pinned host memory), with a 4-byte aligned start;
 * else PGB_EINVAL.  The device id is not checked here. */
int pgb_dl_check(const pgb_dltensor* t, int32_t code, int32_t bits, int32_t ndim, const int64_t* shape,
                 int32_t allow_host);

#ifdef __cplusplus
}
#endif

#endif /* PROBIT_GB300_DLPACK_H */
