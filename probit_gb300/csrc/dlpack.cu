// DLPack entry points of include/probit_gb300_dlpack.h: every tensor is
// checked against the handle's descriptor, then the pointer entry point of
// include/probit_gb300.h is called with data + byte_offset.  Host code only.

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/probit_gb300_dlpack.h"

namespace {

constexpr int32_t kDLCPU = 1;
constexpr int32_t kDLCUDA = 2;
constexpr int32_t kDLCUDAManaged = 13;
constexpr int32_t kInt = 0;
constexpr int32_t kFloat = 2;

using Dl = pgb_dltensor;

void* ptr_of(const Dl* t) { return static_cast<char*>(t->data) + t->byte_offset; }

// The tensor's memory is on the current CUDA device.
int check_device(const Dl* t) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return PGB_ECUDA;
  }
  return t->device.device_id == dev ? PGB_OK : PGB_EINVAL;
}

int check(const Dl* t, int32_t code, int32_t bits, std::initializer_list<int64_t> shape) {
  const std::vector<int64_t> s(shape);
  const int rc = pgb_dl_check(t, code, bits, (int32_t)s.size(), s.data(), 0);
  return rc != PGB_OK ? rc : check_device(t);
}

// float32 scalar: shape () or (1,)
int check_scalar(const Dl* t) {
  if (t && t->ndim == 0) return check(t, kFloat, 32, {});
  return check(t, kFloat, 32, {1});
}

int32_t label_code(const pgb_desc& d) { return d.likelihood == PGB_LIK_GAUSSIAN ? kFloat : kInt; }

// X (n, d), y (n,), theta (T,) of a handle
int check_inputs(const pgb_desc& d, const Dl* X, const Dl* y, const Dl* theta) {
  const int nth = pgb_theta_size(&d);
  if (nth < 0) return nth;
  int rc = check(X, kFloat, 32, {d.n, d.d});
  if (rc == PGB_OK && y) rc = check(y, label_code(d), 32, {d.n});
  if (rc == PGB_OK) rc = check(theta, kFloat, 32, {nth});
  return rc;
}

int desc_of(const pgb_gp* gp, pgb_desc* d) { return gp ? pgb_gp_desc(gp, d) : PGB_EINVAL; }

}  // namespace

extern "C" {

int pgb_dl_check(const pgb_dltensor* t, int32_t code, int32_t bits, int32_t ndim, const int64_t* shape,
                 int32_t allow_host) {
  if (!t || !t->data || ndim < 0 || (ndim > 0 && !shape)) return PGB_EINVAL;
  const int32_t dt = t->device.device_type;
  if (!allow_host && dt != kDLCUDA && dt != kDLCUDAManaged) return PGB_EINVAL;
  if (allow_host && dt != kDLCUDA && dt != kDLCUDAManaged && dt != kDLCPU && dt != 3) return PGB_EINVAL;
  if (t->dtype.code != code || t->dtype.bits != bits || t->dtype.lanes != 1) return PGB_EINVAL;
  if (t->ndim != ndim || (ndim > 0 && !t->shape)) return PGB_EINVAL;
  for (int k = 0; k < ndim; ++k) {
    if (t->shape[k] < 0 || (shape[k] >= 0 && t->shape[k] != shape[k])) return PGB_EINVAL;
  }
  if (t->strides) {
    int64_t expect = 1;
    for (int k = ndim - 1; k >= 0; --k) {
      if (t->shape[k] != 1 && t->strides[k] != expect) return PGB_EINVAL;
      expect *= t->shape[k];
    }
  }
  if ((reinterpret_cast<uintptr_t>(ptr_of(t)) & 3u) != 0) return PGB_EINVAL;
  return PGB_OK;
}

int pgb_dl_weight(pgb_gp* gp, const pgb_dltensor* X, const pgb_dltensor* y, const pgb_dltensor* theta,
                  const pgb_dltensor* a_out, void* stream) {
  pgb_desc d;
  int rc = desc_of(gp, &d);
  if (rc == PGB_OK) rc = check_inputs(d, X, y, theta);
  if (rc == PGB_OK) rc = check(a_out, kFloat, 32, {d.n});
  if (rc != PGB_OK) return rc;
  return pgb_weight(gp, static_cast<const float*>(ptr_of(X)), ptr_of(y), static_cast<const float*>(ptr_of(theta)),
                    static_cast<float*>(ptr_of(a_out)), stream);
}

int pgb_dl_approximate_posterior(pgb_gp* gp, const pgb_dltensor* X, const pgb_dltensor* y,
                                 const pgb_dltensor* theta, const pgb_dltensor* a_out,
                                 const pgb_dltensor* W_out, void* stream) {
  pgb_desc d;
  int rc = desc_of(gp, &d);
  if (rc == PGB_OK) rc = check_inputs(d, X, y, theta);
  if (rc == PGB_OK) rc = check(a_out, kFloat, 32, {d.n});
  if (rc == PGB_OK) rc = check(W_out, kFloat, 32, {d.n});
  if (rc != PGB_OK) return rc;
  return pgb_approximate_posterior(gp, static_cast<const float*>(ptr_of(X)), ptr_of(y),
                                   static_cast<const float*>(ptr_of(theta)), static_cast<float*>(ptr_of(a_out)),
                                   static_cast<float*>(ptr_of(W_out)), stream);
}

int pgb_dl_objective(pgb_gp* gp, const pgb_dltensor* X, const pgb_dltensor* y, const pgb_dltensor* theta,
                     const pgb_dltensor* value_out, void* stream) {
  pgb_desc d;
  int rc = desc_of(gp, &d);
  if (rc == PGB_OK) rc = check_inputs(d, X, y, theta);
  if (rc == PGB_OK) rc = check_scalar(value_out);
  if (rc != PGB_OK) return rc;
  return pgb_objective(gp, static_cast<const float*>(ptr_of(X)), ptr_of(y), static_cast<const float*>(ptr_of(theta)),
                       static_cast<float*>(ptr_of(value_out)), stream);
}

int pgb_dl_value_and_grad(pgb_gp* gp, const pgb_dltensor* X, const pgb_dltensor* y, const pgb_dltensor* theta,
                          const pgb_dltensor* value_out, const pgb_dltensor* grad_out, void* stream) {
  pgb_desc d;
  int rc = desc_of(gp, &d);
  if (rc == PGB_OK) rc = check_inputs(d, X, y, theta);
  if (rc == PGB_OK) rc = check_scalar(value_out);
  if (rc == PGB_OK) rc = check(grad_out, kFloat, 32, {pgb_theta_size(&d)});
  if (rc != PGB_OK) return rc;
  return pgb_value_and_grad(gp, static_cast<const float*>(ptr_of(X)), ptr_of(y),
                            static_cast<const float*>(ptr_of(theta)), static_cast<float*>(ptr_of(value_out)),
                            static_cast<float*>(ptr_of(grad_out)), stream);
}

int pgb_dl_vb_value_and_grad(pgb_gp* gp, const pgb_dltensor* X, const pgb_dltensor* y,
                             const pgb_dltensor* theta, const pgb_dltensor* value_out,
                             const pgb_dltensor* grad_out, void* stream) {
  pgb_desc d;
  int rc = desc_of(gp, &d);
  if (rc == PGB_OK) rc = check_inputs(d, X, y, theta);
  if (rc == PGB_OK) rc = check_scalar(value_out);
  if (rc == PGB_OK) rc = check(grad_out, kFloat, 32, {pgb_theta_size(&d)});
  if (rc != PGB_OK) return rc;
  return pgb_vb_value_and_grad(gp, static_cast<const float*>(ptr_of(X)), ptr_of(y),
                               static_cast<const float*>(ptr_of(theta)), static_cast<float*>(ptr_of(value_out)),
                               static_cast<float*>(ptr_of(grad_out)), stream);
}

int pgb_dl_predict(pgb_gp* gp, const pgb_dltensor* X, const pgb_dltensor* theta, const pgb_dltensor* a,
                   const pgb_dltensor* W, const pgb_dltensor* Xs, const pgb_dltensor* mean_out,
                   const pgb_dltensor* var_out, int32_t reuse_factor, void* stream) {
  pgb_desc d;
  int rc = desc_of(gp, &d);
  if (rc == PGB_OK) rc = check_inputs(d, X, nullptr, theta);
  if (rc == PGB_OK) rc = check(a, kFloat, 32, {d.n});
  if (rc == PGB_OK) rc = check(W, kFloat, 32, {d.n});
  if (rc == PGB_OK) rc = check(Xs, kFloat, 32, {-1, d.d});
  if (rc != PGB_OK) return rc;
  const int64_t m = Xs->shape[0];
  if (m < 1 || m > INT32_MAX || (!mean_out && !var_out)) return PGB_EINVAL;
  if (mean_out && (rc = check(mean_out, kFloat, 32, {m})) != PGB_OK) return rc;
  if (var_out && (rc = check(var_out, kFloat, 32, {m})) != PGB_OK) return rc;
  return pgb_predict(gp, static_cast<const float*>(ptr_of(X)), static_cast<const float*>(ptr_of(theta)),
                     static_cast<const float*>(ptr_of(a)), static_cast<const float*>(ptr_of(W)),
                     static_cast<const float*>(ptr_of(Xs)), (int32_t)m,
                     mean_out ? static_cast<float*>(ptr_of(mean_out)) : nullptr,
                     var_out ? static_cast<float*>(ptr_of(var_out)) : nullptr, reuse_factor, stream);
}

int pgb_dl_batch_value_and_grad(pgb_batch* b, const pgb_dltensor* X, const pgb_dltensor* y,
                                const pgb_dltensor* theta, const pgb_dltensor* values,
                                const pgb_dltensor* grads, void* stream) {
  int32_t count = 0;
  int rc = b ? pgb_batch_size(b, &count) : PGB_EINVAL;
  if (rc != PGB_OK) return rc;
  std::vector<int64_t> xo(count + 1), yo(count + 1), to(count + 1);
  if ((rc = pgb_batch_layout(b, xo.data(), yo.data(), to.data())) != PGB_OK) return rc;
  int gaussian = 0;
  for (int32_t p = 0; p < count; ++p) {
    pgb_desc d;
    if ((rc = pgb_batch_desc(b, p, &d)) != PGB_OK) return rc;
    gaussian += d.likelihood == PGB_LIK_GAUSSIAN;
  }
  rc = check(X, kFloat, 32, {xo[count]});
  if (rc == PGB_OK) {
    if (gaussian == count) rc = check(y, kFloat, 32, {yo[count]});
    else if (gaussian == 0) rc = check(y, kInt, 32, {yo[count]});
    else if (check(y, kFloat, 32, {yo[count]}) != PGB_OK) rc = check(y, kInt, 32, {yo[count]});
  }
  if (rc == PGB_OK) rc = check(theta, kFloat, 32, {to[count]});
  if (rc == PGB_OK) rc = check(values, kFloat, 32, {count});
  if (rc == PGB_OK) rc = check(grads, kFloat, 32, {to[count]});
  if (rc != PGB_OK) return rc;
  return pgb_batch_value_and_grad(b, static_cast<const float*>(ptr_of(X)), ptr_of(y),
                                  static_cast<const float*>(ptr_of(theta)), static_cast<float*>(ptr_of(values)),
                                  static_cast<float*>(ptr_of(grads)), stream);
}

}  // extern "C"
