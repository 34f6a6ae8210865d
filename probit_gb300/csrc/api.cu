// Host orchestration and the extern "C" entry points of include/probit_gb300.h.
//
// A handle owns device workspace for one problem shape.  Each reference
// method becomes one CUDA graph, captured once per handle and replayed:
//   weight      prep -> WHILE(newton step)                       (LaplaceGP.weight)
//   posterior   weight -> precision -> factor of B at the final W (approximate_posterior)
//   objective   posterior + evidence                              (LaplaceGP.objective)
//   value_grad  objective with L^-T + implicit gradient           (value_and_grad)
// The Newton loop is a conditional WHILE node: its last kernel evaluates the
// jaxopt stopping rule on the device and sets the loop condition, so no step
// synchronises with the host.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <climits>
#include <mutex>
#include <vector>

#include "kernels.cuh"

using namespace pgb;

#define PGB_VERSION_STRING "probit_gb300 0.1.0 (sm_103a)"

#define CU_TRY(expr)                                                                    \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess) {                                                            \
      std::fprintf(stderr, "probit_gb300: %s failed: %s (%s:%d)\n", #expr,             \
                   cudaGetErrorString(_e), __FILE__, __LINE__);                         \
      return PGB_ECUDA;                                                                 \
    }                                                                                   \
  } while (0)

namespace {

enum GraphOp { OP_WEIGHT = 0, OP_POSTERIOR = 1, OP_OBJECTIVE = 2, OP_VG = 3, OP_COUNT = 4 };
enum JobSlot { JOB_VEC = 0, JOB_NONE = 1, JOB_IDENT = 2, JOB_CROSS = 3, JOB_COUNT = 4 };

constexpr int kStatusWords = 8;

__global__ void reset_status_kernel(int* status) {
  if (threadIdx.x < kStatusWords) status[threadIdx.x] = 0;
  if (threadIdx.x == 0) status[ST_NOTPD_COL] = INT_MAX;
}

}  // namespace

struct pgb_gp {
  pgb_desc desc;
  Shape sh;
  int n = 0, nt = 0, n_pad = 0, P = 0;
  long long ld = 0;
  int num_sms = 0;
  int device = 0;
  // inputs (copied in per call)
  float* X_in = nullptr;
  void* y_in = nullptr;
  float* theta = nullptr;
  // features and factor
  float* Xf = nullptr;
  float* L = nullptr;
  float* Linv = nullptr;   // inverses of the diagonal tiles of L (nt x T x T)
  float* Rv = nullptr;     // RHS_VEC row tile (T x ld)
  float* Rz = nullptr;     // RHS_IDENT rows (n_pad x ld): L^-T
  float* Binv = nullptr;   // n_pad x ld
  // vectors (n_pad)
  // b holds the Newton residual r = d1 - a, t the right-hand side r / sqrt W
  float *a = nullptr, *f = nullptr, *d1 = nullptr, *W = nullptr, *sw = nullptr, *b = nullptr, *t = nullptr,
        *x = nullptr, *logp = nullptr, *d3 = nullptr, *dsig = nullptr, *svec = nullptr, *rv = nullptr,
        *zbar = nullptr, *tz = nullptr, *y2 = nullptr, *Ky2 = nullptr, *u = nullptr, *c = nullptr,
        *rowdot = nullptr;
  float* sw_prev = nullptr; // sqrt W of the resident factor (bitwise reuse test)
  int* reuse = nullptr;    // [0] factor valid, [1] W differs, [2] reuse decision
  float* scal = nullptr;   // [0] err, [1] value
  float* grad = nullptr;
  int* status = nullptr;
  int* ready = nullptr;    // (2 nt) x nt
  int* counters = nullptr; // [0] dag, [1] trsv (trans), [2] predict dag, [3] trsv (lower)
  int* tflags = nullptr;   // 2 nt: trans solve, lower solve
  double* part = nullptr;
  double* tpart = nullptr;
  double* lpart = nullptr;
  // task lists (device)
  int4* tasks[JOB_COUNT] = {nullptr, nullptr, nullptr, nullptr};
  int ntasks[JOB_COUNT] = {0, 0, 0, 0};
  int2* tiles_lower = nullptr;
  int ntiles_lower = 0;
  DagJob* jobs = nullptr;  // device [JOB_COUNT]
  DagJob hjobs[JOB_COUNT];
  // predict workspace (grown on demand)
  float* Rc = nullptr;
  float* rowsq = nullptr;
  float* Xq = nullptr;
  float* Xq_in = nullptr;
  int* ready_c = nullptr;
  int4* tasks_c = nullptr;
  long long cap_c = 0;     // predict rows allocated
  int m_tasks = -1;
  // graphs
  cudaGraphExec_t gexec[OP_COUNT] = {nullptr, nullptr, nullptr, nullptr};
  cudaStream_t cap_s = nullptr, cap_s2 = nullptr;
  int grad_ready = 0;      // Rz / Binv allocated
  int eager = 0;           // PGB_EAGER=1: launch kernels directly, host-driven Newton loop
  unsigned long long* trace = nullptr;   // PGB_TRACE=1: per-task timestamps of the DAG
  int factor_valid = 0;    // L is the factor of B at the resident W (same theta)
};

namespace {

template <typename Tp>
int dev_alloc(Tp** p, size_t count) {
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(Tp));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return PGB_ENOMEM;
  }
  return PGB_OK;
}

#define ALLOC_TRY(p, n)                   \
  do {                                    \
    int _r = dev_alloc(&(p), (size_t)(n)); \
    if (_r != PGB_OK) return _r;          \
  } while (0)

int validate(const pgb_desc* d) {
  if (!d) return PGB_EINVAL;
  if (d->n < 1 || d->n > (1 << 20)) return PGB_EINVAL;
  if (d->d < 1 || d->d > PGB_MAX_D) return PGB_EINVAL;
  if (d->kernel < PGB_KERNEL_EQ || d->kernel > PGB_KERNEL_EQ_PERIODIC) return PGB_EINVAL;
  if (d->n_lengthscales != 1 && d->n_lengthscales != d->d) return PGB_EINVAL;
  if (d->likelihood < PGB_LIK_GAUSSIAN || d->likelihood > PGB_LIK_PROBIT_STABLE) return PGB_EINVAL;
  if (d->likelihood != PGB_LIK_GAUSSIAN && (d->j < 1 || d->j > 40)) return PGB_EINVAL;
  if (d->kernel == PGB_KERNEL_EQ_PERIODIC && !(d->period > 0.0f)) return PGB_EINVAL;
  if (!(d->tolerance >= 0.0f) || d->maxiter < 1) return PGB_EINVAL;
  if (d->flags != 0) return PGB_EINVAL;
  return PGB_OK;
}

Shape make_shape(const pgb_desc* d) {
  Shape s;
  s.n = d->n;
  s.D = d->d;
  s.Dp = (d->d + 3) / 4 * 4;
  s.kind = d->kernel;
  s.nl = d->n_lengthscales;
  s.lik = d->likelihood;
  s.J = d->likelihood == PGB_LIK_GAUSSIAN ? 0 : d->j;
  s.inv_p = d->kernel == PGB_KERNEL_EQ_PERIODIC ? (float)(1.0 / (double)d->period) : 0.0f;
  return s;
}

std::once_flag g_attr_once;
void setup_attributes() {
  std::call_once(g_attr_once, [] {
    dag_set_attributes();
    trsv_set_attributes();
  });
}

// Column-major topological order of the tile tasks of one factorisation.
std::vector<int4> build_tasks(int job, int nt, int kind, int nrt, bool with_L) {
  std::vector<int4> v;
  for (int j = 0; j < nt; ++j) {
    if (with_L)
      for (int i = j; i < nt; ++i) v.push_back(make_int4(job, i, j, 0));
    if (kind == RHS_VEC) {
      v.push_back(make_int4(job, nt, j, 0));
    } else if (kind == RHS_IDENT) {
      for (int r = 0; r <= j; ++r) v.push_back(make_int4(job, nt + r, j, 0));
    } else if (kind == RHS_CROSS) {
      for (int r = 0; r < nrt; ++r) v.push_back(make_int4(job, nt + r, j, 0));
    }
  }
  return v;
}

int upload_tasks(const std::vector<int4>& v, int4** dst) {
  ALLOC_TRY(*dst, v.size());
  CU_TRY(cudaMemcpy(*dst, v.data(), v.size() * sizeof(int4), cudaMemcpyHostToDevice));
  return PGB_OK;
}

int dag_grid(const pgb_gp* gp, int ntasks) { return std::max(1, std::min(gp->num_sms, ntasks)); }

// ---------------------------------------------------------------- enqueue helpers
void enq_reset_status(pgb_gp* gp, cudaStream_t s) { reset_status_kernel<<<1, 32, 0, s>>>(gp->status); }

void enq_prep(pgb_gp* gp, cudaStream_t s) {
  launch_prep_features(gp->sh, gp->X_in, gp->theta, gp->Xf, gp->n, gp->n_pad, s);
}

void enq_dag(pgb_gp* gp, int job, cudaStream_t s) {
  const int nrt = gp->hjobs[job].nrt;
  cudaMemsetAsync(gp->ready, 0, sizeof(int) * (size_t)(gp->nt + nrt) * gp->nt, s);
  cudaMemsetAsync(gp->counters, 0, sizeof(int), s);
  launch_dag_factor(gp->jobs, gp->tasks[job], gp->ntasks[job], gp->counters, gp->sh.Dp,
                    dag_grid(gp, gp->ntasks[job]), s);
}

void enq_newton_step(pgb_gp* gp, cudaStream_t s, cudaGraphConditionalHandle h, int use_cond) {
  const Shape& sh = gp->sh;
  // f = K a
  launch_gram_matvec(sh, gp->theta, gp->Xf, gp->n, gp->Xf, gp->n, nullptr, 0, gp->a, nullptr, gp->f, s);
  // d1, W, sqrt W, r = d1 - a, t = r / sqrt W
  launch_newton_lik(sh, gp->theta, gp->f, gp->y_in, gp->a, gp->n_pad, gp->d1, gp->W, gp->sw, gp->b, gp->t, s);
  // bitwise-unchanged W keeps the resident factor
  launch_reuse_check(gp->n, gp->sw, gp->sw_prev, gp->reuse, s);
  // new W: L L^T = B and w = L^-1 t in one factorisation (skipped on reuse)
  enq_dag(gp, JOB_VEC, s);
  launch_reuse_mark_valid(gp->reuse, gp->status, s);
  // reused W: w = L^-1 t by the forward wavefront solve (skipped otherwise)
  cudaMemsetAsync(gp->tflags + gp->nt, 0, sizeof(int) * gp->nt, s);
  cudaMemsetAsync(gp->counters + 3, 0, sizeof(int), s);
  launch_trsv(gp->n, gp->nt, gp->ld, gp->L, gp->Linv, gp->t, gp->Rv, 0, gp->tflags + gp->nt, gp->counters + 3, gp->status,
              std::min(gp->nt, gp->num_sms), gp->reuse + 2, 1, s);
  // x = L^-T w
  cudaMemsetAsync(gp->tflags, 0, sizeof(int) * gp->nt, s);
  cudaMemsetAsync(gp->counters + 1, 0, sizeof(int), s);
  launch_trsv(gp->n, gp->nt, gp->ld, gp->L, gp->Linv, gp->Rv, gp->x, 1, gp->tflags, gp->counters + 1, gp->status,
              std::min(gp->nt, gp->num_sms), nullptr, 0, s);
  // a += W^1/2 x, stopping rule
  launch_newton_update(gp->n, gp->sw, gp->x, gp->a, gp->part, s);
  launch_newton_finalize(gp->part, ceil_div(gp->n, 256), gp->desc.tolerance, gp->desc.maxiter, gp->status,
                         gp->scal, h, use_cond, s);
}

void enq_precision(pgb_gp* gp, cudaStream_t s) {
  launch_gram_matvec(gp->sh, gp->theta, gp->Xf, gp->n, gp->Xf, gp->n, nullptr, 0, gp->a, nullptr, gp->f, s);
  launch_lik_full(gp->sh, gp->theta, gp->f, gp->y_in, gp->n_pad, gp->logp, gp->d1, gp->d3, gp->W, gp->sw, s);
}

void enq_grad(pgb_gp* gp, cudaStream_t s) {
  const Shape& sh = gp->sh;
  const int n = gp->n, np = gp->n_pad;
  cudaMemsetAsync(gp->counters + 4, 0, sizeof(int), s);
  launch_syrk_zzt(gp->Rz, gp->ld, gp->nt, gp->tiles_lower, gp->ntiles_lower, gp->Binv, gp->ld, gp->counters + 4,
                  gp->status, std::max(1, std::min(gp->num_sms, gp->ntiles_lower)), s);
  // rowdot_i = sum_j B^-1_ij K_ij sw_j  ->  diag(Sigma)_i = rowdot_i / sw_i
  launch_gram_matvec(sh, gp->theta, gp->Xf, n, gp->Xf, n, gp->Binv, gp->ld, gp->sw, nullptr, gp->rowdot, s);
  launch_grad_vec1(n, np, gp->rowdot, gp->sw, gp->d3, gp->a, gp->d1, gp->dsig, gp->svec, gp->rv, s);
  // zbar = K (a - d1 - s)
  launch_gram_matvec(sh, gp->theta, gp->Xf, n, gp->Xf, n, nullptr, 0, gp->rv, nullptr, gp->zbar, s);
  // u = (I + K W)^-1 zbar = W^-1/2 B^-1 W^1/2 zbar
  launch_scale_vec(n, np, gp->sw, gp->zbar, gp->tz, s);
  launch_dense_matvec(gp->Binv, gp->ld, n, n, gp->tz, nullptr, gp->y2, s);
  launch_grad_vec3(n, np, gp->y2, gp->sw, gp->a, gp->d1, gp->svec, gp->W, gp->u, gp->c, s);
  launch_grad_trace(sh, gp->theta, gp->Xf, gp->Binv, gp->ld, gp->sw, gp->c, gp->a, gp->tiles_lower,
                    gp->ntiles_lower, gp->tpart, s);
  launch_grad_lik_final(sh, gp->theta, gp->f, gp->y_in, gp->dsig, gp->u, gp->tpart, gp->ntiles_lower, gp->lpart,
                        gp->grad, s);
}

int ensure_grad_buffers(pgb_gp* gp) {
  if (gp->grad_ready) return PGB_OK;
  const size_t mat = (size_t)gp->n_pad * gp->ld;
  ALLOC_TRY(gp->Rz, mat);
  ALLOC_TRY(gp->Binv, mat);
  CU_TRY(cudaMemset(gp->Rz, 0, mat * sizeof(float)));
  gp->hjobs[JOB_IDENT].R = gp->Rz;
  CU_TRY(cudaMemcpy(gp->jobs + JOB_IDENT, &gp->hjobs[JOB_IDENT], sizeof(DagJob), cudaMemcpyHostToDevice));
  gp->grad_ready = 1;
  return PGB_OK;
}

void enq_prologue(pgb_gp* gp, cudaStream_t s) {
  enq_reset_status(gp, s);
  enq_prep(gp, s);
  cudaMemsetAsync(gp->a, 0, sizeof(float) * gp->n_pad, s);
  cudaMemsetAsync(gp->reuse, 0, sizeof(int) * 4, s);   // new theta: no resident factor
}

void enq_epilogue(pgb_gp* gp, int op, cudaStream_t s) {
  if (op >= OP_POSTERIOR) {
    enq_precision(gp, s);
    launch_reuse_check(gp->n, gp->sw, gp->sw_prev, gp->reuse, s);
    enq_dag(gp, op == OP_VG ? JOB_IDENT : JOB_NONE, s);
    launch_reuse_mark_valid(gp->reuse, gp->status, s);
    if (op >= OP_OBJECTIVE) launch_evidence(gp->n, gp->logp, gp->f, gp->a, gp->L, gp->ld, gp->part, gp->scal + 1, s);
    if (op == OP_VG) enq_grad(gp, s);
  }
}

// The same work without graphs: kernels launched directly, the Newton loop
// driven from the host (one status read per step).  For profilers that do
// not follow kernels inside conditional graph nodes.
int run_eager(pgb_gp* gp, int op, cudaStream_t s) {
  if (op == OP_VG) {
    int r = ensure_grad_buffers(gp);
    if (r != PGB_OK) return r;
  }
  enq_prologue(gp, s);
  const char* tr = std::getenv("PGB_TRACE");
  const bool trace = tr && tr[0] == '1';
  for (int it = 0; it < gp->desc.maxiter; ++it) {
    enq_newton_step(gp, s, 0, 0);
    int again = 0;
    float err = 0.0f;
    int reuse[4] = {0, 0, 0, 0};
    CU_TRY(cudaMemcpyAsync(&again, gp->status + ST_SPARE0, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (trace) {
      CU_TRY(cudaMemcpyAsync(&err, gp->scal, sizeof(float), cudaMemcpyDeviceToHost, s));
      CU_TRY(cudaMemcpyAsync(reuse, gp->reuse, sizeof(reuse), cudaMemcpyDeviceToHost, s));
    }
    CU_TRY(cudaStreamSynchronize(s));
    if (trace) std::fprintf(stderr, "probit_gb300: newton %d ||delta||=%.6g reuse=%d\n", it + 1, err, reuse[2]);
    if (!again) break;
  }
  enq_epilogue(gp, op, s);
  CU_TRY(cudaGetLastError());
  return PGB_OK;
}

// Capture the graph of one operation.
int build_graph(pgb_gp* gp, int op) {
  if (gp->gexec[op]) return PGB_OK;
  if (op == OP_VG) {
    int r = ensure_grad_buffers(gp);
    if (r != PGB_OK) return r;
  }
  cudaStream_t s = gp->cap_s, s2 = gp->cap_s2;
  cudaGraph_t g = nullptr;
  CU_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
  enq_prologue(gp, s);
  // WHILE node for the Newton loop
  cudaStreamCaptureStatus cs;
  cudaGraph_t cg = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  CU_TRY(cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &ndeps));
  cudaGraphConditionalHandle h;
  CU_TRY(cudaGraphConditionalHandleCreate(&h, cg, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t cnode;
  CU_TRY(cudaGraphAddNode(&cnode, cg, deps, nullptr, ndeps, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CU_TRY(cudaStreamUpdateCaptureDependencies(s, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
  CU_TRY(cudaStreamBeginCaptureToGraph(s2, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  enq_newton_step(gp, s2, h, 1);
  cudaGraph_t body_out = nullptr;
  CU_TRY(cudaStreamEndCapture(s2, &body_out));
  enq_epilogue(gp, op, s);
  CU_TRY(cudaStreamEndCapture(s, &g));
  CU_TRY(cudaGraphInstantiate(&gp->gexec[op], g, 0));
  cudaGraphDestroy(g);
  return PGB_OK;
}

int ingest(pgb_gp* gp, const float* X, const void* y, const float* theta, cudaStream_t s) {
  if (!X || !theta) return PGB_EINVAL;
  CU_TRY(cudaMemcpyAsync(gp->X_in, X, sizeof(float) * (size_t)gp->n * gp->sh.D, cudaMemcpyDeviceToDevice, s));
  CU_TRY(cudaMemcpyAsync(gp->theta, theta, sizeof(float) * gp->P, cudaMemcpyDeviceToDevice, s));
  if (y) CU_TRY(cudaMemcpyAsync(gp->y_in, y, 4 * (size_t)gp->n, cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int run_op(pgb_gp* gp, int op, const float* X, const void* y, const float* theta, cudaStream_t s) {
  if (!y) return PGB_EINVAL;
  if (gp->eager) {
    int r = ingest(gp, X, y, theta, s);
    if (r != PGB_OK) return r;
    r = run_eager(gp, op, s);
    if (r != PGB_OK) return r;
    gp->factor_valid = op >= OP_POSTERIOR;
    return PGB_OK;
  }
  int r = build_graph(gp, op);
  if (r != PGB_OK) return r;
  r = ingest(gp, X, y, theta, s);
  if (r != PGB_OK) return r;
  CU_TRY(cudaGraphLaunch(gp->gexec[op], s));
  gp->factor_valid = op >= OP_POSTERIOR;
  return PGB_OK;
}

}  // namespace

// ==================================================================== C-ABI
extern "C" {

const char* pgb_version(void) { return PGB_VERSION_STRING; }

const char* pgb_strerror(int code) {
  switch (code) {
    case PGB_OK: return "ok";
    case PGB_EINVAL: return "invalid argument";
    case PGB_ENOMEM: return "device allocation failed";
    case PGB_ECUDA: return "CUDA runtime error";
    case PGB_ENOTPD: return "B = I + W^1/2 K W^1/2 is not positive definite";
    case PGB_ENAN: return "NaN in the Newton iteration";
    case PGB_ETIMEOUT: return "device-side wait timed out";
    case PGB_EUNSUPPORTED: return "unsupported shape";
    case PGB_ESTATE: return "operation called out of order";
    default: return "unknown error";
  }
}

int pgb_theta_size(const pgb_desc* desc) {
  int r = validate(desc);
  if (r != PGB_OK) return r;
  return theta_len(desc->n_lengthscales, desc->likelihood, desc->likelihood == PGB_LIK_GAUSSIAN ? 0 : desc->j);
}

int pgb_gp_create(const pgb_desc* desc, pgb_gp** out) {
  if (!out) return PGB_EINVAL;
  *out = nullptr;
  int r = validate(desc);
  if (r != PGB_OK) return r;
  setup_attributes();
  pgb_gp* gp = new pgb_gp();
  gp->desc = *desc;
  gp->sh = make_shape(desc);
  gp->n = desc->n;
  gp->nt = ceil_div(desc->n, T);
  gp->n_pad = gp->nt * T;
  gp->ld = gp->n_pad;
  gp->P = pgb_theta_size(desc);
  CU_TRY(cudaGetDevice(&gp->device));
  CU_TRY(cudaDeviceGetAttribute(&gp->num_sms, cudaDevAttrMultiProcessorCount, gp->device));
  const size_t np = gp->n_pad;
  const size_t mat = np * (size_t)gp->ld;
#define A(p, cnt)                         \
  do {                                    \
    if (dev_alloc(&(p), (cnt)) != PGB_OK) { \
      pgb_gp_destroy(gp);                 \
      return PGB_ENOMEM;                  \
    }                                     \
  } while (0)
  A(gp->X_in, (size_t)gp->n * desc->d);
  {
    int* yy = nullptr;
    A(yy, np);
    gp->y_in = yy;
  }
  A(gp->theta, (size_t)MAX_THETA);
  A(gp->Xf, np * gp->sh.Dp);
  A(gp->L, mat);
  A(gp->Linv, (size_t)gp->nt * T * T);
  A(gp->Rv, (size_t)T * gp->ld);
  float** vecs[] = {&gp->a, &gp->f, &gp->d1, &gp->W, &gp->sw, &gp->b, &gp->t, &gp->x, &gp->logp, &gp->d3,
                    &gp->dsig, &gp->svec, &gp->rv, &gp->zbar, &gp->tz, &gp->y2, &gp->Ky2, &gp->u, &gp->c,
                    &gp->rowdot};
  for (float** v : vecs) A(*v, np);
  A(gp->sw_prev, np);
  A(gp->reuse, 4);
  A(gp->scal, 8);
  A(gp->grad, (size_t)MAX_THETA);
  A(gp->status, kStatusWords);
  A(gp->ready, (size_t)2 * gp->nt * gp->nt);
  A(gp->counters, 8);
  A(gp->tflags, 2 * (size_t)gp->nt);
  A(gp->part, (size_t)ceil_div((int)np, 256) + 8);
  // lower tile pairs
  std::vector<int2> tl;
  for (int I = 0; I < gp->nt; ++I)
    for (int J = 0; J <= I; ++J) tl.push_back(make_int2(I, J));
  gp->ntiles_lower = (int)tl.size();
  A(gp->tiles_lower, tl.size());
  A(gp->tpart, tl.size() * (size_t)(MAX_D + 1));
  A(gp->lpart, (size_t)ceil_div((int)np, 256) * (size_t)(MAX_THETA + 2));
  A(gp->jobs, JOB_COUNT);
#undef A
  CU_TRY(cudaMemcpy(gp->tiles_lower, tl.data(), tl.size() * sizeof(int2), cudaMemcpyHostToDevice));
  CU_TRY(cudaMemset(gp->a, 0, np * sizeof(float)));
  CU_TRY(cudaMemset(gp->Rv, 0, (size_t)T * gp->ld * sizeof(float)));
  CU_TRY(cudaMemset(gp->status, 0, kStatusWords * sizeof(int)));
  CU_TRY(cudaMemset(gp->reuse, 0, 4 * sizeof(int)));
  // jobs
  for (int k = 0; k < JOB_COUNT; ++k) {
    DagJob& j = gp->hjobs[k];
    std::memset(&j, 0, sizeof(j));
    j.n = gp->n;
    j.nt = gp->nt;
    j.ld = gp->ld;
    j.L = gp->L;
    j.Linv = gp->Linv;
    j.Xf = gp->Xf;
    j.sw = gp->sw;
    j.theta = gp->theta;
    j.sh = gp->sh;
    j.ready = gp->ready;
    j.status = gp->status;
    j.reuse = gp->reuse + 2;
    j.reuse_mode = 0;
  }
  gp->hjobs[JOB_VEC].rhs_kind = RHS_VEC;
  gp->hjobs[JOB_VEC].nrt = 1;
  gp->hjobs[JOB_VEC].nrhs = 1;
  gp->hjobs[JOB_VEC].R = gp->Rv;
  gp->hjobs[JOB_VEC].rhs_vec = gp->t;
  gp->hjobs[JOB_VEC].reuse_mode = 2;
  gp->hjobs[JOB_NONE].rhs_kind = RHS_NONE;
  gp->hjobs[JOB_NONE].reuse_mode = 1;
  gp->hjobs[JOB_IDENT].reuse_mode = 1;
  gp->hjobs[JOB_IDENT].rhs_kind = RHS_IDENT;
  gp->hjobs[JOB_IDENT].nrt = gp->nt;
  gp->hjobs[JOB_IDENT].nrhs = gp->n_pad;
  gp->hjobs[JOB_CROSS].rhs_kind = RHS_CROSS;
  CU_TRY(cudaMemcpy(gp->jobs, gp->hjobs, sizeof(gp->hjobs), cudaMemcpyHostToDevice));
  const int kinds[3] = {RHS_VEC, RHS_NONE, RHS_IDENT};
  for (int k = 0; k < 3; ++k) {
    std::vector<int4> v = build_tasks(k, gp->nt, kinds[k], gp->hjobs[k].nrt, true);
    gp->ntasks[k] = (int)v.size();
    int rr = upload_tasks(v, &gp->tasks[k]);
    if (rr != PGB_OK) {
      pgb_gp_destroy(gp);
      return rr;
    }
  }
  {
    const char* e = std::getenv("PGB_EAGER");
    gp->eager = (e && e[0] == '1') ? 1 : 0;
    const char* t = std::getenv("PGB_TRACE");
    if (t && t[0] == '1') {
      size_t mx = 0;
      for (int k = 0; k < JOB_COUNT; ++k) mx = std::max(mx, (size_t)gp->ntasks[k]);
      if (dev_alloc(&gp->trace, mx * 8 + (size_t)gp->nt * 16) == PGB_OK) {
        for (int k = 0; k < JOB_COUNT; ++k) {
          gp->hjobs[k].trace = gp->trace;
          gp->hjobs[k].ptrace = gp->trace + mx * 8;
        }
        CU_TRY(cudaMemcpy(gp->jobs, gp->hjobs, sizeof(gp->hjobs), cudaMemcpyHostToDevice));
      }
    }
  }
  CU_TRY(cudaStreamCreateWithFlags(&gp->cap_s, cudaStreamNonBlocking));
  CU_TRY(cudaStreamCreateWithFlags(&gp->cap_s2, cudaStreamNonBlocking));
  *out = gp;
  return PGB_OK;
}

int pgb_gp_destroy(pgb_gp* gp) {
  if (!gp) return PGB_OK;
  for (int k = 0; k < OP_COUNT; ++k)
    if (gp->gexec[k]) cudaGraphExecDestroy(gp->gexec[k]);
  void* ptrs[] = {gp->trace, gp->Linv, gp->sw_prev, gp->reuse, gp->X_in, gp->y_in, gp->theta, gp->Xf, gp->L, gp->Rv, gp->Rz, gp->Binv, gp->a, gp->f, gp->d1,
                  gp->W, gp->sw, gp->b, gp->t, gp->x, gp->logp, gp->d3, gp->dsig, gp->svec, gp->rv, gp->zbar,
                  gp->tz, gp->y2, gp->Ky2, gp->u, gp->c, gp->rowdot, gp->scal, gp->grad, gp->status, gp->ready,
                  gp->counters, gp->tflags, gp->part, gp->tpart, gp->lpart, gp->tiles_lower, gp->jobs, gp->Rc,
                  gp->rowsq, gp->Xq, gp->Xq_in, gp->ready_c, gp->tasks_c, gp->tasks[0], gp->tasks[1],
                  gp->tasks[2], gp->tasks[3]};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (gp->cap_s) cudaStreamDestroy(gp->cap_s);
  if (gp->cap_s2) cudaStreamDestroy(gp->cap_s2);
  delete gp;
  return PGB_OK;
}

int pgb_gp_status(pgb_gp* gp, pgb_status* out, void* stream) {
  if (!gp || !out) return PGB_EINVAL;
  int h[kStatusWords];
  CU_TRY(cudaMemcpyAsync(h, gp->status, sizeof(h), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  CU_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  out->code = h[ST_CODE];
  out->iterations = h[ST_ITERS];
  out->notpd_col = h[ST_NOTPD_COL] == INT_MAX ? -1 : h[ST_NOTPD_COL];
  out->converged = h[ST_CONVERGED];
  return PGB_OK;
}

int pgb_gram(const pgb_desc* desc, const float* theta, const float* X1, int32_t n1, const float* X2, int32_t n2,
             float* K, int64_t ldk, void* stream) {
  if (validate(desc) != PGB_OK || !theta || !X1 || !X2 || !K || n1 < 0 || n2 < 0 || ldk < n2) return PGB_EINVAL;
  if (n1 == 0 || n2 == 0) return PGB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const Shape sh = make_shape(desc);
  float *f1 = nullptr, *f2 = nullptr;
  CU_TRY(cudaMallocAsync(reinterpret_cast<void**>(&f1), sizeof(float) * (size_t)n1 * sh.Dp, s));
  CU_TRY(cudaMallocAsync(reinterpret_cast<void**>(&f2), sizeof(float) * (size_t)n2 * sh.Dp, s));
  launch_prep_features(sh, X1, theta, f1, n1, n1, s);
  launch_prep_features(sh, X2, theta, f2, n2, n2, s);
  launch_gram_full(sh, theta, f1, n1, f2, n2, K, ldk, s);
  CU_TRY(cudaFreeAsync(f1, s));
  CU_TRY(cudaFreeAsync(f2, s));
  CU_TRY(cudaGetLastError());
  return PGB_OK;
}

int pgb_log_likelihood(const pgb_desc* desc, const float* theta, const float* f, const void* y, int32_t n,
                       float* logp, float* d1, float* d2, float* d3, void* stream) {
  if (validate(desc) != PGB_OK || !theta || !f || !y || n < 0) return PGB_EINVAL;
  if (n == 0) return PGB_OK;
  Shape sh = make_shape(desc);
  sh.n = n;
  launch_lik_eval(sh, theta, f, y, n, logp, d1, d2, d3, (cudaStream_t)stream);
  CU_TRY(cudaGetLastError());
  return PGB_OK;
}

int pgb_weight(pgb_gp* gp, const float* X, const void* y, const float* theta, float* a_out, void* stream) {
  if (!gp || !a_out) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  int r = run_op(gp, OP_WEIGHT, X, y, theta, s);
  if (r != PGB_OK) return r;
  CU_TRY(cudaMemcpyAsync(a_out, gp->a, sizeof(float) * gp->n, cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int pgb_precision(pgb_gp* gp, const float* X, const void* y, const float* theta, const float* a, float* W_out,
                  float* f_out, void* stream) {
  if (!gp || !a || !y) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  int r = ingest(gp, X, y, theta, s);
  if (r != PGB_OK) return r;
  CU_TRY(cudaMemsetAsync(gp->a, 0, sizeof(float) * gp->n_pad, s));
  CU_TRY(cudaMemcpyAsync(gp->a, a, sizeof(float) * gp->n, cudaMemcpyDeviceToDevice, s));
  enq_prep(gp, s);
  enq_precision(gp, s);
  if (W_out) CU_TRY(cudaMemcpyAsync(W_out, gp->W, sizeof(float) * gp->n, cudaMemcpyDeviceToDevice, s));
  if (f_out) CU_TRY(cudaMemcpyAsync(f_out, gp->f, sizeof(float) * gp->n, cudaMemcpyDeviceToDevice, s));
  gp->factor_valid = 0;
  CU_TRY(cudaGetLastError());
  return PGB_OK;
}

int pgb_approximate_posterior(pgb_gp* gp, const float* X, const void* y, const float* theta, float* a_out,
                              float* W_out, void* stream) {
  if (!gp || !a_out || !W_out) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  int r = run_op(gp, OP_POSTERIOR, X, y, theta, s);
  if (r != PGB_OK) return r;
  CU_TRY(cudaMemcpyAsync(a_out, gp->a, sizeof(float) * gp->n, cudaMemcpyDeviceToDevice, s));
  CU_TRY(cudaMemcpyAsync(W_out, gp->W, sizeof(float) * gp->n, cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int pgb_objective(pgb_gp* gp, const float* X, const void* y, const float* theta, float* value_out, void* stream) {
  if (!gp || !value_out) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  int r = run_op(gp, OP_OBJECTIVE, X, y, theta, s);
  if (r != PGB_OK) return r;
  CU_TRY(cudaMemcpyAsync(value_out, gp->scal + 1, sizeof(float), cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int pgb_value_and_grad(pgb_gp* gp, const float* X, const void* y, const float* theta, float* value_out,
                       float* grad_out, void* stream) {
  if (!gp || !value_out || !grad_out) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  int r = run_op(gp, OP_VG, X, y, theta, s);
  if (r != PGB_OK) return r;
  CU_TRY(cudaMemcpyAsync(value_out, gp->scal + 1, sizeof(float), cudaMemcpyDeviceToDevice, s));
  CU_TRY(cudaMemcpyAsync(grad_out, gp->grad, sizeof(float) * gp->P, cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int pgb_factor(pgb_gp* gp, void* stream) {
  if (!gp) return PGB_EINVAL;
  if (!gp->factor_valid) return PGB_ESTATE;
  cudaStream_t s = (cudaStream_t)stream;
  CU_TRY(cudaMemsetAsync(gp->reuse + 2, 0, sizeof(int), s));   // always a full factorisation
  enq_dag(gp, JOB_NONE, s);
  CU_TRY(cudaGetLastError());
  return PGB_OK;
}

int pgb_predict(pgb_gp* gp, const float* X, const float* theta, const float* a, const float* W, const float* Xs,
                int32_t m, float* mean_out, float* var_out, int32_t reuse_factor, void* stream) {
  if (!gp || !X || !theta || !a || !Xs || m < 0 || (!mean_out && !var_out)) return PGB_EINVAL;
  if (m == 0) return PGB_OK;
  if (!reuse_factor && !W) return PGB_EINVAL;
  if (reuse_factor && !gp->factor_valid) return PGB_ESTATE;
  cudaStream_t s = (cudaStream_t)stream;
  const int nt = gp->nt;
  const int mt = ceil_div(m, T);
  const long long mpad = (long long)mt * T;
  // grow the cross-kernel workspace
  if (mpad > gp->cap_c) {
    CU_TRY(cudaStreamSynchronize(s));
    float* ptrs[] = {gp->Rc, gp->rowsq, gp->Xq, gp->Xq_in};
    for (float* p : ptrs)
      if (p) cudaFree(p);
    if (gp->ready_c) cudaFree(gp->ready_c);
    gp->Rc = gp->rowsq = gp->Xq = gp->Xq_in = nullptr;
    gp->ready_c = nullptr;
    ALLOC_TRY(gp->Rc, (size_t)mpad * gp->ld);
    ALLOC_TRY(gp->rowsq, (size_t)mpad * nt);
    ALLOC_TRY(gp->Xq, (size_t)mpad * gp->sh.Dp);
    ALLOC_TRY(gp->Xq_in, (size_t)mpad * gp->sh.D);
    ALLOC_TRY(gp->ready_c, (size_t)(nt + mt) * nt);
    gp->cap_c = mpad;
  }
  if (gp->m_tasks != mt) {
    if (gp->tasks_c) {
      CU_TRY(cudaStreamSynchronize(s));
      cudaFree(gp->tasks_c);
      gp->tasks_c = nullptr;
    }
    std::vector<int4> v = build_tasks(JOB_CROSS, nt, RHS_CROSS, mt, false);
    int r = upload_tasks(v, &gp->tasks_c);
    if (r != PGB_OK) return r;
    gp->ntasks[JOB_CROSS] = (int)v.size();
    gp->m_tasks = mt;
  }
  const Shape& sh = gp->sh;
  if (!reuse_factor) {
    int r = ingest(gp, X, nullptr, theta, s);
    if (r != PGB_OK) return r;
    enq_reset_status(gp, s);
    enq_prep(gp, s);
    launch_sqrt_w(gp->n, gp->n_pad, W, gp->sw, s);
    CU_TRY(cudaMemsetAsync(gp->reuse, 0, sizeof(int) * 4, s));   // factor of the caller's W, not reusable
    enq_dag(gp, JOB_NONE, s);
    gp->factor_valid = 0;
  } else {
    int r = ingest(gp, X, nullptr, theta, s);
    if (r != PGB_OK) return r;
    enq_prep(gp, s);
  }
  CU_TRY(cudaMemcpyAsync(gp->Xq_in, Xs, sizeof(float) * (size_t)m * sh.D, cudaMemcpyDeviceToDevice, s));
  launch_prep_features(sh, gp->Xq_in, gp->theta, gp->Xq, m, (int)mpad, s);
  if (mean_out)
    launch_gram_matvec(sh, gp->theta, gp->Xq, m, gp->Xf, gp->n, nullptr, 0, a, nullptr, mean_out, s);
  if (var_out) {
    DagJob jb = gp->hjobs[JOB_CROSS];
    jb.nrt = mt;
    jb.nrhs = m;
    jb.R = gp->Rc;
    jb.Xq = gp->Xq;
    jb.rowsq = gp->rowsq;
    jb.ready = gp->ready_c;
    CU_TRY(cudaMemcpyAsync(gp->jobs + JOB_CROSS, &jb, sizeof(DagJob), cudaMemcpyHostToDevice, s));
    // L tiles are done: mark them ready; RHS tiles start unready
    CU_TRY(cudaMemsetAsync(gp->ready_c, 1, sizeof(int) * (size_t)nt * nt, s));
    CU_TRY(cudaMemsetAsync(gp->ready_c + (size_t)nt * nt, 0, sizeof(int) * (size_t)mt * nt, s));
    CU_TRY(cudaMemsetAsync(gp->counters + 2, 0, sizeof(int), s));
    launch_dag_factor(gp->jobs, gp->tasks_c, gp->ntasks[JOB_CROSS], gp->counters + 2, sh.Dp,
                      dag_grid(gp, gp->ntasks[JOB_CROSS]), s);
    launch_predict_var(sh, gp->theta, gp->rowsq, nt, m, var_out, s);
  }
  CU_TRY(cudaGetLastError());
  return PGB_OK;
}

// Internal diagnostic entry (not part of the public C-ABI): device pointer of
// one of a handle's intermediate buffers, for the test suite.
void* pgbx_gp_buffer(pgb_gp* gp, const char* name) {
  if (!gp || !name) return nullptr;
  struct Item { const char* n; void* p; };
  const Item items[] = {{"a", gp->a}, {"f", gp->f}, {"d1", gp->d1}, {"W", gp->W}, {"sw", gp->sw}, {"d3", gp->d3},
                        {"dsig", gp->dsig}, {"svec", gp->svec}, {"zbar", gp->zbar}, {"u", gp->u}, {"c", gp->c},
                        {"rowdot", gp->rowdot}, {"L", gp->L}, {"Linv", gp->Linv}, {"Rz", gp->Rz}, {"Binv", gp->Binv},
                        {"logp", gp->logp}, {"grad", gp->grad}, {"scal", gp->scal}, {"reuse", gp->reuse},
                        {"trace", gp->trace}, {"tasks_none", gp->tasks[JOB_NONE]},
                        {"ptrace", gp->hjobs[JOB_NONE].ptrace}};
  for (const Item& it : items)
    if (std::strcmp(it.n, name) == 0) return it.p;
  return nullptr;
}

}  // extern "C"
