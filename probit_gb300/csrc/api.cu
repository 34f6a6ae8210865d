// Host orchestration and the extern "C" entry points of include/probit_gb300.h.
//
// One engine serves any number of independent GP problems (a batch; a single
// GP handle is a batch of one).  Every kernel of the path covers all problems
// of the batch in one launch: per-point and matvec kernels through maps from
// thread block to (problem, local block), the factorisations through one
// merged task list over every problem's tile DAG, the triangular solves
// through one merged claim list.  Each reference method becomes one CUDA
// graph, captured once per engine and replayed:
//   weight      prep -> WHILE(newton step)                       (LaplaceGP.weight)
//   posterior   weight -> precision -> factor of B at the final W (approximate_posterior)
//   objective   posterior + evidence                              (LaplaceGP.objective)
//   value_grad  objective with L^-T + implicit gradient           (value_and_grad)
// The Newton loop is a conditional WHILE node: its last kernels evaluate the
// jaxopt stopping rule of every problem on the device and keep the loop
// going while any problem is still iterating; problems that stopped are
// skipped by every kernel of the step.  No step synchronises with the host.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <vector>

#include "kernels.cuh"

using namespace pgb;

#define PGB_VERSION_STRING "probit_gb300 0.2.0 (sm_103a)"

#define CU_TRY(expr)                                                                    \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess) {                                                            \
      std::fprintf(stderr, "probit_gb300: %s failed: %s (%s:%d)\n", #expr,             \
                   cudaGetErrorString(_e), __FILE__, __LINE__);                         \
      return PGB_ECUDA;                                                                 \
    }                                                                                   \
  } while (0)

#define PGB_TRY(expr)          \
  do {                         \
    int _r = (expr);           \
    if (_r != PGB_OK) return _r; \
  } while (0)

// Descriptor check shared by every entry point that takes a pgb_desc
// (declared in kernels.cuh; pgb_gram_noalloc uses it too).
namespace pgb {
int validate_desc(const pgb_desc* d) {
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
  if (feature_count(d) > MAX_D) return PGB_EUNSUPPORTED;   // eq_periodic: 2 features per input dimension
  return PGB_OK;
}
}  // namespace pgb

namespace {

enum GraphOp {
  OP_WEIGHT = 0, OP_POSTERIOR = 1, OP_OBJECTIVE = 2, OP_VG = 3,   // Laplace
  OP_VB_WEIGHT = 4, OP_VB_OBJECTIVE = 5, OP_VB_VG = 6,          // Variational Bayes
  OP_COUNT = 7
};
bool is_vb(int op) { return op == OP_VB_WEIGHT || op == OP_VB_OBJECTIVE || op == OP_VB_VG; }
bool needs_grad_buffers(int op) { return op == OP_VG || op == OP_VB_VG; }
enum JobSlot { JOB_VEC = 0, JOB_NONE = 1, JOB_IDENT = 2, JOB_CROSS = 3, JOB_VEC_IDENT = 4, JOB_COUNT = 5 };
// Merged task lists: Newton step, factor only, factor with L^-T, and the
// Newton step of an evidence + gradient evaluation (problems with a Gaussian
// likelihood solve their L^-T rows with the factor of the first step, which
// is final since W does not change).
enum TaskList { TL_STEP = 0, TL_NONE = 1, TL_IDENT = 2, TL_VG_STEP = 3, TL_COUNT = 4 };
constexpr int kZLag = 4;
enum Counter { C_DAG = 0, C_TRSV_T = 1, C_PREDICT = 2, C_TRSV_L = 3, C_SYRK = 4, C_COUNT = 8 };

constexpr int kStatusWords = 8;

// Bump allocator over one device allocation (256-byte aligned pieces).  Run
// once with base 0 to size the arena, then with the real base.
struct Bump {
  uintptr_t base = 0;
  size_t off = 0;
  template <class Tp>
  Tp* take(size_t count) {
    off = (off + 255) & ~(size_t)255;
    Tp* p = reinterpret_cast<Tp*>(base + off);
    off += std::max<size_t>(count, 1) * sizeof(Tp);
    return p;
  }
};

int dm_of(int Dp) { return Dp <= 4 ? 4 : (Dp <= 8 ? 8 : 16); }

// Device memory of a handle comes from the stream-ordered allocator on the
// handle's private stream: freeing it never synchronises the device (a
// cudaFree would wait for every stream, stalling other requests in a server).
int ws_alloc(cudaStream_t s, void** p, size_t bytes) {
  if (cudaMallocAsync(p, std::max<size_t>(bytes, 256), s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return PGB_ENOMEM;
  }
  return PGB_OK;
}

void ws_free(cudaStream_t s, void* p) {
  if (p) cudaFreeAsync(p, s);
}

struct MvGroup {
  int kind, DM;
  std::vector<int2> h;
  int2* map = nullptr;
};
struct TraceGroup {
  int DM, periodic;
  std::vector<int4> h;
  int4* tiles = nullptr;
};

// Device state of a batch of problems.
struct Engine {
  int nprob = 0;
  std::vector<pgb_desc> desc;
  std::vector<Shape> sh;
  std::vector<int> nt, th;                 // tiles per dimension, theta size
  std::vector<int> near;                   // near band depth of each problem's factorisations
  std::vector<int> rank;                   // position of each problem in the size order (largest first)
  int whole_max = kWholeMaxTiles;          // problems of at most this many tile rows: one block each
  std::vector<size_t> x_off, y_off, th_off;   // offsets (elements) into the packed inputs
  size_t x_total = 0, y_total = 0, th_total = 0;
  int num_sms = 0, device = 0, dag_dm = 4, nt_max = 1;
  int max_blocks = 0;                      // cap on persistent blocks per launch (0: one per SM)
  std::vector<Prob> hp;                    // host copy of the problem table
  Prob* probs = nullptr;
  void* arena = nullptr;                   // everything but the gradient matrices
  void* garena = nullptr;                  // L^-T and B^-1 of every problem
  float* X_all = nullptr;
  void* y_all = nullptr;
  float* theta_all = nullptr;
  float* value_all = nullptr;
  float* err_all = nullptr;
  float* grad_all = nullptr;
  int* status_all = nullptr;
  int* active_all = nullptr;
  int* enabled_all = nullptr;
  int* reuse_all = nullptr;
  int* counters = nullptr;
  int* any_active = nullptr;
  int* ready_all = nullptr;
  size_t ready_words = 0;
  int* tflags_all = nullptr;
  size_t tflags_words = 0;
  unsigned char* maps_all = nullptr;       // per problem: tensor maps of L, Linv, Rv, Rz (128 B each)
  // block maps
  std::vector<int2> h_vmap, h_bmap, h_claims;
  std::vector<int4> h_syrk;
  std::vector<int4> h_tasks[TL_COUNT];
  int2* vmap = nullptr;
  int nvb = 0;
  int2* bmap = nullptr;
  int nbb = 0;
  std::vector<MvGroup> mv;
  std::vector<TraceGroup> tr;
  int4* syrk_tiles = nullptr;
  int nsyrk = 0;
  DagJob* jobs = nullptr;                  // [problem * JOB_COUNT + slot]
  std::vector<DagJob> hjobs;
  int4* tasks[TL_COUNT] = {};
  int ntasks[TL_COUNT] = {};
  int* zvalid_all = nullptr;
  int has_gauss = 0;                       // some problem has a Gaussian likelihood
  int zlag = kZLag;                        // columns of delay of the identity rows solved beside a factor
  int2* claims = nullptr;
  int nclaims = 0;
  // graphs
  cudaGraphExec_t gexec[OP_COUNT] = {};
  cudaStream_t cap_s = nullptr, cap_s2 = nullptr, cap_s3 = nullptr;   // capture streams (s3: nested bodies)
  int grad_ready = 0;
  int eager = 0;                           // PGB_EAGER=1: kernels launched directly, host-driven loop
  unsigned long long* trace = nullptr;     // PGB_TRACE=1: per-task timestamps of the DAG
};

Shape make_shape(const pgb_desc* d) { return shape_from_desc(d); }

int theta_size_of(const pgb_desc* d) {
  return theta_len(d->n_lengthscales, d->likelihood, d->likelihood == PGB_LIK_GAUSSIAN ? 0 : d->j);
}

std::once_flag g_attr_once;
void setup_attributes() {
  std::call_once(g_attr_once, [] {
    dag_set_attributes();
    trsv_set_attributes();
    // keep freed handle workspaces in this process's pool for the next handle
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
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
    } else if (kind == RHS_VEC_IDENT) {
      v.push_back(make_int4(job, nt, j, 0));
      // w = 1: an identity row solved beside the factorisation (handed out
      // later, see merge_tasks)
      for (int r = 0; r <= j; ++r) v.push_back(make_int4(job, nt + 1 + r, j, 1));
    }
  }
  return v;
}

// The tasks of problem p (nt tile rows) in task list `list`; `gauss`: the
// problem's likelihood is Gaussian (its evaluation Newton step solves L^-T).
std::vector<int4> list_tasks(int p, int nt, int list, bool gauss) {
  switch (list) {
    case TL_STEP: return build_tasks(p * JOB_COUNT + JOB_VEC, nt, RHS_VEC, 1, true);
    case TL_NONE: return build_tasks(p * JOB_COUNT + JOB_NONE, nt, RHS_NONE, 0, true);
    case TL_IDENT: return build_tasks(p * JOB_COUNT + JOB_IDENT, nt, RHS_IDENT, nt, true);
    default:
      return gauss ? build_tasks(p * JOB_COUNT + JOB_VEC_IDENT, nt, RHS_VEC_IDENT, nt + 1, true)
                   : build_tasks(p * JOB_COUNT + JOB_VEC, nt, RHS_VEC, 1, true);
  }
}

// Lookahead stage of tile task (i, j) of a problem with nt tile rows
// (i >= nt: right-hand-side rows) and near band depth `near`:
//   diagonal (j, j) -> 2j,  the `near` tiles below it -> 2j+1,
//   other tiles of column j and right-hand-side tiles -> 2j+3,
// so the diagonal of column j+1 and the tiles below it (the critical path:
// they solve with the panels of L_jj as they are published) are handed out
// before the rest of column j, whose tiles need the inverse of the diagonal
// tile L_jj; by the time they are taken that inverse is usually published,
// and their blocks do not sit waiting for it.  Sorting by (stage, j, i)
// keeps every task after all tasks it waits for: a task (i, j) waits for
// (i, k), (j, k) with k < j (stages <= 2j+1, and at stage 2j+1 only column
// j-1 < j) and for (j, j) (stage 2j).
int dag_stage(int i, int j, int nt, int near) {
  if (i < nt && i == j) return 2 * j;
  if (i < nt && i <= j + near) return 2 * j + 1;
  return 2 * j + 3;
}

// One task list from every problem's tasks: by stage, then problem rank,
// then column, then row.
// A problem of at most `whole_max` tile rows becomes one task (job, -1, 0, 0)
// at stage 0: one block runs all its tiles in order (no waits on other blocks).
// Identity rows solved beside a factorisation (task w = 1) go `zlag` columns
// later than the other right-hand-side tiles of their column: they wait for
// their row's previous tile and for the inverse of the diagonal tile, and a
// block holding one would otherwise sit waiting while factorisation tiles
// are handed out.  Their dependencies all sit in earlier stages still.
std::vector<int4> merge_tasks(const std::vector<std::vector<int4>>& per, const std::vector<int>& nt,
                              const std::vector<int>& rank, const std::vector<int>& near, int whole_max,
                              int zlag = 0) {
  struct Key {
    int stage, rank, j, i;
    int4 t;
  };
  std::vector<Key> all;
  for (size_t p = 0; p < per.size(); ++p)
    if (nt[p] <= whole_max && !per[p].empty())
      all.push_back(Key{0, rank[p], 0, -1, make_int4(per[p][0].x, -1, 0, 0)});
    else
      for (const int4& t : per[p])
        all.push_back(Key{dag_stage(t.y, t.z, nt[p], near[p]) + (t.w ? 2 * zlag : 0), rank[p], t.z, t.y, t});
  std::sort(all.begin(), all.end(), [](const Key& a, const Key& b) {
    if (a.stage != b.stage) return a.stage < b.stage;
    if (a.rank != b.rank) return a.rank < b.rank;
    if (a.j != b.j) return a.j < b.j;
    return a.i < b.i;
  });
  std::vector<int4> out;
  out.reserve(all.size());
  for (const Key& x : all) out.push_back(x.t);
  return out;
}

// Host -> device upload that has landed when it returns.  A plain cudaMemcpy
// from pageable memory may return before its DMA reaches the device and is
// not ordered with non-blocking streams, so work a caller then enqueues on
// its own stream could read the old contents; the copy runs on `s` and `s` is
// synchronised instead.
int h2d(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes == 0) return PGB_OK;
  CU_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
  CU_TRY(cudaStreamSynchronize(s));
  return PGB_OK;
}

template <class Tp>
int upload(Tp* dst, const std::vector<Tp>& v, cudaStream_t s) {
  return h2d(dst, v.data(), v.size() * sizeof(Tp), s);
}

enum MapSlot { MAP_L = 0, MAP_LINV = 1, MAP_RV = 2, MAP_RZ = 3, MAPS_PER_PROB = 4 };

const void* map_slot(const Engine& e, int p, int slot) {
  return e.maps_all + ((size_t)p * MAPS_PER_PROB + slot) * 128;
}

// Encode the tensor maps of every problem's L, Linv, Rv (and Rz when
// allocated) and copy them to the arena.
int upload_maps(Engine& e) {
  std::vector<unsigned char> h((size_t)e.nprob * MAPS_PER_PROB * 128, 0);
  for (int p = 0; p < e.nprob; ++p) {
    const Prob& q = e.hp[p];
    unsigned char* m = h.data() + (size_t)p * MAPS_PER_PROB * 128;
    // the tensor cores read the TF32 hi/lo splits (2 ld columns per row)
    const long long lds = 2 * q.ld;
    bool ok = make_tile_map(m + MAP_L * 128, q.Ls, q.n_pad, lds, lds) &&
              make_tile_map(m + MAP_LINV * 128, q.Linvs, (long long)q.nt * T, 2 * T, 2 * T) &&
              make_tile_map(m + MAP_RV * 128, q.Rvs, T, lds, lds);
    if (ok && q.Rz) ok = make_tile_map(m + MAP_RZ * 128, q.Rz, q.n_pad, lds, lds);
    if (!ok) return PGB_ECUDA;
  }
  return h2d(e.maps_all, h.data(), h.size(), e.cap_s);
}

// Assign every device pointer of the engine from `base` (0: sizing pass).
size_t layout(Engine& e, uintptr_t base) {
  Bump b;
  b.base = base;
  const int np = e.nprob;
  e.X_all = b.take<float>(e.x_total);
  e.y_all = b.take<int>(e.y_total);
  e.theta_all = b.take<float>(e.th_total);
  e.value_all = b.take<float>(np);
  e.err_all = b.take<float>(np);
  e.grad_all = b.take<float>(e.th_total);
  e.status_all = b.take<int>((size_t)np * kStatusWords);
  e.active_all = b.take<int>(np);
  e.enabled_all = b.take<int>(np);
  e.reuse_all = b.take<int>((size_t)np * 4);
  e.counters = b.take<int>(C_COUNT);
  e.any_active = b.take<int>(2);
  e.ready_all = b.take<int>(e.ready_words);
  e.tflags_all = b.take<int>(e.tflags_words);
  e.maps_all = b.take<unsigned char>((size_t)np * MAPS_PER_PROB * 128);
  e.probs = b.take<Prob>(np);
  e.jobs = b.take<DagJob>((size_t)np * JOB_COUNT);
  e.vmap = b.take<int2>(e.h_vmap.size());
  e.bmap = b.take<int2>(e.h_bmap.size());
  e.claims = b.take<int2>(e.h_claims.size());
  e.syrk_tiles = b.take<int4>(e.h_syrk.size());
  for (int k = 0; k < TL_COUNT; ++k) e.tasks[k] = b.take<int4>(e.h_tasks[k].size());
  e.zvalid_all = b.take<int>(np);
  for (MvGroup& g : e.mv) g.map = b.take<int2>(g.h.size());
  for (TraceGroup& g : e.tr) g.tiles = b.take<int4>(g.h.size());
  size_t ready_off = 0, tflags_off = 0;
  for (int p = 0; p < np; ++p) {
    Prob& q = e.hp[p];
    const Shape& s = e.sh[p];
    const int nt = e.nt[p];
    const size_t npad = (size_t)nt * T;
    const size_t ld = npad;
    q.sh = s;
    q.nt = nt;
    q.n_pad = (int)npad;
    q.ld = (long long)ld;
    q.tol = e.desc[p].tolerance;
    q.maxiter = e.desc[p].maxiter;
    q.X = e.X_all + e.x_off[p];
    q.y = static_cast<int*>(e.y_all) + e.y_off[p];
    q.theta = e.theta_all + e.th_off[p];
    q.Xf = b.take<float>(npad * s.Dp);
    q.L = b.take<float>(npad * ld);
    q.Linv = b.take<float>((size_t)nt * T * T);
    q.Rv = b.take<float>((size_t)T * ld);
    q.Ls = b.take<float>(npad * 2 * ld);
    q.Linvs = b.take<float>((size_t)nt * T * 2 * T);
    q.Rvs = b.take<float>((size_t)T * 2 * ld);
    float** vecs[] = {&q.a,    &q.f,    &q.d1, &q.W,    &q.sw, &q.r,  &q.t, &q.x, &q.logp, &q.d3,
                      &q.dsig, &q.svec, &q.rv, &q.zbar, &q.tz, &q.y2, &q.u, &q.c, &q.rowdot, &q.sw_prev, &q.da};
    for (float** v : vecs) *v = b.take<float>(npad);
    const size_t nvb = (size_t)ceil_div((int)npad, VT);
    q.part = b.take<double>(nvb + 8);
    q.tpart = b.take<double>((size_t)nt * (nt + 1) / 2 * (MAX_D + 1));
    q.lpart = b.take<double>(nvb * (MAX_THETA + 2));
    q.err = e.err_all + p;
    q.value = e.value_all + p;
    q.grad = e.grad_all + e.th_off[p];
    q.status = e.status_all + (size_t)p * kStatusWords;
    q.active = e.active_all + p;
    q.enabled = e.enabled_all + p;
    q.reuse = e.reuse_all + (size_t)p * 4;
    q.zvalid = e.zvalid_all + p;
    q.tflags = e.tflags_all + tflags_off;
    tflags_off += 2 * (size_t)nt;
    q.Rz = nullptr;
    q.Binv = nullptr;
    q.tm_Rz = map_slot(e, p, MAP_RZ);
    // factorisation jobs of this problem
    for (int k = 0; k < JOB_COUNT; ++k) {
      DagJob& j = e.hjobs[(size_t)p * JOB_COUNT + k];
      std::memset(&j, 0, sizeof(j));
      j.n = s.n;
      j.nt = nt;
      j.ld = (long long)ld;
      j.near = e.near[p];
      j.L = q.L;
      j.Linv = q.Linv;
      j.Ls = q.Ls;
      j.Linvs = q.Linvs;
      j.Xf = q.Xf;
      j.sw = q.sw;
      j.theta = q.theta;
      j.sh = s;
      j.ready = e.ready_all + ready_off;
      j.progress = e.ready_all + ready_off + (2 * (size_t)nt + 1) * nt;
      j.status = q.status;
      j.reuse = q.reuse + 2;
      j.reuse_mode = 0;
      j.tm_L = map_slot(e, p, MAP_L);
      j.tm_Linv = map_slot(e, p, MAP_LINV);
    }
    ready_off += (2 * (size_t)nt + 1) * nt + 2 * nt;
    DagJob* jb = &e.hjobs[(size_t)p * JOB_COUNT];
    jb[JOB_VEC].rhs_kind = RHS_VEC;
    jb[JOB_VEC].nrt = 1;
    jb[JOB_VEC].nrhs = 1;
    jb[JOB_VEC].R = q.Rv;
    jb[JOB_VEC].Rs = q.Rvs;
    jb[JOB_VEC].rhs_vec = q.t;
    jb[JOB_VEC].reuse_mode = 2;
    jb[JOB_VEC].active = q.active;
    jb[JOB_VEC].tm_R = map_slot(e, p, MAP_RV);
    jb[JOB_NONE].rhs_kind = RHS_NONE;
    jb[JOB_NONE].reuse_mode = 1;
    jb[JOB_NONE].active = q.active;
    jb[JOB_IDENT].rhs_kind = RHS_IDENT;
    jb[JOB_IDENT].reuse_mode = 1;
    jb[JOB_IDENT].active = q.active;
    jb[JOB_IDENT].nrt = nt;
    jb[JOB_IDENT].nrhs = (int)npad;
    jb[JOB_IDENT].tm_R = q.tm_Rz;
    jb[JOB_CROSS].rhs_kind = RHS_CROSS;
    jb[JOB_IDENT].zvalid = q.zvalid;
    jb[JOB_VEC_IDENT] = jb[JOB_VEC];
    jb[JOB_VEC_IDENT].rhs_kind = RHS_VEC_IDENT;
    jb[JOB_VEC_IDENT].nrt = 1 + nt;
    jb[JOB_VEC_IDENT].tm_Z = q.tm_Rz;
    jb[JOB_VEC_IDENT].Zs = q.Rz;
  }
  return b.off;
}

void engine_free(Engine& e) {
  for (int k = 0; k < OP_COUNT; ++k)
    if (e.gexec[k]) cudaGraphExecDestroy(e.gexec[k]);
  if (e.cap_s) {
    ws_free(e.cap_s, e.arena);
    ws_free(e.cap_s, e.garena);
    ws_free(e.cap_s, e.trace);
    cudaStreamSynchronize(e.cap_s);
    cudaStreamDestroy(e.cap_s);
  }
  if (e.cap_s2) cudaStreamDestroy(e.cap_s2);
  if (e.cap_s3) cudaStreamDestroy(e.cap_s3);
  e.arena = e.garena = nullptr;
  e.trace = nullptr;
}

int engine_upload_tables(Engine& e) {
  PGB_TRY(h2d(e.probs, e.hp.data(), sizeof(Prob) * e.hp.size(), e.cap_s));
  return h2d(e.jobs, e.hjobs.data(), sizeof(DagJob) * e.hjobs.size(), e.cap_s);
}

// The three merged DAG task lists (Newton step, factor only, factor with
// L^-T) from every problem's tiles, in lookahead order (dag_stage with the
// problem's near band depth), problems by rank within a stage.  The task
// counts do not depend on the depths.
void build_task_lists(Engine& e) {
  for (int k = 0; k < TL_COUNT; ++k) {
    std::vector<std::vector<int4>> per(e.nprob);
    for (int p = 0; p < e.nprob; ++p) {
      const bool gauss = e.desc[p].likelihood == PGB_LIK_GAUSSIAN;
      per[p] = list_tasks(p, e.nt[p], k, gauss);
    }
    e.h_tasks[k] = merge_tasks(per, e.nt, e.rank, e.near, e.whole_max, e.zlag);
    e.ntasks[k] = (int)e.h_tasks[k].size();
  }
}

// Set the near band depth of every problem (near[p] = 0: the built-in
// rule) and rebuild the task lists and job tables.  Waits for the device
// first: launches in flight read both.  Captured graphs stay valid (they read
// the lists from the same device arrays; the task counts do not change).
int engine_set_near(Engine& e, const int32_t* near) {
  if (!near) return PGB_EINVAL;
  std::vector<int> v(e.nprob);
  for (int p = 0; p < e.nprob; ++p) {
    v[p] = near[p] == 0 ? near_depth(e.nt[p]) : near[p];
    if (v[p] < 1 || v[p] > kMaxNearDepth) return PGB_EINVAL;
  }
  if (v == e.near) return PGB_OK;
  CU_TRY(cudaDeviceSynchronize());
  e.near = v;
  build_task_lists(e);
  for (int p = 0; p < e.nprob; ++p)
    for (int k = 0; k < JOB_COUNT; ++k) e.hjobs[(size_t)p * JOB_COUNT + k].near = v[p];
  for (int k = 0; k < TL_COUNT; ++k) PGB_TRY(upload(e.tasks[k], e.h_tasks[k], e.cap_s));
  return engine_upload_tables(e);
}

// Build the engine of `count` problems: shapes, maps, task lists, one
// arena.  Problems are ranked by size (largest first) for the merged DAG and
// solve orders, so the longest critical paths start first.
int engine_init(Engine& e, const pgb_desc* descs, int count) {
  if (!descs || count < 1) return PGB_EINVAL;
  for (int p = 0; p < count; ++p) PGB_TRY(validate_desc(descs + p));
  setup_attributes();
  e.nprob = count;
  e.desc.assign(descs, descs + count);
  e.sh.resize(count);
  e.nt.resize(count);
  e.th.resize(count);
  e.x_off.resize(count);
  e.y_off.resize(count);
  e.th_off.resize(count);
  e.hp.assign(count, Prob{});
  e.hjobs.assign((size_t)count * JOB_COUNT, DagJob{});
  e.dag_dm = 4;
  e.nt_max = 1;
  for (int p = 0; p < count; ++p) {
    e.sh[p] = make_shape(descs + p);
    e.nt[p] = ceil_div(descs[p].n, T);
    e.th[p] = theta_size_of(descs + p);
    e.x_off[p] = e.x_total;
    e.y_off[p] = e.y_total;
    e.th_off[p] = e.th_total;
    e.x_total += (size_t)descs[p].n * descs[p].d;
    e.y_total += (size_t)descs[p].n;
    e.th_total += (size_t)e.th[p];
    // tile flags of the L rows and of up to nt + 1 right-hand-side row
    // tiles, then the panel counters
    e.ready_words += (2 * (size_t)e.nt[p] + 1) * e.nt[p] + 2 * e.nt[p];
    e.tflags_words += 2 * (size_t)e.nt[p];
    e.dag_dm = std::max(e.dag_dm, dm_of(e.sh[p].Dp));
    if (descs[p].likelihood == PGB_LIK_GAUSSIAN) e.has_gauss = 1;
    e.nt_max = std::max(e.nt_max, e.nt[p]);
  }
  CU_TRY(cudaGetDevice(&e.device));
  CU_TRY(cudaDeviceGetAttribute(&e.num_sms, cudaDevAttrMultiProcessorCount, e.device));
  // size ranking (largest n first, index order among equals)
  std::vector<int> order(count), rank(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return descs[a].n > descs[b].n; });
  for (int r = 0; r < count; ++r) rank[order[r]] = r;
  // per-point map
  for (int p = 0; p < count; ++p)
    for (int blk = 0; blk < ceil_div(e.nt[p] * T, VT); ++blk) e.h_vmap.push_back(make_int2(p, blk));
  e.nvb = (int)e.h_vmap.size();
  // B^-1 row map (8 rows per block)
  for (int p = 0; p < count; ++p)
    for (int blk = 0; blk < ceil_div(descs[p].n, 8); ++blk) e.h_bmap.push_back(make_int2(p, blk));
  e.nbb = (int)e.h_bmap.size();
  // Gram matvec groups by (kernel, feature width)
  {
    std::map<std::pair<int, int>, int> gi;
    for (int pr = 0; pr < count; ++pr) {
      const int p = order[pr];
      const int DM = dm_of(e.sh[p].Dp);
      const auto key = std::make_pair(e.sh[p].kind, DM);
      if (!gi.count(key)) {
        gi[key] = (int)e.mv.size();
        MvGroup g;
        g.kind = key.first;
        g.DM = DM;
        e.mv.push_back(g);
      }
      MvGroup& g = e.mv[gi[key]];
      const int rows = mv_block_rows(DM);
      for (int blk = 0; blk < ceil_div(descs[p].n, rows); ++blk) g.h.push_back(make_int2(p, blk));
    }
  }
  // gradient trace tiles by feature width; B^-1 tiles longest k-range first
  {
    std::map<std::pair<int, int>, int> gi;
    std::vector<std::pair<int, int4>> sy;
    for (int pr = 0; pr < count; ++pr) {
      const int p = order[pr];
      const int DM = dm_of(e.sh[p].Dp);
      const int per = e.sh[p].kind == PGB_KERNEL_EQ_PERIODIC ? 1 : 0;
      const auto key = std::make_pair(DM, per);
      if (!gi.count(key)) {
        gi[key] = (int)e.tr.size();
        TraceGroup g;
        g.DM = DM;
        g.periodic = per;
        e.tr.push_back(g);
      }
      TraceGroup& g = e.tr[gi[key]];
      int ord = 0;
      for (int I = 0; I < e.nt[p]; ++I)
        for (int J = 0; J <= I; ++J) {
          g.h.push_back(make_int4(p, I, J, ord++));
          sy.push_back(std::make_pair(e.nt[p] - I, make_int4(p, I, J, 0)));
        }
    }
    std::stable_sort(sy.begin(), sy.end(), [](const std::pair<int, int4>& a, const std::pair<int, int4>& b) {
      return a.first > b.first;
    });
    for (auto& x : sy) e.h_syrk.push_back(x.second);
    e.nsyrk = (int)e.h_syrk.size();
  }
  // merged DAG task lists in lookahead order (dag_stage), problems by rank
  // within a stage
  e.rank = rank;
  e.near.resize(count);
  for (int p = 0; p < count; ++p) e.near[p] = near_depth(e.nt[p]);
  {
    // PGB_WHOLE_TILES=k: problems of at most k tile rows run whole on one
    // block (0: every tile is its own task)
    const char* wv = std::getenv("PGB_WHOLE_TILES");
    if (wv && wv[0] >= '0' && wv[0] <= '9') e.whole_max = std::atoi(wv);
    // PGB_ZLAG=k: identity rows solved beside a factorisation go k columns late
    const char* zv = std::getenv("PGB_ZLAG");
    if (zv && zv[0] >= '0' && zv[0] <= '9') e.zlag = std::atoi(zv);
  }
  build_task_lists(e);
  // merged solve claims: position by position, problems by rank
  {
    for (int q = 0; q < e.nt_max; ++q)
      for (int r = 0; r < count; ++r) {
        const int p = order[r];
        if (q < e.nt[p]) e.h_claims.push_back(make_int2(p, q));
      }
    e.nclaims = (int)e.h_claims.size();
  }
  // one arena
  CU_TRY(cudaStreamCreateWithFlags(&e.cap_s, cudaStreamNonBlocking));
  CU_TRY(cudaStreamCreateWithFlags(&e.cap_s2, cudaStreamNonBlocking));
  CU_TRY(cudaStreamCreateWithFlags(&e.cap_s3, cudaStreamNonBlocking));
  const size_t bytes = layout(e, 0);
  PGB_TRY(ws_alloc(e.cap_s, &e.arena, bytes));
  layout(e, reinterpret_cast<uintptr_t>(e.arena));
  CU_TRY(cudaMemsetAsync(e.arena, 0, bytes, e.cap_s));
  CU_TRY(cudaStreamSynchronize(e.cap_s));
  {
    const std::vector<int> ones(count, 1);
    PGB_TRY(upload(e.enabled_all, ones, e.cap_s));
  }
  PGB_TRY(upload(e.vmap, e.h_vmap, e.cap_s));
  PGB_TRY(upload(e.bmap, e.h_bmap, e.cap_s));
  PGB_TRY(upload(e.claims, e.h_claims, e.cap_s));
  PGB_TRY(upload(e.syrk_tiles, e.h_syrk, e.cap_s));
  for (int k = 0; k < TL_COUNT; ++k) PGB_TRY(upload(e.tasks[k], e.h_tasks[k], e.cap_s));
  for (MvGroup& g : e.mv) PGB_TRY(upload(g.map, g.h, e.cap_s));
  for (TraceGroup& g : e.tr) PGB_TRY(upload(g.tiles, g.h, e.cap_s));
  {
    const char* ev = std::getenv("PGB_EAGER");
    e.eager = (ev && ev[0] == '1') ? 1 : 0;
    const char* tv = std::getenv("PGB_TRACE");
    if (tv && tv[0] == '1') {
      size_t mx = 0;
      for (int k = 0; k < TL_COUNT; ++k) mx = std::max(mx, (size_t)e.ntasks[k]);
      void* tp = nullptr;
      if (ws_alloc(e.cap_s, &tp, sizeof(unsigned long long) * (mx * 8 + (size_t)e.nt_max * 48)) == PGB_OK) {
        e.trace = static_cast<unsigned long long*>(tp);
        for (DagJob& j : e.hjobs) {
          j.trace = e.trace;
          j.ptrace = e.trace + mx * 8;
        }
      }
    }
  }
  PGB_TRY(upload_maps(e));
  PGB_TRY(engine_upload_tables(e));
  return PGB_OK;
}

// L^-T and B^-1 of every problem, allocated on the first gradient request.
int ensure_grad_buffers(Engine& e) {
  if (e.grad_ready) return PGB_OK;
  size_t total = 0;
  for (int p = 0; p < e.nprob; ++p) total += 3 * (((size_t)e.hp[p].n_pad * e.hp[p].ld * sizeof(float) + 255) & ~(size_t)255);
  PGB_TRY(ws_alloc(e.cap_s, &e.garena, total));
  CU_TRY(cudaMemsetAsync(e.garena, 0, total, e.cap_s));
  CU_TRY(cudaStreamSynchronize(e.cap_s));
  Bump b;
  b.base = reinterpret_cast<uintptr_t>(e.garena);
  for (int p = 0; p < e.nprob; ++p) {
    const size_t mat = (size_t)e.hp[p].n_pad * e.hp[p].ld;
    e.hp[p].Rz = b.take<float>(2 * mat);   // split only: L^-T is read by the tensor cores alone
    e.hp[p].Binv = b.take<float>(mat);
    e.hjobs[(size_t)p * JOB_COUNT + JOB_IDENT].R = nullptr;
    e.hjobs[(size_t)p * JOB_COUNT + JOB_IDENT].Rs = e.hp[p].Rz;
    e.hjobs[(size_t)p * JOB_COUNT + JOB_VEC_IDENT].Zs = e.hp[p].Rz;
  }
  PGB_TRY(upload_maps(e));
  PGB_TRY(engine_upload_tables(e));
  e.grad_ready = 1;
  return PGB_OK;
}

int block_cap(const Engine& e) { return e.max_blocks > 0 ? std::min(e.max_blocks, e.num_sms) : e.num_sms; }
int dag_grid(const Engine& e, int ntasks) { return std::max(1, std::min(block_cap(e), ntasks)); }
int trsv_grid(const Engine& e) { return std::max(1, std::min(e.nclaims, 4 * block_cap(e))); }
// Grid of the kernels with one block per map item (Gram and B^-1 matvecs,
// gradient trace): the whole map, or, on a handle capped to a share of the
// SMs, twice the cap (the blocks stride over the map), so that these wide
// launches leave the other SMs free as the persistent ones do.
int wide_grid(const Engine& e, int nitems) { return e.max_blocks > 0 ? std::min(nitems, 2 * e.max_blocks) : nitems; }

// ---------------------------------------------------------------- enqueue helpers
void enq_matvec(Engine& e, MatvecOp op, cudaStream_t s) {
  for (MvGroup& g : e.mv)
    launch_gram_matvec(g.kind, g.DM, e.probs, g.map, (int)g.h.size(), wide_grid(e, (int)g.h.size()), op, s);
}

void enq_dag(Engine& e, int list, cudaStream_t s) {
  cudaMemsetAsync(e.ready_all, 0, sizeof(int) * e.ready_words, s);
  cudaMemsetAsync(e.counters + C_DAG, 0, sizeof(int), s);
  launch_dag_factor(e.jobs, e.tasks[list], e.ntasks[list], e.counters + C_DAG, e.dag_dm,
                    dag_grid(e, e.ntasks[list]), s);
}

// A conditional handle of the graph being captured on s, with the value it
// takes at each launch of the graph.
int cond_handle(cudaStream_t s, unsigned default_value, cudaGraphConditionalHandle* h) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t cg = nullptr;
  CU_TRY(cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, nullptr, nullptr, nullptr));
  CU_TRY(cudaGraphConditionalHandleCreate(h, cg, default_value, cudaGraphCondAssignDefault));
  return PGB_OK;
}

// Add a conditional node (WHILE or IF) on handle h at the current point of
// the capture on s, whose body is captured on s2 by `body(s2)`.
template <class Body>
int capture_cond(cudaStream_t s, cudaStream_t s2, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                 Body body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t cg = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  CU_TRY(cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &ndeps));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = type;
  cp.conditional.size = 1;
  cudaGraphNode_t cnode;
  CU_TRY(cudaGraphAddNode(&cnode, cg, deps, nullptr, ndeps, &cp));
  cudaGraph_t bodyg = cp.conditional.phGraph_out[0];
  CU_TRY(cudaStreamUpdateCaptureDependencies(s, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
  CU_TRY(cudaStreamBeginCaptureToGraph(s2, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  body(s2);
  cudaGraph_t body_out = nullptr;
  CU_TRY(cudaStreamEndCapture(s2, &body_out));
  return PGB_OK;
}

void enq_newton_step(Engine& e, cudaStream_t s, cudaGraphConditionalHandle h, int use_cond, int list) {
  // f += K da: f follows a by the updates (f = 0, da = a at the start), so
  // the rounding of f shrinks with the step instead of staying at the float32
  // error of a full K a, which would otherwise set a floor under ||da||
  enq_matvec(e, MatvecOp{F_DA, F_NONE, F_F, 0, 1, 1}, s);
  // d1, W, sqrt W, r = d1 - a, t = r / sqrt W
  launch_newton_lik(e.probs, e.vmap, e.nvb, s);
  // bitwise-unchanged W keeps the resident factor
  launch_reuse_check(e.probs, e.vmap, e.nvb, e.nprob, s);
  // new W: L L^T = B and w = L^-1 t in one factorisation (skipped on reuse)
  if (use_cond) {
    // only when some problem needs a new factor this step (after the first
    // steps most have stopped or reuse theirs, and a launch that skips every
    // task still walks the whole merged list)
    cudaGraphConditionalHandle hf;
    if (cond_handle(s, 0, &hf) == PGB_OK) {
      launch_need_factor(e.probs, e.nprob, hf, s);
      capture_cond(s, e.cap_s3, hf, cudaGraphCondTypeIf, [&](cudaStream_t bs) { enq_dag(e, list, bs); });
    }
  } else {
    enq_dag(e, list, s);
  }
  if (list == TL_VG_STEP) launch_mark_z(e.probs, e.nprob, s);
  launch_reuse_mark_valid(e.probs, e.nprob, s);
  // reused W: w = L^-1 t by the forward wavefront solve; then x = L^-T w
  cudaMemsetAsync(e.tflags_all, 0, sizeof(int) * e.tflags_words, s);
  cudaMemsetAsync(e.counters + C_TRSV_T, 0, sizeof(int) * 3, s);
  launch_trsv(e.probs, e.claims, e.nclaims, 0, e.counters + C_TRSV_L, 1, 1, trsv_grid(e), s);
  launch_trsv(e.probs, e.claims, e.nclaims, 1, e.counters + C_TRSV_T, 0, 1, trsv_grid(e), s);
  // a += W^1/2 x, stopping rule
  launch_newton_update(e.probs, e.vmap, e.nvb, s);
  launch_newton_finalize(e.probs, e.nprob, e.any_active, h, use_cond, s);
}

void enq_precision(Engine& e, cudaStream_t s) {
  enq_matvec(e, MatvecOp{F_A, F_NONE, F_F, 0, 1}, s);
  launch_lik_full(e.probs, e.vmap, e.nvb, s);
}

void enq_grad(Engine& e, cudaStream_t s) {
  cudaMemsetAsync(e.counters + C_SYRK, 0, sizeof(int), s);
  launch_syrk_zzt(e.probs, e.syrk_tiles, e.nsyrk, e.counters + C_SYRK, dag_grid(e, e.nsyrk), s);
  // rowdot_i = sum_j B^-1_ij K_ij sw_j  ->  diag(Sigma)_i = rowdot_i / sw_i
  enq_matvec(e, MatvecOp{F_SW, F_NONE, F_ROWDOT, 1, 1}, s);
  launch_grad_vec1(e.probs, e.vmap, e.nvb, s);
  // zbar = K (a - d1 - s)
  enq_matvec(e, MatvecOp{F_RV, F_NONE, F_ZBAR, 0, 1}, s);
  // u = (I + K W)^-1 zbar = W^-1/2 B^-1 W^1/2 zbar
  launch_scale_tz(e.probs, e.vmap, e.nvb, s);
  launch_binv_matvec(e.probs, e.bmap, e.nbb, wide_grid(e, e.nbb), s);
  launch_grad_vec3(e.probs, e.vmap, e.nvb, s);
  for (TraceGroup& g : e.tr) launch_grad_trace(g.DM, g.periodic, e.probs, g.tiles, (int)g.h.size(), wide_grid(e, (int)g.h.size()), s);
  launch_grad_lik_final(e.probs, e.vmap, e.nvb, e.nprob, s);
}

// One step of the VB fixed point w <- (sigma^2 I + K)^-1 (K w + sigma d1(K w))
// with the resident factor of B = I + K / sigma^2: f += K da, t = f + sigma
// d1, x = B^-1 t by the two wavefront solves, w = x / sigma^2, stopping rule.
void enq_vb_step(Engine& e, cudaStream_t s, cudaGraphConditionalHandle h, int use_cond) {
  enq_matvec(e, MatvecOp{F_DA, F_NONE, F_F, 0, 1, 1}, s);
  launch_vb_rhs(e.probs, e.vmap, e.nvb, s);
  cudaMemsetAsync(e.tflags_all, 0, sizeof(int) * e.tflags_words, s);
  cudaMemsetAsync(e.counters + C_TRSV_T, 0, sizeof(int) * 3, s);
  launch_trsv(e.probs, e.claims, e.nclaims, 0, e.counters + C_TRSV_L, 1, 1, trsv_grid(e), s);
  launch_trsv(e.probs, e.claims, e.nclaims, 1, e.counters + C_TRSV_T, 0, 1, trsv_grid(e), s);
  launch_vb_update(e.probs, e.vmap, e.nvb, s);
  launch_newton_finalize(e.probs, e.nprob, e.any_active, h, use_cond, s);
}

void enq_step(Engine& e, int op, cudaStream_t s, cudaGraphConditionalHandle h, int use_cond) {
  if (is_vb(op))
    enq_vb_step(e, s, h, use_cond);
  else
    enq_newton_step(e, s, h, use_cond, (op == OP_VG && e.has_gauss) ? TL_VG_STEP : TL_STEP);
}

void enq_prologue(Engine& e, int op, cudaStream_t s) {
  launch_reset_problems(e.probs, e.vmap, e.nvb, 1, s);
  launch_prep_features(e.probs, e.vmap, e.nvb, s);
  if (is_vb(op)) {
    // B = I + K / sigma^2 does not change along the VB iteration: factor once
    launch_vb_setup(e.probs, e.vmap, e.nvb, s);
    enq_dag(e, TL_NONE, s);
    launch_vb_mark(e.probs, e.nprob, s);
  }
}

// VB objective at the fixed point: f = K w, log p, d1, d2 at f, and the
// objective sum_i [-log p_i + f_i w_i / 2 + log L_ii] (its trace terms
// cancel exactly); zbar = K (w - d1) for the adjoint; the adjoint loop state.
void enq_vb_value(Engine& e, cudaStream_t s) {
  launch_activate_enabled(e.probs, e.nprob, s);
  enq_matvec(e, MatvecOp{F_A, F_NONE, F_F, 0, 1}, s);
  launch_vb_post(e.probs, e.vmap, e.nvb, s);
  launch_evidence(e.probs, e.vmap, e.nvb, e.nprob, s);
}

// Between the VB fixed point and its adjoint loop (OP_VB_VG).
void enq_vb_mid(Engine& e, cudaStream_t s) {
  enq_vb_value(e, s);
  enq_matvec(e, MatvecOp{F_RV, F_NONE, F_ZBAR, 0, 1}, s);   // zbar = K (w - d1)
  launch_vb_adj_reset(e.probs, e.nprob, s);
}

// One step of the adjoint fixed point u <- K (I + sigma D2) A^-1 u + zbar.
void enq_vb_adj_step(Engine& e, cudaStream_t s, cudaGraphConditionalHandle h, int use_cond) {
  cudaMemsetAsync(e.tflags_all, 0, sizeof(int) * e.tflags_words, s);
  cudaMemsetAsync(e.counters + C_TRSV_T, 0, sizeof(int) * 3, s);
  launch_trsv(e.probs, e.claims, e.nclaims, 0, e.counters + C_TRSV_L, 1, 1, trsv_grid(e), s);
  launch_trsv(e.probs, e.claims, e.nclaims, 1, e.counters + C_TRSV_T, 0, 1, trsv_grid(e), s);
  launch_vb_adj_scale(e.probs, e.vmap, e.nvb, s);
  enq_matvec(e, MatvecOp{F_TZ, F_NONE, F_Y2, 0, 1}, s);
  launch_vb_adj_update(e.probs, e.vmap, e.nvb, s);
  launch_vb_adj_finalize(e.probs, e.nprob, e.any_active, h, use_cond, s);
}

void enq_epilogue(Engine& e, int op, cudaStream_t s) {
  if (op == OP_VB_OBJECTIVE) {
    enq_vb_value(e, s);
    return;
  }
  if (op == OP_VB_VG) {
    // v = A^-1 u for the converged u (t = u), then the gradient: the prior
    // trace with R = sw B^-1 sw = A^-1 and c = w/2 - d1 + sigma v d2, and the
    // likelihood-parameter sums
    launch_activate_enabled(e.probs, e.nprob, s);
    cudaMemsetAsync(e.tflags_all, 0, sizeof(int) * e.tflags_words, s);
    cudaMemsetAsync(e.counters + C_TRSV_T, 0, sizeof(int) * 3, s);
    launch_trsv(e.probs, e.claims, e.nclaims, 0, e.counters + C_TRSV_L, 1, 1, trsv_grid(e), s);
    launch_trsv(e.probs, e.claims, e.nclaims, 1, e.counters + C_TRSV_T, 0, 1, trsv_grid(e), s);
    launch_vb_grad_vec(e.probs, e.vmap, e.nvb, s);
    enq_dag(e, TL_IDENT, s);   // L^-T on the resident factor
    cudaMemsetAsync(e.counters + C_SYRK, 0, sizeof(int), s);
    launch_syrk_zzt(e.probs, e.syrk_tiles, e.nsyrk, e.counters + C_SYRK, dag_grid(e, e.nsyrk), s);   // B^-1
    for (TraceGroup& g : e.tr) launch_grad_trace(g.DM, g.periodic, e.probs, g.tiles, (int)g.h.size(), wide_grid(e, (int)g.h.size()), s);
    launch_vb_grad_lik_final(e.probs, e.vmap, e.nvb, e.nprob, s);
    return;
  }
  if (op >= OP_POSTERIOR && !is_vb(op)) {
    launch_activate_enabled(e.probs, e.nprob, s);   // every enabled problem takes part from here on
    enq_precision(e, s);
    launch_reuse_check(e.probs, e.vmap, e.nvb, e.nprob, s);
    enq_dag(e, op == OP_VG ? TL_IDENT : TL_NONE, s);
    launch_reuse_mark_valid(e.probs, e.nprob, s);
    if (op >= OP_OBJECTIVE) launch_evidence(e.probs, e.vmap, e.nvb, e.nprob, s);
    if (op == OP_VG) enq_grad(e, s);
  }
}

// The same work without graphs: kernels launched directly, the Newton loop
// driven from the host (one flag read per step).  For profilers that do not
// follow kernels inside conditional graph nodes.
int run_eager(Engine& e, int op, cudaStream_t s) {
  if (needs_grad_buffers(op)) PGB_TRY(ensure_grad_buffers(e));
  enq_prologue(e, op, s);
  const char* tv = std::getenv("PGB_TRACE");
  const bool trace = tv && tv[0] == '1';
  int maxiter = 1;
  for (const pgb_desc& d : e.desc) maxiter = std::max(maxiter, d.maxiter);
  for (int it = 0; it < maxiter; ++it) {
    enq_step(e, op, s, 0, 0);
    int again = 0;
    float err = 0.0f;
    CU_TRY(cudaMemcpyAsync(&again, e.any_active + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (trace) CU_TRY(cudaMemcpyAsync(&err, e.err_all, sizeof(float), cudaMemcpyDeviceToHost, s));
    CU_TRY(cudaStreamSynchronize(s));
    if (trace) std::fprintf(stderr, "probit_gb300: newton %d ||delta||[0]=%.6g\n", it + 1, err);
    if (!again) break;
  }
  if (op == OP_VB_VG) {
    enq_vb_mid(e, s);
    for (int it = 0; it < maxiter; ++it) {
      enq_vb_adj_step(e, s, 0, 0);
      int again = 0;
      CU_TRY(cudaMemcpyAsync(&again, e.any_active + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
      CU_TRY(cudaStreamSynchronize(s));
      if (!again) break;
    }
  }
  enq_epilogue(e, op, s);
  CU_TRY(cudaGetLastError());
  return PGB_OK;
}

// Add a WHILE node at the current point of the capture on s whose body is
// captured on s2 by `body(s2, handle)`; the body's last kernel sets the
// condition (the loop runs at least once).
template <class Body>
int capture_while(cudaStream_t s, cudaStream_t s2, Body body) {
  cudaGraphConditionalHandle h;
  PGB_TRY(cond_handle(s, 1, &h));
  return capture_cond(s, s2, h, cudaGraphCondTypeWhile, [&](cudaStream_t bs) { body(bs, h); });
}

// Capture the graph of one operation.
int build_graph(Engine& e, int op) {
  if (e.gexec[op]) return PGB_OK;
  if (needs_grad_buffers(op)) PGB_TRY(ensure_grad_buffers(e));
  cudaStream_t s = e.cap_s, s2 = e.cap_s2;
  cudaGraph_t g = nullptr;
  CU_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
  enq_prologue(e, op, s);
  // WHILE node for the fixed-point loop (Newton or VB)
  PGB_TRY(capture_while(s, s2, [&](cudaStream_t bs, cudaGraphConditionalHandle h) { enq_step(e, op, bs, h, 1); }));
  if (op == OP_VB_VG) {
    enq_vb_mid(e, s);
    PGB_TRY(capture_while(s, s2, [&](cudaStream_t bs, cudaGraphConditionalHandle h) {
      enq_vb_adj_step(e, bs, h, 1);
    }));
  }
  enq_epilogue(e, op, s);
  CU_TRY(cudaStreamEndCapture(s, &g));
  CU_TRY(cudaGraphInstantiate(&e.gexec[op], g, 0));
  cudaGraphDestroy(g);
  return PGB_OK;
}

int run_op(Engine& e, int op, cudaStream_t s) {
  if (e.eager) return run_eager(e, op, s);
  PGB_TRY(build_graph(e, op));
  CU_TRY(cudaGraphLaunch(e.gexec[op], s));
  return PGB_OK;
}

// Copy the caller's packed inputs into the engine (stream-ordered).
int ingest(Engine& e, const float* X, const void* y, const float* theta, cudaStream_t s) {
  if (!X || !theta) return PGB_EINVAL;
  CU_TRY(cudaMemcpyAsync(e.X_all, X, sizeof(float) * e.x_total, cudaMemcpyDeviceToDevice, s));
  CU_TRY(cudaMemcpyAsync(e.theta_all, theta, sizeof(float) * e.th_total, cudaMemcpyDeviceToDevice, s));
  if (y) CU_TRY(cudaMemcpyAsync(e.y_all, y, 4 * e.y_total, cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

void status_from_words(const int* h, pgb_status* out) {
  out->code = h[ST_CODE];
  out->iterations = h[ST_ITERS];
  out->notpd_col = h[ST_NOTPD_COL] == INT_MAX ? -1 : h[ST_NOTPD_COL];
  out->converged = h[ST_CONVERGED];
}

}  // namespace

struct pgb_gp {
  Engine e;
  // predict workspace (grown on demand)
  float* Rc = nullptr;     // split of the solved cross-kernel rows (mpad x 2 ld)
  float* rowsq = nullptr;
  float* Xq = nullptr;
  float* Xq_in = nullptr;
  int* ready_c = nullptr;
  void* map_c = nullptr;   // tensor map of Rc (device, 128 B)
  float* mv_ws = nullptr;  // predictive mean and variance when only distributions are asked
  int4* tasks_c = nullptr;
  int ntasks_c = 0;
  long long cap_c = 0;     // predict rows allocated
  int m_tasks = -1;
  int factor_valid = 0;    // L is the factor of B at the resident W (same theta)
};

struct pgb_batch {
  Engine e;
};

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
  int r = validate_desc(desc);
  if (r != PGB_OK) return r;
  return theta_size_of(desc);
}

int pgb_gp_create(const pgb_desc* desc, pgb_gp** out) {
  if (!out) return PGB_EINVAL;
  *out = nullptr;
  int r = validate_desc(desc);
  if (r != PGB_OK) return r;
  pgb_gp* gp = new pgb_gp();
  r = engine_init(gp->e, desc, 1);
  if (r != PGB_OK) {
    pgb_gp_destroy(gp);
    return r;
  }
  *out = gp;
  return PGB_OK;
}

int pgb_gp_destroy(pgb_gp* gp) {
  if (!gp) return PGB_OK;
  void* ptrs[] = {gp->Rc, gp->rowsq, gp->Xq, gp->Xq_in, gp->ready_c, gp->tasks_c, gp->map_c, gp->mv_ws};
  if (gp->e.cap_s)
    for (void* p : ptrs) ws_free(gp->e.cap_s, p);
  engine_free(gp->e);
  delete gp;
  return PGB_OK;
}

int pgb_gp_desc(const pgb_gp* gp, pgb_desc* out) {
  if (!gp || !out) return PGB_EINVAL;
  *out = gp->e.desc[0];
  return PGB_OK;
}

int pgb_gp_set_max_blocks(pgb_gp* gp, int32_t max_blocks) {
  if (!gp || max_blocks < 0) return PGB_EINVAL;
  Engine& e = gp->e;
  if (e.max_blocks == max_blocks) return PGB_OK;
  e.max_blocks = max_blocks;
  for (int k = 0; k < OP_COUNT; ++k)   // graphs were captured with the old grid sizes
    if (e.gexec[k]) {
      cudaGraphExecDestroy(e.gexec[k]);
      e.gexec[k] = nullptr;
    }
  return PGB_OK;
}

int pgb_gp_set_near_depth(pgb_gp* gp, int32_t near_depth) {
  if (!gp) return PGB_EINVAL;
  return engine_set_near(gp->e, &near_depth);
}

int pgb_gp_status(pgb_gp* gp, pgb_status* out, void* stream) {
  if (!gp || !out) return PGB_EINVAL;
  int h[kStatusWords];
  CU_TRY(cudaMemcpyAsync(h, gp->e.status_all, sizeof(h), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  CU_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  status_from_words(h, out);
  return PGB_OK;
}

int pgb_gram(const pgb_desc* desc, const float* theta, const float* X1, int32_t n1, const float* X2, int32_t n2,
             float* K, int64_t ldk, void* stream) {
  if (validate_desc(desc) != PGB_OK || !theta || !X1 || !X2 || !K || n1 < 0 || n2 < 0 || ldk < n2) return PGB_EINVAL;
  if (n1 == 0 || n2 == 0) return PGB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const Shape sh = make_shape(desc);
  float *f1 = nullptr, *f2 = nullptr;
  CU_TRY(cudaMallocAsync(reinterpret_cast<void**>(&f1), sizeof(float) * (size_t)n1 * sh.Dp, s));
  CU_TRY(cudaMallocAsync(reinterpret_cast<void**>(&f2), sizeof(float) * (size_t)n2 * sh.Dp, s));
  launch_prep_features_raw(sh, X1, theta, f1, n1, n1, s);
  launch_prep_features_raw(sh, X2, theta, f2, n2, n2, s);
  launch_gram_full(sh, theta, f1, n1, f2, n2, K, ldk, s);
  CU_TRY(cudaFreeAsync(f1, s));
  CU_TRY(cudaFreeAsync(f2, s));
  CU_TRY(cudaGetLastError());
  return PGB_OK;
}

int pgb_log_likelihood(const pgb_desc* desc, const float* theta, const float* f, const void* y, int32_t n,
                       float* logp, float* d1, float* d2, float* d3, void* stream) {
  if (validate_desc(desc) != PGB_OK || !theta || !f || !y || n < 0) return PGB_EINVAL;
  if (n == 0) return PGB_OK;
  Shape sh = make_shape(desc);
  sh.n = n;
  launch_lik_eval(sh, theta, f, y, n, logp, d1, d2, d3, (cudaStream_t)stream);
  CU_TRY(cudaGetLastError());
  return PGB_OK;
}

int pgb_weight(pgb_gp* gp, const float* X, const void* y, const float* theta, float* a_out, void* stream) {
  if (!gp || !a_out || !y) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  Engine& e = gp->e;
  PGB_TRY(ingest(e, X, y, theta, s));
  PGB_TRY(run_op(e, OP_WEIGHT, s));
  gp->factor_valid = 0;
  CU_TRY(cudaMemcpyAsync(a_out, e.hp[0].a, sizeof(float) * e.sh[0].n, cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int pgb_vb_weight(pgb_gp* gp, const float* X, const void* y, const float* theta, float* w_out, void* stream) {
  if (!gp || !w_out || !y) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  Engine& e = gp->e;
  PGB_TRY(ingest(e, X, y, theta, s));
  PGB_TRY(run_op(e, OP_VB_WEIGHT, s));
  gp->factor_valid = 0;   // the resident factor is of I + K / sigma^2
  CU_TRY(cudaMemcpyAsync(w_out, e.hp[0].a, sizeof(float) * e.sh[0].n, cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int pgb_vb_objective(pgb_gp* gp, const float* X, const void* y, const float* theta, float* value_out,
                     void* stream) {
  if (!gp || !value_out || !y) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  Engine& e = gp->e;
  PGB_TRY(ingest(e, X, y, theta, s));
  PGB_TRY(run_op(e, OP_VB_OBJECTIVE, s));
  gp->factor_valid = 0;
  CU_TRY(cudaMemcpyAsync(value_out, e.value_all, sizeof(float), cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int pgb_vb_value_and_grad(pgb_gp* gp, const float* X, const void* y, const float* theta, float* value_out,
                          float* grad_out, void* stream) {
  if (!gp || !value_out || !grad_out || !y) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  Engine& e = gp->e;
  PGB_TRY(ingest(e, X, y, theta, s));
  PGB_TRY(run_op(e, OP_VB_VG, s));
  gp->factor_valid = 0;
  CU_TRY(cudaMemcpyAsync(value_out, e.value_all, sizeof(float), cudaMemcpyDeviceToDevice, s));
  CU_TRY(cudaMemcpyAsync(grad_out, e.grad_all, sizeof(float) * e.th_total, cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int pgb_precision(pgb_gp* gp, const float* X, const void* y, const float* theta, const float* a, float* W_out,
                  float* f_out, void* stream) {
  if (!gp || !a || !y) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  Engine& e = gp->e;
  const Prob& q = e.hp[0];
  PGB_TRY(ingest(e, X, y, theta, s));
  CU_TRY(cudaMemsetAsync(q.a, 0, sizeof(float) * q.n_pad, s));
  CU_TRY(cudaMemcpyAsync(q.a, a, sizeof(float) * q.sh.n, cudaMemcpyDeviceToDevice, s));
  launch_prep_features(e.probs, e.vmap, e.nvb, s);
  launch_activate_enabled(e.probs, e.nprob, s);
  enq_precision(e, s);
  if (W_out) CU_TRY(cudaMemcpyAsync(W_out, q.W, sizeof(float) * q.sh.n, cudaMemcpyDeviceToDevice, s));
  if (f_out) CU_TRY(cudaMemcpyAsync(f_out, q.f, sizeof(float) * q.sh.n, cudaMemcpyDeviceToDevice, s));
  gp->factor_valid = 0;
  CU_TRY(cudaGetLastError());
  return PGB_OK;
}

int pgb_approximate_posterior(pgb_gp* gp, const float* X, const void* y, const float* theta, float* a_out,
                              float* W_out, void* stream) {
  if (!gp || !a_out || !W_out || !y) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  Engine& e = gp->e;
  PGB_TRY(ingest(e, X, y, theta, s));
  PGB_TRY(run_op(e, OP_POSTERIOR, s));
  gp->factor_valid = 1;
  CU_TRY(cudaMemcpyAsync(a_out, e.hp[0].a, sizeof(float) * e.sh[0].n, cudaMemcpyDeviceToDevice, s));
  CU_TRY(cudaMemcpyAsync(W_out, e.hp[0].W, sizeof(float) * e.sh[0].n, cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int pgb_objective(pgb_gp* gp, const float* X, const void* y, const float* theta, float* value_out, void* stream) {
  if (!gp || !value_out || !y) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  Engine& e = gp->e;
  PGB_TRY(ingest(e, X, y, theta, s));
  PGB_TRY(run_op(e, OP_OBJECTIVE, s));
  gp->factor_valid = 1;
  CU_TRY(cudaMemcpyAsync(value_out, e.value_all, sizeof(float), cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int pgb_value_and_grad(pgb_gp* gp, const float* X, const void* y, const float* theta, float* value_out,
                       float* grad_out, void* stream) {
  if (!gp || !value_out || !grad_out || !y) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  Engine& e = gp->e;
  PGB_TRY(ingest(e, X, y, theta, s));
  PGB_TRY(run_op(e, OP_VG, s));
  gp->factor_valid = 1;
  CU_TRY(cudaMemcpyAsync(value_out, e.value_all, sizeof(float), cudaMemcpyDeviceToDevice, s));
  CU_TRY(cudaMemcpyAsync(grad_out, e.grad_all, sizeof(float) * e.th_total, cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int pgb_factor(pgb_gp* gp, void* stream) {
  if (!gp) return PGB_EINVAL;
  if (!gp->factor_valid) return PGB_ESTATE;
  cudaStream_t s = (cudaStream_t)stream;
  Engine& e = gp->e;
  CU_TRY(cudaMemsetAsync(e.hp[0].reuse + 2, 0, sizeof(int), s));   // always a full factorisation
  launch_activate_enabled(e.probs, e.nprob, s);
  enq_dag(e, TL_NONE, s);
  CU_TRY(cudaGetLastError());
  return PGB_OK;
}

}  // extern "C"

namespace {

// Predictive quantities at m test points: mean (needs a), variance, ordinal
// distribution, full covariance (any subset).  The factor of B is the
// resident one (reuse_factor) or rebuilt from W; the cross-kernel solve
// (L^-1 W^1/2 K_*)^T runs when variance, distribution or covariance is asked.
int predict_impl(pgb_gp* gp, const float* X, const float* theta, const float* a, const float* W, const float* Xs,
                 int32_t m, float* mean_out, float* var_out, float* dist_out, float* cov_out, int64_t ldc,
                 int32_t reuse_factor, void* stream) {
  if (!gp || !X || !theta || !Xs || m < 0) return PGB_EINVAL;
  if (!mean_out && !var_out && !dist_out && !cov_out) return PGB_EINVAL;
  if ((mean_out || dist_out) && !a) return PGB_EINVAL;
  if (cov_out && ldc < m) return PGB_EINVAL;
  if (dist_out && gp->e.sh[0].lik == PGB_LIK_GAUSSIAN) return PGB_EINVAL;
  if (m == 0) return PGB_OK;
  if (!reuse_factor && !W) return PGB_EINVAL;
  if (reuse_factor && !gp->factor_valid) return PGB_ESTATE;
  cudaStream_t s = (cudaStream_t)stream;
  Engine& e = gp->e;
  const Prob& q = e.hp[0];
  const Shape& sh = q.sh;
  const int nt = q.nt;
  const int mt = ceil_div(m, T);
  const long long mpad = (long long)mt * T;
  // grow the cross-kernel workspace
  if (mpad > gp->cap_c) {
    CU_TRY(cudaStreamSynchronize(s));
    void* old[] = {gp->Rc, gp->rowsq, gp->Xq, gp->Xq_in, gp->ready_c, gp->mv_ws};
    for (void* p : old) ws_free(e.cap_s, p);
    gp->Rc = gp->rowsq = gp->Xq = gp->Xq_in = gp->mv_ws = nullptr;
    gp->ready_c = nullptr;
    gp->cap_c = 0;
    auto grab = [&e](void** p, size_t bytes) { return ws_alloc(e.cap_s, p, bytes); };
    // split only (2 ld columns): the solved rows are read back by the tensor
    // cores alone (later right-hand-side tiles, the covariance product)
    PGB_TRY(grab(reinterpret_cast<void**>(&gp->Rc), sizeof(float) * (size_t)mpad * 2 * q.ld));
    PGB_TRY(grab(reinterpret_cast<void**>(&gp->rowsq), sizeof(float) * (size_t)mpad * nt));
    PGB_TRY(grab(reinterpret_cast<void**>(&gp->Xq), sizeof(float) * (size_t)mpad * sh.Dp));
    PGB_TRY(grab(reinterpret_cast<void**>(&gp->Xq_in), sizeof(float) * (size_t)mpad * sh.D));
    PGB_TRY(grab(reinterpret_cast<void**>(&gp->ready_c), sizeof(int) * (size_t)(nt + mt) * nt));
    PGB_TRY(grab(reinterpret_cast<void**>(&gp->mv_ws), sizeof(float) * 2 * (size_t)mpad));
    if (!gp->map_c) PGB_TRY(grab(&gp->map_c, 128));
    alignas(64) unsigned char m[128];
    if (!make_tile_map(m, gp->Rc, mpad, 2 * q.ld, 2 * q.ld)) return PGB_ECUDA;
    PGB_TRY(h2d(gp->map_c, m, sizeof(m), e.cap_s));
    gp->cap_c = mpad;
  }
  if (gp->m_tasks != mt) {
    if (gp->tasks_c) {
      CU_TRY(cudaStreamSynchronize(s));
      ws_free(e.cap_s, gp->tasks_c);
      gp->tasks_c = nullptr;
    }
    std::vector<int4> v = merge_tasks({build_tasks(JOB_CROSS, nt, RHS_CROSS, mt, false)}, {nt}, {0}, {e.near[0]}, 0);
    PGB_TRY(ws_alloc(e.cap_s, reinterpret_cast<void**>(&gp->tasks_c), v.size() * sizeof(int4)));
    PGB_TRY(upload(gp->tasks_c, v, e.cap_s));
    gp->ntasks_c = (int)v.size();
    gp->m_tasks = mt;
  }
  PGB_TRY(ingest(e, X, nullptr, theta, s));
  launch_prep_features(e.probs, e.vmap, e.nvb, s);
  if (!reuse_factor) {
    launch_reset_problems(e.probs, e.vmap, e.nvb, 0, s);
    launch_sqrt_w(sh.n, q.n_pad, W, q.sw, s);
    enq_dag(e, TL_NONE, s);
    gp->factor_valid = 0;   // factor of the caller's W, not of the resident posterior
  }
  CU_TRY(cudaMemcpyAsync(gp->Xq_in, Xs, sizeof(float) * (size_t)m * sh.D, cudaMemcpyDeviceToDevice, s));
  launch_prep_features_raw(sh, gp->Xq_in, q.theta, gp->Xq, m, (int)mpad, s);
  float* mean = mean_out ? mean_out : (dist_out ? gp->mv_ws : nullptr);
  float* var = var_out ? var_out : (dist_out ? gp->mv_ws + mpad : nullptr);
  if (mean) launch_gram_matvec_raw(sh, q.theta, gp->Xq, m, q.Xf, sh.n, a, mean, s);
  if (var || cov_out) {
    DagJob jb = e.hjobs[JOB_CROSS];
    jb.nrt = mt;
    jb.nrhs = m;
    jb.R = nullptr;
    jb.Rs = gp->Rc;
    jb.Xq = gp->Xq;
    jb.rowsq = gp->rowsq;
    jb.ready = gp->ready_c;
    jb.tm_R = gp->map_c;
    CU_TRY(cudaMemcpyAsync(e.jobs + JOB_CROSS, &jb, sizeof(DagJob), cudaMemcpyHostToDevice, s));
    // L tiles are done: mark them ready; RHS tiles start unready
    CU_TRY(cudaMemsetAsync(gp->ready_c, 1, sizeof(int) * (size_t)nt * nt, s));
    CU_TRY(cudaMemsetAsync(gp->ready_c + (size_t)nt * nt, 0, sizeof(int) * (size_t)mt * nt, s));
    CU_TRY(cudaMemsetAsync(e.counters + C_PREDICT, 0, sizeof(int), s));
    launch_dag_factor(e.jobs, gp->tasks_c, gp->ntasks_c, e.counters + C_PREDICT, e.dag_dm,
                      dag_grid(e, gp->ntasks_c), s);
    if (var) launch_predict_var(sh, q.theta, gp->rowsq, nt, m, var, s);
    if (cov_out) {
      // K(Xs, Xs), then minus (L^-1 W^1/2 K_*)^T (L^-1 W^1/2 K_*) on the tensor cores
      launch_gram_full(sh, q.theta, gp->Xq, m, gp->Xq, m, cov_out, ldc, s);
      CU_TRY(cudaMemsetAsync(e.counters + C_PREDICT, 0, sizeof(int), s));
      const int ntiles = mt * (mt + 1) / 2;
      launch_sub_rrt(gp->map_c, m, nt, cov_out, ldc, e.counters + C_PREDICT, e.status_all, dag_grid(e, ntiles), s);
    }
  }
  if (dist_out) launch_predictive_dist(sh, q.theta, mean, var, m, dist_out, s);
  CU_TRY(cudaGetLastError());
  return PGB_OK;
}

}  // namespace

extern "C" {

int pgb_predict(pgb_gp* gp, const float* X, const float* theta, const float* a, const float* W, const float* Xs,
                int32_t m, float* mean_out, float* var_out, int32_t reuse_factor, void* stream) {
  if (!gp || !a || (!mean_out && !var_out)) return PGB_EINVAL;
  return predict_impl(gp, X, theta, a, W, Xs, m, mean_out, var_out, nullptr, nullptr, 0, reuse_factor, stream);
}

int pgb_predict_distributions(pgb_gp* gp, const float* X, const float* theta, const float* a, const float* W,
                              const float* Xs, int32_t m, float* dist_out, float* mean_out, float* var_out,
                              int32_t reuse_factor, void* stream) {
  if (!gp || !dist_out) return PGB_EINVAL;
  return predict_impl(gp, X, theta, a, W, Xs, m, mean_out, var_out, dist_out, nullptr, 0, reuse_factor, stream);
}

int pgb_predict_covariance(pgb_gp* gp, const float* X, const float* theta, const float* W, const float* Xs,
                           int32_t m, float* cov_out, int64_t ldc, int32_t reuse_factor, void* stream) {
  if (!gp || !cov_out) return PGB_EINVAL;
  return predict_impl(gp, X, theta, nullptr, W, Xs, m, nullptr, nullptr, nullptr, cov_out, ldc, reuse_factor,
                      stream);
}

int pgb_predictive_distributions(const pgb_desc* desc, const float* theta, const float* mean, const float* var,
                                 int32_t m, float* dist_out, void* stream) {
  if (validate_desc(desc) != PGB_OK || desc->likelihood == PGB_LIK_GAUSSIAN || !theta || !mean || !var || !dist_out ||
      m < 0)
    return PGB_EINVAL;
  launch_predictive_dist(make_shape(desc), theta, mean, var, m, dist_out, (cudaStream_t)stream);
  CU_TRY(cudaGetLastError());
  return PGB_OK;
}

// ---------------------------------------------------------------- batches
int pgb_batch_create(const pgb_desc* descs, int32_t count, pgb_batch** out) {
  if (!out) return PGB_EINVAL;
  *out = nullptr;
  if (!descs || count < 1) return PGB_EINVAL;
  for (int p = 0; p < count; ++p) PGB_TRY(validate_desc(descs + p));
  pgb_batch* b = new pgb_batch();
  int r = engine_init(b->e, descs, count);
  if (r != PGB_OK) {
    pgb_batch_destroy(b);
    return r;
  }
  *out = b;
  return PGB_OK;
}

int pgb_batch_destroy(pgb_batch* b) {
  if (!b) return PGB_OK;
  engine_free(b->e);
  delete b;
  return PGB_OK;
}

int pgb_batch_set_near_depth(pgb_batch* b, const int32_t* near_depth) {
  if (!b) return PGB_EINVAL;
  return engine_set_near(b->e, near_depth);
}

int pgb_batch_size(const pgb_batch* b, int32_t* count) {
  if (!b || !count) return PGB_EINVAL;
  *count = b->e.nprob;
  return PGB_OK;
}

int pgb_batch_desc(const pgb_batch* b, int32_t index, pgb_desc* out) {
  if (!b || !out || index < 0 || index >= b->e.nprob) return PGB_EINVAL;
  *out = b->e.desc[index];
  return PGB_OK;
}

int pgb_batch_layout(const pgb_batch* b, int64_t* x_offsets, int64_t* y_offsets, int64_t* theta_offsets) {
  if (!b) return PGB_EINVAL;
  const Engine& e = b->e;
  for (int p = 0; p <= e.nprob; ++p) {
    if (x_offsets) x_offsets[p] = (int64_t)(p < e.nprob ? e.x_off[p] : e.x_total);
    if (y_offsets) y_offsets[p] = (int64_t)(p < e.nprob ? e.y_off[p] : e.y_total);
    if (theta_offsets) theta_offsets[p] = (int64_t)(p < e.nprob ? e.th_off[p] : e.th_total);
  }
  return PGB_OK;
}

int pgb_batch_objective(pgb_batch* b, const float* X, const void* y, const float* theta, float* values,
                        void* stream) {
  if (!b || !y || !values) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  Engine& e = b->e;
  PGB_TRY(ingest(e, X, y, theta, s));
  PGB_TRY(run_op(e, OP_OBJECTIVE, s));
  CU_TRY(cudaMemcpyAsync(values, e.value_all, sizeof(float) * e.nprob, cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int pgb_batch_value_and_grad(pgb_batch* b, const float* X, const void* y, const float* theta, float* values,
                             float* grads, void* stream) {
  if (!b || !y || !values || !grads) return PGB_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  Engine& e = b->e;
  PGB_TRY(ingest(e, X, y, theta, s));
  PGB_TRY(run_op(e, OP_VG, s));
  CU_TRY(cudaMemcpyAsync(values, e.value_all, sizeof(float) * e.nprob, cudaMemcpyDeviceToDevice, s));
  CU_TRY(cudaMemcpyAsync(grads, e.grad_all, sizeof(float) * e.th_total, cudaMemcpyDeviceToDevice, s));
  return PGB_OK;
}

int pgb_batch_set_enabled(pgb_batch* b, const int32_t* enabled, void* stream) {
  if (!b || !enabled) return PGB_EINVAL;
  CU_TRY(cudaMemcpyAsync(b->e.enabled_all, enabled, sizeof(int32_t) * b->e.nprob, cudaMemcpyDeviceToDevice,
                         (cudaStream_t)stream));
  return PGB_OK;
}

int pgb_batch_status(pgb_batch* b, pgb_status* out, void* stream) {
  if (!b || !out) return PGB_EINVAL;
  const Engine& e = b->e;
  std::vector<int> h((size_t)e.nprob * kStatusWords);
  CU_TRY(cudaMemcpyAsync(h.data(), e.status_all, sizeof(int) * h.size(), cudaMemcpyDeviceToHost,
                         (cudaStream_t)stream));
  CU_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  for (int p = 0; p < e.nprob; ++p) status_from_words(h.data() + (size_t)p * kStatusWords, out + p);
  return PGB_OK;
}

// Internal test hook (not part of the public C-ABI): makes the bounded
// device-side waits of one problem of a batch run out without any fault.
// The problem's flag waits give up after wait_limit_us microseconds (0: the
// built-in 4 s), and the factorisation tile (tile_i, tile_j), tile_i > tile_j
// (an off-diagonal tile of L), never releases its ready flag, so every task
// that depends on it waits, gives up, and the problem ends with
// PGB_ETIMEOUT while the other problems of the batch finish normally.
// problem < 0 clears the hook of every problem.  Waits for the device first
// (launches in flight read the tables).
int pgbx_batch_test_hook(pgb_batch* b, int32_t problem, int32_t wait_limit_us, int32_t tile_i, int32_t tile_j) {
  if (!b) return PGB_EINVAL;
  Engine& e = b->e;
  if (problem >= e.nprob || wait_limit_us < 0) return PGB_EINVAL;
  if (problem >= 0 && tile_i >= 0 && !(tile_i > tile_j && tile_j >= 0 && tile_i < e.nt[problem])) return PGB_EINVAL;
  CU_TRY(cudaDeviceSynchronize());
  for (int p = 0; p < e.nprob; ++p) {
    const bool on = problem < 0 ? false : p == problem;
    const int wh = (on && tile_i >= 0) ? ((tile_i << 16) | tile_j) + 1 : 0;
    for (int k = 0; k < JOB_COUNT; ++k) e.hjobs[(size_t)p * JOB_COUNT + k].withhold = wh;
    const int us = on ? wait_limit_us : 0;
    PGB_TRY(h2d(e.status_all + (size_t)p * kStatusWords + ST_WAIT_US, &us, sizeof(int), e.cap_s));
  }
  return engine_upload_tables(e);
}

// Internal diagnostic entry (not part of the public C-ABI): device pointer of
// one of a handle's intermediate buffers, for the test suite.
void* pgbx_gp_buffer(pgb_gp* gp, const char* name) {
  if (!gp || !name) return nullptr;
  const Prob& q = gp->e.hp[0];
  struct Item {
    const char* n;
    const void* p;
  };
  const Item items[] = {{"a", q.a},         {"f", q.f},         {"d1", q.d1},       {"W", q.W},
                        {"sw", q.sw},       {"d3", q.d3},       {"dsig", q.dsig},   {"svec", q.svec},
                        {"zbar", q.zbar},   {"u", q.u},         {"c", q.c},         {"rowdot", q.rowdot},
                        {"L", q.L},         {"Linv", q.Linv},   {"Rz", q.Rz},       {"Binv", q.Binv},
                        {"logp", q.logp},   {"grad", q.grad},   {"err", q.err},     {"value", q.value},
                        {"reuse", q.reuse}, {"trace", gp->e.trace}, {"da", q.da},
                        {"tasks_none", gp->e.tasks[JOB_NONE]},
                        {"tasks_ident", gp->e.tasks[JOB_IDENT]},
                        {"ptrace", gp->e.hjobs[JOB_NONE].ptrace}};
  for (const Item& it : items)
    if (std::strcmp(it.n, name) == 0) return const_cast<void*>(it.p);
  return nullptr;
}

// Internal diagnostic entries (not part of the public C-ABI): the merged
// task list of one factorisation kind (0 Newton step, 1 factor only, 2 with
// L^-T) and the per-task timestamps of the last factorisation launch
// (PGB_TRACE=1), for the test suite and profiling scripts.
int pgbx_batch_tasks(pgb_batch* b, int slot, const void** tasks, const void** trace) {
  if (!b || slot < 0 || slot > 2) return -1;
  if (tasks) *tasks = b->e.tasks[slot];
  if (trace) *trace = b->e.trace;
  return b->e.ntasks[slot];
}

// Internal diagnostic entry (host only, no GPU needed): the merged task list
// the engine builds for `count` problems of nt[p] tile rows (kind 0 Newton
// step, 1 factor only, 2 with L^-T, 3 the Newton step of an evidence +
// gradient evaluation with every problem Gaussian: the Newton row and the
// L^-T rows) with near band depths near[p] (NULL:
// the built-in rule) and problems of at most whole_max tile rows as one
// task (job, -1, 0, 0), written to out[4 * task] as (job, i, j, 0); returns
// the task count (call with out = NULL to size).
int pgbx_dag_order(const int32_t* nt, int32_t count, int32_t kind, const int32_t* near, int32_t whole_max,
                   int32_t* out) {
  if (!nt || count < 1 || kind < 0 || kind >= TL_COUNT) return -1;
  std::vector<int> nearv(count);
  for (int p = 0; p < count; ++p) {
    nearv[p] = near ? near[p] : near_depth(nt[p]);
    if (nearv[p] < 1 || nearv[p] > kMaxNearDepth) return -1;
  }
  std::vector<std::vector<int4>> per(count);
  std::vector<int> ntv(nt, nt + count), order(count), rank(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return nt[a] > nt[b]; });
  for (int r = 0; r < count; ++r) rank[order[r]] = r;
  for (int p = 0; p < count; ++p) per[p] = list_tasks(p, nt[p], kind, true);
  std::vector<int4> v = merge_tasks(per, ntv, rank, nearv, whole_max, kZLag);
  if (out)
    for (size_t t = 0; t < v.size(); ++t) {
      out[4 * t] = v[t].x;
      out[4 * t + 1] = v[t].y;
      out[4 * t + 2] = v[t].z;
      out[4 * t + 3] = 0;
    }
  return (int)v.size();
}

}  // extern "C"
