// pgb_gram_noalloc: the kernel matrix of pgb_gram without any device
// allocation.
//
// Who needs it: code that must not call cudaMalloc while it runs — an XLA
// FFI custom call (JAX preallocates most of the GPU and expects custom calls
// to live inside the buffers it hands them), work recorded into a CUDA graph
// by a framework's stream capture (an allocation there either fails the
// capture or escapes it), or a service that reserves all of its memory at
// start-up.  pgb_gram needs a few kilobytes to megabytes of scratch for the
// prepared input features and takes them from the stream-ordered allocator;
// this variant takes them from a fixed array compiled into the library.
//
// The scratch is a file-scope __device__ array of kScratchFloats floats
// (4 MiB): the prepared features of both point sets, (n1 + n2) * ceil4(F)
// floats, where F is the kernel's feature count (d, or 2d for eq_periodic,
// whose inputs become sin/cos pairs).  Every GPU that loads this library
// holds it until the process exits.  All calls share it and each call overwrites what it uses (nothing
// has to start at zero), so two calls whose work overlaps on the GPU — on
// different streams without ordering between them — race on it and give
// wrong results; order them on one stream.
//
// In host code the array's name is only a stand-in, not a device address.
// The first call on each device (with that device current) resolves the
// device address once with cudaGetSymbolAddress and caches it; that first
// call may load the library's device code, so make it before any stream
// capture begins.  The cached address belongs to the device's primary
// context, the one the CUDA runtime uses: it assumes that context lives as
// long as the process (no cudaDeviceReset while the library is in use).
// It calls no cudaMalloc/cudaFree and no allocating library routine.
#include <cstdio>
#include <mutex>

#include "kernels.cuh"

namespace {

constexpr size_t kScratchFloats = size_t(1) << 20;   // 4 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float g_gram_scratch[kScratchFloats];

std::mutex g_scratch_mu;
float* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_gram_scratch on the current device (resolved once).
int scratch_address(float** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PGB_ECUDA;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_gram_scratch);
    if (e != cudaSuccess || p == nullptr) {
      std::fprintf(stderr, "probit_gb300: cudaGetSymbolAddress(scratch) failed: %s\n", cudaGetErrorString(e));
      return PGB_ECUDA;
    }
    g_scratch_ptr[dev] = static_cast<float*>(p);
  }
  *out = g_scratch_ptr[dev];
  return PGB_OK;
}

}  // namespace

extern "C" int pgb_gram_noalloc(const pgb_desc* desc, const float* theta, const float* X1, int32_t n1,
                                const float* X2, int32_t n2, float* K, int64_t ldk, void* stream) {
  // the same descriptor check and error codes as pgb_gram
  if (pgb::validate_desc(desc) != PGB_OK || !theta || !X1 || !X2 || !K || n1 < 0 || n2 < 0 || ldk < n2)
    return PGB_EINVAL;
  if (n1 == 0 || n2 == 0) return PGB_OK;
  const pgb::Shape sh = pgb::shape_from_desc(desc);
  const size_t need = ((size_t)n1 + (size_t)n2) * (size_t)sh.Dp;
  if (need > kScratchFloats) {
    std::fprintf(stderr,
                 "probit_gb300: pgb_gram_noalloc needs %zu scratch floats for %d + %d points of %d features, "
                 "more than its fixed %zu; use pgb_gram\n",
                 need, n1, n2, sh.Dp, kScratchFloats);
    return PGB_EUNSUPPORTED;
  }
  float* scratch = nullptr;
  const int r = scratch_address(&scratch);
  if (r != PGB_OK) return r;
  float* f1 = scratch;
  float* f2 = scratch + (size_t)n1 * sh.Dp;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  pgb::launch_prep_features_raw(sh, X1, theta, f1, n1, n1, s);
  pgb::launch_prep_features_raw(sh, X2, theta, f2, n2, n2, s);
  pgb::launch_gram_full(sh, theta, f1, n1, f2, n2, K, ldk, s);
  return cudaGetLastError() == cudaSuccess ? PGB_OK : PGB_ECUDA;
}
