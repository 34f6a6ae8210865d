// Host-side tensor maps for the tensor-core operand loads.
//
// Every matrix the factorisation reads through the tensor-copy unit (L, the
// right-hand-side rows, the inverses of the diagonal tiles, L^-T) is a
// row-major fp32 array with a row stride that is a multiple of 128 floats;
// its map describes 128-row x CHUNK_COLS-column boxes stored with the
// swizzle of that row width (64 or 128 bytes), the K-major swizzled operand
// layout of tcgen05.mma.  The encoder is the driver's cuTensorMapEncodeTiled, reached
// through the runtime's driver entry point so the library needs no link-time
// dependency on libcuda.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdio>
#include <mutex>

#include "kernels.cuh"

namespace pgb {

namespace {

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

void resolve_encoder() {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
    std::fprintf(stderr, "probit_gb300: cuTensorMapEncodeTiled unavailable (%s)\n", cudaGetErrorString(e));
    cudaGetLastError();
    return;
  }
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
}

}  // namespace

bool make_tile_map(void* map128, const float* base, long long rows, long long cols, long long ld) {
  std::call_once(g_encode_once, resolve_encoder);
  if (!g_encode || !map128 || !base || rows < T || cols < 32 || ld < cols || (ld % 4) != 0) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)CHUNK_COLS, (cuuint32_t)T};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = g_encode(static_cast<CUtensorMap*>(map128), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                              const_cast<float*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                              CHUNK_COLS == 32 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    std::fprintf(stderr, "probit_gb300: cuTensorMapEncodeTiled failed (%d) for a %lld x %lld matrix\n", (int)r, rows,
                 cols);
    return false;
  }
  return true;
}

}  // namespace pgb
