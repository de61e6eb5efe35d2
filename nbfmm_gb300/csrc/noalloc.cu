// noalloc.cu -- the leaf-cell sort (keys, stable radix sort, heads) for callers that cannot allocate device
// memory.
//
// Who needs it: code whose device memory is owned by someone else -- a host application that hands a plugin
// its buffers and a stream and forbids side allocations -- and code that runs where cudaMalloc/cudaFree are
// not acceptable because they synchronise the device or take a global lock (a latency-bound loop sharing the
// GPU with other streams). nbfmm_solver_create allocates the whole workspace up front; this entry point
// instead keeps its sort scratch in one file-scope device array, so a call allocates nothing at all.
//
// Limits and sharing: at most kNoAllocMaxParticles particles per call (scratch ~4.1 MB, held by every GPU
// that loads the library until the process exits). Every call on a device uses the same array, which keeps
// the last call's contents; nothing in it has to start at zero (each call writes every scratch word it
// reads), but calls that overlap on the GPU -- on two streams, or from two host threads -- race on it.
// The device address of the array belongs to one CUDA context: a context of its own that a host application
// makes current, or the device's primary context after cudaDeviceReset, holds the array at another address.
// So every call looks the address up in the current context with cudaGetSymbolAddress (a query that neither
// allocates nor synchronises) instead of keeping one from an earlier call. The first call on a device also
// loads the library's module there, so it should come before any stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <string>

#include "../../include/nbfmm_gb300.h"
#include "engine.cuh"
#include "stars.cuh"

namespace nbfmm_gb300 {
int api_fail(int code, const char* fmt, ...);
}

#define NBFMM_TRY(expr)              \
  do {                               \
    const int _rc = (expr);          \
    if (_rc != NBFMM_OK) return _rc; \
  } while (0)

namespace {

using namespace nbfmm_gb300;

constexpr int kNoAllocMaxParticles = 1 << 18;
constexpr int kNoAllocMaxTiles = (kNoAllocMaxParticles + kSortTile - 1) / kSortTile;
constexpr int kNoAllocRadix = 1 << kRadixMaxBits;

// Word offsets of the scratch regions inside the array.
constexpr size_t kKeysA = 0;
constexpr size_t kValsA = kKeysA + kNoAllocMaxParticles;
constexpr size_t kKeysB = kValsA + kNoAllocMaxParticles;
constexpr size_t kValsB = kKeysB + kNoAllocMaxParticles;
constexpr size_t kCounts = kValsB + kNoAllocMaxParticles;
constexpr size_t kDigitTotal = kCounts + (size_t)kNoAllocRadix * kNoAllocMaxTiles;
constexpr size_t kCount = kDigitTotal + kNoAllocRadix;
constexpr size_t kScratchWords = kCount + 64;  // the particle count, padded to 256 bytes

static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

// The device address of g_noalloc_scratch in the current context, looked up on every call (see the file comment).
int scratch_address(uint32_t** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    cudaGetLastError();
    return api_fail(NBFMM_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
  }
  *out = static_cast<uint32_t*>(p);
  return NBFMM_OK;
}

}  // namespace

extern "C" int nbfmm_sort_cells_noalloc(int num_level, const float position_limits[4], int num_particle,
                                        const float* gpuptr_position, int* gpuptr_perm, int* gpuptr_head,
                                        void* stream) {
  if (num_level < 0 || num_level > kMaxLevels - 1) {
    return api_fail(NBFMM_ERR_INVALID, "num_level %d outside [0, %d]", num_level, kMaxLevels - 1);
  }
  const float* l = position_limits;
  if (!l || !std::isfinite(l[0]) || !std::isfinite(l[1]) || !std::isfinite(l[2]) || !std::isfinite(l[3]) ||
      !(l[0] < l[2]) || !(l[1] < l[3])) {
    return api_fail(NBFMM_ERR_INVALID, "position limits must be finite with min < max");
  }
  if (num_particle < 0 || num_particle > kNoAllocMaxParticles) {
    return api_fail(NBFMM_ERR_INVALID,
                    "nbfmm_sort_cells_noalloc: %d particles exceed its fixed scratch of %d particles",
                    num_particle, kNoAllocMaxParticles);
  }
  if (!gpuptr_head || (num_particle > 0 && (!gpuptr_position || !gpuptr_perm))) {
    return api_fail(NBFMM_ERR_INVALID, "null device pointer");
  }
  // An error left by the caller's earlier work is reported as such, not as this call's failure.
  const cudaError_t pending = cudaGetLastError();
  if (pending != cudaSuccess) {
    return api_fail(NBFMM_ERR_CUDA, "nbfmm_sort_cells_noalloc: a CUDA error was pending before the call: %s",
                    cudaGetErrorString(pending));
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  uint32_t* scratch = nullptr;
  NBFMM_TRY(scratch_address(&scratch));

  const int B = 1 << (num_level + 1);
  Geometry g{};
  g.xmin = l[0];
  g.ymin = l[1];
  g.xmax = l[2];
  g.ymax = l[3];
  g.cell_x = (l[2] - l[0]) / (float)B;  // predo.cu:112-113
  g.cell_y = (l[3] - l[1]) / (float)B;
  g.num_level = num_level;
  g.base_dim = B;
  int* d_n = reinterpret_cast<int*>(scratch + kCount);
  uint32_t* keys_a = scratch + kKeysA;
  uint32_t* vals_a = scratch + kValsA;
  launch_set_int(d_n, num_particle, s);
  launch_keys_from_positions(g, reinterpret_cast<const float2*>(gpuptr_position), d_n, keys_a, vals_a,
                             kNoAllocMaxParticles, s);
  const int where = launch_radix_sort(keys_a, vals_a, scratch + kKeysB, scratch + kValsB, scratch + kCounts,
                                      scratch + kDigitTotal, d_n, kNoAllocMaxParticles, 2 * (num_level + 1), s);
  const uint32_t* skey = where ? scratch + kKeysB : keys_a;
  const uint32_t* perm = where ? scratch + kValsB : vals_a;
  launch_head(skey, d_n, B * B, gpuptr_head, nullptr, s);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && num_particle > 0) {
    e = cudaMemcpyAsync(gpuptr_perm, perm, (size_t)num_particle * sizeof(int), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) cudaGetLastError();
  }
  if (e != cudaSuccess) return api_fail(NBFMM_ERR_CUDA, "nbfmm_sort_cells_noalloc: %s", cudaGetErrorString(e));
  return NBFMM_OK;
}
