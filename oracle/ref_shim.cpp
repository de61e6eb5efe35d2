// ref_shim.cpp -- compiles the reference's own host/device arithmetic for the CPU (TEST INFRASTRUCTURE ONLY).
//
// Built by oracle/build_ref.sh into oracle/_ref/ when the reference sources are present. It includes the
// reference headers where they lie and exports C wrappers, so the tests can pin the oracle's restatement
// against the reference's compiled code:
//   include/nbfmm/core/kernel_function.hpp:29-40   kernelFunction (eps fixed at 1e-1 there)
//   include/nbfmm/utility/operator.hpp:107-109     int2 operator<  (row-major particle order)
//   include/nbfmm/utility/operator.hpp:87-89       int2 operator== (cell key equality)
//   include/nbfmm/utility/operator.hpp:137-139     float2 operator* (x*m of p2mWeight)
//   source/nbfmm/display/stars/display.cu:29-214   displayDevice, run once per star on the CPU (when the recipe
//                                                  could cut it out of its file into oracle/_ref/)
// Nothing else of the reference is compiled: its stage kernels need a GPU and its CMake does not configure.
#include <cuda_runtime_api.h>
#include <vector_functions.h>

#include <math.h>  // the C++ wrapper: floor/sqrt of a float resolve to the float overloads, as in device code
#include <stdint.h>

#include <cmath>

#include <nbfmm/core/kernel_function.hpp>
#include <nbfmm/utility/operator.hpp>

extern "C" {

void ref_kernel_function(float tx, float ty, float sx, float sy, float m, float* out) {
  const float2 r = nbfmm::kernelFunction(make_float2(tx, ty), make_float2(sx, sy), m);
  out[0] = r.x;
  out[1] = r.y;
}

void ref_kernel_function_batch(int n, const float* t, const float* s, const float* m, float* out) {
  for (int i = 0; i < n; ++i) {
    const float2 r = nbfmm::kernelFunction(make_float2(t[2 * i], t[2 * i + 1]),
                                           make_float2(s[2 * i], s[2 * i + 1]), m[i]);
    out[2 * i] = r.x;
    out[2 * i + 1] = r.y;
  }
}

int ref_int2_less(int ax, int ay, int bx, int by) { return make_int2(ax, ay) < make_int2(bx, by); }

int ref_int2_equal(int ax, int ay, int bx, int by) { return make_int2(ax, ay) == make_int2(bx, by); }

void ref_weighted_position(int n, const float* pos, const float* w, float* out) {
  for (int i = 0; i < n; ++i) {
    const float2 r = make_float2(pos[2 * i], pos[2 * i + 1]) * w[i];
    out[2 * i] = r.x;
    out[2 * i + 1] = r.y;
  }
}

}  // extern "C"

#ifdef NBFMM_REF_DISPLAY
namespace ref_display {
struct Index { unsigned int x; };
static Index threadIdx, blockIdx, blockDim;  // one "thread" per call
#undef __global__
#define __global__
#include "display_device.inc"
#undef __global__
}  // namespace ref_display

extern "C" {

// displayDevice for stars [0, n) on a caller's frame buffer (no clearing; the caller pads it, because the
// reference writes before the frame for stars on its top rows).
void ref_display_device(int n, int width, int height, float size_scale, const float* limits, const float* pos,
                        const float* w, uint8_t* board) {
  ref_display::blockDim.x = 1;
  ref_display::threadIdx.x = 0;
  const float4 lim = make_float4(limits[0], limits[1], limits[2], limits[3]);
  for (int i = 0; i < n; ++i) {
    ref_display::blockIdx.x = (unsigned int)i;
    ref_display::displayDevice(n, width, height, size_scale, lim, reinterpret_cast<const float2*>(pos), w, board);
  }
}

int ref_has_display(void) { return 1; }

}  // extern "C"
#else
extern "C" int ref_has_display(void) { return 0; }
#endif

#ifdef NBFMM_REF_PRUNE
#include <thrust/device_ptr.h>
#include <thrust/find.h>
#include <thrust/iterator/zip_iterator.h>
#include <thrust/sort.h>

#include <memory>

namespace ref_prune_kernel {
struct Index { unsigned int x; };
static Index threadIdx, blockIdx, blockDim;  // one "thread" per call
#undef __global__
#define __global__
#include "prune_device.inc"
#undef __global__
}  // namespace ref_prune_kernel

extern "C" {

// Stars::prune (source/nbfmm/display/stars/prune.cu:47-62) on host arrays: the reference's pruneDevice for every
// star, then the sort_by_key of the flags over the zipped (cur, prev, w) arrays and the find of the first flag
// (prune.cu:58-61), on thrust's host system. Returns the new number of stars.
int ref_prune(int num_star, const float* limits, float* cur, float* prev, float* w) {
  std::unique_ptr<bool[]> elimination(new bool[num_star > 0 ? num_star : 1]);
  const float4 lim = make_float4(limits[0], limits[1], limits[2], limits[3]);
  ref_prune_kernel::blockDim.x = 1;
  ref_prune_kernel::threadIdx.x = 0;
  for (int i = 0; i < num_star; ++i) {
    ref_prune_kernel::blockIdx.x = (unsigned int)i;
    ref_prune_kernel::pruneDevice(num_star, lim, reinterpret_cast<const float2*>(cur), elimination.get());
  }
  thrust::device_ptr<float2> thrust_position_cur(reinterpret_cast<float2*>(cur));
  thrust::device_ptr<float2> thrust_position_pre(reinterpret_cast<float2*>(prev));
  thrust::device_ptr<float> thrust_weight(w);
  thrust::device_ptr<bool> thrust_elimination(elimination.get());
  thrust::zip_iterator<thrust::tuple<thrust::device_ptr<float2>, thrust::device_ptr<float2>, thrust::device_ptr<float>>>
      iter(thrust::make_tuple(thrust_position_cur, thrust_position_pre, thrust_weight));
  thrust::sort_by_key(thrust_elimination, thrust_elimination + num_star, iter);
  return (int)(thrust::find(thrust_elimination, thrust_elimination + num_star, 1) - thrust_elimination);
}

int ref_has_prune(void) { return 1; }

}  // extern "C"
#else
extern "C" int ref_has_prune(void) { return 0; }
#endif

#ifdef NBFMM_REF_MODELS
namespace ref_model {
struct Index { unsigned int x; };
static Index threadIdx, blockIdx, blockDim;  // one "thread" per call
// curand_init(0, idx, 0, &s) and curand_uniform(&s) bound to the caller's draws: three per particle idx, taken in
// call order, so the kernels' arithmetic can be compared on identical draws.
struct curandState {
  const float* u;
  int k;
};
static const float* g_draws = nullptr;
static inline void curand_init(unsigned long long, unsigned long long sequence, unsigned long long, curandState* s) {
  s->u = g_draws + 3 * sequence;
  s->k = 0;
}
static inline float curand_uniform(curandState* s) { return s->u[s->k++]; }
using nbfmm::kernelFunction;
#undef __global__
#define __global__
#include "model_circle_center.inc"
#include "model_circle_uniform_center.inc"
#include "model_disk.inc"
#include "model_disk_center.inc"
#include "model_disk_static.inc"
#include "model_rectangle.inc"
#undef __global__

template <class F>
void each_thread(int n, F f) {
  blockDim.x = 1;
  threadIdx.x = 0;
  for (int i = 0; i < n; ++i) {
    blockIdx.x = (unsigned int)i;
    f();
  }
}
}  // namespace ref_model

extern "C" {

// The generators of source/nbfmm/model/*.cu, one kernel "thread" per particle, on draws[3 * n]. The circle models
// compute their angle step with the two host lines of their wrappers (circle_center.cu:85-86,
// circle_uniform_center.cu), included under the wrappers' own parameter names.
void ref_model_circle_center(int num_particle, float cx, float cy, float radius, float weight, float center_weight,
                             float tick, const float* draws, float* cur, float* prev, float* w) {
  using namespace ref_model;
#include "model_circle_center_host.inc"
  g_draws = draws;
  each_thread(num_particle, [&] {
    generateCircleCenterDevice(num_particle, make_float2(cx, cy), radius, weight, center_weight, angle_difference,
                               reinterpret_cast<float2*>(cur), reinterpret_cast<float2*>(prev), w);
  });
}

void ref_model_circle_uniform_center(int num_particle, float cx, float cy, float radius, float weight,
                                     float center_weight, float tick, const float* draws, float* cur, float* prev,
                                     float* w) {
  using namespace ref_model;
#include "model_circle_uniform_center_host.inc"
  g_draws = draws;
  each_thread(num_particle, [&] {
    generateCircleUniformCenterDevice(num_particle, make_float2(cx, cy), radius, weight, center_weight,
                                      angle_difference, reinterpret_cast<float2*>(cur),
                                      reinterpret_cast<float2*>(prev), w);
  });
}

void ref_model_disk(int num_particle, float cx, float cy, float radius, float weight, float tick, const float* draws,
                    float* cur, float* prev, float* w) {
  ref_model::g_draws = draws;
  ref_model::each_thread(num_particle, [&] {
    ref_model::generateDiskDevice(num_particle, make_float2(cx, cy), radius, weight, tick,
                                  reinterpret_cast<float2*>(cur), reinterpret_cast<float2*>(prev), w);
  });
}

void ref_model_disk_center(int num_particle, float cx, float cy, float radius, float weight, float center_weight,
                           float tick, const float* draws, float* cur, float* prev, float* w) {
  ref_model::g_draws = draws;
  ref_model::each_thread(num_particle, [&] {
    ref_model::generateDiskCenterDevice(num_particle, make_float2(cx, cy), radius, weight, center_weight, tick,
                                        reinterpret_cast<float2*>(cur), reinterpret_cast<float2*>(prev), w);
  });
}

void ref_model_disk_static(int num_particle, float cx, float cy, float radius, float weight, const float* draws,
                           float* cur, float* prev, float* w) {
  ref_model::g_draws = draws;
  ref_model::each_thread(num_particle, [&] {
    ref_model::generateDiskStaticDevice(num_particle, make_float2(cx, cy), radius, weight,
                                        reinterpret_cast<float2*>(cur), reinterpret_cast<float2*>(prev), w);
  });
}

void ref_model_rectangle(int num_particle, float cx, float cy, float width, float height, float max_weight,
                         float tick, const float* draws, float* cur, float* prev, float* w) {
  ref_model::g_draws = draws;
  ref_model::each_thread(num_particle, [&] {
    ref_model::generateRectangleDevice(num_particle, make_float2(cx, cy), width, height, max_weight, tick,
                                       reinterpret_cast<float2*>(cur), reinterpret_cast<float2*>(prev), w);
  });
}

int ref_has_models(void) { return 1; }

}  // extern "C"
#else
extern "C" int ref_has_models(void) { return 0; }
#endif
