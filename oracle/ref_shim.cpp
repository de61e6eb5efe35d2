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
