// ref_shim.cpp -- compiles the reference's own host/device arithmetic for the CPU (TEST INFRASTRUCTURE ONLY).
//
// Built by oracle/build_ref.sh into oracle/_ref/ when the reference sources are present. It includes the
// reference headers where they lie and exports C wrappers, so the tests can pin the oracle's restatement
// against the reference's compiled code:
//   include/nbfmm/core/kernel_function.hpp:29-40   kernelFunction (eps fixed at 1e-1 there)
//   include/nbfmm/utility/operator.hpp:107-109     int2 operator<  (row-major particle order)
//   include/nbfmm/utility/operator.hpp:87-89       int2 operator== (cell key equality)
//   include/nbfmm/utility/operator.hpp:137-139     float2 operator* (x*m of p2mWeight)
// Nothing else of the reference is compiled: its stage kernels need a GPU and its CMake does not configure.
#include <cuda_runtime_api.h>
#include <vector_functions.h>

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
