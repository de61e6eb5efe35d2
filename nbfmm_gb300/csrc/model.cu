// model.cu -- the reference's initial-condition models on the GPU (include/nbfmm/model/model.hpp:36-233).
//
// Same arguments and the same random stream as the reference: one XORWOW state per particle from
// curand_init(0, idx, 0) and its first curand_uniform draws (source/nbfmm/model/disk.cu:46-47 and siblings).
// The orbit calibration uses the reference's kernel with its fixed softening 0.1
// (include/nbfmm/core/kernel_function.hpp:35), exactly as the reference generators do. Expressions keep the
// reference's precisions (the 1.0 - ... under acos is double, the angles 2 pi u are formed in double) and the
// multiply-adds the CUDA compiler forms from the reference's float2 operators are written as fmaf.
// Differences from the reference: the double-disk offsets are applied for any N (the reference swaps grid and
// block at double_disk.cu:81-86, an invalid launch above 1,048,576 particles), and arguments are validated
// with a status instead of assert.
// nbfmm_model_set_uniforms installs a device array of draws used instead of curand: a checking hook that lets
// the tests compare this arithmetic with a CPU restatement on identical draws.
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <cmath>

#include "../../include/nbfmm_gb300.h"
#include "engine.cuh"

namespace nbfmm_gb300 {
int api_fail(int code, const char* fmt, ...);
}

using namespace nbfmm_gb300;

namespace {

constexpr float kModelEps = 1e-1f;  // kernel_function.hpp:35
constexpr int kMaxDraws = 3;        // draws per particle (rectangle uses 3)

const float* g_uniforms = nullptr;  // [n * kMaxDraws] when set

struct Draws {
  const float* inject;  // or null: curand
  int idx;
  curandState st;
  int k;
  __device__ __forceinline__ void init(const float* u, int i) {
    inject = u;
    idx = i;
    k = 0;
    if (!u) curand_init(0, i, 0, &st);
  }
  __device__ __forceinline__ float next() {
    const float v = inject ? inject[idx * kMaxDraws + k] : curand_uniform(&st);
    ++k;
    return v;
  }
};

// kernelFunction(0, (r, 0), m).x with eps 0.1 (kernel_function.hpp:29-40).
__device__ __forceinline__ float effect_x(float r, float m) {
  const float rr = sqrtf(__fadd_rn(__fmul_rn(r, r), 0.0f));
  const float tmp = __fdiv_rn(m, __fadd_rn(__fmul_rn(__fmul_rn(rr, rr), rr), kModelEps));
  return __fmul_rn(r, tmp);
}

// acos(1.0 - a t t / r / 2) with the float chain and the double subtraction of disk.cu:51.
__device__ __forceinline__ float angle_step(float ax, float tick, float r) {
  const float q = __fdiv_rn(__fdiv_rn(__fmul_rn(__fmul_rn(ax, tick), tick), r), 2.0f);
  return (float)acos(1.0 - (double)q);
}

__device__ __forceinline__ float two_pi_u(float u) { return (float)(2.0 * M_PI * (double)u); }

__device__ __forceinline__ void place(float2* cur, float2* prev, int i, float2 c, float r, float a_cur, float a_prev) {
  cur[i] = make_float2(fmaf(r, cosf(a_cur), c.x), fmaf(r, sinf(a_cur), c.y));
  prev[i] = make_float2(fmaf(r, cosf(a_prev), c.x), fmaf(r, sinf(a_prev), c.y));
}

// circle_center.cu:24-44 (uniform = 0) and circle_uniform_center.cu:24-42 (uniform = 1).
__global__ void circle_kernel(int n, float2 c, float radius, float weight, float center_weight, float dangle,
                              int evenly, const float* inject, float2* cur, float2* prev, float* w) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (i == 0) {
      cur[0] = c;
      prev[0] = c;
      w[0] = center_weight;
      continue;
    }
    float a;
    if (evenly) {
      a = (float)((2.0 * M_PI * (double)i) / (double)n);
    } else {
      Draws d;
      d.init(inject, i);
      a = two_pi_u(d.next());
    }
    place(cur, prev, i, c, radius, a, __fsub_rn(a, dangle));
    w[i] = weight;
  }
}

// disk.cu:30-57 (center = 0, statik = 0), disk_center.cu:30-60 (center = 1), disk_static.cu:30-51 (statik = 1).
__global__ void disk_kernel(int n, float2 c, float max_radius, float weight, float center_weight, float tick,
                            int center, int statik, const float* inject, float2* cur, float2* prev, float* w) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (center && i == 0) {
      cur[0] = c;
      prev[0] = c;
      w[0] = center_weight;
      continue;
    }
    Draws d;
    d.init(inject, i);
    const float radius = __fmul_rn(__fdiv_rn((float)(i + 1), (float)n), max_radius);
    float dangle = 0.0f;
    if (!statik) {
      const float enclosed = center ? __fadd_rn(__fmul_rn(weight, (float)(i - 1)), center_weight)
                                    : __fmul_rn(weight, (float)i);
      dangle = angle_step(effect_x(radius, enclosed), tick, radius);
    }
    const float a = two_pi_u(d.next());
    place(cur, prev, i, c, radius, a, __fsub_rn(a, dangle));
    w[i] = weight;
  }
}

// rectangle.cu:24-44.
__global__ void rectangle_kernel(int n, float2 c, float width, float height, float max_weight, const float* inject,
                                 float2* cur, float2* prev, float* w) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    Draws d;
    d.init(inject, i);
    const float ux = d.next();
    const float uy = d.next();
    const float uw = d.next();
    const float2 p = make_float2(fmaf(__fsub_rn(ux, 0.5f), width, c.x), fmaf(__fsub_rn(uy, 0.5f), height, c.y));
    cur[i] = p;
    prev[i] = p;
    w[i] = __fmul_rn(max_weight, uw);
  }
}

// double_disk.cu:24-34: previous positions shifted by the orbital offset of the disk.
__global__ void shift_kernel(int n, float2 offset, float2* prev) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    prev[i] = make_float2(__fadd_rn(prev[i].x, offset.x), __fadd_rn(prev[i].y, offset.y));
  }
}

int grid_for(int n) {
  long long g = ((long long)n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g));
}

// Host float arithmetic of the reference's host-side code (kernel_function.hpp, double_disk.cu:58-80).
float2 host_kernel(float2 t, float2 s, float m) {
  const float dx = s.x - t.x, dy = s.y - t.y;
  const float r = std::sqrt(dx * dx + dy * dy);
  const float tmp = m / (r * r * r + kModelEps);
  return make_float2(dx * tmp, dy * tmp);
}

float host_angle_step(float ax, float tick, float r) {
  return (float)std::acos(1.0 - (double)(ax * tick * tick / r / 2.0f));
}

// double_disk.cu:58-80: the offset that sets disk 1 on an orbit about the common centre (eccentricity e).
float2 disk_offset(float2 ca, float2 cb, float mass_b, float ra, float tick, float ecc) {
  const float2 e = host_kernel(ca, cb, mass_b);
  const float a = std::sqrt(e.x * e.x + e.y * e.y);
  float2 o = make_float2(-e.y, e.x);
  const float f = std::sqrt(ra / a) * tick / std::exp2(ecc);
  o.x *= f;
  o.y *= f;
  o.x -= e.x * tick * tick * ecc;
  o.y -= e.y * tick * tick * ecc;
  return o;
}

int check(int n, const float* cur, const float* prev, const float* w) {
  if (n <= 0) return api_fail(NBFMM_ERR_INVALID, "num_particle must be > 0 (model asserts)");
  if (!cur || !prev || !w) return api_fail(NBFMM_ERR_INVALID, "null device pointer");
  return NBFMM_OK;
}

int done(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return api_fail(NBFMM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return NBFMM_OK;
}

float2 f2(const float* p) { return make_float2(p[0], p[1]); }

}  // namespace

extern "C" {

int nbfmm_model_set_uniforms(const float* gpuptr_uniforms) {
  g_uniforms = gpuptr_uniforms;
  return NBFMM_OK;
}

int nbfmm_model_circle_center(int n, const float center[2], float radius, float weight, float center_weight,
                              float tick, float* cur, float* prev, float* w, void* stream) {
  if (check(n, cur, prev, w) != NBFMM_OK) return NBFMM_ERR_INVALID;
  if (!(radius > 0.0f) || !(weight > 0.0f)) return api_fail(NBFMM_ERR_INVALID, "radius and weight must be > 0");
  const float dangle = host_angle_step(host_kernel(make_float2(0, 0), make_float2(radius, 0), center_weight).x, tick,
                                       radius);
  circle_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, f2(center), radius, weight, center_weight, dangle, 0,
                                                              g_uniforms, (float2*)cur, (float2*)prev, w);
  return done("nbfmm_model_circle_center");
}

int nbfmm_model_circle_uniform_center(int n, const float center[2], float radius, float weight, float center_weight,
                                      float tick, float* cur, float* prev, float* w, void* stream) {
  if (check(n, cur, prev, w) != NBFMM_OK) return NBFMM_ERR_INVALID;
  const float dangle = host_angle_step(host_kernel(make_float2(0, 0), make_float2(radius, 0), center_weight).x, tick,
                                       radius);
  circle_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, f2(center), radius, weight, center_weight, dangle, 1,
                                                              g_uniforms, (float2*)cur, (float2*)prev, w);
  return done("nbfmm_model_circle_uniform_center");
}

int nbfmm_model_disk(int n, const float center[2], float radius, float weight, float tick, float* cur, float* prev,
                     float* w, void* stream) {
  if (check(n, cur, prev, w) != NBFMM_OK) return NBFMM_ERR_INVALID;
  if (!(radius > 0.0f) || !(weight > 0.0f)) return api_fail(NBFMM_ERR_INVALID, "radius and weight must be > 0");
  disk_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, f2(center), radius, weight, 0.0f, tick, 0, 0,
                                                            g_uniforms, (float2*)cur, (float2*)prev, w);
  return done("nbfmm_model_disk");
}

int nbfmm_model_disk_center(int n, const float center[2], float radius, float weight, float center_weight, float tick,
                            float* cur, float* prev, float* w, void* stream) {
  if (check(n, cur, prev, w) != NBFMM_OK) return NBFMM_ERR_INVALID;
  disk_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, f2(center), radius, weight, center_weight, tick, 1, 0,
                                                            g_uniforms, (float2*)cur, (float2*)prev, w);
  return done("nbfmm_model_disk_center");
}

int nbfmm_model_disk_static(int n, const float center[2], float radius, float weight, float tick, float* cur,
                            float* prev, float* w, void* stream) {
  if (check(n, cur, prev, w) != NBFMM_OK) return NBFMM_ERR_INVALID;
  disk_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, f2(center), radius, weight, 0.0f, tick, 0, 1,
                                                            g_uniforms, (float2*)cur, (float2*)prev, w);
  return done("nbfmm_model_disk_static");
}

int nbfmm_model_double_disk(int n1, int n2, const float center1[2], const float center2[2], float radius1,
                            float radius2, float weight, float eccentricity, float tick, float* cur, float* prev,
                            float* w, void* stream) {
  if (check(n1, cur, prev, w) != NBFMM_OK || check(n2, cur, prev, w) != NBFMM_OK) return NBFMM_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const int rc1 = nbfmm_model_disk(n1, center1, radius1, weight, tick, cur, prev, w, stream);
  if (rc1 != NBFMM_OK) return rc1;
  const float* g = g_uniforms;  // the second disk's draws follow the first's
  if (g) g_uniforms = g + (size_t)n1 * kMaxDraws;
  const int rc2 = nbfmm_model_disk(n2, center2, radius2, weight, tick, cur + 2 * (size_t)n1, prev + 2 * (size_t)n1,
                                   w + n1, stream);
  g_uniforms = g;
  if (rc2 != NBFMM_OK) return rc2;
  const float2 c1 = f2(center1), c2 = f2(center2);
  const float dx = c1.x - c2.x, dy = c1.y - c2.y;
  const float r = std::sqrt(dx * dx + dy * dy);
  const float r1 = r * n2 / (n1 + n2);
  const float r2 = r * n1 / (n1 + n2);
  const float2 o1 = disk_offset(c1, c2, weight * n2, r1, tick, eccentricity);
  const float2 o2 = disk_offset(c2, c1, weight * n1, r2, tick, eccentricity);
  shift_kernel<<<grid_for(n1), 256, 0, s>>>(n1, o1, (float2*)prev);
  shift_kernel<<<grid_for(n2), 256, 0, s>>>(n2, o2, (float2*)prev + n1);
  return done("nbfmm_model_double_disk");
}

int nbfmm_model_double_disk_center(int n1, int n2, const float center1[2], const float center2[2], float radius1,
                                   float radius2, float weight, float center_weight1, float center_weight2,
                                   float eccentricity, float tick, float* cur, float* prev, float* w, void* stream) {
  if (check(n1, cur, prev, w) != NBFMM_OK || check(n2, cur, prev, w) != NBFMM_OK) return NBFMM_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const int rc1 = nbfmm_model_disk_center(n1, center1, radius1, weight, center_weight1, tick, cur, prev, w, stream);
  if (rc1 != NBFMM_OK) return rc1;
  const float* g = g_uniforms;
  if (g) g_uniforms = g + (size_t)n1 * kMaxDraws;
  const int rc2 = nbfmm_model_disk_center(n2, center2, radius2, weight, center_weight2, tick, cur + 2 * (size_t)n1,
                                          prev + 2 * (size_t)n1, w + n1, stream);
  g_uniforms = g;
  if (rc2 != NBFMM_OK) return rc2;
  const float w1 = weight * (n1 - 1) + center_weight1;
  const float w2 = weight * (n2 - 1) + center_weight2;
  const float2 c1 = f2(center1), c2 = f2(center2);
  const float dx = c1.x - c2.x, dy = c1.y - c2.y;
  const float r = std::sqrt(dx * dx + dy * dy);
  const float r1 = r * w2 / (w1 + w2);
  const float r2 = r * w1 / (w1 + w2);
  const float2 o1 = disk_offset(c1, c2, w2, r1, tick, eccentricity);
  const float2 o2 = disk_offset(c2, c1, w1, r2, tick, eccentricity);
  shift_kernel<<<grid_for(n1), 256, 0, s>>>(n1, o1, (float2*)prev);
  shift_kernel<<<grid_for(n2), 256, 0, s>>>(n2, o2, (float2*)prev + n1);
  return done("nbfmm_model_double_disk_center");
}

int nbfmm_model_rectangle(int n, const float center[2], float width, float height, float max_weight, float tick,
                          float* cur, float* prev, float* w, void* stream) {
  (void)tick;
  if (check(n, cur, prev, w) != NBFMM_OK) return NBFMM_ERR_INVALID;
  rectangle_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, f2(center), width, height, max_weight, g_uniforms,
                                                                 (float2*)cur, (float2*)prev, w);
  return done("nbfmm_model_rectangle");
}

}  // extern "C"
