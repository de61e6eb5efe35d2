// nbfmm_gb300.hpp -- header-only C++ facade over the C ABI (nbfmm_gb300.h) with the reference's signatures.
//
// Code written against emfomy/nbfmm's classes compiles against this header and runs on the engine:
//   nbfmm::Solver  (include/nbfmm/core/solver.hpp:80-103)    constructor, solve
//   nbfmm::Stars   (include/nbfmm/display/stars.hpp:90-126)  constructor, public state, initialize, update, display
//   nbfmm::model   (include/nbfmm/model/model.hpp:36-233)    the eight generators, as Stars::initialize expects
// Where the reference asserts, these throw nbfmm::Error with the engine's message. All work is queued on the
// legacy default stream, as the reference's is; update(num_steps) runs several updates without host
// synchronisation in between.
#ifndef NBFMM_GB300_HPP_
#define NBFMM_GB300_HPP_

#include <vector_functions.h>  // make_float2 / make_float4, as reference code gets them from the CUDA runtime
#include <vector_types.h>

#include <cmath>
#include <cstdint>
#include <stdexcept>

#include "nbfmm_gb300.h"

namespace nbfmm {

class Error : public std::runtime_error {
 public:
  explicit Error(const char* what) : std::runtime_error(what) {}
};

inline void check(int rc) {
  if (rc != NBFMM_OK) throw Error(nbfmm_last_error());
}

class Solver {
 public:
  Solver(int num_level, int max_num_particle, float4 position_limits) {
    const float l[4] = {position_limits.x, position_limits.y, position_limits.z, position_limits.w};
    check(nbfmm_solver_create(num_level, max_num_particle, l, &h_));
  }
  ~Solver() { nbfmm_solver_destroy(h_); }
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;

  void solve(int num_particle, const float2* gpuptr_position_origin, const float* gpuptr_weight_origin,
             float2* gpuptr_effect_origin) {
    check(nbfmm_solver_solve(h_, num_particle, reinterpret_cast<const float*>(gpuptr_position_origin),
                             gpuptr_weight_origin, reinterpret_cast<float*>(gpuptr_effect_origin), nullptr));
  }

  // Engine extension: the kernel softening (the reference fixes 1e-1).
  void set_epsilon(float epsilon) { check(nbfmm_solver_set_epsilon(h_, epsilon)); }
  // Engine extension: near-field arithmetic, NBFMM_ARITH_FAST (default) or NBFMM_ARITH_EXACT.
  void set_arithmetic(int arithmetic) { check(nbfmm_solver_set_arithmetic(h_, arithmetic)); }
  nbfmm_solver* handle() { return h_; }

 private:
  nbfmm_solver* h_ = nullptr;
};

class Stars {
 public:
  Stars(int fmm_level, int num_star, int width, int height, int fps, float tick, float grav_const,
        float size_scale, float4 position_limits, float4 display_limits)
      : width_(width), height_(height), fps_(fps), size_scale_(size_scale),
        display_limits_{display_limits.x, display_limits.y, display_limits.z, display_limits.w} {
    if (width <= 0 || height <= 0 || fps <= 0 || !(size_scale > 0.0f)) {
      throw Error("width, height, fps and size_scale must be > 0");
    }
    if (!(display_limits.x < display_limits.z && display_limits.y < display_limits.w)) {
      throw Error("display limits must satisfy x_min < x_max, y_min < y_max");
    }
    const float l[4] = {position_limits.x, position_limits.y, position_limits.z, position_limits.w};
    check(nbfmm_stars_create(fmm_level, num_star, tick, grav_const, l, &h_));
    float *cur = nullptr, *pre = nullptr, *w = nullptr;
    check(nbfmm_stars_state(h_, &cur, &pre, &w));
    gpuptr_position_cur_ = reinterpret_cast<float2*>(cur);
    gpuptr_position_pre_ = reinterpret_cast<float2*>(pre);
    gpuptr_weight_ = w;
    tick_ = tick * std::sqrt(grav_const);  // stars.cu:31, as the engine computes it
  }
  ~Stars() { nbfmm_stars_destroy(h_); }
  Stars(const Stars&) = delete;
  Stars& operator=(const Stars&) = delete;

  // func(args..., tick_, gpuptr_position_cur_, gpuptr_position_pre_, gpuptr_weight_)  (stars.hpp:111-114)
  template <typename Func, typename... Args>
  void initialize(Func func, Args... args) {
    func(args..., tick_, gpuptr_position_cur_, gpuptr_position_pre_, gpuptr_weight_);
  }

  void update() { check(nbfmm_stars_update(h_, 1, nullptr)); }
  void update(int num_steps) { check(nbfmm_stars_update(h_, num_steps, nullptr)); }
  void display(uint8_t* board) {
    check(nbfmm_stars_display(h_, width_, height_, size_scale_, display_limits_, board, nullptr));
  }

  // num_star_ (stars.hpp:34); synchronises.
  int num_star() {
    int n = 0;
    check(nbfmm_stars_num_star(h_, &n));
    return n;
  }
  int fps() const { return fps_; }
  nbfmm_stars* handle() { return h_; }

  float2* gpuptr_position_cur_ = nullptr;
  float2* gpuptr_position_pre_ = nullptr;
  float* gpuptr_weight_ = nullptr;

 private:
  nbfmm_stars* h_ = nullptr;
  int width_, height_, fps_;
  float size_scale_;
  float display_limits_[4];
  float tick_ = 0.0f;
};

namespace model {

inline void generateCircleCenter(int num_particle, float2 center_position, float radius, float weight,
                                 float center_weight, float tick, float2* gpuptr_position_current,
                                 float2* gpuptr_position_previous, float* gpuptr_weight) {
  const float c[2] = {center_position.x, center_position.y};
  check(nbfmm_model_circle_center(num_particle, c, radius, weight, center_weight, tick,
                                  reinterpret_cast<float*>(gpuptr_position_current),
                                  reinterpret_cast<float*>(gpuptr_position_previous), gpuptr_weight, nullptr));
}

inline void generateCircleUniformCenter(int num_particle, float2 center_position, float radius, float weight,
                                        float center_weight, float tick, float2* gpuptr_position_current,
                                        float2* gpuptr_position_previous, float* gpuptr_weight) {
  const float c[2] = {center_position.x, center_position.y};
  check(nbfmm_model_circle_uniform_center(num_particle, c, radius, weight, center_weight, tick,
                                          reinterpret_cast<float*>(gpuptr_position_current),
                                          reinterpret_cast<float*>(gpuptr_position_previous), gpuptr_weight,
                                          nullptr));
}

inline void generateDisk(int num_particle, float2 center_position, float radius, float weight, float tick,
                         float2* gpuptr_position_current, float2* gpuptr_position_previous, float* gpuptr_weight) {
  const float c[2] = {center_position.x, center_position.y};
  check(nbfmm_model_disk(num_particle, c, radius, weight, tick, reinterpret_cast<float*>(gpuptr_position_current),
                         reinterpret_cast<float*>(gpuptr_position_previous), gpuptr_weight, nullptr));
}

inline void generateDiskCenter(int num_particle, float2 center_position, float radius, float weight,
                               float center_weight, float tick, float2* gpuptr_position_current,
                               float2* gpuptr_position_previous, float* gpuptr_weight) {
  const float c[2] = {center_position.x, center_position.y};
  check(nbfmm_model_disk_center(num_particle, c, radius, weight, center_weight, tick,
                                reinterpret_cast<float*>(gpuptr_position_current),
                                reinterpret_cast<float*>(gpuptr_position_previous), gpuptr_weight, nullptr));
}

inline void generateDiskStatic(int num_particle, float2 center_position, float radius, float weight, float tick,
                               float2* gpuptr_position_current, float2* gpuptr_position_previous,
                               float* gpuptr_weight) {
  const float c[2] = {center_position.x, center_position.y};
  check(nbfmm_model_disk_static(num_particle, c, radius, weight, tick,
                                reinterpret_cast<float*>(gpuptr_position_current),
                                reinterpret_cast<float*>(gpuptr_position_previous), gpuptr_weight, nullptr));
}

inline void generateDoubleDisk(int num_particle1, int num_particle2, float2 center_position1,
                               float2 center_position2, float radius1, float radius2, float weight,
                               float eccentricity, float tick, float2* gpuptr_position_current,
                               float2* gpuptr_position_previous, float* gpuptr_weight) {
  const float c1[2] = {center_position1.x, center_position1.y}, c2[2] = {center_position2.x, center_position2.y};
  check(nbfmm_model_double_disk(num_particle1, num_particle2, c1, c2, radius1, radius2, weight, eccentricity, tick,
                                reinterpret_cast<float*>(gpuptr_position_current),
                                reinterpret_cast<float*>(gpuptr_position_previous), gpuptr_weight, nullptr));
}

inline void generateDoubleDiskCenter(int num_particle1, int num_particle2, float2 center_position1,
                                     float2 center_position2, float radius1, float radius2, float weight,
                                     float center_weight1, float center_weight2, float eccentricity, float tick,
                                     float2* gpuptr_position_current, float2* gpuptr_position_previous,
                                     float* gpuptr_weight) {
  const float c1[2] = {center_position1.x, center_position1.y}, c2[2] = {center_position2.x, center_position2.y};
  check(nbfmm_model_double_disk_center(num_particle1, num_particle2, c1, c2, radius1, radius2, weight,
                                       center_weight1, center_weight2, eccentricity, tick,
                                       reinterpret_cast<float*>(gpuptr_position_current),
                                       reinterpret_cast<float*>(gpuptr_position_previous), gpuptr_weight, nullptr));
}

inline void generateRectangle(int num_particle, float2 center_position, float width, float height,
                              float max_weight, float tick, float2* gpuptr_position_current,
                              float2* gpuptr_position_previous, float* gpuptr_weight) {
  const float c[2] = {center_position.x, center_position.y};
  check(nbfmm_model_rectangle(num_particle, c, width, height, max_weight, tick,
                              reinterpret_cast<float*>(gpuptr_position_current),
                              reinterpret_cast<float*>(gpuptr_position_previous), gpuptr_weight, nullptr));
}

}  // namespace model
}  // namespace nbfmm

#endif  // NBFMM_GB300_HPP_
