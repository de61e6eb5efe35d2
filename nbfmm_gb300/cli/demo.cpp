// demo.cpp -- nbfmm_demo: the reference's demo program (main/demo.cu) on the GB300 engine.
//
// 250 particles in [0, 8] x [-1, 3] drawn with std::default_random_engine (uniform positions, exponential
// weights), their effects by the direct sum on the host and by the engine's solve, printed side by side with
// each particle's leaf cell, in the format of demo.cu:85-91.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <random>
#include <vector>

#include "nbfmm_gb300.h"

using namespace std;

namespace {

void check(int rc, const char* what) {
  if (rc != NBFMM_OK) {
    fflush(stdout);
    fprintf(stderr, "%s: %s\n", what, nbfmm_last_error());
    abort();
  }
}

// The gravitational kernel with the reference's fixed softening (kernel_function.hpp:29-40), on the host.
void kernel(float tx, float ty, float sx, float sy, float m, float* ax, float* ay) {
  const float dx = sx - tx, dy = sy - ty;
  const float r = std::sqrt(dx * dx + dy * dy);
  const float s = m / (r * r * r + 1e-1f);
  *ax = dx * s;
  *ay = dy * s;
}

}  // namespace

int main() {
  cout << "NBFMM " << 1 << "." << 2 << "." << 0 << " demo" << endl << endl;

  const int num_level = 4;
  const int max_num_particle = 256;
  const int num_particle = 250;
  const float limits[4] = {0, -1, 8, 3};

  nbfmm_solver* solver = nullptr;
  check(nbfmm_solver_create(num_level, max_num_particle, limits, &solver), "Solver");

  vector<float> position(2 * max_num_particle), effect0(2 * max_num_particle), effect(2 * max_num_particle);
  vector<float> weight(max_num_particle);
  void *gpuptr_position = nullptr, *gpuptr_effect = nullptr, *gpuptr_weight = nullptr;
  check(nbfmm_device_malloc(max_num_particle * 2 * sizeof(float), &gpuptr_position), "malloc");
  check(nbfmm_device_malloc(max_num_particle * 2 * sizeof(float), &gpuptr_effect), "malloc");
  check(nbfmm_device_malloc(max_num_particle * sizeof(float), &gpuptr_weight), "malloc");

  default_random_engine generator;
  uniform_real_distribution<float> position_x_rand(limits[0], limits[2]);
  uniform_real_distribution<float> position_y_rand(limits[1], limits[3]);
  exponential_distribution<float> weight_rand(1.0);
  for (int i = 0; i < num_particle; ++i) {
    position[2 * i] = position_x_rand(generator);
    position[2 * i + 1] = position_y_rand(generator);
    weight[i] = weight_rand(generator);
  }

  for (int i = 0; i < num_particle; ++i) {
    float ex = 0.0f, ey = 0.0f;
    for (int j = 0; j < num_particle; ++j) {
      if (i != j) {
        float ax, ay;
        kernel(position[2 * i], position[2 * i + 1], position[2 * j], position[2 * j + 1], weight[j], &ax, &ay);
        ex += ax;
        ey += ay;
      }
    }
    effect0[2 * i] = ex;
    effect0[2 * i + 1] = ey;
  }

  check(nbfmm_memcpy_to_device(gpuptr_position, position.data(), num_particle * 2 * sizeof(float)), "copy");
  check(nbfmm_memcpy_to_device(gpuptr_weight, weight.data(), num_particle * sizeof(float)), "copy");
  check(nbfmm_solver_solve(solver, num_particle, (const float*)gpuptr_position, (const float*)gpuptr_weight,
                           (float*)gpuptr_effect, nullptr),
        "solve");
  check(nbfmm_memcpy_to_host(effect.data(), gpuptr_effect, num_particle * 2 * sizeof(float)), "copy");

  // The leaf cell of each particle in the caller's order (the reference's gpuptr_index_ through gpuptr_perm_).
  nbfmm_solver_buffers buf;
  check(nbfmm_solver_get_buffers(solver, &buf), "buffers");
  vector<unsigned int> key(num_particle), perm(num_particle);
  check(nbfmm_memcpy_to_host(key.data(), buf.cell_key, num_particle * sizeof(unsigned int)), "copy");
  check(nbfmm_memcpy_to_host(perm.data(), buf.perm, num_particle * sizeof(unsigned int)), "copy");
  vector<int> index(2 * num_particle);
  for (int i = 0; i < num_particle; ++i) {
    index[2 * perm[i]] = (int)(key[i] % (unsigned int)buf.base_dim);
    index[2 * perm[i] + 1] = (int)(key[i] / (unsigned int)buf.base_dim);
  }

  printf("    Position\t\t\t    Weight\t    Index\t    Effect(CPU)\t\t\t    Effect(FMM)\n");
  for (int i = 0; i < num_particle; ++i) {
    printf("(%12.4f, %12.4f) \t%12.4f \t(%4d, %4d) \t(%12.4f, %12.4f) \t(%12.4f, %12.4f)\n", position[2 * i],
           position[2 * i + 1], weight[i], index[2 * i], index[2 * i + 1], effect0[2 * i], effect0[2 * i + 1],
           effect[2 * i], effect[2 * i + 1]);
  }
  printf("\n");

  check(nbfmm_device_free(gpuptr_position), "free");
  check(nbfmm_device_free(gpuptr_effect), "free");
  check(nbfmm_device_free(gpuptr_weight), "free");
  check(nbfmm_solver_destroy(solver), "Solver");
  return 0;
}
