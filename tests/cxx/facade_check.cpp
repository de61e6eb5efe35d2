// Exercises the C++ facade (include/nbfmm_gb300.hpp) the way code written for the reference uses its classes:
// a Solver solve and a Stars run initialised with a reference model, updated and displayed. Prints one line of
// numbers for the GPU test to compare with the same run through the Python API.
#include <cstdio>
#include <vector>

#include "nbfmm_gb300.hpp"

int main() {
  using namespace nbfmm;
  const int n = 4096;
  Stars stars(4, n, 64, 48, 30, 1e-3f, 1.0f, 0.05f, make_float4(-2, -2, 2, 2), make_float4(-1.5f, -1.5f, 1.5f, 1.5f));
  stars.initialize(model::generateDiskCenter, n, make_float2(0.0f, 0.0f), 1.0f, 1e-4f, 5.0f);
  Solver solver(4, n, make_float4(-2, -2, 2, 2));
  void* eff = nullptr;
  check(nbfmm_device_malloc(n * sizeof(float2), &eff));
  solver.solve(n, stars.gpuptr_position_cur_, stars.gpuptr_weight_, static_cast<float2*>(eff));
  std::vector<float> e(2 * n);
  check(nbfmm_memcpy_to_host(e.data(), eff, e.size() * sizeof(float)));
  stars.update(5);
  void* board = nullptr;
  const long long fb = nbfmm_frame_bytes(64, 48);
  check(nbfmm_device_malloc((unsigned long long)fb, &board));
  stars.display(static_cast<uint8_t*>(board));
  std::vector<unsigned char> f((size_t)fb);
  check(nbfmm_memcpy_to_host(f.data(), board, f.size()));
  double es = 0.0;
  for (float v : e) es += v;
  long lit = 0;
  for (int i = 0; i < 64 * 48; ++i) lit += f[i] == 255;
  std::printf("%.9e %d %ld\n", es, stars.num_star(), lit);
  try {
    Solver bad(4, n, make_float4(1, -2, -1, 2));  // x_min > x_max: the reference asserts
    return 2;
  } catch (const Error&) {
  }
  check(nbfmm_device_free(eff));
  check(nbfmm_device_free(board));
  return 0;
}
