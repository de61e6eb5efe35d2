// make_golden.cpp -- writes the golden vectors of the reference's per-stage tests.
//
// Rebuilds the fixture of check/core/solver.cu:17-69 (num_level 3, 250 particles, limits [0,8]x[-1,2],
// std::default_random_engine with its default seed, exponential(1) masses, random monotone head, random
// shuffle) and evaluates the known answers that the reference's tests compute on the host:
//   postdo  check/core/solver/postdo.cu:35-37      effect_origin[perm[i]] = effect[i]
//   p2p     check/core/solver/p2p.cu:34-41         O(N^2) sum over |dix|,|diy| <= 1, i != j
//   p2m     check/core/solver/p2m.cu:36-46         leaf centre of mass from head ranges
//   m2m     check/core/solver/m2m.cu:32-48         levels 1..L-1 from level 0
//   m2l     check/core/solver/m2l.cu:34-50         parent-neighbour children minus near cells, every level
//   l2l     check/core/solver/l2l.cu:26-37         parent effects summed down to level 0
//   l2p     check/core/solver/l2p.cu:34-36         particle effect += leaf effect
// The arithmetic is the reference's own: kernelFunction and the float2/int2 operators are included from the
// reference headers. Must be compiled with -std=c++14 (std::random_shuffle) and -ffp-contract=off.
// Usage: make_golden <out_dir>; writes one raw little-endian file per array plus manifest.txt.
#include <cuda_runtime_api.h>
#include <vector_functions.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <random>
#include <string>

#include <nbfmm/core/kernel_function.hpp>
#include <nbfmm/utility/operator.hpp>

namespace {

constexpr int kLevels = 3;
constexpr int kDim = 1 << (kLevels + 1);
constexpr int kN = 250;
constexpr int kCellsP1 = kDim * kDim + 1;

std::string g_dir;
FILE* g_manifest = nullptr;

void dump(const char* name, const char* dtype, const void* data, size_t count, size_t elem) {
  const std::string path = g_dir + "/" + name + ".bin";
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { std::perror(path.c_str()); std::exit(1); }
  std::fwrite(data, elem, count, f);
  std::fclose(f);
  std::fprintf(g_manifest, "%s %s %zu\n", name, dtype, count);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) { std::fprintf(stderr, "usage: %s <out_dir>\n", argv[0]); return 2; }
  g_dir = argv[1];
  g_manifest = std::fopen((g_dir + "/manifest.txt").c_str(), "w");
  if (!g_manifest) { std::perror("manifest"); return 1; }

  const float4 limits = make_float4(0, -1, 8, 2);
  static float2 position[kN];
  static float weight[kN];
  static int2 index[kN];
  static int perm[kN];
  static int head[kCellsP1];
  static float2 cell_position[kLevels][kDim][kDim];
  static float cell_weight[kLevels][kDim][kDim];

  std::default_random_engine generator;
  std::uniform_real_distribution<float> rand_x(limits.x, limits.z);
  std::uniform_real_distribution<float> rand_y(limits.y, limits.w);
  std::exponential_distribution<float> rand_w(1.0);
  std::uniform_int_distribution<int> rand_head(0, 255);

  for (int i = 0; i < kN; ++i) {
    position[i].x = rand_x(generator);
    position[i].y = rand_y(generator);
    weight[i] = rand_w(generator);
  }
  for (int l = 0; l < kLevels; ++l) {
    const int cs = 1 << l;
    for (int j = 0; j < kDim; j += cs) {
      for (int i = 0; i < kDim; i += cs) {
        cell_position[l][j][i].x = rand_x(generator);
        cell_position[l][j][i].y = rand_y(generator);
        cell_weight[l][j][i] = rand_w(generator);
      }
    }
  }
  head[0] = 0;
  int rand_sum = 0;
  for (int i = 1; i < kCellsP1; ++i) {
    rand_sum += rand_head(generator);
    head[i] = rand_sum * kN;
  }
  for (int i = 0; i < kCellsP1; ++i) head[i] /= rand_sum;
  std::iota(perm, perm + kN, 0);
  std::random_shuffle(perm, perm + kN);
  for (int c = 0; c < kDim * kDim; ++c) {
    std::fill(index + head[c], index + head[c + 1], make_int2(c % kDim, c / kDim));
  }

  dump("position", "f4", position, 2 * kN, sizeof(float));
  dump("weight", "f4", weight, kN, sizeof(float));
  dump("index", "i4", index, 2 * kN, sizeof(int));
  dump("perm", "i4", perm, kN, sizeof(int));
  dump("head", "i4", head, kCellsP1, sizeof(int));
  dump("cell_position", "f4", cell_position, 2 * kLevels * kDim * kDim, sizeof(float));
  dump("cell_weight", "f4", cell_weight, kLevels * kDim * kDim, sizeof(float));

  // postdo: effect = position, perm = random perm.
  {
    static float2 out[kN];
    for (int i = 0; i < kN; ++i) out[perm[i]] = position[i];
    dump("postdo_effect_origin", "f4", out, 2 * kN, sizeof(float));
  }
  // p2p on (position, weight, index, head).
  {
    static float2 eff[kN];
    for (int i = 0; i < kN; ++i) {
      eff[i] = make_float2(0.0f, 0.0f);
      for (int j = 0; j < kN; ++j) {
        if (std::abs(index[i].x - index[j].x) <= 1 && std::abs(index[i].y - index[j].y) <= 1 && i != j) {
          eff[i] += nbfmm::kernelFunction(position[i], position[j], weight[j]);
        }
      }
    }
    dump("p2p_effect", "f4", eff, 2 * kN, sizeof(float));
  }
  // p2m on (position, weight, head): level-0 cells.
  {
    static float2 cp[kDim * kDim];
    static float cw[kDim * kDim];
    for (int c = 0; c < kDim * kDim; ++c) {
      cp[c] = make_float2(0, 0);
      cw[c] = 0;
      for (int k = head[c]; k < head[c + 1]; ++k) {
        cp[c] += position[k] * weight[k];
        cw[c] += weight[k];
      }
      if (head[c] != head[c + 1]) cp[c] /= cw[c];
    }
    dump("p2m_cell_position", "f4", cp, 2 * kDim * kDim, sizeof(float));
    dump("p2m_cell_weight", "f4", cw, kDim * kDim, sizeof(float));
  }
  // m2m from level 0 of the random cube.
  {
    static float2 cp[kLevels][kDim][kDim];
    static float cw[kLevels][kDim][kDim];
    std::memcpy(cp, cell_position, sizeof(cp));
    std::memcpy(cw, cell_weight, sizeof(cw));
    for (int l = 1; l < kLevels; ++l) {
      const int cs = 1 << l;
      const int off = cs / 2;
      for (int j = 0; j < kDim; j += cs) {
        for (int i = 0; i < kDim; i += cs) {
          cp[l][j][i] = cp[l - 1][j][i] * cw[l - 1][j][i] + cp[l - 1][j][i + off] * cw[l - 1][j][i + off] +
                        cp[l - 1][j + off][i] * cw[l - 1][j + off][i] +
                        cp[l - 1][j + off][i + off] * cw[l - 1][j + off][i + off];
          cw[l][j][i] = cw[l - 1][j][i] + cw[l - 1][j][i + off] + cw[l - 1][j + off][i] + cw[l - 1][j + off][i + off];
          cp[l][j][i] /= cw[l][j][i];
        }
      }
    }
    dump("m2m_cell_position", "f4", cp, 2 * kLevels * kDim * kDim, sizeof(float));
    dump("m2m_cell_weight", "f4", cw, kLevels * kDim * kDim, sizeof(float));
  }
  // m2l on the full random cube.
  {
    static float2 ce[kLevels][kDim][kDim];
    std::memset(ce, 0, sizeof(ce));
    for (int l = 0; l < kLevels; ++l) {
      const int cs = 1 << l;
      const int ps = cs * 2;
      for (int y = 0; y < kDim; y += cs) {
        const int py = (y / (2 * cs)) * (2 * cs);
        for (int x = 0; x < kDim; x += cs) {
          const int px = (x / (2 * cs)) * (2 * cs);
          ce[l][y][x] = make_float2(0.0f, 0.0f);
          for (int j = 0; j < kDim; j += cs) {
            const int pj = (j / (2 * cs)) * (2 * cs);
            for (int i = 0; i < kDim; i += cs) {
              const int pi = (i / (2 * cs)) * (2 * cs);
              if (std::abs(pi - px) <= ps && std::abs(pj - py) <= ps && (std::abs(i - x) > cs || std::abs(j - y) > cs)) {
                ce[l][y][x] += nbfmm::kernelFunction(cell_position[l][y][x], cell_position[l][j][i], cell_weight[l][j][i]);
              }
            }
          }
        }
      }
    }
    dump("m2l_cell_effect", "f4", ce, 2 * kLevels * kDim * kDim, sizeof(float));
  }
  // l2l with the random cell positions as effects.
  {
    static float2 ce[kLevels][kDim][kDim];
    std::memcpy(ce, cell_position, sizeof(ce));
    for (int l = kLevels - 1; l > 0; --l) {
      const int cs = 1 << l;
      const int off = cs / 2;
      for (int j = 0; j < kDim; j += cs) {
        for (int i = 0; i < kDim; i += cs) {
          ce[l - 1][j][i] += ce[l][j][i];
          ce[l - 1][j][i + off] += ce[l][j][i];
          ce[l - 1][j + off][i] += ce[l][j][i];
          ce[l - 1][j + off][i + off] += ce[l][j][i];
        }
      }
    }
    dump("l2l_cell_effect0", "f4", ce, 2 * kDim * kDim, sizeof(float));
  }
  // l2p: effect = position, cell effect = level 0 of the random cell positions.
  {
    static float2 eff[kN];
    for (int i = 0; i < kN; ++i) eff[i] = position[i] + cell_position[0][index[i].y][index[i].x];
    dump("l2p_effect", "f4", eff, 2 * kN, sizeof(float));
  }
  // kernelFunction samples (eps fixed at 1e-1 in the reference).
  {
    std::mt19937 g2(12345);
    std::uniform_real_distribution<float> u(-2.0f, 2.0f);
    std::uniform_real_distribution<float> um(0.0f, 3.0f);
    constexpr int kS = 4096;
    static float t[2 * kS], s[2 * kS], m[kS], out[2 * kS];
    for (int i = 0; i < kS; ++i) {
      t[2 * i] = u(g2); t[2 * i + 1] = u(g2);
      s[2 * i] = (i % 7 == 0) ? t[2 * i] : u(g2);
      s[2 * i + 1] = (i % 7 == 0) ? t[2 * i + 1] : u(g2);
      m[i] = um(g2);
      const float2 r = nbfmm::kernelFunction(make_float2(t[2 * i], t[2 * i + 1]), make_float2(s[2 * i], s[2 * i + 1]), m[i]);
      out[2 * i] = r.x; out[2 * i + 1] = r.y;
    }
    dump("kf_target", "f4", t, 2 * kS, sizeof(float));
    dump("kf_source", "f4", s, 2 * kS, sizeof(float));
    dump("kf_mass", "f4", m, kS, sizeof(float));
    dump("kf_effect", "f4", out, 2 * kS, sizeof(float));
  }
  std::fclose(g_manifest);
  return 0;
}
