/*
 * nbfmm_oracle.c -- CPU restatement of the nbfmm 2D monopole FMM (TEST INFRASTRUCTURE ONLY).
 *
 * Only the tests, __graft_entry__.smoke() and the CPU-baseline leg of bench.py load this library, and only
 * as the checker; the engine never calls it. See nbfmm_oracle.h for the stage list, the reference lines each
 * function follows, and the three reference defects that are neutralised here.
 *
 * Built with -ffp-contract=off so that x86 and Arm hosts round identically; where the engine fuses a
 * multiply-add on purpose the restatement calls fmaf() explicitly.
 */
#include "nbfmm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* include/nbfmm/core/kernel_function.hpp:29-40. The reference fixes eps = 1e-1; here it is a parameter. */
void orc_kernel_function(float tx, float ty, float sx, float sy, float m, float eps, float* ax, float* ay) {
  const float dx = sx - tx;
  const float dy = sy - ty;
  const float r = sqrtf(dx * dx + dy * dy);
  const float tmp = m / (r * r * r + eps);
  *ax = dx * tmp;
  *ay = dy * tmp;
}

int orc_base_dim(int num_level) { return 1 << (num_level + 1); }

/* predo.cu:37-38 with the cell size of predo.cu:112-113 (a float divided by the int base_dim). */
static inline int cell_coord(float v, float lo, float cell, int dim) {
  const float f = floorf((v - lo) / cell);
  if (!(f >= 0.0f)) return 0;            /* NaN and values below the domain land in cell 0 */
  if (f >= (float)dim) return dim - 1;   /* the upper edge and beyond land in the last cell */
  return (int)f;
}

void orc_cell_index(const float limits[4], int base_dim, float x, float y, int* ix, int* iy) {
  const float cx = (limits[2] - limits[0]) / (float)base_dim;
  const float cy = (limits[3] - limits[1]) / (float)base_dim;
  *ix = cell_coord(x, limits[0], cx, base_dim);
  *iy = cell_coord(y, limits[1], cy, base_dim);
}

/*
 * predo.cu:105-135. The reference sorts int2 keys with thrust::sort_by_key under the row-major operator<
 * (operator.hpp:107-109: y first, then x); cub's merge sort keeps equal keys in input order, so the result
 * equals a stable counting sort on key = iy*B + ix, which is what this does. head[c] is the first sorted
 * index whose key is >= c (extractHead, predo.cu:49-74, with every entry written).
 */
void orc_predo(int n, int num_level, const float limits[4], const float* pos, const float* w,
               int* index, int* perm, int* head, float* pos_sorted, float* w_sorted) {
  const int B = orc_base_dim(num_level);
  const int C = B * B;
  int* key = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  int* cnt = (int*)calloc((size_t)C + 1, sizeof(int));
  for (int i = 0; i < n; ++i) {
    int ix, iy;
    orc_cell_index(limits, B, pos[2 * i], pos[2 * i + 1], &ix, &iy);
    key[i] = ix + iy * B;
    cnt[key[i]]++;
  }
  int run = 0;
  for (int c = 0; c < C; ++c) {
    head[c] = run;
    run += cnt[c];
  }
  head[C] = run;
  for (int c = 0; c < C; ++c) cnt[c] = head[c];
  for (int i = 0; i < n; ++i) perm[cnt[key[i]]++] = i; /* stable: input order within a cell */
  for (int i = 0; i < n; ++i) {
    const int p = perm[i];
    index[2 * i] = key[p] % B;
    index[2 * i + 1] = key[p] / B;
    pos_sorted[2 * i] = pos[2 * p];
    pos_sorted[2 * i + 1] = pos[2 * p + 1];
    w_sorted[i] = w[p];
  }
  free(key);
  free(cnt);
}

/* p2p.cu:30-69 (p2pNaive): rows y-1..y+1, cells x-1..x+1, particles in sorted order, self skipped. */
void orc_p2p_naive(int n, int base_dim, const float* pos, const float* w, const int* index, const int* head,
                   float eps, float* eff) {
  const int B = base_dim;
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; ++i) {
    const int px = index[2 * i], py = index[2 * i + 1];
    const float tx = pos[2 * i], ty = pos[2 * i + 1];
    float ex = 0.0f, ey = 0.0f;
    for (int y = py - 1; y <= py + 1; ++y) {
      for (int x = px - 1; x <= px + 1; ++x) {
        if (x < 0 || x >= B || y < 0 || y >= B) continue;
        const int c = x + y * B;
        for (int k = head[c]; k < head[c + 1]; ++k) {
          if (k == i) continue;
          float ax, ay;
          orc_kernel_function(tx, ty, pos[2 * k], pos[2 * k + 1], w[k], eps, &ax, &ay);
          ex += ax;
          ey += ay;
        }
      }
    }
    eff[2 * i] = ex;
    eff[2 * i + 1] = ey;
  }
}

/* p2p.cu:82-161 (p2pBlock): per row a contiguous range, 64-wide chunks, tree reduction per chunk. */
void orc_p2p_block(int n, int base_dim, const float* pos, const float* w, const int* index, const int* head,
                   float eps, float* eff) {
  const int B = base_dim;
  enum { kChunk = 64 };
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < n; ++i) {
    const int px = index[2 * i], py = index[2 * i + 1];
    const float tx = pos[2 * i], ty = pos[2 * i + 1];
    const int left = (px - 1 > 0) ? px - 1 : 0;
    const int right = (px + 1 < B) ? px + 1 : B - 1;
    float ex = 0.0f, ey = 0.0f;
    float tmpx[kChunk], tmpy[kChunk];
    for (int row = 0; row < 3; ++row) {
      const int y = py + row - 1;
      int start = 0, end = 0;
      if (y >= 0 && y < B) {
        start = head[left + y * B];
        end = head[right + y * B + 1];
      }
      const int loops = (end - start) / kChunk + 1;
      for (int l = 0; l < loops; ++l) {
        for (int r = 0; r < kChunk; ++r) {
          const int k = start + l * kChunk + r;
          if (k < end && k != i) {
            orc_kernel_function(tx, ty, pos[2 * k], pos[2 * k + 1], w[k], eps, &tmpx[r], &tmpy[r]);
          } else {
            tmpx[r] = 0.0f;
            tmpy[r] = 0.0f;
          }
        }
        for (int half = kChunk / 2; half >= 1; half /= 2) {
          for (int r = 0; r < half; ++r) {
            tmpx[r] += tmpx[r + half];
            tmpy[r] += tmpy[r + half];
          }
        }
        ex += tmpx[0];
        ey += tmpy[0];
      }
    }
    eff[2 * i] = ex;
    eff[2 * i + 1] = ey;
  }
}

/* p2m: p2mWeight (p2m.cu:24-35) forms x*m; the per-cell sums follow check/core/solver/p2m.cu:36-46
 * (sequential in sorted order); the centre of mass is (sum x*m) / (sum m) per component (p2m.cu:72). */
void orc_p2m(int n, int base_dim, const float* pos, const float* w, const int* head,
             float* cell_pos, float* cell_w) {
  const int C = base_dim * base_dim;
  (void)n;
  for (int c = 0; c < C; ++c) {
    float sx = 0.0f, sy = 0.0f, sw = 0.0f;
    for (int k = head[c]; k < head[c + 1]; ++k) {
      sx += pos[2 * k] * w[k];
      sy += pos[2 * k + 1] * w[k];
      sw += w[k];
    }
    if (head[c] != head[c + 1]) {
      sx = sx / sw;
      sy = sy / sw;
    }
    cell_pos[2 * c] = sx;
    cell_pos[2 * c + 1] = sy;
    cell_w[c] = sw;
  }
}

/* m2m.cu:22-74: parent = mass-weighted mean of its 4 children, summed left to right. */
void orc_m2m(int num_level, int base_dim, float* cell_pos, float* cell_w) {
  const int B = base_dim;
  if (num_level <= 1) return;
  for (int level = 1; level < num_level; ++level) {
    const int cs = 1 << level;
    const int ld = B / cs;
    float* lp = cell_pos + 2 * (size_t)level * B * B;
    float* lw = cell_w + (size_t)level * B * B;
    for (int ty = 0; ty < ld; ++ty) {
      for (int tx = 0; tx < ld; ++tx) {
        const int idx = (tx + ty * B) * cs;
        const int ch = idx - B * B;
        const int ox = cs / 2;
        const int oy = ox * B;
        const int c[4] = {ch, ch + ox, ch + oy, ch + ox + oy};
        float px = lp[2 * c[0]] * lw[c[0]];
        float py = lp[2 * c[0] + 1] * lw[c[0]];
        float ww = lw[c[0]];
        for (int q = 1; q < 4; ++q) {
          px = px + lp[2 * c[q]] * lw[c[q]];
          py = py + lp[2 * c[q] + 1] * lw[c[q]];
          ww = ww + lw[c[q]];
        }
        if (ww == 0.0f) {
          lp[2 * idx] = 0.0f;
          lp[2 * idx + 1] = 0.0f;
        } else {
          lp[2 * idx] = px / ww;
          lp[2 * idx + 1] = py / ww;
        }
        lw[idx] = ww;
      }
    }
  }
}

/* m2l.cu:24-81: sources are the 6x6 children of the parent's 3x3 neighbours minus the target's 3x3. */
void orc_m2l(int num_level, int base_dim, const float* cell_pos, const float* cell_w, float eps, float* cell_eff) {
  const int B = base_dim;
  if (num_level <= 0) return;
  for (int level = 0; level < num_level; ++level) {
    const int cs = 1 << level;
    const int ld = B >> level;
    const float* lp = cell_pos + 2 * (size_t)level * B * B;
    const float* lw = cell_w + (size_t)level * B * B;
    float* le = cell_eff + 2 * (size_t)level * B * B;
#pragma omp parallel for schedule(static)
    for (int ty = 0; ty < ld; ++ty) {
      for (int tx = 0; tx < ld; ++tx) {
        const int px = tx & ~1, py = ty & ~1;
        const int tidx = (tx + ty * B) * cs;
        const float tpx = lp[2 * tidx], tpy = lp[2 * tidx + 1];
        float ex = 0.0f, ey = 0.0f;
        for (int y = py - 2; y < py + 4; ++y) {
          if (y < 0 || y >= ld) continue;
          for (int x = px - 2; x < px + 4; ++x) {
            if (x < 0 || x >= ld) continue;
            if (abs(x - tx) > 1 || abs(y - ty) > 1) {
              const int idx = (x + y * B) * cs;
              float ax, ay;
              orc_kernel_function(tpx, tpy, lp[2 * idx], lp[2 * idx + 1], lw[idx], eps, &ax, &ay);
              ex += ax;
              ey += ay;
            }
          }
        }
        le[2 * tidx] = ex;
        le[2 * tidx + 1] = ey;
      }
    }
  }
}

/* l2l.cu:21-56: from level L-2 down to 0, each cell adds its parent's effect. */
void orc_l2l(int num_level, int base_dim, float* cell_eff) {
  const int B = base_dim;
  if (num_level <= 1) return;
  for (int level = num_level - 2; level >= 0; --level) {
    const int cs = 1 << level;
    const int ld = B / cs;
    float* le = cell_eff + 2 * (size_t)level * B * B;
    for (int ty = 0; ty < ld; ++ty) {
      for (int tx = 0; tx < ld; ++tx) {
        const int idx = (tx + ty * B) * cs;
        const int par = ((tx & ~1) + (ty & ~1) * B) * cs + B * B;
        le[2 * idx] += le[2 * par];
        le[2 * idx + 1] += le[2 * par + 1];
      }
    }
  }
}

/* l2p.cu:23-48 (run for every N; the reference's launch fails above N = 1,048,576). */
void orc_l2p(int n, int base_dim, const int* index, const float* cell_eff, float* eff) {
  for (int i = 0; i < n; ++i) {
    const int c = index[2 * i] + index[2 * i + 1] * base_dim;
    eff[2 * i] += cell_eff[2 * c];
    eff[2 * i + 1] += cell_eff[2 * c + 1];
  }
}

/* postdo.cu:22-45. */
void orc_postdo(int n, const int* perm, const float* eff, float* eff_origin) {
  for (int i = 0; i < n; ++i) {
    eff_origin[2 * perm[i]] = eff[2 * i];
    eff_origin[2 * perm[i] + 1] = eff[2 * i + 1];
  }
}

/* solve.cu:11-27: predo, p2p, p2m, m2m, m2l, l2l, l2p, postdo. */
int orc_solve(int n, int num_level, const float limits[4], float eps, int p2p_block,
              const float* pos, const float* w, float* eff) {
  if (n <= 0) return 0;
  const int B = orc_base_dim(num_level);
  const size_t C = (size_t)B * B;
  const size_t levels = num_level < 2 ? 2 : (size_t)num_level;
  int* index = (int*)malloc(sizeof(int) * 2 * (size_t)n);
  int* perm = (int*)malloc(sizeof(int) * (size_t)n);
  int* head = (int*)malloc(sizeof(int) * (C + 1));
  float* ps = (float*)malloc(sizeof(float) * 2 * (size_t)n);
  float* ws = (float*)malloc(sizeof(float) * (size_t)n);
  float* es = (float*)malloc(sizeof(float) * 2 * (size_t)n);
  float* cp = (float*)calloc(2 * C * levels, sizeof(float));
  float* cw = (float*)calloc(C * levels, sizeof(float));
  float* ce = (float*)calloc(2 * C * levels, sizeof(float));
  if (!index || !perm || !head || !ps || !ws || !es || !cp || !cw || !ce) {
    free(index); free(perm); free(head); free(ps); free(ws); free(es); free(cp); free(cw); free(ce);
    return -1;
  }
  orc_predo(n, num_level, limits, pos, w, index, perm, head, ps, ws);
  if (p2p_block) {
    orc_p2p_block(n, B, ps, ws, index, head, eps, es);
  } else {
    orc_p2p_naive(n, B, ps, ws, index, head, eps, es);
  }
  if (num_level > 0) {
    orc_p2m(n, B, ps, ws, head, cp, cw);
    orc_m2m(num_level, B, cp, cw);
    orc_m2l(num_level, B, cp, cw, eps, ce);
    orc_l2l(num_level, B, ce);
    orc_l2p(n, B, index, ce, es);
  }
  orc_postdo(n, perm, es, eff);
  free(index); free(perm); free(head); free(ps); free(ws); free(es); free(cp); free(cw); free(ce);
  return 0;
}

/* The solve restricted to a list of targets (original indices): the tree is built in full, P2P and L2P
 * run for the listed particles only, in p2pNaive order. eff receives 2 floats per listed target. */
int orc_solve_targets(int n, int num_level, const float limits[4], float eps, const float* pos, const float* w,
                      const int* targets, int n_targets, float* eff) {
  if (n <= 0) return 0;
  const int B = orc_base_dim(num_level);
  const size_t C = (size_t)B * B;
  const size_t levels = num_level < 2 ? 2 : (size_t)num_level;
  int* index = (int*)malloc(sizeof(int) * 2 * (size_t)n);
  int* perm = (int*)malloc(sizeof(int) * (size_t)n);
  int* inv = (int*)malloc(sizeof(int) * (size_t)n);
  int* head = (int*)malloc(sizeof(int) * (C + 1));
  float* ps = (float*)malloc(sizeof(float) * 2 * (size_t)n);
  float* ws = (float*)malloc(sizeof(float) * (size_t)n);
  float* cp = (float*)calloc(2 * C * levels, sizeof(float));
  float* cw = (float*)calloc(C * levels, sizeof(float));
  float* ce = (float*)calloc(2 * C * levels, sizeof(float));
  if (!index || !perm || !inv || !head || !ps || !ws || !cp || !cw || !ce) {
    free(index); free(perm); free(inv); free(head); free(ps); free(ws); free(cp); free(cw); free(ce);
    return -1;
  }
  orc_predo(n, num_level, limits, pos, w, index, perm, head, ps, ws);
  for (int i = 0; i < n; ++i) inv[perm[i]] = i;
  if (num_level > 0) {
    orc_p2m(n, B, ps, ws, head, cp, cw);
    orc_m2m(num_level, B, cp, cw);
    orc_m2l(num_level, B, cp, cw, eps, ce);
    orc_l2l(num_level, B, ce);
  }
#pragma omp parallel for schedule(dynamic, 16)
  for (int t = 0; t < n_targets; ++t) {
    const int i = inv[targets[t]];
    const int px = index[2 * i], py = index[2 * i + 1];
    float ex = 0.0f, ey = 0.0f;
    for (int y = py - 1; y <= py + 1; ++y) {
      for (int x = px - 1; x <= px + 1; ++x) {
        if (x < 0 || x >= B || y < 0 || y >= B) continue;
        const int c = x + y * B;
        for (int k = head[c]; k < head[c + 1]; ++k) {
          if (k == i) continue;
          float ax, ay;
          orc_kernel_function(ps[2 * i], ps[2 * i + 1], ps[2 * k], ps[2 * k + 1], ws[k], eps, &ax, &ay);
          ex += ax;
          ey += ay;
        }
      }
    }
    if (num_level > 0) {
      ex += ce[2 * (px + py * B)];
      ey += ce[2 * (px + py * B) + 1];
    }
    eff[2 * t] = ex;
    eff[2 * t + 1] = ey;
  }
  free(index); free(perm); free(inv); free(head); free(ps); free(ws); free(cp); free(cw); free(ce);
  return 0;
}

/* update.cu:26-55 and prune.cu:28-62. The position update 2x - x_prev + a*tick*tick is evaluated as
 * fmaf(a*tick, tick, 2x - x_prev), the multiply-add the CUDA compiler forms from update.cu:39. */
/* Stars::prune (prune.cu:28-62): flag the stars outside the limits (prune.cu:40-41; NaN is kept), then the
 * stable sort by flag of prune.cu:60, which keeps the survivors first in their order and moves the pruned
 * ones behind them, also in order. Returns the number of survivors. */
int orc_prune(int n, const float limits[4], float* cur, float* prev, float* w) {
  int kept = 0;
  float* dead = (float*)malloc(sizeof(float) * 5 * (size_t)(n > 0 ? n : 1));
  int ndead = 0;
  for (int i = 0; i < n; ++i) {
    const float x = cur[2 * i], y = cur[2 * i + 1];
    const int out = (x < limits[0] || y < limits[1] || x > limits[2] || y > limits[3]);
    if (!out) {
      cur[2 * kept] = x;
      cur[2 * kept + 1] = y;
      prev[2 * kept] = prev[2 * i];
      prev[2 * kept + 1] = prev[2 * i + 1];
      w[kept] = w[i];
      ++kept;
    } else {
      dead[5 * ndead + 0] = x;
      dead[5 * ndead + 1] = y;
      dead[5 * ndead + 2] = prev[2 * i];
      dead[5 * ndead + 3] = prev[2 * i + 1];
      dead[5 * ndead + 4] = w[i];
      ++ndead;
    }
  }
  for (int j = 0; j < ndead; ++j) {
    const int i = kept + j;
    cur[2 * i] = dead[5 * j + 0];
    cur[2 * i + 1] = dead[5 * j + 1];
    prev[2 * i] = dead[5 * j + 2];
    prev[2 * i + 1] = dead[5 * j + 3];
    w[i] = dead[5 * j + 4];
  }
  free(dead);
  return kept;
}

int orc_stars_update(int n, int num_level, const float limits[4], float eps, int p2p_block, float tick_scaled,
                     float* cur, float* prev, float* w, float* acc) {
  if (orc_solve(n, num_level, limits, eps, p2p_block, cur, w, acc) != 0) return -1;
  for (int i = 0; i < n; ++i) {
    for (int d = 0; d < 2; ++d) {
      const float p = cur[2 * i + d];
      const float base = 2.0f * p - prev[2 * i + d];
      cur[2 * i + d] = fmaf(acc[2 * i + d] * tick_scaled, tick_scaled, base);
      prev[2 * i + d] = p;
    }
  }
  return orc_prune(n, limits, cur, prev, w);
}

/* All-pairs direct sum in FP64, the error reference for every result (demo.cu:59-66 pattern). */
void orc_direct_f64(int n, const float* pos, const float* w, double eps, const int* targets, int n_targets,
                    double* eff) {
  const int nt = targets ? n_targets : n;
#pragma omp parallel for schedule(dynamic, 16)
  for (int t = 0; t < nt; ++t) {
    const int i = targets ? targets[t] : t;
    const double tx = pos[2 * i], ty = pos[2 * i + 1];
    double ex = 0.0, ey = 0.0;
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      const double dx = (double)pos[2 * j] - tx;
      const double dy = (double)pos[2 * j + 1] - ty;
      const double r = sqrt(dx * dx + dy * dy);
      const double s = (double)w[j] / (r * r * r + eps);
      ex += dx * s;
      ey += dy * s;
    }
    eff[2 * t] = ex;
    eff[2 * t + 1] = ey;
  }
}

/* FP32 all-pairs direct sum (demo.cu:59-66 pattern), each pair evaluated as kernelFunction does, sources in
 * index order: the CPU direct-sum baseline of the benchmark. */
void orc_direct_f32(int n, const float* pos, const float* w, float eps, const int* targets, int n_targets,
                    float* eff) {
  const int nt = targets ? n_targets : n;
#pragma omp parallel for schedule(dynamic, 16)
  for (int t = 0; t < nt; ++t) {
    const int i = targets ? targets[t] : t;
    const float tx = pos[2 * i], ty = pos[2 * i + 1];
    float ex = 0.0f, ey = 0.0f;
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      float ax, ay;
      orc_kernel_function(tx, ty, pos[2 * j], pos[2 * j + 1], w[j], eps, &ax, &ay);
      ex += ax;
      ey += ay;
    }
    eff[2 * t] = ex;
    eff[2 * t + 1] = ey;
  }
}

long long orc_p2p_pairs(int base_dim, const int* head) {
  const int B = base_dim;
  long long total = 0;
  for (int y = 0; y < B; ++y) {
    for (int x = 0; x < B; ++x) {
      const int c = x + y * B;
      const long long nt = head[c + 1] - head[c];
      if (nt == 0) continue;
      long long ns = 0;
      for (int yy = y - 1; yy <= y + 1; ++yy) {
        if (yy < 0 || yy >= B) continue;
        const int lo = x - 1 > 0 ? x - 1 : 0;
        const int hi = x + 1 < B ? x + 1 : B - 1;
        ns += head[hi + yy * B + 1] - head[lo + yy * B];
      }
      total += nt * (ns - 1);
    }
  }
  return total;
}

/* ---- FP64 checkers for the adjoint ------------------------------------------------------------------------ */

/* Effects of the approximate method in FP64 for positions x (double [2n]) with the leaf key of every particle
 * given: the same stages as orc_solve (p2p.cu, p2m.cu, m2m.cu, m2l.cu, l2l.cu, l2p.cu) in double precision. */
static void fmm64_effects(int n, int num_level, const int* key, const double* x, const double* m, double eps,
                          double* a) {
  const int B = orc_base_dim(num_level);
  const int C = B * B;
  const int levels = num_level < 2 ? 2 : num_level;
  int* cnt = (int*)calloc((size_t)C + 1, sizeof(int));
  int* head = (int*)malloc(sizeof(int) * ((size_t)C + 1));
  int* perm = (int*)malloc(sizeof(int) * (size_t)n);
  double* cp = (double*)calloc(2 * (size_t)C * levels, sizeof(double));
  double* cw = (double*)calloc((size_t)C * levels, sizeof(double));
  double* ce = (double*)calloc(2 * (size_t)C * levels, sizeof(double));
  for (int i = 0; i < n; ++i) cnt[key[i]]++;
  int run = 0;
  for (int c = 0; c < C; ++c) { head[c] = run; run += cnt[c]; }
  head[C] = run;
  for (int c = 0; c < C; ++c) cnt[c] = head[c];
  for (int i = 0; i < n; ++i) perm[cnt[key[i]]++] = i;
  for (int i = 0; i < n; ++i) {
    const int cx = key[i] % B, cy = key[i] / B;
    double ex = 0.0, ey = 0.0;
    for (int y = cy - 1; y <= cy + 1; ++y) {
      for (int xx = cx - 1; xx <= cx + 1; ++xx) {
        if (xx < 0 || xx >= B || y < 0 || y >= B) continue;
        const int c = xx + y * B;
        for (int q = head[c]; q < head[c + 1]; ++q) {
          const int j = perm[q];
          if (j == i) continue;
          const double dx = x[2 * j] - x[2 * i], dy = x[2 * j + 1] - x[2 * i + 1];
          const double r = sqrt(dx * dx + dy * dy);
          const double s = m[j] / (r * r * r + eps);
          ex += dx * s;
          ey += dy * s;
        }
      }
    }
    a[2 * i] = ex;
    a[2 * i + 1] = ey;
  }
  if (num_level > 0) {
    for (int c = 0; c < C; ++c) {
      double sx = 0.0, sy = 0.0, sw = 0.0;
      for (int q = head[c]; q < head[c + 1]; ++q) {
        const int j = perm[q];
        sx += x[2 * j] * m[j];
        sy += x[2 * j + 1] * m[j];
        sw += m[j];
      }
      cp[2 * c] = sw != 0.0 ? sx / sw : 0.0;
      cp[2 * c + 1] = sw != 0.0 ? sy / sw : 0.0;
      cw[c] = sw;
    }
    for (int level = 1; level < num_level; ++level) {
      const int cs = 1 << level, ld = B / cs;
      double* lp = cp + 2 * (size_t)level * C;
      double* lw = cw + (size_t)level * C;
      for (int ty = 0; ty < ld; ++ty) {
        for (int tx = 0; tx < ld; ++tx) {
          const int idx = (tx + ty * B) * cs, ch = idx - C, ox = cs / 2, oy = ox * B;
          const int cc[4] = {ch, ch + ox, ch + oy, ch + ox + oy};
          double px = 0.0, py = 0.0, ww = 0.0;
          for (int k = 0; k < 4; ++k) {
            px += lp[2 * cc[k]] * lw[cc[k]];
            py += lp[2 * cc[k] + 1] * lw[cc[k]];
            ww += lw[cc[k]];
          }
          lp[2 * idx] = ww != 0.0 ? px / ww : 0.0;
          lp[2 * idx + 1] = ww != 0.0 ? py / ww : 0.0;
          lw[idx] = ww;
        }
      }
    }
    for (int level = 0; level < num_level; ++level) {
      const int cs = 1 << level, ld = B >> level;
      const double* lp = cp + 2 * (size_t)level * C;
      const double* lw = cw + (size_t)level * C;
      double* le = ce + 2 * (size_t)level * C;
      for (int ty = 0; ty < ld; ++ty) {
        for (int tx = 0; tx < ld; ++tx) {
          const int px = tx & ~1, py = ty & ~1, tidx = (tx + ty * B) * cs;
          double ex = 0.0, ey = 0.0;
          for (int y = py - 2; y < py + 4; ++y) {
            if (y < 0 || y >= ld) continue;
            for (int xx = px - 2; xx < px + 4; ++xx) {
              if (xx < 0 || xx >= ld) continue;
              if (abs(xx - tx) > 1 || abs(y - ty) > 1) {
                const int idx = (xx + y * B) * cs;
                const double dx = lp[2 * idx] - lp[2 * tidx], dy = lp[2 * idx + 1] - lp[2 * tidx + 1];
                const double r = sqrt(dx * dx + dy * dy);
                const double s = lw[idx] / (r * r * r + eps);
                ex += dx * s;
                ey += dy * s;
              }
            }
          }
          le[2 * tidx] = ex;
          le[2 * tidx + 1] = ey;
        }
      }
    }
    for (int level = num_level - 2; level >= 0; --level) {
      const int cs = 1 << level, ld = B / cs;
      double* le = ce + 2 * (size_t)level * C;
      for (int ty = 0; ty < ld; ++ty) {
        for (int tx = 0; tx < ld; ++tx) {
          const int idx = (tx + ty * B) * cs, par = ((tx & ~1) + (ty & ~1) * B) * cs + C;
          le[2 * idx] += le[2 * par];
          le[2 * idx + 1] += le[2 * par + 1];
        }
      }
    }
    for (int i = 0; i < n; ++i) {
      a[2 * i] += ce[2 * key[i]];
      a[2 * i + 1] += ce[2 * key[i] + 1];
    }
  }
  free(cnt); free(head); free(perm); free(cp); free(cw); free(ce);
}

/* FP64 trajectory of the approximate method (update.cu:39-40 without pruning) from x_{-1} = x0 - v0 tau.
 * keys_in (steps x n) fixes the leaf of every particle at every step; when NULL the keys come from the FP32
 * cell arithmetic on the current positions and are written to keys_out (may be NULL). Returns the loss
 * 0.5 sum m |x(T) - target|^2 and writes x(T) to xT (may be NULL). */
double orc_traj_fmm64(int n, int num_level, const float limits[4], double eps, double tau, int steps,
                      const double* x0, const double* v0, const double* m, const int* keys_in, int* keys_out,
                      const double* target, double* xT) {
  const int B = orc_base_dim(num_level);
  double* x = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  double* xp = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  double* a = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  int* key = (int*)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < 2 * n; ++i) {
    x[i] = x0[i];
    xp[i] = x0[i] - v0[i] * tau;
  }
  for (int t = 0; t < steps; ++t) {
    const int* k = keys_in ? keys_in + (size_t)t * n : key;
    if (!keys_in) {
      for (int i = 0; i < n; ++i) {
        int ix, iy;
        orc_cell_index(limits, B, (float)x[2 * i], (float)x[2 * i + 1], &ix, &iy);
        key[i] = ix + iy * B;
      }
      if (keys_out) memcpy(keys_out + (size_t)t * n, key, sizeof(int) * (size_t)n);
    }
    fmm64_effects(n, num_level, k, x, m, eps, a);
    for (int i = 0; i < 2 * n; ++i) {
      const double p = x[i];
      x[i] = 2.0 * p - xp[i] + a[i] * tau * tau;
      xp[i] = p;
    }
  }
  double loss = 0.0;
  for (int i = 0; i < n; ++i) {
    const double dx = x[2 * i] - target[2 * i], dy = x[2 * i + 1] - target[2 * i + 1];
    loss += 0.5 * m[i] * (dx * dx + dy * dy);
  }
  if (xT) memcpy(xT, x, sizeof(double) * 2 * (size_t)n);
  free(x); free(xp); free(a); free(key);
  return loss;
}

/* The exact all-pairs dynamics in FP64 and the exact gradient of its loss by the adjoint (reverse Verlet with
 * the all-pairs vector-Jacobian products). Returns the loss. */
double orc_traj_direct64_grad(int n, double eps, double tau, int steps, const double* x0, const double* v0,
                              const double* m, const double* target, double* gx0, double* gv0, double* gm) {
  double* xs = (double*)malloc(sizeof(double) * 2 * (size_t)n * (steps + 1));
  double* xp = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  double* a = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  for (int i = 0; i < 2 * n; ++i) {
    xs[i] = x0[i];
    xp[i] = x0[i] - v0[i] * tau;
  }
  for (int t = 0; t < steps; ++t) {
    const double* x = xs + (size_t)t * 2 * n;
    double* xn = xs + (size_t)(t + 1) * 2 * n;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      double ex = 0.0, ey = 0.0;
      for (int j = 0; j < n; ++j) {
        if (j == i) continue;
        const double dx = x[2 * j] - x[2 * i], dy = x[2 * j + 1] - x[2 * i + 1];
        const double r = sqrt(dx * dx + dy * dy);
        const double s = m[j] / (r * r * r + eps);
        ex += dx * s;
        ey += dy * s;
      }
      a[2 * i] = ex;
      a[2 * i + 1] = ey;
    }
    for (int i = 0; i < 2 * n; ++i) {
      xn[i] = 2.0 * x[i] - xp[i] + a[i] * tau * tau;
      xp[i] = x[i];
    }
  }
  const double* xT = xs + (size_t)steps * 2 * n;
  double loss = 0.0;
  double* l1 = (double*)malloc(sizeof(double) * 2 * (size_t)n);  /* lambda_{t+1} */
  double* l2 = (double*)calloc(2 * (size_t)n, sizeof(double));   /* lambda_{t+2} */
  double* g = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  double* gmv = (double*)malloc(sizeof(double) * (size_t)n);
  for (int i = 0; i < n; ++i) {
    const double dx = xT[2 * i] - target[2 * i], dy = xT[2 * i + 1] - target[2 * i + 1];
    loss += 0.5 * m[i] * (dx * dx + dy * dy);
    l1[2 * i] = m[i] * dx;
    l1[2 * i + 1] = m[i] * dy;
    gm[i] = 0.5 * (dx * dx + dy * dy);
  }
  for (int t = steps - 1; t >= 0; --t) {
    const double* x = xs + (size_t)t * 2 * n;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      const double mux = tau * tau * l1[2 * i], muy = tau * tau * l1[2 * i + 1];
      double gx = 0.0, gy = 0.0, gmi = 0.0;
      for (int j = 0; j < n; ++j) {
        if (j == i) continue;
        const double dx = x[2 * j] - x[2 * i], dy = x[2 * j + 1] - x[2 * i + 1];
        const double r = sqrt(dx * dx + dy * dy);
        const double inv = 1.0 / (r * r * r + eps);
        const double mjx = tau * tau * l1[2 * j], mjy = tau * tau * l1[2 * j + 1];
        const double ux = m[i] * mjx - m[j] * mux, uy = m[i] * mjy - m[j] * muy;
        const double k3 = 3.0 * r * inv * inv * (dx * ux + dy * uy);
        gx += ux * inv - k3 * dx;
        gy += uy * inv - k3 * dy;
        gmi -= (mjx * dx + mjy * dy) * inv;
      }
      g[2 * i] = gx;
      g[2 * i + 1] = gy;
      gmv[i] = gmi;
    }
    for (int i = 0; i < 2 * n; ++i) {
      const double l0 = 2.0 * l1[i] + g[i] - l2[i];
      l2[i] = l1[i];
      l1[i] = l0;
    }
    for (int i = 0; i < n; ++i) gm[i] += gmv[i];
  }
  /* now l1 = lambda_0, l2 = lambda_1 */
  for (int i = 0; i < 2 * n; ++i) {
    gx0[i] = l1[i] - l2[i];
    gv0[i] = tau * l2[i];
  }
  free(xs); free(xp); free(a); free(l1); free(l2); free(g); free(gmv);
  return loss;
}

/* ---- Initial-condition models (the files of source/nbfmm/model), given the uniform draws --------------------------- */

static const double kOrcPi = 3.14159265358979323846;

/* kernelFunction(0, (r, 0), m).x with the reference's fixed eps 0.1 (kernel_function.hpp:29-40). */
static float model_effect_x(float r, float m) {
  const float rr = sqrtf(r * r + 0.0f * 0.0f);
  const float tmp = m / (rr * rr * rr + 0.1f);
  return r * tmp;
}

/* acos(1.0 - a t t / r / 2): float chain, double subtraction and acos (disk.cu:51). */
static float model_angle_step(float ax, float tick, float r) {
  const float q = ax * tick * tick / r / 2.0f;
  return (float)acos(1.0 - (double)q);
}

static float model_two_pi_u(float u) { return (float)(2.0 * kOrcPi * (double)u); }

static void model_place(float* cur, float* prev, int i, float cx, float cy, float r, float a, float ap) {
  cur[2 * i] = fmaf(r, cosf(a), cx);
  cur[2 * i + 1] = fmaf(r, sinf(a), cy);
  prev[2 * i] = fmaf(r, cosf(ap), cx);
  prev[2 * i + 1] = fmaf(r, sinf(ap), cy);
}

/* circle_center.cu:24-70 (evenly = 0) and circle_uniform_center.cu:24-66 (evenly = 1); u has 3 draws/particle. */
void orc_model_circle(int n, float cx, float cy, float radius, float weight, float center_weight, float tick,
                      int evenly, const float* u, float* cur, float* prev, float* w) {
  const float dangle = model_angle_step(model_effect_x(radius, center_weight), tick, radius);
  for (int i = 0; i < n; ++i) {
    if (i == 0) {
      cur[0] = prev[0] = cx;
      cur[1] = prev[1] = cy;
      w[0] = center_weight;
      continue;
    }
    const float a = evenly ? (float)((2.0 * kOrcPi * (double)i) / (double)n) : model_two_pi_u(u[3 * i]);
    model_place(cur, prev, i, cx, cy, radius, a, a - dangle);
    w[i] = weight;
  }
}

/* disk.cu:30-81 (center = 0), disk_center.cu:30-83 (center = 1), disk_static.cu:30-74 (statik = 1). */
void orc_model_disk(int n, float cx, float cy, float max_radius, float weight, float center_weight, float tick,
                    int center, int statik, const float* u, float* cur, float* prev, float* w) {
  for (int i = 0; i < n; ++i) {
    if (center && i == 0) {
      cur[0] = prev[0] = cx;
      cur[1] = prev[1] = cy;
      w[0] = center_weight;
      continue;
    }
    const float radius = ((float)(i + 1) / (float)n) * max_radius;
    float dangle = 0.0f;
    if (!statik) {
      const float enclosed = center ? weight * (float)(i - 1) + center_weight : weight * (float)i;
      dangle = model_angle_step(model_effect_x(radius, enclosed), tick, radius);
    }
    const float a = model_two_pi_u(u[3 * i]);
    model_place(cur, prev, i, cx, cy, radius, a, a - dangle);
    w[i] = weight;
  }
}

/* rectangle.cu:24-66: x, y, then the weight draw. */
void orc_model_rectangle(int n, float cx, float cy, float width, float height, float max_weight, const float* u,
                         float* cur, float* prev, float* w) {
  for (int i = 0; i < n; ++i) {
    const float x = fmaf(u[3 * i] - 0.5f, width, cx);
    const float y = fmaf(u[3 * i + 1] - 0.5f, height, cy);
    cur[2 * i] = prev[2 * i] = x;
    cur[2 * i + 1] = prev[2 * i + 1] = y;
    w[i] = max_weight * u[3 * i + 2];
  }
}

/* double_disk.cu:58-80: the previous-position offset of disk a in orbit about the common centre. */
static void model_disk_offset(float ax, float ay, float bx, float by, float mass_b, float ra, float tick, float ecc,
                              float* ox, float* oy) {
  float ex, ey;
  orc_kernel_function(ax, ay, bx, by, mass_b, 0.1f, &ex, &ey);
  const float a = sqrtf(ex * ex + ey * ey);
  float x = -ey, y = ex;
  const float f = sqrtf(ra / a) * tick / exp2f(ecc);
  x *= f;
  y *= f;
  x -= ex * tick * tick * ecc;
  y -= ey * tick * tick * ecc;
  *ox = x;
  *oy = y;
}

/* double_disk.cu:39-87 (center = 0) and double_disk_center.cu:39-91 (center = 1). */
void orc_model_double_disk(int n1, int n2, float c1x, float c1y, float c2x, float c2y, float r1, float r2,
                           float weight, float cw1, float cw2, float ecc, float tick, int center, const float* u,
                           float* cur, float* prev, float* w) {
  orc_model_disk(n1, c1x, c1y, r1, weight, cw1, tick, center, 0, u, cur, prev, w);
  orc_model_disk(n2, c2x, c2y, r2, weight, cw2, tick, center, 0, u + 3 * (size_t)n1, cur + 2 * (size_t)n1,
                 prev + 2 * (size_t)n1, w + n1);
  const float m1 = center ? weight * (n1 - 1) + cw1 : weight * n1;
  const float m2 = center ? weight * (n2 - 1) + cw2 : weight * n2;
  const float dx = c1x - c2x, dy = c1y - c2y;
  const float r = sqrtf(dx * dx + dy * dy);
  const float ra = center ? r * m2 / (m1 + m2) : r * n2 / (n1 + n2);
  const float rb = center ? r * m1 / (m1 + m2) : r * n1 / (n1 + n2);
  float o1x, o1y, o2x, o2y;
  model_disk_offset(c1x, c1y, c2x, c2y, m2, ra, tick, ecc, &o1x, &o1y);
  model_disk_offset(c2x, c2y, c1x, c1y, m1, rb, tick, ecc, &o2x, &o2y);
  for (int i = 0; i < n1; ++i) {
    prev[2 * i] += o1x;
    prev[2 * i + 1] += o1y;
  }
  for (int i = n1; i < n1 + n2; ++i) {
    prev[2 * i] += o2x;
    prev[2 * i + 1] += o2y;
  }
}

/* ---- Frame raster (source/nbfmm/display/stars/display.cu) ------------------------------------------------ */

/* float -> int as the GPU converts (cvt.rzi.s32.f32): toward zero, saturating, NaN -> 0. The C cast is
 * undefined out of range and differs between x86 and Arm there. */
static int display_to_int(float v) {
  if (v != v) return 0;
  if (v >= 2147483648.0f) return 2147483647;
  if (v <= -2147483648.0f) return (-2147483647 - 1);
  return (int)v;
}

/* The pixels displayDevice sets around a star (display.cu:53-212), one row per pixel: the size from which it is
 * drawn, its offset (dx, dy) from the star's pixel, and the guard the reference tests before the write, as
 * x >= xa && x < width - xb && y >= ya && y < height - yb (xb or yb = -1: no upper test; the centre pixel's own
 * test, 0 <= x < width and 0 <= y <= height, always holds when these are evaluated). The guards are the
 * reference's verbatim, including the irregular ones: pixels straight above test only y >= 0
 * (display.cu:62,90,130,182), and several diagonal ones test a wider margin than their offset needs. */
static const signed char kDisplayStamp[48][7] = {
    /* size dx  dy  xa  xb  ya  yb */
    {1, -1, 0, 1, -1, 0, -1},  {1, 1, 0, 0, 1, 0, -1},   {1, 0, -1, 0, -1, 0, -1}, {1, 0, 1, 0, -1, 0, 1},
    {2, -1, -1, 1, -1, 1, -1}, {2, -1, 1, 1, -1, 0, 1},  {2, 1, -1, 0, 1, 1, -1},  {2, 1, 1, 0, 1, 0, 1},
    {3, -2, 0, 2, -1, 0, -1},  {3, 2, 0, 0, 2, 0, -1},   {3, 0, -2, 0, -1, 0, -1}, {3, 0, 2, 0, -1, 0, 2},
    {4, -2, -1, 2, -1, 1, -1}, {4, -1, -2, 1, -1, 2, -1}, {4, -2, 1, 2, -1, 0, 2}, {4, -1, 2, 1, -1, 0, 2},
    {4, 2, -1, 0, 2, 1, -1},   {4, 1, -2, 0, 2, 2, -1},  {4, 2, 1, 0, 2, 0, 2},    {4, 1, 2, 0, 2, 0, 2},
    {5, -3, 0, 3, -1, 0, -1},  {5, 3, 0, 0, 3, 0, -1},   {5, 0, -3, 0, -1, 0, -1}, {5, 0, 3, 0, -1, 0, 3},
    {5, -2, -2, 2, -1, 2, -1}, {5, -2, 2, 2, -1, 0, 2},  {5, 2, -2, 0, 2, 2, -1},  {5, 2, 2, 0, 2, 0, 2},
    {6, -3, -1, 3, -1, 1, -1}, {6, -1, -3, 1, -1, 3, -1}, {6, -3, 1, 3, -1, 0, 3}, {6, -1, 3, 1, -1, 0, 3},
    {6, 3, -1, 0, 3, 1, -1},   {6, 1, -3, 0, 3, 3, -1},  {6, 3, 1, 0, 3, 0, 3},    {6, 1, 3, 0, 3, 0, 3},
    {7, -4, 0, 4, -1, 0, -1},  {7, 4, 0, 0, 4, 0, -1},   {7, 0, -4, 0, -1, 0, -1}, {7, 0, 4, 0, -1, 0, 4},
    {7, -3, -2, 3, -1, 2, -1}, {7, -2, -3, 2, -1, 3, -1}, {7, -3, 2, 3, -1, 0, 3}, {7, -2, 3, 2, -1, 0, 3},
    {7, 3, -2, 0, 3, 2, -1},   {7, 2, -3, 0, 3, 3, -1},  {7, 3, 2, 0, 3, 0, 3},    {7, 2, 3, 0, 3, 0, 3},
};

/* Stars::display (display.cu:219-229) without its prune: Y plane 0, the next width*height/2 bytes 128
 * (display.cu:220-221), then displayDevice (display.cu:29-214) per star. Differences from the reference:
 * writes that would land outside the frame of width*height*3/2 bytes are dropped (the reference writes before
 * the buffer for a star on the top rows, through the y >= 0 guards, which is undefined); everything inside the
 * frame is the reference's, including its acceptance of y == height (display.cu:53), which sets bytes of the
 * chroma plane that follows the Y plane. */
void orc_display(int n, int width, int height, float size_scale, const float limits[4], const float* pos,
                 const float* w, unsigned char* board) {
  const long long plane = (long long)width * height;
  const long long frame = plane * 3 / 2;
  memset(board, 0, (size_t)plane);
  memset(board + plane, 128, (size_t)(plane / 2));
  const float unit_width = (limits[2] - limits[0]) / (float)width;    /* display.cu:45 */
  const float unit_height = (limits[3] - limits[1]) / (float)height;  /* display.cu:46 */
  for (int i = 0; i < n; ++i) {
    const int x = display_to_int(floorf((pos[2 * i] - limits[0]) / unit_width));      /* display.cu:47 */
    const int y = display_to_int(floorf((limits[3] - pos[2 * i + 1]) / unit_height));  /* display.cu:48 */
    const int size = display_to_int(floorf(sqrtf(w[i]) / size_scale));                 /* display.cu:49 */
    if (!(0 <= x && x < width && 0 <= y && y <= height)) continue;                      /* display.cu:53 */
    const long long at = (long long)y * width + x;
    if (at < frame) board[at] = 255;
    for (int k = 0; k < 48 && kDisplayStamp[k][0] <= size; ++k) {
      const signed char* e = kDisplayStamp[k];
      if (!(x >= e[3] && x < width - e[4] && y >= e[5] && y < height - e[6])) continue;
      const long long t = at + (long long)e[2] * width + e[1];
      if (t >= 0 && t < frame) board[t] = 255;
    }
  }
}

/* orc_display over the host threads: each thread draws a slice of the stars into its own frame, and the frames
 * are merged by maximum. Every write stores 255 over a cleared frame, so the merge equals the sequential raster. */
void orc_display_threads(int n, int width, int height, float size_scale, const float limits[4], const float* pos,
                         const float* w, unsigned char* board) {
  const int threads = omp_get_max_threads();
  const long long frame = (long long)width * height * 3 / 2;
  if (threads <= 1 || n < 65536) {
    orc_display(n, width, height, size_scale, limits, pos, w, board);
    return;
  }
  unsigned char* part = (unsigned char*)malloc((size_t)frame * (size_t)threads);
  if (!part) {
    orc_display(n, width, height, size_scale, limits, pos, w, board);
    return;
  }
#pragma omp parallel num_threads(threads)
  {
    const int t = omp_get_thread_num();
    const int lo = (int)((long long)n * t / threads), hi = (int)((long long)n * (t + 1) / threads);
    orc_display(hi - lo, width, height, size_scale, limits, pos + 2 * (size_t)lo, w + lo, part + (size_t)t * frame);
  }
#pragma omp parallel for
  for (long long i = 0; i < frame; ++i) {
    unsigned char v = part[i];
    for (int t = 1; t < threads; ++t) {
      const unsigned char u = part[(size_t)t * frame + i];
      v = u > v ? u : v;
    }
    board[i] = v;
  }
  free(part);
}
