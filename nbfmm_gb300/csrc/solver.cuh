// solver.cuh -- the solver workspace and its sequencing, shared by the C ABI (api.cu) and the adjoint
// (adjoint.cu). Host code only.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "../../include/nbfmm_gb300.h"
#include "engine.cuh"
#include "stars.cuh"

namespace nbfmm_gb300 {
int api_fail(int code, const char* fmt, ...);
}

namespace nbfmm_gb300 {

inline int cuda_check(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return api_fail(NBFMM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return NBFMM_OK;
}

#define NBFMM_TRY(expr)              \
  do {                               \
    const int _rc = (expr);          \
    if (_rc != NBFMM_OK) return _rc; \
  } while (0)

// Allocation-failure injection for tests (nbfmm_debug_fail_allocations_after): true when this allocation must
// fail. Counts every device allocation of the library.
bool injected_alloc_failure();

template <typename T>
int dalloc(T** p, size_t count, const char* what) {
  *p = nullptr;
  if (count == 0) count = 1;
  if (injected_alloc_failure()) return api_fail(NBFMM_ERR_NOMEM, "cudaMalloc(%s): injected failure", what);
  const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return api_fail(e == cudaErrorMemoryAllocation ? NBFMM_ERR_NOMEM : NBFMM_ERR_CUDA,
                    "cudaMalloc(%s, %zu bytes): %s", what, count * sizeof(T), cudaGetErrorString(e));
  }
  return NBFMM_OK;
}

template <typename T>
void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

inline bool limits_ok(const float* l) {
  return l && std::isfinite(l[0]) && std::isfinite(l[1]) && std::isfinite(l[2]) && std::isfinite(l[3]) &&
         l[0] < l[2] && l[1] < l[3];
}

}  // namespace nbfmm_gb300

using namespace nbfmm_gb300;

struct nbfmm_solver {
  Geometry geo{};
  Levels lv{};
  int max_n = 0;
  int num_cells = 0;   // B*B
  int key_bits = 0;    // bits of the largest key the sort sees
  int max_tiles = 0;
  int num_sms = 0;
  float eps = 0.1f;
  int exact = 0;  // NBFMM_ARITH_EXACT: the near field with correctly rounded sqrt and division
  // Passes of 32 targets per P2P work item. Measured on the Stars step: 4 is faster from a few million
  // particles up (16.8M two disks: 15.48 against 16.10 ms of P2P), 2 below, where 4-pass items leave SMs idle
  // (1M disk: 0.570 against 0.577 ms; 16k square: 0.044 against 0.059 ms). Results do not depend on it.
  int item_passes = kP2PPasses;

  uint32_t *keys_a = nullptr, *vals_a = nullptr, *keys_b = nullptr, *vals_b = nullptr;
  uint32_t *counts = nullptr, *digit_total = nullptr;
  int* head = nullptr;
  int2* work = nullptr;
  float4* sorted4 = nullptr;
  float4* rec_tmp = nullptr;  // the record sort's passes in between
  float2* seff = nullptr;
  float4* cell4 = nullptr;
  float2* ceff = nullptr;
  int* ints = nullptr;  // [0] n, [1] n_alive, [2] work count, [3] work counter
  // Where the last sort left its result.
  uint32_t* skey = nullptr;
  uint32_t* perm = nullptr;

  int* d_n() { return ints + 0; }
  int* d_n_alive() { return ints + 1; }
  int* d_work_count() { return ints + 2; }
  int* d_work_next() { return ints + 3; }

  int init(int num_level, int max_num_particle, const float* limits, int extra_key_bits) {
    const int B = 1 << (num_level + 1);
    geo.xmin = limits[0];
    geo.ymin = limits[1];
    geo.xmax = limits[2];
    geo.ymax = limits[3];
    geo.cell_x = (limits[2] - limits[0]) / (float)B;  // predo.cu:112-113
    geo.cell_y = (limits[3] - limits[1]) / (float)B;
    geo.num_level = num_level;
    geo.base_dim = B;
    lv.count = num_level > 0 ? num_level : 1;
    lv.total = 0;
    for (int l = 0; l < lv.count; ++l) {
      lv.dim[l] = B >> l;
      lv.offset[l] = lv.total;
      lv.total += lv.dim[l] * lv.dim[l];
    }
    max_n = max_num_particle;
    item_passes = max_n >= (1 << 22) ? 4 : 2;
    num_cells = B * B;
    key_bits = 2 * (num_level + 1) + extra_key_bits;
    max_tiles = (max_n + kSortTile - 1) / kSortTile;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    NBFMM_TRY(cuda_check("device query"));
    const size_t n = (size_t)max_n;
    NBFMM_TRY(dalloc(&keys_a, n, "keys"));
    NBFMM_TRY(dalloc(&vals_a, n, "values"));
    NBFMM_TRY(dalloc(&keys_b, n, "keys"));
    NBFMM_TRY(dalloc(&vals_b, n, "values"));
    constexpr int kDigits = 1 << (kRecMaxBits > kRadixMaxBits ? kRecMaxBits : kRadixMaxBits);
    const size_t count_tiles = (size_t)(max_n + kRecTile - 1) / kRecTile;  // >= the key/value sort's tiles
    NBFMM_TRY(dalloc(&counts, (size_t)kDigits * count_tiles, "tile counts"));
    NBFMM_TRY(dalloc(&digit_total, (size_t)kDigits, "digit totals"));
    NBFMM_TRY(dalloc(&head, (size_t)num_cells + 2, "head"));
    NBFMM_TRY(dalloc(&work, work_list_capacity(num_cells, n), "work list"));
    NBFMM_TRY(dalloc(&sorted4, n, "sorted particles"));
    NBFMM_TRY(dalloc(&rec_tmp, n, "sort records"));
    NBFMM_TRY(dalloc(&seff, n, "sorted effects"));
    NBFMM_TRY(dalloc(&cell4, (size_t)lv.total, "cells"));
    NBFMM_TRY(dalloc(&ceff, (size_t)lv.total, "cell effects"));
    NBFMM_TRY(dalloc(&ints, 8, "counters"));
    cudaMemset(ints, 0, 8 * sizeof(int));
    cudaMemset(head, 0, ((size_t)num_cells + 2) * sizeof(int));
    cudaMemset(cell4, 0, (size_t)lv.total * sizeof(float4));
    cudaMemset(ceff, 0, (size_t)lv.total * sizeof(float2));
    NBFMM_TRY(cuda_check("workspace clear"));
    skey = keys_a;
    perm = vals_a;
    return NBFMM_OK;
  }

  ~nbfmm_solver() {
    dfree(keys_a); dfree(vals_a); dfree(keys_b); dfree(vals_b);
    dfree(counts); dfree(digit_total); dfree(head); dfree(work);
    dfree(sorted4); dfree(rec_tmp); dfree(seff); dfree(cell4); dfree(ceff); dfree(ints);
  }

  float4* cell0() { return cell4 + lv.offset[0]; }
  float2* ceff0() { return ceff + lv.offset[0]; }

  // Sort (keys_a, vals_a) holding d_n entries; records where the result went.
  void sort(const int* dn, int bits, cudaStream_t s) {
    const int where = launch_radix_sort(keys_a, vals_a, keys_b, vals_b, counts, digit_total, dn, max_n, bits, s);
    skey = where ? keys_b : keys_a;
    perm = where ? vals_b : vals_a;
  }

  // predo.cu:105-135 plus P2M's leaf sums: caller-order positions and weights sorted by leaf cell as records
  // (sorted4 = x, y, m, original index; skey, perm), heads, the P2P work list (paired tails unless the caller's
  // kernel reads plain chunks) and the leaf centres of mass, summed in sorted order.
  void predo(int n, const float2* pos, const float* w, cudaStream_t s, bool pair_tails = true) {
    launch_set_int(d_n(), n, s);
    launch_sort_records(geo, pos, w, d_n(), max_n, 2 * (geo.num_level + 1), sorted4, rec_tmp, keys_a, keys_b,
                        vals_a, counts, digit_total, s);
    skey = keys_a;
    perm = vals_a;
    launch_head(skey, d_n(), num_cells, head, d_n_alive(), s);
    launch_worklist(head, num_cells, work, d_work_count(), pair_tails, s, item_passes);
    launch_p2m(geo, head, sorted4, cell0(), s);
  }

  void far_field(cudaStream_t s) {
    if (geo.num_level <= 0) return;  // p2m.cu:80, m2l.cu:64
    launch_far_field(lv, cell4, ceff, eps, s);  // M2M is a no-op for num_level <= 1 (m2m.cu:60)
  }

  P2PArgs p2p_args() {
    P2PArgs a{};
    a.sorted4 = sorted4;
    a.head = head;
    a.work = work;
    a.pair_tails = 1;  // every single-system work list here pairs tails
    a.d_work_count = d_work_count();
    a.d_work_next = d_work_next();
    a.base_dim = geo.base_dim;
    a.eps = eps;
    a.exact = exact;
    a.series = exact ? 0 : series_degree(geo.cell_x, geo.cell_y, eps);
    a.inv_eps = 1.0f / eps;
    a.ceff0 = geo.num_level > 0 ? ceff0() : nullptr;
    return a;
  }

  int solve(int n, const float* pos, const float* w, float* eff, cudaStream_t s) {
    if (n == 0) return NBFMM_OK;
    predo(n, reinterpret_cast<const float2*>(pos), w, s);
    far_field(s);
    P2PArgs a = p2p_args();
    a.eff_origin = reinterpret_cast<float2*>(eff);
    launch_p2p(a, kSolve, num_sms, s);
    return cuda_check("nbfmm_solver_solve");
  }
};


// Creates and initialises a solver (argument checks of solver.cu:24-27).
int nbfmm_make_solver(int num_level, int max_num_particle, const float* limits, int extra_key_bits, nbfmm_solver** out);
