// batch.cu -- the batched form: many independent systems of uneven N stepped together.
//
// No counterpart in the reference, which steps one system per Stars object (update.cu:47-55). Each system s
// owns particles [offsets[s], offsets[s+1]) of the state arrays, its own limits and tree depth, and evolves
// exactly as an independent Stars::update would: solve, Stormer-Verlet, prune.
//
// Layout: the systems' leaf grids are concatenated into one global leaf-cell space, system s holding cells
// [cell_base[s], cell_base[s] + B_s^2) with key cell_base[s] + iy*B_s + ix. A star pruned from any system gets
// the single key past the last cell, so one stable radix sort orders every system by cell and drops the dead,
// and the single-system kernels for heads, the work list, gather + P2M and P2P (which finds an item's system
// by binary search) serve all systems at once. Cell levels above the leaves are stored per level, systems
// side by side: level l of system s starts at level_offset[l] + level_base[l][s]. M2M and M2L are one launch
// per level covering every system that has that level; a thread (M2M) or a 16x16 tile CTA (M2L) finds its
// system by binary search over the level's prefix table.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <new>
#include <vector>

#include "../../include/nbfmm_gb300.h"
#include "engine.cuh"
#include "stars.cuh"

namespace nbfmm_gb300 {
int api_fail(int code, const char* fmt, ...);
bool injected_alloc_failure();
}

using namespace nbfmm_gb300;

namespace {

__device__ __forceinline__ int find_system(const int* __restrict__ prefix, int num_systems, int k) {
  int lo = 0, hi = num_systems;  // last s with prefix[s] <= k
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (prefix[mid] <= k) lo = mid; else hi = mid;
  }
  return lo;
}

struct BatchDevice {
  int num_systems;
  const Geometry* geo;       // [S]
  const int* sys_of_orig;    // [N] system of each particle (by index in the public arrays)
  const int* cell_base;      // [S + 1] leaf-cell prefix
  const int* dim;            // [S] leaf cells per side
  const int* part_off;       // [S + 1] particle ranges
};

// live_base[s] = sum of counts[t] for t < s, live_base[S] = total (one CTA).
__global__ void batch_live_scan_kernel(const int* __restrict__ counts, int num_systems, int* __restrict__ live_base) {
  __shared__ int carry;
  __shared__ int part[1024];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < num_systems; base += blockDim.x) {
    const int s = base + threadIdx.x;
    const int v = s < num_systems ? counts[s] : 0;
    part[threadIdx.x] = v;
    __syncthreads();
    for (int d = 1; d < (int)blockDim.x; d <<= 1) {  // inclusive Hillis-Steele scan
      const int t = threadIdx.x >= d ? part[threadIdx.x - d] : 0;
      __syncthreads();
      part[threadIdx.x] += t;
      __syncthreads();
    }
    if (s < num_systems) live_base[s] = carry + part[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += part[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) live_base[num_systems] = carry;
}

// Imports each system's live stars [off_s, off_s + counts[s]) into the compact internal state, and files the
// stars a previous call already pruned (the rest of the range) with the last fate, so that the export leaves
// them behind this call's deaths, in their order -- as the reference's update leaves its array tail untouched.
__global__ void batch_import_kernel(BatchDevice bd, StepCounters sc, const int* __restrict__ counts,
                                    const int* __restrict__ live_base, const float2* __restrict__ cur,
                                    const float2* __restrict__ prev, const float* __restrict__ w,
                                    float4* __restrict__ state4, float2* __restrict__ state_prev,
                                    float4* __restrict__ grave, int n, int old_fate) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int s = bd.sys_of_orig[i];
    const int local = i - bd.part_off[s];
    const float2 c = cur[i];
    const float m = w[i];
    if (local < counts[s]) {
      const int slot = live_base[s] + local;
      state4[slot] = make_float4(c.x, c.y, m, __int_as_float(i));
      state_prev[slot] = prev[i];
    } else {
      file_grave(grave, i, c.x, c.y, prev[i], m, old_fate);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *sc.n_cur = live_base[bd.num_systems];
    *sc.n_import = n;
    *sc.step = 1;
    *sc.prune = 0;
  }
}

__global__ void batch_keys_kernel(BatchDevice bd, StepCounters sc, const float4* __restrict__ state4,
                                  const float2* __restrict__ state_prev, uint32_t dead_key,
                                  uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                  float4* __restrict__ grave) {
  const int n = *sc.n_cur;
  const int prune = *sc.prune;
  const int death_rank = *sc.num_steps + 1 - (*sc.step - 1);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = state4[i];
    const int orig = __float_as_int(p.w);
    const int s = bd.sys_of_orig[orig];
    const Geometry g = bd.geo[s];
    uint32_t key;
    if (prune && outside(g, p.x, p.y)) {  // prune.cu:40-41 with the system's limits
      key = dead_key;
      file_grave(grave, orig, p.x, p.y, state_prev[i], p.z, death_rank);
    } else {
      key = (uint32_t)bd.cell_base[s] + leaf_key(g, p.x, p.y);
    }
    keys[i] = key;
    vals[i] = (uint32_t)i;
  }
}

// M2M for level l >= 1 of every system that has it (m2m.cu:40-53).
__global__ void batch_m2m_kernel(float4* __restrict__ cell4, const int* __restrict__ base_c,
                                 const int* __restrict__ base_p, const int* __restrict__ dim, int num_systems,
                                 int off_c, int off_p, int level, int total) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
    const int s = find_system(base_p, num_systems, k);
    const int dim_p = dim[s] >> level, dim_c = dim[s] >> (level - 1);
    const int local = k - base_p[s];
    const int px = local % dim_p, py = local / dim_p;
    const int c0 = off_c + base_c[s] + (2 * py) * dim_c + 2 * px;
    const float4 a = cell4[c0], b = cell4[c0 + 1], c = cell4[c0 + dim_c], d = cell4[c0 + dim_c + 1];
    float sx = __fmul_rn(a.x, a.z);
    float sy = __fmul_rn(a.y, a.z);
    sx = __fadd_rn(sx, __fmul_rn(b.x, b.z));
    sy = __fadd_rn(sy, __fmul_rn(b.y, b.z));
    sx = __fadd_rn(sx, __fmul_rn(c.x, c.z));
    sy = __fadd_rn(sy, __fmul_rn(c.y, c.z));
    sx = __fadd_rn(sx, __fmul_rn(d.x, d.z));
    sy = __fadd_rn(sy, __fmul_rn(d.y, d.z));
    const float sw = __fadd_rn(__fadd_rn(__fadd_rn(a.z, b.z), c.z), d.z);
    float4 out = make_float4(0.0f, 0.0f, sw, 0.0f);
    if (sw != 0.0f) {
      out.x = __fdiv_rn(sx, sw);
      out.y = __fdiv_rn(sy, sw);
    }
    cell4[off_p + k] = out;
  }
}

// M2L (+ L2L on the way down) for level l of every system that has it; one CTA per 16x16 tile.
__global__ void __launch_bounds__(kM2LTile * kM2LTile)
batch_m2l_kernel(const float4* __restrict__ cell4, float2* __restrict__ ceff, const int* __restrict__ tile_base,
                 const int* __restrict__ base_l, const int* __restrict__ base_parent, const int* __restrict__ dim,
                 const int* __restrict__ levels, int num_systems, int off_l, int off_parent, int level, float eps) {
  __shared__ float4 halo[kM2LHalo][kM2LHalo];
  const int s = find_system(tile_base, num_systems, blockIdx.x);
  const int d = dim[s] >> level;
  const int tiles_x = (d + kM2LTile - 1) / kM2LTile;
  const int t = blockIdx.x - tile_base[s];
  const int has_parent = (level + 1 < levels[s]) ? 1 : 0;
  const float4* cells = cell4 + off_l + base_l[s];
  float2* eff = ceff + off_l + base_l[s];
  const float2* parent = has_parent ? ceff + off_parent + base_parent[s] : eff;
  m2l_tile(halo, cells, eff, d, parent, d >> 1, has_parent, (t % tiles_x) * kM2LTile, (t / tiles_x) * kM2LTile, eps);
}

// Final prune of the call, and every star's final state filed by original index (fate 0 = alive).
__global__ void batch_export_fate_kernel(BatchDevice bd, StepCounters sc, const float4* __restrict__ state4,
                                         const float2* __restrict__ state_prev, float4* __restrict__ grave) {
  const int n = *sc.n_cur;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = state4[i];
    const int orig = __float_as_int(p.w);
    file_grave(grave, orig, p.x, p.y, state_prev[i], p.z, outside(bd.geo[bd.sys_of_orig[orig]], p.x, p.y) ? 1 : 0);
  }
}

// Export keys: system-major, then fate, so each system's block keeps survivors first, then the pruned stars,
// most recently pruned first -- the order num_steps reference updates leave that system's arrays in.
__global__ void batch_fate_keys_kernel(BatchDevice bd, StepCounters sc, const float4* __restrict__ grave,
                                       uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const int n = *sc.n_import;
  const int span = *sc.num_steps + 2;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    keys[i] = (uint32_t)(bd.sys_of_orig[i] * span + grave_fate(grave, i));
    vals[i] = (uint32_t)i;
  }
}

__device__ __forceinline__ int lower_bound_u32(const uint32_t* __restrict__ keys, int n, uint32_t v) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (keys[mid] < v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Survivors per system: the number of sorted export keys equal to s*span (fate 0).
__global__ void batch_counts_kernel(const uint32_t* __restrict__ skeys, StepCounters sc, int num_systems,
                                    int* __restrict__ counts) {
  const int n = *sc.n_import;
  const int span = *sc.num_steps + 2;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < num_systems; s += gridDim.x * blockDim.x) {
    const uint32_t k = (uint32_t)(s * span);
    counts[s] = lower_bound_u32(skeys, n, k + 1) - lower_bound_u32(skeys, n, k);
  }
}

int grid_for(long long n, int threads, int cap) {
  long long g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

int bits_for(long long v) {  // bits to hold values in [0, v]
  int b = 1;
  while ((1ll << b) <= v) ++b;
  return b;
}

template <typename T>
int balloc(T** p, size_t count, const char* what) {
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
void bfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

#define BATCH_TRY(expr)              \
  do {                               \
    const int _rc = (expr);          \
    if (_rc != NBFMM_OK) return _rc; \
  } while (0)

int cuda_status(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return api_fail(NBFMM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return NBFMM_OK;
}

}  // namespace

struct nbfmm_batch {
  int S = 0;
  int n = 0;            // total particles
  int max_levels = 0;   // max over systems of the stored levels
  int total_leaf = 0;
  int key_bits = 0;
  int num_sms = 0;
  float tick = 0.0f;
  float eps = 0.1f;
  int exact = 0;  // NBFMM_ARITH_EXACT
  std::vector<int> h_off, h_levels, h_dim, h_level_offset, h_level_total, h_tile_total;

  // Device tables.
  Geometry* geo = nullptr;
  int* sys_of_orig = nullptr;
  int* cell_base = nullptr;
  int* dim = nullptr;
  int* levels = nullptr;
  int* level_base = nullptr;  // [max_levels][S + 1]
  int* tile_base = nullptr;   // [max_levels][S + 1]
  int* sys_passes = nullptr;  // [S] passes of 32 targets per P2P work item of each system (2 or 4)
  int* sys_series = nullptr;  // [S] P2PArgs::series (the series degree) of each system for the current eps
  float2* sys_inv = nullptr;  // [S] RN(1 / cell size) of each system (P2PArgs::sys_inv)
  std::vector<Geometry> h_geo;
  // Sort, tree and P2P workspace.
  uint32_t *keys_a = nullptr, *vals_a = nullptr, *keys_b = nullptr, *vals_b = nullptr;
  uint32_t *counts = nullptr, *digit_total = nullptr;
  int* head = nullptr;
  int head_len = 0;
  int2* work = nullptr;
  float4* sorted4 = nullptr;
  float2* sprev = nullptr;
  float4* cell4 = nullptr;
  float2* ceff = nullptr;
  int total_cells = 0;
  // State.
  float2 *cur = nullptr, *prev = nullptr;
  float* w = nullptr;
  float4* state4 = nullptr;
  float2* state_prev = nullptr;
  float4* grave = nullptr;  // final states by original index: two float4 per star (stars.cuh file_grave)
  uint32_t* order_scratch = nullptr;  // gather_state_ordered_kernel's scratch for large cells
  int* sys_counts = nullptr;  // survivors per system
  int* live_base = nullptr;   // [S + 1] prefix of sys_counts
  int* part_off = nullptr;    // [S + 1] particle ranges
  int* ints = nullptr;        // counters
  StepCounters sc{};
  uint32_t* skey = nullptr;
  uint32_t* perm = nullptr;
  // The re-sort of the steps after a call's first (stars.cuh ResortArrays), over the global leaf-cell space.
  uint32_t* step_key = nullptr;
  uint32_t* step_perm = nullptr;
  int* head_old = nullptr;
  int* stay = nullptr;
  int* imm_cnt = nullptr;
  int* imm_next = nullptr;
  int* tile_sum = nullptr;
  // Graphs (a call's first step sorts in full, the others re-sort) and profiling.
  struct StepGraph {
    cudaGraph_t def = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t node_a = nullptr, node_b = nullptr;
    int kernels = 0;
  };
  StepGraph first_step, next_step;
  bool graphs_built = false;
  cudaStream_t capture_stream = nullptr;
  cudaEvent_t cap_a = nullptr, cap_b = nullptr;
  std::vector<cudaEvent_t> prof_events;
  int prof_max = 0, prof_used = 0;

  int* d_work_count() { return ints + 8; }
  int* d_work_next() { return ints + 9; }

  BatchDevice device() const { return BatchDevice{S, geo, sys_of_orig, cell_base, dim, part_off}; }

  int init(int num_systems, const int* offsets, const int* num_levels, const float* limits, float tick_scaled) {
    S = num_systems;
    tick = tick_scaled;
    h_off.assign(offsets, offsets + S + 1);
    n = h_off[S];
    h_levels.resize(S);
    h_dim.resize(S);
    h_geo.assign(S, Geometry{});
    std::vector<Geometry>& hg = h_geo;
    std::vector<int> h_cell_base(S + 1, 0);
    std::vector<int> h_sys_of_orig(n);
    max_levels = 1;
    long long leaf = 0;
    for (int s = 0; s < S; ++s) {
      const int L = num_levels[s];
      const int B = 1 << (L + 1);
      const float* l = limits + 4 * s;
      Geometry& g = hg[s];
      g.xmin = l[0]; g.ymin = l[1]; g.xmax = l[2]; g.ymax = l[3];
      g.cell_x = (l[2] - l[0]) / (float)B;  // predo.cu:112-113
      g.cell_y = (l[3] - l[1]) / (float)B;
      g.num_level = L;
      g.base_dim = B;
      h_levels[s] = L;
      h_dim[s] = B;
      max_levels = std::max(max_levels, std::max(L, 1));
      h_cell_base[s] = (int)leaf;
      leaf += (long long)B * B;
      for (int i = h_off[s]; i < h_off[s + 1]; ++i) h_sys_of_orig[i] = s;
    }
    if (leaf >= (1ll << 28)) return api_fail(NBFMM_ERR_INVALID, "batch: %lld leaf cells exceed 2^28", leaf);
    total_leaf = (int)leaf;
    h_cell_base[S] = total_leaf;
    key_bits = bits_for(total_leaf);  // the dead key is total_leaf
    // Per-level prefix tables. Level 0 is the leaf space (every system, gather + P2M write it); level l >= 1
    // holds the systems with num_level > l (M2M). M2L tiles cover the systems with num_level > l.
    std::vector<int> h_level_base((size_t)max_levels * (S + 1), 0), h_tile_base((size_t)max_levels * (S + 1), 0);
    h_level_offset.assign(max_levels, 0);
    h_level_total.assign(max_levels, 0);
    h_tile_total.assign(max_levels, 0);
    long long cells = 0;
    for (int lv = 0; lv < max_levels; ++lv) {
      long long run = 0, tiles = 0;
      for (int s = 0; s < S; ++s) {
        h_level_base[(size_t)lv * (S + 1) + s] = (int)run;
        h_tile_base[(size_t)lv * (S + 1) + s] = (int)tiles;
        const int d = h_dim[s] >> lv;
        if (lv == 0 || h_levels[s] > lv) run += (long long)d * d;
        if (h_levels[s] > lv) tiles += (long long)((d + kM2LTile - 1) / kM2LTile) * ((d + kM2LTile - 1) / kM2LTile);
      }
      h_level_base[(size_t)lv * (S + 1) + S] = (int)run;
      h_tile_base[(size_t)lv * (S + 1) + S] = (int)tiles;
      h_level_offset[lv] = (int)cells;
      h_level_total[lv] = (int)run;
      h_tile_total[lv] = (int)tiles;
      cells += run;
    }
    total_cells = (int)cells;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t N = (size_t)std::max(n, 1);
    const int max_tiles = (std::max(n, 1) + kSortTile - 1) / kSortTile;
    head_len = total_leaf + 2;
    BATCH_TRY(balloc(&geo, (size_t)S, "geometry"));
    BATCH_TRY(balloc(&sys_of_orig, N, "system of particle"));
    BATCH_TRY(balloc(&cell_base, (size_t)S + 1, "cell base"));
    BATCH_TRY(balloc(&dim, (size_t)S, "dims"));
    BATCH_TRY(balloc(&levels, (size_t)S, "levels"));
    BATCH_TRY(balloc(&level_base, h_level_base.size(), "level base"));
    BATCH_TRY(balloc(&tile_base, h_tile_base.size(), "tile base"));
    BATCH_TRY(balloc(&sys_passes, (size_t)S, "passes per item"));
    BATCH_TRY(balloc(&sys_series, (size_t)S, "series flags"));
    BATCH_TRY(balloc(&sys_inv, (size_t)S, "cell inverses"));
    BATCH_TRY(balloc(&keys_a, N, "keys"));
    BATCH_TRY(balloc(&vals_a, N, "values"));
    BATCH_TRY(balloc(&keys_b, N, "keys"));
    BATCH_TRY(balloc(&vals_b, N, "values"));
    BATCH_TRY(balloc(&counts, (size_t)(1 << kRadixMaxBits) * max_tiles, "tile counts"));
    BATCH_TRY(balloc(&digit_total, (size_t)(1 << kRadixMaxBits), "digit totals"));
    BATCH_TRY(balloc(&work, work_list_capacity(total_leaf, N), "work list"));
    BATCH_TRY(balloc(&sorted4, N, "sorted particles"));
    BATCH_TRY(balloc(&sprev, N, "sorted previous positions"));
    BATCH_TRY(balloc(&cell4, (size_t)total_cells, "cells"));
    BATCH_TRY(balloc(&ceff, (size_t)total_cells, "cell effects"));
    BATCH_TRY(balloc(&cur, N, "position_cur"));
    BATCH_TRY(balloc(&prev, N, "position_pre"));
    BATCH_TRY(balloc(&w, N, "weight"));
    BATCH_TRY(balloc(&state4, N, "state"));
    BATCH_TRY(balloc(&state_prev, N, "state prev"));
    BATCH_TRY(balloc(&grave, 2 * (size_t)N, "final states"));
    BATCH_TRY(balloc(&order_scratch, (size_t)kOrderScratch * N, "cell order scratch"));
    BATCH_TRY(balloc(&step_key, N, "step keys"));
    BATCH_TRY(balloc(&step_perm, N, "step order"));
    BATCH_TRY(balloc(&head_old, (size_t)total_leaf + 1, "previous heads"));
    BATCH_TRY(balloc(&stay, (size_t)total_leaf, "stayers"));
    BATCH_TRY(balloc(&imm_cnt, (size_t)total_leaf, "immigrants"));
    BATCH_TRY(balloc(&imm_next, (size_t)total_leaf, "immigrant places"));
    BATCH_TRY(balloc(&tile_sum, (size_t)resort_tiles(total_leaf), "re-sort tiles"));
    BATCH_TRY(balloc(&sys_counts, (size_t)S, "system counts"));
    BATCH_TRY(balloc(&live_base, (size_t)S + 1, "live prefix"));
    BATCH_TRY(balloc(&part_off, (size_t)S + 1, "particle offsets"));
    BATCH_TRY(balloc(&ints, 16, "counters"));
    cudaMemcpy(geo, hg.data(), sizeof(Geometry) * S, cudaMemcpyHostToDevice);
    std::vector<float2> h_inv(S);
    for (int s = 0; s < S; ++s) h_inv[s] = make_float2(1.0f / hg[s].cell_x, 1.0f / hg[s].cell_y);
    cudaMemcpy(sys_inv, h_inv.data(), sizeof(float2) * S, cudaMemcpyHostToDevice);
    cudaMemcpy(sys_of_orig, h_sys_of_orig.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemcpy(cell_base, h_cell_base.data(), sizeof(int) * (S + 1), cudaMemcpyHostToDevice);
    const std::vector<int> h_passes(S, kP2PPasses);
    cudaMemcpy(sys_passes, h_passes.data(), sizeof(int) * S, cudaMemcpyHostToDevice);
    cudaMemcpy(part_off, h_off.data(), sizeof(int) * (S + 1), cudaMemcpyHostToDevice);
    cudaMemcpy(dim, h_dim.data(), sizeof(int) * S, cudaMemcpyHostToDevice);
    cudaMemcpy(levels, h_levels.data(), sizeof(int) * S, cudaMemcpyHostToDevice);
    cudaMemcpy(level_base, h_level_base.data(), sizeof(int) * h_level_base.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(tile_base, h_tile_base.data(), sizeof(int) * h_tile_base.size(), cudaMemcpyHostToDevice);
    std::vector<int> h_counts(S);
    for (int s = 0; s < S; ++s) h_counts[s] = h_off[s + 1] - h_off[s];
    cudaMemcpy(sys_counts, h_counts.data(), sizeof(int) * S, cudaMemcpyHostToDevice);
    cudaMemset(ints, 0, 16 * sizeof(int));
    cudaMemset(stay, 0, sizeof(int) * (size_t)total_leaf);
    cudaMemset(imm_cnt, 0, sizeof(int) * (size_t)total_leaf);
    cudaMemset(cell4, 0, sizeof(float4) * (size_t)total_cells);
    cudaMemset(ceff, 0, sizeof(float2) * (size_t)total_cells);  // systems with num_level 0 keep zero far field
    cudaMemset(cur, 0, sizeof(float2) * N);
    cudaMemset(prev, 0, sizeof(float2) * N);
    cudaMemset(w, 0, sizeof(float) * N);
    sc.num_star = ints + 0;
    sc.n_import = ints + 1;
    sc.n_cur = ints + 2;
    sc.n_alive = ints + 3;
    sc.step = ints + 4;
    sc.prune = ints + 5;
    sc.num_steps = ints + 6;
    launch_set_int(sc.num_star, n, nullptr);
    if (cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&cap_a) != cudaSuccess || cudaEventCreate(&cap_b) != cudaSuccess) {
      return cuda_status("batch stream/event create");
    }
    BATCH_TRY(cuda_status("batch init"));
    return cudaDeviceSynchronize() == cudaSuccess ? NBFMM_OK : cuda_status("batch init sync");
  }

  ~nbfmm_batch() {
    drop_graph();
    drop_profile_events();
    if (cap_a) cudaEventDestroy(cap_a);
    if (cap_b) cudaEventDestroy(cap_b);
    if (capture_stream) cudaStreamDestroy(capture_stream);
    bfree(geo); bfree(sys_of_orig); bfree(cell_base); bfree(dim); bfree(levels); bfree(level_base); bfree(tile_base);
    bfree(sys_passes);
    bfree(sys_series);
    bfree(sys_inv);
    bfree(keys_a); bfree(vals_a); bfree(keys_b); bfree(vals_b); bfree(counts); bfree(digit_total);
    bfree(head); bfree(work); bfree(sorted4); bfree(sprev); bfree(cell4); bfree(ceff);
    bfree(cur); bfree(prev); bfree(w); bfree(state4); bfree(state_prev); bfree(grave); bfree(order_scratch); bfree(sys_counts);
    bfree(live_base); bfree(part_off); bfree(ints);
    bfree(step_key); bfree(step_perm); bfree(head_old); bfree(stay); bfree(imm_cnt); bfree(imm_next); bfree(tile_sum);
  }

  int alloc_head() {
    if (!head) BATCH_TRY(balloc(&head, (size_t)head_len, "head"));
    return NBFMM_OK;
  }

  static void drop(StepGraph& g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.def) cudaGraphDestroy(g.def);
    g = StepGraph{};
  }

  void drop_graph() {
    drop(first_step);
    drop(next_step);
    graphs_built = false;
  }

  void set_events(StepGraph& g, cudaEvent_t a, cudaEvent_t b) {
    cudaGraphExecEventRecordNodeSetEvent(g.exec, g.node_a, a);
    cudaGraphExecEventRecordNodeSetEvent(g.exec, g.node_b, b);
  }

  void drop_profile_events() {
    for (cudaEvent_t e : prof_events) cudaEventDestroy(e);
    prof_events.clear();
    prof_max = prof_used = 0;
  }

  void sort(const int* dn, int bits, cudaStream_t s) {
    const int where = launch_radix_sort(keys_a, vals_a, keys_b, vals_b, counts, digit_total, dn, std::max(n, 1), bits, s);
    skey = where ? keys_b : keys_a;
    perm = where ? vals_b : vals_a;
  }

  // One step; a continuing step re-sorts from the previous step's cell order with the keys and counts its P2P
  // epilogue left (stars.cu, "Re-sort of a continuing step"), the first step of a call sorts in full.
  void enqueue_step(cudaStream_t s, bool continuing) {
    const int N = std::max(n, 1);
    const uint32_t* order = nullptr;
    if (!continuing) {
      batch_keys_kernel<<<grid_for(N, 256, 152 * 16), 256, 0, s>>>(device(), sc, state4, state_prev,
                                                                  (uint32_t)total_leaf, keys_a, vals_a, grave);
      sort(sc.n_cur, key_bits, s);
      launch_head(skey, sc.n_cur, total_leaf, head, sc.n_alive, s);
      order = perm;
    } else {
      ResortArrays r{head_old, step_key, stay, imm_cnt, imm_next, tile_sum, step_perm};
      launch_resort(r, total_leaf, N, head, sc.n_alive, s);
      order = step_perm;
    }
    launch_worklist(head, total_leaf, work, d_work_count(), true, s, kP2PPasses, cell_base, sys_passes, S, head_old);
    // gather + P2M over the global leaf space, each cell in index order
    launch_gather_state_ordered(head, total_leaf, order, state4, state_prev, sorted4, sprev, cell4, order_scratch, N,
                                s);
    for (int lv = 1; lv < max_levels; ++lv) {
      if (h_level_total[lv] == 0) continue;
      batch_m2m_kernel<<<grid_for(h_level_total[lv], 256, 152 * 8), 256, 0, s>>>(
          cell4, level_base + (size_t)(lv - 1) * (S + 1), level_base + (size_t)lv * (S + 1), dim, S,
          h_level_offset[lv - 1], h_level_offset[lv], lv, h_level_total[lv]);
    }
    for (int lv = max_levels - 1; lv >= 0; --lv) {
      if (h_tile_total[lv] == 0) continue;
      const int lp = lv + 1 < max_levels ? lv + 1 : lv;
      batch_m2l_kernel<<<h_tile_total[lv], dim3(kM2LTile, kM2LTile), 0, s>>>(
          cell4, ceff, tile_base + (size_t)lv * (S + 1), level_base + (size_t)lv * (S + 1),
          level_base + (size_t)lp * (S + 1), dim, levels, S, h_level_offset[lv], h_level_offset[lp], lv, eps);
    }
    P2PArgs a{};
    a.sorted4 = sorted4;
    a.head = head;
    a.work = work;
    a.pair_tails = 1;  // as a system stepped alone: pairing decides each pair's reciprocal method
    a.d_work_count = d_work_count();
    a.d_work_next = d_work_next();
    a.base_dim = 1;
    a.eps = eps;
    a.exact = exact;
    a.inv_eps = 1.0f / eps;
    a.sys_series = sys_series;
    a.ceff0 = ceff;  // level 0 = the global leaf space
    a.sprev = sprev;
    a.state4 = state4;
    a.state_prev = state_prev;
    a.tick = tick;
    a.num_systems = S;
    a.sys_cell_base = cell_base;
    a.sys_dim = dim;
    a.grave = grave;  // prunes within a call; the call's final states are filed by the export
    a.d_step = sc.step;
    a.d_num_steps = sc.num_steps;
    a.next_key = step_key;
    a.next_stay = stay;
    a.next_imm = imm_cnt;
    a.dead_key = (uint32_t)total_leaf;
    a.sys_geo = geo;
    a.sys_inv = sys_inv;
    cudaEventRecordWithFlags(cap_a, s, cudaEventRecordExternal);
    launch_p2p(a, kVerlet, num_sms, s);
    cudaEventRecordWithFlags(cap_b, s, cudaEventRecordExternal);
    launch_finish_step(sc, s);
  }

  int build_graph(StepGraph& out, bool continuing) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(capture_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      return cuda_status("cudaStreamBeginCapture");
    }
    enqueue_step(capture_stream, continuing);
    const cudaError_t e = cudaStreamEndCapture(capture_stream, &g);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return api_fail(NBFMM_ERR_CUDA, "batch step capture: %s", cudaGetErrorString(e));
    }
    const cudaError_t e2 = cudaGraphInstantiate(&out.exec, g, 0);
    if (e2 != cudaSuccess) {
      cudaGetLastError();
      cudaGraphDestroy(g);
      out.exec = nullptr;
      return api_fail(NBFMM_ERR_CUDA, "batch step graph instantiate: %s", cudaGetErrorString(e2));
    }
    out.def = g;
    size_t count = 0;
    cudaGraphGetNodes(g, nullptr, &count);
    std::vector<cudaGraphNode_t> nodes(count);
    cudaGraphGetNodes(g, nodes.data(), &count);
    out.kernels = 0;
    for (cudaGraphNode_t nd : nodes) {
      cudaGraphNodeType type;
      cudaGraphNodeGetType(nd, &type);
      if (type == cudaGraphNodeTypeKernel) ++out.kernels;
      if (type == cudaGraphNodeTypeEventRecord) {
        cudaEvent_t ev = nullptr;
        cudaGraphEventRecordNodeGetEvent(nd, &ev);
        if (ev == cap_a) out.node_a = nd;
        if (ev == cap_b) out.node_b = nd;
      }
    }
    if (!out.node_a || !out.node_b) return api_fail(NBFMM_ERR_CUDA, "batch step graph: P2P event nodes not found");
    return cuda_status("batch step graph inspection");
  }

  int build_graphs() {
    if (graphs_built) return NBFMM_OK;
    BATCH_TRY(alloc_head());
    // Each system takes the series as it would stepped alone (nbfmm_solver::p2p_args).
    std::vector<int> h_series(S);
    for (int k = 0; k < S; ++k) {
      h_series[k] = exact ? 0 : series_degree(h_geo[k].cell_x, h_geo[k].cell_y, eps);
    }
    if (cudaMemcpy(sys_series, h_series.data(), sizeof(int) * S, cudaMemcpyHostToDevice) != cudaSuccess) {
      return cuda_status("series flags");
    }
    const int rc = build_graph(first_step, false);
    const int rc2 = rc == NBFMM_OK ? build_graph(next_step, true) : rc;
    if (rc2 != NBFMM_OK) {
      drop_graph();
      return rc2;
    }
    graphs_built = true;
    return NBFMM_OK;
  }

  static int fate_bits(int S, int steps) { return bits_for((long long)S * (steps + 2)); }

  int update(int steps, cudaStream_t s) {
    if (steps <= 0 || n == 0) return NBFMM_OK;
    BATCH_TRY(build_graphs());
    const int N = std::max(n, 1);
    batch_live_scan_kernel<<<1, 1024, 0, s>>>(sys_counts, S, live_base);
    batch_import_kernel<<<grid_for(N, 256, 152 * 16), 256, 0, s>>>(device(), sc, sys_counts, live_base, cur, prev, w,
                                                                   state4, state_prev, grave, n, steps + 1);
    launch_set_int(sc.num_steps, steps, s);
    for (int k = 0; k < steps; ++k) {
      StepGraph& g = k == 0 ? first_step : next_step;
      if (prof_used < prof_max) {
        set_events(g, prof_events[2 * prof_used], prof_events[2 * prof_used + 1]);
        ++prof_used;
      } else if (prof_max > 0 && prof_used == prof_max) {
        set_events(first_step, cap_a, cap_b);
        set_events(next_step, cap_a, cap_b);
        ++prof_used;
      }
      if (cudaGraphLaunch(g.exec, s) != cudaSuccess) return cuda_status("cudaGraphLaunch");
    }
    batch_export_fate_kernel<<<grid_for(N, 256, 152 * 16), 256, 0, s>>>(device(), sc, state4, state_prev, grave);
    batch_fate_keys_kernel<<<grid_for(N, 256, 152 * 16), 256, 0, s>>>(device(), sc, grave, keys_a, vals_a);
    sort(sc.n_import, fate_bits(S, steps), s);
    batch_counts_kernel<<<grid_for(S, 256, 152), 256, 0, s>>>(skey, sc, S, sys_counts);
    launch_export_gather(sc, perm, grave, cur, prev, w, N, s);
    return cuda_status("nbfmm_batch_update");
  }
};

extern "C" {

int nbfmm_batch_create(int num_systems, const int* particle_offsets, const int* num_levels,
                       const float* position_limits, float tick, float grav_const, nbfmm_batch** out) {
  if (!out) return api_fail(NBFMM_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if (num_systems < 1 || num_systems > (1 << 20)) return api_fail(NBFMM_ERR_INVALID, "num_systems outside [1, 2^20]");
  if (!particle_offsets || !num_levels || !position_limits) return api_fail(NBFMM_ERR_INVALID, "null table");
  if (particle_offsets[0] != 0) return api_fail(NBFMM_ERR_INVALID, "particle_offsets[0] must be 0");
  for (int s = 0; s < num_systems; ++s) {
    if (particle_offsets[s + 1] < particle_offsets[s]) {
      return api_fail(NBFMM_ERR_INVALID, "particle_offsets must be non-decreasing (system %d)", s);
    }
    if (num_levels[s] < 0 || num_levels[s] > kMaxLevels - 1) {
      return api_fail(NBFMM_ERR_INVALID, "num_levels[%d] = %d outside [0, %d]", s, num_levels[s], kMaxLevels - 1);
    }
    const float* l = position_limits + 4 * s;
    if (!std::isfinite(l[0]) || !std::isfinite(l[1]) || !std::isfinite(l[2]) || !std::isfinite(l[3]) ||
        !(l[0] < l[2]) || !(l[1] < l[3])) {
      return api_fail(NBFMM_ERR_INVALID, "limits of system %d must be finite with min < max", s);
    }
  }
  if (particle_offsets[num_systems] > (1 << 28)) return api_fail(NBFMM_ERR_INVALID, "more than 2^28 particles");
  const float tick_scaled = tick * std::sqrt(grav_const);  // stars.cu:31
  if (!(tick_scaled > 0.0f) || !std::isfinite(tick_scaled)) {
    return api_fail(NBFMM_ERR_INVALID, "tick * sqrt(grav_const) must be finite and > 0");
  }
  nbfmm_batch* h = new (std::nothrow) nbfmm_batch();
  if (!h) return api_fail(NBFMM_ERR_NOMEM, "host allocation failed");
  int rc = h->init(num_systems, particle_offsets, num_levels, position_limits, tick_scaled);
  if (rc == NBFMM_OK) rc = h->alloc_head();
  if (rc != NBFMM_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return NBFMM_OK;
}

int nbfmm_batch_destroy(nbfmm_batch* batch) {
  delete batch;
  return NBFMM_OK;
}

int nbfmm_batch_set_epsilon(nbfmm_batch* batch, float epsilon) {
  if (!batch) return api_fail(NBFMM_ERR_INVALID, "null batch handle");
  if (!(epsilon > 0.0f) || !std::isfinite(epsilon)) return api_fail(NBFMM_ERR_INVALID, "epsilon must be finite and > 0");
  batch->drop_graph();
  batch->eps = epsilon;
  return NBFMM_OK;
}

int nbfmm_batch_set_arithmetic(nbfmm_batch* batch, int arithmetic) {
  if (!batch) return api_fail(NBFMM_ERR_INVALID, "null batch handle");
  if (arithmetic != NBFMM_ARITH_FAST && arithmetic != NBFMM_ARITH_EXACT) {
    return api_fail(NBFMM_ERR_INVALID, "arithmetic must be NBFMM_ARITH_FAST (0) or NBFMM_ARITH_EXACT (1)");
  }
  batch->drop_graph();
  batch->exact = arithmetic;
  return NBFMM_OK;
}

int nbfmm_batch_set_item_passes(nbfmm_batch* batch, const int* passes_per_item) {
  if (!batch) return api_fail(NBFMM_ERR_INVALID, "null batch handle");
  if (!passes_per_item) return api_fail(NBFMM_ERR_INVALID, "null table");
  for (int s = 0; s < batch->S; ++s) {
    if (passes_per_item[s] != 2 && passes_per_item[s] != 4) {
      return api_fail(NBFMM_ERR_INVALID, "passes per item of system %d must be 2 or 4, got %d", s, passes_per_item[s]);
    }
  }
  if (batch->S > 0) {
    const cudaError_t e = cudaMemcpy(batch->sys_passes, passes_per_item, sizeof(int) * batch->S,
                                     cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return api_fail(NBFMM_ERR_CUDA, "nbfmm_batch_set_item_passes: %s", cudaGetErrorString(e));
    }
  }
  return NBFMM_OK;
}

int nbfmm_batch_state(nbfmm_batch* batch, float** gpuptr_position_cur, float** gpuptr_position_pre,
                      float** gpuptr_weight) {
  if (!batch) return api_fail(NBFMM_ERR_INVALID, "null batch handle");
  if (gpuptr_position_cur) *gpuptr_position_cur = reinterpret_cast<float*>(batch->cur);
  if (gpuptr_position_pre) *gpuptr_position_pre = reinterpret_cast<float*>(batch->prev);
  if (gpuptr_weight) *gpuptr_weight = batch->w;
  return NBFMM_OK;
}

int nbfmm_batch_num_stars(nbfmm_batch* batch, int* num_stars) {
  if (!batch || !num_stars) return api_fail(NBFMM_ERR_INVALID, "null argument");
  if (cudaMemcpy(num_stars, batch->sys_counts, sizeof(int) * batch->S, cudaMemcpyDeviceToHost) != cudaSuccess) {
    return cuda_status("nbfmm_batch_num_stars");
  }
  return NBFMM_OK;
}

int nbfmm_batch_update(nbfmm_batch* batch, int num_steps, void* stream) {
  if (!batch) return api_fail(NBFMM_ERR_INVALID, "null batch handle");
  if (num_steps < 0) return api_fail(NBFMM_ERR_INVALID, "num_steps must be >= 0");
  return batch->update(num_steps, reinterpret_cast<cudaStream_t>(stream));
}

int nbfmm_batch_profile_begin(nbfmm_batch* batch, int max_steps) {
  if (!batch) return api_fail(NBFMM_ERR_INVALID, "null batch handle");
  if (max_steps < 0) return api_fail(NBFMM_ERR_INVALID, "max_steps must be >= 0");
  BATCH_TRY(batch->build_graphs());
  batch->drop_profile_events();
  batch->prof_events.resize(2 * (size_t)max_steps, nullptr);
  for (auto& e : batch->prof_events) {
    if (cudaEventCreate(&e) != cudaSuccess) return cuda_status("cudaEventCreate");
  }
  batch->prof_max = max_steps;
  batch->prof_used = 0;
  return NBFMM_OK;
}

int nbfmm_batch_profile_end(nbfmm_batch* batch, float* p2p_ms_total, int* p2p_launches) {
  if (!batch || !p2p_ms_total || !p2p_launches) return api_fail(NBFMM_ERR_INVALID, "null argument");
  const int used = std::min(batch->prof_used, batch->prof_max);
  float total = 0.0f;
  for (int k = 0; k < used; ++k) {
    if (cudaEventSynchronize(batch->prof_events[2 * k + 1]) != cudaSuccess) return cuda_status("cudaEventSynchronize");
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, batch->prof_events[2 * k], batch->prof_events[2 * k + 1]) != cudaSuccess) {
      return cuda_status("cudaEventElapsedTime");
    }
    total += ms;
  }
  if (batch->graphs_built) {
    batch->set_events(batch->first_step, batch->cap_a, batch->cap_b);
    batch->set_events(batch->next_step, batch->cap_a, batch->cap_b);
  }
  batch->drop_profile_events();
  *p2p_ms_total = total;
  *p2p_launches = used;
  return cuda_status("nbfmm_batch_profile_end");
}

int nbfmm_batch_kernel_launches(nbfmm_batch* batch, int num_steps, long long* launches) {
  if (!batch || !launches) return api_fail(NBFMM_ERR_INVALID, "null argument");
  if (num_steps <= 0) {
    *launches = 0;
    return NBFMM_OK;
  }
  BATCH_TRY(batch->build_graphs());
  const int passes = (nbfmm_batch::fate_bits(batch->S, num_steps) + kRadixMaxBits - 1) / kRadixMaxBits;
  const int outside = 3 + 2 + 3 * passes + 1 + 1;  // scan, import, step count, fate, keys, sort, counts, gather
  *launches = batch->first_step.kernels + (long long)(num_steps - 1) * batch->next_step.kernels + outside;
  return NBFMM_OK;
}

}  // extern "C"
