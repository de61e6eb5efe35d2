// engine.cuh -- shared definitions of the GB300 nbfmm engine (sm_103a).
//
// Data layout in HBM (one solver):
//   particles, sorted by leaf cell (row-major key iy*B + ix):
//     sorted4  float4 [max_n]   x, y, mass, original index (int bits)       16 B / particle
//     seff     float2 [max_n]   near-field (and, after L2P, total) effect    8 B / particle
//     skey     uint32 [max_n]   leaf cell key of each sorted particle        4 B / particle
//   sort workspace: keys/values ping-pong (4 x 4 B / particle), per-tile digit counts, digit totals
//   cells, compact per level (level l has D_l = B >> l cells per side, row-major, offset sum_{k<l} D_k^2):
//     cell4    float4 [cells]   centre of mass x, y, mass, 0
//     ceff     float2 [cells]   local (far-field) effect
//   head     int32 [B*B + 1]  first sorted index of each leaf cell
//   work     int2  [...]      non-empty (cell, chunk of up to 128 targets) items for P2P
// B = 2^(num_level + 1) leaf cells per side (source/nbfmm/core/solver.cu:19).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nbfmm_gb300 {

constexpr int kMaxLevels = 11;           // num_level in [0, 10], B <= 2048
constexpr int kSortThreads = 256;        // radix sort CTA
constexpr int kSortItems = 16;           // items per thread
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096 items per tile
constexpr int kRadixMaxBits = 8;         // digit bits per pass of the (key, value) radix sort
constexpr int kRecMaxBits = 10;          // digit bits per pass of the record sort (launch_sort_records)
#ifndef NBFMM_REC_ITEMS
#define NBFMM_REC_ITEMS 16
#endif
constexpr int kRecItems = NBFMM_REC_ITEMS;  // record sort: items per thread
constexpr int kRecTile = kSortThreads * kRecItems;  // 4096 items per tile
constexpr int kP2PThreads = 128;        // 4 independent warps per CTA
#ifndef NBFMM_P2P_ITEM_PASSES
#define NBFMM_P2P_ITEM_PASSES 4
#endif
constexpr int kP2PPasses = NBFMM_P2P_ITEM_PASSES;  // passes of 32 targets in one work item, by default (2 or 4)
constexpr int kP2PChunk = 32 * kP2PPasses;  // targets per work item, by default
constexpr int kP2PMinChunk = 64;             // the smallest work item a work list may use (2 passes)

// A P2P work item is (cell, y). y >= 0: the item runs passes [first, first + passes) of 32 targets of the cell,
// encoded first | passes << 24 (passes 1..4); y = -1: the paired tails of the cell and the next (launch_worklist).
__host__ __device__ __forceinline__ int work_item(int first_pass, int passes) { return first_pass | (passes << 24); }
__host__ __device__ __forceinline__ int item_first_pass(int y) { return y & 0xFFFFFF; }
__host__ __device__ __forceinline__ int item_passes(int y) { return y >> 24; }

// Work list entries a solve may need: a non-empty cell of n targets yields at most n/kP2PMinChunk + 2 items
// (its chunks and one paired-tail item) with paired tails, at most n/kP2PMinChunk + 1 without.
inline size_t work_list_capacity(size_t num_cells, size_t n) { return 2 * num_cells + n / kP2PMinChunk + 1; }

#ifndef NBFMM_P2P_PAIR_TAILS
#define NBFMM_P2P_PAIR_TAILS 1  // 0: never pair tails, whatever a launch asks
#endif

#ifdef __CUDACC__
// True when the last n mod 32 targets of leaf cell c and those of its row neighbour c ^ 1 run together in one
// pass (cells 2i and 2i + 1 always share a row, in every system of a batch too): both cells have such a
// partial pass and together they fill at most 32 lanes.
__device__ __forceinline__ bool tails_paired(const int* __restrict__ head, int c) {
  const int p = c ^ 1;
  const int t = (head[c + 1] - head[c]) & 31, tp = (head[p + 1] - head[p]) & 31;
  return NBFMM_P2P_PAIR_TAILS && t > 0 && tp > 0 && t + tp <= 32;
}
#endif

struct Geometry {
  float xmin, ymin, xmax, ymax;  // position limits [x_min, y_min, x_max, y_max]
  float cell_x, cell_y;          // leaf cell size, (max - min) / B in FP32 (predo.cu:112-113)
  int num_level;                 // L
  int base_dim;                  // B
};

struct Levels {
  int count;                     // number of stored cell levels (max(L, 1))
  int dim[kMaxLevels];           // cells per side of each level
  int offset[kMaxLevels];        // first cell of each level in cell4 / ceff
  int total;                     // total cells over all levels
};

// Leaf cell coordinate of one position component, floorf((v - lo) / cell) as in predo.cu:37-38, with IEEE
// division; NaN and values below the domain give 0, values at or above the upper edge give B - 1.
__device__ __forceinline__ int cell_coord(float v, float lo, float cell, int dim) {
  const float f = floorf(__fdiv_rn(__fsub_rn(v, lo), cell));
  if (!(f >= 0.0f)) return 0;
  if (f >= (float)dim) return dim - 1;
  return (int)f;
}

__device__ __forceinline__ uint32_t leaf_key(const Geometry& g, float x, float y) {
  const int ix = cell_coord(x, g.xmin, g.cell_x, g.base_dim);
  const int iy = cell_coord(y, g.ymin, g.cell_y, g.base_dim);
  return (uint32_t)(ix + iy * g.base_dim);
}

// leaf_key by a multiplication with inv = RN(1/cell): RN(d * inv) is within 1.6 * 2^-23 relative of the correctly
// rounded quotient RN(d / cell) (two roundings of 2^-24 each, plus RN's own), so where the floors of q -/+ 2^-20 |q|
// agree they are the floor of RN(d / cell); near a cell edge (and for NaN or infinities) the IEEE division decides.
__device__ __forceinline__ int cell_coord_mul(float v, float lo, float cell, float inv, int dim) {
  const float d = __fsub_rn(v, lo);
  const float q = __fmul_rn(d, inv);
  const float m = __fmul_rn(fabsf(q), 0x1p-20f);
  float f = floorf(__fsub_rn(q, m));
  if (!(f == floorf(__fadd_rn(q, m)))) f = floorf(__fdiv_rn(d, cell));
  if (!(f >= 0.0f)) return 0;
  if (f >= (float)dim) return dim - 1;
  return (int)f;
}

__device__ __forceinline__ uint32_t leaf_key_mul(const Geometry& g, float2 inv, float x, float y) {
  const int ix = cell_coord_mul(x, g.xmin, g.cell_x, inv.x, g.base_dim);
  const int iy = cell_coord_mul(y, g.ymin, g.cell_y, inv.y, g.base_dim);
  return (uint32_t)(ix + iy * g.base_dim);
}

// Outside the limits, the prune test of source/nbfmm/display/stars/prune.cu:40-41 (NaN is kept).
__device__ __forceinline__ bool outside(const Geometry& g, float x, float y) {
  return x < g.xmin || y < g.ymin || x > g.xmax || y > g.ymax;
}

// kernelFunction (include/nbfmm/core/kernel_function.hpp:29-40) with correctly rounded sqrt and division
// and no fused multiply-add, so that it rounds like the reference compiled for a CPU. Used for the cell
// stages, whose evaluation count is small.
__device__ __forceinline__ float2 kernel_exact(float2 t, float2 s, float m, float eps) {
  const float dx = __fsub_rn(s.x, t.x);
  const float dy = __fsub_rn(s.y, t.y);
  const float r = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
  const float tmp = __fdiv_rn(m, __fadd_rn(__fmul_rn(__fmul_rn(r, r), r), eps));
  return make_float2(__fmul_rn(dx, tmp), __fmul_rn(dy, tmp));
}

// The leaf sums of a cell (sum x*m, sum y*m, sum m), accumulated in sorted order one star at a time, so they
// round exactly like the sequential loop of the reference's P2M check (check/core/solver/p2m.cu:36-46). A warp
// adds one chunk of up to 32 consecutive stars (lane j holds star j): every lane puts its (x*m, y*m, m) into the
// warp's buffer of 32 float4, then lane k < 3 adds component k of stars 0, 1, ... in turn into `acc`. That is one
// shared-memory load and one add per star and component lane, where broadcasting each star to every lane took
// three shuffles. Called by the whole warp with the same `count`; cell_sums_get reads the three sums.
__device__ __forceinline__ void cell_sums_add_chunk(float& acc, float4* __restrict__ buf, float x, float y, float m,
                                                    int count, int lane) {
  buf[lane] = make_float4(__fmul_rn(x, m), __fmul_rn(y, m), m, 0.0f);
  __syncwarp();
  if (lane < 3) {
    const float* b = reinterpret_cast<const float*>(buf) + lane;
#pragma unroll 8
    for (int j = 0; j < count; ++j) acc = __fadd_rn(acc, b[4 * j]);
  }
  __syncwarp();  // the buffer is free for the next chunk
}

// The sums of cell_sums_add_chunk in every lane: (sum x*m, sum y*m, sum m).
__device__ __forceinline__ void cell_sums_get(float acc, float& sx, float& sy, float& sw) {
  sx = __shfl_sync(0xffffffffu, acc, 0);
  sy = __shfl_sync(0xffffffffu, acc, 1);
  sw = __shfl_sync(0xffffffffu, acc, 2);
}

// Centre of mass (p2m.cu:72): (sum x*m) / (sum m) per component; an empty cell is (0, 0) with mass 0.
__device__ __forceinline__ float4 centre_of_mass(float sx, float sy, float sw, bool nonempty) {
  if (!nonempty) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  return make_float4(__fdiv_rn(sx, sw), __fdiv_rn(sy, sw), sw, 0.0f);
}

constexpr int kM2LTile = 16;
constexpr int kM2LHalo = kM2LTile + 4;

// M2L (m2l.cu:24-60) for one 16x16 tile of target cells of one level (x0, y0 even): the 20x20 halo of
// sources is staged in shared memory; each target sums the children of its parent's neighbours minus its own
// 3x3 (y outer, x inner, the reference's order) and, with add_parent, adds its parent's effect afterwards
// (l2l.cu:33-35). `cells`/`eff` point at the level, `parent_eff` at the parent level. Called by all threads of
// a 16x16 CTA.
__device__ __forceinline__ void m2l_tile(float4 (*halo)[kM2LHalo], const float4* __restrict__ cells,
                                         float2* __restrict__ eff, int dim, const float2* __restrict__ parent_eff,
                                         int dim_parent, int add_parent, int x0, int y0, float eps) {
  const int tid = threadIdx.y * kM2LTile + threadIdx.x;
  for (int k = tid; k < kM2LHalo * kM2LHalo; k += kM2LTile * kM2LTile) {
    const int hx = k % kM2LHalo, hy = k / kM2LHalo;
    const int gx = x0 - 2 + hx, gy = y0 - 2 + hy;
    halo[hy][hx] = (gx >= 0 && gx < dim && gy >= 0 && gy < dim) ? cells[gy * dim + gx]
                                                                 : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
  __syncthreads();
  const int tx = x0 + threadIdx.x, ty = y0 + threadIdx.y;
  if (tx >= dim || ty >= dim) return;
  const float4 t = halo[ty - y0 + 2][tx - x0 + 2];
  const float2 tp = make_float2(t.x, t.y);
  const int px = tx & ~1, py = ty & ~1;
  float ex = 0.0f, ey = 0.0f;
  for (int y = py - 2; y < py + 4; ++y) {
    if (y < 0 || y >= dim) continue;
    for (int x = px - 2; x < px + 4; ++x) {
      if (x < 0 || x >= dim) continue;
      if (abs(x - tx) > 1 || abs(y - ty) > 1) {
        const float4 s = halo[y - y0 + 2][x - x0 + 2];
        const float2 k = kernel_exact(tp, make_float2(s.x, s.y), s.z, eps);
        ex = __fadd_rn(ex, k.x);
        ey = __fadd_rn(ey, k.y);
      }
    }
  }
  if (add_parent) {
    const float2 p = parent_eff[(ty >> 1) * dim_parent + (tx >> 1)];
    ex = __fadd_rn(ex, p.x);
    ey = __fadd_rn(ey, p.y);
  }
  eff[ty * dim + tx] = make_float2(ex, ey);
}

// ---- launchers (defined in sort.cu / tree.cu / p2p.cu), all asynchronous on `stream` --------------------

// Keys of positions given as float2 [n] (caller order); values = 0..n-1.
void launch_keys_from_positions(const Geometry& g, const float2* pos, const int* d_n, uint32_t* keys,
                                uint32_t* vals, int max_n, cudaStream_t stream);

// Stable LSD radix sort of (keys, vals) on the low `key_bits` bits; n read from device memory. Passes
// alternate between the two buffer pairs; returns 0 when the result is in (keys_a, vals_a), 1 when it is in
// (keys_b, vals_b).
int launch_radix_sort(uint32_t* keys_a, uint32_t* vals_a, uint32_t* keys_b, uint32_t* vals_b,
                      uint32_t* counts, uint32_t* digit_total, const int* d_n, int max_n, int key_bits,
                      cudaStream_t stream);

// Stable LSD radix sort of caller-order particles by leaf key, carrying each particle's record: on return
// rec_final[i] = (x, y, m, original index bits), key_final[i] its leaf key and perm[i] its original index, in
// key order (ties in caller order). rec_tmp / key_tmp hold the passes in between. counts needs
// 2^kRecMaxBits * ceil(max_n / kRecTile) words and digit_total 2^kRecMaxBits.
int record_sort_passes(int key_bits);
void launch_sort_records(const Geometry& g, const float2* pos, const float* w, const int* d_n, int max_n,
                         int key_bits, float4* rec_final, float4* rec_tmp, uint32_t* key_final, uint32_t* key_tmp,
                         uint32_t* perm, uint32_t* counts, uint32_t* digit_total, cudaStream_t stream);

// head[c] = first index with key >= c, c in [0, num_cells]; *d_n_alive = head[num_cells].
void launch_head(const uint32_t* keys, const int* d_n, int num_cells, int* head, int* d_n_alive,
                 cudaStream_t stream);

// Work list of (cell, chunk) items over non-empty leaf cells; *d_work_count receives the count.
// Work items of the non-empty cells: a cell's passes of 32 targets in items of `passes_per_item` passes (2 or 4;
// with sys_passes, the value of the cell's system, found by binary search over sys_cell_base[0..num_systems]).
// With pair_tails, a cell whose tail is paired (tails_paired) clips its items to its whole passes of 32 targets,
// and the even cell of the pair files one more item, (cell, -1): the tails of cell and cell + 1. p2p_kernel reads
// both layouts (P2PArgs::pair_tails). Measured on GB300: pairing takes 1.4% off P2P on a 16.8M two-disk step and
// 5% off 20k-star steps, and costs 5% on the batched form's launch of 512 small systems. The batched form pairs
// all the same: which sources take the Newton reciprocal follows their place in a pass, so a batched system
// stays bit-identical to the same system stepped alone only if both pair alike. The item size does not change
// any result: a pass is packed with the same neighbour pass (0-1, 2-3) and a cell's odd last pass runs alone
// whether items hold 2 or 4 passes.
// With head_copy, head[0..num_cells] is also copied there (the layout the next step's re-sort starts from).
void launch_worklist(const int* head, int num_cells, int2* work, int* d_work_count, bool pair_tails,
                     cudaStream_t stream, int passes_per_item = kP2PPasses, const int* sys_cell_base = nullptr,
                     const int* sys_passes = nullptr, int num_systems = 0, int* head_copy = nullptr);

// P2M on the sorted particles: leaf centres of mass summed in sorted order (predo, and the stage entry point).
void launch_p2m(const Geometry& g, const int* head, const float4* sorted4, float4* cell0, cudaStream_t stream);

// M2M, every level 1..L-1.
void launch_m2m(const Levels& lv, float4* cell4, cudaStream_t stream);

// M2L on every level; with `with_l2l` the parent effect is added on the way down (M2L + L2L fused).
void launch_m2l(const Levels& lv, const float4* cell4, float2* ceff, float eps, bool with_l2l, cudaStream_t stream);

// The far field of a solve: M2M up every level, then M2L with L2L fused down every level. The levels of at most
// 32 cells per side run in one launch.
void launch_far_field(const Levels& lv, float4* cell4, float2* ceff, float eps, cudaStream_t stream);

// L2L alone (stage entry point).
void launch_l2l(const Levels& lv, float2* ceff, cudaStream_t stream);

// L2P alone: seff[i] += ceff[level 0][skey[i]] (stage entry point).
void launch_l2p(const int* d_n, const uint32_t* skey, const float2* ceff0, float2* seff, int max_n, cudaStream_t stream);

// postdo alone: eff_origin[perm[i]] = seff[i] (stage entry point).
void launch_postdo(const int* d_n, const uint32_t* perm, const float2* seff, float2* eff_origin, int max_n,
                   cudaStream_t stream);

// Sorted leaf keys from head (stage entry point helper): skey[i] = cell of i.
void launch_keys_from_head(const int* head, int num_cells, uint32_t* skey, cudaStream_t stream);

// kVerlet on a batch (P2PArgs::num_systems > 0) runs as kVerletBatch, whose epilogue takes each item's system.
enum P2PEpilogue { kStoreSorted = 0, kSolve = 1, kVerlet = 2, kVerletBatch = 3 };

constexpr uint32_t kStayFlag = 0x80000000u;  // P2PArgs::next_key: the star stays in its cell

struct P2PArgs {
  const float4* sorted4;   // sorted particles
  const int* head;         // leaf heads
  const int2* work;        // (cell, chunk) items
  int pair_tails;          // the work list pairs tails (launch_worklist's pair_tails)
  const int* d_work_count;
  int* d_work_next;        // dynamic scheduling counter, zero before launch
  int base_dim;
  float eps;
  int exact;               // 1: correctly rounded kernelFunction, no contraction (NBFMM_ARITH_EXACT)
  // Fast arithmetic: the degree of the reciprocal series that may replace 1 / (r^3 + eps) in the items away from
  // the leaf grid's edges (series_degree), 0 for none; inv_eps = RN(1 / eps).
  int series;
  float inv_eps;
  const float2* ceff0;     // level-0 local effects (kSolve, kVerlet), may be null when num_level == 0
  float2* seff;            // kStoreSorted: sorted effects
  float2* eff_origin;      // kSolve: effects in caller order
  const float2* sprev;     // kVerlet: sorted previous positions
  float4* state4;          // kVerlet: new state (x', y', m, original index)
  float2* state_prev;      // kVerlet: new previous positions
  float tick;              // kVerlet: tick * sqrt(G)
  // kVerlet: the final states by original index (stars.cuh file_grave), null for none: of the stars the prune at
  // the start of the next step removes, and (one system) of every star on the last step of a call.
  float4* grave;
  const int* d_step;       // 1-based step of the call, and the call's step count
  const int* d_num_steps;
  int* d_sort_n;           // set to *d_n_import when a star leaves in the final prune
  const int* d_n_import;
  // kVerlet: on every step but the call's last, each star's leaf key for the next step by state slot, with
  // kStayFlag when it stays in its cell, or the dead key (B*B; dead_key in a batch) with its final state filed in
  // grave when the next step's prune removes it; null for none. next_stay[c] and next_imm[c] count the stars that
  // stay in cell c and the live stars that move into it (both zero before the launch).
  uint32_t* next_key;
  int* next_stay;
  int* next_imm;
  uint32_t dead_key;       // batch: the dead key, past the last cell of the global space
  Geometry geo;            // kVerlet, one system: leaf geometry and position limits
  float2 inv_cell;         // kVerlet, one system: RN(1 / cell size) per axis (leaf_key_mul)
  // Several systems in one global leaf-cell space (batched form); num_systems == 0 for a single system.
  int num_systems;
  const int* sys_cell_base;  // [num_systems + 1] first global leaf cell of each system
  const int* sys_dim;        // [num_systems] leaf cells per side of each system
  const int* sys_series;     // [num_systems] the series degree of each system (P2PArgs::series), or null
  const Geometry* sys_geo;   // [num_systems] kVerlet with next_key: each system's geometry and limits
  const float2* sys_inv;     // [num_systems] kVerlet with next_key: each system's RN(1 / cell size)
};

void launch_p2p(const P2PArgs& a, P2PEpilogue mode, int num_sms, cudaStream_t stream);

// The series arithmetic of p2p.cu for a leaf grid of these cell sizes and this eps: the farthest pair of an item
// whose neighbourhood avoids the grid's edges is 2 sqrt(2) cells apart, and its v = r^3 / eps decides the degree
// of the series that stays within its error bound: 2, or 0 where it does not apply.
int series_degree(float cell_x, float cell_y, float eps);

}  // namespace nbfmm_gb300
