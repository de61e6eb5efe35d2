// stars.cu -- the time-stepping path of the GB300 engine: Stars::update (solve + Verlet + prune) without
// host synchronisation.
//
// Reference path (source/nbfmm/display/stars/): update.cu:47-55 solves, applies the Stormer-Verlet update
// (update.cu:26-42) in the caller's order, then prune.cu:28-62 stable-partitions the stars still inside the
// limits to the front and reads the new count back to the host (thrust::find, prune.cu:61).
//
// Here the stars live in an internal state kept in the previous step's cell order: state4 = (x, y, m,
// original index), state_prev = previous positions. A step sorts the state by leaf cell, puts each cell back in
// index order (the reference's predo sorts the caller's arrays, so its cells list their stars by index; the sort
// here starts from the previous cell order), gathers it, builds the tree and runs P2P with the L2P + Verlet
// epilogue, which writes the new state in the new cell order.
// Pruning is folded into the next step's keys (the key pass of a call's first step, the P2P epilogue of the step
// before otherwise): a star outside the limits gets the key B*B, sorts behind every live star and drops out
// (head[B*B] is the new count), and its final state is filed under its original index together with its death
// step. A call's first step sorts the state with the radix sort; the steps after it re-sort from the previous
// step's cell order (below). The state of the public arrays (survivors in their previous
// relative order, then the pruned stars, most recent first) is restored once at the end of the call.
#include "engine.cuh"
#include "stars.cuh"

namespace nbfmm_gb300 {

namespace {

__global__ void import_kernel(StepCounters sc, const float2* __restrict__ cur, const float2* __restrict__ prev,
                              const float* __restrict__ w, float4* __restrict__ state4,
                              float2* __restrict__ state_prev) {
  const int n = *sc.num_star;
  // Resuming, the state already holds these stars with these indices (in the last step's cell order).
  const int copy = (sc.resume && sc.resume[0]) ? 0 : n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < copy; i += gridDim.x * blockDim.x) {
    const float2 c = cur[i];
    state4[i] = make_float4(c.x, c.y, w[i], __int_as_float(i));
    state_prev[i] = prev[i];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *sc.n_cur = n;
    *sc.n_import = n;
    *sc.step = 1;
    *sc.prune = 0;
    if (sc.sort_n) *sc.sort_n = 0;  // raised by the export if the call loses a star
    if (sc.first_n) *sc.first_n = copy;
  }
}

// The state a call leaves is in the last step's cell order, and each call imports the public arrays afresh,
// which puts the stars back in caller order and makes the first sort and gather of the call do full work. When
// the previous call lost no star, its export was the identity (public entry i = record i), so public arrays
// equal to the records bit for bit mean that the import would rebuild exactly the stars the state holds, with
// the same original indices; the call then continues from the state. The step's result does not depend on the
// order the state is in (the sort and the in-cell index order fix it), so both ways give the same bits.
__global__ void resume_check_kernel(StepCounters sc, const float2* __restrict__ cur, const float2* __restrict__ prev,
                                    const float* __restrict__ w, const float4* __restrict__ grave) {
  const int n = *sc.num_star;
  if (!sc.resume[0] || n != sc.resume[1]) {
    if (blockIdx.x == 0 && threadIdx.x == 0) sc.resume[0] = 0;
    return;
  }
  bool same = true;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 a = grave[2 * i];
    const float m = grave[2 * i + 1].x;
    const float2 c = cur[i], p = prev[i];
    same &= __float_as_uint(c.x) == __float_as_uint(a.x) && __float_as_uint(c.y) == __float_as_uint(a.y) &&
            __float_as_uint(p.x) == __float_as_uint(a.z) && __float_as_uint(p.y) == __float_as_uint(a.w) &&
            __float_as_uint(w[i]) == __float_as_uint(m);
  }
  if (__any_sync(0xffffffffu, !same) && (threadIdx.x & 31) == 0) sc.resume[0] = 0;
}

__global__ void keys_from_state_kernel(Geometry g, StepCounters sc, const float4* __restrict__ state4,
                                       const float2* __restrict__ state_prev, uint32_t dead_key,
                                       uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                       float4* __restrict__ grave) {
  const int n = sc.first_n ? *sc.first_n : *sc.n_cur;
  const int prune = *sc.prune;
  const int death_rank = *sc.num_steps + 1 - (*sc.step - 1);  // later deaths first in the final order
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = state4[i];
    uint32_t key;
    if (prune && outside(g, p.x, p.y)) {
      key = dead_key;
      file_grave(grave, __float_as_int(p.w), p.x, p.y, state_prev[i], p.z, death_rank);
    } else {
      key = leaf_key(g, p.x, p.y);
    }
    keys[i] = key;
    vals[i] = (uint32_t)i;
  }
}

// ---- Re-sort of a continuing step -----------------------------------------------------------------------------
// Within an update call the state sits in the previous step's cell order (head_old). The previous step's P2P
// epilogue left each star's new leaf key by state slot (kStayFlag set when the star stays in its cell; the dead
// key B*B when the prune at the start of this step removes it) and counted, per cell, the stars that stay and the
// live stars that move in. A step moves most stars by a small fraction of a cell, so most stay. The new cell
// order comes from a counting sort in three short launches instead of the key pass, the radix passes and the
// head search:
//   resort_tile_sum_kernel, resort_head_kernel: heads = exclusive scan of stayers + immigrants per cell, each
//     cell's first immigrant place (head + stayers), and the counts cleared for the next step's epilogue;
//   resort_place_kernel (over the old cells): each stayer goes to its cell's head plus its rank among the cell's
//     stayers in the old order (the order the previous step left each cell in: by index), each immigrant to a
//     place after its new cell's stayers taken from an atomic cursor.
// Dead stars get no place (head[B*B] is the live count). The immigrants' order depends on the atomics, but the
// gather that follows puts every cell in index order, so the step's result does not. The first step of a call that
// continues from the last call's state re-sorts too, with the key word and counts of resume_keys_kernel.
constexpr int kResortThreads = 256;
constexpr int kResortItems = 8;                                // cells per thread in the scan
constexpr int kResortTile = kResortThreads * kResortItems;     // cells per scan tile
constexpr int kPlaceGroup = 16;                                // old cells per warp in resort_place_kernel
constexpr int kPlaceUnroll = 4;                                // chunks of 32 slots whose loads are in flight
constexpr int kMoverCap = 128;

__device__ __forceinline__ int block_sum(int v, int* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  __syncthreads();  // red is free
  if (lane == 0) red[warp] = v;
  __syncthreads();
  int t = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  return t;
}

// Live stars per cell, summed over each tile of kResortTile cells.
__global__ void __launch_bounds__(kResortThreads) resort_tile_sum_kernel(int num_cells, const int* __restrict__ stay,
                                                                         const int* __restrict__ imm_cnt,
                                                                         int* __restrict__ tile_sum,
                                                                         const int* __restrict__ gate) {
  __shared__ int red[kResortThreads / 32];
  if (gate && !*gate) return;
  const int c0 = blockIdx.x * kResortTile;
  int v = 0;
  for (int c = c0 + threadIdx.x; c < min(c0 + kResortTile, num_cells); c += kResortThreads) v += stay[c] + imm_cnt[c];
  v = block_sum(v, red);
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = v;
}

// One tile per CTA: the sum of the tiles before it, then a scan of the tile's counts.
__global__ void __launch_bounds__(kResortThreads) resort_head_kernel(int num_cells, int* __restrict__ stay,
                                                                     int* __restrict__ imm_cnt,
                                                                     const int* __restrict__ tile_sum,
                                                                     int* __restrict__ head, int* __restrict__ imm_next,
                                                                     int* __restrict__ d_n_alive,
                                                                     const int* __restrict__ gate) {
  __shared__ int red[kResortThreads / 32];
  __shared__ int warp_tot[kResortThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (gate && !*gate) {  // not re-sorting: only the counts are cleared
    for (int c = blockIdx.x * kResortTile + threadIdx.x; c < min((int)(blockIdx.x + 1) * kResortTile, num_cells);
         c += kResortThreads) {
      stay[c] = 0;
      imm_cnt[c] = 0;
    }
    return;
  }
  int before = 0;
  for (int t = threadIdx.x; t < (int)blockIdx.x; t += kResortThreads) before += tile_sum[t];
  before = block_sum(before, red);
  const int c0 = blockIdx.x * kResortTile + threadIdx.x * kResortItems;
  int st[kResortItems], cnt[kResortItems], mine = 0;
#pragma unroll
  for (int u = 0; u < kResortItems; ++u) {
    const int c = c0 + u;
    st[u] = c < num_cells ? stay[c] : 0;
    cnt[u] = st[u] + (c < num_cells ? imm_cnt[c] : 0);
    mine += cnt[u];
  }
  int incl = mine;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += y;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  int run = before + incl - mine;
  for (int w = 0; w < warp; ++w) run += warp_tot[w];
#pragma unroll
  for (int u = 0; u < kResortItems; ++u) {
    const int c = c0 + u;
    if (c < num_cells) {
      head[c] = run;
      imm_next[c] = run + st[u];
      stay[c] = 0;  // ready for the next step's epilogue
      imm_cnt[c] = 0;
    }
    run += cnt[u];
    if (c == num_cells - 1) {
      head[num_cells] = run;
      *d_n_alive = run;
    }
  }
}

struct MoverList {
  uint32_t slot[kMoverCap];
  uint32_t key[kMoverCap];
};

// Places the listed immigrants: one atomic per distinct new cell among 32 of them.
__device__ __forceinline__ void place_movers(const MoverList& ml, int count, int* __restrict__ imm_next,
                                             uint32_t* __restrict__ perm, int max_n, int lane) {
  __syncwarp();
  const unsigned below = (1u << lane) - 1u;
  for (int m0 = 0; m0 < count; m0 += 32) {
    const int j = m0 + lane;
    const bool active = j < count;
    const unsigned am = __ballot_sync(0xffffffffu, active);
    if (active) {
      const uint32_t k = ml.key[j];
      const unsigned peers = __match_any_sync(am, k);
      const int leader = __ffs(peers) - 1;
      int first = 0;
      if (lane == leader) first = atomicAdd(&imm_next[k], __popc(peers));
      first = __shfl_sync(peers, first, leader);
      const int at = first + __popc(peers & below);
      if ((unsigned)at < (unsigned)max_n) perm[at] = ml.slot[j];
    }
  }
  __syncwarp();
}

// A warp takes kPlaceGroup consecutive old cells, whose slots form one range starting at a cell's first slot,
// and streams it in chunks of 32. Stayers of one cell carry their cell as key and are contiguous, so a stayer's
// rank in its cell is the number of stayers with its key before it in the chunk, plus those counted in earlier
// chunks when its cell continues the last stayers' cell of the chunk before. Immigrants wait in a per-warp list in
// shared memory.
__global__ void __launch_bounds__(kResortThreads) resort_place_kernel(int num_cells, const int* __restrict__ head_old,
                                                                      const uint32_t* __restrict__ key,
                                                                      const int* __restrict__ head,
                                                                      int* __restrict__ imm_next,
                                                                      uint32_t* __restrict__ perm, int max_n,
                                                                      const int* __restrict__ gate) {
  __shared__ MoverList movers[kResortThreads / 32];
  if (gate && !*gate) return;
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  MoverList& ml = movers[threadIdx.x >> 5];
  const int groups = (num_cells + kPlaceGroup - 1) / kPlaceGroup;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int grp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; grp < groups; grp += warps) {
    const int o0 = grp * kPlaceGroup;
    const int bound = lane < 2 ? head_old[min(o0 + lane * kPlaceGroup, num_cells)] : 0;
    const int begin = __shfl_sync(0xffffffffu, bound, 0), end = __shfl_sync(0xffffffffu, bound, 1);
    uint32_t carry_key = 0xffffffffu;
    int carry = 0, nm = 0;
    for (int base = begin; base < end; base += 32 * kPlaceUnroll) {
      uint32_t w[kPlaceUnroll];
      int h[kPlaceUnroll];
#pragma unroll
      for (int u = 0; u < kPlaceUnroll; ++u) {
        const int i = base + 32 * u + lane;
        w[u] = i < end ? key[i] : (uint32_t)num_cells;  // outside the range: like a dead star
      }
#pragma unroll
      for (int u = 0; u < kPlaceUnroll; ++u) h[u] = (w[u] & kStayFlag) ? head[w[u] & ~kStayFlag] : 0;
#pragma unroll
      for (int u = 0; u < kPlaceUnroll; ++u) {
        const int i = base + 32 * u + lane;
        const uint32_t k = w[u] & ~kStayFlag;
        const bool stays = (w[u] & kStayFlag) != 0;
        const bool moves = !stays && k < (uint32_t)num_cells;
        const unsigned sb = __ballot_sync(0xffffffffu, stays);
        unsigned peers = 0u;
        if (stays) {
          peers = __match_any_sync(sb, k);
          const int at = h[u] + __popc(peers & below) + (k == carry_key ? carry : 0);
          if ((unsigned)at < (unsigned)max_n) perm[at] = (uint32_t)i;
        }
        if (sb) {  // the chunk's last stayers' cell continues into the next chunk
          const int last = 31 - __clz(sb);
          const uint32_t kl = __shfl_sync(0xffffffffu, k, last);
          const int n_last = __popc(__shfl_sync(0xffffffffu, peers, last));
          carry = (kl == carry_key ? carry : 0) + n_last;
          carry_key = kl;
        }
        const unsigned mb = __ballot_sync(0xffffffffu, moves);
        if (nm + __popc(mb) > kMoverCap) {
          place_movers(ml, nm, imm_next, perm, max_n, lane);
          nm = 0;
        }
        if (moves) {
          const int at = nm + __popc(mb & below);
          ml.slot[at] = (uint32_t)i;
          ml.key[at] = k;
        }
        nm += __popc(mb);
      }
    }
    place_movers(ml, nm, imm_next, perm, max_n, lane);
  }
}

__global__ void resume_keys_kernel(Geometry g, float2 inv, StepCounters sc, const float4* __restrict__ sorted4,
                                   const float4* __restrict__ state4, uint32_t* __restrict__ key_word,
                                   int* __restrict__ stay, int* __restrict__ imm_cnt) {
  if (!sc.resume[0]) return;
  const int n = *sc.n_cur;
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * blockDim.x;
  // Whole warps iterate together: the counts are aggregated across the lanes.
  for (int base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
    const int j = base + lane;
    const bool valid = j < n;
    uint32_t old_cell = 0u, key = 0u;
    if (valid) {
      const float4 o = sorted4[j], p = state4[j];
      old_cell = leaf_key_mul(g, inv, o.x, o.y);
      key = leaf_key_mul(g, inv, p.x, p.y);
      key_word[j] = key == old_cell ? key | kStayFlag : key;
    }
    const bool stays = valid && key == old_cell, moves = valid && !stays;
    const unsigned sm = __ballot_sync(0xffffffffu, stays), mm = __ballot_sync(0xffffffffu, moves);
    if (stays) {
      const unsigned peers = __match_any_sync(sm, key);
      if (lane == __ffs(peers) - 1) atomicAdd(&stay[key], __popc(peers));
    }
    if (moves) {
      const unsigned peers = __match_any_sync(mm, key);
      if (lane == __ffs(peers) - 1) atomicAdd(&imm_cnt[key], __popc(peers));
    }
  }
}

__global__ void finish_step_kernel(StepCounters sc) {
  *sc.n_cur = *sc.n_alive;
  *sc.step += 1;
  *sc.prune = 1;
}

// The last prune of the call (prune.cu:40-41 on the final positions) and every star's final state filed by
// original index (fate 0 = alive, fate 1 = pruned by the last step) are done by the last step's P2P epilogue
// (p2p.cu); here only a star lost by an earlier step of the call is noted: the public order then needs the fate
// sort.
__global__ void export_fate_kernel(StepCounters sc) {
  if (sc.sort_n && *sc.n_cur != *sc.n_import) *sc.sort_n = *sc.n_import;
}

__global__ void fate_keys_kernel(StepCounters sc, const float4* __restrict__ grave, uint32_t* __restrict__ keys,
                                 uint32_t* __restrict__ vals) {
  const int n = sc.sort_n ? *sc.sort_n : *sc.n_import;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    keys[i] = (uint32_t)grave_fate(grave, i);
    vals[i] = (uint32_t)i;
  }
}

__global__ void export_gather_kernel(StepCounters sc, const uint32_t* __restrict__ order,
                                     const float4* __restrict__ grave, float2* __restrict__ cur,
                                     float2* __restrict__ prev, float* __restrict__ w, int* __restrict__ mark,
                                     const int* __restrict__ sort_n) {
  const int n = *sc.n_import;
  const bool identity = sort_n && *sort_n == 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (identity) *sc.num_star = n;  // the fate sort and its head ran over nothing
    if (mark) {
      mark[0] = *sc.num_star == n ? 1 : 0;
      mark[1] = *sc.num_star;
    }
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t o = identity ? (uint32_t)i : order[i];
    const float4 a = grave[2 * o];
    cur[i] = make_float2(a.x, a.y);
    prev[i] = make_float2(a.z, a.w);
    w[i] = grave[2 * o + 1].x;
  }
}

__global__ void set_int_kernel(int* p, int v) { *p = v; }

__global__ void prune_keys_kernel(Geometry g, StepCounters sc, const float2* __restrict__ cur,
                                  const float2* __restrict__ prev, const float* __restrict__ w,
                                  uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                  float4* __restrict__ grave) {
  const int n = *sc.num_star;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 c = cur[i];
    const int out = outside(g, c.x, c.y) ? 1 : 0;  // prune.cu:40-41
    keys[i] = (uint32_t)out;
    vals[i] = (uint32_t)i;
    file_grave(grave, i, c.x, c.y, prev[i], w[i], out);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *sc.n_import = n;
}

// ---- Index order inside the leaf cells -------------------------------------------------------------------------
// The reference's predo sorts the caller's arrays stably by leaf cell (predo.cu:127), so each cell lists its stars
// by index. A step here sorts the state, which is kept in the previous step's cell order, so the stars a cell
// received from other cells come as a few increasing runs of indices (one per cell they came from, in that cell's
// order). The helpers below merge those runs (in a global scratch of kOrderScratch words per particle, at the
// cell's own offset) for the cells gather_state_ordered_kernel cannot stage in shared memory.

struct OrderArrays {
  uint32_t *key, *val, *key2, *val2;  // index and state slot, ping-pong
  int *run, *run2, *start;            // run of each element, ping-pong; first element of each run
};

__device__ __forceinline__ OrderArrays order_arrays(uint32_t* base, int stride) {
  OrderArrays a;
  a.key = base;
  a.val = base + stride;
  a.key2 = base + 2 * stride;
  a.val2 = base + 3 * stride;
  a.run = reinterpret_cast<int*>(base + 4 * stride);
  a.run2 = reinterpret_cast<int*>(base + 5 * stride);
  a.start = reinterpret_cast<int*>(base + 6 * stride);
  return a;
}

// True when the cell's stars are not in index order (a descent between neighbours).
__device__ __forceinline__ bool cell_out_of_order(const uint32_t* __restrict__ perm, const float4* __restrict__ state4,
                                                  int h0, int L, int lane) {
  uint32_t last = 0u;
  for (int base = 0; base < L; base += 32) {
    const int i = base + lane;
    const uint32_t o = i < L ? (uint32_t)__float_as_int(state4[perm[h0 + i]].w) : 0xffffffffu;
    uint32_t before = __shfl_up_sync(0xffffffffu, o, 1);
    if (lane == 0) before = base == 0 ? 0u : last;
    if (__any_sync(0xffffffffu, i < L && i > 0 && before > o)) return true;
    last = __shfl_sync(0xffffffffu, o, 31);
  }
  return false;
}

// Loads the cell's (index, slot) pairs and its increasing runs; returns the number of runs. Four chunks of 32 are
// read per round (their slots, then their indices) to keep several loads in flight.
__device__ int order_load(const uint32_t* __restrict__ perm, const float4* __restrict__ state4, int h0, int L,
                          const OrderArrays& a, int lane) {
  int runs = 0;
  uint32_t last = 0u;
  for (int base = 0; base < L; base += 128) {
    uint32_t slot[4], idx[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = base + 32 * u + lane;
      slot[u] = i < L ? perm[h0 + i] : 0u;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = base + 32 * u + lane;
      idx[u] = i < L ? (uint32_t)__float_as_int(state4[slot[u]].w) : 0xffffffffu;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = base + 32 * u + lane;
      if (base + 32 * u >= L) break;  // warp-uniform
      const uint32_t o = idx[u];
      uint32_t before = __shfl_up_sync(0xffffffffu, o, 1);
      if (lane == 0) before = last;
      const bool starts = i < L && (i == 0 || before > o);
      const unsigned ballot = __ballot_sync(0xffffffffu, starts);
      const int r = runs + __popc(ballot & ((2u << lane) - 1u)) - 1;  // (2u << 31) wraps to 0: every lane counted
      if (i < L) {
        a.key[i] = o;
        a.val[i] = slot[u];
        a.run[i] = r;
        if (starts) a.start[r] = i;
      }
      runs += __popc(ballot);
      last = __shfl_sync(0xffffffffu, o, 31);
    }
  }
  __syncwarp();
  return runs;
}

// Merges the runs into index order; returns the slots in that order (a.val or a.val2). Up to kDirectRuns runs,
// each element goes straight to its final place, its offset in its own run plus, for every other run, the number
// of that run's indices below its own (indices are distinct). More runs are merged pairwise, round by round.
constexpr int kDirectRuns = 16;

__device__ const uint32_t* order_merge(int L, int runs, OrderArrays a, int lane) {
  if (runs <= kDirectRuns) {
    for (int i = lane; i < L; i += 32) {
      const uint32_t k = a.key[i];
      const int r = a.run[i];
      int pos = i - a.start[r];
      for (int q = 0; q < runs; ++q) {
        if (q == r) continue;
        int lo = a.start[q], hi = q + 1 < runs ? a.start[q + 1] : L;
        const int sq = lo;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (a.key[mid] < k) lo = mid + 1; else hi = mid;
        }
        pos += lo - sq;
      }
      a.key2[pos] = k;
      a.val2[pos] = a.val[i];
    }
    __syncwarp();
    return a.val2;
  }
  while (runs > 1) {
    for (int i = lane; i < L; i += 32) {
      const uint32_t k = a.key[i];
      const int r = a.run[i];
      const int p = r ^ 1;
      int pos = i;  // an unpaired last run stays in place
      if (p < runs) {
        const int sp = a.start[p], ep = p + 1 < runs ? a.start[p + 1] : L;
        int lo = sp, hi = ep;  // partner elements with a smaller index
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (a.key[mid] < k) lo = mid + 1; else hi = mid;
        }
        const int sr = a.start[r];
        pos = (sr < sp ? sr : sp) + (i - sr) + (lo - sp);
      }
      a.key2[pos] = k;
      a.val2[pos] = a.val[i];
      a.run2[pos] = r >> 1;
    }
    __syncwarp();
    const int merged = (runs + 1) >> 1;
    for (int base = 0; base < merged; base += 32) {  // start[k] = start[2k]
      const int k = base + lane;
      const int st = k < merged ? a.start[2 * k] : 0;
      __syncwarp();
      if (k < merged) a.start[k] = st;
      __syncwarp();
    }
    uint32_t* t = a.key; a.key = a.key2; a.key2 = t;
    t = a.val; a.val = a.val2; a.val2 = t;
    int* u = a.run; a.run = a.run2; a.run2 = u;
    runs = merged;
  }
  return a.val;
}

// Gather + P2M of a step in the reference's order: per leaf cell, the stars in index order (the runs merged when
// the sort left them out of order), their state gathered into cell order and the cell's centre of mass summed in
// that order (p2m.cu:36-46). A warp takes a cell of up to kStageCap stars in one round: it loads the slots, then
// every slot's state (which carries the index) and previous position at once into registers. A cell already in
// index order is written out as loaded. Otherwise each star's final place is worked out from the indices staged
// in shared memory -- usually one long run (the residents) and a few other stars (the arrivals), which are
// sorted across the lanes, placed into the long run by binary search and shift the residents by a prefix count;
// else by its rank across all runs -- the star is written there, and the centre of mass is summed from a
// shared-memory copy in final order. A larger cell, or one of more than kDirectRuns runs and more than 32
// arrivals, is ordered in the global scratch at its own offset and gathered from the state.
constexpr int kStageWarps = 4;
constexpr int kStageChunks = 10;                 // chunks of 32 stars held in registers
constexpr int kStageCap = 32 * kStageChunks;     // 320

struct StageArrays {
  float4 sums[32];  // cell_sums_add_chunk's buffer
  uint32_t key[kStageCap];
  float xs[kStageCap], ys[kStageCap], ms[kStageCap];
  int shift[kStageCap + 1];
  unsigned short run[kStageCap], start[kStageCap], dest[kStageCap];
};

// Sorts one (key, value) pair per lane into ascending key order across the warp (bitonic network).
__device__ __forceinline__ void warp_sort_pairs(uint32_t& k, int& v, int lane) {
#pragma unroll
  for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      const uint32_t ok = __shfl_xor_sync(0xffffffffu, k, stride);
      const int ov = __shfl_xor_sync(0xffffffffu, v, stride);
      const bool ascending = (lane & size) == 0 || size == 32;
      const bool lower = (lane & stride) == 0;
      const bool take = (lower == ascending) ? ok < k : ok > k;
      if (take) {
        k = ok;
        v = ov;
      }
    }
  }
}

// Resident CTAs per SM the ordered gather is compiled and launched for (96 registers at 5, no spills). Measured
// on the 16.8M two-disk step (100 steps, ms per step): 4 CTAs 16.385, 5 CTAs 16.362, 6 CTAs (80 registers,
// spills) 16.409.
#ifndef NBFMM_GATHER_MINB
#define NBFMM_GATHER_MINB 5
#endif

__global__ void __launch_bounds__(kStageWarps * 32, NBFMM_GATHER_MINB) gather_state_ordered_kernel(
    int num_cells, const int* __restrict__ head, const uint32_t* __restrict__ perm, const float4* __restrict__ state4,
    const float2* __restrict__ state_prev, float4* __restrict__ sorted4, float2* __restrict__ sprev,
    float4* __restrict__ cell0, uint32_t* __restrict__ scratch, int max_n) {
  __shared__ StageArrays stage[kStageWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  StageArrays& st = stage[warp];
  const int warps = gridDim.x * kStageWarps;
  for (int c = blockIdx.x * kStageWarps + warp; c < num_cells; c += warps) {
    const int h0 = head[c], h1 = head[c + 1], L = h1 - h0;
    float acc = 0.0f;  // leaf sums, lanes 0-2
    bool done = false;
    if (L <= kStageCap) {
      uint32_t slot[kStageChunks], idx[kStageChunks];
      float4 q[kStageChunks];
      float2 pv[kStageChunks];
#pragma unroll
      for (int u = 0; u < kStageChunks; ++u) {
        const int i = 32 * u + lane;
        slot[u] = i < L ? perm[h0 + i] : 0u;
      }
#pragma unroll
      for (int u = 0; u < kStageChunks; ++u) {
        const int i = 32 * u + lane;
        idx[u] = 0xffffffffu;
        q[u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        pv[u] = make_float2(0.0f, 0.0f);
        if (i < L) {
          q[u] = state4[slot[u]];
          pv[u] = state_prev[slot[u]];
          idx[u] = (uint32_t)__float_as_int(q[u].w);  // the state carries the index
        }
      }
      // Runs of increasing index.
      int runs = 0;
      uint32_t last = 0u;
#pragma unroll
      for (int u = 0; u < kStageChunks; ++u) {
        if (32 * u >= L) break;  // warp-uniform
        const int i = 32 * u + lane;
        uint32_t before = __shfl_up_sync(0xffffffffu, idx[u], 1);
        if (lane == 0) before = last;
        const bool starts = i < L && (i == 0 || before > idx[u]);
        const unsigned ballot = __ballot_sync(0xffffffffu, starts);
        const int r = runs + __popc(ballot & ((2u << lane) - 1u)) - 1;  // (2u << 31) wraps to 0
        if (i < L) {
          st.key[i] = idx[u];
          st.run[i] = (unsigned short)r;
          if (starts) st.start[r] = (unsigned short)i;
        }
        runs += __popc(ballot);
        last = __shfl_sync(0xffffffffu, idx[u], 31);
      }
      __syncwarp();
      if (runs <= 1) {
#pragma unroll
        for (int u = 0; u < kStageChunks; ++u) {
          if (32 * u >= L) break;
          const int i = 32 * u + lane;
          if (i < L) {
            sorted4[h0 + i] = q[u];
            sprev[h0 + i] = pv[u];
          }
          cell_sums_add_chunk(acc, st.sums, q[u].x, q[u].y, q[u].z, min(32, L - 32 * u), lane);
        }
        done = true;
      } else {
        // dest[i] = final place of staged star i. The common case: one long run (the cell's residents) and at
        // most 32 other stars (the arrivals), which are sorted across the lanes, placed into the long run by
        // binary search, and shift the long run's stars by a prefix count.
        int best_len = -1, best_r = 0;
        for (int r = lane; r < runs; r += 32) {
          const int len = (r + 1 < runs ? st.start[r + 1] : L) - st.start[r];
          if (len > best_len) {
            best_len = len;
            best_r = r;
          }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const int ol = __shfl_xor_sync(0xffffffffu, best_len, off);
          const int orr = __shfl_xor_sync(0xffffffffu, best_r, off);
          if (ol > best_len || (ol == best_len && orr < best_r)) {
            best_len = ol;
            best_r = orr;
          }
        }
        const int s0 = st.start[best_r], e0 = s0 + best_len, m = L - best_len;
        bool placed = false;
        if (m <= 32) {
          const int ia = lane < s0 ? lane : e0 + (lane - s0);  // the stars outside the long run
          uint32_t k = lane < m ? st.key[ia] : 0xffffffffu;
          int v = lane < m ? ia : -1;
          warp_sort_pairs(k, v, lane);
          int p = 0;
          if (lane < m) {
            int lo = s0, hi = e0;
            while (lo < hi) {
              const int mid = (lo + hi) >> 1;
              if (st.key[mid] < k) lo = mid + 1; else hi = mid;
            }
            p = lo - s0;
            st.dest[v] = (unsigned short)(p + lane);
          }
          for (int o = lane; o <= best_len; o += 32) st.shift[o] = 0;
          __syncwarp();
          if (lane < m) atomicAdd(&st.shift[p], 1);
          __syncwarp();
          int carry = 0;
          for (int base = 0; base < best_len; base += 32) {  // inclusive prefix of the insertions
            const int o = base + lane;
            int x = o < best_len ? st.shift[o] : 0;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
              const int y = __shfl_up_sync(0xffffffffu, x, off);
              if (lane >= off) x += y;
            }
            if (o < best_len) st.dest[s0 + o] = (unsigned short)(o + carry + x);
            carry += __shfl_sync(0xffffffffu, x, 31);
          }
          placed = true;
        } else if (runs <= kDirectRuns) {  // direct ranks
          for (int i = lane; i < L; i += 32) {
            const uint32_t k = st.key[i];
            const int r = st.run[i];
            int pos = i - st.start[r];
            for (int t = 0; t < runs; ++t) {
              if (t == r) continue;
              int lo = st.start[t], hi = t + 1 < runs ? st.start[t + 1] : L;
              const int s1 = lo;
              while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (st.key[mid] < k) lo = mid + 1; else hi = mid;
              }
              pos += lo - s1;
            }
            st.dest[i] = (unsigned short)pos;
          }
          placed = true;
        }
        if (placed) {
          __syncwarp();
#pragma unroll
          for (int u = 0; u < kStageChunks; ++u) {
            if (32 * u >= L) break;
            const int i = 32 * u + lane;
            if (i < L) {
              const int pos = st.dest[i];
              sorted4[h0 + pos] = q[u];
              sprev[h0 + pos] = pv[u];
              st.xs[pos] = q[u].x;
              st.ys[pos] = q[u].y;
              st.ms[pos] = q[u].z;
            }
          }
          __syncwarp();
          for (int base = 0; base < L; base += 32) {
            const int j = base + lane;
            const bool in = j < L;
            cell_sums_add_chunk(acc, st.sums, in ? st.xs[j] : 0.0f, in ? st.ys[j] : 0.0f, in ? st.ms[j] : 0.0f,
                                min(32, L - base), lane);
          }
          done = true;
        }
      }
    }
    if (!done) {  // a cell larger than the stage, or of many runs
      const uint32_t* order = perm + h0;
      if (L >= 2 && cell_out_of_order(perm, state4, h0, L, lane)) {
        const OrderArrays a = order_arrays(scratch + h0, max_n);
        order = order_merge(L, order_load(perm, state4, h0, L, a, lane), a, lane);
      }
      for (int base = 0; base < L; base += 32) {
        const int i = base + lane;
        float4 q = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (i < L) {
          const uint32_t p = order[i];
          q = state4[p];
          sorted4[h0 + i] = q;
          sprev[h0 + i] = state_prev[p];
        }
        cell_sums_add_chunk(acc, st.sums, q.x, q.y, q.z, min(32, L - base), lane);
      }
    }
    float sx, sy, sw;
    cell_sums_get(acc, sx, sy, sw);
    if (lane == 0) cell0[c] = centre_of_mass(sx, sy, sw, h1 > h0);
    __syncwarp();  // the staging area is free for the next cell
  }
}

int grid_for(long long n, int threads, int cap) {
  long long g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

}  // namespace

void launch_set_int(int* p, int v, cudaStream_t stream) { set_int_kernel<<<1, 1, 0, stream>>>(p, v); }

void launch_import(const StepCounters& sc, const float2* cur, const float2* prev, const float* w, float4* state4,
                   float2* state_prev, int max_n, cudaStream_t stream) {
  import_kernel<<<grid_for(max_n, 256, 152 * 16), 256, 0, stream>>>(sc, cur, prev, w, state4, state_prev);
}

void launch_keys_from_state(const Geometry& g, const StepCounters& sc, const float4* state4, const float2* state_prev,
                            uint32_t dead_key, uint32_t* keys, uint32_t* vals, float4* grave, int max_n,
                            cudaStream_t stream) {
  keys_from_state_kernel<<<grid_for(max_n, 256, 152 * 16), 256, 0, stream>>>(g, sc, state4, state_prev, dead_key, keys,
                                                                             vals, grave);
}

void launch_finish_step(const StepCounters& sc, cudaStream_t stream) { finish_step_kernel<<<1, 1, 0, stream>>>(sc); }

void launch_resort(const ResortArrays& r, int num_cells, int max_n, int* head, int* d_n_alive, cudaStream_t stream,
                   const int* gate) {
  const int tiles = (num_cells + kResortTile - 1) / kResortTile;
  const int groups = (num_cells + kPlaceGroup - 1) / kPlaceGroup;
  resort_tile_sum_kernel<<<tiles, kResortThreads, 0, stream>>>(num_cells, r.stay, r.imm_cnt, r.tile_sum, gate);
  resort_head_kernel<<<tiles, kResortThreads, 0, stream>>>(num_cells, r.stay, r.imm_cnt, r.tile_sum, head,
                                                           r.imm_next, d_n_alive, gate);
  resort_place_kernel<<<grid_for((long long)groups * 32, kResortThreads, 152 * 6), kResortThreads, 0, stream>>>(
      num_cells, r.head_old, r.key, head, r.imm_next, r.perm, max_n, gate);
}

int resort_tiles(int num_cells) { return (num_cells + kResortTile - 1) / kResortTile; }

void launch_resume_keys(const Geometry& g, const StepCounters& sc, const float4* sorted4, const float4* state4,
                        uint32_t* key_word, int* stay, int* imm_cnt, int max_n, cudaStream_t stream) {
  const float2 inv = make_float2(1.0f / g.cell_x, 1.0f / g.cell_y);
  resume_keys_kernel<<<grid_for(max_n, 256, 152 * 8), 256, 0, stream>>>(g, inv, sc, sorted4, state4, key_word, stay,
                                                                       imm_cnt);
}

void launch_export_fate(const StepCounters& sc, cudaStream_t stream) { export_fate_kernel<<<1, 1, 0, stream>>>(sc); }

void launch_fate_keys(const StepCounters& sc, const float4* grave, uint32_t* keys, uint32_t* vals, int max_n,
                      cudaStream_t stream) {
  fate_keys_kernel<<<grid_for(max_n, 256, 152 * 16), 256, 0, stream>>>(sc, grave, keys, vals);
}

void launch_export_gather(const StepCounters& sc, const uint32_t* order, const float4* grave, float2* cur,
                          float2* prev, float* w, int max_n, cudaStream_t stream, int* mark, const int* sort_n) {
  export_gather_kernel<<<grid_for(max_n, 256, 152 * 16), 256, 0, stream>>>(sc, order, grave, cur, prev, w, mark,
                                                                           sort_n);
}

void launch_resume_check(const StepCounters& sc, const float2* cur, const float2* prev, const float* w,
                         const float4* grave, int max_n, cudaStream_t stream) {
  resume_check_kernel<<<grid_for(max_n, 256, 152 * 16), 256, 0, stream>>>(sc, cur, prev, w, grave);
}

void launch_gather_state_ordered(const int* head, int num_cells, const uint32_t* perm, const float4* state4,
                                 const float2* state_prev, float4* sorted4, float2* sprev, float4* cell0,
                                 uint32_t* scratch, int max_n, cudaStream_t stream) {
  gather_state_ordered_kernel<<<grid_for((long long)num_cells * 32, kStageWarps * 32, 152 * NBFMM_GATHER_MINB),
                                kStageWarps * 32, 0,
                                stream>>>(num_cells, head, perm, state4, state_prev, sorted4, sprev, cell0, scratch,
                                          max_n);
}

void launch_prune_keys(const Geometry& g, const StepCounters& sc, const float2* cur, const float2* prev,
                       const float* w, uint32_t* keys, uint32_t* vals, float4* grave, int max_n, cudaStream_t stream) {
  prune_keys_kernel<<<grid_for(max_n, 256, 152 * 16), 256, 0, stream>>>(g, sc, cur, prev, w, keys, vals, grave);
}

}  // namespace nbfmm_gb300
