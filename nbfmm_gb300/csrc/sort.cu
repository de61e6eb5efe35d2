// sort.cu -- preassign for the GB300 engine: leaf keys, a stable LSD radix sort by leaf cell, cell heads
// and the P2P work list.
//
// Replaces predo (source/nbfmm/core/solver/predo.cu:105-135): computeParticleIndex (predo.cu:26-39),
// the iota + thrust::sort_by_key on int2 keys under the row-major operator< (predo.cu:123-127,
// include/nbfmm/utility/operator.hpp:107-109) and extractHead (predo.cu:49-74). The row-major int2 order
// equals the order of the integer key iy*B + ix, and cub's merge sort keeps equal keys in input order, so a
// stable radix sort on that key reproduces the reference's permutation bit for bit.
//
// Sort design: per pass (digits of up to 8 bits), an upsweep writes each 4096-item tile's digit histogram, one
// CTA per digit scans its row of tile counts, and a downsweep ranks each tile's items stably (warp match +
// per-warp digit counters in shared memory) and scatters them. On the step's nearly sorted state, 8-bit digits
// in three passes were measured faster than 10-bit digits in two (0.33 against 0.38 ms at 16.8M): narrower
// digits keep longer runs of a tile together in one store. Loading each round's keys and values inside the
// ranking loop was measured faster here than loading the whole tile first (0.09 against 0.13 ms per pass). Every kernel reads the element count from device memory,
// so the same launches serve any n <= max_n without a host round trip (and can be captured in a graph).
#include "engine.cuh"

namespace nbfmm_gb300 {

namespace {

__device__ __forceinline__ int num_tiles(int n, int tile = kSortTile) { return (n + tile - 1) / tile; }

// Exclusive scan over a 256-thread block; returns the block total in *total.
__device__ __forceinline__ uint32_t block_exclusive_scan_256(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = (lane < kSortThreads / 32) ? warp_sums[lane] : 0u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, s, d);
      if (lane >= d) s += y;
    }
    if (lane < kSortThreads / 32) warp_sums[lane] = s;  // inclusive warp prefix
  }
  __syncthreads();
  const uint32_t warp_prefix = (warp > 0) ? warp_sums[warp - 1] : 0u;
  *total = warp_sums[kSortThreads / 32 - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

// Exclusive scan of up to kSortThreads * 4 values v[tid*4 .. tid*4+3] over a 256-thread block.
__device__ __forceinline__ void block_exclusive_scan_4x256(uint32_t* v4, uint32_t* warp_sums) {
  const uint32_t local = v4[0] + v4[1] + v4[2] + v4[3];
  uint32_t total;
  uint32_t run = block_exclusive_scan_256(local, warp_sums, &total);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint32_t c = v4[k];
    v4[k] = run;
    run += c;
  }
}

__global__ void keys_from_positions_kernel(Geometry g, const float2* __restrict__ pos, const int* __restrict__ d_n,
                                           uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const int n = *d_n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 p = pos[i];
    keys[i] = leaf_key(g, p.x, p.y);
    vals[i] = (uint32_t)i;
  }
}

__global__ void __launch_bounds__(kSortThreads)
radix_upsweep_kernel(const uint32_t* __restrict__ keys, const int* __restrict__ d_n, int shift, int bits,
                     uint32_t* __restrict__ counts, int max_tiles) {
  __shared__ uint32_t hist[1 << kRadixMaxBits];
  const int n = *d_n;
  const int t = blockIdx.x;
  if (t >= num_tiles(n)) return;
  const int nd = 1 << bits;
  const uint32_t mask = (uint32_t)nd - 1u;
  for (int d = threadIdx.x; d < nd; d += kSortThreads) hist[d] = 0u;
  __syncthreads();
  const int base = t * kSortTile;
  const int end = min(base + kSortTile, n);
  for (int i = base + threadIdx.x; i < end; i += kSortThreads) {
    atomicAdd(&hist[(keys[i] >> shift) & mask], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < nd; d += kSortThreads) counts[(size_t)d * max_tiles + t] = hist[d];
}

// One CTA per digit: exclusive scan of that digit's tile counts; the digit's total goes to digit_total.
__global__ void __launch_bounds__(kSortThreads)
radix_scan_kernel(uint32_t* __restrict__ counts, uint32_t* __restrict__ digit_total, const int* __restrict__ d_n,
                  int max_tiles, int tile = kSortTile) {
  __shared__ uint32_t warp_sums[kSortThreads / 32];
  const int nt = num_tiles(*d_n, tile);
  uint32_t* row = counts + (size_t)blockIdx.x * max_tiles;
  uint32_t carry = 0;
  for (int base = 0; base < nt; base += kSortThreads * 4) {
    const int i0 = base + threadIdx.x * 4;
    uint32_t v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = (i0 + k < nt) ? row[i0 + k] : 0u;
    const uint32_t local = v[0] + v[1] + v[2] + v[3];
    uint32_t total;
    uint32_t run = carry + block_exclusive_scan_256(local, warp_sums, &total);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (i0 + k < nt) row[i0 + k] = run;
      run += v[k];
    }
    carry += total;
  }
  if (threadIdx.x == 0) digit_total[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kSortThreads)
radix_downsweep_kernel(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                       uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                       const int* __restrict__ d_n, int shift, int bits, const uint32_t* __restrict__ counts,
                       const uint32_t* __restrict__ digit_total, int max_tiles) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ uint32_t warp_hist[kWarps][1 << kRadixMaxBits];
  __shared__ uint32_t digit_base[1 << kRadixMaxBits];
  __shared__ uint32_t warp_sums[kWarps];
  const int n = *d_n;
  const int t = blockIdx.x;
  if (t >= num_tiles(n)) return;
  const int nd = 1 << bits;
  const uint32_t mask = (uint32_t)nd - 1u;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;

  // Start of every digit in the output: exclusive scan of the digit totals.
  {
    const uint32_t v = (threadIdx.x < nd) ? digit_total[threadIdx.x] : 0u;
    uint32_t total;
    const uint32_t ex = block_exclusive_scan_256(v, warp_sums, &total);
    if (threadIdx.x < nd) digit_base[threadIdx.x] = ex;
  }
  for (int d = lane; d < nd; d += 32) warp_hist[warp][d] = 0u;
  __syncwarp();

  // Warp `warp` owns items [warp*512, warp*512 + 512) of the tile, in 16 rounds of 32 consecutive items.
  const int base = t * kSortTile + warp * (32 * kSortItems);
  const unsigned lt_mask = (1u << lane) - 1u;
  uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const int i = base + r * 32 + lane;
    const bool valid = i < n;
    key[r] = valid ? keys_in[i] : 0u;
    val[r] = valid ? vals_in[i] : 0u;
    const uint32_t digit = valid ? ((key[r] >> shift) & mask) : (uint32_t)nd;  // nd marks an empty slot
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const uint32_t before = valid ? warp_hist[warp][digit] : 0u;
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) warp_hist[warp][digit] = before + __popc(peers);
    __syncwarp();
    rank[r] = before + __popc(peers & lt_mask);
  }
  __syncthreads();
  // Per digit, exclusive prefix over the warps (warp order is item order within the tile).
  for (int d = threadIdx.x; d < nd; d += kSortThreads) {
    uint32_t run = digit_base[d] + counts[(size_t)d * max_tiles + t];
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      const uint32_t c = warp_hist[w][d];
      warp_hist[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const int i = base + r * 32 + lane;
    if (i < n) {
      const uint32_t digit = (key[r] >> shift) & mask;
      const uint32_t dst = warp_hist[warp][digit] + rank[r];
      keys_out[dst] = key[r];
      vals_out[dst] = val[r];
    }
  }
}

// 16-byte asynchronous copy from global to shared memory (no register round trip); completed by
// cp_async_wait_all.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned dst = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;" ::: "memory");
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// ---- Record sort: the solve's predo ----------------------------------------------------------------------
//
// The keys are computed from the caller-order positions inside the passes (never stored in caller order), and
// each particle's record (x, y, m, original index) travels with its key through the passes, so the sorted
// particles come out of the last pass and no gather through the permutation (a random 32-byte sector per 8- or
// 4-byte read) follows. Digits of up to kRecMaxBits bits: two passes for the keys of depth <= 10 leaf grids.
// Per pass: an upsweep of per-tile digit counts, the per-digit scan, and a downsweep that loads the tile's
// items into registers first, ranks them stably (the warp-match ranking of radix_downsweep_kernel) and
// scatters key and record.

template <bool FROM_POS>
__global__ void __launch_bounds__(kSortThreads)
rec_upsweep_kernel(Geometry g, const float2* __restrict__ pos, const uint32_t* __restrict__ keys,
                   const int* __restrict__ d_n, int shift, int bits, uint32_t* __restrict__ counts, int max_tiles) {
  __shared__ uint32_t hist[1 << kRecMaxBits];
  const int n = *d_n;
  const int t = blockIdx.x;
  if (t >= num_tiles(n, kRecTile)) return;
  const int nd = 1 << bits;
  const uint32_t mask = (uint32_t)nd - 1u;
  for (int d = threadIdx.x; d < nd; d += kSortThreads) hist[d] = 0u;
  __syncthreads();
  const int base = t * kRecTile;
  const int end = min(base + kRecTile, n);
  for (int i = base + threadIdx.x; i < end; i += kSortThreads) {
    uint32_t key;
    if (FROM_POS) {
      const float2 p = pos[i];
      key = leaf_key(g, p.x, p.y);
    } else {
      key = keys[i];
    }
    atomicAdd(&hist[(key >> shift) & mask], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < nd; d += kSortThreads) counts[(size_t)d * max_tiles + t] = hist[d];
}

// Tiles of kRecTile items, kRecItems per thread, the keys (or positions) of the tile loaded before the ranking.
// The tile is then staged in shared memory in digit order and written out
// with consecutive threads on consecutive items, so that a digit's run of the tile leaves in one coalesced
// store. (Scattering from registers sends each warp store to ~32 different places, and a profile showed those
// scattered stores, not DRAM, bounding the kernel: about one memory transaction per item and array.)
// Dynamic shared memory: per-warp digit counters [kWarps][nd], the tile's digit starts [nd], the global offset of
// each digit's run [nd], staged keys [kRecTile] and records [kRecTile].
__host__ __device__ constexpr int rec_smem_bytes(int nd) {
  return (kSortThreads / 32) * nd * 4 + 2 * nd * 4 + kRecTile * 4 + kRecTile * 16;
}

#ifndef NBFMM_REC_MINB
#define NBFMM_REC_MINB 2  // resident CTAs per SM the downsweep is compiled for
#endif

template <bool FROM_POS, bool FINAL>
__global__ void __launch_bounds__(kSortThreads, NBFMM_REC_MINB)
rec_downsweep_kernel(Geometry g, const float2* __restrict__ pos, const float* __restrict__ w,
                     const uint32_t* __restrict__ keys_in, const float4* __restrict__ rec_in,
                     uint32_t* __restrict__ keys_out, float4* __restrict__ rec_out, uint32_t* __restrict__ perm_out,
                     const int* __restrict__ d_n, int shift, int bits, const uint32_t* __restrict__ counts,
                     const uint32_t* __restrict__ digit_total, int max_tiles) {
  constexpr int kWarps = kSortThreads / 32;
  extern __shared__ __align__(16) unsigned char rec_smem[];
  __shared__ uint32_t warp_sums[kWarps];
  const int n = *d_n;
  const int t = blockIdx.x;
  if (t >= num_tiles(n, kRecTile)) return;
  const int nd = 1 << bits;
  const uint32_t mask = (uint32_t)nd - 1u;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  uint32_t* warp_hist = reinterpret_cast<uint32_t*>(rec_smem);  // [kWarps][nd]
  uint32_t* local_start = warp_hist + kWarps * nd;               // [nd]
  uint32_t* delta = local_start + nd;                            // [nd]: global - local position of a digit's run
  uint32_t* skey = delta + nd;                                   // [kRecTile]
  float4* srec = reinterpret_cast<float4*>(skey + kRecTile);     // [kRecTile]

  // Warp `warp` owns items [warp*256, warp*256 + 256) of the tile, in kRecItems rounds of 32 consecutive items.
  const int tile0 = t * kRecTile;
  const int tile_n = min(kRecTile, n - tile0);
  const int base = tile0 + warp * (32 * kRecItems);
  // The first pass keeps each record in registers (it computes the key from the position); later passes load
  // the keys now and copy each record from global memory straight into its staged slot (cp.async) once its
  // place is known.
  uint32_t key[kRecItems];
  float4 rec[FROM_POS ? kRecItems : 1];
#pragma unroll
  for (int r = 0; r < kRecItems; ++r) {
    const int i = base + r * 32 + lane;
    if (FROM_POS) {
      float2 p = make_float2(0.0f, 0.0f);
      float m = 0.0f;
      if (i < n) {
        p = pos[i];
        m = w[i];
      }
      rec[FROM_POS ? r : 0] = make_float4(p.x, p.y, m, __int_as_float(i));
    } else {
      key[r] = (i < n) ? keys_in[i] : 0u;
    }
  }
  if (FROM_POS) {
#pragma unroll
    for (int r = 0; r < kRecItems; ++r) key[r] = leaf_key(g, rec[FROM_POS ? r : 0].x, rec[FROM_POS ? r : 0].y);
  }

  for (int d = lane; d < nd; d += 32) warp_hist[warp * nd + d] = 0u;
  __syncwarp();
  const unsigned lt_mask = (1u << lane) - 1u;
  uint32_t rank[kRecItems];
#pragma unroll
  for (int r = 0; r < kRecItems; ++r) {
    const bool valid = base + r * 32 + lane < n;
    const uint32_t digit = valid ? ((key[r] >> shift) & mask) : (uint32_t)nd;  // nd marks an empty slot
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const uint32_t before = valid ? warp_hist[warp * nd + digit] : 0u;
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) warp_hist[warp * nd + digit] = before + __popc(peers);
    __syncwarp();
    rank[r] = before + __popc(peers & lt_mask);
  }
  __syncthreads();
  // Per digit (4 per thread): the tile's count, the warps' exclusive prefix within the digit, the digit's start in
  // the staged tile (a block scan of the counts) and the offset from staged to global position: the digit's
  // global start (scan of the digit totals) plus this tile's offset within the digit (the scanned tile counts).
  {
    uint32_t cnt[4], gstart[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int d = threadIdx.x * 4 + k;
      uint32_t run = 0u;
      if (d < nd) {
#pragma unroll
        for (int wi = 0; wi < kWarps; ++wi) {
          const uint32_t c = warp_hist[wi * nd + d];
          warp_hist[wi * nd + d] = run;
          run += c;
        }
      }
      cnt[k] = run;
      gstart[k] = d < nd ? digit_total[d] : 0u;
    }
    block_exclusive_scan_4x256(gstart, warp_sums);
    block_exclusive_scan_4x256(cnt, warp_sums);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int d = threadIdx.x * 4 + k;
      if (d < nd) {
        local_start[d] = cnt[k];
        delta[d] = gstart[k] + counts[(size_t)d * max_tiles + t] - cnt[k];
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kRecItems; ++r) {
    const int i = base + r * 32 + lane;
    if (i < n) {
      const uint32_t d = (key[r] >> shift) & mask;
      const uint32_t l = local_start[d] + warp_hist[warp * nd + d] + rank[r];
      skey[l] = key[r];
      if (FROM_POS) srec[l] = rec[FROM_POS ? r : 0];
      else cp_async16(&srec[l], &rec_in[i]);
    }
  }
  if (!FROM_POS) cp_async_wait_all();
  __syncthreads();
  for (int l = threadIdx.x; l < tile_n; l += kSortThreads) {
    const uint32_t k = skey[l];
    const uint32_t dst = (uint32_t)l + delta[(k >> shift) & mask];
    const float4 q = srec[l];
    keys_out[dst] = k;
    rec_out[dst] = q;
    if (FINAL) perm_out[dst] = (uint32_t)__float_as_int(q.w);
  }
}

__global__ void head_kernel(const uint32_t* __restrict__ keys, const int* __restrict__ d_n, int num_cells,
                            int* __restrict__ head, int* __restrict__ d_n_alive) {
  const int n = *d_n;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c <= num_cells; c += gridDim.x * blockDim.x) {
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (keys[mid] < (uint32_t)c) lo = mid + 1; else hi = mid;
    }
    head[c] = lo;
    if (c == num_cells && d_n_alive) *d_n_alive = lo;
  }
}

__global__ void worklist_kernel(const int* __restrict__ head, int num_cells, int2* __restrict__ work,
                                int* __restrict__ d_work_count, int pair_tails, int passes_per_item,
                                const int* __restrict__ sys_cell_base, const int* __restrict__ sys_passes,
                                int num_systems, int* __restrict__ head_copy) {
  const int lane = threadIdx.x & 31;
  // Whole warps iterate together so that the warp-wide scan below sees every lane.
  for (int base = blockIdx.x * blockDim.x; base < num_cells; base += gridDim.x * blockDim.x) {
    const int c = base + threadIdx.x;
    int chunks = 0, tails = 0, ppi = passes_per_item, passes = 0;
    if (c < num_cells) {
      if (sys_passes) {  // the cell's system: the last whose first cell is <= c
        int lo = 0, hi = num_systems;
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (sys_cell_base[mid] <= c) lo = mid; else hi = mid;
        }
        ppi = sys_passes[lo];
      }
      const int nt = head[c + 1] - head[c];
      if (head_copy) {
        head_copy[c] = head[c];
        if (c == num_cells - 1) head_copy[num_cells] = head[num_cells];
      }
      const bool paired = pair_tails && tails_paired(head, c);
      passes = ((paired ? nt & ~31 : nt) + 31) >> 5;
      chunks = (passes + ppi - 1) / ppi;
      tails = (paired && !(c & 1)) ? 1 : 0;  // the even cell files the pair
    }
    const int items = chunks + tails;
    int incl = items;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += y;
    }
    int start = 0;
    if (lane == 31 && incl > 0) start = atomicAdd(d_work_count, incl);
    start = __shfl_sync(0xffffffffu, start, 31);
    int2* out = work + start + incl - items;
    for (int k = 0; k < chunks; ++k) out[k] = make_int2(c, work_item(k * ppi, min(ppi, passes - k * ppi)));
    if (tails) out[chunks] = make_int2(c, -1);
  }
}

__global__ void keys_from_head_kernel(const int* __restrict__ head, int num_cells, uint32_t* __restrict__ skey) {
  const int n = head[num_cells];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int lo = 0, hi = num_cells;  // first c with head[c] > i, minus one
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (head[mid] <= i) lo = mid + 1; else hi = mid;
    }
    skey[i] = (uint32_t)(lo - 1);
  }
}

int grid_for(int n, int threads, int cap) {
  long long g = ((long long)n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

}  // namespace

void launch_keys_from_positions(const Geometry& g, const float2* pos, const int* d_n, uint32_t* keys,
                                uint32_t* vals, int max_n, cudaStream_t stream) {
  keys_from_positions_kernel<<<grid_for(max_n, 256, 152 * 16), 256, 0, stream>>>(g, pos, d_n, keys, vals);
}

int launch_radix_sort(uint32_t* keys_a, uint32_t* vals_a, uint32_t* keys_b, uint32_t* vals_b,
                      uint32_t* counts, uint32_t* digit_total, const int* d_n, int max_n, int key_bits,
                      cudaStream_t stream) {
  if (key_bits <= 0) return 0;
  const int max_tiles = (max_n + kSortTile - 1) / kSortTile;
  const int passes = (key_bits + kRadixMaxBits - 1) / kRadixMaxBits;
  const int per_pass = (key_bits + passes - 1) / passes;
  uint32_t* kin = keys_a; uint32_t* vin = vals_a;
  uint32_t* kout = keys_b; uint32_t* vout = vals_b;
  int shift = 0;
  for (int p = 0; p < passes; ++p) {
    const int bits = (shift + per_pass <= key_bits) ? per_pass : key_bits - shift;
    radix_upsweep_kernel<<<max_tiles, kSortThreads, 0, stream>>>(kin, d_n, shift, bits, counts, max_tiles);
    radix_scan_kernel<<<1 << bits, kSortThreads, 0, stream>>>(counts, digit_total, d_n, max_tiles);
    radix_downsweep_kernel<<<max_tiles, kSortThreads, 0, stream>>>(kin, vin, kout, vout, d_n, shift, bits, counts,
                                                                   digit_total, max_tiles);
    shift += bits;
    uint32_t* tk = kin; kin = kout; kout = tk;
    uint32_t* tv = vin; vin = vout; vout = tv;
  }
  return (kin == keys_a) ? 0 : 1;  // which buffer pair holds the result
}

int record_sort_passes(int key_bits) { return key_bits <= kRecMaxBits ? 1 : (key_bits + kRecMaxBits - 1) / kRecMaxBits; }

void launch_sort_records(const Geometry& g, const float2* pos, const float* w, const int* d_n, int max_n,
                         int key_bits, float4* rec_final, float4* rec_tmp, uint32_t* key_final, uint32_t* key_tmp,
                         uint32_t* perm, uint32_t* counts, uint32_t* digit_total, cudaStream_t stream) {
  const int max_tiles = (max_n + kRecTile - 1) / kRecTile;
  const int passes = record_sort_passes(key_bits);
  // The kernels' dynamic shared-memory limit (a per-device function attribute; setting it is a host-side call).
  const int most = rec_smem_bytes(1 << kRecMaxBits);
  cudaFuncSetAttribute(rec_downsweep_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
  cudaFuncSetAttribute(rec_downsweep_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
  cudaFuncSetAttribute(rec_downsweep_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
  cudaFuncSetAttribute(rec_downsweep_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
  const int per_pass = (key_bits + passes - 1) / passes;
  const float4* rin = nullptr;
  const uint32_t* kin = nullptr;
  int shift = 0;
  for (int p = 0; p < passes; ++p) {
    const int bits = (shift + per_pass <= key_bits) ? per_pass : key_bits - shift;
    const bool final_pass = p == passes - 1;
    // Destinations alternate so that the last pass lands in the final buffers.
    const bool to_final = ((passes - 1 - p) & 1) == 0;
    float4* rout = to_final ? rec_final : rec_tmp;
    uint32_t* kout = to_final ? key_final : key_tmp;
    if (p == 0) {
      rec_upsweep_kernel<true><<<max_tiles, kSortThreads, 0, stream>>>(g, pos, nullptr, d_n, shift, bits, counts,
                                                                       max_tiles);
    } else {
      rec_upsweep_kernel<false><<<max_tiles, kSortThreads, 0, stream>>>(g, nullptr, kin, d_n, shift, bits, counts,
                                                                        max_tiles);
    }
    radix_scan_kernel<<<1 << bits, kSortThreads, 0, stream>>>(counts, digit_total, d_n, max_tiles, kRecTile);
    const int smem = rec_smem_bytes(1 << bits);
    if (p == 0 && final_pass) {
      rec_downsweep_kernel<true, true><<<max_tiles, kSortThreads, smem, stream>>>(
          g, pos, w, nullptr, nullptr, kout, rout, perm, d_n, shift, bits, counts, digit_total, max_tiles);
    } else if (p == 0) {
      rec_downsweep_kernel<true, false><<<max_tiles, kSortThreads, smem, stream>>>(
          g, pos, w, nullptr, nullptr, kout, rout, perm, d_n, shift, bits, counts, digit_total, max_tiles);
    } else if (final_pass) {
      rec_downsweep_kernel<false, true><<<max_tiles, kSortThreads, smem, stream>>>(
          g, nullptr, nullptr, kin, rin, kout, rout, perm, d_n, shift, bits, counts, digit_total, max_tiles);
    } else {
      rec_downsweep_kernel<false, false><<<max_tiles, kSortThreads, smem, stream>>>(
          g, nullptr, nullptr, kin, rin, kout, rout, perm, d_n, shift, bits, counts, digit_total, max_tiles);
    }
    rin = rout;
    kin = kout;
    shift += bits;
  }
}

void launch_head(const uint32_t* keys, const int* d_n, int num_cells, int* head, int* d_n_alive,
                 cudaStream_t stream) {
  head_kernel<<<grid_for(num_cells + 1, 256, 152 * 16), 256, 0, stream>>>(keys, d_n, num_cells, head, d_n_alive);
}

void launch_worklist(const int* head, int num_cells, int2* work, int* d_work_count, bool pair_tails,
                     cudaStream_t stream, int passes_per_item, const int* sys_cell_base, const int* sys_passes,
                     int num_systems, int* head_copy) {
  cudaMemsetAsync(d_work_count, 0, sizeof(int), stream);
  worklist_kernel<<<grid_for(num_cells, 256, 152 * 8), 256, 0, stream>>>(
      head, num_cells, work, d_work_count, pair_tails ? 1 : 0, passes_per_item, sys_cell_base, sys_passes,
      num_systems, head_copy);
}

void launch_keys_from_head(const int* head, int num_cells, uint32_t* skey, cudaStream_t stream) {
  keys_from_head_kernel<<<152 * 8, 256, 0, stream>>>(head, num_cells, skey);
}

}  // namespace nbfmm_gb300
