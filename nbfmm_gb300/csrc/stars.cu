// stars.cu -- the time-stepping path of the GB300 engine: Stars::update (solve + Verlet + prune) without
// host synchronisation.
//
// Reference path (source/nbfmm/display/stars/): update.cu:47-55 solves, applies the Stormer-Verlet update
// (update.cu:26-42) in the caller's order, then prune.cu:28-62 stable-partitions the stars still inside the
// limits to the front and reads the new count back to the host (thrust::find, prune.cu:61).
//
// Here the stars live in an internal state kept in the previous step's cell order: state4 = (x, y, m,
// original index), state_prev = previous positions. A step sorts the state by leaf cell, gathers it, builds
// the tree and runs P2P with the L2P + Verlet epilogue, which writes the new state in the new cell order.
// Pruning is folded into the next step's key pass: a star outside the limits gets the key B*B, sorts behind
// every live star and drops out (head[B*B] is the new count), and its final state is filed under its
// original index together with its death step. The state of the public arrays (survivors in their previous
// relative order, then the pruned stars, most recent first) is restored once at the end of the call.
#include "engine.cuh"
#include "stars.cuh"

namespace nbfmm_gb300 {

namespace {

__global__ void import_kernel(StepCounters sc, const float2* __restrict__ cur, const float2* __restrict__ prev,
                              const float* __restrict__ w, float4* __restrict__ state4,
                              float2* __restrict__ state_prev) {
  const int n = *sc.num_star;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 c = cur[i];
    state4[i] = make_float4(c.x, c.y, w[i], __int_as_float(i));
    state_prev[i] = prev[i];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *sc.n_cur = n;
    *sc.n_import = n;
    *sc.step = 1;
    *sc.prune = 0;
  }
}

__global__ void keys_from_state_kernel(Geometry g, StepCounters sc, const float4* __restrict__ state4,
                                       const float2* __restrict__ state_prev, uint32_t dead_key,
                                       uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                       float4* __restrict__ grave) {
  const int n = *sc.n_cur;
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

__global__ void gather_state_p2m_kernel(int num_cells, const int* __restrict__ head, const uint32_t* __restrict__ perm,
                                        const float4* __restrict__ state4, const float2* __restrict__ state_prev,
                                        float4* __restrict__ sorted4, float2* __restrict__ sprev,
                                        float4* __restrict__ cell0) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < num_cells; c += nwarps) {
    const int h0 = head[c], h1 = head[c + 1];
    float sx = 0.0f, sy = 0.0f, sw = 0.0f;
    for (int base = h0; base < h1; base += 32) {
      const int i = base + lane;
      float4 q = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (i < h1) {
        const uint32_t p = perm[i];
        q = state4[p];
        sorted4[i] = q;
        sprev[i] = state_prev[p];
      }
      cell_sums_add_chunk(sx, sy, sw, q.x, q.y, q.z, min(32, h1 - base));
    }
    if (lane == 0) cell0[c] = centre_of_mass(sx, sy, sw, h1 > h0);
  }
}

__global__ void finish_step_kernel(StepCounters sc) {
  *sc.n_cur = *sc.n_alive;
  *sc.step += 1;
  *sc.prune = 1;
}

// The last prune of the call (prune.cu:40-41 on the final positions), and every star's final state filed by
// original index: fate 0 = alive, fate 1 = pruned by the last step.
__global__ void export_fate_kernel(Geometry g, StepCounters sc, const float4* __restrict__ state4,
                                   const float2* __restrict__ state_prev, float4* __restrict__ grave) {
  const int n = *sc.n_cur;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = state4[i];
    file_grave(grave, __float_as_int(p.w), p.x, p.y, state_prev[i], p.z, outside(g, p.x, p.y) ? 1 : 0);
  }
}

__global__ void fate_keys_kernel(StepCounters sc, const float4* __restrict__ grave, uint32_t* __restrict__ keys,
                                 uint32_t* __restrict__ vals) {
  const int n = *sc.n_import;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    keys[i] = (uint32_t)grave_fate(grave, i);
    vals[i] = (uint32_t)i;
  }
}

__global__ void export_gather_kernel(StepCounters sc, const uint32_t* __restrict__ order,
                                     const float4* __restrict__ grave, float2* __restrict__ cur,
                                     float2* __restrict__ prev, float* __restrict__ w) {
  const int n = *sc.n_import;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t o = order[i];
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

void launch_gather_state_p2m(const Geometry& g, const int* head, const uint32_t* perm, const float4* state4,
                             const float2* state_prev, float4* sorted4, float2* sprev, float4* cell0,
                             cudaStream_t stream) {
  const int cells = g.base_dim * g.base_dim;
  gather_state_p2m_kernel<<<grid_for((long long)cells * 32, 256, 152 * 16), 256, 0, stream>>>(
      cells, head, perm, state4, state_prev, sorted4, sprev, cell0);
}

void launch_gather_state_p2m_cells(const int* head, int num_cells, const uint32_t* perm, const float4* state4,
                                   const float2* state_prev, float4* sorted4, float2* sprev, float4* cell0,
                                   cudaStream_t stream) {
  gather_state_p2m_kernel<<<grid_for((long long)num_cells * 32, 256, 152 * 16), 256, 0, stream>>>(
      num_cells, head, perm, state4, state_prev, sorted4, sprev, cell0);
}

void launch_finish_step(const StepCounters& sc, cudaStream_t stream) { finish_step_kernel<<<1, 1, 0, stream>>>(sc); }

void launch_export_fate(const Geometry& g, const StepCounters& sc, const float4* state4, const float2* state_prev,
                        float4* grave, int max_n, cudaStream_t stream) {
  export_fate_kernel<<<grid_for(max_n, 256, 152 * 16), 256, 0, stream>>>(g, sc, state4, state_prev, grave);
}

void launch_fate_keys(const StepCounters& sc, const float4* grave, uint32_t* keys, uint32_t* vals, int max_n,
                      cudaStream_t stream) {
  fate_keys_kernel<<<grid_for(max_n, 256, 152 * 16), 256, 0, stream>>>(sc, grave, keys, vals);
}

void launch_export_gather(const StepCounters& sc, const uint32_t* order, const float4* grave, float2* cur,
                          float2* prev, float* w, int max_n, cudaStream_t stream) {
  export_gather_kernel<<<grid_for(max_n, 256, 152 * 16), 256, 0, stream>>>(sc, order, grave, cur, prev, w);
}

void launch_prune_keys(const Geometry& g, const StepCounters& sc, const float2* cur, const float2* prev,
                       const float* w, uint32_t* keys, uint32_t* vals, float4* grave, int max_n, cudaStream_t stream) {
  prune_keys_kernel<<<grid_for(max_n, 256, 152 * 16), 256, 0, stream>>>(g, sc, cur, prev, w, keys, vals, grave);
}

}  // namespace nbfmm_gb300
