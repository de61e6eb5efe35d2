// tree.cu -- cell stages of the GB300 engine: gather + P2M, M2M, M2L (+ L2L), and the stage-alone L2L, L2P
// and postdo used by the stage entry points.
//
// Reference stages replaced (source/nbfmm/core/solver/):
//   permuteInputVector  predo.cu:86-100    the record sort (sort.cu) carries x, y, m through its passes
//   p2m                 p2m.cu:24-110      per-cell sums by one warp in sorted order, no reduce_by_key, no host sync
//   m2m                 m2m.cu:22-74       one thread per parent cell, compact per-level layout
//   m2l                 m2l.cu:24-81       16x16 target tile per CTA with its 20x20 source halo in shared memory
//   l2l                 l2l.cu:21-56       fused into M2L on the way down (child = m2l + parent)
//   l2p                 l2p.cu:23-48       stage-alone here; fused into the P2P epilogue on the solve path
//   permuteOutputVector postdo.cu:22-45    stage-alone here; fused into the P2P epilogue on the solve path
// The cell arithmetic uses correctly rounded operations without fused multiply-add, in the reference's
// order, so cell values round like the reference compiled for a CPU.
#include <algorithm>

#include "engine.cuh"

namespace nbfmm_gb300 {

namespace {

constexpr int kCellWarps = 8;  // warps per CTA of the one-warp-per-cell kernels

__global__ void p2m_kernel(int num_cells, const int* __restrict__ head, const float4* __restrict__ sorted4,
                           float4* __restrict__ cell0) {
  __shared__ float4 sums[kCellWarps][32];
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < num_cells; c += nwarps) {
    const int h0 = head[c], h1 = head[c + 1];
    float acc = 0.0f;
    for (int base = h0; base < h1; base += 32) {
      const int i = base + lane;
      const float4 q = (i < h1) ? sorted4[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      cell_sums_add_chunk(acc, sums[threadIdx.x >> 5], q.x, q.y, q.z, min(32, h1 - base), lane);
    }
    float sx, sy, sw;
    cell_sums_get(acc, sx, sy, sw);
    if (lane == 0) cell0[c] = centre_of_mass(sx, sy, sw, h1 > h0);
  }
}

// m2m.cu:40-53 for parent k of a level: children (x,y), (x+1,y), (x,y+1), (x+1,y+1) summed left to right; zero
// mass -> (0,0).
__device__ __forceinline__ void m2m_parent(float4* __restrict__ cell4, int off_c, int dim_c, int off_p, int dim_p,
                                           int k) {
  const int px = k % dim_p, py = k / dim_p;
  const int c0 = off_c + (2 * py) * dim_c + 2 * px;
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

__global__ void m2m_kernel(float4* __restrict__ cell4, int off_c, int dim_c, int off_p, int dim_p) {
  const int total = dim_p * dim_p;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
    m2m_parent(cell4, off_c, dim_c, off_p, dim_p, k);
  }
}

// Small levels do not fill the GPU: one launch per level cost 3-14 us, mostly launch and drain, or one thread's
// long serial chain of correctly rounded evaluations. kTopDim: the M2M levels of at most this many cells per side
// run in one launch. kWideDim: the M2L levels of at most this many cells per side evaluate each target's sources
// in parallel across a warp.
constexpr int kTopDim = 64;
constexpr int kWideDim = 128;

// M2M of every level from l0 to the top in one CTA, level after level (__syncthreads between levels).
__global__ void __launch_bounds__(256) m2m_top_kernel(float4* __restrict__ cell4, Levels lv, int l0) {
  for (int l = l0 > 1 ? l0 : 1; l < lv.count; ++l) {
    const int total = lv.dim[l] * lv.dim[l];
    for (int k = threadIdx.x; k < total; k += blockDim.x) {
      m2m_parent(cell4, lv.offset[l - 1], lv.dim[l - 1], lv.offset[l], lv.dim[l], k);
    }
    __syncthreads();
  }
}

// M2L (+ L2L) of a small level with one warp per target cell: lane j evaluates candidate source j of the 6 x 6
// children of the parent's neighbourhood (j and j + 32 for the first four lanes), the valid ones (inside the
// level, outside the target's 3 x 3) are staged in shared memory in the reference's order (y outer, x inner,
// m2l.cu:46-58), and lane 0 adds them one by one, then the parent's effect (l2l.cu:33-35): the arithmetic and
// order of m2l_tile, with the evaluations in parallel instead of one thread's serial chain.
constexpr int kWideWarps = 8;

__global__ void __launch_bounds__(kWideWarps * 32)
m2l_wide_kernel(const float4* __restrict__ cell4, float2* __restrict__ ceff, int off, int dim, int off_parent,
                int dim_parent, int add_parent, float eps) {
  __shared__ float2 terms[kWideWarps][36];
  __shared__ int valid[kWideWarps][36];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c = blockIdx.x * kWideWarps + warp;
  if (c >= dim * dim) return;  // warp-uniform
  const int tx = c % dim, ty = c / dim;
  const float4 t = cell4[off + c];
  const float2 tp = make_float2(t.x, t.y);
  const int px = tx & ~1, py = ty & ~1;
  for (int j = lane; j < 36; j += 32) {
    const int x = px - 2 + j % 6, y = py - 2 + j / 6;
    const bool ok = x >= 0 && x < dim && y >= 0 && y < dim && (abs(x - tx) > 1 || abs(y - ty) > 1);
    valid[warp][j] = ok;
    if (ok) {
      const float4 sc = cell4[off + y * dim + x];
      terms[warp][j] = kernel_exact(tp, make_float2(sc.x, sc.y), sc.z, eps);
    }
  }
  __syncwarp();
  if (lane == 0) {
    float ex = 0.0f, ey = 0.0f;
    for (int j = 0; j < 36; ++j) {
      if (valid[warp][j]) {
        ex = __fadd_rn(ex, terms[warp][j].x);
        ey = __fadd_rn(ey, terms[warp][j].y);
      }
    }
    if (add_parent) {
      const float2 p = ceff[off_parent + (ty >> 1) * dim_parent + (tx >> 1)];
      ex = __fadd_rn(ex, p.x);
      ey = __fadd_rn(ey, p.y);
    }
    ceff[off + c] = make_float2(ex, ey);
  }
}

// m2l.cu:24-60 for one level. Each CTA owns a 16x16 tile of target cells (tile origin even, so the
// children of the parents' neighbours lie in the 20x20 halo around it). With add_parent the parent's
// effect is added afterwards (l2l.cu:33-35): child = m2l + parent.
__global__ void __launch_bounds__(kM2LTile * kM2LTile)
m2l_kernel(const float4* __restrict__ cell4, float2* __restrict__ ceff, int off, int dim, int off_parent,
           int dim_parent, int add_parent, float eps) {
  __shared__ float4 halo[kM2LHalo][kM2LHalo];
  m2l_tile(halo, cell4 + off, ceff + off, dim, ceff + off_parent, dim_parent, add_parent,
           blockIdx.x * kM2LTile, blockIdx.y * kM2LTile, eps);
}

__global__ void l2l_kernel(float2* __restrict__ ceff, int off, int dim, int off_parent, int dim_parent) {
  const int total = dim * dim;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
    const int x = k % dim, y = k / dim;
    const float2 p = ceff[off_parent + (y >> 1) * dim_parent + (x >> 1)];
    float2 e = ceff[off + k];
    e.x = __fadd_rn(e.x, p.x);
    e.y = __fadd_rn(e.y, p.y);
    ceff[off + k] = e;
  }
}

__global__ void l2p_kernel(const int* __restrict__ d_n, const uint32_t* __restrict__ skey,
                           const float2* __restrict__ ceff0, float2* __restrict__ seff) {
  const int n = *d_n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 c = ceff0[skey[i]];
    float2 e = seff[i];
    e.x = __fadd_rn(e.x, c.x);
    e.y = __fadd_rn(e.y, c.y);
    seff[i] = e;
  }
}

// eff_origin[perm[i]] = seff[i] for kPostdoItems items per thread, all loaded before the scattered stores (a
// grid-stride loop with one load-store round trip per iteration was latency-bound). The stores are 8-byte
// pieces of 32-byte sectors at random places; when the output is larger than the L2 can hold, its sectors leave
// the L2 before their four pieces have arrived and go to DRAM several times over. So the original indices are
// taken in windows of at most kPostdoWindowBytes of output, one launch each, every launch reading all of perm
// and seff with evict-first loads and storing only into its window, whose sectors fill up in the L2.
constexpr int kPostdoItems = 4;
constexpr long long kPostdoWindowBytes = 64ll << 20;

__global__ void postdo_kernel(const int* __restrict__ d_n, const uint32_t* __restrict__ perm,
                              const float2* __restrict__ seff, float2* __restrict__ eff_origin, uint32_t lo,
                              uint32_t hi) {
  const int n = *d_n;
  const int base = blockIdx.x * blockDim.x * kPostdoItems + threadIdx.x;
  uint32_t p[kPostdoItems];
  float2 e[kPostdoItems];
#pragma unroll
  for (int k = 0; k < kPostdoItems; ++k) {
    const int i = base + k * blockDim.x;
    p[k] = 0xffffffffu;
    if (i < n) {
      p[k] = __ldcs(perm + i);
      e[k] = __ldcs(seff + i);
    }
  }
#pragma unroll
  for (int k = 0; k < kPostdoItems; ++k) {
    if (p[k] >= lo && p[k] < hi) eff_origin[p[k]] = e[k];
  }
}

int grid_for(long long n, int threads, int cap) {
  long long g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

}  // namespace

void launch_p2m(const Geometry& g, const int* head, const float4* sorted4, float4* cell0, cudaStream_t stream) {
  const int cells = g.base_dim * g.base_dim;
  p2m_kernel<<<grid_for((long long)cells * 32, kCellWarps * 32, 152 * 16), kCellWarps * 32, 0, stream>>>(
      cells, head, sorted4, cell0);
}

void launch_m2m(const Levels& lv, float4* cell4, cudaStream_t stream) {
  for (int l = 1; l < lv.count; ++l) {
    const int total = lv.dim[l] * lv.dim[l];
    m2m_kernel<<<grid_for(total, 256, 152 * 8), 256, 0, stream>>>(cell4, lv.offset[l - 1], lv.dim[l - 1],
                                                                  lv.offset[l], lv.dim[l]);
  }
}

void launch_m2l(const Levels& lv, const float4* cell4, float2* ceff, float eps, bool with_l2l, cudaStream_t stream) {
  for (int l = lv.count - 1; l >= 0; --l) {
    const int dim = lv.dim[l];
    const int has_parent = (with_l2l && l + 1 < lv.count) ? 1 : 0;
    const int lp = has_parent ? l + 1 : l;
    if (dim <= kWideDim) {
      m2l_wide_kernel<<<(dim * dim + kWideWarps - 1) / kWideWarps, kWideWarps * 32, 0, stream>>>(
          cell4, ceff, lv.offset[l], dim, lv.offset[lp], lv.dim[lp], has_parent, eps);
      continue;
    }
    const dim3 grid((dim + kM2LTile - 1) / kM2LTile, (dim + kM2LTile - 1) / kM2LTile);
    m2l_kernel<<<grid, dim3(kM2LTile, kM2LTile), 0, stream>>>(cell4, ceff, lv.offset[l], dim, lv.offset[lp],
                                                               lv.dim[lp], has_parent, eps);
  }
}

void launch_far_field(const Levels& lv, float4* cell4, float2* ceff, float eps, cudaStream_t stream) {
  int l0 = lv.count;  // first level of at most kTopDim cells per side
  for (int l = 0; l < lv.count; ++l) {
    if (lv.dim[l] <= kTopDim) {
      l0 = l;
      break;
    }
  }
  for (int l = 1; l < l0; ++l) {
    const int total = lv.dim[l] * lv.dim[l];
    m2m_kernel<<<grid_for(total, 256, 152 * 8), 256, 0, stream>>>(cell4, lv.offset[l - 1], lv.dim[l - 1],
                                                                  lv.offset[l], lv.dim[l]);
  }
  if (lv.count > 1 && l0 < lv.count) m2m_top_kernel<<<1, 256, 0, stream>>>(cell4, lv, l0);
  launch_m2l(lv, cell4, ceff, eps, true, stream);
}

void launch_l2l(const Levels& lv, float2* ceff, cudaStream_t stream) {
  for (int l = lv.count - 2; l >= 0; --l) {
    const int total = lv.dim[l] * lv.dim[l];
    l2l_kernel<<<grid_for(total, 256, 152 * 8), 256, 0, stream>>>(ceff, lv.offset[l], lv.dim[l], lv.offset[l + 1],
                                                                  lv.dim[l + 1]);
  }
}

void launch_l2p(const int* d_n, const uint32_t* skey, const float2* ceff0, float2* seff, int max_n, cudaStream_t stream) {
  l2p_kernel<<<grid_for(max_n, 256, 152 * 16), 256, 0, stream>>>(d_n, skey, ceff0, seff);
}

void launch_postdo(const int* d_n, const uint32_t* perm, const float2* seff, float2* eff_origin, int max_n,
                   cudaStream_t stream) {
  const long long windows = std::max(1ll, ((long long)max_n * 8 + kPostdoWindowBytes - 1) / kPostdoWindowBytes);
  const long long span = ((long long)max_n + windows - 1) / windows;
  for (long long w = 0; w < windows; ++w) {
    const uint32_t lo = (uint32_t)(w * span), hi = (uint32_t)std::min((long long)max_n, (w + 1) * span);
    postdo_kernel<<<grid_for((long long)max_n, 256 * kPostdoItems, 1 << 30), 256, 0, stream>>>(d_n, perm, seff,
                                                                                              eff_origin, lo, hi);
  }
}

}  // namespace nbfmm_gb300
