// adjoint.cu -- reverse mode of the approximate method itself, through a Stormer-Verlet trajectory.
//
// No counterpart in the reference. The forward trajectory is the solve of solve.cu:11-27 followed by the
// update of update.cu:39-40 (x' = 2x - x_prev + a tau^2, tau = tick * sqrt(G)); stars are not pruned inside an
// adjoint trajectory. The loss is L = 0.5 sum_i m_i |x_i(T) - x*_i|^2. With lambda_t = dL/dx_t,
//   lambda_T = m (x_T - x*),  lambda_t = 2 lambda_{t+1} + J(x_t)^T (tau^2 lambda_{t+1}) - lambda_{t+2},
//   dL/dx_0 = lambda_0 - lambda_1,  dL/dv_0 = tau lambda_1  (x_{-1} = x_0 - v_0 tau),
//   dL/dm = 0.5 |x_T - x*|^2 + sum_t (dA/dm)^T (tau^2 lambda_{t+1}),
// where J and dA/dm are the derivatives of the engine's own effects A(x, m) with the cell assignment held
// fixed (it is piecewise constant in x). The vector-Jacobian product of one solve, for an effect adjoint mu:
//   near field (P2P, p2p.cu:30-69), with d = x_j - x_i, r = |d|, D = r^3 + eps, M(d) = I/D - 3 r d d^T / D^2:
//     g_x[i] += sum_j M(d)(m_i mu_j - m_j mu_i),   g_m[i] += -sum_j mu_j . d / D      (j over the 3x3 cells)
//   far field: Lambda(C) = sum of mu over the particles below cell C (the transpose of L2L and L2P); the
//     transposed M2L (m2l.cu:46-58) over the same, symmetric interaction lists gives per cell
//     G_X(C) = sum_S M(X_S - X_C)(M_C Lambda(S) - M_S Lambda(C)),  G_M(C) = -sum_S Lambda(S).(X_S - X_C)/D;
//     the transposed M2M (m2m.cu:40-53) carries G from parents to children through the centres of mass,
//     G_X(c) += (M_c/M_P) G_X(P),  G_M(c) += G_M(P) + G_X(P).(X_c - X_P)/M_P, and the transposed P2M hands the
//     leaf G to the particles: g_x[i] += (m_i/M_c) G_X(c), g_m[i] += G_M(c) + G_X(c).(x_i - X_c)/M_c.
// Checkpoints (x_t, x_{t-1}) are kept every k steps; the backward pass recomputes each segment forward from its
// checkpoint and then walks it backwards.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <vector>

#include "solver.cuh"

namespace {

constexpr int kAdjWarps = 4;

__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// smu[i] = scale * lam[perm[i]] in sorted order, and the leaf sums Lambda(c) of smu (sorted order, sequential).
__global__ void adj_gather_kernel(int num_cells, const int* __restrict__ head, const uint32_t* __restrict__ perm,
                                  const float2* __restrict__ lam, float scale, float2* __restrict__ smu,
                                  float2* __restrict__ cell_lam0) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < num_cells; c += nwarps) {
    const int h0 = head[c], h1 = head[c + 1];
    float sx = 0.0f, sy = 0.0f;
    for (int base = h0; base < h1; base += 32) {
      const int i = base + lane;
      float2 v = make_float2(0.0f, 0.0f);
      if (i < h1) {
        const float2 l = lam[perm[i]];
        v = make_float2(scale * l.x, scale * l.y);
        smu[i] = v;
      }
      const int count = min(32, h1 - base);
      for (int j = 0; j < count; ++j) {
        sx += __shfl_sync(0xffffffffu, v.x, j);
        sy += __shfl_sync(0xffffffffu, v.y, j);
      }
    }
    if (lane == 0) cell_lam0[c] = make_float2(sx, sy);
  }
}

// Lambda of a parent = sum of its four children (the transpose of L2L, l2l.cu:33-35).
__global__ void adj_up_kernel(float2* __restrict__ cell_lam, int off_c, int dim_c, int off_p, int dim_p) {
  const int total = dim_p * dim_p;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
    const int px = k % dim_p, py = k / dim_p;
    const int c0 = off_c + (2 * py) * dim_c + 2 * px;
    const float2 a = cell_lam[c0], b = cell_lam[c0 + 1], c = cell_lam[c0 + dim_c], d = cell_lam[c0 + dim_c + 1];
    cell_lam[off_p + k] = make_float2(((a.x + b.x) + c.x) + d.x, ((a.y + b.y) + c.y) + d.y);
  }
}

// Transposed M2L of one level (same tiles and halo as m2l_tile): G = (G_X.x, G_X.y, G_M, 0) per cell.
__global__ void __launch_bounds__(kM2LTile * kM2LTile)
adj_m2l_kernel(const float4* __restrict__ cell4, const float2* __restrict__ cell_lam, float4* __restrict__ cell_g,
               int off, int dim, float eps) {
  __shared__ float4 hx[kM2LHalo][kM2LHalo];
  __shared__ float2 hl[kM2LHalo][kM2LHalo];
  const int x0 = blockIdx.x * kM2LTile, y0 = blockIdx.y * kM2LTile;
  const int tid = threadIdx.y * kM2LTile + threadIdx.x;
  for (int k = tid; k < kM2LHalo * kM2LHalo; k += kM2LTile * kM2LTile) {
    const int ix = k % kM2LHalo, iy = k / kM2LHalo;
    const int gx = x0 - 2 + ix, gy = y0 - 2 + iy;
    const bool in = gx >= 0 && gx < dim && gy >= 0 && gy < dim;
    hx[iy][ix] = in ? cell4[off + gy * dim + gx] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    hl[iy][ix] = in ? cell_lam[off + gy * dim + gx] : make_float2(0.0f, 0.0f);
  }
  __syncthreads();
  const int tx = x0 + threadIdx.x, ty = y0 + threadIdx.y;
  if (tx >= dim || ty >= dim) return;
  const float4 C = hx[ty - y0 + 2][tx - x0 + 2];
  const float2 LC = hl[ty - y0 + 2][tx - x0 + 2];
  const int px = tx & ~1, py = ty & ~1;
  float gx = 0.0f, gy = 0.0f, gm = 0.0f;
  for (int y = py - 2; y < py + 4; ++y) {
    if (y < 0 || y >= dim) continue;
    for (int x = px - 2; x < px + 4; ++x) {
      if (x < 0 || x >= dim) continue;
      if (abs(x - tx) > 1 || abs(y - ty) > 1) {
        const float4 S = hx[y - y0 + 2][x - x0 + 2];
        const float2 LS = hl[y - y0 + 2][x - x0 + 2];
        const float dx = S.x - C.x, dy = S.y - C.y;
        const float r2 = dx * dx + dy * dy;
        const float r = sqrtf(r2);
        const float inv = 1.0f / (r2 * r + eps);
        const float ux = C.z * LS.x - S.z * LC.x;
        const float uy = C.z * LS.y - S.z * LC.y;
        const float k3 = 3.0f * r * inv * inv * (dx * ux + dy * uy);
        gx += ux * inv - k3 * dx;
        gy += uy * inv - k3 * dy;
        gm -= (LS.x * dx + LS.y * dy) * inv;
      }
    }
  }
  cell_g[off + ty * dim + tx] = make_float4(gx, gy, gm, 0.0f);
}

// The transposed M2L of every level with at most kAdjWideDim cells per side, in one launch: levels do not depend
// on one another here (G of a level comes from that level's centres and Lambda). One warp per cell: lane j takes
// candidate j of the 6 x 6 children of the parent's neighbourhood (j and j + 32 for the first four lanes), and the
// contributions are summed by a fixed butterfly over the lanes. Cells [first_cell, lv.total) of the compact
// layout.
constexpr int kAdjWideDim = 128;

__device__ __forceinline__ void adj_m2l_pair(const float4 C, const float2 LC, const float4 S, const float2 LS,
                                             float eps, float& gx, float& gy, float& gm) {
  const float dx = S.x - C.x, dy = S.y - C.y;
  const float r2 = dx * dx + dy * dy;
  const float r = sqrtf(r2);
  const float inv = 1.0f / (r2 * r + eps);
  const float ux = C.z * LS.x - S.z * LC.x;
  const float uy = C.z * LS.y - S.z * LC.y;
  const float k3 = 3.0f * r * inv * inv * (dx * ux + dy * uy);
  gx += ux * inv - k3 * dx;
  gy += uy * inv - k3 * dy;
  gm -= (LS.x * dx + LS.y * dy) * inv;
}

__global__ void __launch_bounds__(256) adj_m2l_wide_kernel(const float4* __restrict__ cell4,
                                                           const float2* __restrict__ cell_lam,
                                                           float4* __restrict__ cell_g, Levels lv, int first_cell,
                                                           float eps) {
  const int lane = threadIdx.x & 31;
  const int c = first_cell + (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (c >= lv.total) return;  // warp-uniform
  int l = lv.count - 1;
  while (l > 0 && lv.offset[l] > c) --l;
  const int dim = lv.dim[l], off = lv.offset[l];
  const int k = c - off, tx = k % dim, ty = k / dim;
  const float4 C = cell4[c];
  const float2 LC = cell_lam[c];
  const int px = tx & ~1, py = ty & ~1;
  float gx = 0.0f, gy = 0.0f, gm = 0.0f;
  for (int j = lane; j < 36; j += 32) {
    const int x = px - 2 + j % 6, y = py - 2 + j / 6;
    if (x >= 0 && x < dim && y >= 0 && y < dim && (abs(x - tx) > 1 || abs(y - ty) > 1)) {
      adj_m2l_pair(C, LC, cell4[off + y * dim + x], cell_lam[off + y * dim + x], eps, gx, gy, gm);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    gx += __shfl_xor_sync(0xffffffffu, gx, o);
    gy += __shfl_xor_sync(0xffffffffu, gy, o);
    gm += __shfl_xor_sync(0xffffffffu, gm, o);
  }
  if (lane == 0) cell_g[c] = make_float4(gx, gy, gm, 0.0f);
}

// Lambda up (adj_up_kernel) for levels l_from..top, then nothing else: one CTA, level after level.
__global__ void __launch_bounds__(256) adj_up_top_kernel(float2* __restrict__ cell_lam, Levels lv, int l_from) {
  for (int l = l_from; l < lv.count; ++l) {
    const int dim_p = lv.dim[l], dim_c = lv.dim[l - 1], off_c = lv.offset[l - 1], off_p = lv.offset[l];
    for (int k = threadIdx.x; k < dim_p * dim_p; k += blockDim.x) {
      const int px = k % dim_p, py = k / dim_p;
      const int c0 = off_c + (2 * py) * dim_c + 2 * px;
      const float2 a = cell_lam[c0], b = cell_lam[c0 + 1], c = cell_lam[c0 + dim_c], d = cell_lam[c0 + dim_c + 1];
      cell_lam[off_p + k] = make_float2(((a.x + b.x) + c.x) + d.x, ((a.y + b.y) + c.y) + d.y);
    }
    __syncthreads();
  }
}

// Transposed M2M: a parent's G flows to its children through the centre of mass (m2m.cu:40-53).
__device__ __forceinline__ void adj_down_child(const float4* __restrict__ cell4, float4* __restrict__ cell_g,
                                               int off_c, int dim_c, int off_p, int dim_p, int k) {
  const int x = k % dim_c, y = k / dim_c;
  const int p = off_p + (y >> 1) * dim_p + (x >> 1);
  const float4 P = cell4[p];
  if (P.z == 0.0f) return;  // an empty parent has a fixed (0, 0) centre: nothing flows
  const float4 GP = cell_g[p];
  const float4 ch = cell4[off_c + k];
  float4 g = cell_g[off_c + k];
  const float f = ch.z / P.z;
  g.x += f * GP.x;
  g.y += f * GP.y;
  g.z += GP.z + (GP.x * (ch.x - P.x) + GP.y * (ch.y - P.y)) / P.z;
  cell_g[off_c + k] = g;
}

__global__ void adj_down_kernel(const float4* __restrict__ cell4, float4* __restrict__ cell_g, int off_c, int dim_c,
                                int off_p, int dim_p) {
  const int total = dim_c * dim_c;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
    adj_down_child(cell4, cell_g, off_c, dim_c, off_p, dim_p, k);
  }
}

// adj_down for parent levels top..l_to (children down to level l_to - 1) in one CTA, level after level.
__global__ void __launch_bounds__(256) adj_down_top_kernel(const float4* __restrict__ cell4,
                                                           float4* __restrict__ cell_g, Levels lv, int l_to) {
  for (int l = lv.count - 1; l >= l_to; --l) {
    const int dim_c = lv.dim[l - 1];
    for (int k = threadIdx.x; k < dim_c * dim_c; k += blockDim.x) {
      adj_down_child(cell4, cell_g, lv.offset[l - 1], dim_c, lv.offset[l], lv.dim[l], k);
    }
    __syncthreads();
  }
}

struct AdjP2PArgs {
  const float4* sorted4;  // x, y, m, original index
  const float2* smu;      // effect adjoint, sorted order
  const int* head;
  const int2* work;
  const int* d_work_count;
  int* d_work_next;
  int base_dim;
  float eps;
  const float4* cell0;    // leaf centres of mass (null without far field)
  const float4* g0;       // leaf G (null without far field)
  float2* gx_out;         // original order
  float* gm_out;          // original order
};

typedef unsigned long long f2x;  // two packed floats

__device__ __forceinline__ f2x pk(float lo, float hi) {
  f2x r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}

__device__ __forceinline__ void up(f2x v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

__device__ __forceinline__ f2x sub2(f2x a, f2x b) {
  f2x r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}

__device__ __forceinline__ f2x mul2(f2x a, f2x b) {
  f2x r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}

__device__ __forceinline__ f2x fma2(f2x a, f2x b, f2x c) {
  f2x r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

// A warp's 32-source batch, packed for f32x2: (x, x, y, y), (mu_x, mu_x, mu_y, mu_y), (-m, -m).
struct AdjSlice {
  ulonglong2 xy[32];
  ulonglong2 mu[32];
  f2x mneg[32];
};

// Per pair (d = x_j - x_i, D = r^3 + eps): u = m_i mu_j - m_j mu_i, g_x += u/D - 3 r (d.u) d / D^2,
// s_m += (mu_j . d) / D (g_m = -s_m). Both targets of a packed pair share the source.
struct AdjTargets2 {
  f2x x, y, m, mux, muy;
  f2x gx, gy, sm;
};

__device__ __forceinline__ void adj_pair2(AdjTargets2& t, f2x sx, f2x sy, f2x mjx, f2x mjy, f2x mjneg, f2x eps2,
                                          f2x neg3) {
  const f2x dx = sub2(sx, t.x);
  const f2x dy = sub2(sy, t.y);
  const f2x r2 = fma2(dy, dy, mul2(dx, dx));
  float r2a, r2b;
  up(r2, r2a, r2b);
  const f2x r = pk(sqrt_approx(r2a), sqrt_approx(r2b));
  float da, db;
  up(fma2(r2, r, eps2), da, db);
  const f2x inv = pk(rcp_approx(da), rcp_approx(db));
  const f2x ux = fma2(t.m, mjx, mul2(mjneg, t.mux));
  const f2x uy = fma2(t.m, mjy, mul2(mjneg, t.muy));
  const f2x du = fma2(dy, uy, mul2(dx, ux));
  const f2x w = mul2(mul2(mul2(r, neg3), mul2(inv, inv)), du);
  t.gx = fma2(w, dx, fma2(ux, inv, t.gx));
  t.gy = fma2(w, dy, fma2(uy, inv, t.gy));
  t.sm = fma2(fma2(dy, mjy, mul2(dx, mjx)), inv, t.sm);
}

struct AdjTarget1 {
  float x, y, m, mux, muy;
  float gx, gy, sm;
};

__device__ __forceinline__ void adj_pair1(AdjTarget1& t, float sx, float sy, float mjx, float mjy, float mjneg,
                                          float eps) {
  const float dx = sx - t.x, dy = sy - t.y;
  const float r2 = fmaf(dy, dy, dx * dx);
  const float r = sqrt_approx(r2);
  const float inv = rcp_approx(fmaf(r2, r, eps));
  const float ux = fmaf(t.m, mjx, mjneg * t.mux);
  const float uy = fmaf(t.m, mjy, mjneg * t.muy);
  const float w = -3.0f * r * inv * inv * fmaf(dy, uy, dx * ux);
  t.gx = fmaf(w, dx, fmaf(ux, inv, t.gx));
  t.gy = fmaf(w, dy, fmaf(uy, inv, t.gy));
  t.sm = fmaf(fmaf(dy, mjy, dx * mjx), inv, t.sm);
}

struct AdjRanges {
  int s0, l0, s1, l1, s2, l2;
  __device__ __forceinline__ int total() const { return l0 + l1 + l2; }
  __device__ __forceinline__ int at(int s) const {
    return (s < l0) ? s0 + s : (s < l0 + l1) ? s1 + (s - l0) : s2 + (s - l0 - l1);
  }
};

__device__ __forceinline__ void adj_epilogue(const AdjP2PArgs& a, int j, int cell, float x, float y, float m,
                                             float gx, float gy, float sm) {
  float rm = -sm;
  if (a.cell0) {  // transposed P2M of the far field
    const float4 c = a.cell0[cell];
    const float4 g = a.g0[cell];
    if (c.z != 0.0f) {
      gx += (m / c.z) * g.x;
      gy += (m / c.z) * g.y;
      rm += g.z + (g.x * (x - c.x) + g.y * (y - c.y)) / c.z;
    }
  }
  const int orig = __float_as_int(a.sorted4[j].w);
  a.gx_out[orig] = make_float2(gx, gy);
  a.gm_out[orig] = rm;
}

template <int NP, int ODD>
__device__ __forceinline__ void adj_item(const AdjP2PArgs& a, AdjSlice& sl, int lane, int cell, int first, int last,
                                         const AdjRanges& rg) {
  constexpr int kPasses = 2 * NP + ODD;
  float tx[kPasses], ty[kPasses], tm[kPasses], tux[kPasses], tuy[kPasses];
#pragma unroll
  for (int p = 0; p < kPasses; ++p) {
    const int j = first + p * 32 + lane;
    const bool v = j < last;
    const float4 q = v ? a.sorted4[j] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float2 u = v ? a.smu[j] : make_float2(0.0f, 0.0f);
    tx[p] = q.x; ty[p] = q.y; tm[p] = q.z; tux[p] = u.x; tuy[p] = u.y;
  }
  AdjTargets2 T[NP > 0 ? NP : 1];
#pragma unroll
  for (int q = 0; q < NP; ++q) {
    T[q].x = pk(tx[2 * q], tx[2 * q + 1]);
    T[q].y = pk(ty[2 * q], ty[2 * q + 1]);
    T[q].m = pk(tm[2 * q], tm[2 * q + 1]);
    T[q].mux = pk(tux[2 * q], tux[2 * q + 1]);
    T[q].muy = pk(tuy[2 * q], tuy[2 * q + 1]);
    T[q].gx = 0ull;
    T[q].gy = 0ull;
    T[q].sm = 0ull;
  }
  AdjTarget1 O{tx[kPasses - 1], ty[kPasses - 1], tm[kPasses - 1], tux[kPasses - 1], tuy[kPasses - 1], 0.0f, 0.0f, 0.0f};
  const float eps = a.eps;
  const f2x eps2 = pk(eps, eps);
  const f2x neg3 = pk(-3.0f, -3.0f);
  const int total = rg.total();
  float4 nq = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float2 nu = make_float2(0.0f, 0.0f);
  if (lane < total) {
    const int g = rg.at(lane);
    nq = a.sorted4[g];
    nu = a.smu[g];
  }
  for (int base = 0; base < total; base += 32) {
    __syncwarp();
    sl.xy[lane] = make_ulonglong2(pk(nq.x, nq.x), pk(nq.y, nq.y));
    sl.mu[lane] = make_ulonglong2(pk(nu.x, nu.x), pk(nu.y, nu.y));
    sl.mneg[lane] = pk(-nq.z, -nq.z);  // beyond `total` the source is massless with mu = 0: an exact zero
    __syncwarp();
    nq = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    nu = make_float2(0.0f, 0.0f);
    if (base + 32 + lane < total) {
      const int g = rg.at(base + 32 + lane);
      nq = a.sorted4[g];
      nu = a.smu[g];
    }
#pragma unroll 4
    for (int k = 0; k < 32; ++k) {
      const ulonglong2 s = sl.xy[k];
      const ulonglong2 u = sl.mu[k];
      const f2x mn = sl.mneg[k];
#pragma unroll
      for (int q = 0; q < NP; ++q) adj_pair2(T[q], s.x, s.y, u.x, u.y, mn, eps2, neg3);
      if (ODD) {
        float sx, sy, ux, uy, m, dummy;
        up(s.x, sx, dummy);
        up(s.y, sy, dummy);
        up(u.x, ux, dummy);
        up(u.y, uy, dummy);
        up(mn, m, dummy);
        adj_pair1(O, sx, sy, ux, uy, m, eps);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < NP; ++q) {
    float gx0, gx1, gy0, gy1, s0, s1;
    up(T[q].gx, gx0, gx1);
    up(T[q].gy, gy0, gy1);
    up(T[q].sm, s0, s1);
    const int j0 = first + (2 * q) * 32 + lane, j1 = j0 + 32;
    if (j0 < last) adj_epilogue(a, j0, cell, tx[2 * q], ty[2 * q], tm[2 * q], gx0, gy0, s0);
    if (j1 < last) adj_epilogue(a, j1, cell, tx[2 * q + 1], ty[2 * q + 1], tm[2 * q + 1], gx1, gy1, s1);
  }
  if (ODD) {
    const int j = first + (kPasses - 1) * 32 + lane;
    if (j < last) adj_epilogue(a, j, cell, O.x, O.y, O.m, O.gx, O.gy, O.sm);
  }
}

// Reverse near field + the transposed P2M of the far field. Warps are independent and take (cell, up to 128
// targets) items; the item's sources stream through the warp's own 32-source slice.
__global__ void __launch_bounds__(kAdjWarps * 32, 4) adj_p2p_kernel(const AdjP2PArgs a) {
  __shared__ AdjSlice slices[kAdjWarps];
  const int lane = threadIdx.x & 31;
  AdjSlice& sl = slices[threadIdx.x >> 5];
  const int B = a.base_dim;
  const int work_count = *a.d_work_count;
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(a.d_work_next, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= work_count) break;
    const int2 wc = a.work[item];
    const int cell = wc.x;
    const int cx = cell % B, cy = cell / B;
    const int lo = cx > 0 ? cx - 1 : 0;
    const int hi = cx + 1 < B ? cx + 1 : B - 1;
    AdjRanges rg{0, 0, 0, 0, 0, 0};
    if (cy > 0) { rg.s0 = a.head[lo + (cy - 1) * B]; rg.l0 = a.head[hi + (cy - 1) * B + 1] - rg.s0; }
    rg.s1 = a.head[lo + cy * B];
    rg.l1 = a.head[hi + cy * B + 1] - rg.s1;
    if (cy + 1 < B) { rg.s2 = a.head[lo + (cy + 1) * B]; rg.l2 = a.head[hi + (cy + 1) * B + 1] - rg.s2; }
    const int first = a.head[cell] + item_first_pass(wc.y) * 32;
    const int last = min(first + item_passes(wc.y) * 32, a.head[cell + 1]);
    switch ((last - first + 31) >> 5) {
      case 1: adj_item<0, 1>(a, sl, lane, cell, first, last, rg); break;
      case 2: adj_item<1, 0>(a, sl, lane, cell, first, last, rg); break;
      case 3: adj_item<1, 1>(a, sl, lane, cell, first, last, rg); break;
      default: adj_item<2, 0>(a, sl, lane, cell, first, last, rg); break;
    }
  }
}

// x' = 2x - x_prev + a tau^2 (update.cu:39-40, as the P2P Verlet epilogue rounds it), x_prev = x.
__global__ void adj_verlet_kernel(int n, float tau, float2* __restrict__ x, float2* __restrict__ xp,
                                  const float2* __restrict__ acc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 p = x[i], q = xp[i], e = acc[i];
    const float bx = __fsub_rn(__fmul_rn(2.0f, p.x), q.x);
    const float by = __fsub_rn(__fmul_rn(2.0f, p.y), q.y);
    x[i] = make_float2(__fmaf_rn(__fmul_rn(e.x, tau), tau, bx), __fmaf_rn(__fmul_rn(e.y, tau), tau, by));
    xp[i] = p;
  }
}

// x_{-1} = x_0 - v_0 tau
__global__ void adj_init_kernel(int n, float tau, const float2* __restrict__ x0, const float2* __restrict__ v0,
                                float2* __restrict__ x, float2* __restrict__ xp) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 p = x0[i], v = v0[i];
    x[i] = p;
    // both operations rounded (no fused multiply-add), as x0 - v0 * tau evaluates on a host
    xp[i] = make_float2(__fsub_rn(p.x, __fmul_rn(v.x, tau)), __fsub_rn(p.y, __fmul_rn(v.y, tau)));
  }
}

// lambda_T = m (x_T - x*), grad_m = 0.5 |x_T - x*|^2, and the loss terms (summed on the host side of the test).
__global__ void adj_seed_kernel(int n, const float2* __restrict__ xT, const float2* __restrict__ target,
                                const float* __restrict__ m, float2* __restrict__ lam, float2* __restrict__ lam2,
                                float* __restrict__ gm_acc, float* __restrict__ loss_terms) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float dx = xT[i].x - target[i].x, dy = xT[i].y - target[i].y;
    const float e = 0.5f * (dx * dx + dy * dy);
    lam[i] = make_float2(m[i] * dx, m[i] * dy);
    lam2[i] = make_float2(0.0f, 0.0f);
    gm_acc[i] = e;
    loss_terms[i] = m[i] * e;
  }
}

// lambda_t = 2 lambda_{t+1} + g_x - lambda_{t+2} (written over lambda_{t+2}); grad_m += g_m.
__global__ void adj_step_kernel(int n, const float2* __restrict__ lam1, float2* __restrict__ lam2_to_0,
                                const float2* __restrict__ gx, const float* __restrict__ gm, float* __restrict__ gm_acc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 l1 = lam1[i], l2 = lam2_to_0[i], g = gx[i];
    lam2_to_0[i] = make_float2(2.0f * l1.x + g.x - l2.x, 2.0f * l1.y + g.y - l2.y);
    gm_acc[i] += gm[i];
  }
}

// grad_x0 = lambda_0 - lambda_1, grad_v0 = tau lambda_1, grad_m = accumulated.
__global__ void adj_finish_kernel(int n, float tau, const float2* __restrict__ lam0, const float2* __restrict__ lam1,
                                  const float* __restrict__ gm_acc, float2* __restrict__ gx0, float2* __restrict__ gv0,
                                  float* __restrict__ gm) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 a = lam0[i], b = lam1[i];
    gx0[i] = make_float2(a.x - b.x, a.y - b.y);
    gv0[i] = make_float2(tau * b.x, tau * b.y);
    gm[i] = gm_acc[i];
  }
}

int grid_for(long long n, int threads, int cap) {
  long long g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

}  // namespace

struct nbfmm_adjoint {
  nbfmm_solver* solver = nullptr;
  int n = 0, max_steps = 0, k = 1, steps = 0;
  float tau = 0.0f;
  float2 *x = nullptr, *xp = nullptr, *acc = nullptr;
  float2 *ckpt = nullptr;   // [num_ckpt][2][n]: x_t, x_{t-1} at t = 0, k, 2k, ...
  float2* seg = nullptr;    // [k][n] positions of one segment
  float2 *lam_a = nullptr, *lam_b = nullptr, *gx = nullptr, *smu = nullptr;
  float *gm = nullptr, *gm_acc = nullptr, *loss_terms = nullptr;
  float2* cell_lam = nullptr;
  float4* cell_g = nullptr;
  // Per step of a segment, the sort of that step's positions as its recomputation left it (sorted particles,
  // permutation, heads, cell centres of every level), reused by the step's vector-Jacobian product.
  float4* slot_sorted = nullptr;
  uint32_t* slot_perm = nullptr;
  int* slot_head = nullptr;
  float4* slot_cell = nullptr;
  const float* m = nullptr;  // caller's masses, kept between forward and backward
  float4* own_sorted = nullptr;  // the solver's own sort outputs (bind_slot)
  uint32_t* own_vals = nullptr;
  int* own_head = nullptr;
  float4* own_cell = nullptr;
  float fwd_ms = 0.0f, bwd_ms = 0.0f;

  int init(int num_level, int num_particle, const float* limits, float tau_, int max_steps_, int k_) {
    n = num_particle;
    max_steps = max_steps_;
    k = k_;
    tau = tau_;
    NBFMM_TRY(nbfmm_make_solver(num_level, std::max(n, 1), limits, 0, &solver));
    const size_t N = (size_t)std::max(n, 1);
    const int num_ckpt = (max_steps + k - 1) / k + 1;
    NBFMM_TRY(dalloc(&x, N, "adjoint x"));
    NBFMM_TRY(dalloc(&xp, N, "adjoint x_prev"));
    NBFMM_TRY(dalloc(&acc, N, "adjoint effects"));
    NBFMM_TRY(dalloc(&ckpt, N * 2 * num_ckpt, "checkpoints"));
    NBFMM_TRY(dalloc(&seg, N * k, "segment"));
    NBFMM_TRY(dalloc(&lam_a, N, "lambda"));
    NBFMM_TRY(dalloc(&lam_b, N, "lambda"));
    NBFMM_TRY(dalloc(&gx, N, "g_x"));
    NBFMM_TRY(dalloc(&smu, N, "sorted mu"));
    NBFMM_TRY(dalloc(&gm, N, "g_m"));
    NBFMM_TRY(dalloc(&gm_acc, N, "grad m"));
    NBFMM_TRY(dalloc(&loss_terms, N, "loss terms"));
    NBFMM_TRY(dalloc(&cell_lam, (size_t)solver->lv.total, "cell adjoints"));
    NBFMM_TRY(dalloc(&cell_g, (size_t)solver->lv.total, "cell gradients"));
    NBFMM_TRY(dalloc(&slot_sorted, N * k, "segment sorted particles"));
    NBFMM_TRY(dalloc(&slot_perm, N * k, "segment permutations"));
    NBFMM_TRY(dalloc(&slot_head, ((size_t)solver->num_cells + 2) * k, "segment heads"));
    NBFMM_TRY(dalloc(&slot_cell, (size_t)solver->lv.total * k, "segment cells"));
    own_sorted = solver->sorted4;
    own_vals = solver->vals_a;
    own_head = solver->head;
    own_cell = solver->cell4;
    return cuda_check("adjoint init");
  }

  ~nbfmm_adjoint() {
    dfree(x); dfree(xp); dfree(acc); dfree(ckpt); dfree(seg); dfree(lam_a); dfree(lam_b); dfree(gx); dfree(smu);
    dfree(gm); dfree(gm_acc); dfree(loss_terms); dfree(cell_lam); dfree(cell_g);
    dfree(slot_sorted); dfree(slot_perm); dfree(slot_head); dfree(slot_cell);
    delete solver;
  }

  float2* ck(int i, int which) { return ckpt + ((size_t)i * 2 + which) * (size_t)n; }

  // Points the solver's sort outputs at segment slot `slot` (or back at its own buffers with slot < 0).
  void bind_slot(int slot) {
    nbfmm_solver& v = *solver;
    if (slot < 0) {
      v.sorted4 = own_sorted;
      v.vals_a = own_vals;
      v.head = own_head;
      v.cell4 = own_cell;
      v.perm = own_vals;
      return;
    }
    const size_t N = (size_t)std::max(n, 1);
    v.sorted4 = slot_sorted + slot * N;
    v.vals_a = slot_perm + slot * N;
    v.head = slot_head + slot * ((size_t)v.num_cells + 2);
    v.cell4 = slot_cell + slot * (size_t)v.lv.total;
    v.perm = v.vals_a;
  }

  void step(cudaStream_t s) {  // one forward step on (x, xp)
    solver->solve(n, reinterpret_cast<const float*>(x), m, reinterpret_cast<float*>(acc), s);
    adj_verlet_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(n, tau, x, xp, acc);
  }

  int forward(int num_steps, const float* x0, const float* v0, const float* masses, float* x_final, cudaStream_t s) {
    steps = num_steps;
    m = masses;
    adj_init_kernel<<<grid_for(n, 256, 152 * 16), 256, 0, s>>>(n, tau, reinterpret_cast<const float2*>(x0),
                                                                reinterpret_cast<const float2*>(v0), x, xp);
    for (int t = 0; t < num_steps; ++t) {
      if (t % k == 0) {
        cudaMemcpyAsync(ck(t / k, 0), x, sizeof(float2) * n, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(ck(t / k, 1), xp, sizeof(float2) * n, cudaMemcpyDeviceToDevice, s);
      }
      step(s);
    }
    cudaMemcpyAsync(x_final, x, sizeof(float2) * n, cudaMemcpyDeviceToDevice, s);
    return cuda_check("nbfmm_adjoint_forward");
  }

  // VJP of one solve at positions `pos` (original order) for effect adjoint scale * lam; results in gx, gm. With
  // `cached`, the solver is bound to the slot the step's recomputation sorted pos into (bind_slot), and only the
  // work list is rebuilt (the solve's pairs tails; adj_p2p_kernel reads plain 128-target chunks).
  void vjp(const float2* pos, const float2* lam, float scale, bool cached, cudaStream_t s) {
    nbfmm_solver& v = *solver;
    if (cached) launch_worklist(v.head, v.num_cells, v.work, v.d_work_count(), false, s, v.item_passes);
    else v.predo(n, pos, m, s, false);
    const int cells = v.num_cells;
    adj_gather_kernel<<<grid_for((long long)cells * 32, 256, 152 * 16), 256, 0, s>>>(cells, v.head, v.perm, lam,
                                                                                    scale, smu, cell_lam);
    const bool far = v.geo.num_level > 0;
    if (far) {
      if (!cached) launch_m2m(v.lv, v.cell4, s);  // a cached slot holds every level
      // Lambda up: per level while the parents have more than kAdjSmall cells per side, then one launch.
      constexpr int kAdjSmall = 64;
      int l = 1;
      for (; l < v.lv.count && v.lv.dim[l] > kAdjSmall; ++l) {
        adj_up_kernel<<<grid_for((long long)v.lv.dim[l] * v.lv.dim[l], 256, 152 * 8), 256, 0, s>>>(
            cell_lam, v.lv.offset[l - 1], v.lv.dim[l - 1], v.lv.offset[l], v.lv.dim[l]);
      }
      if (l < v.lv.count) adj_up_top_kernel<<<1, 256, 0, s>>>(cell_lam, v.lv, l);
      // Transposed M2L: large levels per level, the small ones in one launch.
      int lw = v.lv.count;
      for (int q = 0; q < v.lv.count; ++q) {
        if (v.lv.dim[q] <= kAdjWideDim) {
          lw = q;
          break;
        }
      }
      for (int q = 0; q < lw; ++q) {
        const int d = v.lv.dim[q];
        const dim3 grid((d + kM2LTile - 1) / kM2LTile, (d + kM2LTile - 1) / kM2LTile);
        adj_m2l_kernel<<<grid, dim3(kM2LTile, kM2LTile), 0, s>>>(v.cell4, cell_lam, cell_g, v.lv.offset[q], d, v.eps);
      }
      if (lw < v.lv.count) {
        const long long cells_w = (long long)v.lv.total - v.lv.offset[lw];
        adj_m2l_wide_kernel<<<(unsigned)((cells_w * 32 + 255) / 256), 256, 0, s>>>(v.cell4, cell_lam, cell_g, v.lv,
                                                                                  v.lv.offset[lw], v.eps);
      }
      // G down: the small parent levels in one launch, then per level.
      int ld = v.lv.count - 1;
      while (ld >= 1 && v.lv.dim[ld - 1] <= kAdjSmall) --ld;  // parent levels ld+1.. have children of <= kAdjSmall
      if (ld + 1 <= v.lv.count - 1) adj_down_top_kernel<<<1, 256, 0, s>>>(v.cell4, cell_g, v.lv, ld + 1);
      for (int q = ld; q >= 1; --q) {
        adj_down_kernel<<<grid_for((long long)v.lv.dim[q - 1] * v.lv.dim[q - 1], 256, 152 * 8), 256, 0, s>>>(
            v.cell4, cell_g, v.lv.offset[q - 1], v.lv.dim[q - 1], v.lv.offset[q], v.lv.dim[q]);
      }
    }
    AdjP2PArgs a{};
    a.sorted4 = v.sorted4;
    a.smu = smu;
    a.head = v.head;
    a.work = v.work;
    a.d_work_count = v.d_work_count();
    a.d_work_next = v.d_work_next();
    a.base_dim = v.geo.base_dim;
    a.eps = v.eps;
    a.cell0 = far ? v.cell0() : nullptr;
    a.g0 = far ? cell_g + v.lv.offset[0] : nullptr;
    a.gx_out = gx;
    a.gm_out = gm;
    cudaMemsetAsync(v.d_work_next(), 0, sizeof(int), s);
    adj_p2p_kernel<<<v.num_sms * 4, kAdjWarps * 32, 0, s>>>(a);
  }

  int backward(const float* target, float* grad_x0, float* grad_v0, float* grad_m, cudaStream_t s) {
    const int N = n;
    // lam_a = lambda_{t+1}, lam_b = lambda_{t+2}; the final positions are in x.
    adj_seed_kernel<<<grid_for(N, 256, 152 * 16), 256, 0, s>>>(N, x, reinterpret_cast<const float2*>(target), m,
                                                               lam_a, lam_b, gm_acc, loss_terms);
    const float tau2 = tau * tau;
    const int segs = (steps + k - 1) / k;
    for (int sgi = segs - 1; sgi >= 0; --sgi) {
      const int t0 = sgi * k, t1 = std::min(t0 + k, steps);
      cudaMemcpyAsync(x, ck(sgi, 0), sizeof(float2) * N, cudaMemcpyDeviceToDevice, s);
      cudaMemcpyAsync(xp, ck(sgi, 1), sizeof(float2) * N, cudaMemcpyDeviceToDevice, s);
      for (int t = t0; t < t1; ++t) {  // positions x_t for t in [t0, t1); each step's sort kept in its slot
        cudaMemcpyAsync(seg + (size_t)(t - t0) * N, x, sizeof(float2) * N, cudaMemcpyDeviceToDevice, s);
        if (t + 1 < t1) {
          bind_slot(t - t0);
          step(s);
          bind_slot(-1);
        }
      }
      for (int t = t1 - 1; t >= t0; --t) {
        bind_slot(t - t0);
        vjp(seg + (size_t)(t - t0) * N, lam_a, tau2, t + 1 < t1, s);
        bind_slot(-1);
        adj_step_kernel<<<grid_for(N, 256, 152 * 16), 256, 0, s>>>(N, lam_a, lam_b, gx, gm, gm_acc);
        std::swap(lam_a, lam_b);  // lam_a = lambda_t, lam_b = lambda_{t+1}
      }
    }
    adj_finish_kernel<<<grid_for(N, 256, 152 * 16), 256, 0, s>>>(N, tau, lam_a, lam_b, gm_acc,
                                                                 reinterpret_cast<float2*>(grad_x0),
                                                                 reinterpret_cast<float2*>(grad_v0), grad_m);
    return cuda_check("nbfmm_adjoint_backward");
  }
};

extern "C" {

int nbfmm_adjoint_create(int num_level, int num_particle, const float position_limits[4], float tick, float grav_const,
                         int max_steps, int checkpoint_interval, nbfmm_adjoint** out) {
  if (!out) return api_fail(NBFMM_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if (num_particle < 1) return api_fail(NBFMM_ERR_INVALID, "num_particle must be >= 1");
  if (max_steps < 1 || checkpoint_interval < 1) {
    return api_fail(NBFMM_ERR_INVALID, "max_steps and checkpoint_interval must be >= 1");
  }
  const float tau = tick * std::sqrt(grav_const);  // stars.cu:31
  if (!(tau > 0.0f) || !std::isfinite(tau)) return api_fail(NBFMM_ERR_INVALID, "tick * sqrt(grav_const) must be > 0");
  nbfmm_adjoint* h = new (std::nothrow) nbfmm_adjoint();
  if (!h) return api_fail(NBFMM_ERR_NOMEM, "host allocation failed");
  const int rc = h->init(num_level, num_particle, position_limits, tau, max_steps, checkpoint_interval);
  if (rc != NBFMM_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return NBFMM_OK;
}

int nbfmm_adjoint_destroy(nbfmm_adjoint* adj) {
  delete adj;
  return NBFMM_OK;
}

int nbfmm_adjoint_set_epsilon(nbfmm_adjoint* adj, float epsilon) {
  if (!adj) return api_fail(NBFMM_ERR_INVALID, "null adjoint handle");
  return nbfmm_solver_set_epsilon(adj->solver, epsilon);
}

int nbfmm_adjoint_forward(nbfmm_adjoint* adj, int num_steps, const float* gpuptr_position0,
                          const float* gpuptr_velocity0, const float* gpuptr_weight, float* gpuptr_position_final,
                          void* stream) {
  if (!adj) return api_fail(NBFMM_ERR_INVALID, "null adjoint handle");
  if (num_steps < 1 || num_steps > adj->max_steps) {
    return api_fail(NBFMM_ERR_INVALID, "num_steps %d outside [1, %d]", num_steps, adj->max_steps);
  }
  if (!gpuptr_position0 || !gpuptr_velocity0 || !gpuptr_weight || !gpuptr_position_final) {
    return api_fail(NBFMM_ERR_INVALID, "null device pointer");
  }
  return adj->forward(num_steps, gpuptr_position0, gpuptr_velocity0, gpuptr_weight, gpuptr_position_final,
                      reinterpret_cast<cudaStream_t>(stream));
}

int nbfmm_adjoint_backward(nbfmm_adjoint* adj, const float* gpuptr_target, float* gpuptr_grad_position0,
                           float* gpuptr_grad_velocity0, float* gpuptr_grad_weight, float* gpuptr_loss_terms,
                           void* stream) {
  if (!adj) return api_fail(NBFMM_ERR_INVALID, "null adjoint handle");
  if (adj->steps < 1 || !adj->m) return api_fail(NBFMM_ERR_INVALID, "nbfmm_adjoint_forward must run first");
  if (!gpuptr_target || !gpuptr_grad_position0 || !gpuptr_grad_velocity0 || !gpuptr_grad_weight) {
    return api_fail(NBFMM_ERR_INVALID, "null device pointer");
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int rc = adj->backward(gpuptr_target, gpuptr_grad_position0, gpuptr_grad_velocity0, gpuptr_grad_weight, s);
  if (rc == NBFMM_OK && gpuptr_loss_terms) {
    cudaMemcpyAsync(gpuptr_loss_terms, adj->loss_terms, sizeof(float) * adj->n, cudaMemcpyDeviceToDevice, s);
  }
  return rc == NBFMM_OK ? cuda_check("nbfmm_adjoint_backward") : rc;
}

}  // extern "C"
