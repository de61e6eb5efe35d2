// display.cu -- the frame raster of Stars::display and the .y4m movie of the reference's main program.
//
// Reference: source/nbfmm/display/stars/display.cu (displayDevice :29-214, Stars::display :219-229) and the frame
// loop of main/main.cu:228-259 (header :238, "FRAME\n" + width*height*3/2 bytes per frame :242-250).
//
// A frame is YUV 4:2:0: the Y plane (width*height bytes) cleared to 0, the next width*height/2 bytes to 128, and
// every star inside the display limits sets its pixel and, by its size floor(sqrt(w) / size_scale), up to 48
// pixels around it to 255. Many stars share a pixel (a 16.8M-star frame sets each lit pixel ~30 times), so the
// pixels are first collected as bits: each CTA holds one band of the frame's bitmask in shared memory and ORs
// in the pixels of one slice of the stars; the slices' bitmasks are then ORed and expanded into the frame in
// one coalesced pass (raster_bits_kernel, expand_kernel). Frames too large for the bitmask's bands use
// display_kernel, one thread per star storing bytes.
//
// Kept from the reference: its arithmetic (IEEE division and square root, floor, the device's saturating
// float-to-int conversion), its per-pixel guards including the irregular ones, and its acceptance of a star on
// row `height` (display.cu:53), whose pixels fall into the chroma plane. Changed: a write whose byte lies
// outside the frame is dropped, where the reference writes before its buffer for stars on the top rows
// (display.cu:62,90,130,182 test only y >= 0).
//
// The movie keeps two device frames and two pinned host frames: the copy of frame k is queued behind its raster
// on the caller's stream, and the host writes frame k-1 to the file while the GPU works on frame k.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <new>

#include "../../include/nbfmm_gb300.h"
#include "engine.cuh"
#include "stars.cuh"

namespace nbfmm_gb300 {
int api_fail(int code, const char* fmt, ...);
bool injected_alloc_failure();

namespace {

// One pixel of the star stamp: drawn from `size`, at (dx, dy) from the star's pixel, when
// x >= xa && x < width - xb && y >= ya && y < height - yb (xb, yb = -1: no upper test). Rows in the order of
// display.cu:55-212, grouped by size.
struct StampPixel {
  signed char size, dx, dy, xa, xb, ya, yb, pad;
};

__constant__ StampPixel c_stamp[48] = {
    {1, -1, 0, 1, -1, 0, -1, 0},  {1, 1, 0, 0, 1, 0, -1, 0},   {1, 0, -1, 0, -1, 0, -1, 0}, {1, 0, 1, 0, -1, 0, 1, 0},
    {2, -1, -1, 1, -1, 1, -1, 0}, {2, -1, 1, 1, -1, 0, 1, 0},  {2, 1, -1, 0, 1, 1, -1, 0},  {2, 1, 1, 0, 1, 0, 1, 0},
    {3, -2, 0, 2, -1, 0, -1, 0},  {3, 2, 0, 0, 2, 0, -1, 0},   {3, 0, -2, 0, -1, 0, -1, 0}, {3, 0, 2, 0, -1, 0, 2, 0},
    {4, -2, -1, 2, -1, 1, -1, 0}, {4, -1, -2, 1, -1, 2, -1, 0}, {4, -2, 1, 2, -1, 0, 2, 0}, {4, -1, 2, 1, -1, 0, 2, 0},
    {4, 2, -1, 0, 2, 1, -1, 0},   {4, 1, -2, 0, 2, 2, -1, 0},  {4, 2, 1, 0, 2, 0, 2, 0},    {4, 1, 2, 0, 2, 0, 2, 0},
    {5, -3, 0, 3, -1, 0, -1, 0},  {5, 3, 0, 0, 3, 0, -1, 0},   {5, 0, -3, 0, -1, 0, -1, 0}, {5, 0, 3, 0, -1, 0, 3, 0},
    {5, -2, -2, 2, -1, 2, -1, 0}, {5, -2, 2, 2, -1, 0, 2, 0},  {5, 2, -2, 0, 2, 2, -1, 0},  {5, 2, 2, 0, 2, 0, 2, 0},
    {6, -3, -1, 3, -1, 1, -1, 0}, {6, -1, -3, 1, -1, 3, -1, 0}, {6, -3, 1, 3, -1, 0, 3, 0}, {6, -1, 3, 1, -1, 0, 3, 0},
    {6, 3, -1, 0, 3, 1, -1, 0},   {6, 1, -3, 0, 3, 3, -1, 0},  {6, 3, 1, 0, 3, 0, 3, 0},    {6, 1, 3, 0, 3, 0, 3, 0},
    {7, -4, 0, 4, -1, 0, -1, 0},  {7, 4, 0, 0, 4, 0, -1, 0},   {7, 0, -4, 0, -1, 0, -1, 0}, {7, 0, 4, 0, -1, 0, 4, 0},
    {7, -3, -2, 3, -1, 2, -1, 0}, {7, -2, -3, 2, -1, 3, -1, 0}, {7, -3, 2, 3, -1, 0, 3, 0}, {7, -2, 3, 2, -1, 0, 3, 0},
    {7, 3, -2, 0, 3, 2, -1, 0},   {7, 2, -3, 0, 3, 3, -1, 0},  {7, 3, 2, 0, 3, 0, 3, 0},    {7, 2, 3, 0, 3, 0, 3, 0},
};
// Stamp pixels drawn for sizes 1..7 (and above).
__constant__ int c_stamp_count[8] = {0, 4, 8, 12, 20, 28, 36, 48};

__global__ void display_kernel(const int* __restrict__ d_n, int n_host, int width, int height, float size_scale,
                               float4 lim, const float2* __restrict__ pos, const float* __restrict__ w,
                               uint8_t* __restrict__ board, long long frame) {
  const int n = d_n ? *d_n : n_host;
  const float unit_width = __fdiv_rn(__fsub_rn(lim.z, lim.x), (float)width);    // display.cu:45
  const float unit_height = __fdiv_rn(__fsub_rn(lim.w, lim.y), (float)height);  // display.cu:46
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 p = pos[i];
    const int x = __float2int_rz(floorf(__fdiv_rn(__fsub_rn(p.x, lim.x), unit_width)));   // display.cu:47
    const int y = __float2int_rz(floorf(__fdiv_rn(__fsub_rn(lim.w, p.y), unit_height)));  // display.cu:48
    if (!(0 <= x && x < width && 0 <= y && y <= height)) continue;                         // display.cu:53
    const int size = __float2int_rz(floorf(__fdiv_rn(__fsqrt_rn(w[i]), size_scale)));    // display.cu:49
    const long long at = (long long)y * width + x;
    if (at < frame) board[at] = 255;
    const int count = size <= 0 ? 0 : c_stamp_count[size < 7 ? size : 7];
    for (int k = 0; k < count; ++k) {
      const StampPixel e = c_stamp[k];
      if (x >= e.xa && x < width - e.xb && y >= e.ya && y < height - e.yb) {
        const long long t = at + (long long)e.dy * width + e.dx;
        if (t >= 0 && t < frame) board[t] = 255;
      }
    }
  }
}

int grid_for(long long n) {
  long long g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g));
}

bool frame_ok(int width, int height) {
  return width > 0 && height > 0 && (long long)width * height * 3 / 2 < (1LL << 40);
}

// ---- Bitmask raster ------------------------------------------------------------------------------------------
//
// The pixels a frame's stars set are collected as bits: pixel index p = row * width + column over rows
// 0..height (row `height` being the first chroma bytes), at most the frame's size. A CTA owns one band of those
// bits in shared memory and one slice of the stars; for each star it ORs in the star's pixels that fall in its
// band. A star at least 4 pixels from every edge passes all of the stamp's guards, so its pixels are the
// precomputed row masks of its size (at most 9 rows of 9 pixels, one or two 32-bit ORs per row); a star nearer
// an edge evaluates the guards pixel by pixel. The slices' bitmasks are then ORed together and expanded into
// the frame: 255 for a set pixel, else 0 in the Y plane and 128 in the chroma bytes, written 32 bytes per
// thread. The frame is the one the byte-store kernel above writes.

constexpr int kRasterThreads = 1024;
constexpr int kRasterMaxBandWords = 192 * 1024 / 4;  // shared-memory bitmask per CTA (+16 KB of queues)
constexpr int kRasterMaxBands = 16;

// Rows above and below its pixel that the stamp of a size reaches (display.cu:55-212).
__constant__ int c_stamp_radius[8] = {0, 1, 1, 2, 2, 3, 3, 4};

// floor(RN(a / b)) converted as the device converts (display.cu:47-48), from the estimate q = a * rb with
// rb = RN(1 / b). |q - RN(a / b)| <= 1.5 * 2^-23 |q| (two roundings of the estimate, one of the quotient), so
// when q is farther than 4e-7 |q| from every integer both floor to the same value; otherwise (and for NaN,
// infinities and |q| >= 2^23, where q has no fraction) the IEEE division decides.
__device__ __forceinline__ int floor_quotient(float a, float b, float rb) {
  const float q = a * rb;
  const float f = floorf(q);
  const float margin = 4e-7f * fabsf(q);
  if (q - f > margin && (f + 1.0f) - q > margin) return __float2int_rz(f);
  return __float2int_rz(floorf(__fdiv_rn(a, b)));
}

// The star size floor(RN(RN(sqrt(w)) / size_scale)) (display.cu:49), clamped to 8: every size from 7 up draws
// the same stamp. The estimate sqrt.approx(w) * RN(1 / size_scale) is within 4 * 2^-23 relative of the
// quotient; near an integer (and for NaN, negative, zero or subnormal weights) the IEEE operations decide.
__device__ __forceinline__ int star_size(float w, float size_scale, float rscale) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(w));
  const float q = r * rscale;
  if (q >= 8.001f) return 8;
  const float f = floorf(q);
  const float margin = 1e-6f * fabsf(q);
  if (q - f > margin && (f + 1.0f) - q > margin) return __float2int_rz(f);
  const int s = __float2int_rz(floorf(__fdiv_rn(__fsqrt_rn(w), size_scale)));
  return s > 8 ? 8 : s;
}

// One star's pixels ORed into this CTA's band of the bitmask: bits [b0, b1) in s_bits. A star at least 4 pixels
// from every edge passes every guard of the stamp, so its pixels are the precomputed rows of its size; nearer
// an edge the guards are evaluated pixel by pixel.
__device__ __forceinline__ void draw_star_bits(uint32_t* s_bits, int b0, int b1, const unsigned short (*rows)[9],
                                               int x, int y, int size, int width, int height, int nbits) {
  const int at = y * width + x;
  if (x >= 4 && x < width - 4 && y >= 4 && y < height - 4) {
    const int sz = size < 0 ? 0 : (size > 7 ? 7 : size);
    const int r = c_stamp_radius[sz];
    const bool inside = at - r * width - 4 >= b0 && at + r * width + 4 < b1;  // the whole stamp in the band
    for (int dy = -r; dy <= r; ++dy) {
      const unsigned m = rows[sz][dy + 4];
      const int q = at + dy * width - 4 - b0;  // may lie outside the band when !inside: tested per word
      const int word = q >> 5;                 // arithmetic shift: floor for negative q
      const int sh = q & 31;
      const int words = (b1 - b0) >> 5;
      if (inside || (word >= 0 && word < words)) atomicOr(&s_bits[word], m << sh);
      if (sh > 23 && (inside || (word + 1 >= 0 && word + 1 < words))) atomicOr(&s_bits[word + 1], m >> (32 - sh));
    }
  } else {
    if (at < nbits && at >= b0 && at < b1) atomicOr(&s_bits[(at - b0) >> 5], 1u << ((at - b0) & 31));
    const int count = size <= 0 ? 0 : c_stamp_count[size < 7 ? size : 7];
    for (int k = 0; k < count; ++k) {
      const StampPixel e = c_stamp[k];
      if (x >= e.xa && x < width - e.xb && y >= e.ya && y < height - e.yb) {
        const int t = at + e.dy * width + e.dx;
        if (t >= 0 && t < nbits && t >= b0 && t < b1) atomicOr(&s_bits[(t - b0) >> 5], 1u << ((t - b0) & 31));
      }
    }
  }
}

__device__ __forceinline__ void build_stamp_rows(unsigned short (*rows)[9]) {
  if (threadIdx.x < 72) {
    const int size = threadIdx.x / 9, dy = threadIdx.x % 9 - 4;
    unsigned m = dy == 0 ? 1u << 4 : 0u;  // the star's own pixel
    for (int k = 0; k < c_stamp_count[size]; ++k) {
      if (c_stamp[k].dy == dy) m |= 1u << (c_stamp[k].dx + 4);
    }
    rows[size][dy + 4] = (unsigned short)m;
  }
}

// nbits < 2^31 here (at most kRasterMaxBands * kRasterMaxBandWords * 32 bits), so pixel indices are 32-bit.
// Each CTA holds one band of the bitmask and reads one slice of the stars. A warp takes 32 stars at a time,
// computes their rows, and appends the stars whose stamp reaches its band to a warp-local queue; the full
// computation (column, size, pixels) then runs on 32 queued stars at a time, so lanes do not idle on stars of
// other bands.
__global__ void __launch_bounds__(kRasterThreads, 1) raster_bits_kernel(
    const int* __restrict__ d_n, int n_host, int width, int height, float size_scale, float4 lim,
    const float2* __restrict__ pos, const float* __restrict__ w, int nbits, int words_total, int band_words,
    int bands, uint32_t* __restrict__ partial) {
  extern __shared__ uint32_t s_bits[];
  __shared__ unsigned short s_rows[8][9];  // size 0..7, row dy = -4..4: bit dx + 4 drawn
  __shared__ int s_queue[kRasterThreads / 32][64];
  __shared__ int s_queue_y[kRasterThreads / 32][64];
  const int n = d_n ? *d_n : n_host;
  const int slices = gridDim.x / bands;
  const int slice = blockIdx.x / bands, band = blockIdx.x % bands;
  const int wb0 = band * band_words;
  const int wb1 = min(wb0 + band_words, words_total);
  const int b0 = wb0 * 32, b1 = wb1 * 32;
  for (int i = threadIdx.x; i < band_words; i += blockDim.x) s_bits[i] = 0u;
  build_stamp_rows(s_rows);
  __syncthreads();
  const float unit_width = __fdiv_rn(__fsub_rn(lim.z, lim.x), (float)width);    // display.cu:45
  const float unit_height = __fdiv_rn(__fsub_rn(lim.w, lim.y), (float)height);  // display.cu:46
  const float rw = __frcp_rn(unit_width), rh = __frcp_rn(unit_height), rscale = __frcp_rn(size_scale);
  const int row_lo = b0 / width, row_hi = (b1 - 1) / width;
  const int lo = (int)((long long)n * slice / slices), hi = (int)((long long)n * (slice + 1) / slices);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
  int* queue = s_queue[warp];
  int* queue_y = s_queue_y[warp];
  int queued = 0;  // warp-uniform
  for (int base = lo + warp * 32; base < hi + 32 * warps; base += 32 * warps) {
    if (base < hi) {
      const int i = base + lane;
      bool keep = false;
      int y = 0;
      if (i < hi) {
        y = floor_quotient(__fsub_rn(lim.w, pos[i].y), unit_height, rh);   // display.cu:48
        keep = 0 <= y && y <= height && y + 4 >= row_lo && y - 4 <= row_hi;  // display.cu:53, and this band
      }
      const unsigned ballot = __ballot_sync(0xffffffffu, keep);
      if (keep) {
        const int slot = queued + __popc(ballot & ((1u << lane) - 1u));
        queue[slot] = i;
        queue_y[slot] = y;
      }
      queued += __popc(ballot);
      __syncwarp();
    }
    const bool last = base + 32 * warps >= hi + 32 * warps || base >= hi;
    while (queued >= 32 || (last && queued > 0)) {
      const int take = queued >= 32 ? 32 : queued;
      if (lane < take) {
        const int i = queue[queued - take + lane];
        const int y = queue_y[queued - take + lane];
        const int x = floor_quotient(__fsub_rn(pos[i].x, lim.x), unit_width, rw);  // display.cu:47
        if (0 <= x && x < width) {                                                // display.cu:53
          const int size = star_size(w[i], size_scale, rscale);                   // display.cu:49
          draw_star_bits(s_bits, b0, b1, s_rows, x, y, size, width, height, nbits);
        }
      }
      __syncwarp();
      queued -= take;
    }
  }
  __syncthreads();
  uint32_t* out = partial + (size_t)slice * (size_t)words_total + wb0;
  for (int i = threadIdx.x; i < wb1 - wb0; i += blockDim.x) out[i] = s_bits[i];
}

__device__ __forceinline__ uint32_t expand_byte(uint32_t v, int b, long long p, long long plane, long long nbits) {
  const bool set = (v >> b) & 1u;
  return p < plane ? (set ? 255u : 0u) : (set && p < nbits ? 255u : 128u);
}

__global__ void expand_kernel(const uint32_t* __restrict__ partial, int slices, long long words_total,
                              long long nbits, long long plane, long long frame, int aligned,
                              uint8_t* __restrict__ board) {
  const long long frame_words = (frame + 31) / 32;
  for (long long wi = blockIdx.x * (long long)blockDim.x + threadIdx.x; wi < frame_words;
       wi += (long long)gridDim.x * blockDim.x) {
    uint32_t v = 0u;
    if (wi < words_total) {
      for (int g = 0; g < slices; ++g) v |= partial[(size_t)g * (size_t)words_total + wi];
    }
    const long long p0 = wi * 32;
    if (aligned && p0 + 32 <= frame) {
      uint32_t q[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        uint32_t packed = 0u;
#pragma unroll
        for (int b = 0; b < 4; ++b) packed |= expand_byte(v, 4 * k + b, p0 + 4 * k + b, plane, nbits) << (8 * b);
        q[k] = packed;
      }
      uint4* dst = reinterpret_cast<uint4*>(board + p0);
      dst[0] = make_uint4(q[0], q[1], q[2], q[3]);
      dst[1] = make_uint4(q[4], q[5], q[6], q[7]);
    } else {
      for (int b = 0; b < 32 && p0 + b < frame; ++b) board[p0 + b] = (uint8_t)expand_byte(v, b, p0 + b, plane, nbits);
    }
  }
}

// The byte-store raster (clears, then display_kernel): frames whose bitmask needs more than kRasterMaxBands
// bands, or when the bitmask scratch cannot be had.
void launch_display_bytes(const int* d_n, int n_host, int max_n, int width, int height, float size_scale,
                          float4 lim, const float2* pos, const float* w, uint8_t* board, cudaStream_t s) {
  const long long plane = (long long)width * height;
  cudaMemsetAsync(board, 0, (size_t)plane, s);                  // display.cu:220
  cudaMemsetAsync(board + plane, 128, (size_t)(plane / 2), s);  // display.cu:221
  display_kernel<<<grid_for(d_n ? max_n : n_host), 256, 0, s>>>(d_n, n_host, width, height, size_scale, lim, pos,
                                                                w, board, frame_bytes(width, height));
}

}  // namespace

long long frame_bytes(int width, int height) { return (long long)width * height * 3 / 2; }

void launch_display(const int* d_n, int n_host, int max_n, int width, int height, float size_scale,
                    const float* limits, const float2* pos, const float* w, uint8_t* board, cudaStream_t s) {
  const float4 lim = make_float4(limits[0], limits[1], limits[2], limits[3]);
  const long long plane = (long long)width * height, frame = frame_bytes(width, height);
  const long long rows_bits = plane + width;  // rows 0..height
  const long long nbits = rows_bits < frame ? rows_bits : frame;
  const long long words_total = (nbits + 31) / 32;
  const long long bands = (words_total + kRasterMaxBandWords - 1) / kRasterMaxBandWords;
  if (bands > kRasterMaxBands) {
    launch_display_bytes(d_n, n_host, max_n, width, height, size_scale, lim, pos, w, board, s);
    return;
  }
  const int band_words = (int)((words_total + bands - 1) / bands);
  const int smem = band_words * 4;
  int dev = 0, num_sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
  // One CTA of 1024 threads per SM: up to 50 registers a thread leave no room for a second.
  const long long slices_ll = (long long)num_sms / bands;
  const int slices = slices_ll > 0 ? (int)slices_ll : 1;
  uint32_t* partial = nullptr;
  if (injected_alloc_failure() ||
      cudaFuncSetAttribute(raster_bits_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess ||
      cudaMallocAsync(reinterpret_cast<void**>(&partial), (size_t)slices * (size_t)words_total * 4, s) !=
          cudaSuccess) {
    cudaGetLastError();
    launch_display_bytes(d_n, n_host, max_n, width, height, size_scale, lim, pos, w, board, s);
    return;
  }
  raster_bits_kernel<<<slices * (int)bands, kRasterThreads, smem, s>>>(d_n, n_host, width, height, size_scale, lim,
                                                                       pos, w, (int)nbits, (int)words_total,
                                                                       band_words, (int)bands, partial);
  const long long frame_words = (frame + 31) / 32;
  const int aligned = (reinterpret_cast<uintptr_t>(board) & 15) == 0;
  expand_kernel<<<grid_for(frame_words), 256, 0, s>>>(partial, slices, words_total, nbits, plane, frame, aligned,
                                                      board);
  cudaFreeAsync(partial, s);
}

}  // namespace nbfmm_gb300

using namespace nbfmm_gb300;

// The movie of main.cu:228-259 for one Stars handle.
struct nbfmm_movie {
  nbfmm_stars* stars = nullptr;
  FILE* fp = nullptr;
  int width = 0, height = 0;
  float size_scale = 1.0f;
  float limits[4] = {0, 0, 0, 0};
  long long bytes = 0;
  uint8_t* board[2] = {nullptr, nullptr};
  uint8_t* host[2] = {nullptr, nullptr};
  cudaEvent_t copied[2] = {nullptr, nullptr};
  long long frames = 0;   // frames queued
  long long written = 0;  // frames written to the file

  int write_pending() {  // writes the oldest queued frame that is not in the file yet
    const int slot = (int)(written & 1);
    if (cudaEventSynchronize(copied[slot]) != cudaSuccess) {
      return api_fail(NBFMM_ERR_CUDA, "movie frame copy: %s", cudaGetErrorString(cudaGetLastError()));
    }
    if (std::fputs("FRAME\n", fp) < 0 || std::fwrite(host[slot], 1, (size_t)bytes, fp) != (size_t)bytes) {
      return api_fail(NBFMM_ERR_INVALID, "movie: write to the output file failed");
    }
    ++written;
    return NBFMM_OK;
  }

  ~nbfmm_movie() {
    for (int k = 0; k < 2; ++k) {
      if (copied[k]) cudaEventDestroy(copied[k]);
      if (board[k]) cudaFree(board[k]);
      if (host[k]) cudaFreeHost(host[k]);
    }
    if (fp) std::fclose(fp);
  }
};

extern "C" {

int nbfmm_display(int num_star, int width, int height, float size_scale, const float display_limits[4],
                  const float* gpuptr_position, const float* gpuptr_weight, uint8_t* gpuptr_board, void* stream) {
  if (num_star < 0) return api_fail(NBFMM_ERR_INVALID, "num_star must be >= 0");
  if (!frame_ok(width, height)) return api_fail(NBFMM_ERR_INVALID, "width and height must be > 0 (stars.cu:37-38)");
  if (!(size_scale > 0.0f)) return api_fail(NBFMM_ERR_INVALID, "size_scale must be > 0 (stars.cu:41)");
  if (!display_limits || !(display_limits[0] < display_limits[2] && display_limits[1] < display_limits[3])) {
    return api_fail(NBFMM_ERR_INVALID, "display limits must satisfy x_min < x_max, y_min < y_max (stars.cu:43)");
  }
  if (!gpuptr_board || (num_star > 0 && (!gpuptr_position || !gpuptr_weight))) {
    return api_fail(NBFMM_ERR_INVALID, "null device pointer");
  }
  launch_display(nullptr, num_star, num_star, width, height, size_scale, display_limits,
                 reinterpret_cast<const float2*>(gpuptr_position), gpuptr_weight, gpuptr_board,
                 (cudaStream_t)stream);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return api_fail(NBFMM_ERR_CUDA, "nbfmm_display: %s", cudaGetErrorString(e));
  return NBFMM_OK;
}

long long nbfmm_frame_bytes(int width, int height) { return frame_bytes(width, height); }

int nbfmm_movie_open(nbfmm_stars* stars, const char* path, int width, int height, int fps, float size_scale,
                     const float display_limits[4], nbfmm_movie** out) {
  if (!out) return api_fail(NBFMM_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if (!stars || !path) return api_fail(NBFMM_ERR_INVALID, "null argument");
  if (!frame_ok(width, height)) return api_fail(NBFMM_ERR_INVALID, "width and height must be > 0 (stars.cu:37-38)");
  if (fps <= 0) return api_fail(NBFMM_ERR_INVALID, "fps must be > 0 (stars.cu:39)");
  if (!(size_scale > 0.0f)) return api_fail(NBFMM_ERR_INVALID, "size_scale must be > 0 (stars.cu:41)");
  if (!display_limits || !(display_limits[0] < display_limits[2] && display_limits[1] < display_limits[3])) {
    return api_fail(NBFMM_ERR_INVALID, "display limits must satisfy x_min < x_max, y_min < y_max (stars.cu:43)");
  }
  nbfmm_movie* m = new (std::nothrow) nbfmm_movie();
  if (!m) return api_fail(NBFMM_ERR_NOMEM, "host allocation failed");
  m->stars = stars;
  m->width = width;
  m->height = height;
  m->size_scale = size_scale;
  for (int k = 0; k < 4; ++k) m->limits[k] = display_limits[k];
  m->bytes = frame_bytes(width, height);
  for (int k = 0; k < 2; ++k) {
    if (injected_alloc_failure()) {
      delete m;
      return api_fail(NBFMM_ERR_NOMEM, "movie: frame buffers: injected failure");
    }
    if (cudaMalloc(&m->board[k], (size_t)m->bytes) != cudaSuccess ||
        cudaMallocHost(&m->host[k], (size_t)m->bytes) != cudaSuccess ||
        cudaEventCreateWithFlags(&m->copied[k], cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      delete m;
      return api_fail(NBFMM_ERR_NOMEM, "movie: frame buffers could not be allocated");
    }
  }
  m->fp = std::fopen(path, "wb");
  if (!m->fp) {
    delete m;
    return api_fail(NBFMM_ERR_INVALID, "movie: cannot open %s for writing", path);
  }
  // main.cu:238
  if (std::fprintf(m->fp, "YUV4MPEG2 W%d H%d F%d:%d Ip A1:1 C420\n", width, height, fps, 1) < 0) {
    delete m;
    return api_fail(NBFMM_ERR_INVALID, "movie: write to the output file failed");
  }
  *out = m;
  return NBFMM_OK;
}

int nbfmm_movie_frame(nbfmm_movie* movie, void* stream) {
  if (!movie) return api_fail(NBFMM_ERR_INVALID, "null movie handle");
  cudaStream_t s = (cudaStream_t)stream;
  const int slot = (int)(movie->frames & 1);
  if (movie->frames - movie->written >= 2) {  // the slot still holds a frame that is not in the file
    const int rc = movie->write_pending();
    if (rc != NBFMM_OK) return rc;
  }
  const int rc = nbfmm_stars_display(movie->stars, movie->width, movie->height, movie->size_scale, movie->limits,
                                     movie->board[slot], stream);
  if (rc != NBFMM_OK) return rc;
  if (cudaMemcpyAsync(movie->host[slot], movie->board[slot], (size_t)movie->bytes, cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaEventRecord(movie->copied[slot], s) != cudaSuccess) {
    return api_fail(NBFMM_ERR_CUDA, "movie frame copy: %s", cudaGetErrorString(cudaGetLastError()));
  }
  ++movie->frames;
  if (movie->frames - movie->written >= 2) return movie->write_pending();  // the previous frame
  return NBFMM_OK;
}

int nbfmm_movie_close(nbfmm_movie* movie) {
  if (!movie) return NBFMM_OK;
  int rc = NBFMM_OK;
  while (rc == NBFMM_OK && movie->written < movie->frames) rc = movie->write_pending();
  if (movie->fp && std::fclose(movie->fp) != 0 && rc == NBFMM_OK) {
    rc = api_fail(NBFMM_ERR_INVALID, "movie: closing the output file failed");
  }
  movie->fp = nullptr;
  delete movie;
  return rc;
}

}  // extern "C"
