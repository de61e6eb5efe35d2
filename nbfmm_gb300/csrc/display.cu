// display.cu -- the frame raster of Stars::display and the .y4m movie of the reference's main program.
//
// Reference: source/nbfmm/display/stars/display.cu (displayDevice :29-214, Stars::display :219-229) and the frame
// loop of main/main.cu:228-259 (header :238, "FRAME\n" + width*height*3/2 bytes per frame :242-250).
//
// A frame is YUV 4:2:0: the Y plane (width*height bytes) cleared to 0, the next width*height/2 bytes to 128, and
// every star inside the display limits sets its pixel and, by its size floor(sqrt(w) / size_scale), up to 48
// pixels around it to 255. One thread per star; all writes store the same value, so their order and any overlap
// between stars do not matter and no atomics are needed. The frame of a 1080p movie (3 MB) stays in L2; the
// star arrays are read once, coalesced.
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

}  // namespace

long long frame_bytes(int width, int height) { return (long long)width * height * 3 / 2; }

void launch_display(const int* d_n, int n_host, int max_n, int width, int height, float size_scale,
                    const float* limits, const float2* pos, const float* w, uint8_t* board, cudaStream_t s) {
  const long long plane = (long long)width * height;
  cudaMemsetAsync(board, 0, (size_t)plane, s);                    // display.cu:220
  cudaMemsetAsync(board + plane, 128, (size_t)(plane / 2), s);    // display.cu:221
  const float4 lim = make_float4(limits[0], limits[1], limits[2], limits[3]);
  display_kernel<<<grid_for(d_n ? max_n : n_host), 256, 0, s>>>(d_n, n_host, width, height, size_scale, lim, pos,
                                                                w, board, frame_bytes(width, height));
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
