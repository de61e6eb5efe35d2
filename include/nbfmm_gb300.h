/*
 * nbfmm_gb300.h -- C ABI of the GB300-native nbfmm engine (libnbfmm_gb300.so).
 *
 * Drop-in for the hot path of emfomy/nbfmm: nbfmm::Solver (include/nbfmm/core/solver.hpp) and the update
 * path of nbfmm::Stars (include/nbfmm/display/stars.hpp). All pointers named gpuptr_* are device pointers
 * in the reference's layouts: positions and effects are float2 arrays given as float* of 2*n floats,
 * weights are float arrays of n floats, limits are {x_min, y_min, x_max, y_max} (the reference's float4).
 * Streams are cudaStream_t passed as void* (NULL = legacy default stream). Every call returns NBFMM_OK or
 * an error code and leaves a message for nbfmm_last_error(); no call aborts the process. Calls on one
 * handle must not overlap (a handle owns its workspace, as the reference's Solver does).
 */
#ifndef NBFMM_GB300_H_
#define NBFMM_GB300_H_

#ifdef __cplusplus
extern "C" {
#endif

#define NBFMM_GB300_VERSION 1

enum {
  NBFMM_OK = 0,
  NBFMM_ERR_INVALID = 1, /* an argument the reference asserts on (solver.cu:24-27, solve.cu:17, stars.cu:36-43) */
  NBFMM_ERR_CUDA = 2,    /* a CUDA runtime error; the message names the call */
  NBFMM_ERR_NOMEM = 3    /* device memory could not be allocated */
};

typedef struct nbfmm_solver nbfmm_solver;
typedef struct nbfmm_stars nbfmm_stars;

/* Message of the last failed call on this host thread ("" when none). */
const char* nbfmm_last_error(void);
int nbfmm_version(void);

/* ---- Solver ---------------------------------------------------------------------------------------- */

/* nbfmm::Solver::Solver(num_level, max_num_particle, position_limits)  (solver.hpp:80-89, solver.cu:14-46).
 * 0 <= num_level <= 10 (base_dim = 2^(num_level+1)), 1 <= max_num_particle <= 2^28, limits ordered.
 * Allocates the whole workspace; no later call allocates device memory. */
int nbfmm_solver_create(int num_level, int max_num_particle, const float position_limits[4], nbfmm_solver** out);

/* nbfmm::Solver::~Solver  (solver.cu:49-61). NULL is accepted. */
int nbfmm_solver_destroy(nbfmm_solver* solver);

/* Softening of the kernel a = d*m/(|d|^3 + eps); the reference fixes eps = 1e-1
 * (include/nbfmm/core/kernel_function.hpp:35), which is the default here. */
int nbfmm_solver_set_epsilon(nbfmm_solver* solver, float epsilon);

/* Arithmetic of the near field (P2P), per handle. No counterpart in the reference, whose kernelFunction
 * (include/nbfmm/core/kernel_function.hpp:36-39) uses IEEE sqrt and division.
 *   NBFMM_ARITH_FAST (default): hardware square-root and reciprocal approximations and fused multiply-adds, in
 *     the reference's p2pNaive summation order; where leaf cells are small against eps ((2 sqrt(2) cell)^3 / eps
 *     <= 0.0062), part of the reciprocals 1 / (r^3 + eps) are the series (1 / eps)(1 - v + v^2), v = r^3 / eps.
 *     Effects differ from IEEE evaluation in the last bits of each pair, which cancellation can raise above 1e-5
 *     relative on particles whose field nearly cancels.
 *   NBFMM_ARITH_EXACT: every operation of kernelFunction's source rounded once, with correctly rounded sqrt and
 *     division and no fused multiply-add, summed in p2pNaive order (p2p.cu:49-66): the effects round exactly
 *     like the reference's algorithm evaluated in IEEE single precision. Slower near field. */
enum { NBFMM_ARITH_FAST = 0, NBFMM_ARITH_EXACT = 1 };
int nbfmm_solver_set_arithmetic(nbfmm_solver* solver, int arithmetic);

/* nbfmm::Solver::solve(num_particle, position, weight, effect)  (solver.hpp:91-103, solve.cu:11-27).
 * Positions/weights in the caller's order in, effects in the caller's order out; 0 <= n <= max. */
int nbfmm_solver_solve(nbfmm_solver* solver, int num_particle, const float* gpuptr_position_origin,
                       const float* gpuptr_weight_origin, float* gpuptr_effect_origin, void* stream);

/* The stage methods, public in the reference under NBFMM_CHECK (solver.hpp:24-28, 105-209). They run on
 * the solver's own buffers (nbfmm_solver_get_buffers), exactly as the reference's tests drive them. */
int nbfmm_solver_predo(nbfmm_solver* solver, int num_particle, const float* gpuptr_position_origin,
                       const float* gpuptr_weight_origin, void* stream);         /* predo.cu:105-135 */
int nbfmm_solver_p2p(nbfmm_solver* solver, int num_particle, void* stream);     /* p2p.cu:165-176 */
int nbfmm_solver_p2m(nbfmm_solver* solver, int num_particle, void* stream);     /* p2m.cu:79-110 */
int nbfmm_solver_m2m(nbfmm_solver* solver, void* stream);                       /* m2m.cu:58-74 */
int nbfmm_solver_m2l(nbfmm_solver* solver, void* stream);                       /* m2l.cu:63-81 */
int nbfmm_solver_l2l(nbfmm_solver* solver, void* stream);                       /* l2l.cu:39-56 */
int nbfmm_solver_l2p(nbfmm_solver* solver, int num_particle, void* stream);     /* l2p.cu:38-48 */
int nbfmm_solver_postdo(nbfmm_solver* solver, int num_particle, float* gpuptr_effect_origin,
                        void* stream);                                          /* postdo.cu:36-45 */

/* The workspace, the reference's gpuptr_* members (solver.hpp:42-79) in this engine's layout:
 *   particle     float4 [max_num_particle]  sorted x, y, weight, original index (int bits)
 *                                           (gpuptr_position_ + gpuptr_weight_ + gpuptr_perm_)
 *   effect       float2 [max_num_particle]  sorted effects (gpuptr_effect_)
 *   cell_key     uint32 [max_num_particle]  sorted leaf key ix + iy*base_dim (gpuptr_index_)
 *   perm         uint32 [max_num_particle]  sorted -> original index (gpuptr_perm_)
 *   head         int32  [base_dim^2 + 1]    (gpuptr_head_)
 *   cell         float4 [total_cells]       centre of mass x, y, mass, 0 (gpuptr_cell_position_/_weight_)
 *   cell_effect  float2 [total_cells]       (gpuptr_cell_effect_)
 * Cell level l holds level_dim[l]^2 cells, row-major, starting at cell level_offset[l]
 * (the reference's strided cube keeps cell (x,y) of level l at l*B*B + (x + y*B) << l). */
typedef struct {
  int num_level;
  int base_dim;
  int max_num_particle;
  int num_cell_levels;
  int level_dim[11];
  int level_offset[11];
  int total_cells;
  float* particle;
  float* effect;
  unsigned int* cell_key;
  unsigned int* perm;
  int* head;
  float* cell;
  float* cell_effect;
} nbfmm_solver_buffers;

int nbfmm_solver_get_buffers(nbfmm_solver* solver, nbfmm_solver_buffers* out);

/* ---- Stars (the update path) ----------------------------------------------------------------------- */

/* nbfmm::Stars::Stars(fmm_level, num_star, ..., tick, grav_const, ..., position_limits, ...)
 * (stars.hpp:90-98, stars.cu:15-50). The display-only arguments (width, height, fps, size_scale,
 * display_limits) are not part of this path. The effective tick is tick * sqrt(grav_const) (stars.cu:31). */
int nbfmm_stars_create(int fmm_level, int num_star, float tick, float grav_const, const float position_limits[4],
                       nbfmm_stars** out);
int nbfmm_stars_destroy(nbfmm_stars* stars);
int nbfmm_stars_set_epsilon(nbfmm_stars* stars, float epsilon);

/* Near-field arithmetic of the update's solves (nbfmm_solver_set_arithmetic). */
int nbfmm_stars_set_arithmetic(nbfmm_stars* stars, int arithmetic);

/* The public state members (stars.hpp:60-72): gpuptr_position_cur_, gpuptr_position_pre_ (float2 [num_star]),
 * gpuptr_weight_ (float [num_star]). Stars::initialize (stars.hpp:111-114) is the caller writing these. */
int nbfmm_stars_state(nbfmm_stars* stars, float** gpuptr_position_cur, float** gpuptr_position_pre,
                      float** gpuptr_weight);

/* Current number of stars (num_star_, stars.hpp:34). Synchronises with the last update's stream. */
int nbfmm_stars_num_star(nbfmm_stars* stars, int* num_star);

/* num_steps calls of nbfmm::Stars::update() (update.cu:47-55): solve, Stormer-Verlet update, prune.
 * After the call the state arrays hold the surviving stars first, in their previous relative order,
 * followed by the pruned ones, most recently pruned first, as num_steps reference updates leave them.
 * Runs without host synchronisation; the steps are replayed from a captured CUDA graph. */
int nbfmm_stars_update(nbfmm_stars* stars, int num_steps, void* stream);

/* ---- Batched form ----------------------------------------------------------------------------------- */

/* No counterpart in the reference (it steps one system per Stars). Many independent systems stepped together:
 * system s owns particles [particle_offsets[s], particle_offsets[s+1]) of the state arrays, its own limits
 * (position_limits[4s..4s+3]) and tree depth (num_levels[s]); every step of every system is one reference
 * Stars::update of that system alone (solve, Stormer-Verlet, prune). All systems share one sort and one
 * P2P launch per step, and one launch per tree level; a step is replayed from a captured CUDA graph.
 * Tables are host arrays; tick and grav_const are shared (effective tick = tick * sqrt(grav_const)). */
typedef struct nbfmm_batch nbfmm_batch;
int nbfmm_batch_create(int num_systems, const int* particle_offsets, const int* num_levels,
                       const float* position_limits, float tick, float grav_const, nbfmm_batch** out);
int nbfmm_batch_destroy(nbfmm_batch* batch);
int nbfmm_batch_set_epsilon(nbfmm_batch* batch, float epsilon);
int nbfmm_batch_set_arithmetic(nbfmm_batch* batch, int arithmetic); /* nbfmm_solver_set_arithmetic */
/* P2P work-item size per system (host array of num_systems values, 2 or 4 passes of 32 target stars; 4 by
 * default): a tile shape for the autotuner. Results do not depend on it. Takes effect from the next update. */
int nbfmm_batch_set_item_passes(nbfmm_batch* batch, const int* passes_per_item);
/* Device state arrays over all systems (float2 / float2 / float [particle_offsets[num_systems]]). */
int nbfmm_batch_state(nbfmm_batch* batch, float** gpuptr_position_cur, float** gpuptr_position_pre,
                      float** gpuptr_weight);
/* Stars left in each system (host array of num_systems); synchronises. After an update each system's range
 * holds its survivors first, in order, then its pruned stars, most recently pruned first. */
int nbfmm_batch_num_stars(nbfmm_batch* batch, int* num_stars);
int nbfmm_batch_update(nbfmm_batch* batch, int num_steps, void* stream);
int nbfmm_batch_profile_begin(nbfmm_batch* batch, int max_steps);
int nbfmm_batch_profile_end(nbfmm_batch* batch, float* p2p_ms_total, int* p2p_launches);
int nbfmm_batch_kernel_launches(nbfmm_batch* batch, int num_steps, long long* launches);

/* ---- Adjoint --------------------------------------------------------------------------------------- */

/* No counterpart in the reference. Reverse mode of the engine's own approximate method through a
 * Stormer-Verlet trajectory (solve + update.cu:39-40, no pruning inside the trajectory), for the loss
 * L = 0.5 sum_i m_i |x_i(T) - x*_i|^2 with x_{-1} = x_0 - v_0 * tick * sqrt(grav_const). Gradients are taken
 * with the cell assignment of every step held fixed (it is piecewise constant in the positions).
 * Checkpoints every checkpoint_interval steps; the backward pass recomputes each segment from its checkpoint.
 * The weight pointer given to forward must stay valid until backward returns. */
typedef struct nbfmm_adjoint nbfmm_adjoint;
int nbfmm_adjoint_create(int num_level, int num_particle, const float position_limits[4], float tick, float grav_const,
                         int max_steps, int checkpoint_interval, nbfmm_adjoint** out);
int nbfmm_adjoint_destroy(nbfmm_adjoint* adj);
int nbfmm_adjoint_set_epsilon(nbfmm_adjoint* adj, float epsilon);
/* Runs num_steps steps from (x0, v0) with weights m (float2/float2/float [n]); writes x(T). */
int nbfmm_adjoint_forward(nbfmm_adjoint* adj, int num_steps, const float* gpuptr_position0,
                          const float* gpuptr_velocity0, const float* gpuptr_weight, float* gpuptr_position_final,
                          void* stream);
/* dL/dx0, dL/dv0 (float2 [n]) and dL/dm (float [n]) for targets x* (float2 [n]); loss_terms (float [n], may be
 * NULL) receives 0.5 m_i |x_i(T) - x*_i|^2. */
int nbfmm_adjoint_backward(nbfmm_adjoint* adj, const float* gpuptr_target, float* gpuptr_grad_position0,
                           float* gpuptr_grad_velocity0, float* gpuptr_grad_weight, float* gpuptr_loss_terms,
                           void* stream);

/* Stars::prune (prune.cu:28-62) on the public arrays: the stars inside the position limits first, in order, then
 * the others, in order; num_star becomes the number kept. No host synchronisation. */
int nbfmm_stars_prune(nbfmm_stars* stars, void* stream);

/* ---- Frames and the .y4m movie ----------------------------------------------------------------------- */

typedef struct nbfmm_movie nbfmm_movie;

/* Bytes of one YUV 4:2:0 frame, width*height*3/2 (main.cu:234). */
long long nbfmm_frame_bytes(int width, int height);

/* The raster of Stars::display (display.cu:29-221) for any device arrays: clears the frame (Y plane 0, the next
 * width*height/2 bytes 128) and draws stars [0, num_star) of gpuptr_position (float2) and gpuptr_weight inside
 * display_limits {x_min, y_min, x_max, y_max}. gpuptr_board holds nbfmm_frame_bytes(width, height) bytes.
 * The reference's pixels bit for bit, except that writes which would fall outside the frame are dropped (the
 * reference writes before its buffer for stars on the top rows). */
int nbfmm_display(int num_star, int width, int height, float size_scale, const float display_limits[4],
                  const float* gpuptr_position, const float* gpuptr_weight, unsigned char* gpuptr_board,
                  void* stream);

/* Stars::display(board) (display.cu:219-229): the frame of the current stars, then Stars::prune. width, height,
 * size_scale and display_limits are the display arguments of the reference's Stars constructor
 * (stars.hpp:90-92, checked as stars.cu:37-43 asserts them). Use the stream of nbfmm_stars_update. */
int nbfmm_stars_display(nbfmm_stars* stars, int width, int height, float size_scale, const float display_limits[4],
                        unsigned char* gpuptr_board, void* stream);

/* The movie of main.cu:228-259: a .y4m file ("YUV4MPEG2 W H F<fps>:1 Ip A1:1 C420", then "FRAME\n" and the
 * frame per frame) of Stars::display frames. nbfmm_movie_frame displays the stars into the next frame (pruning
 * them, as Stars::display does) and queues its copy to the host on `stream`; the file write of a frame happens
 * in the next nbfmm_movie_frame call, overlapping the GPU work queued in between, or in nbfmm_movie_close. */
int nbfmm_movie_open(nbfmm_stars* stars, const char* path, int width, int height, int fps, float size_scale,
                     const float display_limits[4], nbfmm_movie** out);
int nbfmm_movie_frame(nbfmm_movie* movie, void* stream);
int nbfmm_movie_close(nbfmm_movie* movie);

/* ---- Initial-condition models ---------------------------------------------------------------------- */

/* The reference's generators (include/nbfmm/model/model.hpp:36-233, the files of source/nbfmm/model) with the same
 * arguments: center is {x, y}; cur/prev are float2 [n], w float [n]; tick is the Stars tick (tick * sqrt(G)).
 * Random angles and positions come from curand_init(0, idx, 0) / curand_uniform as in the reference. Calls
 * Stars::initialize makes: func(args..., tick_, cur, prev, w). */
int nbfmm_model_circle_center(int num_particle, const float center[2], float radius, float weight,
                              float center_weight, float tick, float* gpuptr_position_current,
                              float* gpuptr_position_previous, float* gpuptr_weight, void* stream);   /* circle_center.cu:49-70 */
int nbfmm_model_circle_uniform_center(int num_particle, const float center[2], float radius, float weight,
                                      float center_weight, float tick, float* gpuptr_position_current,
                                      float* gpuptr_position_previous, float* gpuptr_weight,
                                      void* stream);                                     /* circle_uniform_center.cu:47-66 */
int nbfmm_model_disk(int num_particle, const float center[2], float radius, float weight, float tick,
                     float* gpuptr_position_current, float* gpuptr_position_previous, float* gpuptr_weight,
                     void* stream);                                                      /* disk.cu:62-81 */
int nbfmm_model_disk_center(int num_particle, const float center[2], float radius, float weight, float center_weight,
                            float tick, float* gpuptr_position_current, float* gpuptr_position_previous,
                            float* gpuptr_weight, void* stream);                         /* disk_center.cu:65-83 */
int nbfmm_model_disk_static(int num_particle, const float center[2], float radius, float weight, float tick,
                            float* gpuptr_position_current, float* gpuptr_position_previous, float* gpuptr_weight,
                            void* stream);                                               /* disk_static.cu:56-74 */
int nbfmm_model_double_disk(int num_particle1, int num_particle2, const float center1[2], const float center2[2],
                            float radius1, float radius2, float weight, float eccentricity, float tick,
                            float* gpuptr_position_current, float* gpuptr_position_previous, float* gpuptr_weight,
                            void* stream);                                               /* double_disk.cu:39-87 */
int nbfmm_model_double_disk_center(int num_particle1, int num_particle2, const float center1[2],
                                   const float center2[2], float radius1, float radius2, float weight,
                                   float center_weight1, float center_weight2, float eccentricity, float tick,
                                   float* gpuptr_position_current, float* gpuptr_position_previous,
                                   float* gpuptr_weight, void* stream);                  /* double_disk_center.cu:39-91 */
int nbfmm_model_rectangle(int num_particle, const float center[2], float width, float height, float max_weight,
                          float tick, float* gpuptr_position_current, float* gpuptr_position_previous,
                          float* gpuptr_weight, void* stream);                           /* rectangle.cu:49-66 */
/* Checking hook (no counterpart in the reference): later model calls on any thread take their draws from this
 * device array (3 floats per particle; the second disk of a double disk continues after the first) instead of
 * curand, so that their arithmetic can be compared with a restatement; NULL restores curand. */
int nbfmm_model_set_uniforms(const float* gpuptr_uniforms);

/* ---- Allocation-free cell sort ---------------------------------------------------------------------- */

/* No counterpart in the reference. The leaf-cell sort of predo (cell keys, stable sort, heads) for callers
 * that cannot allocate device memory: a plugin whose host application owns every device buffer, or code
 * that must not trigger cudaMalloc's device synchronisation. It allocates nothing; its scratch is a fixed
 * device array inside the library (about 4.1 MB per GPU that loads it, held until exit), so at most 262,144
 * particles per call, and calls that overlap on the GPU race on that shared scratch. Every call looks the
 * scratch address up in the current CUDA context (cudaGetSymbolAddress, which neither allocates nor
 * synchronises), so a context the host makes current, or a device reset, is followed; the first call on each
 * device loads the library's module there and should come before any stream capture. A CUDA error pending
 * from earlier work on the calling thread is reported (and cleared) before anything is launched.
 * Outputs: gpuptr_perm [num_particle] = original index of each sorted particle (the reference's
 * gpuptr_perm_), gpuptr_head [base_dim^2 + 1] = first sorted index of each leaf cell (gpuptr_head_). */
int nbfmm_sort_cells_noalloc(int num_level, const float position_limits[4], int num_particle,
                             const float* gpuptr_position, int* gpuptr_perm, int* gpuptr_head, void* stream);

/* ---- Device memory for hosts that link only this library ------------------------------------------- */

/* cudaMalloc, cudaFree and synchronous cudaMemcpy through this library's CUDA runtime, for C hosts (the
 * command-line programs, a cgo or ctypes binding) that do not link the CUDA runtime themselves. The reference's
 * programs call the runtime directly for these (demo.cu:43-45, 69-72, 94-96). */
int nbfmm_device_malloc(unsigned long long bytes, void** gpuptr_out);
int nbfmm_device_free(void* gpuptr);
int nbfmm_memcpy_to_device(void* gpuptr_dst, const void* src, unsigned long long bytes);
int nbfmm_memcpy_to_host(void* dst, const void* gpuptr_src, unsigned long long bytes);

/* ---- Instrumentation (engine-only; the reference has no timing, no events, no counters) ------------ */

/* Times the P2P launch of each of the next `max_steps` update steps with a pair of CUDA events recorded
 * on the update's stream around that launch (the event record nodes of the captured step graph are
 * pointed at a fresh pair per step). */
int nbfmm_stars_profile_begin(nbfmm_stars* stars, int max_steps);

/* Ends the session: total P2P milliseconds and number of timed launches. Synchronises. */
int nbfmm_stars_profile_end(nbfmm_stars* stars, float* p2p_ms_total, int* p2p_launches);

/* Test hook: the next `count` device allocations of the library succeed and every later one fails with
 * NBFMM_ERR_NOMEM (the frame raster then takes its scratch-free path), until called again; count < 0 turns the
 * injection off. Lets tests exercise every allocation failure of the create calls without exhausting a GPU. */
int nbfmm_debug_fail_allocations_after(int count);

/* Number of engine kernels one nbfmm_stars_update(stars, num_steps) call launches. */
int nbfmm_stars_kernel_launches(nbfmm_stars* stars, int num_steps, long long* launches);

#ifdef __cplusplus
}
#endif

#endif /* NBFMM_GB300_H_ */
