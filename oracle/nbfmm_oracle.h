/*
 * nbfmm_oracle.h -- CPU restatement of the nbfmm 2D monopole FMM (TEST INFRASTRUCTURE ONLY).
 *
 * This library is the checker for the GB300 engine: it is linked only by the tests, by
 * __graft_entry__.smoke() and by the CPU-baseline leg of bench.py. The product path never calls it.
 *
 * Every function restates one stage of the reference (emfomy/nbfmm) in plain C, FP32, in the reference's
 * own order of operations, and cites the reference lines it follows. Three reference defects are
 * neutralised rather than replicated (the engine does the same):
 *   A  source/nbfmm/core/solver/predo.cu:49-74  -- head[] tail left unwritten when N % 1024 == 0;
 *                                                 here every head entry is written.
 *   B  source/nbfmm/core/solver/p2m.cu:46-74    -- zero/scatter race in p2mAssigning; here every leaf
 *                                                 cell gets its exact centre of mass.
 *   C  source/nbfmm/core/solver/l2p.cu:47       -- invalid launch for N > 1,048,576 skips L2P; here L2P
 *                                                 always runs.
 * Cell index policy: the reference computes floorf((x - xmin) / cell) without a clamp
 * (predo.cu:37-38); a particle on or beyond the upper limit gets index B (out of range) and the
 * reference's behaviour is undefined. Both the oracle and the engine clamp the index into [0, B-1].
 *
 * Cell arrays use the reference's strided cube layout (solver.cu:35-43, solver.hpp:63-70):
 * level l, cell (x, y) lives at  l*B*B + (x + y*B) << l, with B = 2^(num_level+1).
 */
#ifndef NBFMM_ORACLE_H_
#define NBFMM_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

/* kernelFunction (include/nbfmm/core/kernel_function.hpp:29-40): a = d*m / (|d|^3 + eps), d = src - tgt. */
void orc_kernel_function(float tx, float ty, float sx, float sy, float m, float eps, float* ax, float* ay);

/* Number of base-level cells per side, 2^(num_level+1) (source/nbfmm/core/solver.cu:19). */
int orc_base_dim(int num_level);

/* Leaf cell index of one position (predo.cu:26-39, cell size from predo.cu:112-113), clamped. */
void orc_cell_index(const float limits[4], int base_dim, float x, float y, int* ix, int* iy);

/* predo (predo.cu:105-135): index, stable row-major sort (operator.hpp:107-109), head, permute.
 * index is int2 [n] (sorted), perm [n], head [B*B+1], pos_sorted float2 [n], w_sorted [n]. */
void orc_predo(int n, int num_level, const float limits[4], const float* pos, const float* w,
               int* index, int* perm, int* head, float* pos_sorted, float* w_sorted);

/* p2p in p2pNaive order (p2p.cu:30-69): each target sums its 3x3 leaf cells row by row, in sorted order. */
void orc_p2p_naive(int n, int base_dim, const float* pos, const float* w, const int* index, const int* head,
                   float eps, float* eff);

/* p2p in p2pBlock order (p2p.cu:82-161): 64-wide chunks per row range, tree reduction per chunk. */
void orc_p2p_block(int n, int base_dim, const float* pos, const float* w, const int* index, const int* head,
                   float eps, float* eff);

/* p2m (p2m.cu:79-110, semantics of check/core/solver/p2m.cu:36-46): leaf centre of mass and mass.
 * Writes level 0 of the cube; empty cells get position (0,0), weight 0. */
void orc_p2m(int n, int base_dim, const float* pos, const float* w, const int* head,
             float* cell_pos, float* cell_w);

/* m2m (m2m.cu:22-74): levels 1..L-1 from their four children. Zero mass gives position (0,0). */
void orc_m2m(int num_level, int base_dim, float* cell_pos, float* cell_w);

/* m2l (m2l.cu:24-81): per level, the children of the parent's neighbours minus the 3x3 near cells,
 * evaluated at the target cell's centre of mass. Writes (does not accumulate) cell_eff. */
void orc_m2l(int num_level, int base_dim, const float* cell_pos, const float* cell_w, float eps, float* cell_eff);

/* l2l (l2l.cu:21-56): child effect += parent effect, from level L-2 down to 0. */
void orc_l2l(int num_level, int base_dim, float* cell_eff);

/* l2p (l2p.cu:23-48): particle effect += its leaf cell effect. */
void orc_l2p(int n, int base_dim, const int* index, const float* cell_eff, float* eff);

/* postdo (postdo.cu:22-45): effect_origin[perm[i]] = effect[i]. */
void orc_postdo(int n, const int* perm, const float* eff, float* eff_origin);

/* Full solve (solve.cu:11-27). p2p_block != 0 selects the p2pBlock summation order, which the
 * reference uses for N <= 65535 (p2p.cu:169). Allocates its own workspace. Returns 0 on success. */
int orc_solve(int n, int num_level, const float limits[4], float eps, int p2p_block,
              const float* pos, const float* w, float* eff);

/* The solve for a list of targets (original indices) only: full tree, P2P + L2P for the listed particles
 * (p2pNaive order). eff receives 2 floats per target. Returns 0 on success. */
int orc_solve_targets(int n, int num_level, const float limits[4], float eps, const float* pos, const float* w,
                      const int* targets, int n_targets, float* eff);

/* Stars::prune (prune.cu:28-62): stable partition, stars inside the limits first. Returns the survivors. */
int orc_prune(int n, const float limits[4], float* cur, float* prev, float* w);

/* One Stars::update (update.cu:47-55): solve, Stormer-Verlet (update.cu:26-42), prune (prune.cu:28-62,
 * stable partition of the stars inside the limits). tick_scaled = tick * sqrt(G) (stars.cu:31).
 * acc receives the solve's effects (pre-update order). Returns the new number of stars. */
int orc_stars_update(int n, int num_level, const float limits[4], float eps, int p2p_block, float tick_scaled,
                     float* cur, float* prev, float* w, float* acc);

/* FP64 all-pairs direct sum (demo.cu:59-66 pattern) for the listed targets (all when targets == NULL). */
void orc_direct_f64(int n, const float* pos, const float* w, double eps, const int* targets, int n_targets,
                    double* eff);
/* The same all-pairs direct sum in FP32 with kernelFunction's operations (kernel_function.hpp:36-39), sources in
 * index order: the CPU direct-sum baseline of the benchmark. */
void orc_direct_f32(int n, const float* pos, const float* w, float eps, const int* targets, int n_targets,
                    float* eff);

/* Number of P2P pairs of a sorted system (targets x sources over each 3x3 block, self excluded). */
long long orc_p2p_pairs(int base_dim, const int* head);

/* FP64 trajectory of the approximate method from x_{-1} = x0 - v0 tau, no pruning, with the leaf of every
 * particle at every step given by keys_in (steps x n) or, when keys_in is NULL, computed from the positions
 * with the FP32 cell arithmetic and written to keys_out (may be NULL). Returns 0.5 sum m |x(T) - target|^2. */
double orc_traj_fmm64(int n, int num_level, const float limits[4], double eps, double tau, int steps,
                      const double* x0, const double* v0, const double* m, const int* keys_in, int* keys_out,
                      const double* target, double* xT);

/* Exact all-pairs FP64 dynamics and the exact gradient of the same loss by its adjoint. Returns the loss. */
double orc_traj_direct64_grad(int n, double eps, double tau, int steps, const double* x0, const double* v0,
                              const double* m, const double* target, double* gx0, double* gv0, double* gm);

/* The reference's initial-condition models (the files of source/nbfmm/model) for given uniform draws u (3 per particle;
 * the second disk of a double disk continues after the first). cur/prev float2 [n], w [n]. */
void orc_model_circle(int n, float cx, float cy, float radius, float weight, float center_weight, float tick,
                      int evenly, const float* u, float* cur, float* prev, float* w);
void orc_model_disk(int n, float cx, float cy, float max_radius, float weight, float center_weight, float tick,
                    int center, int statik, const float* u, float* cur, float* prev, float* w);
void orc_model_rectangle(int n, float cx, float cy, float width, float height, float max_weight, const float* u,
                         float* cur, float* prev, float* w);
void orc_model_double_disk(int n1, int n2, float c1x, float c1y, float c2x, float c2y, float r1, float r2,
                           float weight, float cw1, float cw2, float ecc, float tick, int center, const float* u,
                           float* cur, float* prev, float* w);

/* Stars::display without its prune (display.cu:29-229): one YUV 4:2:0 frame of width*height*3/2 bytes.
 * limits are the display limits [x_min, y_min, x_max, y_max]. Writes outside the frame are dropped. */
void orc_display(int n, int width, int height, float size_scale, const float limits[4], const float* pos,
                 const float* w, unsigned char* board);

/* orc_display split over the OpenMP threads (per-thread frames merged by maximum); the same frame. */
void orc_display_threads(int n, int width, int height, float size_scale, const float limits[4], const float* pos,
                         const float* w, unsigned char* board);

/* Number of OpenMP threads the oracle will use. */
int orc_num_threads(void);

#ifdef __cplusplus
}
#endif

#endif /* NBFMM_ORACLE_H_ */
