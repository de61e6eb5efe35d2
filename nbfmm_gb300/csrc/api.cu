// api.cu -- C ABI of the GB300 engine (include/nbfmm_gb300.h): workspace, stage sequencing, the fused
// solve path and the graph-replayed Stars update.
//
// Solve path (solve.cu:11-27 of the reference, reordered so that the far field is ready before P2P and the
// L2P + postdo work rides in the P2P epilogue):
//   keys -> stable radix sort -> head + work list -> gather + P2M -> M2M -> M2L+L2L -> P2P(+L2P+postdo)
// No call allocates device memory after create, and no call synchronises the host except
// nbfmm_stars_num_star and the first nbfmm_stars_update of a handle (graph instantiation).
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "solver.cuh"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

}  // namespace

namespace {
// Allocations still allowed before injected failures begin; -1: no injection (nbfmm_debug_fail_allocations_after).
std::atomic<long> g_alloc_budget{-1};
}  // namespace

// Sets the calling thread's last-error message from another translation unit of the library.
namespace nbfmm_gb300 {

bool injected_alloc_failure() {
  long b = g_alloc_budget.load();
  while (b >= 0) {
    if (b == 0) return true;
    if (g_alloc_budget.compare_exchange_weak(b, b - 1)) return false;
  }
  return false;
}

int api_fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}
}  // namespace nbfmm_gb300

namespace {

int check_solver(nbfmm_solver* h) { return h ? NBFMM_OK : fail(NBFMM_ERR_INVALID, "null solver handle"); }

int check_n(nbfmm_solver* h, int n) {
  if (n < 0 || n > h->max_n) {
    return fail(NBFMM_ERR_INVALID, "num_particle %d outside [0, %d] (solve.cu:17)", n, h->max_n);
  }
  return NBFMM_OK;
}

}  // namespace

int nbfmm_make_solver(int num_level, int max_num_particle, const float* limits, int extra_key_bits, nbfmm_solver** out) {
  if (!out) return fail(NBFMM_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if (num_level < 0 || num_level > kMaxLevels - 1) {
    return fail(NBFMM_ERR_INVALID, "num_level %d outside [0, %d]", num_level, kMaxLevels - 1);
  }
  if (max_num_particle < 1 || max_num_particle > (1 << 28)) {
    return fail(NBFMM_ERR_INVALID, "max_num_particle %d outside [1, 2^28]", max_num_particle);
  }
  if (!limits_ok(limits)) return fail(NBFMM_ERR_INVALID, "position limits must be finite with min < max");
  nbfmm_solver* h = new (std::nothrow) nbfmm_solver();
  if (!h) return fail(NBFMM_ERR_NOMEM, "host allocation failed");
  const int rc = h->init(num_level, max_num_particle, limits, extra_key_bits);
  if (rc != NBFMM_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return NBFMM_OK;
}

namespace {

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

}  // namespace

extern "C" {

const char* nbfmm_last_error(void) { return g_last_error.c_str(); }

int nbfmm_version(void) { return NBFMM_GB300_VERSION; }

int nbfmm_solver_create(int num_level, int max_num_particle, const float position_limits[4], nbfmm_solver** out) {
  return nbfmm_make_solver(num_level, max_num_particle, position_limits, 0, out);
}

int nbfmm_solver_destroy(nbfmm_solver* solver) {
  delete solver;
  return NBFMM_OK;
}

int nbfmm_solver_set_epsilon(nbfmm_solver* solver, float epsilon) {
  NBFMM_TRY(check_solver(solver));
  if (!(epsilon > 0.0f) || !std::isfinite(epsilon)) return fail(NBFMM_ERR_INVALID, "epsilon must be finite and > 0");
  solver->eps = epsilon;
  return NBFMM_OK;
}

int nbfmm_solver_set_arithmetic(nbfmm_solver* solver, int arithmetic) {
  NBFMM_TRY(check_solver(solver));
  if (arithmetic != NBFMM_ARITH_FAST && arithmetic != NBFMM_ARITH_EXACT) {
    return fail(NBFMM_ERR_INVALID, "arithmetic must be NBFMM_ARITH_FAST (0) or NBFMM_ARITH_EXACT (1)");
  }
  solver->exact = arithmetic;
  return NBFMM_OK;
}

int nbfmm_solver_solve(nbfmm_solver* solver, int num_particle, const float* gpuptr_position_origin,
                       const float* gpuptr_weight_origin, float* gpuptr_effect_origin, void* stream) {
  NBFMM_TRY(check_solver(solver));
  NBFMM_TRY(check_n(solver, num_particle));
  if (num_particle > 0 && (!gpuptr_position_origin || !gpuptr_weight_origin || !gpuptr_effect_origin)) {
    return fail(NBFMM_ERR_INVALID, "null device pointer");
  }
  return solver->solve(num_particle, gpuptr_position_origin, gpuptr_weight_origin, gpuptr_effect_origin,
                       as_stream(stream));
}

int nbfmm_solver_predo(nbfmm_solver* solver, int num_particle, const float* gpuptr_position_origin,
                       const float* gpuptr_weight_origin, void* stream) {
  NBFMM_TRY(check_solver(solver));
  NBFMM_TRY(check_n(solver, num_particle));
  if (num_particle > 0 && (!gpuptr_position_origin || !gpuptr_weight_origin)) {
    return fail(NBFMM_ERR_INVALID, "null device pointer");
  }
  solver->predo(num_particle, reinterpret_cast<const float2*>(gpuptr_position_origin), gpuptr_weight_origin,
                as_stream(stream));
  return cuda_check("nbfmm_solver_predo");
}

int nbfmm_solver_p2p(nbfmm_solver* solver, int num_particle, void* stream) {
  NBFMM_TRY(check_solver(solver));
  NBFMM_TRY(check_n(solver, num_particle));
  cudaStream_t s = as_stream(stream);
  launch_worklist(solver->head, solver->num_cells, solver->work, solver->d_work_count(), true, s,
                  solver->item_passes);
  P2PArgs a = solver->p2p_args();
  a.seff = solver->seff;
  launch_p2p(a, kStoreSorted, solver->num_sms, s);
  return cuda_check("nbfmm_solver_p2p");
}

int nbfmm_solver_p2m(nbfmm_solver* solver, int num_particle, void* stream) {
  NBFMM_TRY(check_solver(solver));
  NBFMM_TRY(check_n(solver, num_particle));
  if (solver->geo.num_level <= 0) return NBFMM_OK;  // p2m.cu:80
  launch_p2m(solver->geo, solver->head, solver->sorted4, solver->cell0(), as_stream(stream));
  return cuda_check("nbfmm_solver_p2m");
}

int nbfmm_solver_m2m(nbfmm_solver* solver, void* stream) {
  NBFMM_TRY(check_solver(solver));
  if (solver->geo.num_level <= 1) return NBFMM_OK;  // m2m.cu:60
  launch_m2m(solver->lv, solver->cell4, as_stream(stream));
  return cuda_check("nbfmm_solver_m2m");
}

int nbfmm_solver_m2l(nbfmm_solver* solver, void* stream) {
  NBFMM_TRY(check_solver(solver));
  if (solver->geo.num_level <= 0) return NBFMM_OK;  // m2l.cu:64
  launch_m2l(solver->lv, solver->cell4, solver->ceff, solver->eps, false, as_stream(stream));
  return cuda_check("nbfmm_solver_m2l");
}

int nbfmm_solver_l2l(nbfmm_solver* solver, void* stream) {
  NBFMM_TRY(check_solver(solver));
  if (solver->geo.num_level <= 1) return NBFMM_OK;  // l2l.cu:40
  launch_l2l(solver->lv, solver->ceff, as_stream(stream));
  return cuda_check("nbfmm_solver_l2l");
}

int nbfmm_solver_l2p(nbfmm_solver* solver, int num_particle, void* stream) {
  NBFMM_TRY(check_solver(solver));
  NBFMM_TRY(check_n(solver, num_particle));
  if (solver->geo.num_level <= 0) return NBFMM_OK;  // l2p.cu:39
  cudaStream_t s = as_stream(stream);
  launch_set_int(solver->d_n(), num_particle, s);
  launch_l2p(solver->d_n(), solver->skey, solver->ceff0(), solver->seff, solver->max_n, s);
  return cuda_check("nbfmm_solver_l2p");
}

int nbfmm_solver_postdo(nbfmm_solver* solver, int num_particle, float* gpuptr_effect_origin, void* stream) {
  NBFMM_TRY(check_solver(solver));
  NBFMM_TRY(check_n(solver, num_particle));
  if (num_particle > 0 && !gpuptr_effect_origin) return fail(NBFMM_ERR_INVALID, "null device pointer");
  cudaStream_t s = as_stream(stream);
  launch_set_int(solver->d_n(), num_particle, s);
  launch_postdo(solver->d_n(), solver->perm, solver->seff, reinterpret_cast<float2*>(gpuptr_effect_origin),
                solver->max_n, s);
  return cuda_check("nbfmm_solver_postdo");
}

int nbfmm_solver_get_buffers(nbfmm_solver* solver, nbfmm_solver_buffers* out) {
  NBFMM_TRY(check_solver(solver));
  if (!out) return fail(NBFMM_ERR_INVALID, "null output pointer");
  std::memset(out, 0, sizeof(*out));
  out->num_level = solver->geo.num_level;
  out->base_dim = solver->geo.base_dim;
  out->max_num_particle = solver->max_n;
  out->num_cell_levels = solver->lv.count;
  for (int l = 0; l < solver->lv.count; ++l) {
    out->level_dim[l] = solver->lv.dim[l];
    out->level_offset[l] = solver->lv.offset[l];
  }
  out->total_cells = solver->lv.total;
  out->particle = reinterpret_cast<float*>(solver->sorted4);
  out->effect = reinterpret_cast<float*>(solver->seff);
  out->cell_key = solver->skey;
  out->perm = solver->perm;
  out->head = solver->head;
  out->cell = reinterpret_cast<float*>(solver->cell4);
  out->cell_effect = reinterpret_cast<float*>(solver->ceff);
  return NBFMM_OK;
}

}  // extern "C"

// ---- Stars ---------------------------------------------------------------------------------------------

struct nbfmm_stars {
  nbfmm_solver* solver = nullptr;
  int max_n = 0;
  float tick = 0.0f;  // tick * sqrt(grav_const), stars.cu:31
  // Public state, the reference's layout (stars.hpp:60-72).
  float2* cur = nullptr;
  float2* prev = nullptr;
  float* w = nullptr;
  // Internal state and files by original index.
  float4* state4 = nullptr;
  float2* state_prev = nullptr;
  float2* sprev = nullptr;
  float4* grave = nullptr;  // final states by original index: two float4 per star (stars.cuh file_grave)
  float4* prune_rec = nullptr;  // prune()'s records, same layout
  uint32_t* order_scratch = nullptr;  // gather_state_ordered_kernel's scratch for large cells
  // The re-sort of the steps after a call's first (stars.cuh ResortArrays).
  uint32_t* step_key = nullptr;
  uint32_t* step_perm = nullptr;
  int* head_old = nullptr;
  int* stay = nullptr;
  int* imm_cnt = nullptr;
  int* imm_next = nullptr;
  int* tile_sum = nullptr;
  int* counters = nullptr;
  StepCounters sc{};
  cudaStream_t capture_stream = nullptr;
  // A call's first step sorts the imported (or resumed) state in full; the steps after it re-sort from the
  // previous step's cell order. Each graph has event record nodes around P2P.
  struct StepGraph {
    cudaGraph_t def = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t node_a = nullptr, node_b = nullptr;
    int kernels = 0;
  };
  StepGraph first_step, next_step;
  bool graphs_built = false;
  // The profiling session's events.
  cudaEvent_t cap_a = nullptr, cap_b = nullptr;
  std::vector<cudaEvent_t> prof_events;
  int prof_max = 0, prof_used = 0;

  int init(int fmm_level, int num_star, float tick_scaled, const float* limits) {
    NBFMM_TRY(nbfmm_make_solver(fmm_level, num_star > 0 ? num_star : 1, limits, 1, &solver));
    max_n = num_star > 0 ? num_star : 1;
    tick = tick_scaled;
    const size_t n = (size_t)max_n;
    NBFMM_TRY(dalloc(&cur, n, "position_cur"));
    NBFMM_TRY(dalloc(&prev, n, "position_pre"));
    NBFMM_TRY(dalloc(&w, n, "weight"));
    NBFMM_TRY(dalloc(&state4, n, "state"));
    NBFMM_TRY(dalloc(&state_prev, n, "state prev"));
    NBFMM_TRY(dalloc(&sprev, n, "sorted prev"));
    NBFMM_TRY(dalloc(&grave, 2 * n, "final states"));
    NBFMM_TRY(dalloc(&prune_rec, 2 * n, "prune records"));
    NBFMM_TRY(dalloc(&order_scratch, kOrderScratch * n, "cell order scratch"));
    const size_t cells = (size_t)solver->num_cells;
    NBFMM_TRY(dalloc(&step_key, n, "step keys"));
    NBFMM_TRY(dalloc(&step_perm, n, "step order"));
    NBFMM_TRY(dalloc(&head_old, cells + 1, "previous heads"));
    NBFMM_TRY(dalloc(&stay, cells, "stayers"));
    NBFMM_TRY(dalloc(&imm_cnt, cells, "immigrants"));
    NBFMM_TRY(dalloc(&imm_next, cells, "immigrant places"));
    NBFMM_TRY(dalloc(&tile_sum, (size_t)resort_tiles(solver->num_cells), "re-sort tiles"));
    cudaMemset(imm_cnt, 0, cells * sizeof(int));
    cudaMemset(stay, 0, cells * sizeof(int));
    NBFMM_TRY(dalloc(&counters, 16, "step counters"));
    cudaMemset(cur, 0, n * sizeof(float2));
    cudaMemset(prev, 0, n * sizeof(float2));
    cudaMemset(w, 0, n * sizeof(float));
    cudaMemset(counters, 0, 16 * sizeof(int));
    sc.num_star = counters + 0;
    sc.n_import = counters + 1;
    sc.n_cur = counters + 2;
    sc.n_alive = solver->d_n_alive();
    sc.step = counters + 3;
    sc.prune = counters + 4;
    sc.num_steps = counters + 5;
    sc.resume = counters + 6;  // two ints; 0: the first call imports
    sc.sort_n = counters + 8;
    sc.first_n = counters + 9;
    launch_set_int(sc.num_star, num_star, nullptr);
    if (cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&cap_a) != cudaSuccess || cudaEventCreate(&cap_b) != cudaSuccess) {
      return cuda_check("stream/event create");
    }
    NBFMM_TRY(cuda_check("stars init"));
    return cudaDeviceSynchronize() == cudaSuccess ? NBFMM_OK : cuda_check("stars init sync");
  }

  static void drop(StepGraph& g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.def) cudaGraphDestroy(g.def);
    g = StepGraph{};
  }

  void drop_graph() {
    drop(first_step);
    drop(next_step);
    graphs_built = false;
  }

  void set_events(StepGraph& g, cudaEvent_t a, cudaEvent_t b) {
    cudaGraphExecEventRecordNodeSetEvent(g.exec, g.node_a, a);
    cudaGraphExecEventRecordNodeSetEvent(g.exec, g.node_b, b);
  }

  void drop_profile_events() {
    for (cudaEvent_t e : prof_events) cudaEventDestroy(e);
    prof_events.clear();
    prof_max = prof_used = 0;
  }

  ~nbfmm_stars() {
    drop_graph();
    drop_profile_events();
    if (cap_a) cudaEventDestroy(cap_a);
    if (cap_b) cudaEventDestroy(cap_b);
    if (capture_stream) cudaStreamDestroy(capture_stream);
    dfree(cur); dfree(prev); dfree(w); dfree(state4); dfree(state_prev); dfree(sprev);
    dfree(grave); dfree(prune_rec); dfree(order_scratch); dfree(counters);
    dfree(step_key); dfree(step_perm); dfree(head_old); dfree(stay); dfree(imm_cnt); dfree(imm_next);
    dfree(tile_sum);
    delete solver;
  }

  // One step: the cell order, the work list, gather + P2M, far field, P2P + L2P + Verlet into the state, counters.
  // The steps after a call's first re-sort from the previous step's cell order, whose P2P left the keys and did
  // the prune. A call's first step sorts in full (keys, sort, head) when the call imported its arrays, and
  // re-sorts when it continues from the last call's state: both ways are in its graph, each doing nothing when
  // the resume flag says the other applies.
  void enqueue_step(cudaStream_t s, bool continuing) {
    nbfmm_solver& v = *solver;
    const uint32_t* perm = nullptr;
    if (!continuing) {
      const uint32_t dead = (uint32_t)v.num_cells;
      launch_keys_from_state(v.geo, sc, state4, state_prev, dead, v.keys_a, v.vals_a, grave, max_n, s);
      v.sort(sc.first_n, v.key_bits, s);
      launch_head(v.skey, sc.first_n, v.num_cells, v.head, sc.n_alive, s);
      perm = v.perm;
      launch_resume_keys(v.geo, sc, v.sorted4, state4, step_key, stay, imm_cnt, max_n, s);
      ResortArrays r{head_old, step_key, stay, imm_cnt, imm_next, tile_sum, v.perm};
      launch_resort(r, v.num_cells, max_n, v.head, sc.n_alive, s, sc.resume);
    } else {
      ResortArrays r{head_old, step_key, stay, imm_cnt, imm_next, tile_sum, step_perm};
      launch_resort(r, v.num_cells, max_n, v.head, sc.n_alive, s);
      perm = step_perm;
    }
    launch_worklist(v.head, v.num_cells, v.work, v.d_work_count(), true, s, v.item_passes, nullptr, nullptr, 0,
                    head_old);
    launch_gather_state_ordered(v.head, v.num_cells, perm, state4, state_prev, v.sorted4, sprev, v.cell0(),
                                order_scratch, max_n, s);  // each cell in index order, as the reference sorts
    v.far_field(s);
    P2PArgs a = v.p2p_args();
    a.sprev = sprev;
    a.state4 = state4;
    a.state_prev = state_prev;
    a.tick = tick;
    a.grave = grave;
    a.d_step = sc.step;
    a.d_num_steps = sc.num_steps;
    a.d_sort_n = sc.sort_n;
    a.d_n_import = sc.n_import;
    a.next_key = step_key;
    a.next_stay = stay;
    a.next_imm = imm_cnt;
    a.geo = v.geo;
    a.inv_cell = make_float2(1.0f / v.geo.cell_x, 1.0f / v.geo.cell_y);
    // External records: captured as event record nodes (a plain record is only a capture-ordering marker).
    cudaEventRecordWithFlags(cap_a, s, cudaEventRecordExternal);
    launch_p2p(a, kVerlet, v.num_sms, s);
    cudaEventRecordWithFlags(cap_b, s, cudaEventRecordExternal);
    launch_finish_step(sc, s);
  }

  int build_graph(StepGraph& out, bool continuing) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(capture_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      return cuda_check("cudaStreamBeginCapture");
    }
    enqueue_step(capture_stream, continuing);
    const cudaError_t e = cudaStreamEndCapture(capture_stream, &g);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(NBFMM_ERR_CUDA, "step capture: %s", cudaGetErrorString(e));
    }
    const cudaError_t e2 = cudaGraphInstantiate(&out.exec, g, 0);
    if (e2 != cudaSuccess) {
      cudaGetLastError();
      cudaGraphDestroy(g);
      out.exec = nullptr;
      return fail(NBFMM_ERR_CUDA, "step graph instantiate: %s", cudaGetErrorString(e2));
    }
    out.def = g;
    size_t count = 0;
    cudaGraphGetNodes(g, nullptr, &count);
    std::vector<cudaGraphNode_t> nodes(count);
    cudaGraphGetNodes(g, nodes.data(), &count);
    out.kernels = 0;
    for (cudaGraphNode_t nd : nodes) {
      cudaGraphNodeType type;
      cudaGraphNodeGetType(nd, &type);
      if (type == cudaGraphNodeTypeKernel) ++out.kernels;
      if (type == cudaGraphNodeTypeEventRecord) {
        cudaEvent_t ev = nullptr;
        cudaGraphEventRecordNodeGetEvent(nd, &ev);
        if (ev == cap_a) out.node_a = nd;
        if (ev == cap_b) out.node_b = nd;
      }
    }
    if (!out.node_a || !out.node_b) return fail(NBFMM_ERR_CUDA, "step graph: P2P event nodes not found");
    return cuda_check("step graph inspection");
  }

  int build_graphs() {
    if (graphs_built) return NBFMM_OK;
    const int rc = build_graph(first_step, false);
    const int rc2 = rc == NBFMM_OK ? build_graph(next_step, true) : rc;
    if (rc2 != NBFMM_OK) {
      drop_graph();
      return rc2;
    }
    graphs_built = true;
    return NBFMM_OK;
  }

  // Kernels outside the step graph per update call: import, step count, and the final prune/reorder.
  int sort_passes(int bits) const { return (bits + kRadixMaxBits - 1) / kRadixMaxBits; }
  static int fate_bits(int steps) {
    int bits = 1;
    while ((1 << bits) <= steps + 1) ++bits;
    return bits;
  }

  int update(int steps, cudaStream_t s) {
    if (steps <= 0) return NBFMM_OK;
    NBFMM_TRY(build_graphs());
    nbfmm_solver& v = *solver;
    launch_resume_check(sc, cur, prev, w, grave, max_n, s);
    launch_import(sc, cur, prev, w, state4, state_prev, max_n, s);
    launch_set_int(sc.num_steps, steps, s);
    for (int k = 0; k < steps; ++k) {
      StepGraph& g = k == 0 ? first_step : next_step;
      if (prof_used < prof_max) {  // point the P2P event nodes at this step's pair
        set_events(g, prof_events[2 * prof_used], prof_events[2 * prof_used + 1]);
        ++prof_used;
      } else if (prof_max > 0 && prof_used == prof_max) {
        set_events(first_step, cap_a, cap_b);
        set_events(next_step, cap_a, cap_b);
        ++prof_used;
      }
      if (cudaGraphLaunch(g.exec, s) != cudaSuccess) return cuda_check("cudaGraphLaunch");
    }
    // Final prune and the reference's order: survivors (fate 0) in original order, then the pruned stars,
    // most recent first (fate 1, 2, ...), each group in original order.
    // When the call lost no star (sort_n == 0) the fate keys, the sort and the head run over nothing and the
    // export is the identity.
    launch_export_fate(sc, s);
    launch_fate_keys(sc, grave, v.keys_a, v.vals_a, max_n, s);
    v.sort(sc.sort_n, fate_bits(steps), s);
    launch_head(v.skey, sc.sort_n, 1, v.head, sc.num_star, s);  // head[1] = number of fate-0 stars
    launch_export_gather(sc, v.perm, grave, cur, prev, w, max_n, s, sc.resume, sc.sort_n);
    return cuda_check("nbfmm_stars_update");
  }

  // Stars::prune (prune.cu:28-62) on the public arrays: the one-bit stable sort of prune.cu:60, with the count
  // of kept stars (prune.cu:61) left in the device counter. It keeps its records apart from the final states
  // of the last update call, which the next call compares the public arrays with; a prune that removes stars
  // lowers num_star below that call's count, so the next call imports.
  void prune(cudaStream_t s) {
    nbfmm_solver& v = *solver;
    launch_prune_keys(v.geo, sc, cur, prev, w, v.keys_a, v.vals_a, prune_rec, max_n, s);
    v.sort(sc.n_import, 1, s);
    launch_head(v.skey, sc.n_import, 1, v.head, sc.num_star, s);  // head[1] = number of kept stars
    launch_export_gather(sc, v.perm, prune_rec, cur, prev, w, max_n, s);
  }

  // Stars::display (display.cu:219-229): the frame of the current stars, then prune.
  int display(int width, int height, float size_scale, const float* limits, uint8_t* board, cudaStream_t s) {
    launch_display(sc.num_star, 0, max_n, width, height, size_scale, limits, cur, w, board, s);
    prune(s);
    return cuda_check("nbfmm_stars_display");
  }
};

extern "C" {

int nbfmm_stars_create(int fmm_level, int num_star, float tick, float grav_const, const float position_limits[4],
                       nbfmm_stars** out) {
  if (!out) return fail(NBFMM_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if (num_star < 0) return fail(NBFMM_ERR_INVALID, "num_star must be >= 0 (stars.cu:36)");
  const float tick_scaled = tick * std::sqrt(grav_const);  // stars.cu:31
  if (!(tick_scaled > 0.0f) || !std::isfinite(tick_scaled)) {
    return fail(NBFMM_ERR_INVALID, "tick * sqrt(grav_const) must be finite and > 0 (stars.cu:40)");
  }
  nbfmm_stars* h = new (std::nothrow) nbfmm_stars();
  if (!h) return fail(NBFMM_ERR_NOMEM, "host allocation failed");
  const int rc = h->init(fmm_level, num_star, tick_scaled, position_limits);
  if (rc != NBFMM_OK) {
    delete h;
    return rc;
  }
  *out = h;
  return NBFMM_OK;
}

int nbfmm_stars_destroy(nbfmm_stars* stars) {
  delete stars;
  return NBFMM_OK;
}

int nbfmm_stars_set_epsilon(nbfmm_stars* stars, float epsilon) {
  if (!stars) return fail(NBFMM_ERR_INVALID, "null stars handle");
  stars->drop_graph();  // the graph captured the old value
  return nbfmm_solver_set_epsilon(stars->solver, epsilon);
}

int nbfmm_stars_set_arithmetic(nbfmm_stars* stars, int arithmetic) {
  if (!stars) return fail(NBFMM_ERR_INVALID, "null stars handle");
  NBFMM_TRY(nbfmm_solver_set_arithmetic(stars->solver, arithmetic));
  stars->drop_graph();  // the graph captured the old kernel
  return NBFMM_OK;
}

int nbfmm_stars_state(nbfmm_stars* stars, float** gpuptr_position_cur, float** gpuptr_position_pre,
                      float** gpuptr_weight) {
  if (!stars) return fail(NBFMM_ERR_INVALID, "null stars handle");
  if (gpuptr_position_cur) *gpuptr_position_cur = reinterpret_cast<float*>(stars->cur);
  if (gpuptr_position_pre) *gpuptr_position_pre = reinterpret_cast<float*>(stars->prev);
  if (gpuptr_weight) *gpuptr_weight = stars->w;
  return NBFMM_OK;
}

int nbfmm_stars_num_star(nbfmm_stars* stars, int* num_star) {
  if (!stars || !num_star) return fail(NBFMM_ERR_INVALID, "null argument");
  if (cudaMemcpy(num_star, stars->sc.num_star, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
    return cuda_check("nbfmm_stars_num_star");
  }
  return NBFMM_OK;
}

int nbfmm_stars_update(nbfmm_stars* stars, int num_steps, void* stream) {
  if (!stars) return fail(NBFMM_ERR_INVALID, "null stars handle");
  if (num_steps < 0) return fail(NBFMM_ERR_INVALID, "num_steps must be >= 0");
  return stars->update(num_steps, as_stream(stream));
}

int nbfmm_debug_fail_allocations_after(int count) {
  g_alloc_budget.store(count < 0 ? -1 : count);
  return NBFMM_OK;
}

int nbfmm_device_malloc(unsigned long long bytes, void** gpuptr_out) {
  if (!gpuptr_out) return fail(NBFMM_ERR_INVALID, "null output pointer");
  *gpuptr_out = nullptr;
  if (bytes == 0) return NBFMM_OK;
  if (injected_alloc_failure()) return fail(NBFMM_ERR_NOMEM, "cudaMalloc of %llu bytes: injected failure", bytes);
  if (cudaMalloc(gpuptr_out, (size_t)bytes) != cudaSuccess) {
    cudaGetLastError();
    *gpuptr_out = nullptr;
    return fail(NBFMM_ERR_NOMEM, "cudaMalloc of %llu bytes failed", bytes);
  }
  return NBFMM_OK;
}

int nbfmm_device_free(void* gpuptr) {
  if (gpuptr && cudaFree(gpuptr) != cudaSuccess) return cuda_check("cudaFree");
  return NBFMM_OK;
}

int nbfmm_memcpy_to_device(void* gpuptr_dst, const void* src, unsigned long long bytes) {
  if (bytes == 0) return NBFMM_OK;
  if (!gpuptr_dst || !src) return fail(NBFMM_ERR_INVALID, "null pointer");
  if (cudaMemcpy(gpuptr_dst, src, (size_t)bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    return cuda_check("cudaMemcpy to device");
  }
  return NBFMM_OK;
}

int nbfmm_memcpy_to_host(void* dst, const void* gpuptr_src, unsigned long long bytes) {
  if (bytes == 0) return NBFMM_OK;
  if (!dst || !gpuptr_src) return fail(NBFMM_ERR_INVALID, "null pointer");
  if (cudaMemcpy(dst, gpuptr_src, (size_t)bytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
    return cuda_check("cudaMemcpy to host");
  }
  return NBFMM_OK;
}

int nbfmm_stars_prune(nbfmm_stars* stars, void* stream) {
  if (!stars) return fail(NBFMM_ERR_INVALID, "null stars handle");
  stars->prune(as_stream(stream));
  return cuda_check("nbfmm_stars_prune");
}

int nbfmm_stars_display(nbfmm_stars* stars, int width, int height, float size_scale, const float display_limits[4],
                        uint8_t* gpuptr_board, void* stream) {
  if (!stars) return fail(NBFMM_ERR_INVALID, "null stars handle");
  if (width <= 0 || height <= 0) return fail(NBFMM_ERR_INVALID, "width and height must be > 0 (stars.cu:37-38)");
  if (!(size_scale > 0.0f)) return fail(NBFMM_ERR_INVALID, "size_scale must be > 0 (stars.cu:41)");
  if (!display_limits || !(display_limits[0] < display_limits[2] && display_limits[1] < display_limits[3])) {
    return fail(NBFMM_ERR_INVALID, "display limits must satisfy x_min < x_max, y_min < y_max (stars.cu:43)");
  }
  if (!gpuptr_board) return fail(NBFMM_ERR_INVALID, "null frame pointer");
  return stars->display(width, height, size_scale, display_limits, gpuptr_board, as_stream(stream));
}

int nbfmm_stars_profile_begin(nbfmm_stars* stars, int max_steps) {
  if (!stars) return fail(NBFMM_ERR_INVALID, "null stars handle");
  if (max_steps < 0) return fail(NBFMM_ERR_INVALID, "max_steps must be >= 0");
  NBFMM_TRY(stars->build_graphs());
  stars->drop_profile_events();
  stars->prof_events.resize(2 * (size_t)max_steps, nullptr);
  for (auto& e : stars->prof_events) {
    if (cudaEventCreate(&e) != cudaSuccess) return cuda_check("cudaEventCreate");
  }
  stars->prof_max = max_steps;
  stars->prof_used = 0;
  return NBFMM_OK;
}

int nbfmm_stars_profile_end(nbfmm_stars* stars, float* p2p_ms_total, int* p2p_launches) {
  if (!stars || !p2p_ms_total || !p2p_launches) return fail(NBFMM_ERR_INVALID, "null argument");
  const int used = stars->prof_used < stars->prof_max ? stars->prof_used : stars->prof_max;
  float total = 0.0f;
  for (int k = 0; k < used; ++k) {
    if (cudaEventSynchronize(stars->prof_events[2 * k + 1]) != cudaSuccess) return cuda_check("cudaEventSynchronize");
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, stars->prof_events[2 * k], stars->prof_events[2 * k + 1]) != cudaSuccess) {
      return cuda_check("cudaEventElapsedTime");
    }
    total += ms;
  }
  if (stars->graphs_built) {
    stars->set_events(stars->first_step, stars->cap_a, stars->cap_b);
    stars->set_events(stars->next_step, stars->cap_a, stars->cap_b);
  }
  stars->drop_profile_events();
  *p2p_ms_total = total;
  *p2p_launches = used;
  return cuda_check("nbfmm_stars_profile_end");
}

int nbfmm_stars_kernel_launches(nbfmm_stars* stars, int num_steps, long long* launches) {
  if (!stars || !launches) return fail(NBFMM_ERR_INVALID, "null argument");
  if (num_steps <= 0) {
    *launches = 0;
    return NBFMM_OK;
  }
  NBFMM_TRY(stars->build_graphs());
  const int outside = 3 /* resume check, import, step count */ + 2 /* export fate, fate keys */ +
                      3 * stars->sort_passes(nbfmm_stars::fate_bits(num_steps)) + 1 /* head */ + 1 /* gather */;
  *launches = stars->first_step.kernels + (long long)(num_steps - 1) * stars->next_step.kernels + outside;
  return NBFMM_OK;
}

}  // extern "C"
