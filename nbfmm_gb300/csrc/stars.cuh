// stars.cuh -- device counters and launchers of the time-stepping path (stars.cu).
#pragma once

#include "engine.cuh"

namespace nbfmm_gb300 {

// Counters kept in device memory so that a step needs no host round trip and can be replayed from a graph.
struct StepCounters {
  int* num_star;   // public number of stars (num_star_ of the reference's Stars)
  int* n_import;   // stars at the start of the current update call
  int* n_cur;      // stars in the internal state
  int* n_alive;    // live stars after this step's key pass (head[B*B])
  int* step;       // 1-based step index within the call
  int* prune;      // 0 on the first step of a call (its input was pruned by the previous call)
  int* num_steps;  // steps of the current call
  int* resume;     // Stars only: [0] 1 when the call may continue from the state the last update call left,
                   // [1] the stars in that state (see launch_resume_check)
  int* sort_n;     // Stars only: entries the call's export sorts; 0 when it lost no star (identity export)
  int* first_n;    // Stars only: stars the first step of a call sorts in full; 0 when the call continues from the
                   // last call's state, which its first step re-sorts (launch_resume_keys)
};

// The final state of a star filed under its original index ("grave"): a 32-byte record of two float4,
// (x, y, x_prev, y_prev) and (m, fate as int bits, 0, 0), at grave[2 * orig] and grave[2 * orig + 1]. One thread
// writes both halves, so a record scattered by original index fills one DRAM sector instead of three partial
// ones. Fate 0 = alive at the end of the call; k > 0 orders the pruned stars (smaller = pruned later).
__device__ __forceinline__ void file_grave(float4* __restrict__ grave, int orig, float x, float y, float2 prev, float m,
                                           int fate) {
  grave[2 * orig] = make_float4(x, y, prev.x, prev.y);
  grave[2 * orig + 1] = make_float4(m, __int_as_float(fate), 0.0f, 0.0f);
}

__device__ __forceinline__ int grave_fate(const float4* __restrict__ grave, int orig) {
  return __float_as_int(grave[2 * orig + 1].y);
}

void launch_set_int(int* p, int v, cudaStream_t stream);
void launch_import(const StepCounters& sc, const float2* cur, const float2* prev, const float* w, float4* state4,
                   float2* state_prev, int max_n, cudaStream_t stream);
// Clears sc.resume[0] unless the last update call lost no star, num_star is still the count it left
// (sc.resume[1]), and the public arrays still hold, bit for bit, what it exported: its final states, filed in
// `grave` by original index.
void launch_resume_check(const StepCounters& sc, const float2* cur, const float2* prev, const float* w,
                         const float4* grave, int max_n, cudaStream_t stream);
void launch_keys_from_state(const Geometry& g, const StepCounters& sc, const float4* state4, const float2* state_prev,
                            uint32_t dead_key, uint32_t* keys, uint32_t* vals, float4* grave, int max_n,
                            cudaStream_t stream);
void launch_finish_step(const StepCounters& sc, cudaStream_t stream);

// The cell order of a step that continues a call, from the previous step's (stars.cu, "Re-sort of a continuing
// step"): heads, *d_n_alive = head[B*B] and perm, the state slots in the new cell order (each cell's stayers in
// their old order, then its immigrants). The counts are cleared for the next step's P2P epilogue.
struct ResortArrays {
  const int* head_old;   // [num_cells + 1] the previous step's heads (the state's layout)
  const uint32_t* key;   // [state] P2PArgs::next_key
  int* stay;             // [num_cells] P2PArgs::next_stay, zero between steps
  int* imm_cnt;          // [num_cells] P2PArgs::next_imm, zero between steps
  int* imm_next;         // [num_cells] place of each cell's next immigrant
  int* tile_sum;         // [resort_tiles(num_cells)]
  uint32_t* perm;        // [state]
};
int resort_tiles(int num_cells);
// With `gate`, nothing is re-sorted unless *gate is non-zero (the counts are cleared either way).
void launch_resort(const ResortArrays& r, int num_cells, int max_n, int* head, int* d_n_alive, cudaStream_t stream,
                   const int* gate = nullptr);
// The first step of a call that continues from the last call's state (sc.resume[0] set; nothing otherwise): the
// key word and cell counts of the re-sort, which the last call's final step did not leave. The state is in that
// step's cell order, and its sorted copy `sorted4` still holds the positions that step was sorted by, so each
// slot's old cell is the leaf key of sorted4 and its new cell that of state4 (no prune at a call's first step).
void launch_resume_keys(const Geometry& g, const StepCounters& sc, const float4* sorted4, const float4* state4,
                        uint32_t* key_word, int* stay, int* imm_cnt, int max_n, cudaStream_t stream);
// After the last step of an update call: notes a star lost by a step (the last step's P2P epilogue filed every
// remaining star's final state, P2PArgs::grave).
void launch_export_fate(const StepCounters& sc, cudaStream_t stream);
void launch_fate_keys(const StepCounters& sc, const float4* grave, uint32_t* keys, uint32_t* vals, int max_n,
                      cudaStream_t stream);
// Public arrays from the records: entry i = record order[i], or record i where `sort_n` is given and holds 0
// (nothing was sorted: then num_star = n_import). `mark`, if given (the end of an update call), gets
// mark[0] = 1 if the call lost no star (then the export is the identity and the records describe the state)
// and mark[1] = num_star.
void launch_export_gather(const StepCounters& sc, const uint32_t* order, const float4* grave, float2* cur,
                          float2* prev, float* w, int max_n, cudaStream_t stream, int* mark = nullptr,
                          const int* sort_n = nullptr);

// The gather + P2M of a step over `num_cells` leaf cells of any layout (the batched form's global space too): the
// state gathered into cell order with every leaf cell in index order, the order the reference's stable sort of the
// caller's arrays gives (the step's sort keeps the previous cell order instead), and each cell's centre of mass
// summed in that order. scratch holds kOrderScratch * max_n words for cells too large for shared memory.
constexpr int kOrderScratch = 7;
void launch_gather_state_ordered(const int* head, int num_cells, const uint32_t* perm, const float4* state4,
                                 const float2* state_prev, float4* sorted4, float2* sprev, float4* cell0,
                                 uint32_t* scratch, int max_n, cudaStream_t stream);

// Stars::prune on the public arrays (prune.cu:28-62), step 1: n_import = num_star, keys 1 for the stars outside
// the limits and 0 otherwise, vals the identity, and a copy of the arrays into grave records to gather back from.
void launch_prune_keys(const Geometry& g, const StepCounters& sc, const float2* cur, const float2* prev,
                       const float* w, uint32_t* keys, uint32_t* vals, float4* grave, int max_n, cudaStream_t stream);

// Frame raster of Stars::display (display.cu): clears the frame and draws stars [0, n) where n = *d_n, or n_host
// when d_n is null (grid sized for max_n).
void launch_display(const int* d_n, int n_host, int max_n, int width, int height, float size_scale,
                    const float* limits, const float2* pos, const float* w, uint8_t* board, cudaStream_t s);
long long frame_bytes(int width, int height);

}  // namespace nbfmm_gb300
