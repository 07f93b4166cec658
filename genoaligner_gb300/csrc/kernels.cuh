// kernels.cuh -- argument blocks and launchers of the device kernels.
#pragma once

#include "common.cuh"
#include "sw_sizes.cuh"

namespace ga {

struct WfaArgs {
    PairDesc D;              // a = pattern, b = text
    int32_t smax;
    int32_t trace;
    int32_t* out_score;
    int32_t* out_len;
    char* out_cigar;
    int32_t* stack;          // per warp slot: (smax+1)^2 offsets (trace only)
    int64_t stack_slot;
    int32_t* counter;        // next pair index
    int32_t* err;
    int32_t chunk = 1;       // pairs taken per counter increment
};

struct SwArgs {
    PairDesc D;              // a = text (rows), b = pattern (columns)
    const int32_t* work;     // pair indices handled by this launch
    int32_t nwork;
    int32_t match, mismatch, gap_open, gap_extend;
    int32_t* out_score;
    int32_t* out_pos;        // 4 per pair: start_i, start_j, end_i, end_j
    int32_t* out_len;
    char* out_cigar;
    uint32_t* dirs;          // per warp slot, dir_slot words
    int64_t dir_slot;
    int32_t* edge;           // per warp slot, 2 ints per row (band edge H, E)
    int64_t edge_slot;
    int32_t* counter;
    int32_t* err;
    int64_t coop_cells = -1; // sw32ck: items above this many cells run on a whole block (< 0: none)
    const int32_t* nwork_dev = nullptr;   // when set, the item count is read here at launch (device)
    // Sizes read on the device (no plan read back before the launch): when
    // plan is set, list plan_list of the device-built plan (plan_view) gives
    // the items and the per-warp memory, and dir_cap / edge_cap (words of
    // dirs, ints of edge) bound how many blocks run.
    const long long* plan = nullptr;
    int32_t plan_list = 0;
    int64_t dir_cap = 0, edge_cap = 0;
};

// Two pairs per warp in 16-bit lanes (sw16ck.cu): work holds 2 pair indices
// per item, the second -1 when the item carries one pair.
struct Sw16Args {
    PairDesc D;
    const int32_t* work;
    int32_t nwork;
    int32_t match, mismatch, gap_open, gap_extend;
    int32_t* out_score;
    int32_t* out_pos;
    int32_t* out_len;
    char* out_cigar;
    uint32_t* dirs;
    int64_t dir_slot;
    int32_t* edge;
    int64_t edge_slot;
    int32_t* counter;
    int32_t* err;
    int64_t coop_cells = -1; // sw16ck: items above this many cells run on a whole block (< 0: none)
    int32_t ovf_limit = 1 << 30;          // a pair whose best reaches this is handed over ...
    int32_t* esc_list = nullptr;          // ... to the 32-bit kernel: appended here
    int32_t* esc_count = nullptr;
    const long long* plan = nullptr;      // as in SwArgs
    int32_t plan_list = 0;
    int64_t dir_cap = 0, edge_cap = 0;
};

// The learned-bucketed WFA path (wfa_routed.cu).
struct RoutedArgs {
    WfaArgs A;                   // A.smax = the batch smax
    const int2* big;             // warp queue: (pair, smax), one pair per warp
    const int32_t* big_count;    // device-side count
    int32_t* big_next;
    const int2* small;           // lane queue: (pair, first smax), one pair per lane (null: none)
    const int32_t* small_count;
    int32_t* small_next;
    int2* esc;                   // escalations from the lane queue: (pair, batch smax)
    int32_t* esc_count;
    int32_t* esc_next;
    const int32_t* block_count;  // the first *block_count warp-queue items run on whole blocks (null: none)
    int32_t* block_next;
    uint16_t* lane_rec;          // lane kernel: per warp slot, lane_rec_slot() walk records (trace only)
    int32_t warp_smem;           // warp kernel: shared-memory ints per warp
    int32_t group;               // warp kernel: lanes per warp-queue pair (8, 16 or 32; routed_group)
};

// Packs seq into the 2-bit arena `packed` (packed_arena_words(seq_bytes)
// words; null: purity flags only) and sets pure[2n].
cudaError_t launch_pack(const PairDesc& D, int64_t seq_bytes, uint64_t* packed, uint8_t* pure, cudaStream_t st);
int64_t packed_arena_words(int64_t seq_bytes);
cudaError_t launch_pack_arena(const uint8_t* seq, int64_t seq_bytes, uint64_t* packed, uint32_t* bad, cudaStream_t st);
// Sequences copied to the device as the caller laid them out -- one span per
// side, the sides' bytes in request order -- moved into the staging arena: pair
// p's side a from span_a + src_a[p] to seq + a_off[p] (a_len bytes) where
// src_a[p] >= 0, side b likewise; seq is D.seq, writable (wfa.cu).
cudaError_t launch_gather_sides(const PairDesc& D, uint8_t* seq, const uint8_t* span_a, const uint8_t* span_b,
                                const int64_t* src_a, const int64_t* src_b, cudaStream_t st);
// Each pair's CIGAR (end of its slot) packed 2 bits per op at pk + pk_off[p] (wfa.cu).
cudaError_t launch_cigar_pack(const PairDesc& D, const int32_t* len, const char* cig, const int64_t* pk_off,
                              uint8_t* pk, cudaStream_t st);
// WFA result checks on the device (wfa.cu): flags[p] = rescore_ok | wellformed_ok << 1.
cudaError_t launch_wfa_validate(const PairDesc& D, const int32_t* score, const int32_t* len, const char* cig,
                                uint8_t* flags, cudaStream_t st);
// 3-mer sketch features [n][66]; sw: the scaling of the SW variant model.
cudaError_t launch_sketch(const PairDesc& D, float* feat, int32_t* lb, cudaStream_t st, bool sw = false);
cudaError_t launch_mlp_forward(const float* feat, int n, float* y, cudaStream_t st);
bool cost_model_loaded();
bool sw_model_loaded();
void prepare_mlp();
// SW variant routing by the SW model: try16[p] = 1 for pairs the 16-bit
// kernel should try (feat [n][66] and y [n][2] are scratch).
cudaError_t launch_sw_route(const PairDesc& D, int match, int go, float* feat, float* y, uint8_t* try16,
                            cudaStream_t st);
int route_buckets();
// Warp-queue lanes per pair for a batch smax and a tuned group size.
int routed_group(int smax, int group);
int64_t routed_stack_slot(int smax, int group);
int64_t lane_rec_slot();
int routed_warp_smem(int smax, int group);
int routed_max_slots(int smax, bool trace, int sm_count, int group);
int lane_max_slots(bool trace, int sm_count);
// Fused sketch + lower bound + cost model + queue choice (learned.cu); then
// the queues from the per-pair items (wfa_routed.cu).
cudaError_t launch_route_model(const PairDesc& D, int smax, int lane_smax, bool model, int32_t* item, int32_t* lb,
                               float* y, int32_t* counts, int32_t* out_score, int32_t* out_len, cudaStream_t st);
cudaError_t launch_route(int n, const int32_t* item, int32_t* counts, int32_t* starts, int2* big, int2* small,
                         cudaStream_t st);
// The lane kernel over R.small, then the warp kernel over R.big and the
// lane kernel's escalations.
cudaError_t launch_routed(const RoutedArgs& R, int lane_slots, int slots, cudaStream_t st);

size_t wfa_smem_bytes(int smax);
int wfa_max_slots(int smax, bool trace, int sm_count);
cudaError_t launch_wfa(const WfaArgs& A, int slots, cudaStream_t st);

// Score-only 32-bit kernel (sw.cu): SW_SCORE_C columns per lane.
constexpr int SW_SCORE_C = 8;
int sw_max_slots(int sm_count);
cudaError_t launch_sw(const SwArgs& A, int slots, cudaStream_t st);

// Checkpointed traceback kernels (sw16ck.cu: two 16-bit pairs per warp;
// sw32ck.cu: one 32-bit pair per warp); dir_slot = their *_dir_words.
// The device-built work plan (sw_plan.cu).  Lists, in launch order: the
// 16-bit list (sw16ck, or sw16so score-only: two pairs per item), the 32-bit
// list (sw32ck short shape, or sw_kernel score-only) and the 32-bit long-shape
// list (sw32ck long shape; traceback only).  The record `res` (SP_RES long longs):
// per list its pair count, its length in the flattened work array and its
// offset there, the largest per-warp memory of its items (32-bit words), the
// band-edge slot (2 * the longest text), the 16-bit list's largest item
// (larger row count x larger column count of its two pairs), and the pairs
// taken on the optimistic 16-bit rule only: their count and the largest
// per-warp memory the 32-bit long-shape kernel would need for them.
constexpr int SP_LISTS = 3, SP_L16 = 0, SP_L32 = 1, SP_L32LONG = 2;
constexpr int SP_COUNT = 0, SP_INTS = 3, SP_BASE = 6, SP_DIR = 9, SP_EDGE = 12, SP_MAXC16 = 13, SP_NOPT = 14,
              SP_DIROPT = 15, SP_RES = 16;
// plan_list of the launch that takes the pairs the 16-bit kernel hands over
constexpr int SP_ESC = SP_LISTS;

// One launch's view of the plan.  Without a plan: the launch's own fields.
// With one: the list's items (work0 + its base in the flattened lists; the
// hand-over list: work0 itself and the count at nwork_dev), item count and
// per-warp memory from the record, and whether this block runs: blocks past
// dir_cap / (4 * dir_slot) (and edge_cap / (4 * edge_slot)) return at once.
// A list whose one block of 4 warps does not fit runs nowhere and sets
// ERR_SCRATCH.
struct PlanView {
    const int32_t* work;
    int nwork;
    int64_t dir_slot, edge_slot;
    bool run;
};
__device__ __forceinline__ PlanView plan_view(const long long* plan, int list, const int32_t* work0, int nwork0,
                                              const int32_t* nwork_dev, int64_t dir_slot0, int64_t edge_slot0,
                                              int64_t dir_cap, int64_t edge_cap, int32_t* err)
{
    PlanView v{work0, nwork_dev ? *nwork_dev : nwork0, dir_slot0, edge_slot0, true};
    if (!plan) return v;
    if (list == SP_ESC) {
        v.dir_slot = (plan[SP_DIROPT] + 3) / 4 * 4;
    } else {
        const long long ints = plan[SP_INTS + list];
        v.work = work0 + plan[SP_BASE + list];
        v.nwork = (int)(list == SP_L16 ? ints / 2 : ints);
        v.dir_slot = (plan[SP_DIR + list] + 3) / 4 * 4;
    }
    v.edge_slot = plan[SP_EDGE] > 2 ? plan[SP_EDGE] : 2;
    long long blocks = gridDim.x;
    if (v.dir_slot > 0) blocks = min(blocks, (long long)(dir_cap / (4 * v.dir_slot)));
    if (edge_cap > 0) blocks = min(blocks, (long long)(edge_cap / (4 * v.edge_slot)));
    if (blocks < 1 && v.nwork > 0 && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, ERR_SCRATCH);
    v.run = blockIdx.x < blocks;
    return v;
}
struct SwPlanArgs {
    PairDesc D;                  // a = text (rows), b = pattern (columns); D.pure set
    int32_t match, mismatch, gap_open, gap_extend;
    int64_t cell_limit;          // traceback limit in cells, < 0: none
    int32_t use16;               // the 16-bit kernels may be used
    int32_t window;              // sw16ck recompute window, tiles (2 or 4)
    int32_t opt16_pct;           // optimistic 16-bit eligibility (sw16_eligible_opt), 100: the strict bound
    const uint8_t* try16 = nullptr;   // when set: the optimistic rule per pair (the SW model's routing) instead
    int32_t long_log2;           // sw32ck long shape above 2^long_log2 cells
    int32_t too_large_score;     // score written for pairs above cell_limit
    int32_t score_only;          // 1: lists of the score-only kernels (sw16so, sw_kernel)
    int32_t* out_score;
    int32_t* work;               // flattened work lists (2n + 8 ints)
    long long* res;              // the record above
    int32_t *item, *counts, *starts, *sorted;   // scratch, set by launch_sw_plan
};
int64_t sw_plan_scratch_ints(int n);
cudaError_t launch_sw_plan(SwPlanArgs P, int32_t* scratch, cudaStream_t st);
// Result checks of every pair with a CIGAR (sw_plan.cu): flags[p] =
// rescore_ok | wellformed_ok << 1.
struct ga_sw_scoring_t { int32_t match, mismatch, gap_open, gap_extend; };
cudaError_t launch_sw_validate(const PairDesc& D, const ga_sw_scoring_t& sc, const int32_t* score, const int32_t* pos,
                               const int32_t* len, const char* cig, uint8_t* flags, cudaStream_t st);

// sw32ck has a short-pair shape and a long-pair shape (sw32ck_long); sizes
// in sw_sizes.cuh.
int sw32ck_max_slots(bool long_pairs, int sm_count);
cudaError_t launch_sw32ck(const SwArgs& A, bool long_pairs, int slots, cudaStream_t st);
int sw16ck_max_slots(int sm_count, int window);
int sw16so_max_slots(int sm_count);
cudaError_t launch_sw16so(const Sw16Args& A, int slots, cudaStream_t st);
// blocks: the variant with the whole-block phase (items above A.coop_cells)
cudaError_t launch_sw16ck(const Sw16Args& A, int slots, int window, bool blocks, cudaStream_t st);

}  // namespace ga
