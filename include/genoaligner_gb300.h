/*
 * genoaligner_gb300.h -- C ABI of the GB300-native batched pairwise aligner.
 *
 * This is the drop-in boundary for the reference's pairwise API
 * (include/genoaligner/api.hpp of alrobles/genoaligner).  Plain C: pointers,
 * sizes and fixed-layout structs only, so any FFI (ctypes, cgo, JNI, N-API)
 * can bind it.  The C++ API in include/genoaligner/api.hpp is implemented on
 * top of the same engine and keeps the reference's declarations.
 *
 * Conventions, shared by every entry point:
 *   - status codes map 1:1 onto the reference's Status enums
 *     (api.hpp:158, 306): GA_OK, GA_INVALID_ARGUMENT, GA_DEVICE_ERROR;
 *   - error strings are static, non-NULL iff status != GA_OK (api.hpp:160);
 *   - invalid_argument is decided before any device work and fails the whole
 *     batch; on device_error every result is reset to its defaults and both
 *     counters are 0 (src/api/api.cpp:331-339, 724-732);
 *   - inputs are borrowed for the duration of the call; outputs go to
 *     caller-owned arrays; nothing is retained;
 *   - concurrent calls on disjoint inputs are safe: each call runs on its own
 *     CUDA stream with its own buffers.
 */
#ifndef GENOALIGNER_GB300_H
#define GENOALIGNER_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GA_OK               0
#define GA_INVALID_ARGUMENT 1
#define GA_DEVICE_ERROR     2

/* Largest smax the drop-in entry accepts (src/api/api.cpp:227). */
#define GA_MAX_SMAX 511
/* Largest smax the extension and device-resident WFA entries accept: one
 * warp's wavefronts (2 * (2 smax + 3) offsets) must fit the shared memory of
 * a block of four warps. */
#define GA_MAX_SMAX_DEVICE 3500
/* Per-pair direction-table limit of the drop-in SW entry, in cells
 * (include/genoaligner/api.hpp:256). */
#define GA_SW_MAX_TRACE_CELLS (1 << 26)

/* ------------------------------------------------------------------ WFA -- */

/* One pair to align; mirrors genoaligner::AlignRequest (api.hpp:81-88). */
typedef struct ga_align_request {
    const char* pattern;
    int32_t     pattern_len;
    int32_t     smax;          /* max edit distance searched (reference default 64) */
    const char* text;
    int32_t     text_len;
    int32_t     with_cigar;    /* 0 = score only */
} ga_align_request;

/* Result of one pair; mirrors genoaligner::AlignResult (api.hpp:64-76).  The
 * CIGAR (one char per op over M,X,I,D) is cigar_buf[cigar_offset ..
 * cigar_offset + cigar_len). */
typedef struct ga_align_result {
    int32_t score;             /* edit distance; -1 = unresolved (distance > smax) */
    int32_t resolved;
    int32_t rescore_ok;
    int32_t wellformed_ok;
    int64_t cigar_offset;
    int32_t cigar_len;
    int32_t reserved;
} ga_align_result;

/* Batch outcome; mirrors the counters and status of BatchResult
 * (api.hpp:148-163) and SWBatchResult (api.hpp:301-311). */
typedef struct ga_batch_info {
    int32_t     status;
    int32_t     resolved_count;
    int32_t     unresolved_count;
    int32_t     reserved;
    const char* error;
} ga_batch_info;

/* Bytes of CIGAR storage a batch needs: sum over requests of
 * pattern_len + text_len (negative lengths count as 0). */
int64_t ga_align_cigar_bytes(const ga_align_request* reqs, int32_t n);

/* Replaces genoaligner::align_batch (api.hpp:164, src/api/api.cpp:234-497).
 * One smax for the whole batch, the minimum over the requests; smax outside
 * [0, 511] fails the batch; any with_cigar request puts every resolved pair on
 * the CIGAR path.  results[n]; cigar_buf of ga_align_cigar_bytes() bytes (may
 * be NULL when no request has with_cigar).  Returns the status. */
int32_t ga_align_batch(const ga_align_request* reqs, int32_t n, ga_align_result* results,
                       char* cigar_buf, int64_t cigar_buf_bytes, ga_batch_info* info);

/* ------------------------------------------------------------------- SW -- */

/* Affine scheme; mirrors genoaligner::SWScoring (api.hpp:246-251). */
typedef struct ga_sw_scoring {
    int32_t match;
    int32_t mismatch;
    int32_t gap_open;
    int32_t gap_extend;
} ga_sw_scoring;

/* One pair to locally align; mirrors genoaligner::SWRequest (api.hpp:261-268).
 * text is the row axis, pattern the column axis. */
typedef struct ga_sw_request {
    const char*   text;
    int32_t       text_len;
    int32_t       with_cigar;
    const char*   pattern;
    int32_t       pattern_len;
    int32_t       reserved;
    ga_sw_scoring scoring;
} ga_sw_request;

/* Result of one pair; mirrors genoaligner::SWAlignResult (api.hpp:273-294). */
typedef struct ga_sw_result {
    int32_t score;             /* >= 0 when resolved; -1 when not computed */
    int32_t resolved;
    int32_t start_i, start_j;  /* 0-based first aligned char of text / pattern */
    int32_t end_i, end_j;      /* 0-based last aligned char */
    int32_t rescore_ok;
    int32_t wellformed_ok;
    int32_t too_large;
    int32_t cigar_len;
    int64_t cigar_offset;
} ga_sw_result;

/* Bytes of CIGAR storage an SW batch needs: sum of text_len + pattern_len. */
int64_t ga_align_sw_cigar_bytes(const ga_sw_request* reqs, int32_t n);

/* Replaces genoaligner::align_sw_batch (api.hpp:312, src/api/api.cpp:584-847).
 * One scoring scheme per batch; any with_cigar request runs the trace path for
 * the batch; a pair whose (text_len+1)(pattern_len+1) exceeds 2^26 comes back
 * too_large.  A score-only batch reports score and end cell only, with the end
 * cell the reference's warp kernel reports. */
int32_t ga_align_sw_batch(const ga_sw_request* reqs, int32_t n, ga_sw_result* results,
                          char* cigar_buf, int64_t cigar_buf_bytes, ga_batch_info* info);

/* ------------------------------------------------------ extension entries -- */

/* Options of the extension entries (include/genoaligner/ext.hpp).  Zero
 * fields take the defaults noted. */
typedef struct ga_options {
    int32_t max_smax;          /* accepted smax bound; 0 = 511 (the drop-in bound);
                                  values above GA_MAX_SMAX_DEVICE count as it */
    int32_t learned;           /* 1 = route pairs by the learned cost model;
                                  2 = the same queues keyed by the exact q-gram
                                  lower bound alone (no network: the ablation
                                  that shows what the model adds) */
    int64_t trace_cell_limit;  /* SW per-pair trace limit in cells; 0 = 2^26, <0 = none */
    int32_t reserved[4];
} ga_options;

/* align_batch with the options above (no reference counterpart: the
 * reference caps smax at 511).  Results identical to ga_align_batch whenever
 * the options are the defaults. */
int32_t ga_align_batch_ex(const ga_align_request* reqs, int32_t n, ga_align_result* results,
                          char* cigar_buf, int64_t cigar_buf_bytes, const ga_options* opt,
                          ga_batch_info* info);

/* align_sw_batch with the options above (no reference counterpart: the
 * reference caps the trace at 2^26 cells per pair). */
int32_t ga_align_sw_batch_ex(const ga_sw_request* reqs, int32_t n, ga_sw_result* results,
                             char* cigar_buf, int64_t cigar_buf_bytes, const ga_options* opt,
                             ga_batch_info* info);

/* -------------------------------------------------- device-resident entry -- */

/* A batch whose sequences already sit in device memory (no reference
 * counterpart; used when the data is produced on the device).  seq is one
 * byte arena; sequence a of pair i is seq[a_off[i] .. a_off[i]+a_len[i]), b
 * likewise.  Every offset must be a multiple of 32 and the arena must extend
 * at least 64 bytes past the last sequence.  For WFA a = pattern, b = text;
 * for SW a = text (rows), b = pattern (columns).  All arrays are device
 * pointers.  out_off[i] is the byte offset of pair i's CIGAR slot in
 * out_cigar (capacity a_len[i] + b_len[i]); the CIGAR is written at the END of
 * the slot: out_cigar[out_off[i] + cap - len .. out_off[i] + cap). */
typedef struct ga_device_batch {
    const uint8_t* seq;
    int64_t        seq_bytes;
    const int64_t* a_off;
    const int32_t* a_len;
    const int64_t* b_off;
    const int32_t* b_len;
    const int64_t* out_off;
    int32_t        n;
    int32_t        reserved;
} ga_device_batch;

/* WFA over a device batch.  out_score[i] (-1 unresolved), out_len[i] (CIGAR
 * length, 0 when trace == 0 or unresolved), out_cigar as above.  Enqueued on
 * `stream` (a cudaStream_t; NULL = this call's own stream, synchronised before
 * return).  Returns a status; `err` gets a static string on failure. */
int32_t ga_wfa_device(const ga_device_batch* batch, int32_t smax, int32_t trace,
                      int32_t* out_score, int32_t* out_len, char* out_cigar,
                      void* stream, const char** err);

/* ga_wfa_device with extension options (opt may be NULL): opt->learned = 1
 * routes pairs by the cost model (loaded with ga_cost_model_set) into two
 * bucketed queues served by persistent kernels (one pair per lane for small
 * predicted distances, one pair per warp otherwise), replayed as one CUDA
 * graph; results are the same as without it. */
int32_t ga_wfa_device_ex(const ga_device_batch* batch, int32_t smax, int32_t trace, const ga_options* opt,
                         int32_t* out_score, int32_t* out_len, char* out_cigar, void* stream,
                         const char** err);

/* Routing record of the calling thread's last learned WFA call: out[0] = pairs
 * in the lane queue (one pair per lane), out[1] = pairs in the warp queue (one
 * pair per warp or per group of lanes), out[2] = pairs the lane queue escalated to the warp queue
 * (unresolved within their first smax, or handed over), out[3] = warp-queue
 * pairs run on a whole block (estimated distance >= 256); out[4..] = 0.  A
 * host batch of 262,144 pairs or more runs in up to 4 ranges: the record is
 * then its last range's.  Synchronises the device. */
int32_t ga_wfa_route_stats(int32_t* out, int32_t max);

/* Queue item of every pair of the calling thread's last learned WFA call
 * (out[n], host memory; n must be that call's pair count): -1 = unresolved
 * by the lower bound without search; otherwise bits 0-7 = the bucket (below
 * 32: the warp queue, keyed by the bit length of the estimated distance; 32 +
 * s: the lane queue with first smax s) and bits 8 and up = the smax the pair
 * is first run with.  Synchronises the device. */
int32_t ga_wfa_route_items(int32_t* out, int32_t n);

/* SW over a device batch, score + end cell + start cell + CIGAR.
 * out_pos[4*i .. 4*i+3] = start_i, start_j, end_i, end_j.  Pairs above
 * trace_cell_limit cells (< 0: no limit) get out_score = -2 (too large).
 * trace = 0 is the score-only form: out_len, out_cigar and batch->out_off
 * may be null, and out_pos holds -1, -1 and the end cell of the reference's
 * score-only kernel (-1, -1 for score 0). */
int32_t ga_sw_device(const ga_device_batch* batch, ga_sw_scoring scoring, int32_t trace,
                     int64_t trace_cell_limit, int32_t* out_score, int32_t* out_pos,
                     int32_t* out_len, char* out_cigar, void* stream, const char** err);

/* ga_sw_device with extension options (opt may be NULL): opt->learned = 1
 * lets the SW variant model (model slot 1, ga_model_select) choose, pair by
 * pair, which pure-ACGT pairs beyond the proven 16-bit bound try the 16-bit
 * two-pairs-per-warp kernel (one whose best reaches the 16-bit limit is
 * recomputed in 32 bits); results are the same as without it.  No reference
 * counterpart. */
int32_t ga_sw_device_ex(const ga_device_batch* batch, ga_sw_scoring scoring, int32_t trace,
                        int64_t trace_cell_limit, const ga_options* opt, int32_t* out_score, int32_t* out_pos,
                        int32_t* out_len, char* out_cigar, void* stream, const char** err);

/* ------------------------------------------------------- learned model -- */

/* The learned cost model (no counterpart in the reference): a k-mer sketch
 * and an MLP 66 -> 128 -> 128 -> 2 that predicts log2(edit distance + 1) and
 * log2(wavefront cells + 1) of a pair.  It only routes work (the smax tried
 * first, the kernel variant, the queue); results never depend on it. */
int32_t ga_cost_model_nparams(void);
/* The model the calling thread's ga_cost_model_set / _get, ga_mlp_* calls act
 * on: 0 = the WFA cost model (routes learned WFA calls), 1 = the SW variant
 * model (the same network trained to predict an SW pair's best score as a
 * fraction of its all-match score; routes ga_sw_device_ex / the SW extension
 * entry with learned = 1).  GA_INVALID_ARGUMENT for any other value. */
int32_t ga_model_select(int32_t which);
/* Features [n][66] of an SW device batch (a = text, b = pattern) for the SW
 * variant model: 3-mer count differences / 64, lengths / 8192. */
int32_t ga_sw_features(const ga_device_batch* batch, float* features, void* stream);
/* Load / read the fp32 parameters of the current device's model (layout: W1
 * [128][66], b1 [128], W2 [128][128], b2 [128], W3 [2][128], b3 [2]). */
int32_t ga_cost_model_set(const float* params, int32_t n);
int32_t ga_cost_model_get(float* params, int32_t n);
/* Features [n][66] and the exact q-gram lower bound of the edit distance of
 * every pair of a device batch (a = pattern, b = text).  Device pointers. */
int32_t ga_wfa_features(const ga_device_batch* batch, float* features, int32_t* lower_bound, void* stream);
/* Inference: y[n][2] from features[n][66] (device pointers), fp32 activations
 * (the training forward pass). */
int32_t ga_mlp_forward(const float* features, int32_t n, float* y, void* stream);
/* The routing forward pass on the tensor cores (mma.sync bf16, fp32
 * accumulate; inputs and activations rounded to bf16 at each multiply). */
int32_t ga_mlp_forward_fast(const float* features, int32_t n, float* y, void* stream);
/* Gradient of the mean squared error over a batch (device features and
 * targets [n][2]) with respect to every parameter, copied to grad_host
 * (ga_cost_model_nparams() floats); loss_host gets the summed squared error. */
int32_t ga_mlp_gradient(const float* features, const float* targets, int32_t n, float* grad_host,
                        float* loss_host);
/* One Adam step on a batch (device pointers); loss_host (optional) gets the
 * batch mean squared error before the step. */
int32_t ga_mlp_train_step(const float* features, const float* targets, int32_t n, float lr,
                          float* loss_host, void* stream);

/* WFA over a device batch, like ga_wfa_device, but without allocating any
 * device memory.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc when they align: an application that
 * has handed all device memory to its own pool allocator, or a latency-bound
 * loop that cannot take cudaMalloc's implicit device-wide synchronisation.
 * The caller passes inputs and outputs exactly as for ga_wfa_device; all
 * scratch (2-bit arena, purity flags, wavefront stacks, work counter) comes
 * from one 16 MiB array in the library's device image, which every GPU that
 * loads this library holds until the process exits.
 *
 * Limit: 256 + 2n + (seq_bytes/32 + 2)*8 + ceil(seq_bytes/64)*8 bytes (each
 * term rounded up to 256; the last is the 2-bit arena's per-32-byte masks of
 * non-ACGT bytes) must fit in 16 MiB, plus, when trace != 0, four wavefront stacks of
 * (smax+1)^2 * 4 bytes; a larger batch is refused with GA_INVALID_ARGUMENT and
 * a message, before any device work.
 *
 * smax above GA_MAX_SMAX_DEVICE, or a negative seq_bytes, is refused with
 * GA_INVALID_ARGUMENT.
 *
 * The first call in a CUDA context (normally: the first call on a device, made
 * with that device current) resolves the array's device address
 * (cudaGetSymbolAddress) and keeps it with the context's id; a call in another
 * context, such as after cudaDeviceReset, resolves it again.  Make the first
 * call before any stream capture.  Every call shares the one array: calls
 * whose work can overlap on the GPU (different streams, or threads that do not
 * order their calls) race on it and must be serialised by the caller.  stream
 * NULL runs on the legacy default stream and synchronises before returning;
 * with a stream the call returns once its work is enqueued, and the caller
 * orders the next call after it. */
int32_t ga_wfa_device_noalloc(const ga_device_batch* batch, int32_t smax, int32_t trace,
                              int32_t* out_score, int32_t* out_len, char* out_cigar,
                              void* stream, const char** err);

/* --------------------------------------------------------------- ingest -- */

/* A FASTA file read into one device-ready arena (no counterpart in the
 * reference, whose reader, include/genoaligner/io/fasta.hpp, returns
 * std::strings; that reader is kept in include/genoaligner/io/fasta.hpp with
 * the same rules).  Record i's sequence (raw bytes, line breaks removed) is
 * arena[offsets[i] .. offsets[i] + lengths[i]); offsets are multiples of 32,
 * padding is zero and the arena ends with 64 spare bytes, so the arena can be
 * uploaded as the `seq` of a ga_device_batch as is.  The arena is pinned host
 * memory when a CUDA device is present (ga_fasta_pinned).  Parsing follows the
 * reference's reader rules; a malformed input fails with GA_INVALID_ARGUMENT
 * and the reference's message and line in *err (valid until the calling
 * thread's next failing ga_fasta call). */
typedef struct ga_fasta ga_fasta;
int32_t        ga_fasta_read(const char* path, ga_fasta** out, const char** err);
int32_t        ga_fasta_parse(const char* data, int64_t bytes, ga_fasta** out, const char** err);
int32_t        ga_fasta_count(const ga_fasta* f);
const char*    ga_fasta_id(const ga_fasta* f, int32_t i);
const char*    ga_fasta_description(const ga_fasta* f, int32_t i);
const uint8_t* ga_fasta_arena(const ga_fasta* f, int64_t* bytes);
const int64_t* ga_fasta_offsets(const ga_fasta* f);
const int32_t* ga_fasta_lengths(const ga_fasta* f);
int32_t        ga_fasta_pinned(const ga_fasta* f);
/* Copy the whole arena to device memory (one host-to-device copy on `stream`;
 * NULL: the default stream, synchronised before return). */
int32_t        ga_fasta_upload(const ga_fasta* f, void* device_arena, void* stream);
void           ga_fasta_free(ga_fasta* f);

/* Device-side 2-bit packing of a byte arena (seq: device, 16-byte aligned;
 * seq_bytes a multiple of 32): for every 32-byte chunk c, packed[c] holds its
 * 32 codes, 2 bits each, first byte lowest (A 0, C 1, G 2, T 3 under
 * ((b >> 1) ^ (b >> 2)) & 3), and bit k of mask[c] is set when byte 32c + k is
 * not one of A, C, G, T (upper case).  The WFA path packs its arena this way. */
int32_t ga_pack_2bit_device(const uint8_t* seq, int64_t seq_bytes, uint64_t* packed, uint32_t* mask,
                            void* stream);

/* The reference's WFA result checks (validate, src/api/api.cpp:84-112) on the
 * device, after ga_wfa_device with trace = 1: flags[i] = rescore_ok |
 * wellformed_ok << 1 for pairs with a CIGAR, 0 for the others.  The host entry
 * ga_align_batch runs the same kernel.  Device pointers. */
int32_t ga_wfa_validate_device(const ga_device_batch* batch, const int32_t* score, const int32_t* len,
                               const char* cigar, uint8_t* flags, void* stream);

/* The reference's SW result checks (sw_validate, src/api/api.cpp:114-156) on
 * the device, after ga_sw_device with trace = 1: flags[i] = rescore_ok |
 * wellformed_ok << 1 for pairs with a CIGAR (the ops consume exactly the
 * reported span, M only on equal bytes and X on unequal ones, and re-score to
 * the reported score), 0 for the others.  Device pointers. */
int32_t ga_sw_validate_device(const ga_device_batch* batch, ga_sw_scoring scoring, const int32_t* score,
                              const int32_t* pos, const int32_t* len, const char* cigar, uint8_t* flags,
                              void* stream);

/* CIGAR post-processing of an SW batch of records against one reference
 * (the per-record checks of the reference's tools/gene_qc.cpp), on the
 * device, after ga_sw_device with trace = 1 (a = record text, b = the
 * reference, read in frame `frame` 0..2; genetic code `code` 1 = standard,
 * 2 = vertebrate mitochondrial).  out[4*i .. 4*i+3] = fs_runs (indel runs
 * whose length is not a multiple of 3), fs_net ((inserted - deleted) mod 3,
 * as -1, 0, +1), stops (stop codons read in reference codons fully paired
 * with contiguous text bases, the span's own terminator excluded), stop_end
 * (1 when that terminator was found); zeros for pairs without a positive
 * score.  All pointers are device pointers; score/pos/len/cigar are
 * ga_sw_device's outputs. */
int32_t ga_sw_qc_device(const ga_device_batch* batch, const int32_t* score, const int32_t* pos,
                        const int32_t* len, const char* cigar, int32_t frame, int32_t code, int32_t* out,
                        void* stream);

/* ------------------------------------------------------------- autotuner -- */

/* How work is laid onto the GPU (no counterpart in the reference).  These
 * settings pick kernel variants, tile widths and lanes per pair, never what is
 * computed: every setting gives the same results.  One setting per device,
 * used by every later call on that device (ga_sw_device, ga_align_sw_batch,
 * the learned WFA path). */
typedef struct ga_tune {
    int32_t sw_pack16;      /* SW traceback, pure-ACGT pairs whose scores fit 16 bits:
                               1 = two pairs per warp in 16-bit halves (inter-sequence),
                               0 = one pair per warp in 32 bits (intra-sequence) */
    int32_t sw_window;      /* 16-bit traceback: tiles of 64 columns recomputed per
                               window of the walk, 2 (16 lanes x 4 columns per tile)
                               or 4 (8 lanes x 8 columns) */
    int32_t sw_long_log2;   /* 32-bit traceback: pairs above 2^sw_long_log2 cells take
                               the 512 x 512 tile shape, the rest 64 x 64; 16 .. 30 */
    int32_t wfa_lane_smax;  /* learned WFA: pairs whose first smax is <= this run one
                               per lane, 32 per warp (0 = none: one pair per warp); 0 .. 31 */
    int32_t sw_coop_log2;   /* SW traceback: work items above 2^sw_coop_log2 cells (a 32-bit
                               long-shape pair, or a 16-bit item of two pairs) run their forward
                               pass on the 4 warps of a block (128 lanes) instead of one warp;
                               16 .. 40 (40: never) */
    int32_t sw_opt16_pct;   /* SW traceback: a pure-ACGT pair whose all-match score scaled by
                               sw_opt16_pct / 100 fits 16 bits runs on the 16-bit kernel; one
                               whose best then reaches the 16-bit limit is recomputed in 32 bits
                               (exact either way).  50 .. 100 (100: only pairs whose all-match
                               score fits) */
    int32_t wfa_group;      /* learned WFA at batch smax <= 128: lanes per warp-queue pair,
                               8 or 16 (32 / wfa_group pairs per warp, stepping through the
                               wavefronts together) or 32 (one pair per warp); larger smax: 32 */
    int32_t reserved[1];
} ga_tune;

/* One timed candidate of an autotuning run. */
typedef struct ga_tune_trial {
    ga_tune tune;
    double  ms;             /* mean device time of one call over the timed repetitions */
} ga_tune_trial;

/* The built-in setting (chosen by this tuner on a GB300). */
int32_t ga_tune_default(ga_tune* out);
/* Read / replace the current device's setting; ga_tune_set refuses values out
 * of range with GA_INVALID_ARGUMENT and keeps the old setting. */
int32_t ga_tune_get(ga_tune* out);
int32_t ga_tune_set(const ga_tune* t);

/* Time candidate settings on an SW traceback batch (arguments and outputs as
 * ga_sw_device with trace = 1) and keep the fastest for the current device.
 * Each candidate runs once untimed, then `reps` timed calls (reps <= 0: 2) on
 * the library's own stream.  Coordinate search: sw_pack16, then sw_window
 * (when pack16 is chosen), then sw_long_log2 (when the batch has pairs above
 * 2^20 cells), then sw_coop_log2 (when it has pairs above 2^24 cells), then
 * sw_opt16_pct (when it has pure pairs whose all-match score passes 16 bits).  chosen (may be NULL) gets the setting kept; trials[0 ..
 * *n_trials) (may be NULL) every candidate timed.  The outputs hold the batch's
 * results on return. */
int32_t ga_autotune_sw(const ga_device_batch* batch, ga_sw_scoring scoring, int64_t trace_cell_limit,
                       int32_t* out_score, int32_t* out_pos, int32_t* out_len, char* out_cigar,
                       int32_t reps, ga_tune* chosen, ga_tune_trial* trials, int32_t max_trials,
                       int32_t* n_trials, const char** err);

/* The same for the learned WFA path (arguments as ga_wfa_device_ex with
 * opt->learned = 1; the cost model must be loaded): candidates for
 * wfa_lane_smax, then (smax <= 128) wfa_group. */
int32_t ga_autotune_wfa(const ga_device_batch* batch, int32_t smax, int32_t trace,
                        int32_t* out_score, int32_t* out_len, char* out_cigar,
                        int32_t reps, ga_tune* chosen, ga_tune_trial* trials, int32_t max_trials,
                        int32_t* n_trials, const char** err);

/* Write every device's stored setting to a text file (one line per device:
 * name, then the seven fields in the order above; files with the first six
 * load with the built-in wfa_group), or load such a file:
 * lines naming the current device's model set its setting.  GA_INVALID_ARGUMENT
 * on an unreadable / malformed file (nothing is changed then). */
int32_t ga_tune_save(const char* path);
int32_t ga_tune_load(const char* path);

/* ------------------------------------------------------------ provenance -- */

/* Mirror backend_name / device_name / device_available (api.hpp:485-487). */
const char* ga_backend_name(void);
const char* ga_device_name(void);
int32_t     ga_device_available(void);

/* Kernel launches this library issued since load (for launch accounting). */
int64_t ga_kernel_launches(void);

/* Bytes the calling thread's last ga_align_batch / ga_align_sw_batch call
 * copied host-to-device and device-to-host. */
void ga_last_transfer_bytes(int64_t* h2d, int64_t* d2h);

/* Per-kernel timing: ga_profile(1) resets the totals and records a CUDA event
 * pair around every launch on its launch stream until ga_profile(0);
 * ga_profile_read returns the summed device milliseconds and the launch count
 * of one kernel id (0 .. 15, names from ga_profile_kernel_name). */
void        ga_profile(int32_t on);
int32_t     ga_profile_read(int32_t kernel_id, double* total_ms, int64_t* launches);
const char* ga_profile_kernel_name(int32_t kernel_id);

/* Integer-pipe throughput of this GPU, in lane-operations per second, from a
 * microbenchmark kernel (variant 0: add + max in plain C; 1: __viaddmax_s32;
 * 2: __vimax3_s32_relu).  The Smith-Waterman roofline is built on it. */
int32_t ga_bench_int_peak(int32_t variant, double* lane_ops_per_s);

/* Test hook: make the next batch call fail at the named host step
 * (1 = device allocation, 2 = host-to-device copy, 3 = kernel launch,
 * 4 = device-to-host copy, 5 = a traceback call's first CIGAR length replaced,
 * after the copy back, by one past its slot; 0 = off).  The call then reports
 * device_error with defaults in every result, as a real failure there would
 * (step 5: the host checks every length against its slot before it writes a
 * CIGAR). */
void ga_debug_fail_next(int32_t step);

#ifdef __cplusplus
}
#endif

#endif /* GENOALIGNER_GB300_H */
