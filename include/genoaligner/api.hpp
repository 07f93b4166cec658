// genoaligner/api.hpp -- pairwise alignment API, GB300-native implementation.
//
// Drop-in for the pairwise part of alrobles/genoaligner's public header
// (include/genoaligner/api.hpp:59-313, 485-487): the same namespace, types,
// field names, defaults and functions, so code written against the reference
// compiles and links against libgenoaligner_gb300.so unchanged.  The
// multiple-sequence part of the reference header (msa_align, MsaRequest, ...)
// is not part of this library.
//
// Contract (identical to the reference):
//   * align_batch: edit distance bounded by smax; one smax per batch, the
//     minimum over the requests; smax outside [0, 511] fails the whole batch
//     with Status::invalid_argument; pairs whose distance exceeds smax come back
//     unresolved (score -1, no CIGAR); if any request asks for a CIGAR, every
//     resolved pair gets one.  CIGARs are one char per op over M, X, I, D; I
//     consumes text, D consumes pattern.
//   * align_sw_batch: affine local alignment {match, mismatch, gap_open,
//     gap_extend}, text = rows, pattern = columns; one scheme per batch; the
//     scheme refusals of the reference apply; a pair whose
//     (text_len+1)*(pattern_len+1) exceeds SW_MAX_TRACE_CELLS reports
//     too_large; score 0 resolves with coordinates -1 and both flags true.
//   * rescore_ok / wellformed_ok are computed by the library from the CIGAR.
//   * status device_error means the device path failed: every result is at its
//     defaults and both counters are 0; error is a static string.
//   * Requests hold pointers; callers keep them alive for the call.  Concurrent
//     calls on disjoint inputs are safe (each call runs on its own stream).
#ifndef GENOALIGNER_API_HPP
#define GENOALIGNER_API_HPP

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace genoaligner {

struct AlignResult {
    int         score    = -1;      // edit distance; -1 = unresolved (distance > smax)
    bool        resolved = false;   // score >= 0
    std::string cigar;              // over {M,X,I,D}; empty when unresolved
    bool        rescore_ok    = false;
    bool        wellformed_ok = false;
};

struct AlignRequest {
    const char* pattern     = nullptr;
    int         pattern_len = 0;
    const char* text        = nullptr;
    int         text_len    = 0;
    int         smax        = 64;     // max edit distance searched
    bool        with_cigar  = true;   // false = score only
};

AlignResult align(const AlignRequest& req);

struct BatchResult {
    std::vector<AlignResult> results;
    int resolved_count   = 0;
    int unresolved_count = 0;

    enum class Status { ok, invalid_argument, device_error };
    Status status = Status::ok;
    const char* error = nullptr;    // static string, non-null iff status != ok

    bool ok() const { return status == Status::ok; }
};
BatchResult align_batch(const std::vector<AlignRequest>& reqs);

struct SWScoring {
    int match      = 2;
    int mismatch   = -3;
    int gap_open   = 5;
    int gap_extend = 2;
};

// Largest direction table a pair may need, in cells ((text_len+1)*(pattern_len+1)).
static constexpr int SW_MAX_TRACE_CELLS = 1 << 26;

struct SWRequest {
    const char* text        = nullptr;   // rows
    int         text_len    = 0;
    const char* pattern     = nullptr;   // columns
    int         pattern_len = 0;
    SWScoring   scoring;
    bool        with_cigar  = true;      // false = score + end coordinate only
};

struct SWAlignResult {
    int         score    = -1;
    bool        resolved = false;
    std::string cigar;
    int         start_i = -1;
    int         start_j = -1;
    int         end_i   = -1;
    int         end_j   = -1;
    bool        rescore_ok    = false;
    bool        wellformed_ok = false;
    bool        too_large = false;
};

struct SWBatchResult {
    std::vector<SWAlignResult> results;
    int resolved_count   = 0;
    int unresolved_count = 0;

    enum class Status { ok, invalid_argument, device_error };
    Status status = Status::ok;
    const char* error = nullptr;

    bool ok() const { return status == Status::ok; }
};
SWBatchResult align_sw_batch(const std::vector<SWRequest>& reqs);
SWAlignResult align_sw(const SWRequest& req);

const char* backend_name();       // "cuda-sm_103a"
const char* device_name();        // device 0 as reported by the runtime, or "none"
bool        device_available();   // false when no CUDA device is visible

}  // namespace genoaligner

#endif  // GENOALIGNER_API_HPP
