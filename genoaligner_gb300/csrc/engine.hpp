// engine.hpp -- internal C++ interface of the host engine (shared by the C ABI
// in engine.cu and the C++ drop-in API in api.cpp).
#pragma once

#include <cstdint>
#include <functional>

#include "../../include/genoaligner_gb300.h"

namespace ga {

// Run fn(lo, hi) over [0, n) in chunks of `grain` on the host thread pool
// (the calling thread participates).
void parallel_for(int64_t n, int64_t grain, const std::function<void(int64_t, int64_t)>& fn);

// CIGARs come back from the device packed, 2 bits per op in op order
// (M 0, X 1, I 2, D 3; op t at bits 2 (t % 4) of byte t / 4), each pair's at
// its own byte offset: expand len ops into dst.
void expand_cigar(const uint8_t* src, int len, char* dst);

// Per-pair outputs of a WFA batch (or of one range of it: the batch's pairs
// base .. base + n - 1), valid during the finish callback, indexed by
// q = i - base.  The CIGAR of pair q has len[q] ops packed at pk + pk_off[q];
// its slot in the caller's buffer ends at cig_base + slot_end[q].
struct WfaView {
    const int32_t* score;
    const int32_t* len;
    const uint8_t* pk;
    const int64_t* pk_off;
    const int64_t* slot_end;
    bool trace;
    const uint8_t* vflags;    // checks done on the device: rescore_ok | wellformed_ok << 1 (null: check on the host)
    int64_t base;
    int64_t cig_base;
    void cigar(int64_t q, char* dst) const { expand_cigar(pk + pk_off[q], len[q], dst); }
};
using WfaFinish = std::function<void(int64_t lo, int64_t hi, const WfaView& v)>;

// The reference's SW request checks, in its order and with its messages
// (src/api/api.cpp:600-616 with sw_scheme_ok :515-536); the WFA ones
// (:246-266) run inside wfa_batch's first pass.
int32_t sw_check(const ga_sw_request* reqs, int32_t n, const char** err);

// The align_batch pipeline: validation, planning, transfer, kernels, and the
// finish callback over every pair (in parallel).  Returns a GA_* status; on
// failure *err is a static string and the callback has not run.
// route: 0 plain, 1 queues by the cost model (plain when none is loaded), 2
// queues by the exact lower bound alone.
int route_mode(int requested);
// cig_cap: bytes of the caller's CIGAR buffer (-1: no buffer); a batch whose
// CIGARs need more fails with GA_INVALID_ARGUMENT after the request checks
// (which come first), before any device work.
int32_t wfa_batch(const ga_align_request* reqs, int32_t n, int32_t max_smax, int route,
                  const WfaFinish& fin, const char** err, int64_t cig_cap = INT64_MAX);

// Per-pair outputs of one range of an SW batch (requests [base, base + n)),
// valid during the finish callback, which gets the batch's own indices: pair i
// reads score[i - base] and so on; its CIGAR has len ops packed at
// pk + pk_off[i - base] and goes to bytes cig_base + e - len .. cig_base + e
// of the caller's CIGAR buffer, e = slot_end[i - base].
struct SwView {
    const int32_t* score;     // -1 = too large
    const int32_t* pos;       // start_i, start_j, end_i, end_j per pair
    const int32_t* len;
    const uint8_t* pk;
    const int64_t* pk_off;
    const int64_t* slot_end;
    bool trace;
    const uint8_t* vflags;    // checks done on the device: rescore_ok | wellformed_ok << 1 (null: check on the host)
    int64_t base;
    int64_t cig_base;
    void cigar(int64_t q, char* dst) const { expand_cigar(pk + pk_off[q], len[q], dst); }
};
using SwFinish = std::function<void(int64_t lo, int64_t hi, const SwView& v)>;

int32_t sw_batch(const ga_sw_request* reqs, int32_t n, int64_t cell_limit, const SwFinish& fin,
                 const char** err, bool learned = false);

// Result checks computed in the library (the reference's validate and
// sw_validate semantics, src/api/api.cpp:84-156).
void wfa_validate(const char* cigar, int len, int score, const char* P, int m, const char* T, int n,
                  bool* rescore_ok, bool* wellformed_ok);
void sw_validate(const char* cigar, int len, const char* T, int m, int si, int ei, const char* P,
                 int n, int sj, int ej, const ga_sw_scoring& sc, int score, bool* rescore_ok,
                 bool* wellformed_ok);

}  // namespace ga
