// api.cpp -- the C++ drop-in API (include/genoaligner/api.hpp, ext.hpp) over
// the host engine.  Strings are built straight from the pinned output staging
// on the host thread pool; result semantics follow src/api/api.cpp:456-496 and
// 542-580, 843-846 of the reference.
#include <atomic>
#include <cstring>

#include "../../include/genoaligner/api.hpp"
#include "../../include/genoaligner/ext.hpp"
#include "engine.hpp"

namespace genoaligner {

namespace {

BatchResult::Status wfa_status(int32_t st)
{
    return st == GA_INVALID_ARGUMENT ? BatchResult::Status::invalid_argument : BatchResult::Status::device_error;
}

SWBatchResult::Status sw_status(int32_t st)
{
    return st == GA_INVALID_ARGUMENT ? SWBatchResult::Status::invalid_argument : SWBatchResult::Status::device_error;
}

}  // namespace

BatchResult align_batch_ex(const std::vector<AlignRequest>& reqs, const AlignOptions& opt)
{
    BatchResult out;
    const int32_t n = (int32_t)reqs.size();
    out.results.assign(reqs.size(), AlignResult{});
    if (n == 0) return out;
    std::vector<ga_align_request> cr((size_t)n);
    for (int32_t i = 0; i < n; ++i) {
        const AlignRequest& r = reqs[(size_t)i];
        cr[(size_t)i] = ga_align_request{r.pattern, r.pattern_len, r.smax, r.text, r.text_len, r.with_cigar ? 1 : 0};
    }
    std::atomic<int> resolved{0};
    auto fin = [&](int64_t lo, int64_t hi, const ga::WfaView& v) {
        int res = 0;
        for (int64_t i = lo; i < hi; ++i) {
            AlignResult& r = out.results[(size_t)i];
            const int64_t q = i - v.base;           // index in the range's outputs
            r.score = v.score[q];
            r.resolved = r.score >= 0;
            res += r.resolved;
            if (v.trace && r.resolved && v.len[q] > 0) {
                r.cigar.resize((size_t)v.len[q]);
                v.cigar(q, &r.cigar[0]);
                if (v.vflags) {
                    r.rescore_ok = v.vflags[q] & 1;
                    r.wellformed_ok = (v.vflags[q] >> 1) & 1;
                } else {
                    ga::wfa_validate(r.cigar.data(), (int)r.cigar.size(), r.score, reqs[(size_t)i].pattern,
                                     reqs[(size_t)i].pattern_len, reqs[(size_t)i].text, reqs[(size_t)i].text_len,
                                     &r.rescore_ok, &r.wellformed_ok);
                }
            }
        }
        resolved.fetch_add(res);
    };
    const char* err = nullptr;
    const int32_t st = ga::wfa_batch(cr.data(), n, opt.max_smax, opt.learned, fin, &err);
    if (st != GA_OK) {
        out.results.assign(reqs.size(), AlignResult{});
        out.status = wfa_status(st);
        out.error = err;
        return out;
    }
    out.resolved_count = resolved.load();
    out.unresolved_count = n - out.resolved_count;
    return out;
}

BatchResult align_batch(const std::vector<AlignRequest>& reqs)
{
    return align_batch_ex(reqs, AlignOptions{});
}

AlignResult align(const AlignRequest& req)
{
    BatchResult b = align_batch(std::vector<AlignRequest>{req});
    return b.results.empty() ? AlignResult{} : b.results[0];
}

SWBatchResult align_sw_batch_ex(const std::vector<SWRequest>& reqs, const AlignOptions& opt)
{
    SWBatchResult out;
    const int32_t n = (int32_t)reqs.size();
    out.results.assign(reqs.size(), SWAlignResult{});
    if (n == 0) return out;
    std::vector<ga_sw_request> cr((size_t)n);
    for (int32_t i = 0; i < n; ++i) {
        const SWRequest& r = reqs[(size_t)i];
        ga_sw_request q;
        q.text = r.text;
        q.text_len = r.text_len;
        q.with_cigar = r.with_cigar ? 1 : 0;
        q.pattern = r.pattern;
        q.pattern_len = r.pattern_len;
        q.reserved = 0;
        q.scoring = ga_sw_scoring{r.scoring.match, r.scoring.mismatch, r.scoring.gap_open, r.scoring.gap_extend};
        cr[(size_t)i] = q;
    }
    std::atomic<int> resolved{0};
    auto fin = [&](int64_t lo, int64_t hi, const ga::SwView& v) {
        int res = 0;
        for (int64_t i = lo; i < hi; ++i) {
            SWAlignResult& r = out.results[(size_t)i];
            const int64_t q = i - v.base;           // index in the range's outputs
            const int s = v.score[q];
            if (s < 0) {
                if (v.trace) r.too_large = true;
                continue;
            }
            r.score = s;
            r.resolved = true;
            ++res;
            r.end_i = v.pos[4 * q + 2];
            r.end_j = v.pos[4 * q + 3];
            if (s == 0) { r.rescore_ok = r.wellformed_ok = true; continue; }
            if (!v.trace || !reqs[(size_t)i].with_cigar) continue;
            r.start_i = v.pos[4 * q];
            r.start_j = v.pos[4 * q + 1];
            if (v.len[q] > 0) {
                r.cigar.resize((size_t)v.len[q]);
                v.cigar(q, &r.cigar[0]);
                if (v.vflags) {
                    r.rescore_ok = v.vflags[q] & 1;
                    r.wellformed_ok = (v.vflags[q] >> 1) & 1;
                } else {
                    ga::sw_validate(r.cigar.data(), (int)r.cigar.size(), reqs[(size_t)i].text,
                                    reqs[(size_t)i].text_len, r.start_i, r.end_i, reqs[(size_t)i].pattern,
                                    reqs[(size_t)i].pattern_len, r.start_j, r.end_j, cr[(size_t)i].scoring, s,
                                    &r.rescore_ok, &r.wellformed_ok);
                }
            }
        }
        resolved.fetch_add(res);
    };
    const char* err = nullptr;
    const int64_t limit = opt.trace_cell_limit;
    const int32_t st = ga::sw_batch(cr.data(), n, limit, fin, &err);
    if (st != GA_OK) {
        out.results.assign(reqs.size(), SWAlignResult{});
        out.status = sw_status(st);
        out.error = err;
        return out;
    }
    out.resolved_count = resolved.load();
    out.unresolved_count = n - out.resolved_count;
    return out;
}

SWBatchResult align_sw_batch(const std::vector<SWRequest>& reqs)
{
    return align_sw_batch_ex(reqs, AlignOptions{});
}

SWAlignResult align_sw(const SWRequest& req)
{
    SWBatchResult b = align_sw_batch(std::vector<SWRequest>{req});
    return b.results.empty() ? SWAlignResult{} : b.results[0];
}

const char* backend_name() { return ga_backend_name(); }
const char* device_name() { return ga_device_name(); }
bool device_available() { return ga_device_available() != 0; }

}  // namespace genoaligner
