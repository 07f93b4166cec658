// ref_wrap.cpp -- host build of the reference's own pairwise kernels.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile against the reference
// sources where they lie (REF_ROOT), with the reference's CPU shim, into
// oracle/_ref/libgaref.so.  Nothing of the reference is copied here: this file
// includes src/api/api.cpp, which pulls in wfa_kernel.hip, wfa_score_flat.hip
// and sw_kernel_impl.hip, and calls those bodies directly the way the
// reference's own parity harnesses do (tests/parity/wfa_parity.cpp:266-319,
// tests/sw/test_sw_trace.cpp:152-190).  It exists to pin oracle/ga_oracle.c and
// to generate tests/golden/ fixtures; it is never part of the product.

#define GENOALIGNER_HIP_SHIM 1
#include "src/api/api.cpp"
#include "src/reference/edit_distance_cpu.hpp"

#include <vector>

using namespace genoaligner;

extern "C" {

// One WFA pair with the API's result semantics.  trace=1 runs wfa_trace_kernel
// and then the decode/validate step of src/api/api.cpp:456-469 (the shim
// branch of align_batch returns every pair unresolved by design, so that step
// is applied here); trace=0 runs wfa_score_kernel_flat at blockDim 1, whose
// interior grid-stride loop then covers every diagonal with one thread.
int ref_wfa_pair(const char* P, int m, const char* T, int n, int smax, int trace,
                 int cigar_cap, char* cigar, int* cigar_len, int* rescore_ok,
                 int* wellformed_ok)
{
    *cigar_len = 0;
    *rescore_ok = 0;
    *wellformed_ok = 0;
    PairView pv{T, n, P, m, smax};
    blockIdx = uint3{0, 0, 0};
    threadIdx = uint3{0, 0, 0};
    blockDim = dim3{1, 1, 1};
    int score = -1;
    if (!trace) {
        shim::smem_vec().assign((size_t)2 * (size_t)(2 * smax + 3), 0);
        wfa_score_kernel_flat(&pv, &score, smax);
        return score;
    }
    const int wf_stride = 2 * smax + 3;
    const int wf_alloc_max = (smax + 1) * wf_stride;
    std::vector<int> ws((size_t)wf_alloc_max, 0), cg((size_t)cigar_cap, 0), meta(4, 0);
    wfa_trace_kernel(&pv, &score, cg.data(), meta.data(), ws.data(), smax, wf_stride,
                     wf_alloc_max, wf_alloc_max * (int)sizeof(int), cigar_cap);
    const int used = meta[1], trunc = meta[2];
    if (score >= 0 && !trunc && used > 0) {
        std::string s = decode_cigar(cg.data(), used);
        bool rs = false, wf = false;
        validate(s, score, P, m, T, n, &rs, &wf);
        std::memcpy(cigar, s.data(), s.size());
        *cigar_len = (int)s.size();
        *rescore_ok = rs ? 1 : 0;
        *wellformed_ok = wf ? 1 : 0;
    }
    return score;
}

int ref_edit_distance(const char* P, int m, const char* T, int n)
{
    return edit_distance_cpu(P, m, T, n);
}

// A whole SW batch through the reference's own align_sw_batch, compiled with
// the shim: the trace path runs sw_trace_kernel per pair, a pure score-only
// batch runs sw_score_kernel under the shim's real-thread warp emulation.
// fields: 9 ints per pair {score, resolved, start_i, start_j, end_i, end_j,
// rescore_ok, wellformed_ok, too_large}.  cigars: pair i written at
// cigars + cig_off[i] with length cig_len[i].  Returns the Status value and the
// error string through *err.
int ref_sw_batch(int n, const char* const* texts, const int* tlens,
                 const char* const* pats, const int* plens,
                 int match, int mismatch, int gap_open, int gap_extend,
                 const unsigned char* with_cigar, int* fields, char* cigars,
                 const long long* cig_off, int* cig_len, const char** err)
{
    std::vector<SWRequest> reqs((size_t)n);
    for (int i = 0; i < n; ++i) {
        SWRequest& r = reqs[(size_t)i];
        r.text = texts[i];
        r.text_len = tlens[i];
        r.pattern = pats[i];
        r.pattern_len = plens[i];
        r.scoring = SWScoring{match, mismatch, gap_open, gap_extend};
        r.with_cigar = with_cigar[i] != 0;
    }
    SWBatchResult b = align_sw_batch(reqs);
    *err = b.error;
    for (int i = 0; i < n && i < (int)b.results.size(); ++i) {
        const SWAlignResult& r = b.results[(size_t)i];
        int* f = fields + (size_t)i * 9;
        f[0] = r.score; f[1] = r.resolved; f[2] = r.start_i; f[3] = r.start_j;
        f[4] = r.end_i; f[5] = r.end_j; f[6] = r.rescore_ok; f[7] = r.wellformed_ok;
        f[8] = r.too_large;
        cig_len[i] = (int)r.cigar.size();
        if (cigars && !r.cigar.empty())
            std::memcpy(cigars + cig_off[i], r.cigar.data(), r.cigar.size());
    }
    return (int)b.status;
}

}  // extern "C"
