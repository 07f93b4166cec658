// genoaligner/ext.hpp -- extension entries of the GB300 pairwise aligner.
//
// Additive: these have no counterpart in the reference.  They return the same
// result types as align_batch / align_sw_batch and, with default options,
// results identical to them.  They exist for workloads beyond the reference's
// declared limits (smax above 511, SW traceback above 2^26 cells per pair) and
// to switch on learned routing, which never changes a result.
#ifndef GENOALIGNER_EXT_HPP
#define GENOALIGNER_EXT_HPP

#include "genoaligner/api.hpp"

namespace genoaligner {

struct AlignOptions {
    int       max_smax         = 511;                 // accepted smax bound
    bool      learned          = false;               // route by the learned cost model
    long long trace_cell_limit = SW_MAX_TRACE_CELLS;  // SW per-pair trace limit; < 0 = none
};

BatchResult   align_batch_ex(const std::vector<AlignRequest>& reqs, const AlignOptions& opt);
SWBatchResult align_sw_batch_ex(const std::vector<SWRequest>& reqs, const AlignOptions& opt);

}  // namespace genoaligner

#endif  // GENOALIGNER_EXT_HPP
