// route.cuh -- the routing rule of the learned WFA path, shared by the fused
// sketch + cost-model kernel (learned.cu) and the queue kernels
// (wfa_routed.cu).
#pragma once

#include "common.cuh"

namespace ga {

// Lane queue: pairs run one per lane, 32 per warp.  Eligible: both sides pure
// ACGT, at most LANE_MAXLEN bases, first smax <= the tuned lane_smax, itself
// at most LANE_SMAX (the lane kernel's shared-memory wavefront bound).
constexpr int LANE_SMAX = 31;
constexpr int LANE_MAXLEN = 256;
// Buckets: keys 0 .. ROUTE_BUCKETS-1 are the warp queue by bit length of the
// predicted distance bound, ROUTE_BUCKETS + s the lane queue with first smax s.
constexpr int ROUTE_BUCKETS = 32;
// Warp-queue items whose bucket key (bit length of the estimated distance) is
// at least BLOCK_BITS -- estimated s >= 256 -- run first, each on a whole
// block of the warp kernel (128 threads over the diagonals of one pair).
constexpr int BLOCK_BITS = 9;

__device__ __forceinline__ int bitlen(unsigned x) { return 32 - __clz(x); }

// First smax of a pair from the cost model's log2(d + 1) and the exact lower
// bound: the prediction with a 25 % + 2 margin, never below the bound.
__device__ __forceinline__ int first_smax(float y, int lb, int smax)
{
    const float dhat = exp2f(fmaxf(y, 0.f)) - 1.f;
    int s = (int)ceilf(dhat * 1.25f + 2.f);
    s = max(s, lb);
    s = max(s, 1);
    return min(s, smax);
}

// Queue item of one pair: -1 when the bound proves it unresolved, else
// (bucket key) | (smax the pair is first run with) << 8.  A warp-queue pair
// runs with the batch smax: the warp kernel stops at s = d whatever its smax,
// so a smaller budget there could only add reruns.
__device__ __forceinline__ int route_item(int m, int n, bool pure_a, bool pure_b, int lb, float y0, int smax,
                                          int lane_smax)
{
    if (m <= 0 || n <= 0) return min(bitlen((unsigned)smax), ROUTE_BUCKETS - 1) | (smax << 8);
    if (lb > smax) return -1;
    const int s = first_smax(y0, lb, smax);
    if (s <= lane_smax && s <= LANE_SMAX && m <= LANE_MAXLEN && n <= LANE_MAXLEN && pure_a && pure_b)
        return (ROUTE_BUCKETS + s) | (s << 8);
    return min(bitlen((unsigned)s), ROUTE_BUCKETS - 1) | (smax << 8);
}

}  // namespace ga
