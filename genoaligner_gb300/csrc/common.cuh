// common.cuh -- shared device definitions for the GB300 pairwise aligner.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

namespace ga {

constexpr unsigned FULL = 0xffffffffu;

// Unreachable wavefront offset and its threshold test.  The reference stores
// INT32_MIN/2 and tests reachability with a margin, because +1 applied to the
// sentinel must still read as unreachable (wfa_kernel.hip:103, 110).
constexpr int WFA_NULL = INT32_MIN / 2;
__device__ __forceinline__ bool wfa_live(int off) { return off > WFA_NULL + 1024; }

// Device error word bits (set by kernels, read by the host after a launch).
enum : int {
    ERR_CIGAR_OVERFLOW = 1,   // a walk produced more ops than its slot holds
    ERR_BAD_INPUT      = 2,   // a descriptor violated the layout contract
    ERR_SCRATCH        = 4,   // a launch's per-warp memory exceeded what it was given
};

// Sequences of pair i: a at seq[a_off[i]], b at seq[b_off[i]]; offsets are
// multiples of 32 so the 2-bit arena can use word = offset / 32.
struct PairDesc {
    const uint8_t* seq;
    const uint64_t* packed;   // 2-bit arena (32 bases per word)
    const uint8_t* pure;      // per sequence: 1 if every byte is A, C, G or T
    const int64_t* a_off;
    const int32_t* a_len;
    const int64_t* b_off;
    const int32_t* b_len;
    const int64_t* out_off;   // CIGAR slot of pair i (capacity a_len + b_len)
    int32_t n;
};

// Symbols BITS wide, little-endian within 64-bit words: symbol p of a
// sequence starting at word W[0] occupies bits [p*BITS, p*BITS+BITS) of the
// stream.  Returns the 64/BITS symbols starting at p.  Reads W[p*BITS/64 + 1],
// so every arena carries one spare word past its last sequence.
template <int BITS>
__device__ __forceinline__ uint64_t fetch_syms(const uint64_t* __restrict__ W, int p)
{
    const unsigned bit = (unsigned)p * BITS;
    const unsigned w = bit >> 6, sh = bit & 63u;
    const uint64_t lo = __ldg(W + w);
    const uint64_t hi = __ldg(W + w + 1);
    return sh ? ((lo >> sh) | (hi << (64u - sh))) : lo;
}

// Length of the run of equal symbols of P from v and T from h, bounded by
// both ends.  One XOR and one find-first-set per 64/BITS symbols.
template <int BITS>
__device__ __forceinline__ int match_run(const uint64_t* __restrict__ P, const uint64_t* __restrict__ T,
                                         int v, int h, int m, int n)
{
    constexpr int SYMS = 64 / BITS;
    int run = 0;
    for (;;) {
        const int lim = min(m - v, n - h);
        if (lim <= 0) break;
        const uint64_t x = fetch_syms<BITS>(P, v) ^ fetch_syms<BITS>(T, h);
        int eq = x ? (__ffsll((long long)x) - 1) / BITS : SYMS;
        eq = min(eq, lim);
        run += eq;
        v += eq;
        h += eq;
        if (eq < SYMS) break;
    }
    return run;
}

// Kernel identities for launch accounting and per-kernel timing.
// (names: ga_profile_kernel_name)
enum KernelId : int {
    K_PACK = 0, K_WFA_SCORE, K_WFA_TRACE, K_WFA_LANE, K_WFA_ROUTED, K_SW_SCORE, K_SW32_TRACE, K_SW16X2_TRACE,
    K_SW16X2_SCORE, K_SWPLAN, K_VALIDATE, K_QC, K_PEAK, K_SKETCH, K_MLP, K_ROUTE, K_COUNT
};

// Streaming multiprocessors of the current device (queried once per device).
int device_sms();
// Resident blocks per SM of `func` at `threads` threads and `smem` bytes of
// dynamic shared memory on the current device, cached per (device, func,
// threads, smem); the function's dynamic shared-memory limit is raised to
// smem first (never lowered).
int blocks_per_sm(const void* func, int threads, size_t smem);

// Host side, around every launch this library makes: counts the launch and,
// while profiling is on, records CUDA events on the launch stream.
void launch_begin(int kernel_id, cudaStream_t st);
void launch_end(int kernel_id, cudaStream_t st);

}  // namespace ga
