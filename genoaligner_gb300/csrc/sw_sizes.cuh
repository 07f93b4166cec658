// sw_sizes.cuh -- shapes, eligibility and per-warp memory of the
// Smith-Waterman traceback kernels, shared by the kernels (sw16ck.cu,
// sw32ck.cu), the device planner (sw_plan.cu) and the host.
#pragma once

#include <cmath>
#include <cstdint>

namespace ga {

// ---- 16-bit two-pairs-per-warp kernels --------------------------------------
// Every value is stored as value + BIAS16 so each 16-bit half stays in
// [0, 32767].  A pair qualifies when both sides are pure ACGT and
// match * min(m, n) + BIAS16 + gap_open < 32000, gap_open + gap_extend < BIAS16
// and mismatch + gap_open >= 0 (host-side check; purity comes from the device).
constexpr int BIAS16 = 1024;

__host__ __device__ inline bool sw16_eligible(int m, int n, int match, int mismatch, int go, int ge)
{
    if (m <= 0 || n <= 0) return false;
    if (go + ge >= BIAS16 || mismatch + go < 0 || match + go > 32000) return false;
    const int64_t top = (int64_t)match * (m < n ? m : n) + BIAS16 + go;
    return top < 32000;
}

// Optimistic 16-bit eligibility: the bound above with the all-match score
// scaled by pct / 100 (pct 100: the bound itself).  A pair taken on this
// rule alone may score past 16 bits; the kernel then sees a best value of at
// least sw16_overflow_limit and hands the pair to the 32-bit kernel.
__host__ __device__ inline bool sw16_eligible_opt(int m, int n, int match, int mismatch, int go, int ge, int pct)
{
    if (m <= 0 || n <= 0) return false;
    if (go + ge >= BIAS16 || mismatch + go < 0 || match + go > 32000) return false;
    const int64_t top = (int64_t)match * (m < n ? m : n) * pct / 100 + BIAS16 + go;
    return top < 32000;
}

// The scheme conditions of the 16-bit kernels alone (no score bound): the
// per-pair 16-bit choice of the SW model is taken only under them.
__host__ __device__ inline bool sw16_scheme_ok(int match, int mismatch, int go, int ge)
{
    return go + ge < BIAS16 && mismatch + go >= 0 && match + go <= 32000;
}

// A best value at or above this in the 16-bit forward pass may have passed
// 16 bits somewhere: every cell's value is exact until an H_diag + match
// first wraps, and that H_diag (> 32767 - match) is in the best, so a best
// below the limit proves the whole pass (and the biased windows, values up to
// best + BIAS16 + match) exact.
__host__ __device__ inline int sw16_overflow_limit(int match) { return 32000 - BIAS16 - match; }

// sw16ck.cu: checkpoint rows every CK_K rows, column edges every CK_TW
// columns, recompute windows of `window` tiles of CK_K x CK_TW cells (2 or 4;
// CK_TG is the default).
constexpr int CK_K = 64;
constexpr int CK_TW = 64;
constexpr int CK_TG = 2;
constexpr int CK_C = 16;                 // forward columns per lane, full bands
constexpr int CK_BW = 32 * CK_C;         // forward band width, full bands

__host__ __device__ inline int ck_rows(int M) { return M > 1 ? (M - 1) / CK_K : 0; }

// Forward bands: full bands of CK_BW columns while more than CK_BW columns
// remain, then one band of 32 * CB columns with the smallest CB in
// {2, 4, 8, 16} that reaches column N.
__host__ __device__ inline int ck_last_cb(int rest)
{
    return rest > 8 * 32 ? 16 : (rest > 4 * 32 ? 8 : (rest > 2 * 32 ? 4 : 2));
}
// Columns the forward bands cover (the column extent of the checkpoints).
__host__ __device__ inline int ck_ncol(int N)
{
    const int full = N > 0 ? (N - 1) / CK_BW : 0;
    return full * CK_BW + 32 * ck_last_cb(N - full * CK_BW);
}

// 32-bit words of one warp slot for an item of at most M rows and N columns:
// checkpoint rows, column edges (16-byte aligned end), the window table.
__host__ __device__ inline int64_t sw16ck_dir_words(int M, int N, int window)
{
    const int64_t ncol = ck_ncol(N);
    return 2 * (int64_t)ck_rows(M) * ncol + (2 * (ncol / CK_TW) * (int64_t)M + 3) / 4 * 4 +
           (int64_t)CK_K * window * CK_TW;
}

// Bucket (0..4095, smallest first) of a 16-bit pair of m rows and n columns
// in a list of the two-pairs-per-warp kernels: consecutive entries share a
// warp and run with the larger of their row counts and forward column
// extents, so the key orders by column extent (ck_ncol, in 64-column steps,
// widest first), then by rows (18 buckets per doubling, most first):
// neighbours then have near-equal shapes, not only near-equal cell counts.
// Pairs 1,536 columns wide and more come before all others, by cells (32
// buckets per doubling, largest first), so the longest work starts first and
// whole-block items lead.
__host__ __device__ inline int sw16_shape_key(int m, int n)
{
    const int ncls = ck_ncol(n > 1 ? n : 1) / 64;
    if (ncls >= 24) {
        const float lc = log2f((float)(m > 1 ? m : 1) * (float)(n > 1 ? n : 1));
        const int e = (int)(32.0f * (lc - 20.0f));
        return 1023 - (e < 0 ? 0 : (e > 1023 ? 1023 : e));
    }
    const float lm = log2f((float)(m > 16 ? m : 16) * (1.0f / 16.0f));
    const int mb = (int)(18.0f * lm) < 127 ? (int)(18.0f * lm) : 127;
    return 1024 + (23 - ncls) * 128 + (127 - mb);
}

// 32-bit words of one warp slot of the 16-bit score-only kernel (sw16so in
// sw16ck.cu): per pair and lane the row that last raised the lane's best
// (SO_ROW_WORDS), then the column edges that carry its band boundaries.
constexpr int SO_ROW_WORDS = 2 * 32 * CK_C;
__host__ __device__ inline int64_t sw16so_dir_words(int M, int N)
{
    return SO_ROW_WORDS + (2 * (int64_t)(ck_ncol(N) / CK_TW) * M + 3) / 4 * 4 + 4;
}

// ---- 32-bit one-pair-per-warp checkpointed kernel (sw32ck.cu) ---------------
constexpr int C32_C = 16;                // forward columns per lane, full bands
constexpr int C32_BW = 32 * C32_C;
constexpr int C32_LONG_LOG2 = 24;       // default: the long-pair shape above 2^24 cells
constexpr int C32_COOP_LOG2 = 27;       // default: work items above 2^27 cells run on a whole block
constexpr int C32_MAX_WARPS = 4;        // sw32ck: warps per block

__host__ __device__ inline int c32_rows(int m, int K) { return m > 1 ? (m - 1) / K : 0; }
__host__ __device__ inline int c32_last_cb(int rest) { return rest > 8 * 32 ? 16 : (rest > 4 * 32 ? 8 : 4); }
__host__ __device__ inline int c32_ncol(int n)
{
    const int full = n > 0 ? (n - 1) / C32_BW : 0;
    return full * C32_BW + 32 * c32_last_cb(n - full * C32_BW);
}
// The long-pair shape (512-row blocks, 512-column tiles) for pairs above
// 2^long_log2 cells, the short one (64 x 64) below.
__host__ __device__ inline bool sw32ck_long(int m, int n, int long_log2)
{
    return (int64_t)m * n > ((int64_t)1 << long_log2);
}

// 32-bit words of one warp slot for a pair of m rows and n columns:
// checkpoint rows, column edges, the tile table.
__host__ __device__ inline int64_t sw32ck_dir_words(int m, int n, int long_log2)
{
    const bool lg = sw32ck_long(m, n, long_log2);
    const int K = lg ? 512 : 64, CT = lg ? 16 : 2, TW = 32 * CT, NWT = CT >= 8 ? CT / 8 : 1;
    const int64_t stride = ((int64_t)c32_ncol(n) + TW - 1) / TW * TW;
    return 2 * (int64_t)c32_rows(m, K) * stride + 2 * (stride / TW) * (int64_t)m + (int64_t)(K + 31) * 32 * NWT;
}

}  // namespace ga
