// sw16ck.cu -- Smith-Waterman with traceback, two pairs per warp in 16-bit
// lanes: a score-only forward pass that keeps checkpoints, then the walk over
// windows of 64 x 64 tiles recomputed from them.
//
// Same recurrence, tie rules and walk as the reference's (its
// trace recurrence, include/genoaligner/backend/sw_kernel_impl.hip:286-329,
// walk :198-242, best cell = first strict maximum in row-major order).  What
// changes is where the direction bits come from.  Storing four predicate bits
// for every cell costs three integer instructions per bit and 4 bits of HBM
// traffic per cell, while the walk reads a thin path through the matrix.  So:
//
//   1. forward: H, E, F for every cell with DPX 16x2 max-plus instructions
//      (__viaddmax_s16x2, __vimax3_s16x2_relu), no predicates.  Kept on the
//      way: every CK_K-th row, each column's (H - gap_open, F) (checkpoint
//      rows); every TW-th column, each row's (H - gap_open, E) (column
//      edges); per lane the best value with its first row and column;
//   2. the best cell is the warp's (max value, min row, min column);
//   3. walk: the tile [i0, i] x [TW*b + 1, TW*b + TW] holding the walk's
//      current cell (i0 = the first row of its CK_K-row block) and the TG - 1
//      tiles to its left are recomputed from the checkpoint row above them
//      and the column edges left of them -- TG groups of 32 / TG lanes, one
//      tile each, so the lanes' one-step lag costs 32 / TG - 1 steps, not
//      31 -- and their H values are kept; the walk proceeds inside them
//      (runs of diagonal steps 32 at a time), reading every decision
//      off H values with the reference's tie rules (diagonal, then E, then F;
//      a gap cell opened when its neighbour's H - gap_open equals it, E from
//      a warp-wide max over the row); leaving the window at the top or the
//      left, the tiles there are recomputed.  Both pairs of a warp recompute
//      their windows in one pass, each half of a register at its own rows and
//      columns.
//
// Recomputed values equal the forward pass's, so every decision is the one
// the reference's stored direction bits give.  Eligibility (16-bit scores
// proven, or tried with the overflow check) is decided by the plan
// (sw_plan.cu, sw_sizes.cuh).
//
// The score-only form (sw16so_kernel, at the end) runs step 1 alone, without
// checkpoint rows, and picks the end cell by the reference's score-only rule
// (include/genoaligner/backend/sw_kernel_impl.hip:146,158-167) instead of
// step 2.
#include "kernels.cuh"

namespace ga {

constexpr int TW = CK_TW;                // tile width: a group of 32 / TG lanes x TW * TG / 32 columns
constexpr int CK_BIAS = BIAS16;          // value bias of the recompute pass
constexpr int CK_MAX_TG = 4;             // widest recompute window, tiles
// shared memory words per warp: the forward band profile, or the window
// profile (TW * TG / 32 columns per lane) plus the window's column edges
constexpr int CK_LETTERS = 5;           // forward profile rows per pair: A C G T, then the padding row
constexpr int CK_FWD_WORDS = 2 * CK_LETTERS * (CK_C / 2) * 32;
constexpr int CK_WIN_WORDS = 2 * 4 * (TW * CK_MAX_TG / 64) * 32 + 2 * CK_MAX_TG * CK_K;
constexpr int CK_WARP_WORDS = CK_FWD_WORDS > CK_WIN_WORDS ? CK_FWD_WORDS : CK_WIN_WORDS;

__device__ __forceinline__ int ck_code(uint32_t c) { return (int)(((c >> 1) ^ (c >> 2)) & 3u); }
__device__ __forceinline__ int lo16s(uint32_t x) { return (int)(int16_t)(x & 0xffffu); }
__device__ __forceinline__ int hi16s(uint32_t x) { return (int)(int16_t)(x >> 16); }

// The end-cell key of the reference's score-only kernel
// (include/genoaligner/backend/sw_kernel_impl.hip:146, 158-167): among cells
// holding the maximum, the smallest (bit-reversed column class (j mod 32),
// row, column), j 0-based, i 1-based.
__device__ __forceinline__ uint64_t c9_key(int i, int j)
{
    return ((uint64_t)(__brev((unsigned)j & 31u) >> 27) << 58) | ((uint64_t)(i - 1) << 29) | (uint64_t)j;
}
__device__ __forceinline__ uint64_t c9_join(int hi, int lo) { return ((uint64_t)(uint32_t)hi << 32) | (uint32_t)lo; }

// A lane's CB columns j0 + c (CB a power of two, j0 a multiple of CB, bands
// starting at multiples of 32): their key classes brev5(j mod 32) order like
// c with its log2(CB) bits reversed, the rank q9_rank gives; q9_col inverts it.
template <int CB>
__host__ __device__ constexpr int q9_rank(int c)
{
    int r = 0;
    for (int b = 1; b < CB; b <<= 1) { r = (r << 1) | (c & 1); c >>= 1; }
    return r;
}
template <int CB>
__device__ __forceinline__ int q9_col(int rank)
{
    return CB == 1 ? 0 : (int)(__brev((unsigned)rank) >> (32 - __builtin_ctz(CB)));
}

// (value, row, column) order of the best cell: larger value, then smaller row,
// then smaller column.
__device__ __forceinline__ bool ck_better(int v, int r, int c, int bv, int br, int bc)
{
    return v > bv || (v == bv && (r < br || (r == br && c < bc)));
}

// Forward profile of a band at CB columns per lane:
// prof[((pair * 5 + letter) * (CB / 2) + h) * 32 + t] holds the 16-bit scores
// (s + gap_open) of this lane's columns 2h, 2h+1.  Past a pattern's end, and
// in the padding letter 4 (the rows past a pair's text), a score far below any
// reachable value: there H is at most the best of the rows above less
// gap_open, so padding cells never hold a new best.
template <int CB>
__device__ __forceinline__ void ck_profile_fwd(uint32_t* prof, const uint8_t* patA, const uint8_t* patB, int j0,
                                               int nvA, int nvB, int sm, int sx, int t)
{
    constexpr int PAD = -16384;
    __syncwarp();
#pragma unroll
    for (int h = 0; h < CB / 2; ++h) {
        const int c0 = 2 * h, c1 = 2 * h + 1;
        const int a0 = c0 < nvA ? ck_code(__ldg(patA + j0 + c0)) : 4;
        const int a1 = c1 < nvA ? ck_code(__ldg(patA + j0 + c1)) : 4;
        const int b0 = c0 < nvB ? ck_code(__ldg(patB + j0 + c0)) : 4;
        const int b1 = c1 < nvB ? ck_code(__ldg(patB + j0 + c1)) : 4;
#pragma unroll
        for (int L = 0; L < 4; ++L) {
            const int va0 = a0 == 4 ? PAD : (a0 == L ? sm : sx), va1 = a1 == 4 ? PAD : (a1 == L ? sm : sx);
            const int vb0 = b0 == 4 ? PAD : (b0 == L ? sm : sx), vb1 = b1 == 4 ? PAD : (b1 == L ? sm : sx);
            prof[((0 * CK_LETTERS + L) * (CB / 2) + h) * 32 + t] = ((uint32_t)va0 & 0xffffu) | ((uint32_t)va1 << 16);
            prof[((1 * CK_LETTERS + L) * (CB / 2) + h) * 32 + t] = ((uint32_t)vb0 & 0xffffu) | ((uint32_t)vb1 << 16);
        }
        const uint32_t pad2 = ((uint32_t)PAD & 0xffffu) * 0x10001u;
        prof[((0 * CK_LETTERS + 4) * (CB / 2) + h) * 32 + t] = pad2;
        prof[((1 * CK_LETTERS + 4) * (CB / 2) + h) * 32 + t] = pad2;
    }
    __syncwarp();
}

// What one forward band pass reads and writes.
struct FwdCtx {
    const uint8_t *textA, *textB, *patA, *patB;
    int mA, nA, mB, nB, M, ncol;
    uint32_t* ck;            // checkpoint rows [q][col][2]
    uint32_t* ce;            // column edges [k][row][2]
    uint32_t* prof;
    int sm, sx;
    uint32_t NGO2, NGE2, GO2;
    uint32_t* rows = nullptr; // Q9: per pair and lane, the row that last raised the lane's best
};

// Q9 end-cell bookkeeping of one pair (half h) in one lane: best value v, the
// smallest key found among its cells (k1:k0, all ones when none), and the row
// `pend` that last raised v, whose H - go words sit in `rows` until a tie or
// the band's end needs its key.  Rows below the warp's best of the pair (taken
// every 32 steps) are skipped: they cannot hold the end cell.
template <int CB>
__device__ __forceinline__ void q9_store(uint32_t* dst, const uint32_t (&w)[CB])
{
    if constexpr (CB >= 4) {
#pragma unroll
        for (int q = 0; q < CB / 4; ++q)
            reinterpret_cast<uint4*>(dst)[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
    } else {
        *reinterpret_cast<uint2*>(dst) = make_uint2(w[0], w[1]);
    }
}

// mask (key order) of the lane's columns of half h holding H = v
template <int CB>
__device__ __forceinline__ uint32_t q9_mask(const uint32_t (&w)[CB], int v, int h, uint32_t GO2, uint32_t valid)
{
    const uint32_t tgt = __vsub2((uint32_t)v * 0x10001u, GO2);
    uint32_t m = 0u;
#pragma unroll
    for (int c = 0; c < CB; ++c) {
        const uint32_t eq = __vcmpeq2(w[c], tgt);
        m |= (h ? eq >> 31 : eq & 1u) << q9_rank<CB>(c);
    }
    return m & valid;
}

// merge row i's smallest key among cells of half h holding v into (k1, k0)
template <int CB>
__device__ __forceinline__ void q9_merge_row(const uint32_t (&w)[CB], int i, int v, int h, int j0, uint32_t GO2,
                                             uint32_t valid, int& k1, int& k0)
{
    const uint32_t m = q9_mask<CB>(w, v, h, GO2, valid);
    if (m) {
        const uint64_t key = c9_key(i, j0 + q9_col<CB>(__ffs(m) - 1));
        if (key < c9_join(k1, k0)) { k1 = (int)(key >> 32); k0 = (int)(uint32_t)key; }
    }
}

// the pending row of half h (stored at src) merged into (k1, k0)
template <int CB>
__device__ __forceinline__ void q9_resolve(const uint32_t* src, int& pend, int v, int h, int j0, uint32_t GO2,
                                           uint32_t valid, int& k1, int& k0)
{
    if (pend <= 0) return;
    uint32_t w[CB];
    if constexpr (CB >= 4) {
#pragma unroll
        for (int q = 0; q < CB / 4; ++q) {
            const uint4 x = reinterpret_cast<const uint4*>(src)[q];
            w[4 * q] = x.x; w[4 * q + 1] = x.y; w[4 * q + 2] = x.z; w[4 * q + 3] = x.w;
        }
    } else {
        const uint2 x = *reinterpret_cast<const uint2*>(src);
        w[0] = x.x; w[1] = x.y;
    }
    q9_merge_row<CB>(w, pend, v, h, j0, GO2, valid, k1, k0);
    pend = 0;
}

// Band starting at column b0 (0-based), CB columns per lane (the band covers
// 32 CB columns; the last band of a pair takes the smallest CB that reaches
// its last column).  Updates the lane's best (value, row, column) per pair.
// COOP: the band is one of an item's bands run by the warps of a block
// together (fwd16_coop); the warp then meets the block's barrier after every
// 32 steps, ceil((M + 31) / 32) times per band.
// Q9: the score-only form (sw16so_kernel): no checkpoint rows, and per pair
// the best value with the end-cell key of the reference's score-only kernel
// (c9_key) in (r, c) as its high and low words.
template <int CB, bool COOP, bool Q9 = false>
__device__ void fwd_band(const FwdCtx& X, int b0, int t, int& vA, int& rA, int& cA, int& vB, int& rB, int& cB,
                         int* pend = nullptr)
{
    constexpr int NH = CB / 2;
    const uint32_t MIN2 = 0x80008000u, K2 = 0x80008000u;
    const uint32_t NGO2 = X.NGO2, NGE2 = X.NGE2;
    const int M = X.M, mA = X.mA, mB = X.mB;
    const int j0 = b0 + t * CB;
    const int nvA = max(0, min(CB, X.nA - j0)), nvB = max(0, min(CB, X.nB - j0));
    ck_profile_fwd<CB>(X.prof, X.patA, X.patB, j0, nvA, nvB, X.sm, X.sx, t);
    uint32_t hgu[CB], fv[CB];
#pragma unroll
    for (int c = 0; c < CB; ++c) { hgu[c] = NGO2; fv[c] = 0u; }
    uint32_t validA = 0u, validB = 0u;                     // Q9: the pairs' columns, in key order
    uint32_t* rowsA = Q9 ? X.rows + t * CK_C : nullptr;
    uint32_t* rowsB = Q9 ? X.rows + (32 + t) * CK_C : nullptr;
    if constexpr (Q9) {
#pragma unroll
        for (int c = 0; c < CB; ++c) {
            validA |= (uint32_t)(c < nvA) << q9_rank<CB>(c);
            validB |= (uint32_t)(c < nvB) << q9_rank<CB>(c);
        }
    }
    uint32_t diag_in = NGO2, out_hg = NGO2, out_e = 0u;
    // left boundary: the column edge at column b0
    const uint32_t* left = b0 > 0 ? X.ce + 2 * (int64_t)(b0 / TW - 1) * M : nullptr;
    // this lane writes the column edge after its last column when that column is a multiple of TW
    const int kout = (j0 + CB) % TW == 0 && j0 + CB < X.ncol ? (j0 + CB) / TW : 0;
    uint32_t* eout = kout ? X.ce + 2 * (int64_t)(kout - 1) * M : nullptr;
    // each row's profile offsets (per pair, its text letter's rows; the padding
    // letter past the pair's text) travel along the lanes with the boundary
    // values.  Lane 0's inputs of 32 rows at a time -- the offsets and the left
    // edge -- are read by all lanes together (lane u: row 32k + u) and handed
    // to lane 0 by a shuffle each step, so no step runs a lane-0-only branch.
    auto row_off = [&](int r) -> uint32_t {
        const int la = r < mA ? ck_code(__ldg(X.textA + r)) : CK_LETTERS - 1;
        const int lb = r < mB ? ck_code(__ldg(X.textB + r)) : CK_LETTERS - 1;
        return (uint32_t)(la * NH * 32) | ((uint32_t)((CK_LETTERS + lb) * NH * 32) << 16);
    };
    uint32_t rb_off = 0u, rb_hg = NGO2, rb_e = 0u;       // this lane's row of the current 32
    uint32_t ch = 0;
    uint32_t bmax = 0u, brow = 0u;                        // this band: best and its first row, per half
    const int steps = M + 31;
    for (int tau = 0; tau < steps; ++tau) {
        if ((tau & 31) == 0 && tau < M) {
            const int r = tau + t;
            if (r < M) {
                rb_off = row_off(r);
                if (left) {
                    const uint2 lv = *reinterpret_cast<const uint2*>(left + 2 * r);
                    rb_hg = lv.x;
                    rb_e = lv.y;
                }
            }
            if constexpr (Q9) {
                // the pairs' best so far over the warp: a lower bound of their
                // final best, below which no cell can be the end cell
                pend[2] = __reduce_max_sync(FULL, vA);
                pend[3] = __reduce_max_sync(FULL, vB);
            }
        }
        uint32_t in_hg = __shfl_up_sync(FULL, out_hg, 1);
        uint32_t in_e = __shfl_up_sync(FULL, out_e, 1);
        ch = __shfl_up_sync(FULL, ch, 1);
        const uint32_t l_off = __shfl_sync(FULL, rb_off, tau & 31);
        const uint32_t l_hg = __shfl_sync(FULL, rb_hg, tau & 31);
        const uint32_t l_e = __shfl_sync(FULL, rb_e, tau & 31);
        const int i = tau - t + 1;
        if (t == 0) {
            ch = l_off;
            in_hg = l_hg;
            in_e = l_e;
        }
        if (i >= 1 && i <= M) {
        const uint32_t* pA = X.prof + (ch & 0xffffu) + t;
        const uint32_t* pB = X.prof + (ch >> 16) + t;
        uint32_t hgd = diag_in, hgl = in_hg, el = in_e;
        uint32_t rowmax = 0u;
#pragma unroll
        for (int cc = 0; cc < CB; cc += 2) {
            const uint32_t wa = pA[(cc >> 1) * 32], wb = pB[(cc >> 1) * 32];
            const uint32_t S0 = __byte_perm(wa, wb, 0x5410), S1 = __byte_perm(wa, wb, 0x7632);
            uint32_t hh2[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int cu = cc + u;
                const uint32_t S = u ? S1 : S0;
                const uint32_t e = __viaddmax_s16x2(el, NGE2, hgl);         // max(E_left - ge, H_left - go)
                const uint32_t f = __viaddmax_s16x2(fv[cu], NGE2, hgu[cu]); // max(F_up - ge, H_up - go)
                const uint32_t h1 = __viaddmax_s16x2(hgd, S, e);            // max(H_diag + s, E)
                const uint32_t hh = __vimax3_s16x2_relu(h1, f, f);          // max(h1, F, 0)
                const uint32_t hg = __viaddmax_s16x2(hh, NGO2, MIN2);       // H - go
                hh2[u] = hh;
                hgd = hgu[cu];
                hgu[cu] = hg;
                fv[cu] = f;
                hgl = hg;
                el = e;
            }
            rowmax = __vimax3_s16x2(rowmax, hh2[0], hh2[1]);
        }
        diag_in = in_hg;
        out_hg = hgl;
        out_e = el;
        if (eout) *reinterpret_cast<uint2*>(eout + 2 * (i - 1)) = make_uint2(out_hg, out_e);
        if constexpr (Q9) {
            // a row whose maximum reaches a pair's best so far: that maximum
            // sits in a column of the pair (padding columns score PAD and
            // trail the pair's last column by a gap).  A raise stores the row
            // and defers its key; a tie takes the keys of both rows.
            const int ra = lo16s(rowmax), rb = hi16s(rowmax);
            const bool ka = ra > 0 && ra >= max(vA, pend[2]) && i <= X.mA;
            const bool kb = rb > 0 && rb >= max(vB, pend[3]) && i <= X.mB;
            if (ka || kb) {
                if (ka) {
                    if (ra > vA) {
                        vA = ra; rA = cA = -1; pend[0] = i;
                        q9_store<CB>(rowsA, hgu);
                    } else {
                        q9_resolve<CB>(rowsA, pend[0], vA, 0, j0, X.GO2, validA, rA, cA);
                        q9_merge_row<CB>(hgu, i, vA, 0, j0, X.GO2, validA, rA, cA);
                    }
                }
                if (kb) {
                    if (rb > vB) {
                        vB = rb; rB = cB = -1; pend[1] = i;
                        q9_store<CB>(rowsB, hgu);
                    } else {
                        q9_resolve<CB>(rowsB, pend[1], vB, 1, j0, X.GO2, validB, rB, cB);
                        q9_merge_row<CB>(hgu, i, vB, 1, j0, X.GO2, validB, rB, cB);
                    }
                }
            }
        } else {
        if ((i & (CK_K - 1)) == 0 && i < M) {                     // checkpoint row i
            uint4* dst = reinterpret_cast<uint4*>(X.ck + 2 * ((int64_t)(i / CK_K - 1) * X.ncol + j0));
#pragma unroll
            for (int c = 0; c < CB; c += 2) dst[c >> 1] = make_uint4(hgu[c], fv[c], hgu[c + 1], fv[c + 1]);
        }
        // strict improvement per half (bits 15 / 31 of d clear): this band's
        // best and the first row holding it; the column is found when the walk
        // recomputes that row
        const uint32_t d = bmax - rowmax + K2;
        const uint32_t imp = ((~d & K2) >> 15) * 0xffffu;
        bmax = __vmaxs2(bmax, rowmax);
        brow = (brow & ~imp) | ((uint32_t)i * 0x10001u & imp);
        }
        }
        if (COOP && ((tau & 31) == 31 || tau == steps - 1)) __syncthreads();
    }
    if constexpr (Q9) {                                   // the band's pending rows
        q9_resolve<CB>(rowsA, pend[0], vA, 0, j0, X.GO2, validA, rA, cA);
        q9_resolve<CB>(rowsB, pend[1], vB, 1, j0, X.GO2, validB, rB, cB);
    } else {
        // merge the band into the lane's best; the column kept is the first of
        // the lane's span in this band (spans order like their columns)
        const int v = lo16s(bmax), r = (int)(brow & 0xffffu);
        if (v > 0 && ck_better(v, r, j0 + 1, vA, rA, cA)) { vA = v; rA = r; cA = j0 + 1; }
        const int v2 = hi16s(bmax), r2 = (int)(brow >> 16);
        if (v2 > 0 && ck_better(v2, r2, j0 + 1, vB, rB, cB)) { vB = v2; rB = r2; cB = j0 + 1; }
    }
    __syncwarp();
}

// fwd_band's traceback form for a warp alone, two rows per step: lane t
// takes rows i = 2 (tau - t) + 1 and i + 1 of its CB columns.  Row i + 1's
// cell in column c needs only row i's cells in columns c - 1 and c, so the
// two rows' dependency chains (E along a row, H through E) are independent at
// equal column and interleave: twice the independent integer work per lane
// between the same per-row shuffles and profile reads.  Values, checkpoint
// rows, column edges and the best (value, first row) per pair are
// fwd_band's exactly.
template <int CB>
__device__ void fwd_band2(const FwdCtx& X, int b0, int t, int& vA, int& rA, int& cA, int& vB, int& rB, int& cB)
{
    constexpr int NH = CB / 2;
    const uint32_t MIN2 = 0x80008000u, K2 = 0x80008000u;
    const uint32_t NGO2 = X.NGO2, NGE2 = X.NGE2;
    const int M = X.M, mA = X.mA, mB = X.mB;
    const int j0 = b0 + t * CB;
    const int nvA = max(0, min(CB, X.nA - j0)), nvB = max(0, min(CB, X.nB - j0));
    ck_profile_fwd<CB>(X.prof, X.patA, X.patB, j0, nvA, nvB, X.sm, X.sx, t);
    uint32_t hgu[CB], fv[CB];
#pragma unroll
    for (int c = 0; c < CB; ++c) { hgu[c] = NGO2; fv[c] = 0u; }
    // the left neighbour's H - go at the row above this step's first row; what
    // this lane hands right for its two rows
    uint32_t diag_in = NGO2, out_hg0 = NGO2, out_e0 = 0u, out_hg1 = NGO2, out_e1 = 0u;
    const uint32_t* left = b0 > 0 ? X.ce + 2 * (int64_t)(b0 / TW - 1) * M : nullptr;
    const int kout = (j0 + CB) % TW == 0 && j0 + CB < X.ncol ? (j0 + CB) / TW : 0;
    uint32_t* eout = kout ? X.ce + 2 * (int64_t)(kout - 1) * M : nullptr;
    auto row_off = [&](int r) -> uint32_t {
        const int la = r < mA ? ck_code(__ldg(X.textA + r)) : CK_LETTERS - 1;
        const int lb = r < mB ? ck_code(__ldg(X.textB + r)) : CK_LETTERS - 1;
        return (uint32_t)(la * NH * 32) | ((uint32_t)((CK_LETTERS + lb) * NH * 32) << 16);
    };
    // lane 0's inputs of 64 rows at a time (lane u: rows 64k + 2u and + 1,
    // 0-based), handed to lane 0 by shuffles
    uint32_t rb_off0 = 0u, rb_hg0 = NGO2, rb_e0 = 0u, rb_off1 = 0u, rb_hg1 = NGO2, rb_e1 = 0u;
    uint32_t ch0 = 0, ch1 = 0;
    uint32_t bmax = 0u, brow = 0u;
    const int steps = (M + 1) / 2 + 31;
    for (int tau = 0; tau < steps; ++tau) {
        if ((tau & 31) == 0 && 2 * tau < M) {
            const int r = 2 * (tau + t);
            if (r < M) {
                rb_off0 = row_off(r);
                if (left) {
                    const uint2 lv = *reinterpret_cast<const uint2*>(left + 2 * r);
                    rb_hg0 = lv.x;
                    rb_e0 = lv.y;
                }
            }
            if (r + 1 < M) {
                rb_off1 = row_off(r + 1);
                if (left) {
                    const uint2 lv = *reinterpret_cast<const uint2*>(left + 2 * (r + 1));
                    rb_hg1 = lv.x;
                    rb_e1 = lv.y;
                }
            }
        }
        uint32_t in_hg0 = __shfl_up_sync(FULL, out_hg0, 1);
        uint32_t in_e0 = __shfl_up_sync(FULL, out_e0, 1);
        uint32_t in_hg1 = __shfl_up_sync(FULL, out_hg1, 1);
        uint32_t in_e1 = __shfl_up_sync(FULL, out_e1, 1);
        ch0 = __shfl_up_sync(FULL, ch0, 1);
        ch1 = __shfl_up_sync(FULL, ch1, 1);
        const uint32_t l_off0 = __shfl_sync(FULL, rb_off0, tau & 31);
        const uint32_t l_hg0 = __shfl_sync(FULL, rb_hg0, tau & 31);
        const uint32_t l_e0 = __shfl_sync(FULL, rb_e0, tau & 31);
        const uint32_t l_off1 = __shfl_sync(FULL, rb_off1, tau & 31);
        const uint32_t l_hg1 = __shfl_sync(FULL, rb_hg1, tau & 31);
        const uint32_t l_e1 = __shfl_sync(FULL, rb_e1, tau & 31);
        const int i = 2 * (tau - t) + 1;
        if (t == 0) {
            ch0 = l_off0; in_hg0 = l_hg0; in_e0 = l_e0;
            ch1 = l_off1; in_hg1 = l_hg1; in_e1 = l_e1;
        }
        if (i >= 1 && i <= M) {
            const uint32_t* pA0 = X.prof + (ch0 & 0xffffu) + t;
            const uint32_t* pB0 = X.prof + (ch0 >> 16) + t;
            const uint32_t* pA1 = X.prof + (ch1 & 0xffffu) + t;
            const uint32_t* pB1 = X.prof + (ch1 >> 16) + t;
            // row i: diagonal, left; row i + 1: diagonal (row i's left neighbour), left
            uint32_t hgd0 = diag_in, hgl0 = in_hg0, el0 = in_e0;
            uint32_t hgd1 = in_hg0, hgl1 = in_hg1, el1 = in_e1;
            uint32_t rowmax0 = 0u, rowmax1 = 0u;
#pragma unroll
            for (int cc = 0; cc < CB; cc += 2) {
                const uint32_t wa0 = pA0[(cc >> 1) * 32], wb0 = pB0[(cc >> 1) * 32];
                const uint32_t wa1 = pA1[(cc >> 1) * 32], wb1 = pB1[(cc >> 1) * 32];
                const uint32_t S00 = __byte_perm(wa0, wb0, 0x5410), S01 = __byte_perm(wa0, wb0, 0x7632);
                const uint32_t S10 = __byte_perm(wa1, wb1, 0x5410), S11 = __byte_perm(wa1, wb1, 0x7632);
                uint32_t hh0[2], hh1[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int cu = cc + u;
                    // row i, column cu
                    const uint32_t e0 = __viaddmax_s16x2(el0, NGE2, hgl0);
                    const uint32_t f0 = __viaddmax_s16x2(fv[cu], NGE2, hgu[cu]);
                    const uint32_t h10 = __viaddmax_s16x2(hgd0, u ? S01 : S00, e0);
                    const uint32_t hv0 = __vimax3_s16x2_relu(h10, f0, f0);
                    const uint32_t hg0 = __viaddmax_s16x2(hv0, NGO2, MIN2);
                    hgd0 = hgu[cu];
                    // row i + 1, column cu: up is row i's cell just computed
                    const uint32_t e1 = __viaddmax_s16x2(el1, NGE2, hgl1);
                    const uint32_t f1 = __viaddmax_s16x2(f0, NGE2, hg0);
                    const uint32_t h11 = __viaddmax_s16x2(hgd1, u ? S11 : S10, e1);
                    const uint32_t hv1 = __vimax3_s16x2_relu(h11, f1, f1);
                    const uint32_t hg1 = __viaddmax_s16x2(hv1, NGO2, MIN2);
                    hgd1 = hg0;
                    hgu[cu] = hg1;
                    fv[cu] = f1;
                    hgl0 = hg0; el0 = e0;
                    hgl1 = hg1; el1 = e1;
                    hh0[u] = hv0;
                    hh1[u] = hv1;
                }
                rowmax0 = __vimax3_s16x2(rowmax0, hh0[0], hh0[1]);
                rowmax1 = __vimax3_s16x2(rowmax1, hh1[0], hh1[1]);
            }
            diag_in = in_hg1;
            out_hg0 = hgl0; out_e0 = el0;
            out_hg1 = hgl1; out_e1 = el1;
            const bool two = i + 1 <= M;
            if (eout) {
                *reinterpret_cast<uint2*>(eout + 2 * (i - 1)) = make_uint2(out_hg0, out_e0);
                if (two) *reinterpret_cast<uint2*>(eout + 2 * i) = make_uint2(out_hg1, out_e1);
            }
            if (((i + 1) & (CK_K - 1)) == 0 && i + 1 < M) {           // checkpoint row i + 1 (i is odd)
                uint4* dst = reinterpret_cast<uint4*>(X.ck + 2 * ((int64_t)((i + 1) / CK_K - 1) * X.ncol + j0));
#pragma unroll
                for (int c = 0; c < CB; c += 2) dst[c >> 1] = make_uint4(hgu[c], fv[c], hgu[c + 1], fv[c + 1]);
            }
            {
                const uint32_t d = bmax - rowmax0 + K2;
                const uint32_t imp = ((~d & K2) >> 15) * 0xffffu;
                bmax = __vmaxs2(bmax, rowmax0);
                brow = (brow & ~imp) | ((uint32_t)i * 0x10001u & imp);
            }
            if (two) {
                const uint32_t d = bmax - rowmax1 + K2;
                const uint32_t imp = ((~d & K2) >> 15) * 0xffffu;
                bmax = __vmaxs2(bmax, rowmax1);
                brow = (brow & ~imp) | ((uint32_t)(i + 1) * 0x10001u & imp);
            }
        }
    }
    const int v = lo16s(bmax), r = (int)(brow & 0xffffu);
    if (v > 0 && ck_better(v, r, j0 + 1, vA, rA, cA)) { vA = v; rA = r; cA = j0 + 1; }
    const int v2 = hi16s(bmax), r2 = (int)(brow >> 16);
    if (v2 > 0 && ck_better(v2, r2, j0 + 1, vB, rB, cB)) { vB = v2; rB = r2; cB = j0 + 1; }
    __syncwarp();
}

// Tile profile of one pair for a lane of a tile group (CT columns per lane):
// prof[((pair * 4 + letter) * CT/2 + h) * 32 + t] holds the 16-bit scores of
// the lane's columns col0 + 2h, col0 + 2h + 1 (0-based); past the pattern's
// end or left of column 0: mismatch.
template <int CT>
__device__ __forceinline__ void ck_profile_tile(uint32_t* prof, const uint8_t* pat, int n, int col0, int pair,
                                                int sm, int sx, int t)
{
#pragma unroll
    for (int h = 0; h < CT / 2; ++h) {
        const int c0 = col0 + 2 * h, c1 = c0 + 1;
        const int a0 = (c0 >= 0 && c0 < n) ? ck_code(__ldg(pat + c0)) : 4;
        const int a1 = (c1 >= 0 && c1 < n) ? ck_code(__ldg(pat + c1)) : 4;
#pragma unroll
        for (int L = 0; L < 4; ++L) {
            const int v0 = a0 == L ? sm : sx, v1 = a1 == L ? sm : sx;
            prof[((pair * 4 + L) * (CT / 2) + h) * 32 + t] = ((uint32_t)v0 & 0xffffu) | ((uint32_t)v1 << 16);
        }
    }
}

// The forward pass of one item by the 4 warps of a block: band b runs on warp
// b % 4, starting at 32-step chunk start(b) = max(start(b-1) + 2, start(b-4) +
// chunks per band), so each band's first lane reads the left edge of rows
// 32c+1 .. 32c+32 (written by the band before it up to its step 32c + 62)
// after the barrier that closed that band's chunk c + 1, and each warp runs
// its bands one after the other.  Every warp meets the block barrier once per
// chunk, idle or not: start(last band) + chunks per band times in all.
__device__ void fwd16_coop(const FwdCtx& X, int N, int t, int wib, int& vA, int& rA, int& cA, int& vB, int& rB,
                           int& cB)
{
    const int nck = (X.M + 62) / 32;                  // ceil((M + 31) / 32)
    int g = 0, prev = -2, b = 0;
    int st4[4] = {0, 0, 0, 0};
    for (int b0 = 0; b0 < N; ++b) {
        const int rest = N - b0;
        const int cb = rest > CK_BW ? CK_C : ck_last_cb(rest);
        const int s = max(prev + 2, b >= 4 ? st4[b & 3] + nck : 0);
        prev = s;
        st4[b & 3] = s;
        if ((b & 3) == wib) {
            for (; g < s; ++g) __syncthreads();
            if (cb == 16) fwd_band<16, true>(X, b0, t, vA, rA, cA, vB, rB, cB);
            else if (cb == 8) fwd_band<8, true>(X, b0, t, vA, rA, cA, vB, rB, cB);
            else if (cb == 4) fwd_band<4, true>(X, b0, t, vA, rA, cA, vB, rB, cB);
            else fwd_band<2, true>(X, b0, t, vA, rA, cA, vB, rB, cB);
            g += nck;
        }
        b0 += 32 * cb;
    }
    const int G = prev + nck;
    for (; g < G; ++g) __syncthreads();
}

// One work item (two pairs): the forward pass (by this warp, or by the
// block's 4 warps when coop), the best cells, the windows and walks (this
// warp, or warp 0 of the block) and the outputs.  wslot: the item's
// checkpoint memory (warp 0's slot when coop); prof: this warp's shared
// memory.  In coop every warp returns after the same barriers; the caller
// closes the item with one more barrier.
template <int TG, bool PLAN>
__device__ void ck_item(const Sw16Args& A, const int32_t* __restrict__ pwork, int w, bool coop, int wib, int t,
                        uint32_t* wslot, uint32_t* prof, int (*s_best)[6])
{
    const int32_t* work = PLAN ? pwork : A.work;
    const int go = A.gap_open, ge = A.gap_extend;
    const int sm = A.match + go, sx = A.mismatch + go;
    // unbiased forward constants (per half)
    const uint32_t NGO2 = ((uint32_t)(-go) & 0xffffu) * 0x10001u;
    const uint32_t NGE2 = ((uint32_t)(-ge) & 0xffffu) * 0x10001u;
    const uint32_t GO2 = (uint32_t)go * 0x10001u;
    const uint32_t MIN2 = 0x80008000u;
    // biased recompute constants (every value + BIAS16, sw_sizes.cuh)
    const uint32_t B2 = (uint32_t)CK_BIAS * 0x10001u;

    const int pa = work[2 * w];
    const bool has_b = work[2 * w + 1] >= 0;
    const int pb = has_b ? work[2 * w + 1] : pa;
    const int mA = A.D.a_len[pa], nA = A.D.b_len[pa];
    const int mB = A.D.a_len[pb], nB = A.D.b_len[pb];
    const uint8_t* textA = A.D.seq + A.D.a_off[pa];
    const uint8_t* patA = A.D.seq + A.D.b_off[pa];
    const uint8_t* textB = A.D.seq + A.D.a_off[pb];
    const uint8_t* patB = A.D.seq + A.D.b_off[pb];
    const int M = max(mA, mB), N = max(nA, nB);
    const int ncol = ck_ncol(N);
    const int nq = ck_rows(M);
    // slot layout: checkpoint rows [q][col][2], column edges [k][row][2],
    // tile tables [pair][step][lane]
    uint32_t* ck = wslot;
    uint32_t* ce = ck + 2 * (int64_t)nq * ncol;
    uint32_t* tiles = ce + (2 * (int64_t)(ncol / TW) * M + 3) / 4 * 4;     // 16-byte aligned

    // ------------------------------------------------ forward pass --
    int vA = 0, rA = 0, cA = 0, vB = 0, rB = 0, cB = 0;          // lane's best per pair
    {
        FwdCtx X{textA, textB, patA, patB, mA, nA, mB, nB, M, ncol, ck, ce, prof, sm, sx, NGO2, NGE2, GO2};
        if (coop) {
            fwd16_coop(X, N, t, wib, vA, rA, cA, vB, rB, cB);
        } else {
            for (int b0 = 0; b0 < N;) {
                const int rest = N - b0;                          // columns from this band on
                const int cb = rest > CK_BW ? CK_C : ck_last_cb(rest);
                if (cb == 16) fwd_band2<16>(X, b0, t, vA, rA, cA, vB, rB, cB);
                else if (cb == 8) fwd_band2<8>(X, b0, t, vA, rA, cA, vB, rB, cB);
                else if (cb == 4) fwd_band2<4>(X, b0, t, vA, rA, cA, vB, rB, cB);
                else fwd_band2<2>(X, b0, t, vA, rA, cA, vB, rB, cB);
                b0 += 32 * cb;
            }
        }
    }
    // per pair over the warp: (max value, min row, min span); the best cell
    // is the first column of that row holding the value -- in that span, as
    // any earlier column holding it would belong to an earlier span
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const int ov = __shfl_xor_sync(FULL, vA, o), orr = __shfl_xor_sync(FULL, rA, o), oc = __shfl_xor_sync(FULL, cA, o);
        if (ov > 0 && ck_better(ov, orr, oc, vA, rA, cA)) { vA = ov; rA = orr; cA = oc; }
        const int ov2 = __shfl_xor_sync(FULL, vB, o), orr2 = __shfl_xor_sync(FULL, rB, o), oc2 = __shfl_xor_sync(FULL, cB, o);
        if (ov2 > 0 && ck_better(ov2, orr2, oc2, vB, rB, cB)) { vB = ov2; rB = orr2; cB = oc2; }
    }
    if (coop) {
        // the block's best per pair: every warp reduces the four warps' bests in the same order
        if (t == 0) {
            s_best[wib][0] = vA; s_best[wib][1] = rA; s_best[wib][2] = cA;
            s_best[wib][3] = vB; s_best[wib][4] = rB; s_best[wib][5] = cB;
        }
        __syncthreads();
        vA = s_best[0][0]; rA = s_best[0][1]; cA = s_best[0][2];
        vB = s_best[0][3]; rB = s_best[0][4]; cB = s_best[0][5];
        for (int q = 1; q < 4; ++q) {
            if (s_best[q][0] > 0 && ck_better(s_best[q][0], s_best[q][1], s_best[q][2], vA, rA, cA)) {
                vA = s_best[q][0]; rA = s_best[q][1]; cA = s_best[q][2];
            }
            if (s_best[q][3] > 0 && ck_better(s_best[q][3], s_best[q][4], s_best[q][5], vB, rB, cB)) {
                vB = s_best[q][3]; rB = s_best[q][4]; cB = s_best[q][5];
            }
        }
        if (wib != 0) return;                     // the windows and walks are warp 0's
    }

    // ----------------------------------------------------- the walks --
    // per pair: cell, state (0 H, 1 E, 2 F), tracked value, CIGAR cursor, tile
    int wi[2] = {rA, rB}, wj[2] = {cA, cB}, wst[2] = {0, 0}, wv[2] = {vA, vB};
    int wpos[2] = {mA + nA, mB + nB};
    bool done[2] = {vA <= 0, !has_b || vB <= 0};
    // a pair whose best reached the limit may have passed 16 bits (a pair taken
    // on the optimistic rule): it goes to the 32-bit kernel, which writes it
    const bool ovf[2] = {vA >= A.ovf_limit, has_b && vB >= A.ovf_limit};
#pragma unroll
    for (int x = 0; x < 2; ++x) {
        if (x == 1 && !has_b) break;
        if (t == 0) {
            const int p = x ? pb : pa;
            if (ovf[x]) {
                A.esc_list[atomicAdd(A.esc_count, 1)] = p;
            } else if (done[x]) {
                A.out_score[p] = 0;
                A.out_pos[4 * p] = A.out_pos[4 * p + 1] = A.out_pos[4 * p + 2] = A.out_pos[4 * p + 3] = -1;
                A.out_len[p] = 0;
            } else {
                A.out_score[p] = x ? vB : vA;
                A.out_pos[4 * p + 2] = (x ? rB : rA) - 1;
            }
        }
    }
    done[0] = done[0] || ovf[0];
    done[1] = done[1] || ovf[1];
    bool first[2] = {!done[0], !done[1]};                // the best cell's column not yet found
    const int best_of[2] = {vA, vB};
    int ti0[2] = {1, 1}, tb[2] = {0, 0};
#pragma unroll
    for (int x = 0; x < 2; ++x) {
        ti0[x] = done[x] ? 1 : ((wi[x] - 1) / CK_K) * CK_K + 1;
        tb[x] = done[x] ? 0 : (wj[x] - 1) / TW;
    }
    // window table: H of the window's cells, [row][TG * TW columns], both
    // pairs in the 16-bit halves (biased)
    constexpr int WCOL = TG * TW;
    uint32_t* Ht = tiles;
    constexpr int LG = 32 / TG, CT = TW / LG;                   // lanes per tile group, columns per lane
    const int g = t / LG, tl = t % LG;                          // tile group, lane in group
    while (!(done[0] && done[1])) {
        // ---- recompute, per pair x, the window of TG tiles tb-TG+1 .. tb over rows
        // [ti0, wi]: group g takes tile tb - TG + 1 + g, lane tl its columns
        // CT tl .. CT tl + CT - 1
        const int rows0 = done[0] ? 0 : wi[0] - ti0[0] + 1, rows1 = done[1] ? 0 : wi[1] - ti0[1] + 1;
        const int R = max(rows0, rows1);
        const int tgA = tb[0] - (TG - 1) + g, tgB = tb[1] - (TG - 1) + g;   // this group's tiles
        const int colA = TW * tgA + CT * tl, colB = TW * tgB + CT * tl;    // this lane's first columns
        __syncwarp();
        ck_profile_tile<CT>(prof, patA, nA, colA, 0, sm, sx, t);
        ck_profile_tile<CT>(prof, patB, nB, colB, 1, sm, sx, t);
        uint32_t hgu[CT], fv[CT];
        uint32_t diag_in;
        {
            const int qa = (ti0[0] - 1) / CK_K - 1, qb = (ti0[1] - 1) / CK_K - 1;
            const uint32_t* ca = ck + 2 * (int64_t)max(qa, 0) * ncol;
            const uint32_t* cb = ck + 2 * (int64_t)max(qb, 0) * ncol;
            const bool oka = qa >= 0 && tgA >= 0, okb = qb >= 0 && tgB >= 0;
#pragma unroll
            for (int c = 0; c < CT; ++c) {
                const uint2 va = oka ? *reinterpret_cast<const uint2*>(ca + 2 * (colA + c)) : make_uint2(NGO2, 0u);
                const uint2 vb = okb ? *reinterpret_cast<const uint2*>(cb + 2 * (colB + c)) : make_uint2(NGO2, 0u);
                hgu[c] = __viaddmax_s16x2(__byte_perm(va.x, vb.x, 0x7610), B2, MIN2);
                fv[c] = __viaddmax_s16x2(__byte_perm(va.y, vb.y, 0x7610), B2, MIN2);
            }
            // H[i0-1][first column - 1] - go: the left lane's last column; for a
            // group's first lane the checkpoint left of its tile (0 on row 0 and column 0)
            uint32_t lft = __shfl_up_sync(FULL, hgu[CT - 1], 1, LG);
            if (tl == 0) {
                const uint32_t ha = (qa >= 0 && tgA > 0) ? ca[2 * (colA - 1)] : NGO2;
                const uint32_t hb = (qb >= 0 && tgB > 0) ? cb[2 * (colB - 1)] : NGO2;
                lft = __viaddmax_s16x2(__byte_perm(ha, hb, 0x7610), B2, MIN2);
            }
            diag_in = lft;
        }
        // the groups' left boundaries per tile row (column edges at TW * tile),
        // combined and biased into shared memory: edg[(group * CK_K + row) * 2]
        uint32_t* edg = prof + 2 * 4 * (CT / 2) * 32;
        for (int idx = t; idx < TG * CK_K; idx += 32) {
            const int gg = idx / CK_K, r = idx - gg * CK_K;
            const int ka = tb[0] - (TG - 1) + gg, kb = tb[1] - (TG - 1) + gg;
            const bool ina = ka > 0 && r < rows0, inb = kb > 0 && r < rows1;
            const uint2 la = ina ? *reinterpret_cast<const uint2*>(ce + 2 * ((int64_t)(ka - 1) * M + (ti0[0] - 1 + r)))
                                 : make_uint2(NGO2, 0u);
            const uint2 lb = inb ? *reinterpret_cast<const uint2*>(ce + 2 * ((int64_t)(kb - 1) * M + (ti0[1] - 1 + r)))
                                 : make_uint2(NGO2, 0u);
            edg[2 * idx] = __viaddmax_s16x2(__byte_perm(la.x, lb.x, 0x7610), B2, MIN2);
            edg[2 * idx + 1] = __viaddmax_s16x2(__byte_perm(la.y, lb.y, 0x7610), B2, MIN2);
        }
        __syncwarp();
        const uint32_t* eg = edg + 2 * g * CK_K;
        uint32_t out_hg = B2 - GO2, out_e = B2;
        const uint8_t* tA = textA + (ti0[0] - 1);
        const uint8_t* tB = textB + (ti0[1] - 1);
        // each row's profile offsets travel along a group's lanes with the
        // boundary values; the groups' first lanes get theirs, and the row's
        // left edge, without a branch of their own: the offsets of 64 rows at
        // a time are read by all lanes (lane u: rows 64k + 2u and + 1) and
        // shuffled out.  Two rows per step, as in fwd_band2: lane tl takes
        // window rows i = 2 (tau - tl) + 1 and i + 1, whose dependency chains
        // interleave.
        uint32_t ch0 = 0, ch1 = 0, rb_ch0 = 0, rb_ch1 = 0;
        uint32_t out_hg1 = B2 - GO2, out_e1 = B2;
        const uint32_t* pA0 = prof + (0 * 4 * (CT / 2)) * 32 + t;
        const uint32_t* pB0 = prof + (1 * 4 * (CT / 2)) * 32 + t;
        uint32_t* hrow = Ht + g * TW + CT * tl;                         // + (row - 1) * WCOL
        const int steps2 = (R + 1) / 2 + LG - 1;
        for (int tau = 0; tau < steps2; ++tau) {
            if ((tau & 31) == 0 && 2 * tau < R) {
                const int r = 2 * (tau + t);
                if (r < R) {
                    const int la = r < rows0 ? ck_code(__ldg(tA + r)) : 0;
                    const int lb = r < rows1 ? ck_code(__ldg(tB + r)) : 0;
                    rb_ch0 = (uint32_t)(la * (CT / 2) * 32) | ((uint32_t)(lb * (CT / 2) * 32) << 16);
                }
                if (r + 1 < R) {
                    const int la = r + 1 < rows0 ? ck_code(__ldg(tA + r + 1)) : 0;
                    const int lb = r + 1 < rows1 ? ck_code(__ldg(tB + r + 1)) : 0;
                    rb_ch1 = (uint32_t)(la * (CT / 2) * 32) | ((uint32_t)(lb * (CT / 2) * 32) << 16);
                }
            }
            uint32_t in_hg0 = __shfl_up_sync(FULL, out_hg, 1, LG);
            uint32_t in_e0 = __shfl_up_sync(FULL, out_e, 1, LG);
            uint32_t in_hg1 = __shfl_up_sync(FULL, out_hg1, 1, LG);
            uint32_t in_e1 = __shfl_up_sync(FULL, out_e1, 1, LG);
            ch0 = __shfl_up_sync(FULL, ch0, 1, LG);
            ch1 = __shfl_up_sync(FULL, ch1, 1, LG);
            const uint32_t l_ch0 = __shfl_sync(FULL, rb_ch0, tau & 31);
            const uint32_t l_ch1 = __shfl_sync(FULL, rb_ch1, tau & 31);
            const int er0 = min(2 * tau, CK_K - 1), er1 = min(2 * tau + 1, CK_K - 1);
            const uint32_t l_hg0 = eg[2 * er0], l_e0 = eg[2 * er0 + 1];
            const uint32_t l_hg1 = eg[2 * er1], l_e1 = eg[2 * er1 + 1];
            const int i = 2 * (tau - tl) + 1;                            // window rows i, i + 1 (1-based)
            if (tl == 0) {
                ch0 = l_ch0; in_hg0 = l_hg0; in_e0 = l_e0;
                ch1 = l_ch1; in_hg1 = l_hg1; in_e1 = l_e1;
            }
            if (i < 1 || i > R) continue;
            const uint32_t* pA_0 = pA0 + (ch0 & 0xffffu);
            const uint32_t* pB_0 = pB0 + (ch0 >> 16);
            const uint32_t* pA_1 = pA0 + (ch1 & 0xffffu);
            const uint32_t* pB_1 = pB0 + (ch1 >> 16);
            uint32_t hgd0 = diag_in, hgl0 = in_hg0, el0 = in_e0;
            uint32_t hgd1 = in_hg0, hgl1 = in_hg1, el1 = in_e1;
            uint32_t hv0[CT], hv1[CT];
#pragma unroll
            for (int cc = 0; cc < CT; cc += 2) {
                const uint32_t wa0 = pA_0[(cc >> 1) * 32], wb0 = pB_0[(cc >> 1) * 32];
                const uint32_t wa1 = pA_1[(cc >> 1) * 32], wb1 = pB_1[(cc >> 1) * 32];
                const uint32_t S00 = __byte_perm(wa0, wb0, 0x5410), S01 = __byte_perm(wa0, wb0, 0x7632);
                const uint32_t S10 = __byte_perm(wa1, wb1, 0x5410), S11 = __byte_perm(wa1, wb1, 0x7632);
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int cu = cc + u;
                    const uint32_t e0 = __viaddmax_s16x2(el0, NGE2, hgl0);
                    const uint32_t f0 = __viaddmax_s16x2(fv[cu], NGE2, hgu[cu]);
                    const uint32_t h10 = __viaddmax_s16x2(hgd0, u ? S01 : S00, e0);
                    const uint32_t hh0 = __vimax3_s16x2(h10, f0, B2);
                    const uint32_t hg0 = hh0 - GO2;
                    hv0[cu] = hh0;
                    hgd0 = hgu[cu];
                    const uint32_t e1 = __viaddmax_s16x2(el1, NGE2, hgl1);
                    const uint32_t f1 = __viaddmax_s16x2(f0, NGE2, hg0);
                    const uint32_t h11 = __viaddmax_s16x2(hgd1, u ? S11 : S10, e1);
                    const uint32_t hh1 = __vimax3_s16x2(h11, f1, B2);
                    const uint32_t hg1 = hh1 - GO2;
                    hv1[cu] = hh1;
                    hgd1 = hg0;
                    hgu[cu] = hg1;
                    fv[cu] = f1;
                    hgl0 = hg0; el0 = e0;
                    hgl1 = hg1; el1 = e1;
                }
            }
            uint4* dst0 = reinterpret_cast<uint4*>(hrow + (i - 1) * WCOL);
#pragma unroll
            for (int c = 0; c < CT; c += 4) dst0[c >> 2] = make_uint4(hv0[c], hv0[c + 1], hv0[c + 2], hv0[c + 3]);
            if (i + 1 <= R) {
                uint4* dst1 = reinterpret_cast<uint4*>(hrow + i * WCOL);
#pragma unroll
                for (int c = 0; c < CT; c += 4) dst1[c >> 2] = make_uint4(hv1[c], hv1[c + 1], hv1[c + 2], hv1[c + 3]);
            }
            diag_in = in_hg1;
            out_hg = hgl0; out_e = el0;
            out_hg1 = hgl1; out_e1 = el1;
        }
        __syncwarp();
        // the best cell's column (a pair's first window): first column of row i*
        // holding the best value -- row i* is the window's last row
#pragma unroll
        for (int x = 0; x < 2; ++x) {
            if (!first[x]) continue;
            const int rows = x ? rows1 : rows0, n = x ? nB : nA;
            const int wc0 = TW * (tb[x] - (TG - 1));                    // 0-based column of window column 0
            int jf = INT32_MAX;
            constexpr int PER = WCOL / 32;
#pragma unroll
            for (int c = PER - 1; c >= 0; --c) {
                const int col = wc0 + PER * t + c;
                if (col >= 0 && col < n) {
                    const uint32_t w = Ht[(rows - 1) * WCOL + PER * t + c];
                    if ((int)(x ? (w >> 16) : (w & 0xffffu)) - CK_BIAS == best_of[x]) jf = col + 1;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) jf = min(jf, __shfl_xor_sync(FULL, jf, o));
            first[x] = false;
            const int p = x ? pb : pa;
            if (jf == INT32_MAX) {                 // cannot happen: the forward pass saw the value here
                if (t == 0) atomicOr(A.err, ERR_BAD_INPUT);
                done[x] = true;
                continue;
            }
            wj[x] = jf;
            if (t == 0) A.out_pos[4 * p + 3] = jf - 1;
        }
        // ---- walk each pair inside its window, tracking the exact value of the
        // current cell's H (state 0), E (1) or F (2).  Every decision is the
        // reference's tie rule read off H values: H came from the diagonal iff
        // H[i-1][j-1] + s == H (the diagonal wins ties), else from E iff E == H
        // (E wins ties with F), else from F; a gap cell was opened iff the
        // neighbour's H - gap_open equals it (opening wins ties).
#pragma unroll
        for (int x = 0; x < 2; ++x) {
            if (done[x]) continue;
            const int p = x ? pb : pa;
            const int m = x ? mB : mA, n = x ? nB : nA;
            const uint8_t* text = x ? textB : textA;
            const uint8_t* pat = x ? patB : patA;
            char* slotc = A.out_cigar + A.D.out_off[p];
            const int i0 = ti0[x], jlo = TW * (tb[x] - (TG - 1)) + 1;     // first window row / column
            const int q = (i0 - 1) / CK_K - 1;                              // checkpoint row i0 - 1
            const uint32_t* crow = ck + 2 * (int64_t)max(q, 0) * ncol;
            const int kedge = (jlo - 1) / TW;                               // column edge at jlo - 1 (if >= 1)
            const uint32_t* cedge = kedge > 0 ? ce + 2 * (int64_t)(kedge - 1) * M : nullptr;
            auto half = [x](uint32_t w) { return x ? hi16s(w) : lo16s(w); };
            // H[ii][jj] for ii in [i0 - 1, i], jj in [jlo - 1, j]
            auto Hv = [&](int ii, int jj) -> int {
                if (ii <= 0 || jj <= 0) return 0;
                if (ii == i0 - 1) return half(crow[2 * (jj - 1)]) + go;
                if (jj == jlo - 1) return half(cedge[2 * (ii - 1)]) + go;
                const uint32_t w = Ht[(ii - i0) * WCOL + (jj - jlo)];
                return (int)(x ? (w >> 16) : (w & 0xffffu)) - CK_BIAS;
            };
            // E[ii][jj] from the row's H values left of jj within the window and the
            // column edge's E (E[ii][0] = 0): warp-parallel max over the gap lengths
            auto Ev = [&](int ii, int jj) -> int {
                const int kl = max(jlo - 1, 0);
                int e = INT32_MIN / 2;
                for (int k = jj - 1 - t; k >= kl; k -= 32) e = max(e, Hv(ii, k) - go - (jj - 1 - k) * ge);
                if (t == 0) {
                    const int eb = (kl > 0) ? half(cedge[2 * (ii - 1) + 1]) : 0;
                    e = max(e, eb - (jj - kl) * ge);
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(FULL, e, o));
                return e;
            };
            int i = wi[x], j = wj[x], state = wst[x], v = wv[x], pos = wpos[x];
            bool fin = false;
            for (;;) {
                if (i <= 0 || j <= 0 || (state == 0 && v == 0)) { fin = true; break; }
                if (i < i0 || j < jlo) break;                               // left the window
                if (state == 0) {
                    // a run of diagonal steps resolved at once: lane u takes the step from
                    // cell (i - u, j - u), whose value is the H lane u - 1 read; the run
                    // ends at the first step that is not diagonal or starts at H = 0
                    const int U = min(min(32, pos), min(i - max(i0, 1), j - max(jlo, 1)) + 1);
                    int hd = 0;
                    bool eq = false;
                    if (t < U) {
                        eq = __ldg(text + i - 1 - t) == __ldg(pat + j - 1 - t);
                        hd = Hv(i - 1 - t, j - 1 - t);
                    }
                    int vu = __shfl_up_sync(FULL, hd, 1);
                    if (t == 0) vu = v;
                    const bool ok = t < U && vu != 0 && hd + (eq ? A.match : A.mismatch) == vu;
                    const unsigned run = __ballot_sync(FULL, ok);
                    const int r = run == FULL ? 32 : __ffs(~run) - 1;
                    if (r > 0) {
                        if (t < r) slotc[pos - 1 - t] = eq ? 'M' : 'X';
                        v = __shfl_sync(FULL, hd, r - 1);
                        i -= r;
                        j -= r;
                        pos -= r;
                        continue;
                    }
                }
                char op;
                if (state == 0) {
                    const uint8_t ta = __ldg(text + i - 1), pc = __ldg(pat + j - 1);
                    const int hd = Hv(i - 1, j - 1);
                    if (hd + (ta == pc ? A.match : A.mismatch) == v) {
                        op = ta == pc ? 'M' : 'X';
                        v = hd;
                        --i;
                        --j;
                    } else if (Ev(i, j) == v) {
                        op = 'D';
                        if (Hv(i, j - 1) - go == v) { v += go; } else { state = 1; v += ge; }
                        --j;
                    } else {
                        op = 'I';
                        if (Hv(i - 1, j) - go == v) { v += go; } else { state = 2; v += ge; }
                        --i;
                    }
                } else if (state == 1) {
                    op = 'D';
                    if (Hv(i, j - 1) - go == v) { v += go; state = 0; } else { v += ge; }
                    --j;
                } else {
                    op = 'I';
                    if (Hv(i - 1, j) - go == v) { v += go; state = 0; } else { v += ge; }
                    --i;
                }
                if (pos <= 0) {
                    if (t == 0) atomicOr(A.err, ERR_CIGAR_OVERFLOW);
                    fin = true;
                    break;
                }
                --pos;
                if (t == 0) slotc[pos] = op;
            }
            // Diagonal shortcut.  Standing in H on a checkpoint row (where the
            // walk leaves a window at its top): if the straight diagonal up to
            // the next checkpoint row (or to row or column 0, where H is 0)
            // scores exactly the current value, it is the walk's own path.  H
            // at each cell is at least its diagonal predecessor's plus the
            // step's score, so along such a diagonal every predecessor holds
            // exactly the partial sum, each step is diagonal (the diagonal wins
            // ties) and no window is needed for it.  Taken while every cell it
            // steps from stays above 0 (a 0 ends the walk: the window path
            // finds it).  (Hops that also end on column edges measured no
            // faster on the 200,000-pair batch.)
            while (!fin && state == 0 && v > 0 && i >= 1 && j >= 1 && (i & (CK_K - 1)) == 0) {
                const int L = min(min(CK_K, i), j);                     // steps (at most 64)
                if (L > pos) break;
                const int ie = i - L, je = j - L;                            // the end cell
                const int he = (ie == 0 || je == 0)
                                   ? 0 : half(ck[2 * ((int64_t)(ie / CK_K - 1) * ncol + (je - 1))]) + go;
                bool e0 = false, e1 = false;
                int p0 = 0, p1 = 0;                                          // step t, step t + 32: its score
                if (t < L) {
                    e0 = __ldg(text + i - 1 - t) == __ldg(pat + j - 1 - t);
                    p0 = e0 ? A.match : A.mismatch;
                }
                if (t + 32 < L) {
                    e1 = __ldg(text + i - 33 - t) == __ldg(pat + j - 33 - t);
                    p1 = e1 ? A.match : A.mismatch;
                }
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {                          // inclusive prefix sums
                    const int y0 = __shfl_up_sync(FULL, p0, o), y1 = __shfl_up_sync(FULL, p1, o);
                    if (t >= o) { p0 += y0; p1 += y1; }
                }
                p1 += __shfl_sync(FULL, p0, 31);
                const int total = __shfl_sync(FULL, p1, 31);
                // the cell after step u holds v - prefix(u); all before the end cell must stay above 0
                const bool low = (t < L - 1 && v - p0 <= 0) || (t + 32 < L - 1 && v - p1 <= 0);
                if (v - total != he || __any_sync(FULL, low)) break;
                if (t < L) slotc[pos - 1 - t] = e0 ? 'M' : 'X';
                if (t + 32 < L) slotc[pos - 33 - t] = e1 ? 'M' : 'X';
                pos -= L;
                i = ie;
                j = je;
                v = he;
                if (i <= 0 || j <= 0 || v == 0) fin = true;
            }
            wi[x] = i; wj[x] = j; wst[x] = state; wv[x] = v; wpos[x] = pos;
            if (fin) {
                done[x] = true;
                if (t == 0) {
                    A.out_pos[4 * p] = i;
                    A.out_pos[4 * p + 1] = j;
                    A.out_len[p] = m + n - pos;
                }
            } else {
                // next window: the block above (left its top) or the tiles to the left
                if (i < i0) ti0[x] = ((i - 1) / CK_K) * CK_K + 1;
                tb[x] = (j - 1) / TW;
            }
        }
        __syncwarp();
    }
}

// TG: tiles recomputed per window pass, the walk's and the TG - 1 to its left.
// Work items come largest first.  Items above A.coop_cells cells (larger row
// count x larger column count of the two pairs) are taken by a whole block,
// whose 4 warps share the forward pass; from the first smaller item on, each
// warp takes items of its own.
// BLK: the variant with the whole-block phase; without it every warp takes
// items of its own and no block barrier is met.
// PLAN: items and per-warp memory from the device-built plan (plan_view),
// the list and its length kept in shared memory; otherwise the launch's own.
template <int TG, bool BLK, bool PLAN>
__global__ void __launch_bounds__(128, 4) sw16ck_kernel(Sw16Args A)
{
    static_assert(TG == 2 || TG == 4, "tile groups split the warp evenly, window rows are 16-byte vectors");
    extern __shared__ uint32_t ck_smem[];
    __shared__ int s_item;
    __shared__ int s_best[4][6];
    __shared__ const int32_t* s_work;
    __shared__ int s_nwork;
    const int t = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    int64_t dir_slot = A.dir_slot;
    if constexpr (PLAN) {
        const PlanView V = plan_view(A.plan, A.plan_list, A.work, A.nwork, nullptr, A.dir_slot, A.edge_slot,
                                     A.dir_cap, A.edge_cap, A.err);
        if (!V.run) return;
        dir_slot = V.dir_slot;
        if (threadIdx.x == 0) { s_work = V.work; s_nwork = V.nwork; }
        __syncthreads();
    }
    uint32_t* wslot = A.dirs + ((int64_t)blockIdx.x * (blockDim.x >> 5) + wib) * dir_slot;
    uint32_t* bslot = A.dirs + (int64_t)blockIdx.x * (blockDim.x >> 5) * dir_slot;
    uint32_t* prof = ck_smem + wib * CK_WARP_WORDS;
#define SW16_NWORK (PLAN ? s_nwork : A.nwork)
#define SW16_WORK (PLAN ? s_work : A.work)

    // one call site of ck_item, so its body is in the kernel once
    bool block_phase = BLK && A.coop_cells >= 0;
    for (;;) {
        int w = -1;
        bool coop = false;
        if (block_phase) {
            if (threadIdx.x == 0) s_item = atomicAdd(A.counter, 1);
            __syncthreads();
            const int wb = s_item;
            __syncthreads();
            if (wb >= SW16_NWORK) break;
            const int pa = SW16_WORK[2 * wb], pb = SW16_WORK[2 * wb + 1];
            const int M = max(A.D.a_len[pa], pb >= 0 ? A.D.a_len[pb] : 0);
            const int N = max(A.D.b_len[pa], pb >= 0 ? A.D.b_len[pb] : 0);
            if ((int64_t)M * N > A.coop_cells) {
                w = wb;
                coop = true;
            } else {
                block_phase = false;                  // warp 0 keeps this item, the others draw their own
                if (wib == 0) w = wb;
            }
        }
        if (!coop && w < 0) {
            if (t == 0) w = atomicAdd(A.counter, 1);
            w = __shfl_sync(FULL, w, 0);
            if (w >= SW16_NWORK) break;
        }
        __syncwarp();
        ck_item<TG, PLAN>(A, s_work, w, coop, wib, t, coop ? bslot : wslot, prof, s_best);
        if (coop) __syncthreads();
    }
}

// Score-only Smith-Waterman, two pairs per warp in 16-bit halves: the forward
// pass of sw16ck_kernel without checkpoint rows (column edges every TW columns
// carry the band boundaries), the end cell by the reference's score-only rule
// (c9_key).  dir_slot = sw16so_dir_words.  Outputs: score, and end_i / end_j
// (0-based) for a positive score, -1 otherwise; start cells -1.
template <bool PLAN>
__global__ void __launch_bounds__(128, 4) sw16so_kernel(Sw16Args A)
{
    extern __shared__ uint32_t ck_smem[];
    __shared__ const int32_t* s_work;
    __shared__ int s_nwork;
    const int t = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    int64_t dir_slot = A.dir_slot;
    if constexpr (PLAN) {
        const PlanView V = plan_view(A.plan, A.plan_list, A.work, A.nwork, nullptr, A.dir_slot, A.edge_slot,
                                     A.dir_cap, A.edge_cap, A.err);
        if (!V.run) return;
        dir_slot = V.dir_slot;
        if (threadIdx.x == 0) { s_work = V.work; s_nwork = V.nwork; }
        __syncthreads();
    }
    uint32_t* rows = A.dirs + ((int64_t)blockIdx.x * (blockDim.x >> 5) + wib) * dir_slot;
    uint32_t* ce = rows + SO_ROW_WORDS;
    uint32_t* prof = ck_smem + wib * CK_WARP_WORDS;
    const int go = A.gap_open, ge = A.gap_extend;
    const int sm = A.match + go, sx = A.mismatch + go;
    const uint32_t NGO2 = ((uint32_t)(-go) & 0xffffu) * 0x10001u;
    const uint32_t NGE2 = ((uint32_t)(-ge) & 0xffffu) * 0x10001u;
    const uint32_t GO2 = (uint32_t)go * 0x10001u;
    for (;;) {
        int w = 0;
        if (t == 0) w = atomicAdd(A.counter, 1);
        w = __shfl_sync(FULL, w, 0);
        if (w >= SW16_NWORK) break;
        __syncwarp();
        const int pa = SW16_WORK[2 * w];
        const bool has_b = SW16_WORK[2 * w + 1] >= 0;
        const int pb = has_b ? SW16_WORK[2 * w + 1] : pa;
        const int mA = A.D.a_len[pa], nA = A.D.b_len[pa];
        const int mB = A.D.a_len[pb], nB = A.D.b_len[pb];
        const int M = max(mA, mB), N = max(nA, nB);
        FwdCtx X{A.D.seq + A.D.a_off[pa], A.D.seq + A.D.a_off[pb], A.D.seq + A.D.b_off[pa], A.D.seq + A.D.b_off[pb],
                 mA, nA, mB, nB, M, ck_ncol(N), nullptr, ce, prof, sm, sx, NGO2, NGE2, GO2, rows};
        int vA = 0, kA1 = -1, kA0 = -1, vB = 0, kB1 = -1, kB0 = -1;    // best and its key (high, low word)
        int pend[4] = {0, 0, 0, 0};      // pending rows of A and B, the warp's best of A and B
        for (int b0 = 0; b0 < N;) {
            const int rest = N - b0;
            const int cb = rest > CK_BW ? CK_C : ck_last_cb(rest);
            if (cb == 16) fwd_band<16, false, true>(X, b0, t, vA, kA1, kA0, vB, kB1, kB0, pend);
            else if (cb == 8) fwd_band<8, false, true>(X, b0, t, vA, kA1, kA0, vB, kB1, kB0, pend);
            else if (cb == 4) fwd_band<4, false, true>(X, b0, t, vA, kA1, kA0, vB, kB1, kB0, pend);
            else fwd_band<2, false, true>(X, b0, t, vA, kA1, kA0, vB, kB1, kB0, pend);
            b0 += 32 * cb;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            int ov = __shfl_xor_sync(FULL, vA, o), o1 = __shfl_xor_sync(FULL, kA1, o), o0 = __shfl_xor_sync(FULL, kA0, o);
            if (ov > vA || (ov == vA && ov > 0 && c9_join(o1, o0) < c9_join(kA1, kA0))) { vA = ov; kA1 = o1; kA0 = o0; }
            ov = __shfl_xor_sync(FULL, vB, o); o1 = __shfl_xor_sync(FULL, kB1, o); o0 = __shfl_xor_sync(FULL, kB0, o);
            if (ov > vB || (ov == vB && ov > 0 && c9_join(o1, o0) < c9_join(kB1, kB0))) { vB = ov; kB1 = o1; kB0 = o0; }
        }
        if (t == 0) {
#pragma unroll
            for (int x = 0; x < 2; ++x) {
                if (x == 1 && !has_b) break;
                const int p = x ? pb : pa;
                const int v = x ? vB : vA;
                const uint64_t key = x ? c9_join(kB1, kB0) : c9_join(kA1, kA0);
                A.out_score[p] = v;
                A.out_pos[4 * p] = -1;
                A.out_pos[4 * p + 1] = -1;
                A.out_pos[4 * p + 2] = v > 0 ? (int)((key >> 29) & 0x1fffffffu) : -1;
                A.out_pos[4 * p + 3] = v > 0 ? (int)(key & 0x1fffffffu) : -1;
                if (A.out_len) A.out_len[p] = 0;
            }
        }
        __syncwarp();
    }
}

static size_t sw16ck_smem() { return (size_t)4 * CK_WARP_WORDS * sizeof(uint32_t); }

#undef SW16_NWORK
#undef SW16_WORK

int sw16so_max_slots(int sm_count)
{
    return blocks_per_sm((const void*)sw16so_kernel<false>, 128, sw16ck_smem()) * sm_count * 4;
}

cudaError_t launch_sw16so(const Sw16Args& A, int slots, cudaStream_t st)
{
    if (A.nwork <= 0 && !A.plan) return cudaSuccess;
    if (slots < 4) return cudaErrorInvalidValue;
    launch_begin(K_SW16X2_SCORE, st);
    if (A.plan) sw16so_kernel<true><<<slots / 4, 128, sw16ck_smem(), st>>>(A);
    else sw16so_kernel<false><<<slots / 4, 128, sw16ck_smem(), st>>>(A);
    launch_end(K_SW16X2_SCORE, st);
    return cudaGetLastError();
}

int sw16ck_max_slots(int sm_count, int window)
{
    const int per_sm = window == 4 ? blocks_per_sm((const void*)sw16ck_kernel<4, true, false>, 128, sw16ck_smem())
                                   : blocks_per_sm((const void*)sw16ck_kernel<2, true, false>, 128, sw16ck_smem());
    return per_sm * sm_count * 4;
}

cudaError_t launch_sw16ck(const Sw16Args& A, int slots, int window, bool blocks, cudaStream_t st)
{
    if (A.nwork <= 0 && !A.plan) return cudaSuccess;
    if (window != 2 && window != 4) return cudaErrorInvalidValue;
    const int grid = (slots + 3) / 4;
    launch_begin(K_SW16X2_TRACE, st);
    const bool plan = A.plan != nullptr;
    if (window == 4) {
        if (blocks) plan ? sw16ck_kernel<4, true, true><<<grid, 128, sw16ck_smem(), st>>>(A)
                         : sw16ck_kernel<4, true, false><<<grid, 128, sw16ck_smem(), st>>>(A);
        else plan ? sw16ck_kernel<4, false, true><<<grid, 128, sw16ck_smem(), st>>>(A)
                  : sw16ck_kernel<4, false, false><<<grid, 128, sw16ck_smem(), st>>>(A);
    } else {
        if (blocks) plan ? sw16ck_kernel<2, true, true><<<grid, 128, sw16ck_smem(), st>>>(A)
                         : sw16ck_kernel<2, true, false><<<grid, 128, sw16ck_smem(), st>>>(A);
        else plan ? sw16ck_kernel<2, false, true><<<grid, 128, sw16ck_smem(), st>>>(A)
                  : sw16ck_kernel<2, false, false><<<grid, 128, sw16ck_smem(), st>>>(A);
    }
    launch_end(K_SW16X2_TRACE, st);
    return cudaGetLastError();
}

}  // namespace ga
