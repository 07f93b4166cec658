// sw32ck.cu -- Smith-Waterman with traceback in 32-bit lanes, one pair per
// warp: a score-only forward pass that keeps checkpoints, then the walk over
// 64 x 64 tiles recomputed with direction bits.
//
// The 32-bit form of sw16ck.cu, for pairs the 16-bit kernels cannot take
// (bytes other than A/C/G/T, or scores that could pass 16 bits: long pairs).
// Same recurrence, tie rules and walk as sw.cu (the reference's trace
// recurrence, include/genoaligner/backend/sw_kernel_impl.hip:286-329, walk
// :198-242, best cell = first strict maximum in row-major order):
//
//   1. forward: lanes of CB columns (16 in full bands; the last band takes the
//      smallest of 4, 8, 16 that reaches the last column), H/E/F with DPX
//      (__viaddmax_s32, __vimax3_s32_relu), no predicates; every CK_K-th row
//      each column's (H - gap_open, F) goes to a checkpoint row, every TW-th
//      column each row's (H - gap_open, E) to a column edge; per lane the best
//      value with its first row and column;
//   2. the best cell is the warp's (max value, min row, min column);
//   3. the walk recomputes the K x TW tile holding its current cell from the
//      checkpoint row above and the column edge left of it, with the nibble
//      of predicates sw.cu stores (E chosen, F chosen, E extended, F
//      extended, from __vibmax_s32), and walks inside it.
//
// Two shapes: K = TW = 64 (2 columns per lane in a tile) for pairs up to a
// few million cells, and K = TW = 512 (16 columns per lane) for long pairs,
// whose checkpoints would otherwise take hundreds of MB per warp: the
// checkpoint memory per cell is 16 B / K + 16 B / TW.
//
// Substitution scores: a shared-memory profile for pure-ACGT pairs, byte
// equality otherwise (the reference compares bytes).
#include "kernels.cuh"

namespace ga {

constexpr int C32_PAD = -(1 << 28);      // score past a pattern's end: below any reachable value

__device__ __forceinline__ int c32_code(uint32_t c) { return (int)(((c >> 1) ^ (c >> 2)) & 3u); }

__device__ __forceinline__ bool c32_better(int v, int r, int c, int bv, int br, int bc)
{
    return v > bv || (v == bv && (r < br || (r == br && c < bc)));
}

struct Fwd32 {
    const uint8_t *text, *pat;
    int m, n, ncol;          // ncol: columns the forward bands cover
    int stride;              // checkpoint row stride: ncol rounded up to TW
    int K, TW;               // checkpoint interval (rows), column-edge interval (columns); powers of 2
    int32_t* ck;             // checkpoint rows [q][col][2]
    int32_t* ce;             // column edges [k][row][2]
    int4* prof;              // per warp: 4 letters x CB/4 quads x 32 lanes
    int sm, sx, go, ge;
};

// One band of the forward pass, two rows per step: lane t takes rows
// i = 2 (tau - t) + 1 and i + 1 of its CB columns.  Row i + 1's cell in
// column c needs only row i's cells in columns c - 1 and c, so the two rows'
// dependency chains (E along a row, H through E) are independent at equal
// column and interleave.  COOP: the band is one of a pair's bands run by the
// warps of a block together (fwd32_coop); the warp then meets the block's
// barrier after every 32 steps, ceil(steps / 32) times per band.
template <int CB, bool PROF, bool COOP>
__device__ void fwd32_band(const Fwd32& X, int b0, int t, int& vb, int& rb, int& cb)
{
    constexpr int NQ = CB / 4;
    const int go = X.go, ge = X.ge, m = X.m;
    const int j0 = b0 + t * CB;
    const int nv = max(0, min(CB, X.n - j0));
    uint32_t pb[PROF ? 1 : CB];
    if constexpr (PROF) {
        __syncwarp();
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            int code[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) code[k] = (4 * q + k < nv) ? c32_code(__ldg(X.pat + j0 + 4 * q + k)) : 4;
#pragma unroll
            for (int L = 0; L < 4; ++L) {
                int v[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) v[k] = code[k] == 4 ? C32_PAD : (code[k] == L ? X.sm : X.sx);
                X.prof[(L * NQ + q) * 32 + t] = make_int4(v[0], v[1], v[2], v[3]);
            }
        }
        __syncwarp();
    } else {
#pragma unroll
        for (int c = 0; c < CB; ++c) pb[c] = (c < nv) ? __ldg(X.pat + j0 + c) : 0x100u;
    }
    int hgu[CB], fv[CB];
#pragma unroll
    for (int c = 0; c < CB; ++c) { hgu[c] = -go; fv[c] = 0; }
    // the left neighbour's H - go at the row above this step's first row; what
    // this lane hands right for its two rows
    int diag_in = -go, out_hg0 = -go, out_e0 = 0, out_hg1 = -go, out_e1 = 0;
    const int32_t* left = b0 > 0 ? X.ce + 2 * (int64_t)(b0 / X.TW - 1) * m : nullptr;
    const int kout = (j0 + CB) % X.TW == 0 && j0 + CB < X.ncol ? (j0 + CB) / X.TW : 0;
    int32_t* eout = kout ? X.ce + 2 * (int64_t)(kout - 1) * m : nullptr;
    // each row's text byte (its profile offset with PROF) travels along the lanes
    // with the boundary values; lane 0's inputs of 64 rows at a time -- that and
    // the left edge -- are read by all lanes (lane u: rows 64k + 2u and + 1) and
    // shuffled to lane 0 each step, so no step runs a lane-0-only branch
    uint32_t ch0 = 0, ch1 = 0, rb_ch0 = 0, rb_ch1 = 0;
    int rb_hg0 = -go, rb_e0 = 0, rb_hg1 = -go, rb_e1 = 0;
    int bv = 0, br = 0;                               // this band's best and the first row holding it
    const int steps = (m + 1) / 2 + 31;
    for (int tau = 0; tau < steps; ++tau) {
        if ((tau & 31) == 0 && 2 * tau < m) {
            const int r = 2 * (tau + t);
            if (r < m) {
                const uint32_t c = __ldg(X.text + r);
                rb_ch0 = PROF ? (uint32_t)(c32_code(c) * NQ * 32) : c;
                if (left) {
                    const int2 lv = *reinterpret_cast<const int2*>(left + 2 * r);
                    rb_hg0 = lv.x;
                    rb_e0 = lv.y;
                }
            }
            if (r + 1 < m) {
                const uint32_t c = __ldg(X.text + r + 1);
                rb_ch1 = PROF ? (uint32_t)(c32_code(c) * NQ * 32) : c;
                if (left) {
                    const int2 lv = *reinterpret_cast<const int2*>(left + 2 * (r + 1));
                    rb_hg1 = lv.x;
                    rb_e1 = lv.y;
                }
            }
        }
        int in_hg0 = __shfl_up_sync(FULL, out_hg0, 1);
        int in_e0 = __shfl_up_sync(FULL, out_e0, 1);
        int in_hg1 = __shfl_up_sync(FULL, out_hg1, 1);
        int in_e1 = __shfl_up_sync(FULL, out_e1, 1);
        ch0 = __shfl_up_sync(FULL, ch0, 1);
        ch1 = __shfl_up_sync(FULL, ch1, 1);
        const uint32_t l_ch0 = __shfl_sync(FULL, rb_ch0, tau & 31);
        const int l_hg0 = __shfl_sync(FULL, rb_hg0, tau & 31);
        const int l_e0 = __shfl_sync(FULL, rb_e0, tau & 31);
        const uint32_t l_ch1 = __shfl_sync(FULL, rb_ch1, tau & 31);
        const int l_hg1 = __shfl_sync(FULL, rb_hg1, tau & 31);
        const int l_e1 = __shfl_sync(FULL, rb_e1, tau & 31);
        const int i = 2 * (tau - t) + 1;
        if (t == 0) {
            ch0 = l_ch0; in_hg0 = l_hg0; in_e0 = l_e0;
            ch1 = l_ch1; in_hg1 = l_hg1; in_e1 = l_e1;
        }
        if (i >= 1 && i <= m) {
            int s0[CB], s1[CB];
            if constexpr (PROF) {
#pragma unroll
                for (int q = 0; q < NQ; ++q) {
                    const int4 v = X.prof[ch0 + q * 32 + t];
                    s0[4 * q] = v.x; s0[4 * q + 1] = v.y; s0[4 * q + 2] = v.z; s0[4 * q + 3] = v.w;
                    const int4 w = X.prof[ch1 + q * 32 + t];
                    s1[4 * q] = w.x; s1[4 * q + 1] = w.y; s1[4 * q + 2] = w.z; s1[4 * q + 3] = w.w;
                }
            } else {
#pragma unroll
                for (int c = 0; c < CB; ++c) {
                    s0[c] = c < nv ? (ch0 == pb[c] ? X.sm : X.sx) : C32_PAD;
                    s1[c] = c < nv ? (ch1 == pb[c] ? X.sm : X.sx) : C32_PAD;
                }
            }
            int hgd0 = diag_in, hgl0 = in_hg0, el0 = in_e0;
            int hgd1 = in_hg0, hgl1 = in_hg1, el1 = in_e1;
            int rowmax0 = 0, rowmax1 = 0;
#pragma unroll
            for (int c = 0; c < CB; ++c) {
                // row i
                const int e0 = __viaddmax_s32(el0, -ge, hgl0);        // max(E_left - ge, H_left - go)
                const int f0 = __viaddmax_s32(fv[c], -ge, hgu[c]);    // max(F_up - ge, H_up - go)
                const int h0 = __vimax3_s32_relu(hgd0 + s0[c], e0, f0); // max(H_diag + s, E, F, 0)
                const int hg0 = h0 - go;
                rowmax0 = max(rowmax0, h0);
                hgd0 = hgu[c];
                // row i + 1: up is row i's cell just computed
                const int e1 = __viaddmax_s32(el1, -ge, hgl1);
                const int f1 = __viaddmax_s32(f0, -ge, hg0);
                const int h1 = __vimax3_s32_relu(hgd1 + s1[c], e1, f1);
                const int hg1 = h1 - go;
                rowmax1 = max(rowmax1, h1);
                hgd1 = hg0;
                hgu[c] = hg1;
                fv[c] = f1;
                hgl0 = hg0; el0 = e0;
                hgl1 = hg1; el1 = e1;
            }
            diag_in = in_hg1;
            out_hg0 = hgl0; out_e0 = el0;
            out_hg1 = hgl1; out_e1 = el1;
            const bool two = i + 1 <= m;
            if (eout) {
                *reinterpret_cast<int2*>(eout + 2 * (i - 1)) = make_int2(out_hg0, out_e0);
                if (two) *reinterpret_cast<int2*>(eout + 2 * i) = make_int2(out_hg1, out_e1);
            }
            if (((i + 1) & (X.K - 1)) == 0 && i + 1 < m) {           // checkpoint row i + 1 (i is odd, K even)
                int4* dst = reinterpret_cast<int4*>(X.ck + 2 * ((int64_t)((i + 1) / X.K - 1) * X.stride + j0));
#pragma unroll
                for (int c = 0; c < CB; c += 2) dst[c >> 1] = make_int4(hgu[c], fv[c], hgu[c + 1], fv[c + 1]);
            }
            if (rowmax0 > bv) { bv = rowmax0; br = i; }        // first row holding this lane's best
            if (two && rowmax1 > bv) { bv = rowmax1; br = i + 1; }
        }
        if (COOP && ((tau & 31) == 31 || tau == steps - 1)) __syncthreads();
    }
    // the column kept is the first of the lane's span in this band (spans
    // order like their columns); the walk finds the cell's column in that row
    if (bv > 0 && c32_better(bv, br, j0 + 1, vb, rb, cb)) { vb = bv; rb = br; cb = j0 + 1; }
    __syncwarp();
}

template <bool PROF>
__device__ void fwd32(const Fwd32& X, int t, int& vb, int& rb, int& cb)
{
    for (int b0 = 0; b0 < X.n;) {
        const int rest = X.n - b0;
        const int w = rest > C32_BW ? C32_C : c32_last_cb(rest);
        if (w == 16) fwd32_band<16, PROF, false>(X, b0, t, vb, rb, cb);
        else if (w == 8) fwd32_band<8, PROF, false>(X, b0, t, vb, rb, cb);
        else fwd32_band<4, PROF, false>(X, b0, t, vb, rb, cb);
        b0 += 32 * w;
    }
}

// The forward pass of one pair by the W warps of a block (W = blockDim / 32,
// 4 or 8): band b runs on warp b % W, starting at 32-step chunk start(b) =
// max(start(b-1) + 2, start(b-W) + chunks per band), so each band's first lane reads the left edge of rows
// 64c+1 .. 64c+64 (written by the band before it up to its step 32c + 62)
// after the barrier that closed that band's chunk c + 1, and each warp runs
// its bands one after the other.  Every warp meets the block barrier once per
// chunk, idle or not: start(last band) + chunks per band times in all.
template <bool PROF>
__device__ void fwd32_coop(const Fwd32& X, int t, int wib, int& vb, int& rb, int& cb)
{
    const int W = blockDim.x >> 5;                    // warps of the block (at most C32_MAX_WARPS)
    const int nck = ((X.m + 1) / 2 + 62) / 32;        // chunks per band: ceil(steps / 32)
    int g = 0, prev = -2, b = 0;
    int stw[C32_MAX_WARPS];                           // start of the last band of each warp
#pragma unroll
    for (int q = 0; q < C32_MAX_WARPS; ++q) stw[q] = 0;
    for (int b0 = 0; b0 < X.n; ++b) {
        const int rest = X.n - b0;
        const int w = rest > C32_BW ? C32_C : c32_last_cb(rest);
        const int ow = b % W;
        int own = 0;
#pragma unroll
        for (int q = 0; q < C32_MAX_WARPS; ++q)
            if (q == ow) own = stw[q];
        const int s = max(prev + 2, b >= W ? own + nck : 0);
        prev = s;
#pragma unroll
        for (int q = 0; q < C32_MAX_WARPS; ++q)
            if (q == ow) stw[q] = s;
        if (ow == wib) {
            for (; g < s; ++g) __syncthreads();
            if (w == 16) fwd32_band<16, PROF, true>(X, b0, t, vb, rb, cb);
            else if (w == 8) fwd32_band<8, PROF, true>(X, b0, t, vb, rb, cb);
            else fwd32_band<4, PROF, true>(X, b0, t, vb, rb, cb);
            g += nck;
        }
        b0 += 32 * w;
    }
    const int G = prev + nck;
    for (; g < G; ++g) __syncthreads();
}

// Shared memory per warp: the forward profile (4 letters x 4 quads x 32
// lanes of int4), reused by a tile's profile (4 letters x CT/4 quads x 32
// lanes, or int2 pairs for CT = 2) followed by its K left-edge rows.
__host__ __device__ constexpr int c32_warp_smem_bytes(int K, int CT)
{
    return (4 * (C32_C / 4) * 32 * 16) > (4 * CT * 32 * 4 + K * 8) ? (4 * (C32_C / 4) * 32 * 16)
                                                                      : (4 * CT * 32 * 4 + K * 8);
}

// One pair: the forward pass (by this warp, or by the block's 4 warps when
// coop), the best cell, the walk (this warp, or warp 0 of the block) and the
// outputs.  wslot: the pair's checkpoint/tile memory (warp 0's slot when
// coop); wsm: this warp's shared memory.  In coop every warp returns after
// the same barriers; the caller closes the pair with one more barrier.
template <int K, int CT>
__device__ void c32_pair(const SwArgs& A, int p, bool coop, int wib, int t, uint32_t* wslot, unsigned char* wsm,
                         int (*s_best)[3])
{
    constexpr int TW = 32 * CT;
    constexpr int NWT = CT >= 8 ? CT / 8 : 1;            // nibble words per lane and step
    int4* prof = reinterpret_cast<int4*>(wsm);
    const int go = A.gap_open, ge = A.gap_extend;
    const int sm = A.match + go, sx = A.mismatch + go;
    const int m = A.D.a_len[p], n = A.D.b_len[p];
    const uint8_t* text = A.D.seq + A.D.a_off[p];
    const uint8_t* pat = A.D.seq + A.D.b_off[p];
    if (m <= 0 || n <= 0) {
        if (t == 0 && (!coop || wib == 0)) {
            A.out_score[p] = 0;
            A.out_pos[4 * p] = A.out_pos[4 * p + 1] = A.out_pos[4 * p + 2] = A.out_pos[4 * p + 3] = -1;
            A.out_len[p] = 0;
        }
        return;
    }
    const bool pure = A.D.pure && A.D.pure[p] && A.D.pure[A.D.n + p];
    // tiles reach up to a multiple of TW: checkpoint rows are that wide (the
    // columns past the forward bands are padding, never read into a real cell)
    const int ncol = c32_ncol(n);
    const int stride = (ncol + TW - 1) / TW * TW;
    const int nq = c32_rows(m, K);
    int32_t* ck = reinterpret_cast<int32_t*>(wslot);
    int32_t* ce = ck + 2 * (int64_t)nq * stride;
    uint32_t* tile = reinterpret_cast<uint32_t*>(ce + 2 * (int64_t)(stride / TW) * m);

    // ------------------------------------------------ forward pass --
    int vb = 0, rb = 0, cb = 0;
    {
        Fwd32 X{text, pat, m, n, ncol, stride, K, TW, ck, ce, prof, sm, sx, go, ge};
        if (coop) {
            if (pure) fwd32_coop<true>(X, t, wib, vb, rb, cb);
            else fwd32_coop<false>(X, t, wib, vb, rb, cb);
        } else {
            if (pure) fwd32<true>(X, t, vb, rb, cb);
            else fwd32<false>(X, t, vb, rb, cb);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const int ov = __shfl_xor_sync(FULL, vb, o), orr = __shfl_xor_sync(FULL, rb, o), oc = __shfl_xor_sync(FULL, cb, o);
        if (ov > 0 && c32_better(ov, orr, oc, vb, rb, cb)) { vb = ov; rb = orr; cb = oc; }
    }
    if (coop) {
        // the block's best: every warp reduces the four warps' bests in the same order
        if (t == 0) { s_best[wib][0] = vb; s_best[wib][1] = rb; s_best[wib][2] = cb; }
        __syncthreads();
        vb = s_best[0][0]; rb = s_best[0][1]; cb = s_best[0][2];
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) {
            const int ov = s_best[q][0], orr = s_best[q][1], oc = s_best[q][2];
            if (ov > 0 && c32_better(ov, orr, oc, vb, rb, cb)) { vb = ov; rb = orr; cb = oc; }
        }
        if (wib != 0) return;                     // the walk is warp 0's
    }
    if (vb <= 0) {
        if (t == 0) {
            A.out_score[p] = 0;
            A.out_pos[4 * p] = A.out_pos[4 * p + 1] = A.out_pos[4 * p + 2] = A.out_pos[4 * p + 3] = -1;
            A.out_len[p] = 0;
        }
        return;
    }

    // ----------------------------------------------------- the walk --
    char* slotc = A.out_cigar + A.D.out_off[p];
    int pos = m + n;
    int i = rb, j = cb, state = 0, v = vb;
    int ti0 = ((i - 1) / K) * K + 1, tb = (j - 1) / TW;
    bool first = true;                                          // the best cell's column not yet found
    int* edg = reinterpret_cast<int*>(wsm + 4 * CT * 32 * 4);     // [row][2], after the tile profile
    bool fin = false;
    while (!fin) {
        const int rows = i - ti0 + 1;
        const int steps = rows + 31;
        const int col0 = TW * tb;
        __syncwarp();
        // tile profile (pure pairs) or bytes, top state, left edges
        uint32_t pbt[CT];
        {
            const int cl = col0 + CT * t;
            if (pure) {
                int code[CT];
#pragma unroll
                for (int c = 0; c < CT; ++c) code[c] = cl + c < n ? c32_code(__ldg(pat + cl + c)) : 4;
                if constexpr (CT == 2) {
                    int2* tp = reinterpret_cast<int2*>(wsm);
#pragma unroll
                    for (int L = 0; L < 4; ++L) tp[L * 32 + t] = make_int2(code[0] == L ? sm : sx, code[1] == L ? sm : sx);
                } else {
                    int4* tp = reinterpret_cast<int4*>(wsm);
#pragma unroll
                    for (int L = 0; L < 4; ++L)
#pragma unroll
                        for (int q4 = 0; q4 < CT / 4; ++q4)
                            tp[(L * (CT / 4) + q4) * 32 + t] =
                                make_int4(code[4 * q4] == L ? sm : sx, code[4 * q4 + 1] == L ? sm : sx,
                                          code[4 * q4 + 2] == L ? sm : sx, code[4 * q4 + 3] == L ? sm : sx);
                }
            }
#pragma unroll
            for (int c = 0; c < CT; ++c) pbt[c] = (!pure && cl + c < n) ? __ldg(pat + cl + c) : 0x100u;
        }
        const int q = (ti0 - 1) / K - 1;
        const int32_t* crow = ck + 2 * (int64_t)max(q, 0) * stride;
        int hgu[CT], fv[CT];
#pragma unroll
        for (int c = 0; c < CT; ++c) {
            hgu[c] = q >= 0 ? crow[2 * (col0 + CT * t + c)] : -go;
            fv[c] = q >= 0 ? crow[2 * (col0 + CT * t + c) + 1] : 0;
        }
        int diag_in = __shfl_up_sync(FULL, hgu[CT - 1], 1);
        if (t == 0) diag_in = (q >= 0 && tb > 0) ? crow[2 * (col0 - 1)] : -go;
        {
            const int32_t* le = tb > 0 ? ce + 2 * ((int64_t)(tb - 1) * m + (ti0 - 1)) : nullptr;
            for (int r = t; r < K; r += 32) {
                edg[2 * r] = (le && r < rows) ? le[2 * r] : -go;
                edg[2 * r + 1] = (le && r < rows) ? le[2 * r + 1] : 0;
            }
        }
        __syncwarp();
        int out_hg = -go, out_e = 0;
        int jfound = INT32_MAX;
        const uint8_t* tx = text + (ti0 - 1);
        uint32_t ch = 0, ch_next = t == 0 ? (uint32_t)__ldg(tx) : 0u;
        for (int tau = 0; tau < steps; ++tau) {
            int in_hg = __shfl_up_sync(FULL, out_hg, 1);
            int in_e = __shfl_up_sync(FULL, out_e, 1);
            ch = __shfl_up_sync(FULL, ch, 1);
            const int r = tau - t + 1;                                  // tile row, 1-based
            if (t == 0) {
                ch = ch_next;
                if (r < rows) ch_next = __ldg(tx + r);
                if (r <= rows) { in_hg = edg[2 * (r - 1)]; in_e = edg[2 * (r - 1) + 1]; }
            }
            if (r < 1 || r > rows) continue;
            int s[CT];
            if (pure) {
                const int L = c32_code(ch);
                if constexpr (CT == 2) {
                    const int2 v2 = reinterpret_cast<const int2*>(wsm)[L * 32 + t];
                    s[0] = v2.x;
                    s[1] = v2.y;
                } else {
#pragma unroll
                    for (int q4 = 0; q4 < CT / 4; ++q4) {
                        const int4 v4 = reinterpret_cast<const int4*>(wsm)[(L * (CT / 4) + q4) * 32 + t];
                        s[4 * q4] = v4.x; s[4 * q4 + 1] = v4.y; s[4 * q4 + 2] = v4.z; s[4 * q4 + 3] = v4.w;
                    }
                }
            } else {
#pragma unroll
                for (int c = 0; c < CT; ++c) s[c] = ch == pbt[c] ? sm : sx;
            }
            int hgd = diag_in, hgl = in_hg, el = in_e;
            uint32_t nib[NWT];
#pragma unroll
            for (int wq = 0; wq < NWT; ++wq) nib[wq] = 0;
#pragma unroll
            for (int c = 0; c < CT; ++c) {
                bool pe, pf, p1, p2;
                const int h0 = hgd + s[c];
                const int e = __vibmax_s32(hgl, el - ge, &pe);            // open wins ties
                const int f = __vibmax_s32(hgu[c], fv[c] - ge, &pf);
                const int h1 = __vibmax_s32(h0, e, &p1);                  // diagonal wins ties
                const int h2 = __vibmax_s32(h1, f, &p2);
                const int h = max(h2, 0);
                nib[c >> 3] |= ((uint32_t)!p1 | ((uint32_t)!p2 << 1) | ((uint32_t)!pe << 2) | ((uint32_t)!pf << 3))
                               << (4 * (c & 7));
                const int hg = h - go;
                hgd = hgu[c];
                hgu[c] = hg;
                fv[c] = f;
                hgl = hg;
                el = e;
            }
#pragma unroll
            for (int wq = 0; wq < NWT; ++wq) tile[(tau * 32 + t) * NWT + wq] = nib[wq];
            if (first && r == rows) {                           // the best cell's row
#pragma unroll
                for (int c = CT - 1; c >= 0; --c) {
                    const int col = col0 + CT * t + c;
                    if (col < n && hgu[c] + go == vb) jfound = col + 1;
                }
            }
            diag_in = in_hg;
            out_hg = hgl;
            out_e = el;
        }
        __syncwarp();
        if (first) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) jfound = min(jfound, __shfl_xor_sync(FULL, jfound, o));
            first = false;
            if (jfound == INT32_MAX) {             // cannot happen: the forward pass saw the value here
                if (t == 0) atomicOr(A.err, ERR_BAD_INPUT);
                break;
            }
            j = jfound;
            cb = jfound;
        }
        // walk inside the tile: state 0 on H, 1 in an E run ('D'), 2 in an F run ('I')
        const int jlo = col0 + 1;
        for (;;) {
            if (i <= 0 || j <= 0 || (state == 0 && v == 0)) { fin = true; break; }
            if (i < ti0 || j < jlo) break;
            if (state == 0) {
                // a run of diagonal steps resolved at once: lane u takes the step from
                // cell (i - u, j - u); its value is v less the scores of steps 0 .. u-1
                const int U = min(min(32, pos), min(i - max(ti0, 1), j - max(jlo, 1)) + 1);
                bool diag = false, eq = false;
                int s = 0;
                if (t < U) {
                    const int jq = j - t - jlo;
                    const int tq = jq / CT, cq = jq - tq * CT;
                    const uint32_t nq = tile[(((i - t - ti0) + tq) * 32 + tq) * NWT + (cq >> 3)] >> (4 * (cq & 7));
                    diag = (nq & 3u) == 0u;
                    eq = __ldg(text + i - 1 - t) == __ldg(pat + j - 1 - t);
                    s = eq ? A.match : A.mismatch;
                }
                int incl = s;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(FULL, incl, o);
                    if (t >= o) incl += y;
                }
                const bool ok = t < U && diag && v - (incl - s) != 0;
                const unsigned run = __ballot_sync(FULL, ok);
                const int r = run == FULL ? 32 : __ffs(~run) - 1;
                if (r > 0) {
                    if (t < r) slotc[pos - 1 - t] = eq ? 'M' : 'X';
                    v -= __shfl_sync(FULL, incl, r - 1);
                    i -= r;
                    j -= r;
                    pos -= r;
                    continue;
                }
            }
            const int jj = j - jlo;
            const int tt = jj / CT, c = jj - tt * CT;
            const uint32_t nb4 = (tile[(((i - ti0) + tt) * 32 + tt) * NWT + (c >> 3)] >> (4 * (c & 7))) & 15u;
            char op;
            if (state == 0) {
                if (nb4 & 2u) {
                    op = 'I';
                    if (nb4 & 8u) { state = 2; v += ge; } else { v += go; }
                    --i;
                } else if (nb4 & 1u) {
                    op = 'D';
                    if (nb4 & 4u) { state = 1; v += ge; } else { v += go; }
                    --j;
                } else {
                    const uint8_t ta = __ldg(text + i - 1), pc = __ldg(pat + j - 1);
                    op = ta == pc ? 'M' : 'X';
                    v -= ta == pc ? A.match : A.mismatch;
                    --i;
                    --j;
                }
            } else if (state == 1) {
                op = 'D';
                if (nb4 & 4u) { v += ge; } else { v += go; state = 0; }
                --j;
            } else {
                op = 'I';
                if (nb4 & 8u) { v += ge; } else { v += go; state = 0; }
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
        if (!fin) {
            if (i < ti0) ti0 = ((i - 1) / K) * K + 1;
            tb = (j - 1) / TW;
        }
    }
    if (t == 0) {
        A.out_score[p] = vb;
        A.out_pos[4 * p] = i;
        A.out_pos[4 * p + 1] = j;
        A.out_pos[4 * p + 2] = rb - 1;
        A.out_pos[4 * p + 3] = cb - 1;
        A.out_len[p] = m + n - pos;
    }
}

// Work items come largest first.  Items above A.coop_cells cells are taken by
// a whole block (its 4 warps share the forward pass); from the first smaller
// item on, each warp takes items of its own.
// PLAN: items and per-warp memory from the device-built plan (plan_view),
// the list and its length kept in shared memory; otherwise the launch's own.
template <int K, int CT, bool PLAN>
__global__ void __launch_bounds__(128, 4) sw32ck_kernel(SwArgs A)
{
    constexpr int WSB = c32_warp_smem_bytes(K, CT);
    extern __shared__ int4 c32_smem[];
    __shared__ int s_item;
    __shared__ int s_best[C32_MAX_WARPS][3];
    __shared__ const int32_t* s_work;
    __shared__ int s_nwork;
    const int t = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    int64_t dir_slot = A.dir_slot;
    if constexpr (PLAN) {
        const PlanView V = plan_view(A.plan, A.plan_list, A.work, A.nwork, A.nwork_dev, A.dir_slot, A.edge_slot,
                                     A.dir_cap, A.edge_cap, A.err);
        if (!V.run) return;
        dir_slot = V.dir_slot;
        if (threadIdx.x == 0) { s_work = V.work; s_nwork = V.nwork; }
        __syncthreads();
    }
    uint32_t* wslot = A.dirs + ((int64_t)blockIdx.x * (blockDim.x >> 5) + wib) * dir_slot;
    uint32_t* bslot = A.dirs + (int64_t)blockIdx.x * (blockDim.x >> 5) * dir_slot;
    unsigned char* wsm = reinterpret_cast<unsigned char*>(c32_smem) + wib * WSB;
    const int nwork = PLAN ? s_nwork : (A.nwork_dev ? *A.nwork_dev : A.nwork);
#define SW32_WORK (PLAN ? s_work : A.work)
    // one call site of c32_pair, so its body is in the kernel once
    bool block_phase = A.coop_cells >= 0;
    for (;;) {
        int w = -1;
        bool coop = false;
        if (block_phase) {
            if (threadIdx.x == 0) s_item = atomicAdd(A.counter, 1);
            __syncthreads();
            const int wb = s_item;
            __syncthreads();
            if (wb >= nwork) break;
            const int p = SW32_WORK[wb];
            if ((int64_t)A.D.a_len[p] * A.D.b_len[p] > A.coop_cells) {
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
            if (w >= nwork) break;
        }
        __syncwarp();
        c32_pair<K, CT>(A, SW32_WORK[w], coop, wib, t, coop ? bslot : wslot, wsm, s_best);
        if (coop) __syncthreads();
    }
}
#undef SW32_WORK

template <int K, int CT>
static size_t c32_smem(int warps = 4) { return (size_t)warps * c32_warp_smem_bytes(K, CT); }

int sw32ck_max_slots(bool long_pairs, int sm_count)
{
    if (long_pairs) {
        // both variants launch with this shared memory: raise both limits
        blocks_per_sm((const void*)sw32ck_kernel<512, 16, true>, 128, c32_smem<512, 16>());
        return blocks_per_sm((const void*)sw32ck_kernel<512, 16, false>, 128, c32_smem<512, 16>()) * sm_count * 4;
    }
    blocks_per_sm((const void*)sw32ck_kernel<64, 2, true>, 128, c32_smem<64, 2>());
    return blocks_per_sm((const void*)sw32ck_kernel<64, 2, false>, 128, c32_smem<64, 2>()) * sm_count * 4;
}

// slots: warp slots of A.dirs, a multiple of 4 (blocks of 4 warps).
cudaError_t launch_sw32ck(const SwArgs& A, bool long_pairs, int slots, cudaStream_t st)
{
    if (A.nwork <= 0 && !A.nwork_dev && !A.plan) return cudaSuccess;
    if (slots < 4) return cudaErrorInvalidValue;
    launch_begin(K_SW32_TRACE, st);
    if (A.plan) {
        if (long_pairs) sw32ck_kernel<512, 16, true><<<slots / 4, 128, c32_smem<512, 16>(), st>>>(A);
        else sw32ck_kernel<64, 2, true><<<slots / 4, 128, c32_smem<64, 2>(), st>>>(A);
    } else {
        if (long_pairs) sw32ck_kernel<512, 16, false><<<slots / 4, 128, c32_smem<512, 16>(), st>>>(A);
        else sw32ck_kernel<64, 2, false><<<slots / 4, 128, c32_smem<64, 2>(), st>>>(A);
    }
    launch_end(K_SW32_TRACE, st);
    return cudaGetLastError();
}

}  // namespace ga
