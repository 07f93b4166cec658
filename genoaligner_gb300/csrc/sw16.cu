// sw16.cu -- Smith-Waterman traceback kernel, two pairs per warp in 16-bit lanes.
//
// Same recurrence, tie rules and walk as sw.cu (the reference's trace
// recurrence, include/genoaligner/backend/sw_kernel_impl.hip:286-329, and walk
// :198-242); what changes is the arithmetic width.  On this GPU the integer
// max/compare/logic pipe retires 64 lanes per clock per SM and is what bounds
// the 32-bit kernel, while DPX 16x2 operations (__viaddmax_s16x2,
// __vimax3_s16x2, __vmaxs2) retire one instruction for two cells.  So a warp
// here carries two pairs at once, pair A in the low and pair B in the high
// 16 bits of every register, through the same lagged-lane schedule as sw.cu.
//
// Eligibility (checked on the host): both pairs consist of A, C, G, T only;
// match * min(m, n) + BIAS < 32000, gap_open + gap_extend < BIAS, and
// mismatch + gap_open >= 0.  Every value v is stored as v + BIAS, so each half
// stays in [0, 32767]: 32-bit additions of non-negative per-half constants
// never carry across halves, and signed 16-bit max works unchanged.
//
// Direction predicates come from sign bits: for a >= b in both halves,
// d = a - b + 0x80008000 has bit 15 (pair A) and bit 31 (pair B) set.  Per
// group of 8 cells, four accumulators collect those bits by shift-and-or
// (cell c ends up at bit 8+c and 24+c), and two byte permutes split them into
// one 32-bit word per pair: byte k = predicate k, bit c = cell c, with
//   k = 0: H did not come from E      (diag >= e)
//   k = 1: H did not come from F      (max(diag, e) >= f)
//   k = 2: E was opened, not extended (H_left - go >= E_left - ge)
//   k = 3: F was opened, not extended (H_up - go >= F_up - ge)
#include "kernels.cuh"

namespace ga {


__device__ __forceinline__ int code2_16(uint32_t c) { return (int)(((c >> 1) ^ (c >> 2)) & 3u); }

// two 16-bit halves -> unbiased signed ints
__device__ __forceinline__ int lo16(uint32_t x) { return (int)(x & 0xffffu) - BIAS16; }
__device__ __forceinline__ int hi16(uint32_t x) { return (int)(x >> 16) - BIAS16; }

template <int C>
__global__ void __launch_bounds__(128) sw16_kernel(Sw16Args A)
{
    constexpr int BW = 32 * C, NW = C / 8, NH = C / 2;
    extern __shared__ uint32_t prof16_smem[];
    const int t = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int64_t slot = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    uint32_t* dslot = A.dirs + slot * A.dir_slot;               // pair A table, then pair B table
    uint32_t* eslot = reinterpret_cast<uint32_t*>(A.edge + slot * A.edge_slot);
    // profile: [pair][letter][column pair h][lane], 16-bit scores packed per column pair
    uint32_t* prof = prof16_smem + wib * (2 * 4 * NH * 32);
    const int go = A.gap_open, ge = A.gap_extend;
    const uint32_t B2 = (uint32_t)BIAS16 * 0x10001u;
    const uint32_t NGE2 = (uint32_t)(-ge) & 0xffffu;
    const uint32_t NGE2x = NGE2 | (NGE2 << 16);
    const uint32_t K2 = 0x80008000u;
    const uint32_t GO2 = (uint32_t)go * 0x10001u;
    const uint32_t KGE2 = K2 + (uint32_t)ge * 0x10001u;

    for (;;) {
        int w = 0;
        if (t == 0) w = atomicAdd(A.counter, 1);
        w = __shfl_sync(FULL, w, 0);
        if (w >= A.nwork) break;
        __syncwarp();
        const int pa = A.work[2 * w], pb = A.work[2 * w + 1] >= 0 ? A.work[2 * w + 1] : A.work[2 * w];
        const bool has_b = A.work[2 * w + 1] >= 0;
        const int mA = A.D.a_len[pa], nA = A.D.b_len[pa];
        const int mB = A.D.a_len[pb], nB = A.D.b_len[pb];
        const uint8_t* textA = A.D.seq + A.D.a_off[pa];
        const uint8_t* patA = A.D.seq + A.D.b_off[pa];
        const uint8_t* textB = A.D.seq + A.D.a_off[pb];
        const uint8_t* patB = A.D.seq + A.D.b_off[pb];
        const int M = max(mA, mB), N = max(nA, nB);
        const int nb = (N + BW - 1) / BW;
        const int steps = M + 31;
        const int64_t table = (int64_t)nb * steps * 32 * NW;      // words per pair table
        int bestA = 0, biA = 0, bjA = 0, bestB = 0, biB = 0, bjB = 0;

        for (int b = 0; b < nb; ++b) {
            const int j0 = b * BW + t * C;
            const int nvA = max(0, min(C, nA - j0)), nvB = max(0, min(C, nB - j0));
            __syncwarp();
#pragma unroll
            for (int h = 0; h < NH; ++h) {
                const int c0 = 2 * h, c1 = 2 * h + 1;
                const int a0 = c0 < nvA ? code2_16(__ldg(patA + j0 + c0)) : 4;
                const int a1 = c1 < nvA ? code2_16(__ldg(patA + j0 + c1)) : 4;
                const int b0 = c0 < nvB ? code2_16(__ldg(patB + j0 + c0)) : 4;
                const int b1 = c1 < nvB ? code2_16(__ldg(patB + j0 + c1)) : 4;
                const int sm = A.match + go, sx = A.mismatch + go;
#pragma unroll
                for (int L = 0; L < 4; ++L) {
                    prof[((0 * 4 + L) * NH + h) * 32 + t] =
                        (uint32_t)(a0 == L ? sm : sx) | ((uint32_t)(a1 == L ? sm : sx) << 16);
                    prof[((1 * 4 + L) * NH + h) * 32 + t] =
                        (uint32_t)(b0 == L ? sm : sx) | ((uint32_t)(b1 == L ? sm : sx) << 16);
                }
            }
            __syncwarp();
            uint32_t hgu[C], fv[C];
#pragma unroll
            for (int c = 0; c < C; ++c) { hgu[c] = B2 - GO2; fv[c] = B2; }
            uint32_t diag_in = B2 - GO2, out_hg = B2 - GO2, out_e = B2;
            const bool left_edge = (t == 0) && (b > 0);
            uint32_t nxt_hg = B2 - GO2, nxt_e = B2;
            if (left_edge) { nxt_hg = eslot[0]; nxt_e = eslot[1]; }
            uint32_t aA_next = (t == 0) ? __ldg(textA) : 'A', aB_next = (t == 0) ? __ldg(textB) : 'A';
            for (int tau = 0; tau < steps; ++tau) {
                uint32_t in_hg = __shfl_up_sync(FULL, out_hg, 1);
                uint32_t in_e = __shfl_up_sync(FULL, out_e, 1);
                const int i = tau - t + 1;
                const uint32_t aA = aA_next, aB = aB_next;
                if (i >= 0 && i < M) {
                    aA_next = i < mA ? __ldg(textA + i) : 'A';
                    aB_next = i < mB ? __ldg(textB + i) : 'A';
                }
                if (t == 0) {
                    if (b == 0) { in_hg = B2 - GO2; in_e = B2; }
                    else { in_hg = nxt_hg; in_e = nxt_e; }
                    if (left_edge && i >= 1 && i < M) { nxt_hg = eslot[2 * i]; nxt_e = eslot[2 * i + 1]; }
                }
                if (i < 1 || i > M) continue;
                const uint32_t* pA = prof + ((0 * 4 + code2_16(aA)) * NH) * 32 + t;
                const uint32_t* pB = prof + ((1 * 4 + code2_16(aB)) * NH) * 32 + t;
                uint32_t hgd = diag_in, hgl = in_hg, el = in_e;
                uint32_t rowmax = B2;
                uint32_t dwA[NW], dwB[NW];
#pragma unroll
                for (int g = 0; g < NW; ++g) {
                    uint32_t acc0 = 0, acc1 = 0, acc2 = 0, acc3 = 0;
#pragma unroll
                    for (int cc = 0; cc < 8; cc += 2) {
                        const int c = 8 * g + cc;
                        const uint32_t wa = pA[(c >> 1) * 32], wb = pB[(c >> 1) * 32];
                        const uint32_t S0 = __byte_perm(wa, wb, 0x5410), S1 = __byte_perm(wa, wb, 0x7632);
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            const int cu = c + u;
                            const uint32_t S = u ? S1 : S0;
                            const uint32_t e = __viaddmax_s16x2(el, NGE2x, hgl);      // max(E_left - ge, H_left - go)
                            const uint32_t f = __viaddmax_s16x2(fv[cu], NGE2x, hgu[cu]);
                            const uint32_t h0 = hgd + S;                              // H_diag + s (biased)
                            const uint32_t h1 = __vmaxs2(h0, e);
                            const uint32_t hh = __vimax3_s16x2(h1, f, B2);            // max(h0, e, f, 0)
                            acc0 = (acc0 >> 1) | ((h0 - e + K2) & K2);
                            acc1 = (acc1 >> 1) | ((h1 - f + K2) & K2);
                            acc2 = (acc2 >> 1) | ((hgl - el + KGE2) & K2);
                            acc3 = (acc3 >> 1) | ((hgu[cu] - fv[cu] + KGE2) & K2);
                            const uint32_t hg = hh - GO2;
                            hgd = hgu[cu];
                            hgu[cu] = hg;
                            fv[cu] = f;
                            hgl = hg;
                            el = e;
                            rowmax = __vmaxs2(rowmax, hh);
                        }
                    }
                    const uint32_t t01 = __byte_perm(acc0, acc1, 0x7351);
                    const uint32_t t23 = __byte_perm(acc2, acc3, 0x7351);
                    dwA[g] = __byte_perm(t01, t23, 0x5410);
                    dwB[g] = __byte_perm(t01, t23, 0x7632);
                }
                diag_in = in_hg;
                out_hg = hgl;
                out_e = el;
                {
                    uint32_t* dA = dslot + ((int64_t)(b * steps + tau) * 32 + t) * NW;
                    uint32_t* dB = dA + table;
                    if constexpr (NW == 1) { dA[0] = dwA[0]; dB[0] = dwB[0]; }
                    else if constexpr (NW == 2) {
                        *reinterpret_cast<uint2*>(dA) = make_uint2(dwA[0], dwA[1]);
                        *reinterpret_cast<uint2*>(dB) = make_uint2(dwB[0], dwB[1]);
                    } else {
                        *reinterpret_cast<uint4*>(dA) = make_uint4(dwA[0], dwA[1], dwA[2], dwA[3]);
                        *reinterpret_cast<uint4*>(dB) = make_uint4(dwB[0], dwB[1], dwB[2], dwB[3]);
                    }
                }
                if (t == 31 && b + 1 < nb) { eslot[2 * (i - 1)] = out_hg; eslot[2 * (i - 1) + 1] = out_e; }
                // best cells (row-major first), per pair; padding columns and rows
                // never exceed the running best (mismatch < 0), so the masked scan
                // runs only when a valid cell may improve it
                const int rA = lo16(rowmax), rB = hi16(rowmax);
                if (nvA > 0 && i <= mA && (rA > bestA || (rA == bestA && rA > 0 && i < biA))) {
                    int mx = 0, first = -1;
#pragma unroll
                    for (int c = 0; c < C; ++c) {
                        const int h = lo16(hgu[c]) + go;
                        if (c < nvA && h > mx) { mx = h; first = c; }
                    }
                    if (first >= 0 && (mx > bestA || (mx == bestA && i < biA))) { bestA = mx; biA = i; bjA = j0 + first + 1; }
                }
                if (nvB > 0 && i <= mB && (rB > bestB || (rB == bestB && rB > 0 && i < biB))) {
                    int mx = 0, first = -1;
#pragma unroll
                    for (int c = 0; c < C; ++c) {
                        const int h = hi16(hgu[c]) + go;
                        if (c < nvB && h > mx) { mx = h; first = c; }
                    }
                    if (first >= 0 && (mx > bestB || (mx == bestB && i < biB))) { bestB = mx; biB = i; bjB = j0 + first + 1; }
                }
            }
            __syncwarp();
        }

        // per pair: warp reduction of the best cell, then the walk
        for (int which = 0; which < (has_b ? 2 : 1); ++which) {
            int best = which ? bestB : bestA, bi = which ? biB : biA, bj = which ? bjB : bjA;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const int ob = __shfl_xor_sync(FULL, best, o);
                const int oi = __shfl_xor_sync(FULL, bi, o);
                const int oj = __shfl_xor_sync(FULL, bj, o);
                if (ob > best || (ob == best && ob > 0 && (oi < bi || (oi == bi && oj < bj)))) {
                    best = ob; bi = oi; bj = oj;
                }
            }
            const int p = which ? pb : pa;
            const int m = which ? mB : mA, n = which ? nB : nA;
            const uint8_t* text = which ? textB : textA;
            const uint8_t* pat = which ? patB : patA;
            if (best <= 0) {
                if (t == 0) {
                    A.out_score[p] = 0;
                    A.out_pos[4 * p] = A.out_pos[4 * p + 1] = A.out_pos[4 * p + 2] = A.out_pos[4 * p + 3] = -1;
                    A.out_len[p] = 0;
                }
                continue;
            }
            __syncwarp();
            const uint32_t* tab = dslot + (which ? table : 0);
            char* slotc = A.out_cigar + A.D.out_off[p];
            int pos = m + n;
            int i = bi, j = bj, state = 0, v = best;
            while (i > 0 && j > 0) {
                if (state == 0 && v == 0) break;
                const int jj = j - 1;
                const int bb = jj / BW;
                const int r = jj - bb * BW;
                const int tt = r / C, c = r - tt * C;
                const uint32_t word = tab[((int64_t)(bb * steps + (i - 1) + tt) * 32 + tt) * NW + (c >> 3)];
                const int bit = c & 7;
                const bool notE = (word >> bit) & 1u, notF = (word >> (8 + bit)) & 1u;
                const bool eopen = (word >> (16 + bit)) & 1u, fopen = (word >> (24 + bit)) & 1u;
                char op;
                if (state == 0) {
                    if (!notF) {
                        op = 'I';
                        if (!fopen) { state = 2; v += ge; } else { v += go; }
                        --i;
                    } else if (!notE) {
                        op = 'D';
                        if (!eopen) { state = 1; v += ge; } else { v += go; }
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
                    if (!eopen) { v += ge; } else { v += go; state = 0; }
                    --j;
                } else {
                    op = 'I';
                    if (!fopen) { v += ge; } else { v += go; state = 0; }
                    --i;
                }
                if (pos <= 0) {
                    if (t == 0) atomicOr(A.err, ERR_CIGAR_OVERFLOW);
                    break;
                }
                --pos;
                if (t == 0) slotc[pos] = op;
            }
            if (t == 0) {
                A.out_score[p] = best;
                A.out_pos[4 * p] = i;
                A.out_pos[4 * p + 1] = j;
                A.out_pos[4 * p + 2] = bi - 1;
                A.out_pos[4 * p + 3] = bj - 1;
                A.out_len[p] = m + n - pos;
            }
        }
    }
}

int64_t sw16_dir_words(int M, int N, int C)
{
    const int64_t nb = (N + 32 * C - 1) / (32 * C);
    return 2 * nb * (int64_t)(M + 31) * 32 * (C / 8);
}

static size_t sw16_smem(int C) { return (size_t)4 * 2 * 4 * (C / 2) * 32 * sizeof(uint32_t); }

template <int C>
static int sw16_slots_for()
{
    const size_t smem = sw16_smem(C);
    if (smem > 48 * 1024) cudaFuncSetAttribute(sw16_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sw16_kernel<C>, 128, smem);
    return per_sm < 1 ? 1 : per_sm;
}

int sw16_max_slots(int C, int sm_count)
{
    const int per_sm = C == 8 ? sw16_slots_for<8>() : (C == 16 ? sw16_slots_for<16>() : sw16_slots_for<32>());
    return per_sm * sm_count * 4;
}

cudaError_t launch_sw16(const Sw16Args& A, int C, int slots, cudaStream_t st)
{
    if (A.nwork <= 0) return cudaSuccess;
    const int blocks = (slots + 3) / 4;
    const size_t smem = sw16_smem(C);
    const int id = K_SW16X2_TRACE;
    launch_begin(id, st);
    if (C == 8) sw16_kernel<8><<<blocks, 128, smem, st>>>(A);
    else if (C == 16) sw16_kernel<16><<<blocks, 128, smem, st>>>(A);
    else sw16_kernel<32><<<blocks, 128, smem, st>>>(A);
    launch_end(id, st);
    return cudaGetLastError();
}

}  // namespace ga
