// sw.cu -- score-only affine Smith-Waterman kernel for 32-bit pairs (sm_103a).
//
// The score-only path of pairs the two-pairs-per-warp 16-bit kernel cannot
// take (bytes outside A/C/G/T, or scores that could pass 16 bits).  The
// recurrence is the reference's (include/genoaligner/backend/sw_kernel_impl.hip:
// 286-329): E and F extend only when strictly greater than opening; h <= 0
// restarts; boundaries H = E = F = 0.
//
// GB300 shape (the reference's score kernel is one warp per pair with a
// shared-memory row and 14 shuffles per 32 cells):
//
//   * one warp per pair, persistent over a work list sorted by size;
//   * lane t owns C = 8 consecutive columns of a band of 256 columns and keeps
//     their H - gap_open and F in registers; rows stream through the warp with
//     a one-step lag per lane, so at step tau lane t computes row tau - t + 1
//     and takes the left neighbour's last-column values of the same row with
//     two shuffles -- no shared-memory traffic for the recurrence, no barriers;
//   * patterns wider than one band are processed band by band; the band edge
//     (H - gap_open and E per row) passes through a per-warp buffer;
//   * for pairs made only of A, C, G, T the substitution score comes from a
//     query profile in shared memory (score + gap_open per letter and column,
//     16-byte loads); other pairs compare bytes;
//   * E, F and H are one DPX instruction each (__viaddmax_s32 twice,
//     __vimax3_s32_relu).
//
// The end cell is the one the reference's warp kernel reports
// (sw_kernel_impl.hip:146, 158-167): among cells holding the maximum, the one
// of the lane class (j-1) mod 32 that its xor-butterfly keeps -- the class
// with the smallest bit-reversed 5-bit index -- and within that class the
// row-major-first cell.
#include "kernels.cuh"

namespace ga {

__device__ __forceinline__ unsigned brev5(unsigned x) { return __brev(x) >> 27; }
__device__ __forceinline__ int code2(uint32_t c) { return (int)(((c >> 1) ^ (c >> 2)) & 3u); }

// Forward pass over every band of one pair; returns the best value and its
// end-cell key through best/bi/bj (1-based)/bkey.
template <int C, bool PROF>
__device__ __forceinline__ void sw_forward(const SwArgs& A, int m, int n, const uint8_t* __restrict__ text,
                                           const uint8_t* __restrict__ pat, int32_t* eslot, int4* prof, int t,
                                           int& best, int& bi, int& bj, uint64_t& bkey)
{
    constexpr int BW = 32 * C, NQ = C / 4;
    const int go = A.gap_open, ge = A.gap_extend;
    const int sm = A.match + go, sx = A.mismatch + go;
    const int nb = (n + BW - 1) / BW;
    const int steps = m + 31;
    for (int b = 0; b < nb; ++b) {
        const int j0 = b * BW + t * C;
        const int nv = max(0, min(C, n - j0));
        uint32_t pb[PROF ? 1 : C];
        if constexpr (PROF) {
            __syncwarp();
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                int code[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) code[k] = (4 * q + k < nv) ? code2(__ldg(pat + j0 + 4 * q + k)) : 4;
#pragma unroll
                for (int L = 0; L < 4; ++L)
                    prof[(L * NQ + q) * 32 + t] = make_int4(code[0] == L ? sm : sx, code[1] == L ? sm : sx,
                                                            code[2] == L ? sm : sx, code[3] == L ? sm : sx);
            }
            __syncwarp();
        } else {
#pragma unroll
            for (int c = 0; c < C; ++c) pb[c] = (c < nv) ? __ldg(pat + j0 + c) : 0x100u;
        }
        int hgu[C], fv[C];
#pragma unroll
        for (int c = 0; c < C; ++c) { hgu[c] = -go; fv[c] = 0; }
        int diag_in = -go;                      // H[i-1][j0-1] - go for the row in flight
        int out_hg = -go, out_e = 0;            // this lane's last column: H - go, E
        const bool left_edge = (t == 0) && (b > 0);
        int nxt_hg = -go, nxt_e = 0;
        if (left_edge) { nxt_hg = eslot[0]; nxt_e = eslot[1]; }
        uint32_t a_next = (t == 0) ? __ldg(text) : 0u;
        for (int tau = 0; tau < steps; ++tau) {
            int in_hg = __shfl_up_sync(FULL, out_hg, 1);
            int in_e = __shfl_up_sync(FULL, out_e, 1);
            const int i = tau - t + 1;
            const uint32_t a = a_next;
            if (i >= 0 && i < m) a_next = __ldg(text + i);          // next step's row is i + 1
            if (t == 0) {
                if (b == 0) { in_hg = -go; in_e = 0; }
                else { in_hg = nxt_hg; in_e = nxt_e; }
                if (left_edge && i >= 1 && i < m) { nxt_hg = eslot[2 * i]; nxt_e = eslot[2 * i + 1]; }
            }
            if (i < 1 || i > m) continue;
            int s[C];
            if constexpr (PROF) {
                const int L = code2(a);
#pragma unroll
                for (int q = 0; q < NQ; ++q) {
                    const int4 v = prof[(L * NQ + q) * 32 + t];
                    s[4 * q] = v.x; s[4 * q + 1] = v.y; s[4 * q + 2] = v.z; s[4 * q + 3] = v.w;
                }
            } else {
#pragma unroll
                for (int c = 0; c < C; ++c) s[c] = (a == pb[c]) ? sm : sx;
            }
            int hgd = diag_in, hgl = in_hg, el = in_e;
            int rowmax = 0;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const int h0 = hgd + s[c];                          // H[i-1][j-1] + s
                const int e = __viaddmax_s32(el, -ge, hgl);
                const int f = __viaddmax_s32(fv[c], -ge, hgu[c]);
                const int h = __vimax3_s32_relu(h0, e, f);
                const int hg = h - go;
                hgd = hgu[c];
                hgu[c] = hg;
                fv[c] = f;
                hgl = hg;
                el = e;
                rowmax = max(rowmax, h);
            }
            diag_in = in_hg;
            out_hg = hgl;
            out_e = el;
            if (t == 31 && b + 1 < nb) { eslot[2 * (i - 1)] = out_hg; eslot[2 * (i - 1) + 1] = out_e; }
            // Padding columns (c >= nv) take part in rowmax; with mismatch < 0 they
            // never exceed this lane's running best, so the exact (masked) scan
            // below runs only when a valid column may improve it.
            if (nv == 0) continue;
            if (rowmax > 0 && rowmax >= best) {
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    const int h = hgu[c] + go;
                    if (c < nv && h > 0 && h >= best) {
                        const unsigned j = (unsigned)(j0 + c);          // 0-based column
                        const uint64_t key = ((uint64_t)brev5(j & 31u) << 58) | ((uint64_t)(i - 1) << 29) | j;
                        if (h > best || key < bkey) { best = h; bkey = key; bi = i; bj = j + 1; }
                    }
                }
            }
        }
        __syncwarp();
    }
}

// PLAN: items and band-edge memory from the device-built plan (plan_view).
template <int C, bool PLAN>
__global__ void __launch_bounds__(128) sw_kernel(SwArgs A)
{
    extern __shared__ int4 prof_smem[];
    const int t = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int64_t slot = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    PlanView V{A.work, A.nwork, A.dir_slot, A.edge_slot, true};
    if constexpr (PLAN) {
        V = plan_view(A.plan, A.plan_list, A.work, A.nwork, nullptr, A.dir_slot, A.edge_slot, A.dir_cap, A.edge_cap,
                      A.err);
        if (!V.run) return;
    }
    int32_t* eslot = A.edge + slot * V.edge_slot;
    int4* prof = prof_smem + wib * (C * 32);           // 4 letters x C/4 quads x 32 lanes

    for (;;) {
        int w = 0;
        if (t == 0) w = atomicAdd(A.counter, 1);
        w = __shfl_sync(FULL, w, 0);
        if (w >= V.nwork) break;
        __syncwarp();
        const int p = V.work[w];
        const int m = A.D.a_len[p];            // rows (text)
        const int n = A.D.b_len[p];            // columns (pattern)
        const uint8_t* text = A.D.seq + A.D.a_off[p];
        const uint8_t* pat = A.D.seq + A.D.b_off[p];
        int best = 0, bi = 0, bj = 0;
        uint64_t bkey = ~0ull;
        if (m > 0 && n > 0) {
            const bool pure = A.D.pure && A.D.pure[p] && A.D.pure[A.D.n + p];
            if (pure) sw_forward<C, true>(A, m, n, text, pat, eslot, prof, t, best, bi, bj, bkey);
            else      sw_forward<C, false>(A, m, n, text, pat, eslot, prof, t, best, bi, bj, bkey);
            // warp reduction of the best cell: the smallest key among the maxima
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const int ob = __shfl_xor_sync(FULL, best, o);
                const int oi = __shfl_xor_sync(FULL, bi, o);
                const int oj = __shfl_xor_sync(FULL, bj, o);
                const unsigned long long ok = __shfl_xor_sync(FULL, (unsigned long long)bkey, o);
                if (ob > best || (ob == best && ob > 0 && ok < bkey)) { best = ob; bi = oi; bj = oj; bkey = ok; }
            }
        }
        if (t == 0) {
            A.out_score[p] = best;
            A.out_pos[4 * p] = -1;
            A.out_pos[4 * p + 1] = -1;
            A.out_pos[4 * p + 2] = best > 0 ? bi - 1 : -1;
            A.out_pos[4 * p + 3] = best > 0 ? bj - 1 : -1;
            if (A.out_len) A.out_len[p] = 0;
        }
    }
}

static size_t sw_smem(int C) { return (size_t)4 * C * 32 * sizeof(int4); }

int sw_max_slots(int sm_count)
{
    const size_t smem = sw_smem(SW_SCORE_C);
    return blocks_per_sm((const void*)sw_kernel<SW_SCORE_C, false>, 128, smem) * sm_count * 4;
}

cudaError_t launch_sw(const SwArgs& A, int slots, cudaStream_t st)
{
    if (A.nwork <= 0 && !A.plan) return cudaSuccess;
    const int blocks = (slots + 3) / 4;
    launch_begin(K_SW_SCORE, st);
    if (A.plan) sw_kernel<SW_SCORE_C, true><<<blocks, 128, sw_smem(SW_SCORE_C), st>>>(A);
    else sw_kernel<SW_SCORE_C, false><<<blocks, 128, sw_smem(SW_SCORE_C), st>>>(A);
    launch_end(K_SW_SCORE, st);
    return cudaGetLastError();
}

}  // namespace ga
