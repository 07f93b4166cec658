// sw.cu -- affine Smith-Waterman kernels (sm_103a).
//
// Recurrence and tie rules are the reference's trace recurrence
// (include/genoaligner/backend/sw_kernel_impl.hip:286-329), which the result
// contract fixes: E and F extend only when strictly greater than opening; H
// takes the diagonal, then E if strictly greater, then F if strictly greater;
// h <= 0 stops; boundaries H = E = F = 0.  The direction nibble per cell uses
// the reference's bit meaning (hsrc in bits 0-1: 0 stop, 1 diag, 2 E, 3 F;
// bit 2: E extended; bit 3: F extended, sw_kernel.hip:218-223) and the walk
// follows the same state machine (sw_kernel_impl.hip:198-242).
//
// GB300 shape (nothing of it comes from the reference, whose trace kernel is
// one thread per pair):
//
//   * one warp per pair, persistent over a work list sorted by size;
//   * thread t owns C consecutive columns of a band of 32*C columns and keeps
//     their H and F in registers; rows stream through the warp with a one-step
//     lag per lane, so at step tau lane t computes row tau - t + 1 and receives
//     the left neighbour's last-column H and E of the same row by one shuffle
//     each -- two shuffles per C cells, no shared memory, no barriers;
//   * patterns wider than a band are processed band by band, the band edge
//     (H, E per row) passing through a per-warp global buffer;
//   * 4-bit direction nibbles, 8 per 32-bit word, stored step-major: at every
//     step the warp writes 32 * C/2 contiguous bytes;
//   * the best cell is the row-major-first maximum (per lane, then a warp
//     reduction on (score desc, row asc, column asc));
//   * the walk runs warp-uniformly right after the forward pass and writes the
//     CIGAR back to front into the pair's output slot.
//
// The score-only kernel (no directions) reports the end cell the reference's
// warp kernel reports (sw_kernel_impl.hip:146, 158-167): among cells holding
// the maximum, the one of the lane class (j-1) mod 32 that the xor-butterfly
// keeps -- the class with the smallest bit-reversed 5-bit index -- and within
// that class the row-major-first cell.
#include "kernels.cuh"

namespace ga {

__device__ __forceinline__ unsigned brev5(unsigned x) { return __brev(x) >> 27; }

template <int C, bool TRACE>
__global__ void __launch_bounds__(128) sw_kernel(SwArgs A)
{
    constexpr int BW = 32 * C;                 // columns per band
    constexpr int NW = C / 8;                  // direction words per lane per step
    const int t = threadIdx.x & 31;
    const int64_t slot = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    uint32_t* dslot = TRACE ? A.dirs + slot * A.dir_slot : nullptr;
    int32_t* eslot = A.edge + slot * A.edge_slot;
    const int go = A.gap_open, ge = A.gap_extend;

    for (;;) {
        int w = 0;
        if (t == 0) w = atomicAdd(A.counter, 1);
        w = __shfl_sync(FULL, w, 0);
        if (w >= A.nwork) break;
        __syncwarp();
        const int p = A.work[w];
        const int m = A.D.a_len[p];            // rows (text)
        const int n = A.D.b_len[p];            // columns (pattern)
        const uint8_t* text = A.D.seq + A.D.a_off[p];
        const uint8_t* pat = A.D.seq + A.D.b_off[p];
        if (m <= 0 || n <= 0) {
            if (t == 0) {
                A.out_score[p] = 0;
                A.out_pos[4 * p] = A.out_pos[4 * p + 1] = A.out_pos[4 * p + 2] = A.out_pos[4 * p + 3] = -1;
                if (A.out_len) A.out_len[p] = 0;
            }
            continue;
        }
        const int nb = (n + BW - 1) / BW;
        const int steps = m + 31;
        int best = 0, bi = 0, bj = 0;          // 1-based cell; best == 0 means none
        uint64_t bkey = ~0ull;                 // score-only end-cell key

        for (int b = 0; b < nb; ++b) {
            const int j0 = b * BW + t * C;     // 0-based first column of this lane
            const int nv = max(0, min(C, n - j0));
            uint8_t pc[C];
#pragma unroll
            for (int c = 0; c < C; ++c) pc[c] = (c < nv) ? __ldg(pat + j0 + c) : 0;
            int hup[C], fv[C];
#pragma unroll
            for (int c = 0; c < C; ++c) { hup[c] = 0; fv[c] = 0; }
            int diag_in = 0;                   // H[i-1][j0-1] for the row in flight
            int out_h = 0, out_e = 0;          // this lane's last-column H and E
            const bool left_edge = (t == 0) && (b > 0);
            int nxt_h = 0, nxt_e = 0;          // band-edge values for the next row (lane 0)
            if (left_edge) { nxt_h = eslot[0]; nxt_e = eslot[1]; }
            for (int tau = 0; tau < steps; ++tau) {
                int in_h = __shfl_up_sync(FULL, out_h, 1);
                int in_e = __shfl_up_sync(FULL, out_e, 1);
                const int i = tau - t + 1;
                const bool row = (i >= 1) && (i <= m);
                if (t == 0) {
                    if (b == 0) { in_h = 0; in_e = 0; }
                    else { in_h = nxt_h; in_e = nxt_e; }
                    if (left_edge && i < m) { nxt_h = eslot[2 * i]; nxt_e = eslot[2 * i + 1]; }
                }
                const uint8_t a = (row) ? __ldg(text + i - 1) : 0;
                if (row) {
                    int diag = diag_in;
                    int hl = in_h, el = in_e;
                    int rowmax = 0;
                    uint32_t dw[NW];
#pragma unroll
                    for (int q = 0; q < NW; ++q) dw[q] = 0;
#pragma unroll
                    for (int c = 0; c < C; ++c) {
                        int e = hl - go;
                        uint32_t bits = 0;
                        if (el - ge > e) { e = el - ge; bits = 4; }
                        int f = hup[c] - go;
                        if (fv[c] - ge > f) { f = fv[c] - ge; bits |= 8; }
                        int h = diag + (a == pc[c] ? A.match : A.mismatch);
                        uint32_t src = 1;
                        if (e > h) { h = e; src = 2; }
                        if (f > h) { h = f; src = 3; }
                        if (h <= 0) { h = 0; src = 0; }
                        if (TRACE) dw[c >> 3] |= (bits | src) << (4 * (c & 7));
                        diag = hup[c];
                        hup[c] = h;
                        fv[c] = f;
                        hl = h;
                        el = e;
                        if (c < nv) rowmax = max(rowmax, h);
                    }
                    diag_in = in_h;
                    out_h = hl;
                    out_e = el;
                    if (TRACE) {
                        uint32_t* dst = dslot + ((int64_t)(b * steps + tau) * 32 + t) * NW;
                        if constexpr (NW == 4) *reinterpret_cast<uint4*>(dst) = make_uint4(dw[0], dw[1], dw[2], dw[3]);
                        else if constexpr (NW == 2) *reinterpret_cast<uint2*>(dst) = make_uint2(dw[0], dw[1]);
                        else *dst = dw[0];
                    }
                    if (t == 31 && b + 1 < nb) { eslot[2 * (i - 1)] = out_h; eslot[2 * (i - 1) + 1] = out_e; }
                    if (TRACE) {
                        // row-major-first maximum: a later band may hold the same
                        // score in an earlier row
                        if (rowmax > best || (rowmax == best && rowmax > 0 && i < bi)) {
                            int fc = 0;
#pragma unroll
                            for (int c = C - 1; c >= 0; --c) if (c < nv && hup[c] == rowmax) fc = c;
                            best = rowmax; bi = i; bj = j0 + fc + 1;
                        }
                    } else if (rowmax > 0 && rowmax >= best) {
#pragma unroll
                        for (int c = 0; c < C; ++c) {
                            if (c < nv && hup[c] == rowmax) {
                                const unsigned j = (unsigned)(j0 + c);          // 0-based column
                                const uint64_t key = ((uint64_t)brev5(j & 31u) << 58) |
                                                     ((uint64_t)(i - 1) << 29) | j;
                                if (rowmax > best || key < bkey) { best = rowmax; bkey = key; bi = i; bj = j + 1; }
                            }
                        }
                    }
                }
            }
            __syncwarp();
        }

        // warp reduction of the best cell
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const int ob = __shfl_xor_sync(FULL, best, o);
            const int oi = __shfl_xor_sync(FULL, bi, o);
            const int oj = __shfl_xor_sync(FULL, bj, o);
            const unsigned long long ok = __shfl_xor_sync(FULL, (unsigned long long)bkey, o);
            bool take;
            if (TRACE) take = ob > best || (ob == best && ob > 0 && (oi < bi || (oi == bi && oj < bj)));
            else       take = ob > best || (ob == best && ob > 0 && ok < bkey);
            if (take) { best = ob; bi = oi; bj = oj; bkey = ok; }
        }

        if (!TRACE || best <= 0) {
            if (t == 0) {
                A.out_score[p] = best;
                A.out_pos[4 * p] = -1;
                A.out_pos[4 * p + 1] = -1;
                A.out_pos[4 * p + 2] = best > 0 ? bi - 1 : -1;
                A.out_pos[4 * p + 3] = best > 0 ? bj - 1 : -1;
                if (A.out_len) A.out_len[p] = 0;
            }
            continue;
        }

        // walk (warp-uniform): state 0 on H, 1 in an E run ('D'), 2 in an F run ('I')
        __syncwarp();
        char* slotc = A.out_cigar + A.D.out_off[p];
        int pos = m + n;
        int i = bi, j = bj, state = 0;
        while (i > 0 && j > 0) {
            const int jj = j - 1;
            const int bb = jj / BW;
            const int r = jj - bb * BW;
            const int tt = r / C, cc = r - tt * C;
            const int64_t word = ((int64_t)(bb * steps + (i - 1) + tt) * 32 + tt) * NW + (cc >> 3);
            const uint32_t nib = (dslot[word] >> (4 * (cc & 7))) & 15u;
            char op;
            if (state == 0) {
                const uint32_t src = nib & 3u;
                if (src == 0) break;
                if (src == 1) {
                    op = (__ldg(text + i - 1) == __ldg(pat + j - 1)) ? 'M' : 'X';
                    --i; --j;
                } else if (src == 2) {
                    op = 'D';
                    state = (nib & 4u) ? 1 : 0;
                    --j;
                } else {
                    op = 'I';
                    state = (nib & 8u) ? 2 : 0;
                    --i;
                }
            } else if (state == 1) {
                op = 'D';
                --j;
                if (!(nib & 4u)) state = 0;
            } else {
                op = 'I';
                --i;
                if (!(nib & 8u)) state = 0;
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

// Column width per lane for a pattern of n columns: the narrowest band that
// covers the pattern, 32*C columns per band.
int sw_width_for(int n)
{
    if (n <= 256) return 8;
    if (n <= 512) return 16;
    return 32;
}

// Direction-table words one warp slot needs for an m x n pair at width C.
int64_t sw_dir_words(int m, int n, int C)
{
    const int64_t nb = (n + 32 * C - 1) / (32 * C);
    return nb * (int64_t)(m + 31) * 32 * (C / 8);
}

template <int C, bool TRACE>
static int sw_slots_for()
{
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sw_kernel<C, TRACE>, 128, 0);
    return per_sm < 1 ? 1 : per_sm;
}

int sw_max_slots(int C, bool trace, int sm_count)
{
    int per_sm = 1;
    switch (C) {
        case 8:  per_sm = trace ? sw_slots_for<8, true>()  : sw_slots_for<8, false>();  break;
        case 16: per_sm = trace ? sw_slots_for<16, true>() : sw_slots_for<16, false>(); break;
        default: per_sm = trace ? sw_slots_for<32, true>() : sw_slots_for<32, false>(); break;
    }
    return per_sm * sm_count * 4;
}

cudaError_t launch_sw(const SwArgs& A, int C, bool trace, int slots, cudaStream_t st)
{
    if (A.nwork <= 0) return cudaSuccess;
    const int blocks = (slots + 3) / 4;
    const int id = (trace ? K_SW8_TRACE : K_SW8_SCORE) + (C == 8 ? 0 : (C == 16 ? 1 : 2));
    launch_begin(id, st);
    switch (C) {
        case 8:
            if (trace) sw_kernel<8, true><<<blocks, 128, 0, st>>>(A);
            else sw_kernel<8, false><<<blocks, 128, 0, st>>>(A);
            break;
        case 16:
            if (trace) sw_kernel<16, true><<<blocks, 128, 0, st>>>(A);
            else sw_kernel<16, false><<<blocks, 128, 0, st>>>(A);
            break;
        default:
            if (trace) sw_kernel<32, true><<<blocks, 128, 0, st>>>(A);
            else sw_kernel<32, false><<<blocks, 128, 0, st>>>(A);
            break;
    }
    launch_end(id, st);
    return cudaGetLastError();
}

}  // namespace ga
