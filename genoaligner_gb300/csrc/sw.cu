// sw.cu -- affine Smith-Waterman kernels (sm_103a).
//
// Recurrence and tie rules are the reference's trace recurrence
// (include/genoaligner/backend/sw_kernel_impl.hip:286-329), which the result
// contract fixes: E and F extend only when strictly greater than opening; H
// takes the diagonal, then E if strictly greater, then F if strictly greater;
// h <= 0 restarts; boundaries H = E = F = 0; the best cell is the first
// strictly greater one in row-major order.  The walk is the reference's state
// machine (sw_kernel_impl.hip:198-242).
//
// GB300 shape (the reference's trace kernel is one thread per pair):
//
//   * one warp per pair, persistent over a work list sorted by size;
//   * lane t owns C consecutive columns of a band of 32*C columns and keeps
//     their H - gap_open and F in registers; rows stream through the warp with
//     a one-step lag per lane, so at step tau lane t computes row tau - t + 1
//     and takes the left neighbour's last-column values of the same row with
//     two shuffles -- no shared-memory traffic for the recurrence, no barriers;
//   * patterns wider than one band are processed band by band; the band edge
//     (H - gap_open and E per row) passes through a per-warp buffer;
//   * for pairs made only of A, C, G, T the substitution score comes from a
//     query profile in shared memory (score + gap_open per letter and column,
//     16-byte loads, C/4 per row); other pairs compare bytes;
//   * max and "which operand won" come together from DPX __vibmax_s32;
//   * each cell stores a nibble of four predicates -- E chosen, F chosen, E
//     extended, F extended -- 8 per word, step-major, so the warp writes
//     32 * C/2 contiguous bytes per step.  The stop state is not stored: the
//     walk carries the exact H/E/F value along its path (diagonal: h - s; gap
//     open: e + gap_open; gap extend: e + gap_extend) and stops where H is 0,
//     which is exactly where the reference's recurrence records a stop.
//
// The score-only kernel reports the end cell the reference's warp kernel
// reports (sw_kernel_impl.hip:146, 158-167): among cells holding the maximum,
// the one of the lane class (j-1) mod 32 that its xor-butterfly keeps -- the
// class with the smallest bit-reversed 5-bit index -- and within that class
// the row-major-first cell.
#include <cstdlib>

#include "kernels.cuh"

namespace ga {

__device__ __forceinline__ unsigned brev5(unsigned x) { return __brev(x) >> 27; }
__device__ __forceinline__ int code2(uint32_t c) { return (int)(((c >> 1) ^ (c >> 2)) & 3u); }

// Forward pass over every band of one pair; returns the best cell through
// best/bi/bj (1-based) and, score-only, its end-cell key.
template <int C, bool TRACE, bool PROF>
__device__ __forceinline__ void sw_forward(const SwArgs& A, int m, int n, const uint8_t* __restrict__ text,
                                           const uint8_t* __restrict__ pat, uint32_t* dslot, int32_t* eslot,
                                           int4* prof, int t, int& best, int& bi, int& bj, uint64_t& bkey)
{
    constexpr int BW = 32 * C, NW = C / 8, NQ = C / 4;
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
            uint32_t dw[NW];
#pragma unroll
            for (int q = 0; q < NW; ++q) dw[q] = 0;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                int h, e, f;
                const int h0 = hgd + s[c];                          // H[i-1][j-1] + s
                if constexpr (TRACE) {
                    bool pe, pf, p1, p2;
                    e = __vibmax_s32(hgl, el - ge, &pe);          // open wins ties
                    f = __vibmax_s32(hgu[c], fv[c] - ge, &pf);
                    const int h1 = __vibmax_s32(h0, e, &p1);      // diagonal wins ties
                    const int h2 = __vibmax_s32(h1, f, &p2);
                    h = max(h2, 0);
                    dw[c >> 3] |= ((uint32_t)!p1 | ((uint32_t)!p2 << 1) | ((uint32_t)!pe << 2) |
                                   ((uint32_t)!pf << 3)) << (4 * (c & 7));
                } else {
                    e = __viaddmax_s32(el, -ge, hgl);
                    f = __viaddmax_s32(fv[c], -ge, hgu[c]);
                    h = __vimax3_s32_relu(h0, e, f);
                }
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
            if constexpr (TRACE) {
                uint32_t* dst = dslot + ((int64_t)(b * steps + tau) * 32 + t) * NW;
                if constexpr (NW == 4) *reinterpret_cast<uint4*>(dst) = make_uint4(dw[0], dw[1], dw[2], dw[3]);
                else if constexpr (NW == 2) *reinterpret_cast<uint2*>(dst) = make_uint2(dw[0], dw[1]);
                else *dst = dw[0];
            }
            if (t == 31 && b + 1 < nb) { eslot[2 * (i - 1)] = out_hg; eslot[2 * (i - 1) + 1] = out_e; }
            // Padding columns (c >= nv) take part in rowmax; with mismatch < 0 they
            // never exceed this lane's running best, so the exact (masked) scan
            // below runs only when a valid column may improve it.
            if (nv == 0) continue;
            if constexpr (TRACE) {
                if (rowmax > best || (rowmax == best && rowmax > 0 && i < bi)) {
                    int mx = 0, first = -1;             // first valid column holding the row's maximum
#pragma unroll
                    for (int c = 0; c < C; ++c) {
                        const int h = hgu[c] + go;
                        if (c < nv && h > mx) { mx = h; first = c; }
                    }
                    if (first >= 0 && (mx > best || (mx == best && i < bi))) {
                        best = mx;
                        bi = i;
                        bj = j0 + first + 1;
                    }
                }
            } else if (rowmax > 0 && rowmax >= best) {
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

template <int C, bool TRACE>
__global__ void __launch_bounds__(128) sw_kernel(SwArgs A)
{
    constexpr int BW = 32 * C, NW = C / 8;
    extern __shared__ int4 prof_smem[];
    const int t = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int64_t slot = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    uint32_t* dslot = TRACE ? A.dirs + slot * A.dir_slot : nullptr;
    int32_t* eslot = A.edge + slot * A.edge_slot;
    int4* prof = prof_smem + wib * (C * 32);           // 4 letters x C/4 quads x 32 lanes

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
        int best = 0, bi = 0, bj = 0;
        uint64_t bkey = ~0ull;
        const bool pure = A.D.pure && A.D.pure[p] && A.D.pure[A.D.n + p];
        if (pure) sw_forward<C, TRACE, true>(A, m, n, text, pat, dslot, eslot, prof, t, best, bi, bj, bkey);
        else      sw_forward<C, TRACE, false>(A, m, n, text, pat, dslot, eslot, prof, t, best, bi, bj, bkey);

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

        // walk (warp-uniform): state 0 on H, 1 in an E run ('D'), 2 in an F run ('I');
        // v is the exact value of the current cell's H (state 0), E (1) or F (2)
        __syncwarp();
        const int go = A.gap_open, ge = A.gap_extend;
        const int steps = m + 31;
        char* slotc = A.out_cigar + A.D.out_off[p];
        int pos = m + n;
        int i = bi, j = bj, state = 0, v = best;
        while (i > 0 && j > 0) {
            if (state == 0 && v == 0) break;                   // the reference's stop cell
            const int jj = j - 1;
            const int bb = jj / BW;
            const int r = jj - bb * BW;
            const int tt = r / C, cc = r - tt * C;
            const int64_t word = ((int64_t)(bb * steps + (i - 1) + tt) * 32 + tt) * NW + (cc >> 3);
            const uint32_t nib = (dslot[word] >> (4 * (cc & 7))) & 15u;
            char op;
            if (state == 0) {
                if (nib & 2u) {                                 // H came from F
                    op = 'I';
                    if (nib & 8u) { state = 2; v += ge; } else { v += go; }
                    --i;
                } else if (nib & 1u) {                          // H came from E
                    op = 'D';
                    if (nib & 4u) { state = 1; v += ge; } else { v += go; }
                    --j;
                } else {                                        // diagonal
                    const uint8_t ta = __ldg(text + i - 1), pb = __ldg(pat + j - 1);
                    op = ta == pb ? 'M' : 'X';
                    v -= ta == pb ? A.match : A.mismatch;
                    --i;
                    --j;
                }
            } else if (state == 1) {
                op = 'D';
                if (nib & 4u) { v += ge; } else { v += go; state = 0; }
                --j;
            } else {
                op = 'I';
                if (nib & 8u) { v += ge; } else { v += go; state = 0; }
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

// Column width per lane for a pattern of n columns: the narrowest band that
// covers the pattern, 32*C columns per band.
int sw_maxc()
{
    static const int maxc = [] {
        const char* e = getenv("GA_SW_MAXC");
        const int v = e ? atoi(e) : 8;
        return (v == 8 || v == 16) ? v : 32;
    }();
    return maxc;
}

int sw_width_for(int n)
{
    const int maxc = sw_maxc();
    if (n <= 256 || maxc == 8) return 8;
    if (n <= 512 || maxc == 16) return 16;
    return 32;
}

// Direction-table words one warp slot needs for an m x n pair at width C.
int64_t sw_dir_words(int m, int n, int C)
{
    const int64_t nb = (n + 32 * C - 1) / (32 * C);
    return nb * (int64_t)(m + 31) * 32 * (C / 8);
}

static size_t sw_smem(int C) { return (size_t)4 * C * 32 * sizeof(int4); }

template <int C, bool TRACE>
static int sw_slots_for()
{
    const size_t smem = sw_smem(C);
    if (smem > 48 * 1024) cudaFuncSetAttribute(sw_kernel<C, TRACE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sw_kernel<C, TRACE>, 128, smem);
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
    const size_t smem = sw_smem(C);
    const int id = (trace ? K_SW8_TRACE : K_SW8_SCORE) + (C == 8 ? 0 : (C == 16 ? 1 : 2));
    launch_begin(id, st);
    switch (C) {
        case 8:
            if (trace) sw_kernel<8, true><<<blocks, 128, smem, st>>>(A);
            else sw_kernel<8, false><<<blocks, 128, smem, st>>>(A);
            break;
        case 16:
            if (trace) sw_kernel<16, true><<<blocks, 128, smem, st>>>(A);
            else sw_kernel<16, false><<<blocks, 128, smem, st>>>(A);
            break;
        default:
            if (trace) sw_kernel<32, true><<<blocks, 128, smem, st>>>(A);
            else sw_kernel<32, false><<<blocks, 128, smem, st>>>(A);
            break;
    }
    launch_end(id, st);
    return cudaGetLastError();
}

}  // namespace ga
