// sw_plan.cu -- the Smith-Waterman traceback work plan, built on the device.
//
// The plan sorts the pairs of a batch into the kernels' work lists, largest
// first: the two-pairs-per-warp 16-bit list (pure-ACGT pairs whose scores fit
// 16 bits; consecutive entries share a warp) and the 32-bit lists (short and
// long shapes of sw32ck.cu).  It is a counting sort on a size key (16-bit
// pairs: forward column extent, then rows; 32-bit pairs: 64 buckets per
// doubling of (m + 31) * n) in four kernels -- classify and
// count, scan, scatter, pack -- and leaves on the device the work lists in
// the order the launches read them plus, per list, its length and the largest
// per-warp memory its items need.  The host entry's launches read that small
// record on the device (plan mode: grids and memory sized from host bounds);
// the device entry reads it back to size its memory exactly.
#include "kernels.cuh"

namespace ga {

constexpr int SP_NB = 4096;              // size buckets per list

// Bucket of a 16-bit pair (sw16_shape_key).
__device__ __forceinline__ int sp_key16(int m, int n) { return sw16_shape_key(m, n); }

// Bucket of a 32-bit pair of m rows and n columns, largest first.
__device__ __forceinline__ int sp_key(int m, int n)
{
    const uint64_t c = (uint64_t)(max(m, 0) + 31) * (uint64_t)max(n, 1);
    const int lz = __clzll((long long)c), e = 63 - lz;
    const int frac = (int)(((c << lz) >> 57) & 63u);
    return SP_NB - 1 - min(SP_NB - 1, e * 64 + frac);
}

__global__ void sp_classify_kernel(SwPlanArgs P)
{
    const int lane = threadIdx.x & 31;
    const int n = P.D.n;
    const int stride = gridDim.x * blockDim.x;
    for (int p0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); p0 < n; p0 += stride) {
        const int p = p0 + lane;
        int it = -1;
        if (p < n) {
            const int m = P.D.a_len[p], nn = P.D.b_len[p];
            if (P.cell_limit >= 0 && m > 0 && nn > 0 && ((int64_t)m + 1) * ((int64_t)nn + 1) > P.cell_limit) {
                P.out_score[p] = P.too_large_score;                  // too large: no trace
            } else {
                const bool pure = P.use16 && P.D.pure[p] && P.D.pure[n + p];
                const bool strict = pure && sw16_eligible(m, nn, P.match, P.mismatch, P.gap_open, P.gap_extend);
                const bool opt = P.try16 ? (P.try16[p] != 0 && m > 0 && nn > 0 &&
                                            sw16_scheme_ok(P.match, P.mismatch, P.gap_open, P.gap_extend))
                                         : sw16_eligible_opt(m, nn, P.match, P.mismatch, P.gap_open, P.gap_extend,
                                                             P.opt16_pct);
                const bool u16 = strict || (!P.score_only && pure && opt);
                if (u16 && !strict) {           // may be handed to the 32-bit long-shape kernel
                    atomicAdd(reinterpret_cast<unsigned long long*>(P.res + SP_NOPT), 1ull);
                    atomicMax(reinterpret_cast<unsigned long long*>(P.res + SP_DIROPT),
                              (unsigned long long)sw32ck_dir_words(m, nn, 0));
                }
                const int list = u16 ? SP_L16
                                     : ((!P.score_only && sw32ck_long(m, nn, P.long_log2)) ? SP_L32LONG : SP_L32);
                it = list * SP_NB + (u16 ? sp_key16(m, nn) : sp_key(m, nn));
                atomicMax(reinterpret_cast<unsigned long long*>(P.res + SP_EDGE), (unsigned long long)(2 * max(m, 0)));
            }
            P.item[p] = it;
        }
        const unsigned same = __match_any_sync(FULL, it);
        if (it >= 0 && lane == __ffs(same) - 1) atomicAdd(&P.counts[it], __popc(same));
    }
}

// One warp per list: exclusive scan of its bucket counts (bucket order is
// largest first), then the lists' lengths in the flattened work array and
// their offsets there (16-bit lists hold two entries per warp item).
__global__ void sp_scan_kernel(SwPlanArgs P)
{
    __shared__ long long total[SP_LISTS];
    const int lane = threadIdx.x & 31, L = threadIdx.x >> 5;
    if (L < SP_LISTS) {
        const int per = SP_NB / 32;
        const int32_t* cnt = P.counts + L * SP_NB + lane * per;
        int32_t* st = P.starts + L * SP_NB + lane * per;
        int sum = 0;
        for (int b = 0; b < per; ++b) sum += cnt[b];
        int incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += v;
        }
        int acc = incl - sum;
        for (int b = 0; b < per; ++b) {
            st[b] = acc;
            acc += cnt[b];
        }
        if (lane == 31) total[L] = incl;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long base = 0;
        for (int l = 0; l < SP_LISTS; ++l) {
            const long long ints = l == SP_L16 ? 2 * ((total[l] + 1) / 2) : total[l];
            P.res[SP_COUNT + l] = total[l];
            P.res[SP_INTS + l] = ints;
            P.res[SP_BASE + l] = base;
            base += ints;
        }
    }
}

__global__ void sp_scatter_kernel(SwPlanArgs P)
{
    const int lane = threadIdx.x & 31;
    const int n = P.D.n;
    const int stride = gridDim.x * blockDim.x;
    for (int p0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); p0 < n; p0 += stride) {
        const int p = p0 + lane;
        const int it = p < n ? P.item[p] : -1;
        const unsigned same = __match_any_sync(FULL, it);
        const int leader = __ffs(same) - 1;
        int base = 0;
        if (it >= 0 && lane == leader) base = atomicAdd(&P.starts[it], __popc(same));
        base = __shfl_sync(FULL, base, leader);
        if (it >= 0) P.sorted[(int64_t)(it / SP_NB) * n + base + __popc(same & ((1u << lane) - 1u))] = p;
    }
}

// Work items in launch order, and each list's largest per-warp memory.
__global__ void sp_pack_kernel(SwPlanArgs P)
{
    const int n = P.D.n;
    const int stride = gridDim.x * blockDim.x;
    for (int l = 0; l < SP_LISTS; ++l) {
        const long long cnt = P.res[SP_COUNT + l];
        if (cnt == 0) continue;
        const int32_t* srt = P.sorted + (int64_t)l * n;
        int32_t* w = P.work + P.res[SP_BASE + l];
        unsigned long long* mx = reinterpret_cast<unsigned long long*>(P.res + SP_DIR + l);
        unsigned long long local = 0, cmax = 0;
        if (l == SP_L16) {
            const long long items = (cnt + 1) / 2;
            for (long long q = blockIdx.x * blockDim.x + threadIdx.x; q < items; q += stride) {
                const int a = srt[2 * q], b = 2 * q + 1 < cnt ? srt[2 * q + 1] : -1;
                w[2 * q] = a;
                w[2 * q + 1] = b;
                const int M = max(P.D.a_len[a], b >= 0 ? P.D.a_len[b] : 0);
                const int N = max(P.D.b_len[a], b >= 0 ? P.D.b_len[b] : 0);
                local = max(local, (unsigned long long)(P.score_only ? sw16so_dir_words(M, N)
                                                                     : sw16ck_dir_words(M, N, P.window)));
                if (l == SP_L16) cmax = max(cmax, (unsigned long long)M * (unsigned long long)N);
            }
        } else {
            for (long long q = blockIdx.x * blockDim.x + threadIdx.x; q < cnt; q += stride) {
                const int a = srt[q];
                w[q] = a;
                if (!P.score_only)
                    local = max(local, (unsigned long long)sw32ck_dir_words(P.D.a_len[a], P.D.b_len[a], P.long_log2));
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            local = max(local, __shfl_xor_sync(FULL, local, o));
            cmax = max(cmax, __shfl_xor_sync(FULL, cmax, o));
        }
        if ((threadIdx.x & 31) == 0 && local) atomicMax(mx, local);
        if ((threadIdx.x & 31) == 0 && cmax)
            atomicMax(reinterpret_cast<unsigned long long*>(P.res + SP_MAXC16), cmax);
    }
}

// ------------------------------------------------------------ validation --
// The result checks of the reference's sw_validate (src/api/api.cpp:114-156),
// one warp per pair over its CIGAR (written at the end of its slot), 32 ops at
// a time: each lane's op steps the text and/or the pattern, a warp prefix sum
// gives its cell, and the lanes check their ops together.  The ops must
// consume exactly the span [start, end] of both sequences, M only on equal
// bytes and X on unequal ones (wellformed), and re-score to the reported
// score (rescore), each gap run costing gap_open + (L - 1) * gap_extend:
// L * gap_extend per gap op plus gap_open - gap_extend per run, a run
// starting at an I (or D) whose previous op is not one.  flags[p] =
// rescore_ok | wellformed_ok << 1 for pairs with a CIGAR, 0 otherwise.
__global__ void sw_validate_kernel(PairDesc D, int match, int mismatch, int go, int ge, const int32_t* __restrict__ score,
                                   const int32_t* __restrict__ pos, const int32_t* __restrict__ len,
                                   const char* __restrict__ cig, uint8_t* __restrict__ flags)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < D.n; p += nw) {
        const int s = score[p], L = len[p];
        if (s <= 0 || L <= 0) {
            if (lane == 0) flags[p] = 0;
            continue;
        }
        const int m = D.a_len[p], n = D.b_len[p];
        const uint8_t* T = D.seq + D.a_off[p];
        const uint8_t* P = D.seq + D.b_off[p];
        const char* cg = cig + D.out_off[p] + (m + n) - L;
        const int si = pos[4 * p], sj = pos[4 * p + 1], ei = pos[4 * p + 2], ej = pos[4 * p + 3];
        int i0 = si, j0 = sj, total = 0;
        bool bad = false;
        char prev_last = 0;                                        // the previous chunk's last op
        for (int q0 = 0; q0 < L; q0 += 32) {
            const int q = q0 + lane;
            const bool in = q < L;
            const char op = in ? cg[q] : 0;
            const bool mx = op == 'M' || op == 'X';
            const int di = mx || op == 'I', dj = mx || op == 'D';
            int v = di << 16 | dj;                                 // inclusive prefix of both steps
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(FULL, v, o);
                if (lane >= o) v += y;
            }
            const int i = i0 + (v >> 16) - di, j = j0 + (v & 0xffff) - dj;
            char prev = __shfl_up_sync(FULL, op, 1);
            if (lane == 0) prev = prev_last;
            bool b = false;
            int sc = 0;
            if (in) {
                if (mx) {
                    b = i > ei || j > ej || i >= m || j >= n || ((T[i] == P[j]) != (op == 'M'));
                    sc = op == 'M' ? match : mismatch;
                } else if (op == 'I') {
                    b = i > ei || i >= m;
                    sc = -ge - (prev != 'I' ? go - ge : 0);
                } else if (op == 'D') {
                    b = j > ej || j >= n;
                    sc = -ge - (prev != 'D' ? go - ge : 0);
                } else {
                    b = true;
                }
            }
            bad |= __any_sync(FULL, b);
            total += __reduce_add_sync(FULL, sc);
            const int tot = __shfl_sync(FULL, v, 31);
            i0 += tot >> 16;
            j0 += tot & 0xffff;
            prev_last = __shfl_sync(FULL, op, 31);
        }
        const bool ok = !bad && i0 == ei + 1 && j0 == ej + 1;
        if (lane == 0) flags[p] = (uint8_t)((ok && total == s ? 1 : 0) | (ok ? 2 : 0));
    }
}

cudaError_t launch_sw_validate(const PairDesc& D, const ga_sw_scoring_t& sc, const int32_t* score, const int32_t* pos,
                               const int32_t* len, const char* cig, uint8_t* flags, cudaStream_t st)
{
    if (D.n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<int64_t>(((int64_t)D.n + 3) / 4, (int64_t)device_sms() * 16);   // a warp per pair
    launch_begin(K_VALIDATE, st);
    sw_validate_kernel<<<blocks, 128, 0, st>>>(D, sc.match, sc.mismatch, sc.gap_open, sc.gap_extend, score, pos, len,
                                               cig, flags);
    launch_end(K_VALIDATE, st);
    return cudaGetLastError();
}

int64_t sw_plan_scratch_ints(int n) { return (int64_t)n + 2 * SP_LISTS * SP_NB + (int64_t)SP_LISTS * n; }

cudaError_t launch_sw_plan(SwPlanArgs P, int32_t* scratch, cudaStream_t st)
{
    const int n = P.D.n;
    P.item = scratch;
    P.counts = scratch + n;
    P.starts = P.counts + SP_LISTS * SP_NB;
    P.sorted = P.starts + SP_LISTS * SP_NB;
    cudaError_t e = cudaMemsetAsync(P.counts, 0, sizeof(int32_t) * SP_LISTS * SP_NB, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(P.res, 0, sizeof(long long) * SP_RES, st);
    if (e != cudaSuccess || n <= 0) return e;
    int blocks = (n + 255) / 256;
    blocks = std::min(blocks, device_sms() * 8);
    launch_begin(K_SWPLAN, st);
    sp_classify_kernel<<<blocks, 256, 0, st>>>(P);
    launch_end(K_SWPLAN, st);
    launch_begin(K_SWPLAN, st);
    sp_scan_kernel<<<1, 32 * SP_LISTS, 0, st>>>(P);
    launch_end(K_SWPLAN, st);
    launch_begin(K_SWPLAN, st);
    sp_scatter_kernel<<<blocks, 256, 0, st>>>(P);
    launch_end(K_SWPLAN, st);
    launch_begin(K_SWPLAN, st);
    sp_pack_kernel<<<blocks, 256, 0, st>>>(P);
    launch_end(K_SWPLAN, st);
    return cudaGetLastError();
}

}  // namespace ga
