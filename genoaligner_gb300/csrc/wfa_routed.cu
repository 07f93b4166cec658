// wfa_routed.cu -- the learned-bucketed WFA path: routing and a persistent
// kernel over bucketed queues with 32-lane and 8-lane groups.
//
// Same recurrence and walk as wfa.cu (the reference's wfa_trace_kernel,
// include/genoaligner/backend/wfa_kernel.hip:119-145, 338-437); what changes is
// how pairs reach it:
//
//   * the cost model (learned.cu) gives each pair a predicted distance and the
//     sketch an exact lower bound; a pair whose bound exceeds the batch smax is
//     unresolved at once (the full search would prove the same);
//   * every other pair gets a first smax -- the prediction with a margin,
//     never below the bound, never above the batch smax -- and a queue: first
//     smax <= SMALL_SMAX goes to the small queue, served by 8-lane groups (four
//     pairs per warp), the rest to the big queue, served by whole warps;
//   * the router sorts both queues by first smax, largest first (a counting
//     sort in three kernels), so neighbours in a queue cost alike;
//   * a pair not resolved within its first smax escalates: it is appended to
//     an escalation list with smax doubled (capped at the batch smax) and the
//     next launch of the same kernel takes that list as its big queue; a pair
//     still unresolved at the batch smax is final.
//
// Results do not depend on the smax a pair is tried with: wavefront s is the
// same for every smax >= s, so a pair resolved at any smax >= d returns the
// reference's score and CIGAR.  All counts live in device memory, so the
// whole sequence of launches is a fixed graph.
#include "kernels.cuh"

namespace ga {

constexpr int SMALL_SMAX = 15;
constexpr int ROUTE_BUCKETS = 16;        // by first smax: bucket = bit length of smax

__device__ __forceinline__ int bitlen(unsigned x) { return 32 - __clz(x); }

template <int G>
__device__ __forceinline__ void gsync(unsigned gmask)
{
    if (G == 32) __syncwarp();
    else __syncwarp(gmask);
}

template <int G>
__device__ __forceinline__ int emit_run_g(char* slot, int pos, int len, char c, int gl, int* err)
{
    if (len <= 0) return pos;
    if (len > pos) {
        if (gl == 0) atomicOr(err, ERR_CIGAR_OVERFLOW);
        len = pos;
    }
    for (int q = gl; q < len; q += G) slot[pos - len + q] = c;
    return pos - len;
}

// One pair on a group of G lanes with the given smax.  Returns the score
// (-1 when unresolved within smax); writes the outputs only when the pair is
// resolved or `final`.
template <bool TRACE, int BITS, int G>
__device__ int wfa_pair_g(const RoutedArgs& R, int p, int smax, bool final, const uint64_t* __restrict__ P,
                          const uint64_t* __restrict__ T, int m, int n, int32_t* wf0, int32_t* wf1, int32_t* stk,
                          int gl, unsigned gmask)
{
    const WfaArgs& A = R.A;
    const int WS = 2 * smax + 3;
    const int base = smax + 1;
    for (int t = gl; t < WS; t += G) { wf0[t] = WFA_NULL; wf1[t] = WFA_NULL; }
    const int off0 = match_run<BITS>(P, T, 0, 0, m, n);
    gsync<G>(gmask);
    if (gl == 0) {
        wf0[base] = off0;
        if (TRACE) stk[0] = off0;
    }
    const int kfinal = n - m;
    int score = -1;
    if (kfinal == 0 && off0 >= n) {
        score = 0;
    } else if (kfinal >= -smax && kfinal <= smax) {
        int32_t* prev = wf0;
        int32_t* cur = wf1;
        for (int s = 1; s <= smax; ++s) {
            gsync<G>(gmask);
            for (int k = gl - s; k <= s; k += G) {
                const int ins = prev[base + k - 1];
                const int del = prev[base + k + 1];
                const int mis = prev[base + k];
                int x = max(del, max(ins, mis) + 1);
                if (!wfa_live(x) || x > n || x - k > m) x = WFA_NULL;
                else x += match_run<BITS>(P, T, x - k, x, m, n);
                cur[base + k] = x;
                if (TRACE) stk[s * s + s + k] = x;
            }
            gsync<G>(gmask);
            if (kfinal >= -s && kfinal <= s) {
                const int fo = cur[base + kfinal];
                if (wfa_live(fo) && fo >= n) { score = s; break; }
            }
            int32_t* t = prev; prev = cur; cur = t;
        }
    }
    if (score < 0 && !final) return score;
    if (!TRACE || score < 0) {
        if (gl == 0) {
            A.out_score[p] = score;
            if (A.out_len) A.out_len[p] = 0;
        }
        return score;
    }
    char* slot = A.out_cigar + A.D.out_off[p];
    int pos = m + n;
    if (score == 0) {
        pos = emit_run_g<G>(slot, pos, n, 'M', gl, A.err);
    } else {
        gsync<G>(gmask);
        int s = score, k = kfinal;
        int off = stk[s * s + s + k];
        int h = off, v = off - k;
        pos = emit_run_g<G>(slot, pos, v - m, 'D', gl, A.err);
        pos = emit_run_g<G>(slot, pos, h - n, 'I', gl, A.err);
        v = min(v, m);
        h = min(h, n);
        while (v > 0 && h > 0 && s > 0) {
            const int sp = s - 1;
            const int32_t* W = stk + sp * sp + sp;
            const int c_mis = (k >= -sp && k <= sp) ? W[k] + 1 : WFA_NULL;
            const int c_ins = (k - 1 >= -sp && k - 1 <= sp) ? W[k - 1] + 1 : WFA_NULL;
            const int c_del = (k + 1 >= -sp && k + 1 <= sp) ? W[k + 1] : WFA_NULL;
            int best = WFA_NULL;
            char op = 0;
            if (wfa_live(c_mis) && c_mis >= best) { best = c_mis; op = 'X'; }
            if (wfa_live(c_ins) && c_ins > best)  { best = c_ins; op = 'I'; }
            if (wfa_live(c_del) && c_del > best)  { best = c_del; op = 'D'; }
            if (!op) break;
            pos = emit_run_g<G>(slot, pos, off - best, 'M', gl, A.err);
            pos = emit_run_g<G>(slot, pos, 1, op, gl, A.err);
            off = best;
            if (op == 'X')      { off -= 1; }
            else if (op == 'I') { k -= 1; off -= 1; }
            else                { k += 1; }
            h = off;
            v = off - k;
            --s;
        }
        if (v > 0 && h > 0) {
            const int run = min(v, h);
            pos = emit_run_g<G>(slot, pos, run, 'M', gl, A.err);
            v -= run;
            h -= run;
        }
        pos = emit_run_g<G>(slot, pos, v, 'D', gl, A.err);
        pos = emit_run_g<G>(slot, pos, h, 'I', gl, A.err);
    }
    if (gl == 0) {
        A.out_score[p] = score;
        A.out_len[p] = m + n - pos;
    }
    return score;
}

template <bool TRACE, int G>
__device__ void run_item(const RoutedArgs& R, int2 item, int32_t* wf0, int32_t* wf1, int32_t* stk, int gl,
                         unsigned gmask)
{
    const WfaArgs& A = R.A;
    const int p = item.x, smax = item.y;
    const int m = A.D.a_len[p], n = A.D.b_len[p];
    if (m <= 0 || n <= 0) {
        const int len = m <= 0 ? max(n, 0) : m;
        if (TRACE) emit_run_g<G>(A.out_cigar + A.D.out_off[p], len, len, m <= 0 ? 'I' : 'D', gl, A.err);
        if (gl == 0) {
            A.out_score[p] = len;
            if (A.out_len) A.out_len[p] = TRACE ? len : 0;
        }
        return;
    }
    const bool final = smax >= A.smax;
    int score;
    if (A.D.pure[p] && A.D.pure[A.D.n + p]) {
        score = wfa_pair_g<TRACE, 2, G>(R, p, smax, final, A.D.packed + (A.D.a_off[p] >> 5),
                                        A.D.packed + (A.D.b_off[p] >> 5), m, n, wf0, wf1, stk, gl, gmask);
    } else {
        score = wfa_pair_g<TRACE, 8, G>(R, p, smax, final, reinterpret_cast<const uint64_t*>(A.D.seq + A.D.a_off[p]),
                                        reinterpret_cast<const uint64_t*>(A.D.seq + A.D.b_off[p]), m, n, wf0, wf1,
                                        stk, gl, gmask);
    }
    if (score < 0 && !final && gl == 0) {
        const int q = atomicAdd(R.esc_count, 1);
        R.esc[q] = make_int2(p, min(2 * smax, A.smax));
    }
}

// Persistent: whole warps drain the big queue, then 8-lane groups the small one.
template <bool TRACE>
__global__ void __launch_bounds__(128) wfa_routed_kernel(RoutedArgs R)
{
    extern __shared__ int32_t rsmem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int wsz = R.warp_smem;
    int32_t* wsm = rsmem + wib * wsz;
    const int64_t slot = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    int32_t* stk = TRACE ? R.A.stack + slot * R.A.stack_slot : nullptr;
    const int nbig = *R.big_count;
    for (;;) {
        int q = 0;
        if (lane == 0) q = atomicAdd(R.big_next, 1);
        q = __shfl_sync(FULL, q, 0);
        if (q >= nbig) break;
        __syncwarp();
        const int2 it = R.big[q];
        const int WS = 2 * it.y + 3;
        run_item<TRACE, 32>(R, it, wsm, wsm + WS, stk, lane, FULL);
    }
    // small queue: four independent 8-lane groups per warp
    const int g = lane >> 3, gl = lane & 7;
    const unsigned gmask = 0xffu << (8 * g);
    const int WSs = 2 * SMALL_SMAX + 3;
    int32_t* gsm = wsm + g * 2 * WSs;
    int32_t* gstk = TRACE ? stk + g * (SMALL_SMAX + 1) * (SMALL_SMAX + 1) : nullptr;
    const int nsmall = R.small_count ? *R.small_count : 0;
    __syncwarp();
    for (;;) {
        int q = 0;
        if (gl == 0) q = atomicAdd(R.small_next, 1);
        q = __shfl_sync(gmask, q, 8 * g);
        if (q >= nsmall) break;
        __syncwarp(gmask);
        const int2 it = R.small[q];
        run_item<TRACE, 8>(R, it, gsm, gsm + 2 * it.y + 3, gstk, gl, gmask);
    }
}

// ------------------------------------------------------------- routing --
// First smax of pair p from the cost model's log2(d + 1) and the bound.
__device__ __forceinline__ int first_smax(float y, int lb, int smax)
{
    const float dhat = exp2f(fmaxf(y, 0.f)) - 1.f;
    int s = (int)ceilf(dhat * 1.25f + 2.f);
    s = max(s, lb);
    s = max(s, 1);
    return min(s, smax);
}

__global__ void route_count_kernel(PairDesc D, const float* __restrict__ y, const int32_t* __restrict__ lb, int smax,
                                   int32_t* __restrict__ out_score, int32_t* __restrict__ out_len,
                                   int32_t* __restrict__ counts)
{
    __shared__ int local[2 * ROUTE_BUCKETS];
    if (threadIdx.x < 2 * ROUTE_BUCKETS) local[threadIdx.x] = 0;
    __syncthreads();
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < D.n; p += gridDim.x * blockDim.x) {
        const int m = D.a_len[p], n = D.b_len[p];
        if (m > 0 && n > 0 && lb[p] > smax) {             // provably beyond smax
            out_score[p] = -1;
            if (out_len) out_len[p] = 0;
            continue;
        }
        const int s = (m > 0 && n > 0) ? first_smax(y[2 * p], lb[p], smax) : smax;
        const int small = (s <= SMALL_SMAX && m > 0 && n > 0) ? 1 : 0;
        atomicAdd(&local[small * ROUTE_BUCKETS + min(bitlen((unsigned)s), ROUTE_BUCKETS - 1)], 1);
    }
    __syncthreads();
    if (threadIdx.x < 2 * ROUTE_BUCKETS && local[threadIdx.x]) atomicAdd(&counts[threadIdx.x], local[threadIdx.x]);
}

// counts[2*NB] -> start offsets (largest bucket first within each queue) and
// the two queue totals (counts[2*NB], counts[2*NB+1]).
__global__ void route_scan_kernel(int32_t* counts, int32_t* starts)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int q = 0; q < 2; ++q) {
        int acc = 0;
        for (int b = ROUTE_BUCKETS - 1; b >= 0; --b) {
            starts[q * ROUTE_BUCKETS + b] = acc;
            acc += counts[q * ROUTE_BUCKETS + b];
        }
        counts[2 * ROUTE_BUCKETS + q] = acc;
    }
}

// Warp-aggregated: lanes with the same (queue, bucket) take one atomic.
__global__ void route_scatter_kernel(PairDesc D, const float* __restrict__ y, const int32_t* __restrict__ lb, int smax,
                                     int32_t* __restrict__ starts, int2* __restrict__ big, int2* __restrict__ small)
{
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    for (int p0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); p0 < D.n; p0 += stride) {
        const int p = p0 + lane;
        int key = -1, s = 0;
        if (p < D.n) {
            const int m = D.a_len[p], n = D.b_len[p];
            if (!(m > 0 && n > 0 && lb[p] > smax)) {
                s = (m > 0 && n > 0) ? first_smax(y[2 * p], lb[p], smax) : smax;
                const int isb = (s <= SMALL_SMAX && m > 0 && n > 0) ? 1 : 0;
                key = isb * ROUTE_BUCKETS + min(bitlen((unsigned)s), ROUTE_BUCKETS - 1);
            }
        }
        const unsigned same = __match_any_sync(FULL, key);
        const int leader = __ffs(same) - 1;
        int base = 0;
        if (lane == leader && key >= 0) base = atomicAdd(&starts[key], __popc(same));
        base = __shfl_sync(FULL, base, leader);
        if (key >= 0) {
            const int at = base + __popc(same & ((1u << lane) - 1u));
            (key >= ROUTE_BUCKETS ? small : big)[at] = make_int2(p, s);
        }
    }
}

int route_buckets() { return ROUTE_BUCKETS; }
int routed_small_smax() { return SMALL_SMAX; }

// Stack ints per warp slot: one big item at the batch smax, or four small ones.
int64_t routed_stack_slot(int smax)
{
    const int64_t big = (int64_t)(smax + 1) * (smax + 1);
    const int64_t small = 4 * (int64_t)(SMALL_SMAX + 1) * (SMALL_SMAX + 1);
    return big > small ? big : small;
}

cudaError_t launch_route(const PairDesc& D, const float* y, const int32_t* lb, int smax, int32_t* out_score,
                         int32_t* out_len, int32_t* counts, int32_t* starts, int2* big, int2* small, cudaStream_t st)
{
    if (D.n <= 0) return cudaSuccess;
    int blocks = (D.n + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    launch_begin(K_ROUTE, st);
    route_count_kernel<<<blocks, 256, 0, st>>>(D, y, lb, smax, out_score, out_len, counts);
    launch_end(K_ROUTE, st);
    launch_begin(K_ROUTE, st);
    route_scan_kernel<<<1, 32, 0, st>>>(counts, starts);
    launch_end(K_ROUTE, st);
    launch_begin(K_ROUTE, st);
    route_scatter_kernel<<<blocks, 256, 0, st>>>(D, y, lb, smax, starts, big, small);
    launch_end(K_ROUTE, st);
    return cudaGetLastError();
}

int routed_warp_smem(int smax)
{
    const int big = 2 * (2 * smax + 3);
    const int small = 4 * 2 * (2 * SMALL_SMAX + 3);
    return big > small ? big : small;
}

int routed_max_slots(int smax, bool trace, int sm_count)
{
    const size_t smem = (size_t)4 * routed_warp_smem(smax) * sizeof(int32_t);
    int per_sm = 0;
    if (trace) {
        if (smem > 48 * 1024) cudaFuncSetAttribute(wfa_routed_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wfa_routed_kernel<true>, 128, smem);
    } else {
        if (smem > 48 * 1024) cudaFuncSetAttribute(wfa_routed_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wfa_routed_kernel<false>, 128, smem);
    }
    if (per_sm < 1) per_sm = 1;
    return per_sm * sm_count * 4;
}

cudaError_t launch_routed(const RoutedArgs& R, int slots, cudaStream_t st)
{
    const int blocks = (slots + 3) / 4;
    const size_t smem = (size_t)4 * R.warp_smem * sizeof(int32_t);
    const int id = R.A.trace ? K_WFA_TRACE : K_WFA_SCORE;
    launch_begin(id, st);
    if (R.A.trace) wfa_routed_kernel<true><<<blocks, 128, smem, st>>>(R);
    else wfa_routed_kernel<false><<<blocks, 128, smem, st>>>(R);
    launch_end(id, st);
    return cudaGetLastError();
}

}  // namespace ga
