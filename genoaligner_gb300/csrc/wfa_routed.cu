// wfa_routed.cu -- the learned-bucketed WFA path: routing and two persistent
// kernels over two bucketed queues, one served by single lanes, one by
// groups of lanes, warps or whole blocks.
//
// Same recurrence and walk as wfa.cu (the reference's wfa_trace_kernel,
// include/genoaligner/backend/wfa_kernel.hip:119-145, 338-437); what changes is
// how pairs reach it:
//
//   * the cost model (learned.cu) gives each pair a predicted distance and the
//     sketch an exact lower bound; a pair whose bound exceeds the batch smax is
//     unresolved at once (the full search would prove the same);
//   * every other pair gets a first smax -- the prediction with a margin,
//     never below the bound, never above the batch smax -- and a queue.  A
//     pure-ACGT pair of at most LANE_MAXLEN bases a side whose first smax is
//     <= LANE_SMAX goes to the lane queue: one pair per lane, 32 pairs per
//     warp in lockstep over (s, k), sequences and wavefront staged in shared
//     memory.  Every other pair goes to the warp queue, with the batch smax:
//     one pair per group of lanes (8 or 16 lanes, several pairs per warp
//     stepping through their wavefronts together, at batch smax <= 128; else
//     one pair per warp), lanes over the diagonals of a wavefront; items
//     estimated at s >= 256 first on whole blocks;
//   * the router sorts both queues, largest first -- the lane queue by first
//     smax, the warp queue by the bit length of the estimate -- with a
//     counting sort (bucket counts in the route pass, then a scan and a
//     scatter), so the pairs of a lane batch or of a warp cost alike;
//   * a lane-queue pair not resolved within its first smax escalates: it is
//     appended to an escalation list with the batch smax, which the warp
//     kernel takes after its own queue (it starts again from s = 0); a pair
//     unresolved at the batch smax is final.
//
// Results do not depend on the smax a pair is tried with: wavefront s is the
// same for every smax >= s, so a pair resolved at any smax >= d returns the
// reference's score and CIGAR.  All counts live in device memory, so the
// whole sequence of launches is a fixed graph.
#include "kernels.cuh"
#include "route.cuh"

namespace ga {

// Lane queue (route.cuh): per warp in shared memory, both sequences of its
// 32 pairs as 32-bit words of 16 2-bit codes [word][lane] (LANE_WORDS = 16
// data words + 1 read by the two-word fetch window) and one wavefront of
// 16-bit offsets [k][lane] (offsets are at most LANE_MAXLEN; LANE_NULL marks
// a dead diagonal), updated in place.  The walk reads a 16-bit record per (s, k):
// the predecessor (0 mismatch, 1 insertion, 2 deletion) and the extension
// length, [idx][lane] in the warp's global stack slot.
constexpr int LANE_WORDS = LANE_MAXLEN / 16 + 1;
constexpr int LANE_WS = 2 * LANE_SMAX + 3;
constexpr int LANE_STACK = (LANE_SMAX + 1) * (LANE_SMAX + 1);
constexpr int LANE_WARP_SMEM = 2 * LANE_WORDS * 32 + LANE_WS * 16;    // ints per warp
// Dead-diagonal offset of the lane wavefront: below every live offset (>= 0),
// and NULL + 1 stays negative, so x < 0 is the liveness test.
constexpr int LANE_NULL = -16384;
// Hand-over rule: past wavefront LANE_HAND_S, once at most 1/LANE_HAND_DIV of
// a warp's pairs are still unresolved, they move to the warp queue.
constexpr int LANE_HAND_S = 6;
constexpr int LANE_HAND_DIV = 16;

template <int G>
__device__ __forceinline__ void gsync(unsigned gmask)
{
    if (G == 128) __syncthreads();
    else if (G == 32) __syncwarp();
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

// ------------------------------------------------------------ lane queue --
// One lane writes ops [pos - len, pos) of its own slot: bytes up to a 4-byte
// boundary, then words, then bytes.
__device__ __forceinline__ int emit_lane(char* slot, int pos, int len, char c, int* err)
{
    if (len <= 0) return pos;
    if (len > pos) {
        atomicOr(err, ERR_CIGAR_OVERFLOW);
        len = pos;
    }
    char* lo = slot + (pos - len);
    char* const hi = slot + pos;
    while (lo < hi && ((uintptr_t)lo & 3u)) *lo++ = c;
    const uint32_t w4 = (uint32_t)(uint8_t)c * 0x01010101u;
    while (hi - lo >= 4) { *reinterpret_cast<uint32_t*>(lo) = w4; lo += 4; }
    while (lo < hi) *lo++ = c;
    return pos - len;
}

// 16 codes of a staged sequence from position p (p < LANE_MAXLEN).
__device__ __forceinline__ uint32_t lane_fetch(const uint32_t* S, int p)
{
    const int w = p >> 4;
    return __funnelshift_r(S[w * 32], S[(w + 1) * 32], 2u * (unsigned)(p & 15));
}

// Match run of P from v and T from h; SP, ST point at this lane's column.
__device__ __forceinline__ int lane_run(const uint32_t* SP, const uint32_t* ST, int v, int h, int m, int n)
{
    int run = 0;
    for (;;) {
        const int lim = min(m - v, n - h);
        if (lim <= 0) break;
        const uint32_t x = lane_fetch(SP, v) ^ lane_fetch(ST, h);
        int eq = x ? (__ffs((int)x) - 1) >> 1 : 16;
        eq = min(eq, lim);
        run += eq;
        v += eq;
        h += eq;
        if (eq < 16) break;
    }
    return run;
}

// Pairs of the lane queue, 32 per warp: each lane runs the whole forward
// pass and walk of its own pair.  All lanes of a warp step through the same
// (s, k) until the last of them resolves or reaches its first smax, so the
// shared-memory wavefront [k][lane] and sequences [word][lane] are read
// without bank conflicts and the walk records coalesce.  The predecessor code
// the forward pass stores is the argmax the reference's walk recomputes
// (mismatch on >=, insertion on >, deletion on >), so the walk needs no
// wavefront values: the offset before extension is the offset minus the
// stored extension length.
template <bool TRACE>
__device__ void lane_phase(const RoutedArgs& R, uint32_t* smem, uint16_t* rec, int lane)
{
    const WfaArgs& A = R.A;
    const uint32_t* SP = smem + lane;
    const uint32_t* ST = smem + LANE_WORDS * 32 + lane;
    int16_t* WF = reinterpret_cast<int16_t*>(smem + 2 * LANE_WORDS * 32) + (LANE_SMAX + 1) * 32 + lane;   // WF[k * 32]
    const int nlane = R.small_count ? *R.small_count : 0;
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(R.small_next, 32);
        base = __shfl_sync(FULL, base, 0);
        if (base >= nlane) break;
        const int q = base + lane;
        const bool have = q < nlane;
        int p = 0, smx = 0, m = 0, n = 0;
        bool misrouted = false;
        if (have) {
            const int2 it = R.small[q];
            p = it.x;
            smx = it.y;
            m = A.D.a_len[p];
            n = A.D.b_len[p];
            // the router sends only pairs that fit; anything else goes back to
            // the warp queue at the same smax
            misrouted = m <= 0 || n <= 0 || m > LANE_MAXLEN || n > LANE_MAXLEN || smx < 1 || smx > LANE_SMAX ||
                        !A.D.pure[p] || !A.D.pure[A.D.n + p];
        }
        const bool run = have && !misrouted;
        // stage both sequences: 32-bit words 0 .. (len-1)/16 + 1 lie in the arena
        {
            const uint32_t* gP = reinterpret_cast<const uint32_t*>(A.D.packed + (run ? (A.D.a_off[p] >> 5) : 0));
            const uint32_t* gT = reinterpret_cast<const uint32_t*>(A.D.packed + (run ? (A.D.b_off[p] >> 5) : 0));
            const int lastP = run ? ((m - 1) >> 4) + 1 : -1, lastT = run ? ((n - 1) >> 4) + 1 : -1;
            uint32_t* sp = smem + lane;
#pragma unroll
            for (int w = 0; w < LANE_WORDS; ++w) {
                sp[w * 32] = w <= lastP ? __ldg(gP + w) : 0u;
                sp[(LANE_WORDS + w) * 32] = w <= lastT ? __ldg(gT + w) : 0u;
            }
        }
        const int kfinal = n - m;
        int score = -1;
        bool act = run;
        if (run) {
            const int off0 = lane_run(SP, ST, 0, 0, m, n);
            WF[0] = (int16_t)off0;
            WF[-32] = LANE_NULL;
            WF[32] = LANE_NULL;
            if (TRACE) rec[lane] = (uint16_t)(off0 << 2);
            if (kfinal == 0 && off0 >= n) { score = 0; act = false; }
        }
        // When only a few lanes are still running well after the others have
        // resolved, they are handed to the warp queue (rerun from s = 0
        // there): the other lanes would otherwise idle.
        const int started = __popc(__ballot_sync(FULL, act));
        bool handed = false;
        for (int s = 1;; ++s) {
            const unsigned am = __ballot_sync(FULL, act);
            if (!am) break;
            if (s > LANE_HAND_S && __popc(am) * LANE_HAND_DIV <= started) {
                handed = act;
                act = false;
                break;
            }
            if (act) {
                WF[(s + 1) * 32] = LANE_NULL;
                WF[-(s + 1) * 32] = LANE_NULL;
                int carry = LANE_NULL;                           // wavefront s-1 at k-1
                for (int k = -s; k <= s; ++k) {
                    const int mis = WF[k * 32];
                    const int del = WF[(k + 1) * 32];
                    int x = mis + 1, code = 0;
                    if (carry + 1 > x) { x = carry + 1; code = 1; }
                    if (del > x) { x = del; code = 2; }
                    carry = mis;
                    int ext = 0;
                    if (x < 0 || x > n || x - k > m) x = LANE_NULL;
                    else { ext = lane_run(SP, ST, x - k, x, m, n); x += ext; }
                    WF[k * 32] = (int16_t)x;
                    if (TRACE) rec[(s * s + s + k) * 32 + lane] = (uint16_t)(code | (ext << 2));
                }
                if (kfinal >= -s && kfinal <= s) {
                    const int fo = WF[kfinal * 32];
                    if (fo >= n) { score = s; act = false; }
                }
                if (act && s >= smx) act = false;
            }
        }
        // unresolved within the first smax (or handed over): escalate to the
        // warp queue at the batch smax, warp-aggregated; unresolved at the
        // batch smax itself: final
        const bool esc = misrouted || handed || (run && score < 0 && smx < A.smax);
        const unsigned em = __ballot_sync(FULL, esc);
        if (em) {
            int eb = 0;
            if (lane == 0) eb = atomicAdd(R.esc_count, __popc(em));
            eb = __shfl_sync(FULL, eb, 0);
            if (esc) R.esc[eb + __popc(em & ((1u << lane) - 1u))] = make_int2(p, A.smax);
        }
        if (!have || esc) continue;
        if (!TRACE || score < 0) {
            A.out_score[p] = score;
            if (A.out_len) A.out_len[p] = 0;
            continue;
        }
        char* slot = A.out_cigar + A.D.out_off[p];
        int pos = m + n;
        if (score == 0) {
            pos = emit_lane(slot, pos, n, 'M', A.err);
        } else {
            // the final cell's offset is n (clipped at n, reached >= n)
            int s = score, k = kfinal, off = n;
            int h = off, v = off - k;
            while (v > 0 && h > 0 && s > 0) {
                const uint32_t r = rec[(s * s + s + k) * 32 + lane];
                const int ext = (int)(r >> 2), code = (int)(r & 3u);
                pos = emit_lane(slot, pos, ext, 'M', A.err);
                pos = emit_lane(slot, pos, 1, code == 0 ? 'X' : (code == 1 ? 'I' : 'D'), A.err);
                off -= ext;
                if (code == 0)      { off -= 1; }
                else if (code == 1) { k -= 1; off -= 1; }
                else                { k += 1; }
                h = off;
                v = off - k;
                --s;
            }
            if (v > 0 && h > 0) {
                const int r = min(v, h);
                pos = emit_lane(slot, pos, r, 'M', A.err);
                v -= r;
                h -= r;
            }
            pos = emit_lane(slot, pos, v, 'D', A.err);
            pos = emit_lane(slot, pos, h, 'I', A.err);
        }
        A.out_score[p] = score;
        A.out_len[p] = m + n - pos;
    }
}

// The walk of a resolved pair (score >= 0) on the G lanes of its group, from
// the wavefront stack the forward pass left (stk[s * s + s + k]: wavefront s
// at diagonal k), written backwards from the end of the pair's CIGAR slot.
// Every lane of the group runs the same walk; the runs are written by all of
// them.  Returns the position of the CIGAR's first op in the slot.
template <int G>
__device__ int walk_g(const WfaArgs& A, int p, int score, int kfinal, int m, int n, const int32_t* stk, int gl)
{
    char* slot = A.out_cigar + A.D.out_off[p];
    int pos = m + n;
    if (score == 0) {
        pos = emit_run_g<G>(slot, pos, n, 'M', gl, A.err);
    } else {
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
    return pos;
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
    if (score > 0) gsync<G>(gmask);
    const int pos = walk_g<G>(A, p, score, n - m, m, n, stk, gl);
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
        R.esc[q] = make_int2(p, A.smax);
    }
}

// Warp-queue items on groups of G lanes (G = 8 or 16), 32 / G pairs per warp:
// the warp takes 32 / G consecutive items of a list (the lists are sorted by
// predicted distance, so the pairs of a warp cost alike) and its groups step
// through s together -- every group at the same s has the same 2s + 1
// diagonals, so the groups' loops stay converged -- each lane over the
// diagonals k = gl - s, gl - s + G, ...  A group whose pair resolves idles
// until the last pair of the warp resolves or reaches the batch smax, then
// the groups walk their own pairs.  Items of these lists carry the batch smax
// and are final.  Each group has its own two wavefronts in the warp's shared
// memory and its own stack of (smax + 1)^2 offsets in the warp's stack slot.
template <bool TRACE, int G>
__device__ void group_phase(const RoutedArgs& R, const int2* __restrict__ items, int cnt, int32_t* next, int first,
                            int32_t* wsm, int32_t* wstk, int lane)
{
    constexpr int NG = 32 / G;
    const WfaArgs& A = R.A;
    const int grp = lane / G, gl = lane % G;
    const int smax = A.smax;
    const int WS = 2 * smax + 3, base = smax + 1;
    int32_t* const wfa = wsm + grp * 2 * WS;
    int32_t* const wfb = wfa + WS;
    int32_t* const stk = TRACE ? wstk + grp * (int64_t)(smax + 1) * (smax + 1) : nullptr;
    for (;;) {
        int q0 = 0;
        if (lane == 0) q0 = atomicAdd(next, NG);
        q0 = __shfl_sync(FULL, q0, 0) + first;
        if (q0 >= cnt) break;
        const int q = q0 + grp;
        int p = 0, m = 0, n = 0;
        bool have = q < cnt;
        if (have) {
            p = items[q].x;
            m = A.D.a_len[p];
            n = A.D.b_len[p];
            if (m <= 0 || n <= 0) {
                const int len = m <= 0 ? max(n, 0) : m;
                if (TRACE) emit_run_g<G>(A.out_cigar + A.D.out_off[p], len, len, m <= 0 ? 'I' : 'D', gl, A.err);
                if (gl == 0) {
                    A.out_score[p] = len;
                    if (A.out_len) A.out_len[p] = TRACE ? len : 0;
                }
                have = false;
            }
        }
        // 2-bit codes when both sides are pure ACGT, else bytes
        const bool packed = have && A.D.pure[p] && A.D.pure[A.D.n + p];
        const uint64_t* P = nullptr;
        const uint64_t* T = nullptr;
        if (have) {
            P = packed ? A.D.packed + (A.D.a_off[p] >> 5) : reinterpret_cast<const uint64_t*>(A.D.seq + A.D.a_off[p]);
            T = packed ? A.D.packed + (A.D.b_off[p] >> 5) : reinterpret_cast<const uint64_t*>(A.D.seq + A.D.b_off[p]);
        }
        for (int t = gl; t < WS; t += G) { wfa[t] = WFA_NULL; wfb[t] = WFA_NULL; }
        int off0 = 0;
        if (have) off0 = packed ? match_run<2>(P, T, 0, 0, m, n) : match_run<8>(P, T, 0, 0, m, n);
        __syncwarp();
        if (have && gl == 0) {
            wfa[base] = off0;
            if (TRACE) stk[0] = off0;
        }
        const int kfinal = n - m;
        int score = -1;
        bool act = have && kfinal >= -smax && kfinal <= smax;
        if (have && kfinal == 0 && off0 >= n) { score = 0; act = false; }
        int32_t* prev = wfa;
        int32_t* cur = wfb;
        for (int s = 1; s <= smax; ++s) {
            if (!__any_sync(FULL, act)) break;
            __syncwarp();
            if (act) {
                for (int k = gl - s; k <= s; k += G) {
                    const int ins = prev[base + k - 1];
                    const int del = prev[base + k + 1];
                    const int mis = prev[base + k];
                    int x = max(del, max(ins, mis) + 1);
                    if (!wfa_live(x) || x > n || x - k > m) x = WFA_NULL;
                    else x += packed ? match_run<2>(P, T, x - k, x, m, n) : match_run<8>(P, T, x - k, x, m, n);
                    cur[base + k] = x;
                    if (TRACE) stk[s * s + s + k] = x;
                }
            }
            __syncwarp();
            if (act && kfinal >= -s && kfinal <= s) {
                const int fo = cur[base + kfinal];
                if (wfa_live(fo) && fo >= n) { score = s; act = false; }
            }
            int32_t* t = prev; prev = cur; cur = t;
        }
        if (have) {
            int len = 0;
            if (TRACE && score >= 0) len = m + n - walk_g<G>(A, p, score, kfinal, m, n, stk, gl);
            if (gl == 0) {
                A.out_score[p] = score;
                if (A.out_len) A.out_len[p] = len;
            }
        }
        __syncwarp();
    }
}

// Lane queue, one pair per lane (persistent, 32 pairs per grab).  Runs
// before the warp kernel so that its escalations are complete when that
// kernel reaches them.
template <bool TRACE>
__global__ void __launch_bounds__(128) wfa_lane_kernel(RoutedArgs R)
{
    extern __shared__ __align__(16) uint32_t lsmem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t slot = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    uint16_t* rec = TRACE ? R.lane_rec + slot * (int64_t)LANE_STACK * 32 : nullptr;
    lane_phase<TRACE>(R, lsmem + wib * LANE_WARP_SMEM, rec, lane);
}

// Warp queue (persistent): the routed pairs largest first, then the lane
// queue's escalations, one pair per warp (G = 32) or per group of G lanes.
// Every item runs with the batch smax and is final.
template <bool TRACE, int G>
__global__ void __launch_bounds__(128) wfa_routed_kernel(RoutedArgs R)
{
    extern __shared__ __align__(16) int32_t rsmem[];
    __shared__ int s_q;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    int32_t* wsm = rsmem + wib * R.warp_smem;
    const int64_t slot = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    int32_t* stk = TRACE ? R.A.stack + slot * R.A.stack_slot : nullptr;
    // the warp queue's largest items first, each on the whole block: its 128
    // threads split the diagonals of every step (one block barrier a step),
    // in warp 0's shared memory and stack
    const int nblock = R.block_count ? *R.block_count : 0;
    if (nblock > 0) {
        int32_t* bstk = TRACE ? R.A.stack + (int64_t)blockIdx.x * (blockDim.x >> 5) * R.A.stack_slot : nullptr;
        for (;;) {
            if (threadIdx.x == 0) s_q = atomicAdd(R.block_next, 1);
            __syncthreads();
            const int q = s_q;
            __syncthreads();
            if (q >= nblock) break;
            const int2 it = R.big[q];
            run_item<TRACE, 128>(R, it, rsmem, rsmem + 2 * it.y + 3, bstk, threadIdx.x, FULL);
            __syncthreads();
        }
    }
    for (int list = 0; list < 2; ++list) {
        const int2* items = list ? R.esc : R.big;
        const int cnt = list ? *R.esc_count : *R.big_count;
        int32_t* next = list ? R.esc_next : R.big_next;
        const int first = list ? 0 : nblock;            // (items before it ran on blocks)
        if constexpr (G < 32) {
            group_phase<TRACE, G>(R, items, cnt, next, first, wsm, stk, lane);
            __syncwarp();
            continue;
        }
        for (;;) {
            int q = 0;
            if (lane == 0) q = atomicAdd(next, 1) + first;
            q = __shfl_sync(FULL, q, 0);
            if (q >= cnt) break;
            __syncwarp();
            const int2 it = items[q];
            run_item<TRACE, 32>(R, it, wsm, wsm + 2 * it.y + 3, stk, lane, FULL);
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------- routing --
// The fused kernel in learned.cu writes every pair's queue item (route.cuh)
// and the bucket counts; a scan turns counts into queue offsets and a scatter
// fills the queues.
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
            if (q == 0 && b == BLOCK_BITS) counts[2 * ROUTE_BUCKETS + 2] = acc;   // whole-block items
        }
        counts[2 * ROUTE_BUCKETS + q] = acc;
    }
}

// Warp-aggregated: lanes with the same (queue, bucket) take one atomic.
__global__ void route_scatter_kernel(int n, const int32_t* __restrict__ item, int32_t* __restrict__ starts,
                                     int2* __restrict__ big, int2* __restrict__ small)
{
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    for (int p0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); p0 < n; p0 += stride) {
        const int p = p0 + lane;
        const int it = p < n ? item[p] : -1;
        const int key = it < 0 ? -1 : (it & 0xff), s = it >> 8;
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

// Lanes per warp-queue pair the warp kernel uses: `group` (8, 16 or 32) when
// the two wavefronts of 32 / group pairs at the batch smax fit a warp's share
// of shared memory comfortably (smax <= GROUP_SMAX_MAX), else 32.
constexpr int GROUP_SMAX_MAX = 128;
int routed_group(int smax, int group)
{
    return (group == 8 || group == 16) && smax <= GROUP_SMAX_MAX ? group : 32;
}

// Stack ints per warp slot of the warp kernel: one pair per group at the batch
// smax.
int64_t routed_stack_slot(int smax, int group) { return (int64_t)(32 / group) * (smax + 1) * (smax + 1); }

// 16-bit walk records per warp slot of the lane kernel.
int64_t lane_rec_slot() { return (int64_t)LANE_STACK * 32; }

cudaError_t launch_route(int n, const int32_t* item, int32_t* counts, int32_t* starts, int2* big, int2* small,
                         cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    int blocks = (n + 255) / 256;
    blocks = std::min(blocks, device_sms() * 8);
    launch_begin(K_ROUTE, st);
    route_scan_kernel<<<1, 32, 0, st>>>(counts, starts);
    launch_end(K_ROUTE, st);
    launch_begin(K_ROUTE, st);
    route_scatter_kernel<<<blocks, 256, 0, st>>>(n, item, starts, big, small);
    launch_end(K_ROUTE, st);
    return cudaGetLastError();
}

// Shared-memory ints per warp of the warp kernel: two wavefronts per group (a
// multiple of 4, so every warp's area is 16-byte aligned).
int routed_warp_smem(int smax, int group) { return ((32 / group) * 2 * (2 * smax + 3) + 3) / 4 * 4; }

template <typename K>
static int per_sm_for(K kernel, size_t smem)
{
    return blocks_per_sm((const void*)kernel, 128, smem);
}

template <bool TRACE>
static const void* routed_kernel(int group)
{
    if (group == 8) return (const void*)wfa_routed_kernel<TRACE, 8>;
    if (group == 16) return (const void*)wfa_routed_kernel<TRACE, 16>;
    return (const void*)wfa_routed_kernel<TRACE, 32>;
}

int routed_max_slots(int smax, bool trace, int sm_count, int group)
{
    const size_t smem = (size_t)4 * routed_warp_smem(smax, group) * sizeof(int32_t);
    const int per_sm = blocks_per_sm(trace ? routed_kernel<true>(group) : routed_kernel<false>(group), 128, smem);
    return per_sm * sm_count * 4;
}

int lane_max_slots(bool trace, int sm_count)
{
    const size_t smem = (size_t)4 * LANE_WARP_SMEM * sizeof(uint32_t);
    const int per_sm = trace ? per_sm_for(wfa_lane_kernel<true>, smem) : per_sm_for(wfa_lane_kernel<false>, smem);
    return per_sm * sm_count * 4;
}

cudaError_t launch_routed(const RoutedArgs& R, int lane_slots, int slots, cudaStream_t st)
{
    const size_t lsm = (size_t)4 * LANE_WARP_SMEM * sizeof(uint32_t);
    launch_begin(K_WFA_LANE, st);
    if (R.A.trace) wfa_lane_kernel<true><<<(lane_slots + 3) / 4, 128, lsm, st>>>(R);
    else wfa_lane_kernel<false><<<(lane_slots + 3) / 4, 128, lsm, st>>>(R);
    launch_end(K_WFA_LANE, st);
    const size_t smem = (size_t)4 * R.warp_smem * sizeof(int32_t);
    const int blocks = (slots + 3) / 4;
    launch_begin(K_WFA_ROUTED, st);
    if (R.group == 8) {
        if (R.A.trace) wfa_routed_kernel<true, 8><<<blocks, 128, smem, st>>>(R);
        else wfa_routed_kernel<false, 8><<<blocks, 128, smem, st>>>(R);
    } else if (R.group == 16) {
        if (R.A.trace) wfa_routed_kernel<true, 16><<<blocks, 128, smem, st>>>(R);
        else wfa_routed_kernel<false, 16><<<blocks, 128, smem, st>>>(R);
    } else {
        if (R.A.trace) wfa_routed_kernel<true, 32><<<blocks, 128, smem, st>>>(R);
        else wfa_routed_kernel<false, 32><<<blocks, 128, smem, st>>>(R);
    }
    launch_end(K_WFA_ROUTED, st);
    return cudaGetLastError();
}

}  // namespace ga
