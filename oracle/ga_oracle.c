/*
 * ga_oracle.c -- CPU oracle for batched pairwise alignment.
 *
 * TEST INFRASTRUCTURE ONLY. This file is a plain-C restatement of the
 * reference's CPU path for align_batch (WFA edit distance + CIGAR) and
 * align_sw_batch (affine Smith-Waterman + CIGAR).  It is loaded by the test
 * suite, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and
 * only there, as the checker.  The product (genoaligner_gb300/) never links
 * or calls it.
 *
 * Parity is pinned: tests/golden/ holds vectors produced by the reference's
 * own kernel bodies compiled for the host (oracle/ref_wrap.cpp), and
 * tests/test_oracle.py checks this file against them.
 *
 * Every function cites the reference code it restates (paths are relative to
 * the reference project root).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define ORA_NULL (INT32_MIN / 2)          /* wfa_kernel.hip:103 (WFA_NEG) */

/* Threshold reachability test: a NULL offset that had +1 applied is still
 * unreachable.  wfa_kernel.hip:110 */
static inline int ora_live(int off) { return off > ORA_NULL + 1024; }

/* CIGAR op codes shared by WFA and SW (wfa_kernel.hip:297-313,
 * sw_kernel.hip:212-215). */
enum { OP_M = 0, OP_X = 1, OP_I = 2, OP_D = 3 };
static const char OP_CHAR[4] = {'M', 'X', 'I', 'D'};

/* Append one op to a reversed CIGAR, refusing past the capacity.
 * wfa_kernel.hip:297-302, sw_kernel_impl.hip:182-188 */
static inline int push_op(int8_t* rev, int cap, int* used, int op)
{
    if (*used >= cap) return 0;
    rev[*used] = (int8_t)op;
    *used += 1;
    return 1;
}

/* ------------------------------------------------------------------ WFA -- */

/* Number of int32 slots the WFA trace workspace needs for one pair:
 * one wavefront of 2*smax+3 slots per score 0..smax (api.cpp:390-392). */
size_t ora_wfa_ws_slots(int smax)
{
    return (size_t)(smax + 1) * (size_t)(2 * smax + 3);
}

/* Backward walk over the stored wavefronts, edit-distance case.
 * Restates wfa_traceback (wfa_kernel.hip:338-437): candidates from score s-1
 * are misms = W[k]+1, ins = W[k-1]+1, del = W[k+1]; misms wins ties, ins and
 * del must be strictly better; the gap between the current offset and the
 * chosen candidate is a run of matches; ops are emitted in reverse. */
static void wfa_walk(int m, int n, int smax, int score_total, const int32_t* ws,
                     int stride, int8_t* rev, int cap, int* used)
{
#define WS(s, k) ws[(size_t)(s) * (size_t)stride + (size_t)((k) + smax + 1)]
    const int kfinal = n - m;
    int s = score_total, k = kfinal;
    if (k < -s || k > s) return;
    int off = WS(s, k);
    if (off == ORA_NULL) return;
    int h = off, v = off - k;
    /* ops that fall outside the grid come last in reading order
     * (wfa_kernel.hip:309-313) */
    for (int t = v - m; t > 0; --t) push_op(rev, cap, used, OP_D);
    for (int t = h - n; t > 0; --t) push_op(rev, cap, used, OP_I);
    if (v > m) v = m;
    if (h > n) h = n;
    while (v > 0 && h > 0 && s > 0) {
        const int sp = s - 1;
        int c_mis = ORA_NULL, c_ins = ORA_NULL, c_del = ORA_NULL;
        if (k >= -sp && k <= sp)         c_mis = WS(sp, k) + 1;
        if (k - 1 >= -sp && k - 1 <= sp) c_ins = WS(sp, k - 1) + 1;
        if (k + 1 >= -sp && k + 1 <= sp) c_del = WS(sp, k + 1);
        int best = ORA_NULL, op = -1;
        if (ora_live(c_mis) && c_mis >= best) { best = c_mis; op = OP_X; }
        if (ora_live(c_ins) && c_ins >  best) { best = c_ins; op = OP_I; }
        if (ora_live(c_del) && c_del >  best) { best = c_del; op = OP_D; }
        if (op < 0) break;
        for (int t = off - best; t > 0; --t) push_op(rev, cap, used, OP_M);
        off = best;
        push_op(rev, cap, used, op);
        if (op == OP_X)      { off -= 1; }
        else if (op == OP_I) { k -= 1; off -= 1; }
        else                 { k += 1; }
        h = off;
        v = off - k;
        s -= 1;
    }
    /* leading matches, then leading D, then leading I (wfa_kernel.hip:429-436) */
    if (v > 0 && h > 0) {
        const int run = v < h ? v : h;
        for (int t = 0; t < run; ++t) push_op(rev, cap, used, OP_M);
        v -= run;
        h -= run;
    }
    for (; v > 0; --v) push_op(rev, cap, used, OP_D);
    for (; h > 0; --h) push_op(rev, cap, used, OP_I);
#undef WS
}

/* One pair through the WFA trace path: restates wfa_trace_kernel
 * (wfa_kernel.hip:467-592).  `ws` must hold ora_wfa_ws_slots(smax) ints; the
 * whole slice is reset to NULL first, as the reference does (:531-532), so the
 * CPU cost of this function tracks the reference's.  Returns the score (-1 when
 * the distance exceeds smax) and the reversed op codes in `rev`. */
int ora_wfa_trace_pair(const char* P, int m, const char* T, int n, int smax,
                       int32_t* ws, int8_t* rev, int cap, int* used, int* trunc)
{
    *used = 0;
    *trunc = 0;
    if (m <= 0 || n <= 0) {
        /* degenerate: the other length, all I (m==0) then all D (n==0) */
        for (int i = 0; i < n; ++i) push_op(rev, cap, used, OP_I);
        for (int i = 0; i < m; ++i) push_op(rev, cap, used, OP_D);
        *trunc = (*used >= cap) ? 1 : 0;
        return (m <= 0) ? n : m;
    }
    const int stride = 2 * smax + 3;
    const size_t slots = ora_wfa_ws_slots(smax);
    for (size_t t = 0; t < slots; ++t) ws[t] = ORA_NULL;
#define WS(s, k) ws[(size_t)(s) * (size_t)stride + (size_t)((k) + smax + 1)]
    int o = 0;
    while (o < m && o < n && P[o] == T[o]) ++o;
    WS(0, 0) = o;
    const int kfinal = n - m;
    int score = -1;
    if (kfinal == 0 && o >= n) {
        score = 0;
    } else {
        for (int s = 1; s <= smax; ++s) {
            for (int k = -s; k <= s; ++k) {
                /* compute-next: wfa_kernel.hip:119-127 */
                const int ins = WS(s - 1, k - 1);
                const int del = WS(s - 1, k + 1);
                const int mis = WS(s - 1, k);
                const int mid = ins > mis ? ins : mis;
                int x = del > mid + 1 ? del : mid + 1;
                if (!ora_live(x) || x > n || x - k > m) {
                    x = ORA_NULL;
                } else {
                    /* extension: wfa_kernel.hip:130-136 */
                    int vv = x - k, hh = x;
                    while (vv < m && hh < n && P[vv] == T[hh]) { ++vv; ++hh; ++x; }
                }
                WS(s, k) = x;
            }
            if (kfinal >= -s && kfinal <= s) {
                const int fo = WS(s, kfinal);
                if (ora_live(fo) && fo >= n) { score = s; break; }
            }
        }
    }
#undef WS
    if (score < 0) return -1;
    if (score == 0) {
        for (int i = 0; i < n; ++i) push_op(rev, cap, used, OP_M);
        *trunc = (*used >= cap) ? 1 : 0;
        return 0;
    }
    wfa_walk(m, n, smax, score, ws, stride, rev, cap, used);
    *trunc = (*used > 0 && *used >= cap) ? 1 : 0;
    return score;
}

/* Score-only WFA: restates wfa_score_kernel_flat (wfa_score_flat.hip:63-140)
 * with two ping-pong wavefronts.  `ws` must hold 2*(2*smax+3) ints. */
int ora_wfa_score_pair(const char* P, int m, const char* T, int n, int smax, int32_t* ws)
{
    if (m <= 0 || n <= 0) return (m <= 0) ? n : m;
    const int stride = 2 * smax + 3;
    int32_t* prev = ws;
    int32_t* cur = ws + stride;
    for (int t = 0; t < 2 * stride; ++t) ws[t] = ORA_NULL;
    int o = 0;
    while (o < m && o < n && P[o] == T[o]) ++o;
    prev[smax + 1] = o;
    const int kfinal = n - m;
    if (kfinal == 0 && o >= n) return 0;
    for (int s = 1; s <= smax; ++s) {
        for (int k = -s; k <= s; ++k) {
            const int ins = prev[k - 1 + smax + 1];
            const int del = prev[k + 1 + smax + 1];
            const int mis = prev[k + smax + 1];
            const int mid = ins > mis ? ins : mis;
            int x = del > mid + 1 ? del : mid + 1;
            if (!ora_live(x) || x > n || x - k > m) {
                x = ORA_NULL;
            } else {
                int vv = x - k, hh = x;
                while (vv < m && hh < n && P[vv] == T[hh]) { ++vv; ++hh; ++x; }
            }
            cur[k + smax + 1] = x;
        }
        if (kfinal >= -s && kfinal <= s) {
            const int fo = cur[kfinal + smax + 1];
            if (ora_live(fo) && fo >= n) return s;
        }
        int32_t* t = prev; prev = cur; cur = t;
    }
    return -1;
}

/* Levenshtein distance by the O(mn) rolling-row DP: restates edit_distance_cpu
 * (src/reference/edit_distance_cpu.hpp:19-39). */
int ora_edit_distance(const char* P, int m, const char* T, int n)
{
    if (m == 0) return n;
    if (n == 0) return m;
    int* prev = (int*)malloc(sizeof(int) * (size_t)(n + 1) * 2);
    if (!prev) return -2;
    int* cur = prev + n + 1;
    for (int j = 0; j <= n; ++j) prev[j] = j;
    for (int i = 1; i <= m; ++i) {
        cur[0] = i;
        for (int j = 1; j <= n; ++j) {
            int v = prev[j - 1] + (P[i - 1] == T[j - 1] ? 0 : 1);
            if (prev[j] + 1 < v) v = prev[j] + 1;
            if (cur[j - 1] + 1 < v) v = cur[j - 1] + 1;
            cur[j] = v;
        }
        int* t = prev; prev = cur; cur = t;
    }
    const int r = prev[n];
    free(prev < cur ? prev : cur);
    return r;
}

/* The WFA result check: M only on equal bytes, X only on unequal, every X/I/D
 * costs one, both sequences consumed exactly.  Restates validate
 * (src/api/api.cpp:84-106). */
void ora_wfa_validate(const char* cigar, int len, int score, const char* P, int m,
                      const char* T, int n, int* rescore_ok, int* wellformed_ok)
{
    int s = 0, pi = 0, ti = 0, wf = 1;
    for (int c = 0; c < len; ++c) {
        switch (cigar[c]) {
            case 'M':
                if (pi >= m || ti >= n || P[pi] != T[ti]) wf = 0;
                ++pi; ++ti; break;
            case 'X':
                if (pi >= m || ti >= n || P[pi] == T[ti]) wf = 0;
                ++pi; ++ti; ++s; break;
            case 'I': ++ti; ++s; break;
            case 'D': ++pi; ++s; break;
            default: wf = 0; break;
        }
    }
    if (pi != m || ti != n) wf = 0;
    *wellformed_ok = wf;
    *rescore_ok = (s == score);
}

/* API-level WFA result for one pair, given the batch's smax, whether the batch
 * runs the trace path (any request with_cigar) and the batch CIGAR capacity.
 * Restates src/api/api.cpp:456-469 (trace path) and :485-488 (score path).
 * `cigar` receives the decoded string (forward order), `cigar_len` its length
 * (0 when no CIGAR is reported). */
int ora_wfa_result(const char* P, int m, const char* T, int n, int smax, int trace,
                   int cigar_cap, int32_t* ws, int8_t* rev, char* cigar, int* cigar_len,
                   int* rescore_ok, int* wellformed_ok)
{
    *cigar_len = 0;
    *rescore_ok = 0;
    *wellformed_ok = 0;
    if (!trace) return ora_wfa_score_pair(P, m, T, n, smax, ws);
    int used = 0, trunc = 0;
    const int score = ora_wfa_trace_pair(P, m, T, n, smax, ws, rev, cigar_cap, &used, &trunc);
    if (score >= 0 && !trunc && used > 0) {
        for (int j = 0; j < used; ++j) cigar[j] = OP_CHAR[rev[used - 1 - j]];
        *cigar_len = used;
        ora_wfa_validate(cigar, used, score, P, m, T, n, rescore_ok, wellformed_ok);
    }
    return score;
}

/* ------------------------------------------------------------------- SW -- */

typedef struct { int match, mismatch, gap_open, gap_extend; } ora_sw_scoring;

/* Direction byte fields of the trace recurrence (sw_kernel.hip:218-223). */
enum { D_STOP = 0, D_DIAG = 1, D_E = 2, D_F = 3, D_EEXT = 4, D_FEXT = 8 };

/* Too-large sentinel of the trace kernel (sw_kernel.hip:227). */
#define ORA_SW_TOO_BIG (-(1 << 30))

/* Affine local alignment with one direction byte per cell, then the backward
 * walk.  Restates sw_trace_kernel (sw_kernel_impl.hip:252-336) and
 * sw_trace_walk (:198-242): e/f extend only when strictly greater than
 * opening; H takes diag, then E if strictly greater, then F if strictly
 * greater; h <= 0 is a stop; the best cell is the first strictly greater one
 * in row-major order; the walk follows hsrc, then stays in a gap while the
 * current cell's extend bit is set.
 *
 * text is the row axis (m), pattern the column axis (n).  `dir_limit` is the
 * caller's direction-table capacity in cells: a pair with (m+1)(n+1) above it
 * returns ORA_SW_TOO_BIG (sw_kernel_impl.hip:275-280).  `dirs` must hold
 * (m+1)(n+1) bytes and `rowbuf` 2(n+1) ints.  Coordinates come back 0-based,
 * -1 for score 0. */
int ora_sw_trace_pair(const char* T, int m, const char* P, int n, ora_sw_scoring sc,
                      long long dir_limit, uint8_t* dirs, int32_t* rowbuf,
                      int8_t* rev, int cap, int* used, int* trunc,
                      int* start_i, int* start_j, int* end_i, int* end_j)
{
    *used = 0;
    *trunc = 0;
    *start_i = *start_j = *end_i = *end_j = -1;
    if (m <= 0 || n <= 0) return 0;
    const int rs = n + 1;
    if ((long long)(m + 1) * (long long)rs > dir_limit) return ORA_SW_TOO_BIG;
    int32_t* hrow = rowbuf;
    int32_t* frow = rowbuf + rs;
    for (int j = 0; j <= n; ++j) { hrow[j] = 0; frow[j] = 0; dirs[j] = D_STOP; }
    for (int i = 0; i <= m; ++i) dirs[(size_t)i * rs] = D_STOP;
    const int go = sc.gap_open, ge = sc.gap_extend;
    int best = 0, bi = -1, bj = -1;
    for (int i = 1; i <= m; ++i) {
        const char a = T[i - 1];
        int hleft = 0, eleft = 0, diag = 0;
        uint8_t* drow = dirs + (size_t)i * rs;
        for (int j = 1; j <= n; ++j) {
            int e = hleft - go, eb = 0;
            if (eleft - ge > e) { e = eleft - ge; eb = D_EEXT; }
            int f = hrow[j] - go, fb = 0;
            if (frow[j] - ge > f) { f = frow[j] - ge; fb = D_FEXT; }
            int h = diag + (a == P[j - 1] ? sc.match : sc.mismatch);
            int src = D_DIAG;
            if (e > h) { h = e; src = D_E; }
            if (f > h) { h = f; src = D_F; }
            if (h <= 0) { h = 0; src = D_STOP; }
            drow[j] = (uint8_t)(src | eb | fb);
            diag = hrow[j];
            hrow[j] = h;
            frow[j] = f;
            hleft = h;
            eleft = e;
            if (h > best) { best = h; bi = i; bj = j; }
        }
    }
    if (best <= 0) return 0;
    /* backward walk: state 0 = on H, 1 = in an E run (D ops), 2 = in an F run (I ops) */
    int i = bi, j = bj, state = 0, ok = 1;
    while (i > 0 && j > 0) {
        const uint8_t b = dirs[(size_t)i * rs + j];
        if (state == 0) {
            const int src = b & 3;
            if (src == D_STOP) break;
            if (src == D_DIAG) {
                ok &= push_op(rev, cap, used, T[i - 1] == P[j - 1] ? OP_M : OP_X);
                --i; --j;
            } else if (src == D_E) {
                ok &= push_op(rev, cap, used, OP_D);
                state = (b & D_EEXT) ? 1 : 0;
                --j;
            } else {
                ok &= push_op(rev, cap, used, OP_I);
                state = (b & D_FEXT) ? 2 : 0;
                --i;
            }
        } else if (state == 1) {
            ok &= push_op(rev, cap, used, OP_D);
            --j;
            if (!(b & D_EEXT)) state = 0;
        } else {
            ok &= push_op(rev, cap, used, OP_I);
            --i;
            if (!(b & D_FEXT)) state = 0;
        }
    }
    *start_i = i;
    *start_j = j;
    *end_i = bi - 1;
    *end_j = bj - 1;
    *trunc = ok ? 0 : 1;
    return best;
}

/* Score-only SW with the reference's end-cell rule (sw_kernel_impl.hip:22-168).
 * The H values are the plain recurrence's; the end cell is chosen the way the
 * warp kernel chooses it: lane L (of `warp` lanes) owns columns j with
 * (j-1) mod warp == L and keeps the first cell, in row-major order, whose H is
 * strictly above its running best (starting at 0); the lanes then reduce with
 * an xor butterfly in which a lane adopts its partner's triple only when the
 * partner's score is strictly greater, and lane 0 reports.  The butterfly is
 * simulated step by step here.  `rowbuf` must hold 2(n+1) ints. */
int ora_sw_score_pair(const char* T, int m, const char* P, int n, ora_sw_scoring sc,
                      int warp, int32_t* rowbuf, int* end_i, int* end_j)
{
    *end_i = *end_j = -1;
    if (m <= 0 || n <= 0) return 0;
    if (warp < 1 || warp > 64) return -2;
    int lb[64], li[64], lj[64];
    for (int l = 0; l < warp; ++l) { lb[l] = 0; li[l] = -1; lj[l] = -1; }
    int32_t* hrow = rowbuf;
    int32_t* frow = rowbuf + (n + 1);
    for (int j = 0; j <= n; ++j) { hrow[j] = 0; frow[j] = 0; }
    const int go = sc.gap_open, ge = sc.gap_extend;
    for (int i = 1; i <= m; ++i) {
        const char a = T[i - 1];
        int hleft = 0, eleft = 0, diag = 0;
        for (int j = 1; j <= n; ++j) {
            int e = hleft - go;
            if (eleft - ge > e) e = eleft - ge;
            int f = hrow[j] - go;
            if (frow[j] - ge > f) f = frow[j] - ge;
            int h = diag + (a == P[j - 1] ? sc.match : sc.mismatch);
            if (e > h) h = e;
            if (f > h) h = f;
            if (h < 0) h = 0;
            diag = hrow[j];
            hrow[j] = h;
            frow[j] = f;
            hleft = h;
            eleft = e;
            const int l = (j - 1) % warp;
            if (h > lb[l]) { lb[l] = h; li[l] = i - 1; lj[l] = j - 1; }
        }
    }
    for (int off = warp / 2; off > 0; off >>= 1) {
        int nb[64], ni[64], nj[64];
        for (int l = 0; l < warp; ++l) {
            const int p = l ^ off;
            nb[l] = lb[l]; ni[l] = li[l]; nj[l] = lj[l];
            if (lb[p] > lb[l]) { nb[l] = lb[p]; ni[l] = li[p]; nj[l] = lj[p]; }
        }
        memcpy(lb, nb, sizeof(int) * (size_t)warp);
        memcpy(li, ni, sizeof(int) * (size_t)warp);
        memcpy(lj, nj, sizeof(int) * (size_t)warp);
    }
    *end_i = li[0];
    *end_j = lj[0];
    return lb[0];
}

/* The SW result check over the reported span: a run of k consecutive I (or D)
 * ops is one gap costing gap_open + (k-1)*gap_extend; M needs equal bytes, X
 * unequal; the walk must land exactly one past each end.  Restates sw_validate
 * (src/api/api.cpp:114-156). */
void ora_sw_validate(const char* cigar, int len, const char* T, int m, int si, int ei,
                     const char* P, int n, int sj, int ej, ora_sw_scoring sc, int score,
                     int* rescore_ok, int* wellformed_ok)
{
    int i = si, j = sj, s = 0, run = 0, wf = 1;
    for (int c = 0; c < len; ++c) {
        const char op = cigar[c];
        if (op == 'M' || op == 'X') {
            if (run != 0) {
                const int L = run > 0 ? run : -run;
                s -= sc.gap_open + (L - 1) * sc.gap_extend;
                run = 0;
            }
            if (i > ei || j > ej || i >= m || j >= n) wf = 0;
            else if ((op == 'M') != (T[i] == P[j])) wf = 0;
            s += (op == 'M') ? sc.match : sc.mismatch;
            ++i; ++j;
        } else if (op == 'I') {
            if (run < 0) { s -= sc.gap_open + (-run - 1) * sc.gap_extend; run = 0; }
            if (i > ei || i >= m) wf = 0;
            ++i; ++run;
        } else if (op == 'D') {
            if (run > 0) { s -= sc.gap_open + (run - 1) * sc.gap_extend; run = 0; }
            if (j > ej || j >= n) wf = 0;
            ++j; --run;
        } else {
            wf = 0;
        }
    }
    if (run != 0) {
        const int L = run > 0 ? run : -run;
        s -= sc.gap_open + (L - 1) * sc.gap_extend;
    }
    if (i != ei + 1 || j != ej + 1) wf = 0;
    *wellformed_ok = wf;
    *rescore_ok = wf && (s == score);
}

/* --------------------------------------------------------- batch drivers -- */

/* One WFA pair's result fields, laid out for numpy structured arrays. */
typedef struct {
    int32_t score, resolved, rescore_ok, wellformed_ok;
    int64_t cigar_off;
    int32_t cigar_len, pad;
} ora_wfa_out;

/* One SW pair's result fields. */
typedef struct {
    int32_t score, resolved, start_i, start_j, end_i, end_j;
    int32_t rescore_ok, wellformed_ok, too_large, pad;
    int64_t cigar_off;
    int32_t cigar_len, pad2;
} ora_sw_out;

typedef struct {
    /* inputs: sequence i's bytes are buf[off[i] .. off[i]+len[i]) */
    const char* pbuf; const int64_t* poff; const int32_t* plen;
    const char* tbuf; const int64_t* toff; const int32_t* tlen;
    const uint8_t* want_cigar;   /* per pair; SW only */
    int32_t n, smax, trace, cigar_cap;
    ora_sw_scoring sc;
    long long dir_limit;
    /* outputs */
    char* cigars; const int64_t* cig_off;   /* cigar of pair i at cigars + cig_off[i] */
    void* out;
    /* work split */
    int32_t next;
    pthread_mutex_t mu;
    int error;
} ora_job;

static int job_take(ora_job* J, int chunk, int* lo, int* hi)
{
    pthread_mutex_lock(&J->mu);
    *lo = J->next;
    J->next += chunk;
    pthread_mutex_unlock(&J->mu);
    if (*lo >= J->n) return 0;
    *hi = *lo + chunk < J->n ? *lo + chunk : J->n;
    return 1;
}

static void* wfa_worker(void* arg)
{
    ora_job* J = (ora_job*)arg;
    int32_t* ws = (int32_t*)malloc(sizeof(int32_t) * (ora_wfa_ws_slots(J->smax) + 8));
    int maxlen = J->cigar_cap + 8;
    int8_t* rev = (int8_t*)malloc((size_t)maxlen);
    if (!ws || !rev) { J->error = 1; free(ws); free(rev); return NULL; }
    ora_wfa_out* out = (ora_wfa_out*)J->out;
    int lo, hi;
    while (job_take(J, 16, &lo, &hi)) {
        for (int i = lo; i < hi; ++i) {
            ora_wfa_out* o = &out[i];
            char* cg = J->cigars ? J->cigars + J->cig_off[i] : NULL;
            int rs = 0, wf = 0, cl = 0;
            char dummy[1];
            o->score = ora_wfa_result(J->pbuf + J->poff[i], J->plen[i],
                                      J->tbuf + J->toff[i], J->tlen[i], J->smax, J->trace,
                                      J->cigar_cap, ws, rev, cg ? cg : dummy, &cl, &rs, &wf);
            o->resolved = o->score >= 0;
            o->rescore_ok = rs;
            o->wellformed_ok = wf;
            o->cigar_len = cl;
            o->cigar_off = J->cig_off ? J->cig_off[i] : 0;
        }
    }
    free(ws);
    free(rev);
    return NULL;
}

static int run_workers(ora_job* J, void* (*fn)(void*), int threads)
{
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t tid[256];
    pthread_mutex_init(&J->mu, NULL);
    J->next = 0;
    J->error = 0;
    int started = 0;
    for (int t = 1; t < threads; ++t)
        if (pthread_create(&tid[started], NULL, fn, J) == 0) ++started;
    fn(J);
    for (int t = 0; t < started; ++t) pthread_join(tid[t], NULL);
    pthread_mutex_destroy(&J->mu);
    return J->error ? -1 : 0;
}

/* WFA batch.  `smax` is the batch smax (the requests' minimum), `trace` is 1
 * when any request asks for a CIGAR, `cigar_cap` the batch capacity
 * max(m+n+2).  CIGAR i is written at cigars + cig_off[i] (room for m+n
 * bytes), or nowhere when cigars is NULL. */
int ora_wfa_batch(int32_t n, const char* pbuf, const int64_t* poff, const int32_t* plen,
                  const char* tbuf, const int64_t* toff, const int32_t* tlen,
                  int32_t smax, int32_t trace, int32_t cigar_cap,
                  char* cigars, const int64_t* cig_off, ora_wfa_out* out, int32_t threads)
{
    ora_job J;
    memset(&J, 0, sizeof(J));
    J.pbuf = pbuf; J.poff = poff; J.plen = plen;
    J.tbuf = tbuf; J.toff = toff; J.tlen = tlen;
    J.n = n; J.smax = smax; J.trace = trace; J.cigar_cap = cigar_cap;
    J.cigars = cigars; J.cig_off = cig_off; J.out = out;
    return run_workers(&J, wfa_worker, threads);
}

static void* sw_worker(void* arg)
{
    ora_job* J = (ora_job*)arg;
    ora_sw_out* out = (ora_sw_out*)J->out;
    size_t dir_cap = 0, row_cap = 0, rev_cap = 0;
    uint8_t* dirs = NULL;
    int32_t* rowbuf = NULL;
    int8_t* rev = NULL;
    int lo, hi;
    while (job_take(J, 1, &lo, &hi)) {
        for (int i = lo; i < hi; ++i) {
            ora_sw_out* o = &out[i];
            const int m = J->tlen[i], n = J->plen[i];
            const char* T = J->tbuf + J->toff[i];
            const char* P = J->pbuf + J->poff[i];
            memset(o, 0, sizeof(*o));
            o->score = -1;
            o->start_i = o->start_j = o->end_i = o->end_j = -1;
            o->cigar_off = J->cig_off ? J->cig_off[i] : 0;
            const size_t need_row = 2 * (size_t)(n + 1) + 2;
            if (need_row > row_cap) {
                free(rowbuf);
                row_cap = need_row;
                rowbuf = (int32_t*)malloc(sizeof(int32_t) * row_cap);
                if (!rowbuf) { J->error = 1; return NULL; }
            }
            if (!J->trace) {
                int ei = -1, ej = -1;
                const int s = ora_sw_score_pair(T, m, P, n, J->sc, 32, rowbuf, &ei, &ej);
                if (s < 0) continue;
                o->score = s; o->resolved = 1; o->end_i = ei; o->end_j = ej;
                if (s == 0) { o->rescore_ok = o->wellformed_ok = 1; }
                continue;
            }
            const long long cells = (long long)(m + 1) * (long long)(n + 1);
            if (m > 0 && n > 0 && cells <= J->dir_limit && (size_t)cells > dir_cap) {
                free(dirs);
                dir_cap = (size_t)cells;
                dirs = (uint8_t*)malloc(dir_cap);
                if (!dirs) { J->error = 1; return NULL; }
            }
            const size_t need_rev = (size_t)J->cigar_cap + 8;
            if (need_rev > rev_cap) {
                free(rev);
                rev_cap = need_rev;
                rev = (int8_t*)malloc(rev_cap);
                if (!rev) { J->error = 1; return NULL; }
            }
            int used = 0, trunc = 0, si, sj, ei, ej;
            const int s = ora_sw_trace_pair(T, m, P, n, J->sc, J->dir_limit, dirs, rowbuf,
                                            rev, J->cigar_cap, &used, &trunc, &si, &sj, &ei, &ej);
            /* result fill: restates sw_fill_trace_results (src/api/api.cpp:542-580) */
            if (s == ORA_SW_TOO_BIG) { o->too_large = 1; continue; }
            if (s < 0) continue;
            o->score = s; o->resolved = 1; o->end_i = ei; o->end_j = ej;
            if (s == 0) { o->rescore_ok = o->wellformed_ok = 1; continue; }
            if (J->want_cigar && !J->want_cigar[i]) continue;
            o->start_i = si; o->start_j = sj;
            if (!trunc && used > 0 && J->cigars) {
                char* cg = J->cigars + J->cig_off[i];
                for (int q = 0; q < used; ++q) cg[q] = OP_CHAR[rev[used - 1 - q]];
                o->cigar_len = used;
                int rs = 0, wf = 0;
                ora_sw_validate(cg, used, T, m, si, ei, P, n, sj, ej, J->sc, s, &rs, &wf);
                o->rescore_ok = rs;
                o->wellformed_ok = wf;
            }
        }
    }
    free(dirs);
    free(rowbuf);
    free(rev);
    return NULL;
}

/* SW batch.  text is the row axis.  `trace` is 1 when any request asks for a
 * CIGAR (the trace kernel then serves every pair, src/api/api.cpp:750-784);
 * `want_cigar[i]` says whether pair i asked; `dir_limit` is the per-pair
 * direction-table limit in cells; `cigar_cap` is max_m+max_n+4. */
int ora_sw_batch(int32_t n, const char* tbuf, const int64_t* toff, const int32_t* tlen,
                 const char* pbuf, const int64_t* poff, const int32_t* plen,
                 int32_t match, int32_t mismatch, int32_t gap_open, int32_t gap_extend,
                 int32_t trace, const uint8_t* want_cigar, long long dir_limit,
                 int32_t cigar_cap, char* cigars, const int64_t* cig_off,
                 ora_sw_out* out, int32_t threads)
{
    ora_job J;
    memset(&J, 0, sizeof(J));
    J.pbuf = pbuf; J.poff = poff; J.plen = plen;
    J.tbuf = tbuf; J.toff = toff; J.tlen = tlen;
    J.want_cigar = want_cigar;
    J.n = n; J.trace = trace; J.cigar_cap = cigar_cap;
    J.sc.match = match; J.sc.mismatch = mismatch;
    J.sc.gap_open = gap_open; J.sc.gap_extend = gap_extend;
    J.dir_limit = dir_limit;
    J.cigars = cigars; J.cig_off = cig_off; J.out = out;
    return run_workers(&J, sw_worker, threads);
}

/* Batch edit distance (score cross-check). */
typedef struct { ora_job* J; int32_t* out; } ed_arg;

static void* ed_worker(void* arg)
{
    ora_job* J = (ora_job*)arg;
    int32_t* out = (int32_t*)J->out;
    int lo, hi;
    while (job_take(J, 64, &lo, &hi))
        for (int i = lo; i < hi; ++i)
            out[i] = ora_edit_distance(J->pbuf + J->poff[i], J->plen[i], J->tbuf + J->toff[i], J->tlen[i]);
    return NULL;
}

/* edit_distance_cpu over a batch, on `threads` threads. */
int ora_edit_distance_batch(int32_t n, const char* pbuf, const int64_t* poff, const int32_t* plen,
                            const char* tbuf, const int64_t* toff, const int32_t* tlen,
                            int32_t* out, int32_t threads)
{
    ora_job J;
    memset(&J, 0, sizeof(J));
    J.pbuf = pbuf; J.poff = poff; J.plen = plen;
    J.tbuf = tbuf; J.toff = toff; J.tlen = tlen;
    J.n = n;
    J.out = out;
    return run_workers(&J, ed_worker, threads);
}
