// wfa.cu -- sequence packing and the WFA edit-distance kernels (sm_103a).
//
// Algorithm: the wavefront recurrence of the reference's wfa_trace_kernel /
// wfa_score_kernel_flat (include/genoaligner/backend/wfa_kernel.hip:119-145,
// 467-592; wfa_score_flat.hip:63-140).  Offsets are text coordinates h,
// v = h - k, the alignment diagonal is n - m; compute-next takes
// max(del, max(ins, mism) + 1) and clips to NULL past either end before
// extending; the walk prefers mismatch on ties, then insertion, then deletion
// (strictly).  These steps are fixed by the result contract -- the scores and
// CIGAR strings must be the reference's -- so they are kept, expressed for a
// warp:
//
//   * one warp per pair, persistent: warps pull pair indices from a counter,
//     so long and short pairs balance across the grid;
//   * the diagonals of wavefront s are spread over the 32 lanes; the previous
//     and current wavefront live in a per-warp shared-memory ping-pong;
//   * extension compares 32 bases per step on the 2-bit arena (XOR +
//     find-first-set); pairs with any byte outside ACGT compare 8 raw bytes
//     per step instead, so byte-equality semantics hold for N, lowercase, etc.;
//   * for CIGARs every wavefront is also written to a per-warp triangular stack
//     in global memory (wavefront s at s*s, 2s+1 entries); the walk then runs
//     warp-uniformly over it and writes the CIGAR back to front into the
//     pair's output slot, runs of matches written by all lanes at once.
#include "kernels.cuh"

namespace ga {

// ---------------------------------------------------------------- packing --
// The 2-bit arena: one thread per 32-byte chunk of the byte arena -> one
// 64-bit word (A=0 C=1 G=2 T=3 under ((c>>1)^(c>>2))&3, little-endian).
// Sequences start on 32-byte boundaries, so word index = byte offset / 32 and
// no per-sequence bookkeeping is needed.
__global__ void __launch_bounds__(256) pack_chunks_kernel(const uint8_t* __restrict__ seq, int64_t nchunks,
                                                          uint64_t* __restrict__ packed, uint32_t* __restrict__ bad)
{
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nchunks; c += (int64_t)gridDim.x * blockDim.x) {
        const uint4* src = reinterpret_cast<const uint4*>(seq + 32 * c);
        const uint4 x0 = __ldg(src), x1 = __ldg(src + 1);
        const uint32_t parts[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
        uint64_t word = 0;
        uint32_t badbits = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const uint32_t v = parts[q];
            // four codes of one 32-bit part: ((c >> 1) ^ (c >> 2)) & 3 per byte
            const uint32_t codes = ((v >> 1) ^ (v >> 2)) & 0x03030303u;
            const uint32_t packed4 = (codes & 3u) | ((codes >> 6) & 0xcu) | ((codes >> 12) & 0x30u) | ((codes >> 18) & 0xc0u);
            word |= (uint64_t)packed4 << (8 * q);
            // a byte is A, C, G or T iff it equals "ACGT"[its code]
            const uint32_t sel = (codes & 3u) | ((codes >> 4) & 0x30u) | ((codes >> 8) & 0x300u) | ((codes >> 12) & 0x3000u);
            const uint32_t diff = __byte_perm(0x54474341u, 0u, sel) ^ v;
            const uint32_t nz = ((((diff & 0x7f7f7f7fu) + 0x7f7f7f7fu) | diff) >> 7) & 0x01010101u;
            badbits |= ((nz * 0x10204080u) >> 28) << (4 * q);       // bit 8q+b of nz -> bit 4q+b
        }
        packed[c] = word;
        bad[c] = badbits;
    }
}

// 1 when byte c is one of A, C, G, T.
__device__ __forceinline__ uint32_t acgt_byte(uint32_t c)
{
    // 'A'=0x41 'C'=0x43 'G'=0x47 'T'=0x54: all in 0x40..0x5f; low 5 bits 1, 3, 7, 20
    return ((c >> 5) == 2u) & ((0x0010008au >> (c & 31u)) & 1u);
}

// Purity flag per sequence (a-sides q < n, then b-sides) from the per-chunk
// masks of pack_chunks_kernel: bit b of bad[c] = byte 32c + b is not A/C/G/T.
__global__ void __launch_bounds__(256) purity_mask_kernel(PairDesc D, const uint32_t* __restrict__ bad,
                                                          uint8_t* __restrict__ pure)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 2 * D.n; q += gridDim.x * blockDim.x) {
        const bool is_a = q < D.n;
        const int p = is_a ? q : q - D.n;
        const int64_t c0 = (is_a ? D.a_off[p] : D.b_off[p]) >> 5;
        const int len = is_a ? D.a_len[p] : D.b_len[p];
        const int full = len >> 5, rest = len & 31;
        uint32_t acc = 0;
        for (int w = 0; w < full; ++w) acc |= __ldg(bad + c0 + w);
        if (rest) acc |= __ldg(bad + c0 + full) & ((1u << rest) - 1u);
        pure[q] = (uint8_t)(acc == 0);
    }
}

// Purity flag per sequence straight from the bytes, one thread each (the
// Smith-Waterman paths, which read bytes and build no 2-bit arena).
__global__ void __launch_bounds__(256) purity_kernel(PairDesc D, uint8_t* __restrict__ pure)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 2 * D.n; q += gridDim.x * blockDim.x) {
        const bool is_a = q < D.n;
        const int p = is_a ? q : q - D.n;
        const uint8_t* s = D.seq + (is_a ? D.a_off[p] : D.b_off[p]);
        const int len = is_a ? D.a_len[p] : D.b_len[p];
        uint32_t ok = 1;
        for (int o = 0; o < len && ok; o += 16) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(s + o));
            const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int b = 0; b < 16; ++b)
                if (o + b < len) ok &= acgt_byte((w[b >> 2] >> (8 * (b & 3))) & 0xffu);
        }
        pure[q] = (uint8_t)ok;
    }
}

// ------------------------------------------------------------------- WFA --
// Cooperative emission of a run of `len` copies of `c` ending just before
// slot[pos]; returns the new (lower) position.
__device__ __forceinline__ int emit_run(char* slot, int pos, int len, char c, int lane, int* err)
{
    if (len <= 0) return pos;
    if (len > pos) {
        if (lane == 0) atomicOr(err, ERR_CIGAR_OVERFLOW);
        len = pos;
    }
    for (int q = lane; q < len; q += 32) slot[pos - len + q] = c;
    return pos - len;
}

template <bool TRACE, int BITS>
__device__ void wfa_pair(const WfaArgs& A, int p, const uint64_t* __restrict__ P,
                         const uint64_t* __restrict__ T, int m, int n, int32_t* wf0, int32_t* wf1,
                         int32_t* stk, int lane)
{
    const int smax = A.smax;
    const int WS = 2 * smax + 3;
    const int base = smax + 1;                 // slot of diagonal 0
    for (int t = lane; t < WS; t += 32) { wf0[t] = WFA_NULL; wf1[t] = WFA_NULL; }
    const int off0 = match_run<BITS>(P, T, 0, 0, m, n);   // computed redundantly by every lane
    __syncwarp();
    if (lane == 0) {
        wf0[base] = off0;
        if (TRACE) stk[0] = off0;
    }
    const int kfinal = n - m;
    int score = -1;
    if (kfinal == 0 && off0 >= n) {
        score = 0;
    } else {
        int32_t* prev = wf0;
        int32_t* cur = wf1;
        for (int s = 1; s <= smax; ++s) {
            __syncwarp();
            for (int k = lane - s; k <= s; k += 32) {
                const int ins = prev[base + k - 1];
                const int del = prev[base + k + 1];
                const int mis = prev[base + k];
                int x = max(del, max(ins, mis) + 1);
                if (!wfa_live(x) || x > n || x - k > m) x = WFA_NULL;
                else x += match_run<BITS>(P, T, x - k, x, m, n);
                cur[base + k] = x;
                if (TRACE) stk[s * s + s + k] = x;
            }
            __syncwarp();
            if (kfinal >= -s && kfinal <= s) {
                const int fo = cur[base + kfinal];
                if (wfa_live(fo) && fo >= n) { score = s; break; }
            }
            int32_t* t = prev; prev = cur; cur = t;
        }
    }
    if (!TRACE || score < 0) {
        if (lane == 0) {
            A.out_score[p] = score;
            if (A.out_len) A.out_len[p] = 0;
        }
        return;
    }
    char* slot = A.out_cigar + A.D.out_off[p];
    int pos = m + n;
    if (score == 0) {
        pos = emit_run(slot, pos, n, 'M', lane, A.err);
    } else {
        __syncwarp();                      // stack writes of every lane are visible below
        int s = score, k = kfinal;
        int off = stk[s * s + s + k];
        int h = off, v = off - k;
        pos = emit_run(slot, pos, v - m, 'D', lane, A.err);
        pos = emit_run(slot, pos, h - n, 'I', lane, A.err);
        v = min(v, m);
        h = min(h, n);
        while (v > 0 && h > 0 && s > 0) {
            const int sp = s - 1;
            const int32_t* W = stk + sp * sp + sp;     // W[k] = offset of diagonal k at score sp
            const int c_mis = (k >= -sp && k <= sp) ? W[k] + 1 : WFA_NULL;
            const int c_ins = (k - 1 >= -sp && k - 1 <= sp) ? W[k - 1] + 1 : WFA_NULL;
            const int c_del = (k + 1 >= -sp && k + 1 <= sp) ? W[k + 1] : WFA_NULL;
            int best = WFA_NULL;
            char op = 0;
            if (wfa_live(c_mis) && c_mis >= best) { best = c_mis; op = 'X'; }
            if (wfa_live(c_ins) && c_ins > best)  { best = c_ins; op = 'I'; }
            if (wfa_live(c_del) && c_del > best)  { best = c_del; op = 'D'; }
            if (!op) break;
            pos = emit_run(slot, pos, off - best, 'M', lane, A.err);
            pos = emit_run(slot, pos, 1, op, lane, A.err);
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
            pos = emit_run(slot, pos, run, 'M', lane, A.err);
            v -= run;
            h -= run;
        }
        pos = emit_run(slot, pos, v, 'D', lane, A.err);
        pos = emit_run(slot, pos, h, 'I', lane, A.err);
    }
    if (lane == 0) {
        A.out_score[p] = score;
        A.out_len[p] = m + n - pos;
    }
}

template <bool TRACE>
__global__ void __launch_bounds__(128) wfa_kernel(WfaArgs A)
{
    extern __shared__ int32_t smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int WS = 2 * A.smax + 3;
    int32_t* wf0 = smem + wib * 2 * WS;
    int32_t* wf1 = wf0 + WS;
    const int64_t slot = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    int32_t* stk = TRACE ? A.stack + slot * A.stack_slot : nullptr;
    for (;;) {
        int p0 = 0;
        if (lane == 0) p0 = atomicAdd(A.counter, A.chunk);
        p0 = __shfl_sync(FULL, p0, 0);
        if (p0 >= A.D.n) break;
        const int pend = min(p0 + A.chunk, A.D.n);
        for (int p = p0; p < pend; ++p) {
        __syncwarp();
        const int m = A.D.a_len[p];       // pattern
        const int n = A.D.b_len[p];       // text
        if (m <= 0 || n <= 0) {
            // one side empty: the score is the other length, whatever smax is;
            // the CIGAR is all insertions (empty pattern) or all deletions
            // (wfa_kernel.hip:480-502)
            const int len = m <= 0 ? max(n, 0) : m;
            if (TRACE) emit_run(A.out_cigar + A.D.out_off[p], len, len, m <= 0 ? 'I' : 'D', lane, A.err);
            if (lane == 0) {
                A.out_score[p] = len;
                if (A.out_len) A.out_len[p] = TRACE ? len : 0;
            }
            continue;
        }
        const bool pure = A.D.pure[p] && A.D.pure[A.D.n + p];
        if (pure) {
            const uint64_t* P = A.D.packed + (A.D.a_off[p] >> 5);
            const uint64_t* T = A.D.packed + (A.D.b_off[p] >> 5);
            wfa_pair<TRACE, 2>(A, p, P, T, m, n, wf0, wf1, stk, lane);
        } else {
            const uint64_t* P = reinterpret_cast<const uint64_t*>(A.D.seq + A.D.a_off[p]);
            const uint64_t* T = reinterpret_cast<const uint64_t*>(A.D.seq + A.D.b_off[p]);
            wfa_pair<TRACE, 8>(A, p, P, T, m, n, wf0, wf1, stk, lane);
        }
        }
    }
}

// --------------------------------------------------------------- launchers --
cudaError_t launch_pack(const PairDesc& D, int64_t seq_bytes, uint64_t* packed, uint8_t* pure, cudaStream_t st)
{
    if (D.n <= 0) return cudaSuccess;
    int blocks = (2 * D.n + 255) / 256;
    blocks = std::min(blocks, device_sms() * 32);
    if (packed) {
        // every sequence ends >= 64 bytes before the arena's end, so the whole
        // chunks cover them all and no read passes seq_bytes
        const int64_t nchunks = seq_bytes / 32;
        uint32_t* bad = reinterpret_cast<uint32_t*>(packed + nchunks + 2);
        int64_t cblocks = (nchunks + 255) / 256;
        cblocks = std::min<int64_t>(cblocks, device_sms() * 32);
        launch_begin(K_PACK, st);
        pack_chunks_kernel<<<(int)cblocks, 256, 0, st>>>(D.seq, nchunks, packed, bad);
        launch_end(K_PACK, st);
        launch_begin(K_PACK, st);
        purity_mask_kernel<<<blocks, 256, 0, st>>>(D, bad, pure);
        launch_end(K_PACK, st);
        return cudaGetLastError();
    }
    launch_begin(K_PACK, st);
    purity_kernel<<<blocks, 256, 0, st>>>(D, pure);
    launch_end(K_PACK, st);
    return cudaGetLastError();
}

// The 2-bit words and non-ACGT masks of a whole byte arena (seq_bytes a
// multiple of 32, seq 16-byte aligned): packed[c], bad[c] for every chunk c.
cudaError_t launch_pack_arena(const uint8_t* seq, int64_t seq_bytes, uint64_t* packed, uint32_t* bad, cudaStream_t st)
{
    const int64_t nchunks = seq_bytes / 32;
    if (nchunks <= 0) return cudaSuccess;
    int64_t cblocks = (nchunks + 255) / 256;
    cblocks = std::min<int64_t>(cblocks, device_sms() * 32);
    launch_begin(K_PACK, st);
    pack_chunks_kernel<<<(int)cblocks, 256, 0, st>>>(seq, nchunks, packed, bad);
    launch_end(K_PACK, st);
    return cudaGetLastError();
}

// The result checks of the reference's validate (src/api/api.cpp:84-112), one
// warp per pair over its CIGAR (at the end of its slot), 32 ops at a time:
// each lane's op steps the pattern and/or the text, a warp prefix sum gives
// its position, and the lanes check their M / X bytes together (the ops and
// the bytes they compare are read contiguously).  Wellformed when the ops
// consume exactly the pattern and the text with M only on equal bytes and X
// only on unequal ones; rescore when the X, I and D ops number the score.
// flags[p] = rescore_ok | wellformed_ok << 1 for pairs with a CIGAR, 0 for
// the others.
__global__ void wfa_validate_kernel(PairDesc D, const int32_t* __restrict__ score, const int32_t* __restrict__ len,
                                    const char* __restrict__ cig, uint8_t* __restrict__ flags)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < D.n; p += nw) {
        const int s = score[p], L = len[p];
        if (s < 0 || L <= 0) {
            if (lane == 0) flags[p] = 0;
            continue;
        }
        const int m = D.a_len[p], n = D.b_len[p];
        const uint8_t* P = D.seq + D.a_off[p];
        const uint8_t* T = D.seq + D.b_off[p];
        const char* cg = cig + D.out_off[p] + (m + n) - L;
        int pi0 = 0, ti0 = 0, cost = 0;
        bool bad = false;
        for (int q0 = 0; q0 < L; q0 += 32) {
            const int q = q0 + lane;
            const char op = q < L ? cg[q] : 'I';
            const bool mx = op == 'M' || op == 'X';
            const int dp = (mx || op == 'D') && q < L, dt = (mx || op == 'I') && q < L;
            int v = dp << 16 | dt;                                 // inclusive prefix of both steps
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(FULL, v, o);
                if (lane >= o) v += y;
            }
            const int pi = pi0 + (v >> 16) - dp, ti = ti0 + (v & 0xffff) - dt;
            bool b = false;
            if (q < L) {
                if (mx) b = pi >= m || ti >= n || ((P[pi] == T[ti]) != (op == 'M'));
                else b = op != 'I' && op != 'D';
            }
            bad |= __any_sync(FULL, b);
            cost += __popc(__ballot_sync(FULL, q < L && (op == 'X' || op == 'I' || op == 'D')));
            const int tot = __shfl_sync(FULL, v, 31);
            pi0 += tot >> 16;
            ti0 += tot & 0xffff;
        }
        if (lane == 0) flags[p] = (uint8_t)((cost == s ? 1 : 0) | (!bad && pi0 == m && ti0 == n ? 2 : 0));
    }
}

// Every pair's CIGAR (the last len[p] bytes of its slot of a_len + b_len) packed
// for the copy back, 2 bits per op in op order (M 0, X 1, I 2, D 3; op t at
// bits 2 (t % 4) of byte t / 4), at byte pk_off[p] of pk.  One warp per pair,
// a lane per output byte: the slot is read and the packed bytes written
// contiguously.
__global__ void cigar_pack_kernel(PairDesc D, const int32_t* __restrict__ len, const char* __restrict__ cig,
                                  const int64_t* __restrict__ pk_off, uint8_t* __restrict__ pk)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < D.n; p += nw) {
        const int L = len[p];
        if (L <= 0) continue;
        const char* src = cig + D.out_off[p] + ((int64_t)D.a_len[p] + D.b_len[p]) - L;
        uint8_t* dst = pk + pk_off[p];
        for (int b = lane; 4 * b < L; b += 32) {
            uint32_t v = 0;
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                if (4 * b + t < L) {
                    const char c = src[4 * b + t];
                    v |= (uint32_t)(c == 'M' ? 0 : (c == 'X' ? 1 : (c == 'I' ? 2 : 3))) << (2 * t);
                }
            }
            dst[b] = (uint8_t)v;
        }
    }
}

// A warp per pair, each side's bytes copied 32 at a time (one sector read and
// written per step; the destination is 32-byte aligned).
__global__ void gather_sides_kernel(PairDesc D, uint8_t* __restrict__ seq, const uint8_t* __restrict__ span_a,
                                    const uint8_t* __restrict__ span_b, const int64_t* __restrict__ src_a,
                                    const int64_t* __restrict__ src_b)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < D.n; p += nw) {
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const int64_t src = side ? src_b[p] : src_a[p];
            if (src < 0) continue;
            const int len = side ? D.b_len[p] : D.a_len[p];
            const uint8_t* s = (side ? span_b : span_a) + src;
            uint8_t* d = seq + (side ? D.b_off[p] : D.a_off[p]);
            for (int k = lane; k < len; k += 32) d[k] = s[k];
        }
    }
}

cudaError_t launch_gather_sides(const PairDesc& D, uint8_t* seq, const uint8_t* span_a, const uint8_t* span_b,
                                const int64_t* src_a, const int64_t* src_b, cudaStream_t st)
{
    if (D.n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<int64_t>(((int64_t)D.n + 3) / 4, (int64_t)device_sms() * 16);   // a warp per pair
    launch_begin(K_PACK, st);
    gather_sides_kernel<<<blocks, 128, 0, st>>>(D, seq, span_a, span_b, src_a, src_b);
    launch_end(K_PACK, st);
    return cudaGetLastError();
}

cudaError_t launch_cigar_pack(const PairDesc& D, const int32_t* len, const char* cig, const int64_t* pk_off,
                              uint8_t* pk, cudaStream_t st)
{
    if (D.n <= 0) return cudaSuccess;
    int blocks = (D.n + 7) / 8;
    blocks = std::min(blocks, device_sms() * 16);
    launch_begin(K_VALIDATE, st);
    cigar_pack_kernel<<<blocks, 256, 0, st>>>(D, len, cig, pk_off, pk);
    launch_end(K_VALIDATE, st);
    return cudaGetLastError();
}

cudaError_t launch_wfa_validate(const PairDesc& D, const int32_t* score, const int32_t* len, const char* cig,
                                uint8_t* flags, cudaStream_t st)
{
    if (D.n <= 0) return cudaSuccess;
    const int blocks = (int)std::min<int64_t>(((int64_t)D.n + 3) / 4, (int64_t)device_sms() * 16);   // a warp per pair
    launch_begin(K_VALIDATE, st);
    wfa_validate_kernel<<<blocks, 128, 0, st>>>(D, score, len, cig, flags);
    launch_end(K_VALIDATE, st);
    return cudaGetLastError();
}

// 64-bit words of a packed arena for seq_bytes of sequence: the 2-bit words
// (+2 spare, read by two-word fetch windows) then one 32-bit mask per chunk.
int64_t packed_arena_words(int64_t seq_bytes)
{
    const int64_t nchunks = seq_bytes / 32;
    return nchunks + 2 + (nchunks + 1) / 2;
}

size_t wfa_smem_bytes(int smax) { return (size_t)4 * 2 * (2 * smax + 3) * sizeof(int32_t); }

int wfa_max_slots(int smax, bool trace, int sm_count)
{
    const size_t smem = wfa_smem_bytes(smax);
    const int per_sm = trace ? blocks_per_sm((const void*)wfa_kernel<true>, 128, smem)
                             : blocks_per_sm((const void*)wfa_kernel<false>, 128, smem);
    return per_sm * sm_count * 4;
}

cudaError_t launch_wfa(const WfaArgs& A, int slots, cudaStream_t st)
{
    if (A.D.n <= 0) return cudaSuccess;
    const int blocks = (slots + 3) / 4;
    const size_t smem = wfa_smem_bytes(A.smax);
    const int id = A.trace ? K_WFA_TRACE : K_WFA_SCORE;
    launch_begin(id, st);
    if (A.trace) wfa_kernel<true><<<blocks, 128, smem, st>>>(A);
    else         wfa_kernel<false><<<blocks, 128, smem, st>>>(A);
    launch_end(id, st);
    return cudaGetLastError();
}

}  // namespace ga
