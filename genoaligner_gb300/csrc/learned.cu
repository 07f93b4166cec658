// learned.cu -- the learned cost model: k-mer sketch, MLP forward/backward,
// Adam, all hand-written kernels.
//
// Features of one pair (66 floats): for each of the 64 DNA 3-mers, (count in
// a - count in b) / 8, then len(a) / 256 and len(b) / 256.  3-mers are taken
// on the 2-bit codes ((c >> 1) ^ (c >> 2)) & 3 of the raw bytes, so A/C/G/T
// map to 0..3 and any other byte aliases onto one of them.
//
// The sketch also yields an exact lower bound on the edit distance: an edit
// changes at most 3 3-mers of each string, so d >= L1(count difference) / 6,
// and d >= |len(a) - len(b)|.  Aliasing only merges characters, which can only
// lower the distance of the aliased strings, so the bound holds for the
// original strings.  A pair whose bound exceeds the batch smax is unresolved
// without running WFA -- the same answer the full search gives.
//
// MLP: 66 -> 128 (ReLU) -> 128 (ReLU) -> 2, weights stored as bf16 and
// computed in fp32 (fp32 master copy for Adam).  Outputs: log2(d + 1) and
// log2(wavefront cells + 1) with wavefront cells = (d + 1)^2.  It is a tiny
// GEMM (25k multiply-adds per pair), run as shared-memory-tiled FMA: 64 pairs
// per block, 256 threads, every thread 32 outputs of one pair.
#include <mutex>
#include <vector>

#include "../../include/genoaligner_gb300.h"
#include "kernels.cuh"
#include "route.cuh"
#include <cuda_bf16.h>

namespace ga {

constexpr int NF = 66, NH1 = 128, NH2 = 128, NO = 2;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH1 * NF, OFF_W2 = OFF_B1 + NH1, OFF_B2 = OFF_W2 + NH2 * NH1,
              OFF_W3 = OFF_B2 + NH2, OFF_B3 = OFF_W3 + NO * NH2, NPARAM = OFF_B3 + NO;
constexpr int TILE = 64;

void prepare_mlp();
const __nv_bfloat16* cost_model_weights();

// ------------------------------------------------------------------ sketch --
// One warp per pair: 3-mer histograms of both sides in shared memory.
__global__ void __launch_bounds__(256) sketch_kernel(PairDesc D, float* __restrict__ feat,
                                                     int32_t* __restrict__ lower_bound, float s_diff, float s_len)
{
    __shared__ int hist[8][64];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < D.n; p += nwarps) {
        hist[wib][lane] = 0;
        hist[wib][lane + 32] = 0;
        __syncwarp();
        for (int side = 0; side < 2; ++side) {
            const uint8_t* s = D.seq + (side ? D.b_off[p] : D.a_off[p]);
            const int L = side ? D.b_len[p] : D.a_len[p];
            const int sign = side ? -1 : 1;
            for (int q = lane; q + 2 < L; q += 32) {
                const uint32_t c0 = __ldg(s + q), c1 = __ldg(s + q + 1), c2 = __ldg(s + q + 2);
                const int k = (int)((((c0 >> 1) ^ (c0 >> 2)) & 3u) * 16 + (((c1 >> 1) ^ (c1 >> 2)) & 3u) * 4 +
                                    (((c2 >> 1) ^ (c2 >> 2)) & 3u));
                atomicAdd(&hist[wib][k], sign);
            }
        }
        __syncwarp();
        const int d0 = hist[wib][lane], d1 = hist[wib][lane + 32];
        feat[(int64_t)p * NF + lane] = d0 * s_diff;
        feat[(int64_t)p * NF + lane + 32] = d1 * s_diff;
        int l1 = abs(d0) + abs(d1);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) l1 += __shfl_xor_sync(FULL, l1, o);
        if (lane == 0) {
            const int m = D.a_len[p], n = D.b_len[p];
            feat[(int64_t)p * NF + 64] = m * s_len;
            feat[(int64_t)p * NF + 65] = n * s_len;
            if (lower_bound) lower_bound[p] = max(abs(m - n), (l1 + 5) / 6);
        }
        __syncwarp();
    }
}

// The same sketch from the 2-bit arena (D.packed).  Lanes 0-15 take side a,
// lanes 16-31 side b; a lane counts the 16 3-mers starting in its 16-base
// stretch from one 64-bit window (3-mer i is bits [2i, 2i+6) of the window).
// The histogram is indexed by the window's own order, c0 + 4 c1 + 16 c2; the
// feature order 16 c0 + 4 c1 + c2 is applied when the features are written.
__global__ void __launch_bounds__(256) sketch_packed_kernel(PairDesc D, float* __restrict__ feat,
                                                            int32_t* __restrict__ lower_bound, float s_diff,
                                                            float s_len)
{
    __shared__ int hist[8][64];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int side = lane >> 4, sl = lane & 15;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < D.n; p += nwarps) {
        hist[wib][lane] = 0;
        hist[wib][lane + 32] = 0;
        __syncwarp();
        const uint64_t* P = D.packed + ((side ? D.b_off[p] : D.a_off[p]) >> 5);
        const int L = side ? D.b_len[p] : D.a_len[p];
        const int sign = side ? -1 : 1;
        for (int q = 16 * sl; q + 2 < L; q += 256) {
            const uint64_t v = fetch_syms<2>(P, q);
            const int cnt = min(16, L - 2 - q);
#pragma unroll
            for (int i = 0; i < 16; ++i)
                if (i < cnt) atomicAdd(&hist[wib][(int)((v >> (2 * i)) & 63u)], sign);
        }
        __syncwarp();
        // feature k = 16 c0 + 4 c1 + c2 lives in bin c0 + 4 c1 + 16 c2
        const int k0 = lane, k1 = lane + 32;
        const int d0 = hist[wib][((k0 & 3) << 4) | (k0 & 12) | (k0 >> 4)];
        const int d1 = hist[wib][((k1 & 3) << 4) | (k1 & 12) | (k1 >> 4)];
        feat[(int64_t)p * NF + k0] = d0 * s_diff;
        feat[(int64_t)p * NF + k1] = d1 * s_diff;
        int l1 = abs(d0) + abs(d1);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) l1 += __shfl_xor_sync(FULL, l1, o);
        if (lane == 0) {
            const int m = D.a_len[p], n = D.b_len[p];
            feat[(int64_t)p * NF + 64] = m * s_len;
            feat[(int64_t)p * NF + 65] = n * s_len;
            if (lower_bound) lower_bound[p] = max(abs(m - n), (l1 + 5) / 6);
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------- MLP --
struct MlpParams {
    const __nv_bfloat16* w;   // NPARAM bf16 (weights and biases)
};

// Shared-memory image of one tile's layers.
struct MlpSmem {
    float W[NH2 * NH1];        // the current layer's weights, transposed [in][out]
    float X[TILE * (NF + 2)];
    float H1[TILE * (NH1 + 1)];
    float H2[TILE * (NH2 + 1)];
};

// out[r][o] = act(sum_i in[r][i] * W[o][i] + b[o]) for the tile's rows; W is
// staged transposed in smem with outputs interleaved by 4 (o = 4k + oq) so the
// four output groups of a warp read four different banks.
template <int IN, int OUT, bool RELU>
__device__ __forceinline__ void dense(const __nv_bfloat16* __restrict__ w, const __nv_bfloat16* __restrict__ b,
                                      float* Ws, const float* in, int in_stride, float* out, int out_stride,
                                      int rows)
{
    __syncthreads();
    for (int idx = threadIdx.x; idx < IN * OUT; idx += blockDim.x) {
        const int o = idx / IN, i = idx - o * IN;
        Ws[i * OUT + o] = __bfloat162float(w[idx]);
    }
    __syncthreads();
    constexpr int PER = OUT / 4;                  // outputs per thread (4 threads per row)
    const int r = threadIdx.x >> 2, oq = threadIdx.x & 3;
    if (r < rows) {
        float acc[PER];
#pragma unroll
        for (int k = 0; k < PER; ++k) acc[k] = __bfloat162float(b[4 * k + oq]);
        for (int i = 0; i < IN; ++i) {
            const float x = in[r * in_stride + i];
            const float* wr = Ws + i * OUT;
#pragma unroll
            for (int k = 0; k < PER; ++k) acc[k] = fmaf(x, wr[4 * k + oq], acc[k]);
        }
#pragma unroll
        for (int k = 0; k < PER; ++k) out[r * out_stride + 4 * k + oq] = RELU ? fmaxf(acc[k], 0.f) : acc[k];
    }
}

// The output layer (2 outputs) by one thread per row.
__device__ __forceinline__ void dense_out(const __nv_bfloat16* __restrict__ w, const float* H2, float* y, int rows)
{
    const int r = threadIdx.x;
    if (r < rows) {
        float a0 = __bfloat162float(w[OFF_B3]), a1 = __bfloat162float(w[OFF_B3 + 1]);
        for (int i = 0; i < NH2; ++i) {
            const float h = H2[r * (NH2 + 1) + i];
            a0 = fmaf(h, __bfloat162float(w[OFF_W3 + i]), a0);
            a1 = fmaf(h, __bfloat162float(w[OFF_W3 + NH2 + i]), a1);
        }
        y[2 * r] = a0;
        y[2 * r + 1] = a1;
    }
}

__device__ __forceinline__ void forward_tile(const __nv_bfloat16* w, const float* __restrict__ feat, int64_t base,
                                             int rows, MlpSmem& S, float* ytile)
{
    for (int idx = threadIdx.x; idx < rows * NF; idx += blockDim.x) {
        const int r = idx / NF, i = idx - r * NF;
        S.X[r * (NF + 2) + i] = feat[(base + r) * NF + i];
    }
    dense<NF, NH1, true>(w + OFF_W1, w + OFF_B1, S.W, S.X, NF + 2, S.H1, NH1 + 1, rows);
    dense<NH1, NH2, true>(w + OFF_W2, w + OFF_B2, S.W, S.H1, NH1 + 1, S.H2, NH2 + 1, rows);
    __syncthreads();
    dense_out(w, S.H2, ytile, rows);
    __syncthreads();
}

__global__ void __launch_bounds__(256) mlp_forward_kernel(const __nv_bfloat16* __restrict__ w,
                                                          const float* __restrict__ feat, int n, float* __restrict__ y)
{
    extern __shared__ float mlp_smem[];
    MlpSmem& S = *reinterpret_cast<MlpSmem*>(mlp_smem);
    __shared__ float ytile[2 * TILE];
    for (int64_t base = (int64_t)blockIdx.x * TILE; base < n; base += (int64_t)gridDim.x * TILE) {
        const int rows = (n - base < TILE) ? (int)(n - base) : TILE;
        forward_tile(w, feat, base, rows, S, ytile);
        for (int idx = threadIdx.x; idx < 2 * rows; idx += blockDim.x) y[2 * base + idx] = ytile[idx];
        __syncthreads();
    }
}

// Forward + backward of the mean squared error over the batch; gradients of
// every parameter (with respect to the bf16-rounded weights) accumulate into
// grad (fp32) and the summed squared error into loss.
__global__ void __launch_bounds__(256) mlp_backward_kernel(const __nv_bfloat16* __restrict__ w,
                                                           const float* __restrict__ feat,
                                                           const float* __restrict__ target, int n,
                                                           float inv_batch, float* __restrict__ grad,
                                                           float* __restrict__ loss)
{
    extern __shared__ float mlp_smem[];
    MlpSmem& S = *reinterpret_cast<MlpSmem*>(mlp_smem);
    __shared__ float ytile[2 * TILE];
    __shared__ float dy[2 * TILE];
    for (int64_t base = (int64_t)blockIdx.x * TILE; base < n; base += (int64_t)gridDim.x * TILE) {
        const int rows = (n - base < TILE) ? (int)(n - base) : TILE;
        forward_tile(w, feat, base, rows, S, ytile);
        // dL/dy = 2 (y - t) / B
        float lsum = 0.f;
        for (int idx = threadIdx.x; idx < 2 * TILE; idx += blockDim.x) {
            float g = 0.f;
            if (idx < 2 * rows) {
                const float e = ytile[idx] - target[2 * base + idx];
                lsum += e * e;
                g = 2.f * e * inv_batch;
            }
            dy[idx] = g;
        }
        for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(FULL, lsum, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(loss, lsum);
        __syncthreads();
        // output layer: dW3, db3; dH2 = dy W3 * relu'(H2) (H2 overwritten in place)
        for (int idx = threadIdx.x; idx < NO * NH2; idx += blockDim.x) {
            const int o = idx / NH2, i = idx - o * NH2;
            float g = 0.f;
            for (int r = 0; r < rows; ++r) g = fmaf(dy[2 * r + o], S.H2[r * (NH2 + 1) + i], g);
            atomicAdd(&grad[OFF_W3 + idx], g);
        }
        if (threadIdx.x < NO) {
            float g = 0.f;
            for (int r = 0; r < rows; ++r) g += dy[2 * r + threadIdx.x];
            atomicAdd(&grad[OFF_B3 + threadIdx.x], g);
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < rows * NH2; idx += blockDim.x) {
            const int r = idx / NH2, i = idx - r * NH2;
            float* h = &S.H2[r * (NH2 + 1) + i];
            const float g = dy[2 * r] * __bfloat162float(w[OFF_W3 + i]) + dy[2 * r + 1] * __bfloat162float(w[OFF_W3 + NH2 + i]);
            *h = (*h > 0.f) ? g : 0.f;
        }
        __syncthreads();
        // layer 2: dW2[o][i] = sum_r dH2[r][o] H1[r][i]; db2; dH1 = dH2 W2 * relu'(H1)
        for (int idx = threadIdx.x; idx < NH2 * NH1; idx += blockDim.x) {
            const int o = idx / NH1, i = idx - o * NH1;
            float g = 0.f;
            for (int r = 0; r < rows; ++r) g = fmaf(S.H2[r * (NH2 + 1) + o], S.H1[r * (NH1 + 1) + i], g);
            atomicAdd(&grad[OFF_W2 + idx], g);
        }
        for (int o = threadIdx.x; o < NH2; o += blockDim.x) {
            float g = 0.f;
            for (int r = 0; r < rows; ++r) g += S.H2[r * (NH2 + 1) + o];
            atomicAdd(&grad[OFF_B2 + o], g);
        }
        // W2 (not transposed) into S.W: W[o][i]
        for (int idx = threadIdx.x; idx < NH2 * NH1; idx += blockDim.x) S.W[idx] = __bfloat162float(w[OFF_W2 + idx]);
        __syncthreads();
        for (int idx = threadIdx.x; idx < rows * NH1; idx += blockDim.x) {
            const int r = idx / NH1, i = idx - r * NH1;
            float g = 0.f;
            for (int o = 0; o < NH2; ++o) g = fmaf(S.H2[r * (NH2 + 1) + o], S.W[o * NH1 + i], g);
            // each thread reads and overwrites only its own H1 entry: dH1 in place
            const float h = S.H1[r * (NH1 + 1) + i];
            S.H1[r * (NH1 + 1) + i] = (h > 0.f) ? g : 0.f;
        }
        __syncthreads();
        // layer 1: dW1[o][i] = sum_r dH1[r][o] X[r][i]; db1
        for (int idx = threadIdx.x; idx < NH1 * NF; idx += blockDim.x) {
            const int o = idx / NF, i = idx - o * NF;
            float g = 0.f;
            for (int r = 0; r < rows; ++r) g = fmaf(S.H1[r * (NH1 + 1) + o], S.X[r * (NF + 2) + i], g);
            atomicAdd(&grad[OFF_W1 + idx], g);
        }
        for (int o = threadIdx.x; o < NH1; o += blockDim.x) {
            float g = 0.f;
            for (int r = 0; r < rows; ++r) g += S.H1[r * (NH1 + 1) + o];
            atomicAdd(&grad[OFF_B1 + o], g);
        }
        __syncthreads();
    }
}

// Adam on the fp32 master copy, then the bf16 copy the forward pass reads.
__global__ void adam_kernel(float* __restrict__ master, __nv_bfloat16* __restrict__ w, const float* __restrict__ grad,
                            float* __restrict__ m1, float* __restrict__ m2, int n, float lr, float b1, float b2,
                            float eps, float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float g = grad[i];
        const float a = b1 * m1[i] + (1.f - b1) * g;
        const float v = b2 * m2[i] + (1.f - b2) * g * g;
        m1[i] = a;
        m2[i] = v;
        const float p = master[i] - lr * (a * c1) / (sqrtf(v * c2) + eps);
        master[i] = p;
        w[i] = __float2bfloat16(p);
    }
}

__global__ void to_bf16_kernel(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = __float2bfloat16(src[i]);
}

// ------------------------------------------------- tensor-core inference --
// The routing forward pass on the tensor cores: mma.sync m16n8k16 bf16 with
// fp32 accumulation, one warp per 16 pairs; the inputs and each hidden layer
// are rounded to bf16 as they enter a multiply.  Layer outputs go from the
// accumulator registers straight into the next layer's A fragments (the m16n8
// accumulator layout of two adjacent n-tiles is the A layout of one k16 step).
// Weights are staged once per block in shared memory, rows padded (88 and 136
// bf16) so the eight row groups of a fragment load hit eight bank groups.
constexpr int TK1 = 80, TS1 = 88, TS2 = 136;

struct TcSmem {
    __nv_bfloat16 W1[NH1 * TS1];
    __nv_bfloat16 W2[NH2 * TS2];
    __nv_bfloat16 W3[8 * TS2];
    float b1[NH1], b2[NH2], b3[8];
};

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// Weights and biases of a bf16 model into a block's shared memory.
__device__ void load_tc_weights(TcSmem& S, const __nv_bfloat16* __restrict__ w)
{
    for (int idx = threadIdx.x; idx < NH1 * TS1; idx += blockDim.x) {
        const int o = idx / TS1, i = idx - o * TS1;
        S.W1[idx] = i < NF ? w[OFF_W1 + o * NF + i] : __float2bfloat16(0.f);
    }
    for (int idx = threadIdx.x; idx < NH2 * TS2; idx += blockDim.x) {
        const int o = idx / TS2, i = idx - o * TS2;
        S.W2[idx] = i < NH1 ? w[OFF_W2 + o * NH1 + i] : __float2bfloat16(0.f);
    }
    for (int idx = threadIdx.x; idx < 8 * TS2; idx += blockDim.x) {
        const int o = idx / TS2, i = idx - o * TS2;
        S.W3[idx] = (o < NO && i < NH2) ? w[OFF_W3 + o * NH2 + i] : __float2bfloat16(0.f);
    }
    for (int i = threadIdx.x; i < NH1; i += blockDim.x) S.b1[i] = __bfloat162float(w[OFF_B1 + i]);
    for (int i = threadIdx.x; i < NH2; i += blockDim.x) S.b2[i] = __bfloat162float(w[OFF_B2 + i]);
    if (threadIdx.x < 8) S.b3[threadIdx.x] = threadIdx.x < NO ? __bfloat162float(w[OFF_B3 + threadIdx.x]) : 0.f;
}

// One 16-pair tile through the network.  a: the input A fragments (rows g
// and g + 8 of the tile, columns 16 kt + 2 tg (+1, +8, +9)); o: outputs of
// rows g (o[0], o[1]) and g + 8 (o[2], o[3]), valid in lanes with tg == 0.
__device__ __forceinline__ void tc_tile_forward(const TcSmem& S, const uint32_t (&a)[TK1 / 16][4], float (&o)[4])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, tg = lane & 3;
    float c[16][4];
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
        const float b0 = S.b1[8 * nt + 2 * tg], bb1 = S.b1[8 * nt + 2 * tg + 1];
        c[nt][0] = b0; c[nt][1] = bb1; c[nt][2] = b0; c[nt][3] = bb1;
        const __nv_bfloat16* wr = S.W1 + (8 * nt + g) * TS1 + 2 * tg;
#pragma unroll
        for (int kt = 0; kt < TK1 / 16; ++kt)
            mma_bf16(c[nt], a[kt], *reinterpret_cast<const uint32_t*>(wr + 16 * kt),
                     *reinterpret_cast<const uint32_t*>(wr + 16 * kt + 8));
    }
    uint32_t h[8][4];
#pragma unroll
    for (int kt = 0; kt < 8; ++kt) {
        h[kt][0] = pack_bf16(fmaxf(c[2 * kt][0], 0.f), fmaxf(c[2 * kt][1], 0.f));
        h[kt][1] = pack_bf16(fmaxf(c[2 * kt][2], 0.f), fmaxf(c[2 * kt][3], 0.f));
        h[kt][2] = pack_bf16(fmaxf(c[2 * kt + 1][0], 0.f), fmaxf(c[2 * kt + 1][1], 0.f));
        h[kt][3] = pack_bf16(fmaxf(c[2 * kt + 1][2], 0.f), fmaxf(c[2 * kt + 1][3], 0.f));
    }
#pragma unroll
    for (int nt = 0; nt < 16; ++nt) {
        const float b0 = S.b2[8 * nt + 2 * tg], bb1 = S.b2[8 * nt + 2 * tg + 1];
        c[nt][0] = b0; c[nt][1] = bb1; c[nt][2] = b0; c[nt][3] = bb1;
        const __nv_bfloat16* wr = S.W2 + (8 * nt + g) * TS2 + 2 * tg;
#pragma unroll
        for (int kt = 0; kt < 8; ++kt)
            mma_bf16(c[nt], h[kt], *reinterpret_cast<const uint32_t*>(wr + 16 * kt),
                     *reinterpret_cast<const uint32_t*>(wr + 16 * kt + 8));
    }
#pragma unroll
    for (int kt = 0; kt < 8; ++kt) {
        h[kt][0] = pack_bf16(fmaxf(c[2 * kt][0], 0.f), fmaxf(c[2 * kt][1], 0.f));
        h[kt][1] = pack_bf16(fmaxf(c[2 * kt][2], 0.f), fmaxf(c[2 * kt][3], 0.f));
        h[kt][2] = pack_bf16(fmaxf(c[2 * kt + 1][0], 0.f), fmaxf(c[2 * kt + 1][1], 0.f));
        h[kt][3] = pack_bf16(fmaxf(c[2 * kt + 1][2], 0.f), fmaxf(c[2 * kt + 1][3], 0.f));
    }
    o[0] = S.b3[2 * tg]; o[1] = S.b3[2 * tg + 1]; o[2] = S.b3[2 * tg]; o[3] = S.b3[2 * tg + 1];
    const __nv_bfloat16* wr = S.W3 + g * TS2 + 2 * tg;
#pragma unroll
    for (int kt = 0; kt < 8; ++kt)
        mma_bf16(o, h[kt], *reinterpret_cast<const uint32_t*>(wr + 16 * kt),
                 *reinterpret_cast<const uint32_t*>(wr + 16 * kt + 8));
}

__global__ void __launch_bounds__(256) mlp_forward_tc_kernel(const __nv_bfloat16* __restrict__ w,
                                                             const float* __restrict__ feat, int n,
                                                             float* __restrict__ y)
{
    extern __shared__ __align__(16) unsigned char tc_raw[];
    TcSmem& S = *reinterpret_cast<TcSmem*>(tc_raw);
    load_tc_weights(S, w);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, tg = lane & 3;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; tile * 16 < n; tile += warps) {
        const int r0 = tile * 16 + g, r1 = r0 + 8;
        auto X = [&](int r, int c) -> float { return (r < n && c < NF) ? __ldg(feat + (int64_t)r * NF + c) : 0.f; };
        uint32_t a[TK1 / 16][4];
#pragma unroll
        for (int kt = 0; kt < TK1 / 16; ++kt) {
            const int c0 = 16 * kt + 2 * tg, c1 = c0 + 8;
            a[kt][0] = pack_bf16(X(r0, c0), X(r0, c0 + 1));
            a[kt][1] = pack_bf16(X(r1, c0), X(r1, c0 + 1));
            a[kt][2] = pack_bf16(X(r0, c1), X(r0, c1 + 1));
            a[kt][3] = pack_bf16(X(r1, c1), X(r1, c1 + 1));
        }
        float o[4];
        tc_tile_forward(S, a, o);
        if (tg == 0) {
            if (r0 < n) { y[2 * (int64_t)r0] = o[0]; y[2 * (int64_t)r0 + 1] = o[1]; }
            if (r1 < n) { y[2 * (int64_t)r1] = o[2]; y[2 * (int64_t)r1 + 1] = o[3]; }
        }
    }
}

// ------------------------------------------ fused routing inference --
// Sketch, lower bound, tensor-core forward pass and queue choice of every pair
// of a WFA batch in one pass, one warp per 16 pairs: lane l < 16 counts the
// 3-mers of side a of pair l of the tile, lane l + 16 those of side b, into a
// private histogram column hist[bin][lane] (bin = c0 + 4 c1 + 16 c2, the 2-bit
// window's own order); the A fragments read feature k = 16 c0 + 4 c1 + c2 as
// hist[bin][r] - hist[bin][r + 16].  Features, bf16 rounding and the network
// are those of ga_wfa_features + ga_mlp_forward_fast, so the prediction is the
// same; nothing but the queue item (route.cuh) leaves the kernel.  MODEL =
// false is the same pass without the network: the queue item comes from the
// exact lower bound alone (the prediction replaced by log2(bound + 1)), for
// measuring what the network adds.
constexpr int RM_WARPS = 16;

template <bool MODEL>
__global__ void __launch_bounds__(512) route_model_kernel(const __nv_bfloat16* __restrict__ w, PairDesc D, int smax,
                                                          int lane_smax,
                                                          int32_t* __restrict__ item, int32_t* __restrict__ lb_out,
                                                          float* __restrict__ y_out, int32_t* __restrict__ counts,
                                                          int32_t* __restrict__ out_score, int32_t* __restrict__ out_len)
{
    extern __shared__ __align__(16) unsigned char rm_raw[];
    TcSmem& S = *reinterpret_cast<TcSmem*>(rm_raw);
    int* hist_all = reinterpret_cast<int*>(rm_raw + sizeof(TcSmem));
    __shared__ int local[2 * ROUTE_BUCKETS];
    if (MODEL) load_tc_weights(S, w);
    if (threadIdx.x < 2 * ROUTE_BUCKETS) local[threadIdx.x] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, g = lane >> 2, tg = lane & 3;
    const int side = lane >> 4, sl = lane & 15;
    int* H = hist_all + wib * 64 * 32 + lane;                 // H[bin * 32]: this lane's column
    const int* Hw = hist_all + wib * 64 * 32;
    const int n = D.n;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; tile * 16 < n; tile += warps) {
#pragma unroll 8
        for (int b = 0; b < 64; ++b) H[b * 32] = 0;
        const int p = tile * 16 + sl;
        int m = 0, nn = 0;
        if (p < n) {
            m = D.a_len[p];
            nn = D.b_len[p];
            const uint64_t* P = D.packed + ((side ? D.b_off[p] : D.a_off[p]) >> 5);
            const int L = side ? nn : m;
            // 256 symbols at a time: the 8 words that hold them and the next
            // one (3-mers straddle it) are loaded together, then counted
            for (int q0 = 0; q0 + 2 < L; q0 += 256) {
                uint64_t wd[9];
                const int wlast = ((L - 1) >> 5) - (q0 >> 5) + 1;     // words past this lie beyond the arena's spare
#pragma unroll
                for (int j = 0; j < 9; ++j) wd[j] = j <= wlast ? __ldg(P + (q0 >> 5) + j) : 0ull;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int q = q0 + 16 * j;
                    if (q + 2 >= L) break;
                    const uint64_t v = (j & 1) ? ((wd[j >> 1] >> 32) | (wd[(j >> 1) + 1] << 32)) : wd[j >> 1];
                    const int cnt = min(16, L - 2 - q);
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        if (i < cnt) ++H[(int)((v >> (2 * i)) & 63u) * 32];   // the lane's own column: no atomic
                }
            }
        }
        __syncwarp();
        // exact lower bound: lanes l and l + 16 each sum half the bins of pair l
        int l1 = 0;
#pragma unroll 8
        for (int b = side * 32; b < side * 32 + 32; ++b) l1 += abs(Hw[b * 32 + sl] - Hw[b * 32 + sl + 16]);
        l1 += __shfl_xor_sync(FULL, l1, 16);
        const int lb = max(abs(m - nn), (l1 + 5) / 6);
        // A fragments
        const int r0 = g, r1 = g + 8;
        const int m0 = __shfl_sync(FULL, m, r0), n0 = __shfl_sync(FULL, nn, r0);
        const int m1 = __shfl_sync(FULL, m, r1), n1 = __shfl_sync(FULL, nn, r1);
        auto X = [&](int r, int c, int mr, int nr) -> float {
            if (c < 64) {
                const int bin = ((c & 3) << 4) | (c & 12) | (c >> 4);
                return (float)(Hw[bin * 32 + r] - Hw[bin * 32 + r + 16]) * 0.125f;
            }
            if (c == 64) return mr * (1.0f / 256.0f);
            if (c == 65) return nr * (1.0f / 256.0f);
            return 0.f;
        };
        float o[4];
        const int lb0 = __shfl_sync(FULL, lb, r0), lb1 = __shfl_sync(FULL, lb, r1);
        if constexpr (MODEL) {
            uint32_t a[TK1 / 16][4];
#pragma unroll
            for (int kt = 0; kt < TK1 / 16; ++kt) {
                const int c0 = 16 * kt + 2 * tg, c1 = c0 + 8;
                a[kt][0] = pack_bf16(X(r0, c0, m0, n0), X(r0, c0 + 1, m0, n0));
                a[kt][1] = pack_bf16(X(r1, c0, m1, n1), X(r1, c0 + 1, m1, n1));
                a[kt][2] = pack_bf16(X(r0, c1, m0, n0), X(r0, c1 + 1, m0, n0));
                a[kt][3] = pack_bf16(X(r1, c1, m1, n1), X(r1, c1 + 1, m1, n1));
            }
            tc_tile_forward(S, a, o);
        } else {
            (void)X;
            o[0] = o[1] = log2f((float)lb0 + 1.f);
            o[2] = o[3] = log2f((float)lb1 + 1.f);
        }
        if (tg == 0) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = h ? r1 : r0;
                const int pr = tile * 16 + r;
                if (pr >= n) continue;
                const int mr = h ? m1 : m0, nr = h ? n1 : n0, lbr = h ? lb1 : lb0;
                const float y0 = h ? o[2] : o[0];
                const int it = route_item(mr, nr, D.pure[pr] != 0, D.pure[n + pr] != 0, lbr, y0, smax, lane_smax);
                item[pr] = it;
                if (lb_out) lb_out[pr] = lbr;
                if (y_out) { y_out[2 * (int64_t)pr] = y0; y_out[2 * (int64_t)pr + 1] = h ? o[3] : o[1]; }
                if (it < 0) {
                    out_score[pr] = -1;
                    if (out_len) out_len[pr] = 0;
                } else {
                    atomicAdd(&local[it & 0xff], 1);
                }
            }
        }
        __syncwarp();
    }
    __syncthreads();
    if (threadIdx.x < 2 * ROUTE_BUCKETS && local[threadIdx.x]) atomicAdd(&counts[threadIdx.x], local[threadIdx.x]);
}

static size_t route_model_smem() { return sizeof(TcSmem) + (size_t)RM_WARPS * 64 * 32 * sizeof(int); }

// The fused routing pass over a WFA batch (D.packed and D.pure set): per pair
// the queue item, lower bound and prediction; bucket totals into counts.
// model = false: the queue items from the lower bound alone.
cudaError_t launch_route_model(const PairDesc& D, int smax, int lane_smax, bool model, int32_t* item, int32_t* lb,
                               float* y, int32_t* counts, int32_t* out_score, int32_t* out_len, cudaStream_t st)
{
    const __nv_bfloat16* w = cost_model_weights();
    if (model && !w) return cudaErrorNotReady;
    if (D.n <= 0) return cudaSuccess;
    int blocks = (D.n + 16 * RM_WARPS - 1) / (16 * RM_WARPS);
    blocks = std::min(blocks, device_sms());
    launch_begin(K_MLP, st);
    if (model)
        route_model_kernel<true><<<blocks, 32 * RM_WARPS, route_model_smem(), st>>>(w, D, smax, lane_smax, item, lb, y,
                                                                                    counts, out_score, out_len);
    else
        route_model_kernel<false><<<blocks, 32 * RM_WARPS, route_model_smem(), st>>>(w, D, smax, lane_smax, item, lb,
                                                                                     y, counts, out_score, out_len);
    launch_end(K_MLP, st);
    return cudaGetLastError();
}

static cudaError_t run_forward_tc(const __nv_bfloat16* w, const float* feat, int n, float* y, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    prepare_mlp();
    int blocks = (n + 127) / 128;
    blocks = std::min(blocks, device_sms() * 2);
    launch_begin(K_MLP, st);
    mlp_forward_tc_kernel<<<blocks, 256, sizeof(TcSmem), st>>>(w, feat, n, y);
    launch_end(K_MLP, st);
    return cudaGetLastError();
}

// --------------------------------------------------------- model state --
// One model per device: fp32 master, bf16 working copy, Adam moments, grads.
struct Model {
    float* master = nullptr;
    __nv_bfloat16* w = nullptr;
    float *m1 = nullptr, *m2 = nullptr, *grad = nullptr, *loss = nullptr;
    int step = 0;
    bool ready = false;
};
// Two models per device, the same network: slot 0 the WFA cost model (edit
// distance and wavefront work), slot 1 the Smith-Waterman variant model (best
// score as a fraction of the all-match score).  The C API's set / get /
// forward / gradient / train calls act on the calling thread's selected slot
// (ga_model_select); each routing pass reads its own slot.
constexpr int N_MODEL_SLOTS = 2;
static std::mutex g_model_mu;
static Model g_models[16][N_MODEL_SLOTS];
static thread_local int t_model_slot = 0;

static Model* model_for(int slot, bool create)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16) { cudaGetLastError(); return nullptr; }
    Model& M = g_models[dev][slot];
    if (!M.master && create) {
        if (cudaMalloc(&M.master, NPARAM * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&M.w, NPARAM * sizeof(__nv_bfloat16)) != cudaSuccess ||
            cudaMalloc(&M.m1, NPARAM * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&M.m2, NPARAM * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&M.grad, NPARAM * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&M.loss, sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
    }
    return M.master ? &M : nullptr;
}

static size_t mlp_smem_bytes() { return sizeof(MlpSmem); }

// Kernel attributes are set outside any stream capture (prepare_mlp is called
// while planning a batch).
void prepare_mlp()
{
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_smem_bytes());
        cudaFuncSetAttribute(mlp_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_smem_bytes());
        cudaFuncSetAttribute(mlp_forward_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TcSmem));
        cudaFuncSetAttribute(route_model_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)route_model_smem());
        cudaFuncSetAttribute(route_model_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)route_model_smem());
    });
}

static cudaError_t run_forward(const __nv_bfloat16* w, const float* feat, int n, float* y, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    prepare_mlp();
    int blocks = (n + TILE - 1) / TILE;
    blocks = std::min(blocks, device_sms() * 2);
    launch_begin(K_MLP, st);
    mlp_forward_kernel<<<blocks, 256, mlp_smem_bytes(), st>>>(w, feat, n, y);
    launch_end(K_MLP, st);
    return cudaGetLastError();
}

static cudaError_t run_backward(const __nv_bfloat16* w, const float* feat, const float* target, int n, float* grad,
                                float* loss, cudaStream_t st)
{
    prepare_mlp();
    cudaMemsetAsync(grad, 0, NPARAM * sizeof(float), st);
    cudaMemsetAsync(loss, 0, sizeof(float), st);
    int blocks = (n + TILE - 1) / TILE;
    blocks = std::min(blocks, device_sms() * 2);
    launch_begin(K_MLP, st);
    mlp_backward_kernel<<<blocks, 256, mlp_smem_bytes(), st>>>(w, feat, target, n, 1.0f / (float)n, grad, loss);
    launch_end(K_MLP, st);
    return cudaGetLastError();
}

cudaError_t launch_sketch(const PairDesc& D, float* feat, int32_t* lb, cudaStream_t st, bool sw)
{
    if (D.n <= 0) return cudaSuccess;
    int blocks = (D.n + 7) / 8;
    blocks = std::min(blocks, device_sms() * 16);
    // WFA pairs (150-10,000 bases): differences / 8, lengths / 256; SW pairs
    // (text with flanks, up to tens of kb): differences / 64, lengths / 8192
    const float s_diff = sw ? 1.0f / 64.0f : 0.125f, s_len = sw ? 1.0f / 8192.0f : 1.0f / 256.0f;
    launch_begin(K_SKETCH, st);
    if (D.packed) sketch_packed_kernel<<<blocks, 256, 0, st>>>(D, feat, lb, s_diff, s_len);
    else sketch_kernel<<<blocks, 256, 0, st>>>(D, feat, lb, s_diff, s_len);
    launch_end(K_SKETCH, st);
    return cudaGetLastError();
}

static Model* model_for_current(bool create) { return model_for(t_model_slot, create); }

// A slot's weights on the current device for inference, or null when none is loaded.
static const __nv_bfloat16* model_weights(int slot)
{
    std::lock_guard<std::mutex> lk(g_model_mu);
    Model* M = model_for(slot, false);
    return (M && M->ready) ? M->w : nullptr;
}
const __nv_bfloat16* cost_model_weights() { return model_weights(0); }

bool cost_model_loaded() { return cost_model_weights() != nullptr; }
bool sw_model_loaded() { return model_weights(1) != nullptr; }

// Inference of the selected slot's model: the tensor-core forward pass.
cudaError_t launch_mlp_forward(const float* feat, int n, float* y, cudaStream_t st)
{
    const __nv_bfloat16* w = model_weights(t_model_slot);
    if (!w) return cudaErrorNotReady;
    return run_forward_tc(w, feat, n, y, st);
}

// SW variant routing: features of every pair (a = text, b = pattern), the
// SW model's prediction of the best score as a fraction of the all-match
// score match * min(m, n), and try16[p] = 1 for a pair the 16-bit kernel
// should try: its predicted score with a margin (x 1.15 + 8 matches) fits 16
// bits (sw16_eligible_opt's test).  Purity and the exact hand-over at the
// 16-bit limit are the planner's and the kernel's, so a wrong prediction only
// costs time.
__global__ void sw_route_kernel(PairDesc D, const float* __restrict__ y, int match, int go, uint8_t* __restrict__ try16)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < D.n; p += gridDim.x * blockDim.x) {
        const int m = D.a_len[p], n = D.b_len[p];
        const float frac = fminf(fmaxf(y[2 * (int64_t)p], 0.f), 1.f);
        const float all = (float)match * (float)min(max(m, 0), max(n, 0));
        const float pred = frac * all * 1.15f + 8.f * (float)match;
        try16[p] = (m > 0 && n > 0 && pred + (float)(BIAS16 + go) < 32000.f) ? 1 : 0;
    }
}

cudaError_t launch_sw_route(const PairDesc& D, int match, int go, float* feat, float* y, uint8_t* try16, cudaStream_t st)
{
    const __nv_bfloat16* w = model_weights(1);
    if (!w) return cudaErrorNotReady;
    if (D.n <= 0) return cudaSuccess;
    cudaError_t e = launch_sketch(D, feat, nullptr, st, true);
    if (e == cudaSuccess) e = run_forward_tc(w, feat, D.n, y, st);
    if (e != cudaSuccess) return e;
    int blocks = std::min((D.n + 255) / 256, device_sms() * 8);
    launch_begin(K_ROUTE, st);
    sw_route_kernel<<<blocks, 256, 0, st>>>(D, y, match, go, try16);
    launch_end(K_ROUTE, st);
    return cudaGetLastError();
}

}  // namespace ga

using namespace ga;

extern "C" {

int32_t ga_cost_model_nparams(void) { return NPARAM; }

int32_t ga_model_select(int32_t which)
{
    if (which < 0 || which >= N_MODEL_SLOTS) return GA_INVALID_ARGUMENT;
    t_model_slot = which;
    return GA_OK;
}

int32_t ga_cost_model_set(const float* params, int32_t n)
{
    if (!params || n != NPARAM) return GA_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(g_model_mu);
    Model* M = model_for_current(true);
    if (!M) return GA_DEVICE_ERROR;
    if (cudaMemcpy(M->master, params, NPARAM * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(M->m1, 0, NPARAM * sizeof(float)) != cudaSuccess ||
        cudaMemset(M->m2, 0, NPARAM * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        return GA_DEVICE_ERROR;
    }
    to_bf16_kernel<<<64, 256>>>(M->master, M->w, NPARAM);
    if (cudaDeviceSynchronize() != cudaSuccess) { cudaGetLastError(); return GA_DEVICE_ERROR; }
    M->step = 0;
    M->ready = true;
    return GA_OK;
}

int32_t ga_cost_model_get(float* params, int32_t n)
{
    if (!params || n != NPARAM) return GA_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(g_model_mu);
    Model* M = model_for_current(false);
    if (!M || !M->ready) return GA_INVALID_ARGUMENT;
    if (cudaMemcpy(params, M->master, NPARAM * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return GA_DEVICE_ERROR;
    }
    return GA_OK;
}

int32_t ga_wfa_features(const ga_device_batch* b, float* feat, int32_t* lower_bound, void* stream)
{
    if (!b || b->n < 0 || !feat) return GA_INVALID_ARGUMENT;
    PairDesc D;
    D.seq = b->seq; D.packed = nullptr; D.pure = nullptr;
    D.a_off = b->a_off; D.a_len = b->a_len; D.b_off = b->b_off; D.b_len = b->b_len; D.out_off = b->out_off; D.n = b->n;
    cudaStream_t st = (cudaStream_t)stream;
    if (launch_sketch(D, feat, lower_bound, st, false) != cudaSuccess) { cudaGetLastError(); return GA_DEVICE_ERROR; }
    if (!stream && cudaStreamSynchronize(st) != cudaSuccess) { cudaGetLastError(); return GA_DEVICE_ERROR; }
    return GA_OK;
}

int32_t ga_sw_features(const ga_device_batch* b, float* feat, void* stream)
{
    if (!b || b->n < 0 || !feat) return GA_INVALID_ARGUMENT;
    PairDesc D;
    D.seq = b->seq; D.packed = nullptr; D.pure = nullptr;
    D.a_off = b->a_off; D.a_len = b->a_len; D.b_off = b->b_off; D.b_len = b->b_len; D.out_off = b->out_off; D.n = b->n;
    cudaStream_t st = (cudaStream_t)stream;
    if (launch_sketch(D, feat, nullptr, st, true) != cudaSuccess) { cudaGetLastError(); return GA_DEVICE_ERROR; }
    if (!stream && cudaStreamSynchronize(st) != cudaSuccess) { cudaGetLastError(); return GA_DEVICE_ERROR; }
    return GA_OK;
}

int32_t ga_mlp_forward(const float* feat, int32_t n, float* y, void* stream)
{
    if (!feat || !y || n < 0) return GA_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    const __nv_bfloat16* w = model_weights(t_model_slot);
    if (!w) return GA_INVALID_ARGUMENT;
    const cudaError_t e = run_forward(w, feat, n, y, st);
    if (e == cudaErrorNotReady) return GA_INVALID_ARGUMENT;
    if (e != cudaSuccess) { cudaGetLastError(); return GA_DEVICE_ERROR; }
    if (!stream && cudaStreamSynchronize(st) != cudaSuccess) { cudaGetLastError(); return GA_DEVICE_ERROR; }
    return GA_OK;
}

int32_t ga_mlp_forward_fast(const float* feat, int32_t n, float* y, void* stream)
{
    if (!feat || !y || n < 0) return GA_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    const cudaError_t e = launch_mlp_forward(feat, n, y, st);
    if (e == cudaErrorNotReady) return GA_INVALID_ARGUMENT;
    if (e != cudaSuccess) { cudaGetLastError(); return GA_DEVICE_ERROR; }
    if (!stream && cudaStreamSynchronize(st) != cudaSuccess) { cudaGetLastError(); return GA_DEVICE_ERROR; }
    return GA_OK;
}

int32_t ga_mlp_gradient(const float* feat, const float* target, int32_t n, float* grad_host, float* loss_host)
{
    if (!feat || !target || n <= 0 || !grad_host) return GA_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(g_model_mu);
    Model* M = model_for_current(false);
    if (!M || !M->ready) return GA_INVALID_ARGUMENT;
    if (run_backward(M->w, feat, target, n, M->grad, M->loss, 0) != cudaSuccess ||
        cudaMemcpy(grad_host, M->grad, NPARAM * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
        (loss_host && cudaMemcpy(loss_host, M->loss, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)) {
        cudaGetLastError();
        return GA_DEVICE_ERROR;
    }
    return GA_OK;
}

int32_t ga_mlp_train_step(const float* feat, const float* target, int32_t n, float lr, float* loss_host, void* stream)
{
    if (!feat || !target || n <= 0) return GA_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(g_model_mu);
    Model* M = model_for_current(false);
    if (!M || !M->ready) return GA_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (run_backward(M->w, feat, target, n, M->grad, M->loss, st) != cudaSuccess) { cudaGetLastError(); return GA_DEVICE_ERROR; }
    M->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f / (1.f - powf(b1, (float)M->step)), c2 = 1.f / (1.f - powf(b2, (float)M->step));
    launch_begin(K_MLP, st);
    adam_kernel<<<64, 256, 0, st>>>(M->master, M->w, M->grad, M->m1, M->m2, NPARAM, lr, b1, b2, 1e-8f, c1, c2);
    launch_end(K_MLP, st);
    if (cudaGetLastError() != cudaSuccess) return GA_DEVICE_ERROR;
    if (loss_host) {
        if (cudaMemcpyAsync(loss_host, M->loss, sizeof(float), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            cudaGetLastError();
            return GA_DEVICE_ERROR;
        }
        *loss_host /= (float)n;
    }
    return GA_OK;
}

}  // extern "C"
