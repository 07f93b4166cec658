// qc.cu -- CIGAR post-processing of a one-reference-against-many SW batch on
// the device: the per-record checks of the reference's gene QC tool
// (tools/gene_qc.cpp:170-234), one thread per pair over its CIGAR where the
// SW kernels left it, so only four integers per pair come back to the host.
//
// Per pair with a positive score, walking the CIGAR from (start_i, start_j)
// (i in the text, j in the reference, whose reading frame is `frame`):
//   - stops: reference codons (codon position (j - frame) mod 3) whose three
//     columns all pair a text base, contiguous in the text, and read a stop
//     codon of genetic code `code` (1: TAA TAG TGA; 2: TAA TAG AGA AGG);
//   - fs_runs: runs of I or D whose length is not a multiple of 3;
//   - fs_net: (inserted - deleted) mod 3, signed to -1, 0 or +1;
//   - stop_end: 1 when the last stop found sits in the span's last complete
//     codon (the gene's own terminator); it is then not counted in stops.
#include "../../include/genoaligner_gb300.h"
#include "kernels.cuh"

namespace ga {

__device__ __forceinline__ bool qc_stop(uint8_t a, uint8_t b, uint8_t c, int code)
{
    if (a == 'T' && b == 'A' && (c == 'A' || c == 'G')) return true;
    if (code == 1 && a == 'T' && b == 'G' && c == 'A') return true;
    if (code == 2 && a == 'A' && b == 'G' && (c == 'A' || c == 'G')) return true;
    return false;
}

__global__ void qc_kernel(PairDesc D, const int32_t* __restrict__ score, const int32_t* __restrict__ pos,
                          const int32_t* __restrict__ len, const char* __restrict__ cig, int frame, int code,
                          int32_t* __restrict__ out)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < D.n; p += gridDim.x * blockDim.x) {
        int fs = 0, fs_net = 0, stops = 0, stop_end = 0;
        const int L = len[p];
        if (score[p] > 0 && L > 0) {
            const int m = D.a_len[p], n = D.b_len[p];
            const uint8_t* T = D.seq + D.a_off[p];
            const char* cg = cig + D.out_off[p] + (m + n) - L;
            int i = pos[4 * p], j = pos[4 * p + 1];
            uint8_t codon[3] = {0, 0, 0};
            int fill = -1, i0 = -1, last_codon_j = -1, stop_at = -1;
            long long ins = 0, del = 0;
            char run_op = 0;
            int run = 0;
            for (int q = 0; q <= L; ++q) {
                const char op = q < L ? cg[q] : 0;
                // indel runs (a run ends at the first different op)
                if (op != run_op) {
                    if (run_op == 'I' || run_op == 'D') {
                        if (run % 3 != 0) ++fs;
                        if (run_op == 'I') ins += run; else del += run;
                    }
                    run_op = op;
                    run = 0;
                }
                ++run;
                if (q == L) break;
                if (op == 'M' || op == 'X') {
                    const int ph = ((j - frame) % 3 + 3) % 3;
                    if (ph == 0) { fill = 0; i0 = i; }
                    if (fill == ph && i >= 0 && i < m) codon[fill++] = T[i];
                    else fill = -1;
                    if (fill == 3) {
                        if (i == i0 + 2) {
                            last_codon_j = j - 2;
                            if (qc_stop(codon[0], codon[1], codon[2], code)) {
                                ++stops;
                                stop_at = j - 2;
                            }
                        }
                        fill = -1;
                    }
                    ++i;
                    ++j;
                } else if (op == 'I') {
                    ++i;
                } else if (op == 'D') {
                    fill = -1;
                    ++j;
                }
            }
            fs_net = (int)(((ins - del) % 3 + 3) % 3);
            if (fs_net > 1) fs_net -= 3;
            if (stops > 0 && stop_at == last_codon_j) {
                stop_end = 1;
                --stops;
            }
        }
        out[4 * p] = fs;
        out[4 * p + 1] = fs_net;
        out[4 * p + 2] = stops;
        out[4 * p + 3] = stop_end;
    }
}

cudaError_t launch_qc(const PairDesc& D, const int32_t* score, const int32_t* pos, const int32_t* len, const char* cig,
                      int frame, int code, int32_t* out, cudaStream_t st)
{
    if (D.n <= 0) return cudaSuccess;
    int blocks = (D.n + 127) / 128;
    blocks = std::min(blocks, device_sms() * 16);
    launch_begin(K_QC, st);
    qc_kernel<<<blocks, 128, 0, st>>>(D, score, pos, len, cig, frame, code, out);
    launch_end(K_SWPLAN, st);
    return cudaGetLastError();
}

}  // namespace ga

extern "C" int32_t ga_sw_qc_device(const ga_device_batch* b, const int32_t* score, const int32_t* pos,
                                   const int32_t* len, const char* cigar, int32_t frame, int32_t code, int32_t* out,
                                   void* stream)
{
    if (!b || b->n < 0 || frame < 0 || frame > 2 || (code != 1 && code != 2) ||
        (b->n > 0 && (!b->seq || !b->a_off || !b->a_len || !b->b_len || !b->out_off || !score || !pos || !len ||
                      !cigar || !out)))
        return GA_INVALID_ARGUMENT;
    ga::PairDesc D;
    D.seq = b->seq; D.packed = nullptr; D.pure = nullptr;
    D.a_off = b->a_off; D.a_len = b->a_len; D.b_off = b->b_off; D.b_len = b->b_len;
    D.out_off = b->out_off; D.n = b->n;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = ga::launch_qc(D, score, pos, len, cigar, frame, code, out, st);
    if (e == cudaSuccess && !stream) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return GA_DEVICE_ERROR;
    }
    return GA_OK;
}
