// peak.cu -- integer-pipe throughput microbenchmark (the Smith-Waterman
// roofline's denominator).  Eight independent dependency chains per thread, a
// full grid, timed with CUDA events; the rate is reported in lane-operations
// per second (one C-level integer operation on one lane = 1).
//
//   variant 0: a = max(a + x, y) written as plain C    (2 ops per step)
//   variant 1: a = __viaddmax_s32(a, x, y)              (1 op per step)
//   variant 2: a = __vimax3_s32_relu(a, x, y)           (1 op per step)
//   3-10 and 11-13: other integer/DPX forms, one C-level operation each
//   (11: __vimax3_s16x2_relu, 12: __vimax3_s16x2, 13: __vmaxs2)
#include "common.cuh"
#include "../../include/genoaligner_gb300.h"

namespace ga {

template <int V>
__global__ void __launch_bounds__(256) int_peak_kernel(int iters, int x, int* out)
{
    int a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = (int)threadIdx.x * (k + 1) - 77 * k;
    const int y = (int)(threadIdx.x ^ blockIdx.x) - 1000;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if constexpr (V == 0) a[k] = max(a[k] + x, y + k);
                else if constexpr (V == 1) a[k] = __viaddmax_s32(a[k], x, y + k);
                else if constexpr (V == 2) a[k] = __vimax3_s32_relu(a[k], x - k, y);
                else if constexpr (V == 3) a[k] = max(a[k], y + k) ^ x;             // max + xor
                else if constexpr (V == 4) a[k] = a[k] + (y + k);                   // add
                else if constexpr (V == 5) a[k] = (int)__vmaxs2((unsigned)a[k], (unsigned)(y + k)) ^ x;
                else if constexpr (V == 6) a[k] = (int)__viaddmax_s16x2((unsigned)a[k], (unsigned)x, (unsigned)(y + k));
                else if constexpr (V == 7) {
                    bool ph, pl;
                    a[k] = (int)__vibmax_s16x2((unsigned)a[k], (unsigned)(y + k), &ph, &pl) + (ph ? 1 : 0) + (pl ? 2 : 0);
                } else if constexpr (V == 8) {
                    bool p;
                    a[k] = __vibmax_s32(a[k], y + k, &p) + (p ? 1 : 0);
                } else if constexpr (V == 9) a[k] = (int)__vcmpgtu2((unsigned)a[k], (unsigned)(y + k)) ^ x;
                else if constexpr (V == 11) a[k] = (int)__vimax3_s16x2_relu((unsigned)a[k], (unsigned)(y + k), (unsigned)x);
                else if constexpr (V == 12) a[k] = (int)__vimax3_s16x2((unsigned)a[k], (unsigned)(y + k), (unsigned)x);
                else if constexpr (V == 13) a[k] = (int)__vmaxs2((unsigned)a[k], (unsigned)(y + k));
                else a[k] = (a[k] & (y + k)) | (x ^ k);                              // logic
            }
        }
    }
    int s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s ^= a[k];
    if (s == 0x7fffffff) out[0] = s;          // keeps the chains live
}

}  // namespace ga

using namespace ga;

extern "C" int32_t ga_bench_int_peak(int32_t variant, double* lane_ops_per_s)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return GA_DEVICE_ERROR;
    }
    int* out = nullptr;
    if (cudaMalloc(&out, sizeof(int)) != cudaSuccess) { cudaGetLastError(); return GA_DEVICE_ERROR; }
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 8, threads = 256, iters = 2048;
    auto launch = [&] {
        launch_begin(K_PEAK, st);
        switch (variant) {
            case 0: int_peak_kernel<0><<<blocks, threads, 0, st>>>(iters, 3, out); break;
            case 1: int_peak_kernel<1><<<blocks, threads, 0, st>>>(iters, 3, out); break;
            case 2: int_peak_kernel<2><<<blocks, threads, 0, st>>>(iters, 3, out); break;
            case 3: int_peak_kernel<3><<<blocks, threads, 0, st>>>(iters, 3, out); break;
            case 4: int_peak_kernel<4><<<blocks, threads, 0, st>>>(iters, 3, out); break;
            case 5: int_peak_kernel<5><<<blocks, threads, 0, st>>>(iters, 3, out); break;
            case 6: int_peak_kernel<6><<<blocks, threads, 0, st>>>(iters, 3, out); break;
            case 7: int_peak_kernel<7><<<blocks, threads, 0, st>>>(iters, 3, out); break;
            case 8: int_peak_kernel<8><<<blocks, threads, 0, st>>>(iters, 3, out); break;
            case 9: int_peak_kernel<9><<<blocks, threads, 0, st>>>(iters, 3, out); break;
            case 11: int_peak_kernel<11><<<blocks, threads, 0, st>>>(iters, 3, out); break;
            case 12: int_peak_kernel<12><<<blocks, threads, 0, st>>>(iters, 3, out); break;
            case 13: int_peak_kernel<13><<<blocks, threads, 0, st>>>(iters, 3, out); break;
            default: int_peak_kernel<10><<<blocks, threads, 0, st>>>(iters, 3, out); break;
        }
        launch_end(K_PEAK, st);
    };
    launch();                                   // warm-up
    cudaEventRecord(a, st);
    const int reps = 5;
    for (int r = 0; r < reps; ++r) launch();
    cudaEventRecord(b, st);
    int32_t rc = GA_OK;
    float ms = 0.f;
    if (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess || ms <= 0.f) {
        cudaGetLastError();
        rc = GA_DEVICE_ERROR;
    } else {
        const double steps = (double)blocks * threads * iters * 16 * 8 * reps;
        const double ops = steps * (variant == 0 ? 2.0 : 1.0);
        *lane_ops_per_s = ops / (ms * 1e-3);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaStreamDestroy(st);
    cudaFree(out);
    return rc;
}
