// measure.cu -- throughput probe of the FP64 pipe, the denominator of the
// plain FP64 form's roofline.
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so the plain FP64
// leapfrog (whose per-site arithmetic must be IEEE double in the reference's
// order) is bound by the FP64 pipe, not by HBM.  This kernel issues only
// independent FP64 operations of one kind (8 chains per thread, no memory
// traffic in the loop) on every SM and reports thread instructions per second.
#include <cuda_runtime.h>

#include "../../include/iegpu.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreadsRate = 256;

template <int OP>
__global__ void __launch_bounds__(kThreadsRate) k_fp64_rate(double* out, double a, double b, int iters) {
    double x[kChains];
#pragma unroll
    for (int q = 0; q < kChains; ++q) x[q] = 1.0 + 1e-3 * (double)(threadIdx.x + q);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int q = 0; q < kChains; ++q) {
            if (OP == 0) x[q] = fma(x[q], a, b);
            else if (OP == 1) x[q] = x[q] + b;
            else x[q] = x[q] * a;
        }
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < kChains; ++q) s += x[q];
    if (s == 12345.678) out[blockIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" int iegpu_measure_fp64_rate(int op, double* inst_per_s) {
    if (!inst_per_s || op < 0 || op > 2) return IEGPU_EINVAL;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return IEGPU_ECUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return IEGPU_ECUDA;
    const int blocks = sms * 8;
    const int iters = 4096;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * (size_t)blocks) != cudaSuccess) return IEGPU_ENOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const double a = 1.0 - 1e-9, b = 1e-12;
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        if (op == 0) k_fp64_rate<0><<<blocks, kThreadsRate>>>(out, a, b, iters);
        else if (op == 1) k_fp64_rate<1><<<blocks, kThreadsRate>>>(out, a, b, iters);
        else k_fp64_rate<2><<<blocks, kThreadsRate>>>(out, a, b, iters);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;  // the first launch is a warm-up
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return IEGPU_ECUDA;
    const double inst = (double)blocks * kThreadsRate * kChains * (double)iters;
    *inst_per_s = inst / (best * 1e-3);
    return IEGPU_OK;
}
