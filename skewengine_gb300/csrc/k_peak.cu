// FP32 pipe throughput probe: the roofline denominator of the total-viewshed
// sweep, whose work is FP32 lane operations (subtract, divide, compare per
// line-of-sight step) rather than bytes or tensor-core FLOPs.
//
// Each thread runs 8 independent chains of fused multiply-adds, scalar
// (fma.rn.f32) or packed two-wide (fma.rn.f32x2), long enough to run ~10 ms per
// launch.  Reported as FP32 lane operations per second, one fused multiply-add
// counted as one operation (it is one issue of one lane).
#include <algorithm>
#include <cstdint>

#include "kernels.h"

namespace ske {

namespace {

constexpr int kChains = 8;

__global__ void k_fma_scalar(float* out, float a, float b, int iters) {
    float acc[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) acc[c] = a + c + threadIdx.x;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) acc[c] = __fmaf_rn(acc[c], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += acc[c];
    if (s == 1.2345f) out[0] = s;  // keeps the chains live
}

__global__ void k_fma_packed(float* out, float a, float b, int iters) {
    uint64_t acc[kChains], va, vb;
    asm("mov.b64 %0, {%1,%1};" : "=l"(va) : "f"(a));
    asm("mov.b64 %0, {%1,%1};" : "=l"(vb) : "f"(b));
#pragma unroll
    for (int c = 0; c < kChains; c++) {
        const float lo = a + c + threadIdx.x, hi = lo + 0.5f;
        asm("mov.b64 %0, {%1,%2};" : "=l"(acc[c]) : "f"(lo), "f"(hi));
    }
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(acc[c]) : "l"(va), "l"(vb));
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kChains; c++) {
        float lo, hi;
        asm("mov.b64 {%0,%1}, %2;" : "=f"(lo), "=f"(hi) : "l"(acc[c]));
        s += lo + hi;
    }
    if (s == 1.2345f) out[0] = s;
}

__global__ void k_dfma(double* out, double a, double b, int iters) {
    double acc[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) acc[c] = a + c + threadIdx.x;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) acc[c] = __fma_rn(acc[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += acc[c];
    if (s == 1.2345) out[0] = s;
}

}  // namespace

// Best of `reps` timed launches of the binary64 probe: DFMA lane ops/s.
cudaError_t measure_fp64_peak(int num_sms, int reps, double* dfma_ops) {
    double* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(double));
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int threads = 256, blocks = num_sms * 4, iters = 256;
    double best = 0;
    for (int r = 0; r < reps + 1 && e == cudaSuccess; r++) {
        cudaEventRecord(a);
        k_dfma<<<blocks, threads>>>(d, 0.999, 0.001, iters);
        cudaEventRecord(b);
        e = cudaEventSynchronize(b);
        if (e == cudaSuccess) e = cudaGetLastError();
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        const double lanes = (double)blocks * threads * iters * kChains;
        if (r > 0 && ms > 0) best = std::max(best, lanes / (ms * 1e-3));
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(d);
    *dfma_ops = best;
    return e;
}

// Best of `reps` timed launches of each probe; returns lane-op/s (scalar, packed).
cudaError_t measure_fp32_peak(int num_sms, int reps, double* scalar_ops, double* packed_ops) {
    float* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(float));
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int threads = 256, blocks = num_sms * 8, iters = 4096;
    double best[2] = {0, 0};
    for (int kind = 0; kind < 2 && e == cudaSuccess; kind++) {
        for (int r = 0; r < reps + 1 && e == cudaSuccess; r++) {  // first launch warms up
            cudaEventRecord(a);
            if (kind == 0) k_fma_scalar<<<blocks, threads>>>(d, 0.999f, 0.001f, iters);
            else k_fma_packed<<<blocks, threads>>>(d, 0.999f, 0.001f, iters);
            cudaEventRecord(b);
            e = cudaEventSynchronize(b);
            if (e == cudaSuccess) e = cudaGetLastError();
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            const double lanes = (double)blocks * threads * iters * kChains * (kind ? 2 : 1);
            if (r > 0 && ms > 0) best[kind] = std::max(best[kind], lanes / (ms * 1e-3));
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(d);
    *scalar_ops = best[0];
    *packed_ops = best[1];
    return e;
}

}  // namespace ske
