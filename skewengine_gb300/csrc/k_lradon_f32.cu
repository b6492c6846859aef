// Local Radon transform in float32 (SKE_FLAG_LOCAL_RADON_F32): the same
// quantity as k_lradon (pointRadon, src/kernelRADN.h:114-182), computed on the
// FP32 pipes instead of the reference's binary64 FFTs.
//
// For every valid skewed cell (i, j) of a sector:
//   W(k, j) = sum of the 65 staged cells l = j-32 .. j+32 of row k (float32, in
//             increasing l; cells outside a row's valid range are 0)
//   x[m]    = W(i-32+m, j) * gauss[m]                      m = 0..63
//   Y[k]    = taper[k] * (sum_m x[m] cos(2 pi k m / 64)) / 8      k = 0..25
//             (the real part of the 64-point transform of the real x, scaled
//             by 1/sqrt(64) as the reference's (0.125, 0) product)
//   Z[m]    = (sum_k Y[k] e^(-2 pi i k m / 64)) / 8               m = 4..31
//   out     = |Z[m-1]|^2 for the first m >= 5 with |Z[m]|^2 > |Z[m-1]|^2, else 0.
// Only the transform bins the reference reads are formed, as direct sums: the
// 64 x 26 cosine products of Y and the 26 x 28 complex products of Z.  The
// twiddles (cosines and sines of 2 pi (k m mod 64) / 64, rounded to float on
// the host) sit in shared memory as one row per m, read by every thread at the
// same address (broadcast, 16 bytes per load), with the 26 bins unrolled in
// registers.  Two cells per thread (a twiddle row serves both); a CTA of 256
// threads owns a 32 x 32 tile of cells, stages the skewed rows it needs (95
// rows x 96 columns) and forms each W once.
// The order of the float32 sums differs from the reference's binary64 FFT, so
// values differ in their last bits, and where two successive |Z|^2 nearly tie
// the first ascent can fall on another bin: the rate of output cells that
// differ by more than a relative 1e-3 from the reference is measured and
// stated (tests/test_local_radon.py).  Ownership of cells past a row's span
// follows owner_row as in k_lradon.
#include <cmath>

#include "kernels.h"

namespace ske {

namespace {

constexpr int kW = kLocalRadonWindow;  // 64
constexpr int kHalf = kW / 2;          // 32
constexpr int kKeep = kLocalRadonKeep;  // 26
constexpr int kTI = 32, kTJ = 32;
constexpr int kRows = kTI + kW - 1;  // 95 W rows a tile needs
constexpr int kCols = kTJ + kW;      // 96 staged columns
constexpr int kThreads = 256;
constexpr int kZ0 = 4, kZ1 = 32;  // |Z_m|^2 formed for m = kZ0 .. kZ1 - 1
constexpr int kZn = kZ1 - kZ0;
constexpr int kKP = 28;  // twiddle row pitch (kKeep padded to 16 bytes)

// Row m of the first transform: cos(2 pi k m / 64); rows m = kZ0.. of the
// second: cos and sin of 2 pi k m / 64; k < kKeep, zero padding.
__constant__ float c_tx[kW * kKP];
__constant__ float c_tzc[kZn * kKP];
__constant__ float c_tzs[kZn * kKP];

struct SmemF {
    float s[kRows][kCols];
    float w[kRows][kTJ];
    float gauss[kW];
    float taper[kKP];
    float tx[kW][kKP];
    float tzc[kZn][kKP];
    float tzs[kZn][kKP];
};

__global__ void __launch_bounds__(kThreads)
    k_lradon_f32(DevGeometry g, Batch b, const float* __restrict__ SI, float* __restrict__ SO, int64_t stride,
                 int tiles_j, const double* __restrict__ gauss_all, const double* __restrict__ taper) {
    extern __shared__ __align__(16) float smem_f[];
    SmemF& sm = *reinterpret_cast<SmemF*>(smem_f);
    const int slot = blockIdx.y;
    const SectorDesc& d = g.desc[b.angle[slot]];
    const int i0 = (blockIdx.x / tiles_j) * kTI, j0 = (blockIdx.x % tiles_j) * kTJ;
    if (i0 >= d.H) return;
    const int32_t* first = g.first + d.row_off;
    const int32_t* last = g.last + d.row_off;
    int any = 0;
    for (int r = threadIdx.x; r < kTI; r += blockDim.x) {
        const int i = i0 + r;
        if (i < d.H && first[i] < j0 + kTJ && last[i] > j0 && first[i] < last[i]) any = 1;
    }
    if (!__syncthreads_or(any)) return;

    const float* in = SI + slot * stride;
    for (int t = threadIdx.x; t < kRows * kCols; t += blockDim.x) {
        const int r = t / kCols, c = t % kCols;
        const int k = i0 - kHalf + r, l = j0 - kHalf + c;
        float v = 0.0f;
        if (k >= 0 && k < d.H && l >= first[k] && l < last[k]) v = in[(int64_t)k * d.dim_i + l];
        sm.s[r][c] = v;
    }
    for (int t = threadIdx.x; t < kW; t += blockDim.x) sm.gauss[t] = (float)gauss_all[(int64_t)b.angle[slot] * kW + t];
    for (int t = threadIdx.x; t < kKeep; t += blockDim.x) sm.taper[t] = (float)taper[t];
    for (int t = threadIdx.x; t < kW * kKP; t += blockDim.x) (&sm.tx[0][0])[t] = c_tx[t];
    for (int t = threadIdx.x; t < kZn * kKP; t += blockDim.x) {
        (&sm.tzc[0][0])[t] = c_tzc[t];
        (&sm.tzs[0][0])[t] = c_tzs[t];
    }
    __syncthreads();
    // Window sums: warp per row, lane per column, 65 sequential adds.
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = warp; r < kRows; r += kThreads / 32) {
        float acc = 0.0f;
#pragma unroll 5
        for (int l = 0; l <= kW; l++) acc = __fadd_rn(acc, sm.s[r][lane + l]);
        sm.w[r][lane] = acc;
    }
    __syncthreads();

    // Two cells per thread, rows ci and ci + kTI/2 of the tile: every twiddle
    // row and window weight read from shared memory serves both.
    float* out = SO + slot * stride;
    for (int ca = warp; ca < kTI / 2; ca += kThreads / 32) {
        const int cj = lane, j = j0 + cj;
        int64_t p[2];
        bool valid[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int i = i0 + ca + u * (kTI / 2);
            valid[u] = i < d.H && j >= first[i] && j < last[i];
            p[u] = (int64_t)i * d.dim_i + j;
            if (valid[u] && j >= d.dim_i && owner_row(d, first, last, p[u]) != i) valid[u] = false;
        }
        if (!valid[0] && !valid[1]) continue;
        float re[2][kKeep];
#pragma unroll
        for (int u = 0; u < 2; u++)
#pragma unroll
            for (int k = 0; k < kKeep; k++) re[u][k] = 0.0f;
#pragma unroll 2
        for (int m = 0; m < kW; m++) {
            const float gm = sm.gauss[m];
            const float x0 = __fmul_rn(sm.w[ca + m][cj], gm);
            const float x1 = __fmul_rn(sm.w[ca + kTI / 2 + m][cj], gm);
            const float4* t4 = reinterpret_cast<const float4*>(sm.tx[m]);
#pragma unroll
            for (int q = 0; q < kKP / 4; q++) {
                const float4 t = t4[q];
                const float tv[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
                for (int e = 0; e < 4; e++)
                    if (4 * q + e < kKeep) {
                        re[0][4 * q + e] = __fmaf_rn(x0, tv[e], re[0][4 * q + e]);
                        re[1][4 * q + e] = __fmaf_rn(x1, tv[e], re[1][4 * q + e]);
                    }
            }
        }
#pragma unroll
        for (int u = 0; u < 2; u++)
#pragma unroll
            for (int k = 0; k < kKeep; k++) re[u][k] = __fmul_rn(sm.taper[k], __fmul_rn(re[u][k], 0.125f));
        float prev[2] = {0.0f, 0.0f}, found[2] = {0.0f, 0.0f};
        bool done[2] = {false, false};
#pragma unroll 2
        for (int m = kZ0; m < kZ1; m++) {
            float zr[2] = {0.0f, 0.0f}, zi[2] = {0.0f, 0.0f};
            const float4* tc4 = reinterpret_cast<const float4*>(sm.tzc[m - kZ0]);
            const float4* ts4 = reinterpret_cast<const float4*>(sm.tzs[m - kZ0]);
#pragma unroll
            for (int q = 0; q < kKP / 4; q++) {
                const float4 c = tc4[q], sn = ts4[q];
                const float cv[4] = {c.x, c.y, c.z, c.w}, sv[4] = {sn.x, sn.y, sn.z, sn.w};
#pragma unroll
                for (int e = 0; e < 4; e++)
                    if (4 * q + e < kKeep) {
#pragma unroll
                        for (int u = 0; u < 2; u++) {
                            zr[u] = __fmaf_rn(re[u][4 * q + e], cv[e], zr[u]);
                            zi[u] = __fmaf_rn(re[u][4 * q + e], sv[e], zi[u]);
                        }
                    }
            }
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const float a = __fmul_rn(zr[u], 0.125f), bq = __fmul_rn(zi[u], 0.125f);
                const float nm = __fadd_rn(__fmul_rn(a, a), __fmul_rn(bq, bq));
                if (m > kZ0 && !done[u] && nm > prev[u]) {
                    found[u] = prev[u];
                    done[u] = true;
                }
                prev[u] = nm;
            }
        }
#pragma unroll
        for (int u = 0; u < 2; u++)
            if (valid[u]) out[p[u]] = found[u];
    }
}

}  // namespace

int lradon_f32_init_tables() {
    static float tx[kW * kKP], tzc[kZn * kKP], tzs[kZn * kKP];
    for (int m = 0; m < kW; m++)
        for (int k = 0; k < kKP; k++)
            tx[m * kKP + k] = k < kKeep ? (float)std::cos(2.0 * M_PI * ((k * m) % kW) / kW) : 0.0f;
    for (int m = kZ0; m < kZ1; m++)
        for (int k = 0; k < kKP; k++) {
            const double a = 2.0 * M_PI * ((k * m) % kW) / kW;
            tzc[(m - kZ0) * kKP + k] = k < kKeep ? (float)std::cos(a) : 0.0f;
            tzs[(m - kZ0) * kKP + k] = k < kKeep ? (float)std::sin(a) : 0.0f;
        }
    if (cudaMemcpyToSymbol(c_tx, tx, sizeof(tx)) != cudaSuccess) return -1;
    if (cudaMemcpyToSymbol(c_tzc, tzc, sizeof(tzc)) != cudaSuccess) return -1;
    if (cudaMemcpyToSymbol(c_tzs, tzs, sizeof(tzs)) != cudaSuccess) return -1;
    return 0;
}

cudaError_t launch_local_radon_f32(const DevGeometry& g, const Batch& b, const float* SI, float* SO, int64_t stride,
                                   int max_H, int max_cols, const double* gauss, const double* taper,
                                   cudaStream_t st) {
    if (b.count == 0) return cudaSuccess;
    const int tiles_i = (max_H + kTI - 1) / kTI, tiles_j = (max_cols + kTJ - 1) / kTJ;
    const size_t smem = sizeof(SmemF);
    cudaError_t e = cudaFuncSetAttribute(k_lradon_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_lradon_f32<<<dim3((unsigned)(tiles_i * tiles_j), b.count), kThreads, smem, st>>>(g, b, SI, SO, stride, tiles_j,
                                                                                     gauss, taper);
    return cudaGetLastError();
}

}  // namespace ske
