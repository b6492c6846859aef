// Cepstrum motion-blur estimation (kernelBLUR, src/kernelBLUR.h:267-302 ->
// lineCepstrum :153-228 -> select_subarray :69-85, getBlurParameter2 :88-110).
//
// For every valid skewed cell j of row r: a 64-cell window of the row centred at
// j (cells outside [first, last) are zero; the effective window is 64 because
// kernelRADN.h:19 wins the shared KERNELCOMMONS guard), X = FFT(window)/8,
// c = FFT(log|X_k|^2, k < 32)/sqrt(32), s_k = -min(0, Re c_k) for k < 16, and
// the output is (float)(10000 * peak(s)).
//
// One warp per cell: the window lives in shared memory as complex doubles and
// each lane performs one butterfly per stage of the reference radix-2
// decimation-in-frequency FFT (helper.h:59-106) with the reference's twiddle
// sequence, in binary64 without fused operations; cells whose FFT input is
// finite use warp_fft_real (same values up to the sign of zeros, which the
// outputs cannot see).  The logarithm is CUDA's double-precision log().
#include "kernels.h"

namespace ske {

namespace {

constexpr int kWin = kBlurWindow;  // 64
constexpr int kWarpsPerBlock = 8;

__global__ void __launch_bounds__(kWarpsPerBlock * 32, 6)
    k_cepstrum(DevGeometry g, Batch b, const float* __restrict__ SI, float* __restrict__ SO, int64_t stride,
               int64_t len, const double* __restrict__ tw64, const double* __restrict__ tw32) {
    __shared__ cd xs[kWarpsPerBlock][kWin];
    __shared__ double twa[2 * (kWin - 1)], twb[2 * (kWin / 2 - 1)];
    for (int i = threadIdx.x; i < 2 * (kWin - 1); i += blockDim.x) twa[i] = tw64[i];
    for (int i = threadIdx.x; i < 2 * (kWin / 2 - 1); i += blockDim.x) twb[i] = tw32[i];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    cd* x = xs[warp];
    const int slot = blockIdx.y;
    const SectorDesc d = g.desc[b.angle[slot]];
    const int32_t* first = g.first + d.row_off;
    const int32_t* last = g.last + d.row_off;
    const float* in = SI + slot * stride;
    float* out = SO + slot * stride;
    const double norm64 = __ddiv_rn(1.0, __dsqrt_rn(64.0));
    const double norm32 = __ddiv_rn(1.0, __dsqrt_rn(32.0));
    const int64_t warps = (int64_t)gridDim.x * kWarpsPerBlock;
    for (int64_t p = (int64_t)blockIdx.x * kWarpsPerBlock + warp; p < len; p += warps) {
        const int r = owner_row(d, first, last, p);  // warp-uniform
        if (r < 0) {
            if (lane == 0) out[p] = 0.0f;
            continue;
        }
        const int64_t base = (int64_t)r * d.dim_i;
        const int j = (int)(p - base);
        const int f = first[r], l = last[r];
        bool fin = true;
        for (int m = lane; m < kWin; m += 32) {
            const int idx = j - kWin / 2 + m;
            x[m] = (idx < f || idx >= l) ? cd{0.0, 0.0} : cd{(double)in[base + idx], 0.0};
            fin = fin && isfinite(x[m].re);
        }
        __syncwarp();
        // Finite real input: the reduced-work FFT gives the same values up to the
        // sign of zeros, which neither |X|^2 nor -min(0, c) can see.
        if (__all_sync(0xffffffffu, fin)) warp_fft_real<kKeepLow>(x, kWin, twa, lane);  // X_k, k < 32
        else warp_fft(x, kWin, twa, lane);
        // |X_k|^2 of the 1/sqrt(64)-scaled spectrum, k < 32, then its log.
        {
            const cd v = x[lane];
            const double re = __dmul_rn(v.re, norm64), im = __dmul_rn(v.im, norm64);
            const double ps = __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im));
            __syncwarp();
            x[lane] = {log(ps), 0.0};
        }
        __syncwarp();
        // A zero power gives log = -inf: such cells keep the exact FFT.
        if (__all_sync(0xffffffffu, isfinite(x[lane].re)))
            warp_fft_real<kKeepLowRe>(x, kWin / 2, twb, lane);  // Re c_k, k < 16
        else warp_fft(x, kWin / 2, twb, lane);
        // s_k = -min(0, c_k) for k < 16 (lane k), then getBlurParameter2: from
        // index 5 skip the non-ascending head; the result is the sample before
        // the first ascent or any larger sample after the ascending one.  The
        // samples are -0 or positive (never +0 or NaN), so the reference's
        // sequential `s > best` scan and a max reduction give the same value.
        const int k = lane & (kWin / 4 - 1);
        const double c = __dmul_rn(x[k].re, norm32);
        const double sk = -((c < 0.0) ? c : 0.0);  // -std::min(0.0, c)
        const double prev = __shfl_up_sync(0xffffffffu, sk, 1);
        const unsigned asc = __ballot_sync(0xffffffffu, lane >= 5 && lane < kWin / 4 && sk > prev);
        double best = 0.0;
        if (asc) {
            const int i = __ffs(asc) - 1;  // first ascent
            double m = (lane == i - 1 || (lane > i && lane < kWin / 4)) ? sk : -0.0;
            for (int o = 16; o > 0; o >>= 1) {
                const double t = __shfl_xor_sync(0xffffffffu, m, o);
                m = t > m ? t : m;
            }
            best = m;
        }
        if (lane == 0) out[p] = __double2float_rn(__dmul_rn(best, 10000.0));
        __syncwarp();
    }
}

}  // namespace

cudaError_t launch_cepstrum(const DevGeometry& g, const Batch& b, const float* SI, float* SO, int64_t stride,
                            int64_t len, const double* tw64, const double* tw32, cudaStream_t st) {
    int64_t blocks = (len + kWarpsPerBlock - 1) / kWarpsPerBlock;
    if (blocks > 8192) blocks = 8192;
    k_cepstrum<<<dim3((unsigned)blocks, b.count), kWarpsPerBlock * 32, 0, st>>>(g, b, SI, SO, stride, len, tw64,
                                                                                 tw32);
    return cudaGetLastError();
}

}  // namespace ske
