// Local Radon transform (pointRadon, src/kernelRADN.h:114-182), the reference's
// Radon operator with its LRT switch set (kernelRADN.h:212-220).
//
// For every valid skewed cell (i, j) of a sector:
//   W(k, j) = sum over l = j-32 .. j+32 of S[k, l]   (binary64, in increasing l;
//             columns outside row k's valid range and rows outside the grid add 0)
//   x[m]    = W(i-32+m, j) * gauss[m],  m < 64,  gauss from the sector's scale
//   X       = FFT(x) / 8;  Y[k] = taper[k] * Re X[k] for k <= 25, else 0
//   Z       = FFT(Y) / 8;  out = getParameter(Z): from m = 5 the first
//             |Z_m|^2 > |Z_{m-1}|^2 gives |Z_{m-1}|^2 (none: 0), stored as float.
//
// GB300 mapping
//  * W(k, j) is shared by the 64 cells (k-32 .. k+31, j): a CTA takes a tile of
//    kTI x kTJ cells, stages the skewed rows it needs (kTI+63 rows, kTJ+64
//    columns, zeros outside the valid ranges) in shared memory and forms every
//    W of the tile once, each as the reference's sequential binary64 sum, so
//    the result is the reference's to the bit.
//  * One warp per cell then gathers its column of 64 W values, applies the
//    weights and runs both 64-point FFTs with one butterfly per lane per stage
//    (warp_fft: the reference's DIF order and twiddle sequence, binary64,
//    no fused operations).  The 1/sqrt(64) scaling is the reference's complex
//    multiplication by (0.125, 0).
//  * Tiles whose staged values are all finite use warp_fft_real (real-input
//    first stage, multiplication-free last stage) and real scalings: the same
//    values up to the sign of zeros, so the squared magnitudes, and the output,
//    are bit-identical; other tiles keep every operation of the reference.
//  * The Gaussian weights and the taper use host libm (local_radon_tables), as
//    the reference computes them on the host.
//  * Output cells past a row's span of the flat grid belong to the last row
//    covering them (owner_row), as in the reference's row-order writes.
#include <climits>

#include "kernels.h"

namespace ske {

namespace {

constexpr int kW = kLocalRadonWindow;  // 64
constexpr int kHalf = kW / 2;          // 32
constexpr int kTI = 32;                // cell rows per tile
constexpr int kTJ = 32;                // cell columns per tile
constexpr int kRows = kTI + kW - 1;    // W rows a tile needs
constexpr int kCols = kTJ + kW;        // staged columns: kTJ windows of 65
constexpr int kWarps = 8;

struct Smem {
    float s[kRows][kCols];
    double w[kRows][kTJ];
    cd x[kWarps][kW];  // per-warp FFT buffer; before the cell loop, a row's prefix sums
    double gauss[kW];
    double taper[kLocalRadonKeep];
    double tw[2 * (kW - 1)];
};

__global__ void __launch_bounds__(kWarps * 32)
    k_lradon(DevGeometry g, Batch b, const float* __restrict__ SI, float* __restrict__ SO, int64_t stride,
             int tiles_j, const double* __restrict__ gauss_all, const double* __restrict__ taper,
             const double* __restrict__ tw64) {
    extern __shared__ double smem_d[];
    Smem& sm = *reinterpret_cast<Smem*>(smem_d);
    const int slot = blockIdx.y;
    const SectorDesc& d = g.desc[b.angle[slot]];
    const int i0 = (blockIdx.x / tiles_j) * kTI, j0 = (blockIdx.x % tiles_j) * kTJ;
    if (i0 >= d.H) return;
    const int32_t* first = g.first + d.row_off;
    const int32_t* last = g.last + d.row_off;
    // Skip tiles without a valid cell.
    int any = 0;
    for (int r = threadIdx.x; r < kTI; r += blockDim.x) {
        const int i = i0 + r;
        if (i < d.H && first[i] < j0 + kTJ && last[i] > j0 && first[i] < last[i]) any = 1;
    }
    if (!__syncthreads_or(any)) return;

    const float* in = SI + slot * stride;
    int bad = 0;
    for (int t = threadIdx.x; t < kRows * kCols; t += blockDim.x) {
        const int r = t / kCols, c = t % kCols;
        const int k = i0 - kHalf + r, l = j0 - kHalf + c;
        float v = 0.0f;
        if (k >= 0 && k < d.H && l >= first[k] && l < last[k]) v = in[(int64_t)k * d.dim_i + l];
        sm.s[r][c] = v;
        bad |= !isfinite(v);
    }
    // Finite tiles take the reduced-work FFT (warp_fft_real); any non-finite
    // input keeps every operation of the reference.
    const bool finite = !__syncthreads_or(bad);
    for (int t = threadIdx.x; t < kW; t += blockDim.x) sm.gauss[t] = gauss_all[(int64_t)b.angle[slot] * kW + t];
    for (int t = threadIdx.x; t < kLocalRadonKeep; t += blockDim.x) sm.taper[t] = taper[t];
    for (int t = threadIdx.x; t < 2 * (kW - 1); t += blockDim.x) sm.tw[t] = tw64[t];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // Window sums, one warp per staged row.  Every float is an integer multiple
    // of 2^(e - 150); when the row's exponents span at most 28 binades and the
    // sum of its magnitudes in units of its smallest 2^e stays below 2^53, every
    // partial sum of the reference's sequential binary64 loop is exact, so each
    // window sum is the exact sum: a difference of two 64-bit integer prefix
    // sums.  Other rows (or a non-finite value) keep the sequential adds.
    static_assert(kCols == 3 * 32, "three staged cells per lane");
    static_assert(sizeof(cd) * kW >= sizeof(long long) * (kCols + 1), "prefix sums fit the FFT buffer");
    for (int r = warp; r < kRows; r += kWarps) {
        const float* row = sm.s[r];
        unsigned u[3], m[3];
        int ee[3], emin = INT_MAX, emax = 0;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            u[k] = __float_as_uint(row[3 * lane + k]);
            const int e8 = (int)((u[k] >> 23) & 0xffu);
            m[k] = (u[k] & 0x7fffffu) | (e8 ? 0x800000u : 0u);
            ee[k] = m[k] ? max(e8, 1) : INT_MAX;
            emin = min(emin, ee[k]);
            emax = max(emax, e8);
        }
        for (int o = 16; o > 0; o >>= 1) {
            emin = min(emin, __shfl_xor_sync(0xffffffffu, emin, o));
            emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
        }
        bool exact = emax != 0xff && (emin == INT_MAX || emax - emin <= 28);
        if (exact && emin != INT_MAX) {
            long long v[3];
            unsigned long long mag = 0;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const long long x = m[k] ? (long long)m[k] << (ee[k] - emin) : 0;  // < 2^52
                v[k] = (u[k] >> 31) ? -x : x;
                mag += (unsigned long long)x;
            }
            long long incl = v[0] + v[1] + v[2];
            for (int o = 1; o < 32; o <<= 1) {
                const long long t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            for (int o = 16; o > 0; o >>= 1) mag += __shfl_xor_sync(0xffffffffu, mag, o);
            exact = mag < (1ull << 53);
            if (exact) {
                long long* pre = reinterpret_cast<long long*>(sm.x[warp]);  // idle until the cell loop
                const long long excl = incl - (v[0] + v[1] + v[2]);
                pre[3 * lane] = excl;
                pre[3 * lane + 1] = excl + v[0];
                pre[3 * lane + 2] = excl + v[0] + v[1];
                if (lane == 31) pre[kCols] = incl;
                __syncwarp();
                const double scale = __longlong_as_double((long long)(emin - 150 + 1023) << 52);
                sm.w[r][lane] = __dmul_rn(__ll2double_rn(pre[lane + kW + 1] - pre[lane]), scale);
                __syncwarp();
            }
        } else if (exact) {
            sm.w[r][lane] = 0.0;  // all cells zero
        }
        if (!exact) {
            double acc = 0.0;
            for (int k = 0; k <= kW; k++) acc = __dadd_rn(acc, (double)row[lane + k]);
            sm.w[r][lane] = acc;
        }
    }
    __syncthreads();

    cd* x = sm.x[warp];
    const cd scale{0.125, 0.0};  // 1/sqrt(64) (helper.h:102-104)
    float* out = SO + slot * stride;
    for (int cell = warp; cell < kTI * kTJ; cell += kWarps) {
        const int ci = cell / kTJ, cj = cell % kTJ;
        const int i = i0 + ci, j = j0 + cj;
        if (i >= d.H || j < first[i] || j >= last[i]) continue;  // warp-uniform
        const int64_t p = (int64_t)i * d.dim_i + j;
        if (j >= d.dim_i && owner_row(d, first, last, p) != i) continue;
        for (int m = lane; m < kW; m += 32) x[m] = cd{__dmul_rn(sm.w[ci + m][cj], sm.gauss[m]), 0.0};
        __syncwarp();
        // Only Re X_k for k < 26 is read: the pruned FFT forms Re X_k, k < 32.
        if (finite) warp_fft_real<kKeepLowRe>(x, kW, sm.tw, lane);
        else warp_fft(x, kW, sm.tw, lane);
        for (int m = lane; m < kW; m += 32) {
            double y = 0.0;
            if (m < kLocalRadonKeep) {
                // Finite: x * (0.125, 0) is (re/8, im/8) up to the sign of zeros.
                const double re = finite ? __dmul_rn(x[m].re, 0.125) : cmul(x[m], scale).re;
                y = __dmul_rn(sm.taper[m], re);
            }
            x[m] = cd{y, 0.0};
        }
        __syncwarp();
        // Y is zero from bin 26 on; only Z_m for m < 32 is read.
        if (finite) warp_fft_real<kKeepLow, true>(x, kW, sm.tw, lane);
        else warp_fft(x, kW, sm.tw, lane);
        x[lane] = finite ? cd{__dmul_rn(x[lane].re, 0.125), __dmul_rn(x[lane].im, 0.125)} : cmul(x[lane], scale);
        __syncwarp();
        // getParameter: from m = 5 the first |Z_m|^2 > |Z_{m-1}|^2 gives
        // |Z_{m-1}|^2 (none: 0).  Lane m forms |Z_m|^2 (the reference's
        // products and sum); a ballot finds the first ascent.
        const double nm = __dadd_rn(__dmul_rn(x[lane].re, x[lane].re), __dmul_rn(x[lane].im, x[lane].im));
        const double prev = __shfl_up_sync(0xffffffffu, nm, 1);
        const unsigned asc = __ballot_sync(0xffffffffu, lane >= 5 && lane < kHalf && nm > prev);
        const int ia = asc ? __ffs(asc) - 1 : 1;
        const double v = __shfl_sync(0xffffffffu, nm, ia - 1);
        if (lane == 0) out[p] = __double2float_rn(asc ? v : 0.0);
        __syncwarp();
    }
}

}  // namespace

cudaError_t launch_local_radon(const DevGeometry& g, const Batch& b, const float* SI, float* SO, int64_t stride,
                               int max_H, int max_cols, const double* gauss, const double* taper, const double* tw64,
                               cudaStream_t st) {
    if (b.count == 0) return cudaSuccess;
    const int tiles_i = (max_H + kTI - 1) / kTI, tiles_j = (max_cols + kTJ - 1) / kTJ;
    const size_t smem = sizeof(Smem);
    cudaError_t e = cudaFuncSetAttribute(k_lradon, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_lradon<<<dim3((unsigned)(tiles_i * tiles_j), b.count), kWarps * 32, smem, st>>>(g, b, SI, SO, stride, tiles_j,
                                                                                      gauss, taper, tw64);
    return cudaGetLastError();
}

}  // namespace ske
