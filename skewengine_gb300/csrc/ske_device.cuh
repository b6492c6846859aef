// Device helpers shared by the engine's CUDA kernels.
//
// Bit-exactness: the reference's arithmetic is plain IEEE binary32/binary64 with
// round-to-nearest and no fused multiply-add (its x86-64 host build).  Every
// value the kernels must reproduce is therefore computed with the explicit
// _rn intrinsics below, which the compiler neither contracts nor reorders.
#pragma once

#include <cstdint>

#include "ske_internal.h"

namespace ske {

// Device pointers to one grid's geometry tables (built by build_geometry).
struct DevGeometry {
    const SectorDesc* desc;
    const int32_t* target;
    const float* weight;
    const int32_t* first;
    const int32_t* last;
};

// A batch of sectors processed by one launch: entries index DevGeometry::desc
// and the batch's per-sector buffers (slot s owns [s*stride, (s+1)*stride)).
constexpr int kMaxBatch = 180;
struct Batch {
    int count;
    int angle[kMaxBatch];
};

// Skewed input value of cell (r, c), r < H: the two source contributions of the
// reference scatter (skewEngine.cuh:615-620).  Source row r-t-1 contributes
// w*x (the reference adds it first: lower loop index), row r-t contributes
// (1-w)*x, onto a cell that starts at 0.
__device__ __forceinline__ float skew_gather(const SectorDesc& d, const int32_t* __restrict__ tgt,
                                             const float* __restrict__ wgt, const float* __restrict__ src,
                                             int r, int c) {
    const int t = tgt[c];
    const float w = wgt[c];
    const int i0 = r - t - 1;
    // Branch-free: both loads predicated, the additions selected.
    const bool v0 = (unsigned)i0 < (unsigned)d.dim_o, v1 = (unsigned)(i0 + 1) < (unsigned)d.dim_o;
    const float* p0 = src + ((int64_t)i0 * d.dim_i + c);
    const float a = v0 ? p0[0] : 0.0f;
    const float b = v1 ? p0[d.dim_i] : 0.0f;
    float acc = 0.0f;
    acc = v0 ? __fadd_rn(acc, __fmul_rn(w, a)) : acc;
    acc = v1 ? __fadd_rn(acc, __fmul_rn(__fsub_rn(1.0f, w), b)) : acc;
    return acc;
}

// The last (largest) skewed row whose valid range [r*dim_i+first, r*dim_i+last)
// covers flat index p, or -1.  Rows can overrun their own width when dim_l >
// dim_i (non-square grids, transposed sectors: skewEngine.cuh:581 initialises
// last[] with dim_l); the reference then writes such cells from several rows in
// row order, so the last covering row's value is the one that stays.
__device__ __forceinline__ int owner_row(const SectorDesc& d, const int32_t* __restrict__ first,
                                         const int32_t* __restrict__ last, int64_t p) {
    int r = (int)(p / d.dim_i);
    if (r > d.H - 1) r = d.H - 1;
    for (; r >= 0; r--) {
        const int64_t base = (int64_t)r * d.dim_i;
        if (base + d.diml <= p) break;  // no earlier row can reach p either
        if (p >= base + first[r] && p < base + last[r]) return r;
    }
    return -1;
}

// Grid-stride helpers.
__device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int64_t gstride() { return (int64_t)gridDim.x * blockDim.x; }

// Complex double, multiplied the way GCC's std::complex<double> does at -O3
// without -ffast-math: (ac - bd, ad + bc), and when both parts come out NaN the
// infinity recovery of ISO C99 Annex G.5.1 (_Cmultd), which libgcc's __muldc3
// implements.
struct cd {
    double re, im;
};

__device__ __forceinline__ cd cadd(cd a, cd b) { return {__dadd_rn(a.re, b.re), __dadd_rn(a.im, b.im)}; }
__device__ __forceinline__ cd csub(cd a, cd b) { return {__dsub_rn(a.re, b.re), __dsub_rn(a.im, b.im)}; }

static __device__ __noinline__ cd cmul_recover(double a, double b, double c, double d) {
    const double ac = __dmul_rn(a, c), bd = __dmul_rn(b, d), ad = __dmul_rn(a, d), bc = __dmul_rn(b, c);
    bool recalc = false;
    if (isinf(a) || isinf(b)) {
        a = copysign(isinf(a) ? 1.0 : 0.0, a);
        b = copysign(isinf(b) ? 1.0 : 0.0, b);
        if (isnan(c)) c = copysign(0.0, c);
        if (isnan(d)) d = copysign(0.0, d);
        recalc = true;
    }
    if (isinf(c) || isinf(d)) {
        c = copysign(isinf(c) ? 1.0 : 0.0, c);
        d = copysign(isinf(d) ? 1.0 : 0.0, d);
        if (isnan(a)) a = copysign(0.0, a);
        if (isnan(b)) b = copysign(0.0, b);
        recalc = true;
    }
    if (!recalc && (isinf(ac) || isinf(bd) || isinf(ad) || isinf(bc))) {
        if (isnan(a)) a = copysign(0.0, a);
        if (isnan(b)) b = copysign(0.0, b);
        if (isnan(c)) c = copysign(0.0, c);
        if (isnan(d)) d = copysign(0.0, d);
        recalc = true;
    }
    if (recalc) {
        const double inf = __longlong_as_double(0x7ff0000000000000LL);
        return {__dmul_rn(inf, __dsub_rn(__dmul_rn(a, c), __dmul_rn(b, d))),
                __dmul_rn(inf, __dadd_rn(__dmul_rn(a, d), __dmul_rn(b, c)))};
    }
    return {__dsub_rn(ac, bd), __dadd_rn(ad, bc)};
}

__device__ __forceinline__ cd cmul(cd x, cd y) {
    const double re = __dsub_rn(__dmul_rn(x.re, y.re), __dmul_rn(x.im, y.im));
    const double im = __dadd_rn(__dmul_rn(x.re, y.im), __dmul_rn(x.im, y.re));
    if (isnan(re) && isnan(im)) return cmul_recover(x.re, x.im, y.re, y.im);
    return {re, im};
}

// 32-bit bit reversal of the low `bits` bits.
__device__ __forceinline__ unsigned bitrev(unsigned v, unsigned bits) {
    return bits ? (__brev(v) >> (32 - bits)) : 0u;
}

// helper::fft (helper.h:59-106) of x[0..n) (n <= 64, a power of two) by one
// warp, in place: radix-2 decimation in frequency, one butterfly per lane per
// stage, with the reference's twiddle sequence tw (fft_twiddles: for the stage
// of half-span h, entries 2*(n - 2h) .. give T^l as (re, im)), then the bit
// reversal.  No scaling.
__device__ __forceinline__ void warp_fft(cd* x, int n, const double* __restrict__ tw, int lane) {
    for (int h = n >> 1; h >= 1; h >>= 1) {
        const double* t = tw + 2 * (n - 2 * h);
        for (int k = lane; k < (n >> 1); k += 32) {
            const int l = k & (h - 1);
            const int a = (k / h) * 2 * h + l;
            const int bb = a + h;
            const cd xa = x[a], xb = x[bb];
            x[a] = cadd(xa, xb);
            x[bb] = cmul(csub(xa, xb), cd{t[2 * l], t[2 * l + 1]});
        }
        __syncwarp();
    }
    const unsigned bits = 31 - __clz(n);
    for (int i = lane; i < n; i += 32) {
        const int j = (int)bitrev((unsigned)i, bits);
        if (j > i) {
            const cd tmp = x[i];
            x[i] = x[j];
            x[j] = tmp;
        }
    }
    __syncwarp();
}

// The product of cmul without its infinity recovery, for operands known to be
// finite with finite products.
__device__ __forceinline__ cd cmul_finite(cd x, cd y) {
    return {__dsub_rn(__dmul_rn(x.re, y.re), __dmul_rn(x.im, y.im)),
            __dadd_rn(__dmul_rn(x.re, y.im), __dmul_rn(x.im, y.re))};
}

// Outputs a warp_fft_real caller reads: all of them, X_k for k < n/2, or only
// Re X_k for k < n/2.  The pruned variants leave out work whose results are
// never read; the values they do produce are the same.
enum FftKeep { kKeepAll = 0, kKeepLow = 1, kKeepLowRe = 2 };

// warp_fft for finite input whose imaginary parts are all zero (n = 64 or 32),
// with the same values as warp_fft up to the sign of zero results:
//  * first stage: the operands are real, so (a - b) * T is (d*T.re, d*T.im)
//    (the reference's extra terms are products with an exact zero);
//  * last stage: its only twiddle is exactly (1, 0), so x[b] = a - b;
//  * other stages: cmul_finite.  Finite float-derived values stay far from
//    overflow, so no NaN arises and the reference's infinity recovery never
//    applies.  Callers use it only when every
// input is finite; results that feed squared magnitudes or comparisons of
// magnitudes are then bit-identical to warp_fft's.
// kKeep: the last stage's butterfly (2k, 2k+1) produces X_r and X_{r+n/2}
// (r = bitrev(2k)), so kKeepLow forms only the sums; kKeepLowRe also forms
// only the real parts in the last two stages.  With kZeroHigh the upper half
// of the input is known to be zero: the first stage's sums are the lower
// half itself (up to zero signs).
template <int kKeep = kKeepAll, bool kZeroHigh = false>
__device__ __forceinline__ void warp_fft_real(cd* x, int n, const double* __restrict__ tw, int lane) {
    {  // first stage, h = n/2: butterfly k pairs k and k + n/2 with twiddle T^k
        const int h = n >> 1;
        const double* t = tw;  // stage of half-span n/2 starts at entry 0
        for (int k = lane; k < h; k += 32) {
            const double xa = x[k].re;
            if (kZeroHigh) {
                x[k] = cd{xa, 0.0};
                x[k + h] = cd{__dmul_rn(xa, t[2 * k]), __dmul_rn(xa, t[2 * k + 1])};
            } else {
                const double xb = x[k + h].re;
                const double d = __dsub_rn(xa, xb);
                x[k] = cd{__dadd_rn(xa, xb), 0.0};
                x[k + h] = cd{__dmul_rn(d, t[2 * k]), __dmul_rn(d, t[2 * k + 1])};
            }
        }
        __syncwarp();
    }
    for (int h = n >> 2; h >= 2; h >>= 1) {
        const double* t = tw + 2 * (n - 2 * h);
        for (int k = lane; k < (n >> 1); k += 32) {
            const int l = k & (h - 1);
            const int a = (k / h) * 2 * h + l;
            const int bb = a + h;
            const cd xa = x[a], xb = x[bb];
            if (kKeep == kKeepLowRe && h == 2) {
                // Only the real parts feed the last stage's real sums.
                const cd dd = csub(xa, xb);
                x[a].re = __dadd_rn(xa.re, xb.re);
                x[bb].re = __dsub_rn(__dmul_rn(dd.re, t[2 * l]), __dmul_rn(dd.im, t[2 * l + 1]));
            } else {
                x[a] = cadd(xa, xb);
                x[bb] = cmul_finite(csub(xa, xb), cd{t[2 * l], t[2 * l + 1]});
            }
        }
        __syncwarp();
    }
    for (int k = lane; k < (n >> 1); k += 32) {  // last stage, h = 1, twiddle (1, 0)
        const cd xa = x[2 * k], xb = x[2 * k + 1];
        if (kKeep == kKeepLowRe) {
            x[2 * k].re = __dadd_rn(xa.re, xb.re);
        } else {
            x[2 * k] = cadd(xa, xb);
            if (kKeep == kKeepAll) x[2 * k + 1] = csub(xa, xb);
        }
    }
    __syncwarp();
    const unsigned bits = 31 - __clz(n);
    for (int i = lane; i < n; i += 32) {
        const int j = (int)bitrev((unsigned)i, bits);
        if (j > i) {
            const cd tmp = x[i];
            x[i] = x[j];
            x[j] = tmp;
        }
    }
    __syncwarp();
}

}  // namespace ske
