// Radon ray sums + ramp-filtered back-projection (kernelRADN global mode,
// src/kernelRADN.h:221-258).
//
// Per sector: p_r = sum of the valid cells of skewed row r (double, in column
// order), P = FFT(p) over H2 = 2^ceil(log2 H) points, P_i *= i/H for i <= H/2
// and 0 above, q = IFFT(P), and every valid cell of row r gets (float)Re q_r.
// The FFT is the reference's radix-2 decimation-in-frequency transform
// (helper.h:59-106) with its exact twiddle sequence, computed in binary64 with
// no fused operations, so the result is bit-identical to the reference.
//
// Three launches per batch: row sums (one warp per row), transform (one CTA per
// sector), back-projection (one thread per cell).  For sectors whose rows stay
// within their width the engine skips the back-projection (its deskew reads the
// filtered row values) and the skew (the row sums gather the skewed cells from
// the oriented input themselves), and runs sums and transform as one fused
// sector kernel (k_radon_sector, a thread-block cluster per sector).
#include <climits>

#include <cooperative_groups.h>

#include "kernels.h"

namespace ske {

namespace {

__device__ __forceinline__ int pow2_at_least(int h) {
    int p = 1;
    while (p < h) p <<= 1;
    return p;
}

// Row sums p[r] = the reference's left-to-right binary64 sum of row r's valid
// cells (kernelRADN.h:223-229); p[r] = 0 for H <= r < H2.  One warp per row.
// Every float is m * 2^e with an integer m of at most 24 bits; in units of the
// row's smallest 2^e the values are integers, and when the sum of their
// magnitudes stays below 2^53 every partial sum of the reference is exactly
// representable, i.e. its result is the exact sum, which does not depend on the
// order of additions.  The warp then forms that sum with coalesced loads and
// 64-bit integer partial sums (exponent spread <= 28, rows <= 2048 cells: no
// overflow) and returns sum * 2^emin.  Rows with a non-finite value or failing
// these conditions are added in binary64, left to right, by one lane.
//
// kGather: the cells are formed from the oriented input as the skew forms them
// (skew_gather), instead of read from the skewed grid; only for sectors whose
// rows stay within dim_i, where cell (r, j) is the skew's value at r*dim_i + j.
constexpr int kSumWarps = 8;
constexpr int kMaxSpread = 28;
constexpr int kMaxExactRow = 2048;

// x << n for 0 <= n; n >= 64 gives 0 (PTX clamps the shift amount).
__device__ __forceinline__ unsigned long long shl64(unsigned long long x, int n) {
    unsigned long long y;
    asm("shl.b64 %0, %1, %2;" : "=l"(y) : "l"(x), "r"(n));
    return y;
}

// Per-lane part of an exact row sum.  A float with biased exponent field e8
// and significand m (hidden bit included) is m * 2^(max(e8, 1) - 150).  The
// lane keeps the sums of its positive and of its negative values as integers
// in units of 2^(emin - 150), emin its smallest exponent of a nonzero value so
// far (they are shifted left when emin drops); emax is its largest exponent
// field (255 for an infinity or NaN).  Values far apart in exponent may wrap
// the integers: the spread test at the end rejects those rows.
struct ExactPart {
    unsigned long long pos = 0, neg = 0;
    int emin = INT_MAX, emax = 0;
    __device__ __forceinline__ void add(float v) {
        const unsigned u = __float_as_uint(v);
        const int e8 = (int)((u >> 23) & 0xffu);
        const unsigned m = (u & 0x7fffffu) | (e8 ? 0x800000u : 0u);
        const int ee = m ? max(e8, 1) : INT_MAX;  // zeros leave emin alone
        if (ee < emin) {
            const int sh = emin == INT_MAX ? 0 : emin - ee;
            pos = shl64(pos, sh);
            neg = shl64(neg, sh);
            emin = ee;
        }
        emax = max(emax, e8);
        const unsigned long long x = shl64(m, ee - emin);  // m = 0: shift clamps, x = 0
        const unsigned long long xn = (u >> 31) ? x : 0ull;
        neg += xn;
        pos += x - xn;
    }
    // Not an exact candidate: a non-finite value or a spread above kMaxSpread.
    __device__ __forceinline__ bool bad() const {
        return emax == 0xff || (emin != INT_MAX && emax - emin > kMaxSpread);
    }
};

template <bool kGather>
__global__ void __launch_bounds__(kSumWarps * 32)
    k_radon_sums(DevGeometry g, Batch b, const float* __restrict__ SI, int64_t stride, const float* __restrict__ orient,
                 int64_t n_cells, cd* __restrict__ P, int64_t pstride) {
    const int lane = threadIdx.x & 31;
    const int slot = blockIdx.y;
    const SectorDesc d = g.desc[b.angle[slot]];
    const int H2 = pow2_at_least(d.H);
    const float* in = SI + slot * stride;
    const float* src = orient + (int64_t)d.type * n_cells;
    const int32_t* tgt = g.target + d.col_off;
    const float* wgt = g.weight + d.col_off;
    cd* p = P + slot * pstride;
    const int nwarps = gridDim.x * kSumWarps;
    for (int r = blockIdx.x * kSumWarps + (threadIdx.x >> 5); r < H2; r += nwarps) {
        if (r >= d.H) {
            if (lane == 0) p[r] = {0.0, 0.0};
            continue;
        }
        const int f = g.first[d.row_off + r], l = g.last[d.row_off + r];
        const float* row = in + (int64_t)r * d.dim_i;
        auto cell = [&](int j) { return kGather ? skew_gather(d, tgt, wgt, src, r, j) : row[j]; };
        ExactPart a;
#pragma unroll 2
        for (int j = f + lane; j < l; j += 32) a.add(cell(j));
        const bool lane_bad = a.bad();
        int gmin = a.emin, gmax = a.emax;
        for (int o = 16; o > 0; o >>= 1) {
            gmin = min(gmin, __shfl_xor_sync(0xffffffffu, gmin, o));
            gmax = max(gmax, __shfl_xor_sync(0xffffffffu, gmax, o));
        }
        bool bad = __any_sync(0xffffffffu, lane_bad) || l - f > kMaxExactRow ||
                   (gmin != INT_MAX && gmax - gmin > kMaxSpread);  // gmax: largest field, >= any nonzero's

        double s = 0.0;
        if (!bad && gmin != INT_MAX) {
            // Units of 2^(gmin - 150): every value < 2^52, at most 2048 of them.
            const int sh = a.emin == INT_MAX ? 0 : a.emin - gmin;
            unsigned long long pos = shl64(a.pos, sh), neg = shl64(a.neg, sh);
            for (int o = 16; o > 0; o >>= 1) {
                pos += __shfl_xor_sync(0xffffffffu, pos, o);
                neg += __shfl_xor_sync(0xffffffffu, neg, o);
            }
            if (pos + neg < (1ull << 53)) {  // every partial sum exact: the exact sum
                const double scale = __longlong_as_double((long long)(gmin - 150 + 1023) << 52);
                s = __dmul_rn(__ll2double_rn((long long)(pos - neg)), scale);
            } else {
                bad = true;
            }
        }
        if (bad && lane == 0)
            for (int j = f; j < l; j++) s = __dadd_rn(s, (double)cell(j));
        if (lane == 0) p[r] = {s, 0.0};
    }
}

// In-place reference DIF FFT of x[0..n) by one CTA, then bit reversal.
// kFinite (every input finite): butterflies with the twiddle (1, 0) skip the
// multiplication, the others use cmul_finite, and with kRealIn (all imaginary
// parts zero) the first stage multiplies the real difference only.  The values
// are the reference's up to the sign of zero results (finite float-derived
// sums cannot overflow, so no infinity or NaN arises).
template <bool kFinite, bool kRealIn>
__device__ void cta_fft(cd* x, int n, const double* __restrict__ tw) {
    for (int h = n >> 1; h >= 1; h >>= 1) {
        const double* t = tw + 2 * (size_t)(n - 2 * h);
        const bool real_stage = kRealIn && h == (n >> 1);
        for (int k = threadIdx.x; k < (n >> 1); k += blockDim.x) {
            const int l = k & (h - 1);
            const int a = ((k - l) << 1) + l;
            const int bb = a + h;
            const cd xa = x[a], xb = x[bb];
            if (!kFinite) {
                x[a] = cadd(xa, xb);
                x[bb] = cmul(csub(xa, xb), cd{t[2 * l], t[2 * l + 1]});
            } else if (real_stage) {
                const double dr = __dsub_rn(xa.re, xb.re);
                x[a] = cd{__dadd_rn(xa.re, xb.re), 0.0};
                x[bb] = cd{__dmul_rn(dr, t[2 * l]), __dmul_rn(dr, t[2 * l + 1])};
            } else {
                x[a] = cadd(xa, xb);
                x[bb] = l == 0 ? csub(xa, xb) : cmul_finite(csub(xa, xb), cd{t[2 * l], t[2 * l + 1]});
            }
        }
        __syncthreads();
    }
    const unsigned bits = 31 - __clz(n);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int j = (int)bitrev((unsigned)i, bits);
        if (j > i) {
            const cd tmp = x[i];
            x[i] = x[j];
            x[j] = tmp;
        }
    }
    __syncthreads();
}

// Ramp filter: i > H/2 -> 0, else (i/H) * P_i (real scalar times complex),
// then the conjugation that starts the inverse transform (helper.h:110).
__device__ void ramp_filter(cd* x, int H, int H2) {
    for (int i = threadIdx.x; i < H2; i += blockDim.x) {
        cd v = x[i];
        if (i > H / 2) {
            v = {0.0, 0.0};
        } else {
            const double s = __ddiv_rn((double)i, (double)H);
            v = {__dmul_rn(v.re, s), __dmul_rn(v.im, s)};
        }
        x[i] = {v.re, -v.im};
    }
    __syncthreads();
}

// One CTA per sector.  Sectors with H2 <= kSmemH2 transform a copy of their
// row sums in shared memory (smem > 0), larger ones work in place in P.  The
// final division by H2 (kernelRADN.h:255) is a multiplication by the exact
// power of two 1/H2: the same correctly rounded quotient.
constexpr int kTransformThreads = 256;
constexpr int kSmemH2 = 8192;

__global__ void __launch_bounds__(kTransformThreads)
    k_radon_transform(DevGeometry g, Batch b, cd* __restrict__ P, int64_t pstride,
                      const double* __restrict__ twiddles, const int64_t* __restrict__ tw_off, int smem) {
    extern __shared__ cd xs[];
    const int slot = blockIdx.x;
    const SectorDesc d = g.desc[b.angle[slot]];
    const int H = d.H;
    const int H2 = pow2_at_least(H);
    cd* p = P + slot * pstride;
    cd* x = smem ? xs : p;
    const double* tw = twiddles + tw_off[31 - __clz(H2)];
    int bad = 0;
    for (int i = threadIdx.x; i < H2; i += blockDim.x) {
        const cd v = p[i];
        if (smem) x[i] = v;
        bad |= !isfinite(v.re);
    }
    if (!__syncthreads_or(bad)) {
        cta_fft<true, true>(x, H2, tw);
        ramp_filter(x, H, H2);
        cta_fft<true, false>(x, H2, tw);
    } else {
        cta_fft<false, false>(x, H2, tw);
        ramp_filter(x, H, H2);
        cta_fft<false, false>(x, H2, tw);
    }
    // conj, then divide by H2: only the real part is used (kernelRADN.h:255).
    const double inv = 1.0 / (double)H2;
    for (int i = threadIdx.x; i < H; i += blockDim.x) p[i].re = __dmul_rn(x[i].re, inv);
}

// The whole Radon operator of a sector whose rows stay within its width, in
// one launch: a cluster of kClusterCtas CTAs per sector.  Every CTA of the
// cluster forms exact row sums (as k_radon_sums, gathering the skewed cells
// from the oriented input) for its share of the rows and stores them straight
// into the leader CTA's shared memory (distributed shared memory); after the
// cluster barrier the leader applies the transform, ramp filter and inverse
// transform in place (as k_radon_transform) and writes the filtered row values
// q to P, which the deskew reads.  The other CTAs exit at the barrier, so
// their SM slots take other sectors' sums while the leaders run the binary64
// transforms.  Bit-identical to the three-launch path.
constexpr int kClusterCtas = 8;

__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kTransformThreads, 6)
    k_radon_sector(DevGeometry g, Batch b, const float* __restrict__ orient, int64_t n_cells, cd* __restrict__ P,
                   int64_t pstride, const double* __restrict__ twiddles, const int64_t* __restrict__ tw_off) {
    namespace cg = cooperative_groups;
    extern __shared__ cd xs[];
    cg::cluster_group cluster = cg::this_cluster();
    const unsigned rank = cluster.block_rank();
    const int lane = threadIdx.x & 31;
    const int slot = blockIdx.y;
    const SectorDesc d = g.desc[b.angle[slot]];
    const int H = d.H;
    const int H2 = pow2_at_least(H);
    const float* src = orient + (int64_t)d.type * n_cells;
    const int32_t* tgt = g.target + d.col_off;
    const float* wgt = g.weight + d.col_off;
    cd* x0 = cluster.map_shared_rank(xs, 0);  // the leader's buffer
    constexpr int kWarps = kTransformThreads / 32;
    for (int r = rank * kWarps + (threadIdx.x >> 5); r < H2; r += kClusterCtas * kWarps) {
        if (r >= H) {
            if (lane == 0) x0[r] = {0.0, 0.0};
            continue;
        }
        const int f = g.first[d.row_off + r], l = g.last[d.row_off + r];
        ExactPart a;
#pragma unroll 2
        for (int j = f + lane; j < l; j += 32) a.add(skew_gather(d, tgt, wgt, src, r, j));
        const bool lane_bad = a.bad();
        int gmin = a.emin, gmax = a.emax;
        for (int o = 16; o > 0; o >>= 1) {
            gmin = min(gmin, __shfl_xor_sync(0xffffffffu, gmin, o));
            gmax = max(gmax, __shfl_xor_sync(0xffffffffu, gmax, o));
        }
        bool bad = __any_sync(0xffffffffu, lane_bad) || l - f > kMaxExactRow ||
                   (gmin != INT_MAX && gmax - gmin > kMaxSpread);
        double s = 0.0;
        if (!bad && gmin != INT_MAX) {
            const int sh = a.emin == INT_MAX ? 0 : a.emin - gmin;
            unsigned long long pos = shl64(a.pos, sh), neg = shl64(a.neg, sh);
            for (int o = 16; o > 0; o >>= 1) {
                pos += __shfl_xor_sync(0xffffffffu, pos, o);
                neg += __shfl_xor_sync(0xffffffffu, neg, o);
            }
            if (pos + neg < (1ull << 53)) {
                const double scale = __longlong_as_double((long long)(gmin - 150 + 1023) << 52);
                s = __dmul_rn(__ll2double_rn((long long)(pos - neg)), scale);
            } else {
                bad = true;
            }
        }
        if (bad && lane == 0)
            for (int j = f; j < l; j++) s = __dadd_rn(s, (double)skew_gather(d, tgt, wgt, src, r, j));
        if (lane == 0) x0[r] = {s, 0.0};
    }
    cluster.sync();  // every row sum is in the leader's shared memory
    if (rank != 0) return;
    const double* tw = twiddles + tw_off[31 - __clz(H2)];
    int bad = 0;
    for (int i = threadIdx.x; i < H2; i += blockDim.x) bad |= !isfinite(xs[i].re);
    if (!__syncthreads_or(bad)) {
        cta_fft<true, true>(xs, H2, tw);
        ramp_filter(xs, H, H2);
        cta_fft<true, false>(xs, H2, tw);
    } else {
        cta_fft<false, false>(xs, H2, tw);
        ramp_filter(xs, H, H2);
        cta_fft<false, false>(xs, H2, tw);
    }
    cd* p = P + slot * pstride;
    const double inv = 1.0 / (double)H2;
    for (int i = threadIdx.x; i < H; i += blockDim.x) p[i].re = __dmul_rn(xs[i].re, inv);
}

// ---- float32 mode (SKE_FLAG_RADON_F32) -------------------------------------
// The same operator on the FP32 pipes: row sums in float (a warp per row,
// lanes over columns, a shuffle tree), the radix-2 DIF transform, ramp filter
// and inverse transform in float in shared memory (twiddles rounded from the
// binary64 table), the filtered row values written to P as doubles for the
// deskew or back-projection.  Values differ from the reference's binary64 in
// their low bits (the sums' order and float rounding); the relative error of
// the output is measured and stated (tests/test_gpu_parity.py).
template <bool kGather>
__global__ void __launch_bounds__(kSumWarps * 32)
    k_radon_sums_f32(DevGeometry g, Batch b, const float* __restrict__ SI, int64_t stride,
                     const float* __restrict__ orient, int64_t n_cells, cd* __restrict__ P, int64_t pstride) {
    const int lane = threadIdx.x & 31;
    const int slot = blockIdx.y;
    const SectorDesc d = g.desc[b.angle[slot]];
    const int H2 = pow2_at_least(d.H);
    const float* in = SI + slot * stride;
    const float* src = orient + (int64_t)d.type * n_cells;
    const int32_t* tgt = g.target + d.col_off;
    const float* wgt = g.weight + d.col_off;
    cd* p = P + slot * pstride;
    const int nwarps = gridDim.x * kSumWarps;
    for (int r = blockIdx.x * kSumWarps + (threadIdx.x >> 5); r < H2; r += nwarps) {
        if (r >= d.H) {
            if (lane == 0) p[r] = {0.0, 0.0};
            continue;
        }
        const int f = g.first[d.row_off + r], l = g.last[d.row_off + r];
        const float* row = in + (int64_t)r * d.dim_i;
        float acc = 0.0f;
        for (int j = f + lane; j < l; j += 32) acc += kGather ? skew_gather(d, tgt, wgt, src, r, j) : row[j];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) p[r] = {(double)acc, 0.0};
    }
}

__device__ void cta_fft_f32(float2* x, int n, const double* __restrict__ tw) {
    for (int h = n >> 1; h >= 1; h >>= 1) {
        const double* t = tw + 2 * (size_t)(n - 2 * h);
        for (int k = threadIdx.x; k < (n >> 1); k += blockDim.x) {
            const int l = k & (h - 1);
            const int a = ((k - l) << 1) + l;
            const int bb = a + h;
            const float2 xa = x[a], xb = x[bb];
            const float dr = xa.x - xb.x, di = xa.y - xb.y;
            const float c = (float)t[2 * l], sn = (float)t[2 * l + 1];
            x[a] = make_float2(xa.x + xb.x, xa.y + xb.y);
            x[bb] = make_float2(dr * c - di * sn, dr * sn + di * c);
        }
        __syncthreads();
    }
    const unsigned bits = 31 - __clz(n);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int j = (int)bitrev((unsigned)i, bits);
        if (j > i) {
            const float2 tmp = x[i];
            x[i] = x[j];
            x[j] = tmp;
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kTransformThreads)
    k_radon_transform_f32(DevGeometry g, Batch b, cd* __restrict__ P, int64_t pstride,
                          const double* __restrict__ twiddles, const int64_t* __restrict__ tw_off) {
    extern __shared__ float2 xf[];
    const int slot = blockIdx.x;
    const SectorDesc d = g.desc[b.angle[slot]];
    const int H = d.H;
    const int H2 = pow2_at_least(H);
    cd* p = P + slot * pstride;
    const double* tw = twiddles + tw_off[31 - __clz(H2)];
    for (int i = threadIdx.x; i < H2; i += blockDim.x) xf[i] = make_float2((float)p[i].re, 0.0f);
    __syncthreads();
    cta_fft_f32(xf, H2, tw);
    for (int i = threadIdx.x; i < H2; i += blockDim.x) {  // ramp filter, then the conjugation
        float2 v = xf[i];
        if (i > H / 2) {
            v = make_float2(0.0f, 0.0f);
        } else {
            const float sc = __fdiv_rn((float)i, (float)H);
            v = make_float2(v.x * sc, v.y * sc);
        }
        xf[i] = make_float2(v.x, -v.y);
    }
    __syncthreads();
    cta_fft_f32(xf, H2, tw);
    const float inv = 1.0f / (float)H2;
    for (int i = threadIdx.x; i < H; i += blockDim.x) p[i].re = (double)(xf[i].x * inv);
}

__global__ void k_radon_backproject(DevGeometry g, Batch b, const cd* __restrict__ P, int64_t pstride,
                                    float* __restrict__ SO, int64_t stride, int64_t len) {
    const int slot = blockIdx.y;
    const SectorDesc d = g.desc[b.angle[slot]];
    const int32_t* first = g.first + d.row_off;
    const int32_t* last = g.last + d.row_off;
    const cd* q = P + slot * pstride;
    float* out = SO + slot * stride;
    for (int64_t p = gtid(); p < len; p += gstride()) {
        // Rows that can cover p, in increasing order (`+=` in row order).
        int rhi = (int)(p / d.dim_i);
        if (rhi > d.H - 1) rhi = d.H - 1;
        int64_t lo_row = (p - d.diml) / d.dim_i;
        int rlo = lo_row < 0 ? 0 : (int)lo_row;
        float v = 0.0f;
        for (int r = rlo; r <= rhi; r++) {
            const int64_t base = (int64_t)r * d.dim_i;
            if (p >= base + first[r] && p < base + last[r]) v = (float)__dadd_rn((double)v, q[r].re);
        }
        out[p] = v;
    }
}

}  // namespace

// 0: the fused sector kernel where it applies; 1 (default): row sums and
// transform as two launches, measured faster (radon_select).
int g_radon_path = 1;

int radon_launches(bool rows_only, int max_H2, bool f32) {
    if (f32 && max_H2 <= kSmemH2) return rows_only ? 2 : 3;
    return rows_only ? (max_H2 <= kSmemH2 && g_radon_path == 0 ? 1 : 2) : 3;
}

int radon_select(int path) {
    if (path != 0 && path != 1) return -1;
    g_radon_path = path;
    return 0;
}

cudaError_t launch_radon(const DevGeometry& g, const Batch& b, const float* SI, float* SO, int64_t stride,
                         int64_t len, double* P, int64_t pstride, const double* twiddles, const int64_t* tw_off,
                         int max_H2, cudaStream_t st, bool backproject, const float* orient, int64_t n_cells,
                         bool f32) {
    if (orient && backproject) return cudaErrorInvalidValue;  // the gathered cells are not kept for SO
    cd* Pc = reinterpret_cast<cd*>(P);
    if (f32 && max_H2 <= kSmemH2) {
        dim3 g1((max_H2 + kSumWarps - 1) / kSumWarps, b.count);
        if (orient)
            k_radon_sums_f32<true><<<g1, kSumWarps * 32, 0, st>>>(g, b, SI, stride, orient, n_cells, Pc, pstride);
        else
            k_radon_sums_f32<false><<<g1, kSumWarps * 32, 0, st>>>(g, b, SI, stride, orient, n_cells, Pc, pstride);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        const int smem = max_H2 * (int)sizeof(float2);
        if (smem > 48 * 1024) {
            e = cudaFuncSetAttribute(k_radon_transform_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
        }
        k_radon_transform_f32<<<b.count, kTransformThreads, smem, st>>>(g, b, Pc, pstride, twiddles, tw_off);
        e = cudaGetLastError();
        if (e != cudaSuccess || !backproject) return e;
        int64_t blocks = (len + 255) / 256;
        if (blocks > 4096) blocks = 4096;
        k_radon_backproject<<<dim3((unsigned)blocks, b.count), 256, 0, st>>>(g, b, Pc, pstride, SO, stride, len);
        return cudaGetLastError();
    }
    if (orient && max_H2 <= kSmemH2 && g_radon_path == 0) {  // one fused launch: a cluster per sector
        const int smem = max_H2 * (int)sizeof(cd);
        cudaError_t e = cudaSuccess;
        if (smem > 48 * 1024) e = cudaFuncSetAttribute(k_radon_sector, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        k_radon_sector<<<dim3(kClusterCtas, b.count), kTransformThreads, smem, st>>>(g, b, orient, n_cells, Pc, pstride,
                                                                                   twiddles, tw_off);
        return cudaGetLastError();
    }
    dim3 g1((max_H2 + kSumWarps - 1) / kSumWarps, b.count);
    if (orient)
        k_radon_sums<true><<<g1, kSumWarps * 32, 0, st>>>(g, b, SI, stride, orient, n_cells, Pc, pstride);
    else
        k_radon_sums<false><<<g1, kSumWarps * 32, 0, st>>>(g, b, SI, stride, orient, n_cells, Pc, pstride);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int smem = max_H2 <= kSmemH2 ? max_H2 * (int)sizeof(cd) : 0;
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(k_radon_transform, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
    }
    k_radon_transform<<<b.count, kTransformThreads, smem, st>>>(g, b, Pc, pstride, twiddles, tw_off, smem);
    e = cudaGetLastError();
    if (e != cudaSuccess || !backproject) return e;
    int64_t blocks = (len + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_radon_backproject<<<dim3((unsigned)blocks, b.count), 256, 0, st>>>(g, b, Pc, pstride, SO, stride, len);
    return cudaGetLastError();
}

}  // namespace ske
