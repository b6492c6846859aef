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
// Three launches per batch: row sums (one thread per row, sequential double
// adds), transform (one CTA per sector), back-projection (one thread per cell).
#include "kernels.h"

namespace ske {

namespace {

__device__ __forceinline__ int pow2_at_least(int h) {
    int p = 1;
    while (p < h) p <<= 1;
    return p;
}

__global__ void k_radon_sums(DevGeometry g, Batch b, const float* __restrict__ SI, int64_t stride,
                             cd* __restrict__ P, int64_t pstride) {
    const int slot = blockIdx.y;
    const SectorDesc d = g.desc[b.angle[slot]];
    const int H2 = pow2_at_least(d.H);
    const float* in = SI + slot * stride;
    cd* p = P + slot * pstride;
    for (int64_t r = gtid(); r < H2; r += gstride()) {
        double s = 0.0;
        if (r < d.H) {
            const int f = g.first[d.row_off + r], l = g.last[d.row_off + r];
            const float* row = in + r * d.dim_i;
            for (int j = f; j < l; j++) s = __dadd_rn(s, (double)row[j]);
        }
        p[r] = {s, 0.0};
    }
}

// In-place reference DIF FFT of x[0..n) by one CTA, then bit reversal.
__device__ void cta_fft(cd* x, int n, const double* __restrict__ tw) {
    for (int h = n >> 1; h >= 1; h >>= 1) {
        const double* t = tw + 2 * (size_t)(n - 2 * h);
        for (int k = threadIdx.x; k < (n >> 1); k += blockDim.x) {
            const int l = k & (h - 1);
            const int a = (k / h) * 2 * h + l;
            const int bb = a + h;
            const cd xa = x[a], xb = x[bb];
            x[a] = cadd(xa, xb);
            x[bb] = cmul(csub(xa, xb), cd{t[2 * l], t[2 * l + 1]});
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

__global__ void k_radon_transform(DevGeometry g, Batch b, cd* __restrict__ P, int64_t pstride,
                                  const double* __restrict__ twiddles, const int64_t* __restrict__ tw_off) {
    const int slot = blockIdx.x;
    const SectorDesc d = g.desc[b.angle[slot]];
    const int H = d.H;
    const int H2 = pow2_at_least(H);
    cd* x = P + slot * pstride;
    const double* tw = twiddles + tw_off[31 - __clz(H2)];
    cta_fft(x, H2, tw);
    // Ramp filter: i > H/2 -> 0, else (i/H) * P_i (real scalar times complex),
    // then the conjugation that starts the inverse transform (helper.h:110).
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
    cta_fft(x, H2, tw);
    // conj, then divide by H2: only the real part is used (kernelRADN.h:255).
    for (int i = threadIdx.x; i < H; i += blockDim.x) x[i].re = __ddiv_rn(x[i].re, (double)H2);
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

cudaError_t launch_radon(const DevGeometry& g, const Batch& b, const float* SI, float* SO, int64_t stride,
                         int64_t len, double* P, int64_t pstride, const double* twiddles, const int64_t* tw_off,
                         int max_H2, cudaStream_t st, bool backproject) {
    cd* Pc = reinterpret_cast<cd*>(P);
    dim3 g1((max_H2 + 255) / 256, b.count);
    k_radon_sums<<<g1, 256, 0, st>>>(g, b, SI, stride, Pc, pstride);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_radon_transform<<<b.count, 1024, 0, st>>>(g, b, Pc, pstride, twiddles, tw_off);
    e = cudaGetLastError();
    if (e != cudaSuccess || !backproject) return e;
    int64_t blocks = (len + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_radon_backproject<<<dim3((unsigned)blocks, b.count), 256, 0, st>>>(g, b, Pc, pstride, SO, stride, len);
    return cudaGetLastError();
}

}  // namespace ske
