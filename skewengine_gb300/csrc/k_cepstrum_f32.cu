// Cepstrum blur estimation in float32, fused over the whole sector loop
// (kernelBLUR, src/kernelBLUR.h:267-302 -> lineCepstrum :153-228, with the
// max+angle deskew of skewEngine.cuh:774-785), for batches of square images.
//
// The reference computes each skewed cell's cepstrum in binary64; the engine's
// exact operator (k_cepstrum.cu) does the same and is FP64-pipe bound.  This
// mode computes the same quantities in float32 on the FP32 pipes:
//   X = FFT64(window)/8          64-sample real window as a 32-point complex
//                                FFT in registers (even/odd packing) and the
//                                real-input split;
//   l_k = log(|X_k|^2), k < 32   (CUDA's logf);
//   c_k = sum_n l_n cos(2 pi k n / 32) / sqrt(32), k < 16, folded (l_n and
//                                l_{32-n} share a cosine);
//   s_k = -min(0, c_k), the reference's peak search, output 10000 * peak.
// Rounding differs from the reference's, so an output can land in another
// 1000-wide bin where a value sits at a bin edge: the bin-mismatch rate against
// the exact operator is measured and stated, and the exact operator stays the
// parity mode.
//
// Fusion: a CTA owns a 128 x 32 tile of one orientation's accumulator of one
// image and walks that orientation's sectors in angle order.  Per sector it
// gathers the skewed rows the tile needs (the reference's skew, gathered from
// the orientation: skew_gather) as 96-cell row segments into shared memory,
// computes the cepstrum of every band cell (one thread per cell, the 64-cell
// window read from the staged segment), and max-deskews into the tile's
// registers.  The skewed input and output never reach HBM; the orientations
// (4 x N floats per image) stay L2-resident.
#include "kernels.h"

namespace ske {

namespace {

constexpr int kCRows = 128;            // accumulator tile rows
constexpr int kCBand = kCRows + 34;    // skewed rows of a tile per sector (drift <= 32 over 32 columns)
constexpr int kCSeg = 96;              // staged cells per band row: columns j0-32 .. j0+63
constexpr int kCThreads = 256;
constexpr int kCPer = kCRows / 8;      // accumulator rows per thread

// W64^k = exp(-2 pi i k / 64) as float (cos, -sin), filled on the host.
__constant__ float2 c_w64[64];

__device__ __forceinline__ void cmulf(float ar, float ai, float br, float bi, float& r, float& i) {
    r = __fsub_rn(__fmul_rn(ar, br), __fmul_rn(ai, bi));
    i = __fadd_rn(__fmul_rn(ar, bi), __fmul_rn(ai, br));
}

// 32-point complex FFT in registers, radix-2 decimation in time: input in
// bit-reversed order, output in natural order.
__device__ __forceinline__ void fft32(float (&re)[32], float (&im)[32]) {
#pragma unroll
    for (int span = 1; span < 32; span <<= 1) {
#pragma unroll
        for (int start = 0; start < 32; start += 2 * span) {
#pragma unroll
            for (int k = 0; k < span; k++) {
                const int a = start + k, b = a + span;
                const float2 w = c_w64[k * (32 / span)];  // W_{2 span}^k = W64^(k * 64 / (2 span))
                float tr, ti;
                if (k == 0) {
                    tr = re[b];
                    ti = im[b];
                } else {
                    cmulf(re[b], im[b], w.x, w.y, tr, ti);
                }
                re[b] = __fsub_rn(re[a], tr);
                im[b] = __fsub_rn(im[a], ti);
                re[a] = __fadd_rn(re[a], tr);
                im[a] = __fadd_rn(im[a], ti);
            }
        }
    }
}

__device__ __forceinline__ constexpr int brev5(int v) {
    return ((v & 1) << 4) | ((v & 2) << 2) | (v & 4) | ((v & 8) >> 2) | ((v & 16) >> 4);
}

// Cepstrum peak of the 64-sample window w[0..63] (zeros outside the row), as
// lineCepstrum computes it, in float32.
__device__ __forceinline__ float cepstrum_f32(const float* __restrict__ w) {
    float re[32], im[32];
#pragma unroll
    for (int n = 0; n < 32; n++) {  // z_n = w[2n] + i w[2n+1], stored bit-reversed
        re[brev5(n)] = w[2 * n];
        im[brev5(n)] = w[2 * n + 1];
    }
    fft32(re, im);
    // X_k = E_k + W64^k O_k, E = (Z_k + conj Z_{32-k}) / 2, O = -i (Z_k - conj Z_{32-k}) / 2;
    // l_k = log(|X_k / 8|^2).
    float l[32];
#pragma unroll
    for (int k = 0; k < 32; k++) {
        const int m = (32 - k) & 31;
        const float er = __fmul_rn(0.5f, __fadd_rn(re[k], re[m]));
        const float ei = __fmul_rn(0.5f, __fsub_rn(im[k], im[m]));
        const float orr = __fmul_rn(0.5f, __fadd_rn(im[k], im[m]));
        const float oi = __fmul_rn(-0.5f, __fsub_rn(re[k], re[m]));
        float xr, xi;
        if (k == 0) {
            xr = __fadd_rn(er, orr);
            xi = __fadd_rn(ei, oi);
        } else {
            const float2 t = c_w64[k];
            float pr, pi;
            cmulf(orr, oi, t.x, t.y, pr, pi);
            xr = __fadd_rn(er, pr);
            xi = __fadd_rn(ei, pi);
        }
        xr = __fmul_rn(xr, 0.125f);
        xi = __fmul_rn(xi, 0.125f);
        l[k] = logf(__fadd_rn(__fmul_rn(xr, xr), __fmul_rn(xi, xi)));
    }
    // c_k = (l_0 + (-1)^k l_16 + sum_{n=1}^{15} (l_n + l_{32-n}) cos(2 pi k n / 32)) / sqrt(32)
    float e[16];
#pragma unroll
    for (int n = 1; n < 16; n++) e[n] = __fadd_rn(l[n], l[32 - n]);
    const float inv = 0.17677669529663687f;  // 1 / sqrt(32)
    float s[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        float acc = (k & 1) ? __fsub_rn(l[0], l[16]) : __fadd_rn(l[0], l[16]);
#pragma unroll
        for (int n = 1; n < 16; n++) acc = __fmaf_rn(e[n], c_w64[(2 * k * n) & 63].x, acc);
        const float c = __fmul_rn(acc, inv);
        s[k] = c < 0.0f ? -c : -0.0f;  // -std::min(0, c)
    }
    // getBlurParameter2 (kernelBLUR.h:88-110): from index 5 skip the
    // non-ascending head; the peak is the sample before the first ascent or any
    // larger sample after the ascending one.
    float best = 0.0f;
    int asc = 16;
#pragma unroll
    for (int i = 15; i >= 5; i--)
        if (s[i] > s[i - 1]) asc = i;
    if (asc < 16) {
#pragma unroll
        for (int i = 4; i < 16; i++) {
            if (i == asc - 1) best = s[i];
        }
#pragma unroll
        for (int i = 6; i < 16; i++)
            if (i > asc && s[i] > best) best = s[i];
    }
    return __fmul_rn(best, 10000.0f);
}

// One launch: blockIdx.y = image; blockIdx.x = (type, tile row, tile column).
__global__ void __launch_bounds__(kCThreads, 2)
    k_cepstrum_fused(BatchTables T, DevGeometry g, TypeLists tl, int dim, int tiles_x, int tiles_y) {
    __shared__ float seg[kCBand][kCSeg];
    __shared__ float val[kCBand][32];
    const int per_type = tiles_x * tiles_y;
    const int t = blockIdx.x / per_type;
    const int tile = blockIdx.x - t * per_type;
    const int cnt = tl.count[t];
    if (cnt == 0) return;
    const BatchGrid& G = T.grids[blockIdx.y];
    const int64_t n = G.n;
    const int j0 = (tile % tiles_x) * 32, i0 = (tile / tiles_x) * kCRows;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int j = j0 + tx;
    const bool col_ok = j < dim;
    const int jlast = min(j0 + 32, dim) - 1;
    const int i_end = min(i0 + kCRows, dim);
    const int ib = ty * kCPer;
    const int nv = min(kCPer, i_end - i0 - ib);
    float* A = G.acc + t * n;
    const float* src = G.orient + t * n;
    float o[kCPer];
#pragma unroll
    for (int k = 0; k < kCPer; k++) {
        const int i = i0 + ib + k;
        o[k] = (col_ok && i < i_end) ? A[(int64_t)i * dim + j] : 0.0f;
    }
    for (int q = 0; q < cnt; q++) {
        const SectorDesc d = g.desc[tl.angle[t][q]];
        const int32_t* tg = g.target + d.col_off;
        const float* wg = g.weight + d.col_off;
        const int32_t* rfirst = g.first + d.row_off;
        const int32_t* rlast = g.last + d.row_off;
        const int tmin = tg[j0], tmax = tg[jlast];
        const int r0 = i0 + tmin;
        const int nrows = (i_end - i0) + 1 + (tmax - tmin);  // <= kCBand for square grids
        // Stage the band's row segments (skewed cells gathered from the orientation).
        for (int idx = threadIdx.x; idx < nrows * kCSeg; idx += kCThreads) {
            const int rr = idx / kCSeg, u = idx - rr * kCSeg;
            const int r = r0 + rr, x = j0 - 32 + u;
            float v = 0.0f;
            if (r < d.H && x >= rfirst[r] && x < rlast[r]) v = skew_gather(d, tg, wg, src, r, x);
            seg[rr][u] = v;
        }
        __syncthreads();
        // Cepstrum of every valid band cell: warp = band row, lane = column.
        for (int rr = ty; rr < nrows; rr += kCThreads / 32) {
            const int r = r0 + rr;
            float v = 0.0f;
            if (r < d.H && j >= rfirst[r] && j < rlast[r]) v = cepstrum_f32(&seg[rr][tx]);
            val[rr][tx] = v;
        }
        __syncthreads();
        if (col_ok && nv > 0) {
            const int off = tg[j] - tmin;
#pragma unroll
            for (int k = 0; k < kCPer; k++) {
                if (k >= nv) continue;
                const float lo = val[ib + k + off][tx], hi = val[ib + k + 1 + off][tx];
                const float m = (lo < hi) ? hi : lo;  // std::max(lo, hi)
                const float v = (o[k] < m) ? m : o[k];
                // a + 1000*(int)(v/1000): the low decimal digits carry the angle.
                o[k] = __int2float_rn(d.angle + 1000 * __float2int_rz(__fdiv_rn(v, 1000.0f)));
            }
        }
        __syncthreads();  // seg and val are rewritten for the next sector
    }
    if (!col_ok) return;
#pragma unroll
    for (int k = 0; k < kCPer; k++) {
        const int i = i0 + ib + k;
        if (i < i_end) A[(int64_t)i * dim + j] = o[k];
    }
}

}  // namespace

cudaError_t cepstrum_f32_init_tables() {
    float2 w[64];
    for (int k = 0; k < 64; k++) {
        const double a = 2.0 * 3.14159265358979323846 * k / 64.0;
        w[k] = make_float2((float)cos(a), (float)-sin(a));
    }
    return cudaMemcpyToSymbol(c_w64, w, sizeof(w));
}

cudaError_t launch_cepstrum_f32(const BatchTables& t, int images, const DevGeometry& g, const TypeLists& tl, int dim,
                                cudaStream_t st) {
    if (images <= 0) return cudaSuccess;
    const int tiles_x = (dim + 31) / 32, tiles_y = (dim + kCRows - 1) / kCRows;
    const int64_t blocks = (int64_t)4 * tiles_x * tiles_y;
    if (blocks > 0x7fffffff || images > 65535) return cudaErrorInvalidValue;
    k_cepstrum_fused<<<dim3((unsigned)blocks, (unsigned)images), kCThreads, 0, st>>>(t, g, tl, dim, tiles_x, tiles_y);
    return cudaGetLastError();
}

}  // namespace ske
