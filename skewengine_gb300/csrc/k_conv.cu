// Convolutions of the learned total-viewshed surrogate (a U-Net over 256x256
// DEM tiles): 3x3, stride 1, zero padding 1, NHWC bfloat16 activations,
// float32 accumulation.  The reference has no counterpart; the surrogate is an
// approximation of the engine's own total-viewshed output, trained on it.
//
// Forward (and the data gradient, which is the same convolution of the output
// gradient with the flipped, transposed weights) is an implicit GEMM:
//   Y[m][co] = bias[co] + sum_k A[m][k] * Wt[co][k],  m = (n, y, x), k = (ky, kx, ci)
//   A[m][k]  = X[n][y+ky-1][x+kx-1][ci] (zero outside the image)
// Cin is a multiple of 8, so every 8 consecutive k of a row of A are 16
// contiguous bytes of X (or all zero).  A CTA of 4 warps computes a 128 x 64
// tile of Y; k advances in slices of 32 that cp.async copies into a double
// buffer in shared memory (zero-filled where A is padding), ldmatrix feeds
// mma.sync m16n8k16 (bf16 in, f32 accumulate), and the epilogue adds the bias,
// optionally applies ReLU and stores bf16 pairs.
//
// The weight gradient dW[co][k] = sum_m dY[m][co] * A[m][k] runs over a chunk of
// pixels per CTA with the same tiles (A and dY staged in shared memory, read
// with transposing ldmatrix), and the chunks' partial sums are added into a
// float32 dW with atomics.
#include <cuda_bf16.h>

#include <cstdint>

#include "../../include/skewengine.h"

namespace {

typedef __nv_bfloat16 bf16;

constexpr int kBM = 128, kBN = 64, kBK = 32, kThreads = 128;
constexpr int kPitch = kBK + 8;  // shared row pitch in bf16: 80 bytes, ldmatrix conflict-free

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// 16-byte async copy; nbytes = 0 fills the destination with zeros.
__device__ __forceinline__ void cp_async16(void* dst, const void* src, int nbytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(nbytes));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;"); }
template <int kN>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(kN));
}

__device__ __forceinline__ void ldsm_x4(unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3, const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3, const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float* d, const unsigned* a, const unsigned* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// The pixel (n, y, x) of output row m, or y = -1e6 for rows past M.
struct Pix {
    int base;  // n*H*W
    int y, x;
};

__device__ __forceinline__ Pix pixel_of(int m, int M, int H, int W) {
    Pix p;
    if (m >= M) {
        p.base = 0;
        p.y = -1000000;
        p.x = 0;
        return p;
    }
    const int hw = H * W;
    const int n = m / hw, r = m - n * hw;
    p.base = n * hw;
    p.y = r / W;
    p.x = r - p.y * W;
    return p;
}

// Source of the 8 k values k .. k+7 of a row of A (k a multiple of 8), or null.
__device__ __forceinline__ const bf16* a_src(const bf16* __restrict__ X, const Pix& p, int k, int Cin, int H, int W) {
    const int tap = k / Cin;
    if (tap >= 9) return nullptr;
    const int ci = k - tap * Cin;
    const int ky = tap / 3, kx = tap - 3 * (tap / 3);
    const int iy = p.y + ky - 1, ix = p.x + kx - 1;
    if (iy < 0 || iy >= H || ix < 0 || ix >= W) return nullptr;
    return X + ((int64_t)(p.base + iy * W + ix) * Cin + ci);
}

// kUpCat: the input is the channel concatenation of X (C1 channels at half the
// resolution, nearest-upsampled) and X2 (C2 channels at full resolution), read
// in place: A's 8-channel chunk at (y, x) comes from X at (y/2, x/2) for
// channels below C1, else from X2.  The same products in the same order as on
// the materialised concatenation.
template <bool kUpCat>
__global__ void __launch_bounds__(kThreads, 4) k_conv3x3(const bf16* __restrict__ X, const bf16* __restrict__ Wt,
                                                      const float* __restrict__ bias, bf16* __restrict__ Y, int M,
                                                      int H, int W, int Cin, int Cout, int Kpad, int relu,
                                                      const bf16* __restrict__ X2, int C1) {
    __shared__ __align__(16) bf16 As[2][kBM][kPitch];
    __shared__ __align__(16) bf16 Bs[2][kBN][kPitch];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
    const int wm = (warp >> 1) * 64, wn = (warp & 1) * 32;

    // This thread's 4 A rows (pixels) share one 8-wide k offset kc: their
    // (tap, channel) pair is tracked incrementally as k advances by kBK, so each
    // chunk costs a bounds test and an add (no division per chunk and slice).
    const int kc = (tid & 3) * 8;
    const bf16* prow[4];
    int py[4], px[4], pn[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const Pix p = pixel_of(m0 + ((tid + i * kThreads) >> 2), M, H, W);
        py[i] = p.y;
        px[i] = p.x;
        pn[i] = p.y >= 0 ? p.base / (H * W) : 0;
        prow[i] = (!kUpCat && p.y >= 0) ? X + (int64_t)(p.base + p.y * W + p.x) * Cin : X;
    }
    int tap = kc / Cin, ci = kc - (kc / Cin) * Cin;  // k = k0 + kc at the next load
    auto load = [&](int stage, int k0) {  // called with k0 = 0, kBK, 2*kBK, ... in order
        const int ky = tap / 3, kx = tap - 3 * (tap / 3);
        const int64_t toff = ((int64_t)(ky - 1) * W + (kx - 1)) * Cin + ci;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int iy = py[i] + ky - 1, ix = px[i] + kx - 1;
            const bool ok = tap < 9 && iy >= 0 && iy < H && ix >= 0 && ix < W;
            const bf16* src = X;
            if (ok) {
                if (!kUpCat)
                    src = prow[i] + toff;
                else if (ci < C1)
                    src = X + ((int64_t)(pn[i] * (H >> 1) + (iy >> 1)) * (W >> 1) + (ix >> 1)) * C1 + ci;
                else
                    src = X2 + ((int64_t)(pn[i] * H + iy) * W + ix) * (Cin - C1) + (ci - C1);
            }
            cp_async16(&As[stage][(tid + i * kThreads) >> 2][kc], src, ok ? 16 : 0);
        }
        for (ci += kBK; ci >= Cin; ci -= Cin) tap++;
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int c = tid + i * kThreads;
            const int co = n0 + (c >> 2), kc = (c & 3) * 8;
            const bool ok = co < Cout;
            cp_async16(&Bs[stage][c >> 2][kc], ok ? Wt + (int64_t)co * Kpad + k0 + kc : Wt, ok ? 16 : 0);
        }
        cp_commit();
    };

    float acc[4][4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[i][j][e] = 0.0f;

    const int KT = Kpad / kBK;
    load(0, 0);
    for (int kt = 0; kt < KT; kt++) {
        const int s = kt & 1;
        if (kt + 1 < KT) {
            load(s ^ 1, (kt + 1) * kBK);
            cp_wait<1>();
        } else {
            cp_wait<0>();
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kBK; kk += 16) {
            unsigned af[4][4], bfr[4][2];
#pragma unroll
            for (int i = 0; i < 4; i++)
                ldsm_x4(af[i][0], af[i][1], af[i][2], af[i][3], &As[s][wm + i * 16 + (lane & 15)][kk + (lane >> 4) * 8]);
#pragma unroll
            for (int j = 0; j < 4; j += 2)
                ldsm_x4(bfr[j][0], bfr[j][1], bfr[j + 1][0], bfr[j + 1][1],
                        &Bs[s][wn + j * 8 + (lane >> 4) * 8 + (lane & 7)][kk + ((lane >> 3) & 1) * 8]);
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bfr[j]);
        }
        __syncthreads();  // the next load overwrites this stage
    }

#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int co = n0 + wn + j * 8 + (lane & 3) * 2;
            if (co >= Cout) continue;
            const float b0 = bias ? bias[co] : 0.0f, b1 = bias ? bias[co + 1] : 0.0f;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int m = m0 + wm + i * 16 + (lane >> 2) + h * 8;
                if (m >= M) continue;
                float v0 = acc[i][j][2 * h] + b0, v1 = acc[i][j][2 * h + 1] + b1;
                if (relu) v0 = fmaxf(v0, 0.0f), v1 = fmaxf(v1, 0.0f);
                *reinterpret_cast<__nv_bfloat162*>(Y + (int64_t)m * Cout + co) = __floats2bfloat162_rn(v0, v1);
            }
        }
}

// Weight gradient: a CTA owns a 64 (co) x 64 (k) tile of dW and a chunk of
// kWgChunk pixels; per slice of 32 pixels it stages dY[m][co] and A[m][k]
// (rows m) and reads both with transposing ldmatrix: dY^T as the row-major
// operand (co x m), A as the column operand (m x k).
constexpr int kWgChunk = 2048;
constexpr int kWgPitch = 64 + 8;  // 144-byte rows: conflict-free ldmatrix

__global__ void __launch_bounds__(kThreads) k_conv3x3_wgrad(const bf16* __restrict__ X, const bf16* __restrict__ dY,
                                                            float* __restrict__ dW, int M, int H, int W, int Cin,
                                                            int Cout, int Kpad) {
    __shared__ __align__(16) bf16 Ds[2][32][kWgPitch];
    __shared__ __align__(16) bf16 As[2][32][kWgPitch];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int k0 = blockIdx.x * 64, c0 = blockIdx.y * 64;
    const int mbeg = blockIdx.z * kWgChunk, mend = min(mbeg + kWgChunk, M);
    const int wc = (warp >> 1) * 32, wk = (warp & 1) * 32;
    auto load = [&](int stage, int mt) {
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int c = tid + i * kThreads;
            const int r = c >> 3, off = (c & 7) * 8;
            const int m = mt + r;
            const bool okd = m < mend && c0 + off < Cout;
            cp_async16(&Ds[stage][r][off], okd ? dY + (int64_t)m * Cout + c0 + off : dY, okd ? 16 : 0);
            const bf16* src = (m < mend && k0 + off < Kpad) ? a_src(X, pixel_of(m, M, H, W), k0 + off, Cin, H, W)
                                                             : nullptr;
            cp_async16(&As[stage][r][off], src ? src : X, src ? 16 : 0);
        }
        cp_commit();
    };
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[i][j][e] = 0.0f;
    const int nt = (mend - mbeg + 31) / 32;
    if (nt > 0) load(0, mbeg);
    for (int t = 0; t < nt; t++) {
        const int s = t & 1;
        if (t + 1 < nt) {
            load(s ^ 1, mbeg + (t + 1) * 32);
            cp_wait<1>();
        } else {
            cp_wait<0>();
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 32; kk += 16) {
            unsigned af[2][4], bfr[4][2];
#pragma unroll
            for (int i = 0; i < 2; i++)
                ldsm_x4_t(af[i][0], af[i][1], af[i][2], af[i][3],
                          &Ds[s][kk + (lane & 7) + ((lane >> 4) << 3)][wc + i * 16 + ((lane >> 3) & 1) * 8]);
#pragma unroll
            for (int j = 0; j < 4; j += 2)
                ldsm_x4_t(bfr[j][0], bfr[j][1], bfr[j + 1][0], bfr[j + 1][1],
                          &As[s][kk + (lane & 7) + ((lane >> 3) & 1) * 8][wk + j * 8 + (lane >> 4) * 8]);
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bfr[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int k = k0 + wk + j * 8 + (lane & 3) * 2;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int co = c0 + wc + i * 16 + (lane >> 2) + h * 8;
                if (co >= Cout || k >= Kpad) continue;
                atomicAdd(dW + (int64_t)co * Kpad + k, acc[i][j][2 * h]);
                atomicAdd(dW + (int64_t)co * Kpad + k + 1, acc[i][j][2 * h + 1]);
            }
        }
}

// cp.async copies 16 bytes: tensors must start on 16-byte boundaries (outputs:
// 4 bytes, for the bf16 pairs of the epilogue).
bool aligned(const void* p, uintptr_t a) { return ((uintptr_t)p & (a - 1)) == 0; }

}  // namespace

extern "C" int ske_conv3x3_bf16(const void* x, const void* w, const float* bias, void* y, int n, int h, int w_,
                                int cin, int cout, int relu, void* stream) {
    if (!x || !w || !y || n < 1 || h < 1 || w_ < 1 || cin < 8 || cin % 8 || cout < 2 || cout % 2)
        return SKE_ERR_INVALID;
    if (!aligned(x, 16) || !aligned(w, 16) || !aligned(y, 4) || !aligned(bias, 4)) return SKE_ERR_INVALID;
    const int64_t m = (int64_t)n * h * w_;
    if (m > 0x7fffffff / 2 || (int64_t)cin * 9 > 0x7fffffff / 2) return SKE_ERR_INVALID;
    const int kpad = (9 * cin + kBK - 1) / kBK * kBK;
    const dim3 grid((unsigned)((m + kBM - 1) / kBM), (unsigned)((cout + kBN - 1) / kBN));
    k_conv3x3<false><<<grid, kThreads, 0, (cudaStream_t)stream>>>((const bf16*)x, (const bf16*)w, bias, (bf16*)y,
                                                                  (int)m, h, w_, cin, cout, kpad, relu, nullptr, 0);
    return cudaGetLastError() == cudaSuccess ? SKE_OK : SKE_ERR_CUDA;
}

extern "C" int ske_conv3x3_upcat_bf16(const void* xlow, const void* xskip, const void* w, const float* bias, void* y,
                                      int n, int h, int w_, int c1, int c2, int cout, int relu, void* stream) {
    if (!xlow || !xskip || !w || !y || n < 1 || h < 2 || w_ < 2 || h % 2 || w_ % 2 || c1 < 8 || c1 % 8 ||
        c2 < 8 || c2 % 8 || cout < 2 || cout % 2)
        return SKE_ERR_INVALID;
    if (!aligned(xlow, 16) || !aligned(xskip, 16) || !aligned(w, 16) || !aligned(y, 4) || !aligned(bias, 4))
        return SKE_ERR_INVALID;
    const int64_t m = (int64_t)n * h * w_;
    const int cin = c1 + c2;
    if (m > 0x7fffffff / 2 || (int64_t)cin * 9 > 0x7fffffff / 2) return SKE_ERR_INVALID;
    const int kpad = (9 * cin + kBK - 1) / kBK * kBK;
    const dim3 grid((unsigned)((m + kBM - 1) / kBM), (unsigned)((cout + kBN - 1) / kBN));
    k_conv3x3<true><<<grid, kThreads, 0, (cudaStream_t)stream>>>((const bf16*)xlow, (const bf16*)w, bias, (bf16*)y,
                                                                 (int)m, h, w_, cin, cout, kpad, relu,
                                                                 (const bf16*)xskip, c1);
    return cudaGetLastError() == cudaSuccess ? SKE_OK : SKE_ERR_CUDA;
}

extern "C" int ske_conv3x3_wgrad_bf16(const void* x, const void* dy, float* dw, int n, int h, int w_, int cin,
                                      int cout, void* stream) {
    if (!x || !dy || !dw || n < 1 || h < 1 || w_ < 1 || cin < 8 || cin % 8 || cout < 8 || cout % 8)
        return SKE_ERR_INVALID;
    if (!aligned(x, 16) || !aligned(dy, 16) || !aligned(dw, 4)) return SKE_ERR_INVALID;
    const int64_t m = (int64_t)n * h * w_;
    if (m > 0x7fffffff / 2) return SKE_ERR_INVALID;
    const int kpad = (9 * cin + kBK - 1) / kBK * kBK;
    const dim3 grid((unsigned)((kpad + 63) / 64), (unsigned)((cout + 63) / 64),
                    (unsigned)((m + kWgChunk - 1) / kWgChunk));
    k_conv3x3_wgrad<<<grid, kThreads, 0, (cudaStream_t)stream>>>((const bf16*)x, (const bf16*)dy, dw, (int)m, h, w_,
                                                                 cin, cout, kpad);
    return cudaGetLastError() == cudaSuccess ? SKE_OK : SKE_ERR_CUDA;
}
