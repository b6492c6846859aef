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
// contiguous bytes of X (or all zero).  It runs on the 5th-generation tensor
// cores (tcgen05.mma with the accumulator in tensor memory; k_conv3x3 below).
//
// The weight gradient dW[co][k] = sum_m dY[m][co] * A[m][k] runs over a chunk of
// pixels per CTA (A and dY staged in shared memory, read with transposing
// ldmatrix into mma.sync m16n8k16), and the chunks' partial sums are added into
// a float32 dW with atomics.
#include <cstdio>
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cstdint>

#include "../../include/skewengine.h"

namespace {

typedef __nv_bfloat16 bf16;

constexpr int kBK = 32, kThreads = 128;

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// 16-byte async copy; nbytes = 0 fills the destination with zeros.
__device__ __forceinline__ void cp_async16(void* dst, const void* src, int nbytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(nbytes));
}
// The same through L1 (.ca): the nine taps of a 3x3 window re-read each input
// pixel, mostly within one CTA or its neighbours on the SM.
__device__ __forceinline__ void cp_async16_ca(void* dst, const void* src, int nbytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(nbytes));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;"); }
template <int kN>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(kN));
}
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

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

// ---- forward convolution on the tensor cores (tcgen05) ----------------------
//
// A CTA of 4 warps computes a 128 x BN tile of Y (BN = Cout rounded up to a
// multiple of 16, at most 128) with tcgen05.mma kind::f16 (bfloat16 A and B,
// float32 accumulator in tensor memory, BN columns of its 128 lanes).  K
// advances in slices of 32, two MMAs of K = 16 each.  Every thread copies its
// share of a slice's A rows (the im2col gather, zero where A is padding) and B
// rows (weights) with cp.async through L1 into a kTcStages-deep ring in shared
// memory, in the canonical K-major layout without swizzle: core matrices of 8
// rows x 16 bytes (128 contiguous bytes), the 4 core matrices of a row group's
// slice adjacent (leading byte offset 128), row groups 512 bytes apart (stride
// byte offset).  Slices are fetched kTcPrefetch ahead.  Once every thread's
// copies of a slice have landed (wait_group, proxy fence, barrier) thread 0
// issues its MMAs and commits them to the stage's mbarrier.  A stage is refilled with the slice kTcStages after
// the one it held, which was issued kTcStages - kTcPrefetch = 2 slices earlier,
// so the tensor pipe keeps a slice queued while the next one's barrier passes.
// The epilogue reads the accumulator with tcgen05.ld (warp w owns lanes
// 32w..32w+31, i.e. output rows), adds the bias, applies ReLU and stores
// bfloat16.  Every wait is bounded: one that runs out sets g_conv_status,
// skips the remaining MMAs and the epilogue, and the CTA still releases its
// tensor memory.
//
// kUpCat: the input is the channel concatenation of X (C1 channels at half the
// resolution, nearest-upsampled) and X2 (C2 channels at full resolution), read
// in place: A's 8-channel chunk at (y, x) comes from X at (y/2, x/2) for
// channels below C1, else from X2.  The same products in the same order as on
// the materialised concatenation.
constexpr int kTcBM = 128, kTcBK = 32, kTcStages = 4, kTcPrefetch = 2, kTcMaxBN = 128;
constexpr int kTcABytes = kTcBM * kTcBK * 2;  // 8 KB of A per stage
constexpr int kTcSBO = (kTcBK / 8) * 128;     // bytes between row groups
constexpr long long kTcWaitLimit = 1ll << 22;

__device__ int g_conv_status;  // 1: a tensor-core wait ran out

__host__ __device__ constexpr int tc_smem_bytes(int bn) {
    return kTcStages * (kTcABytes + bn * kTcBK * 2) + kTcStages * 8 + 16;
}

__device__ __forceinline__ void tc_mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool tc_mbar_wait(uint64_t* bar, int parity) {
    for (long long i = 0; i < kTcWaitLimit; i++) {
        unsigned ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: start address, leading byte offset 128,
// stride byte offset kTcSBO (all in 16-byte units), descriptor version 1, no
// swizzle.
__device__ __forceinline__ uint64_t tc_desc(unsigned saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(kTcSBO >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor, kind::f16: f32 accumulator (bits 4-5 = 1), A and B
// bfloat16 (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bit 17,
// M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t tc_idesc(int bn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(kTcBM >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(unsigned dtmem, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::
            "r"(dtmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 16 consecutive f32 columns of this warp's 32 lanes (lane = row) from tensor memory.
__device__ __forceinline__ void tc_ld16(unsigned taddr, float* v) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// 32 consecutive f32 columns of this warp's 32 lanes from tensor memory.
__device__ __forceinline__ void tc_ld32(unsigned taddr, float* v) {
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// The same load without its wait (tc_ld32_wait completes it).
__device__ __forceinline__ void tc_ld32_issue(unsigned taddr, unsigned* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
}
// Waits for this thread's tensor-memory loads; the registers of the last one
// pass through the statement, so their uses stay after it.
__device__ __forceinline__ void tc_ld32_wait(unsigned* r) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                   "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                   "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
                 :
                 : "memory");
}

template <bool kUpCat>
__global__ void __launch_bounds__(kThreads) k_conv3x3(const bf16* __restrict__ X, const bf16* __restrict__ Wt,
                                                      const float* __restrict__ bias, bf16* __restrict__ Y, int M,
                                                      int H, int W, int Cin, int Cout, int Kpad, int relu,
                                                      const bf16* __restrict__ X2, int C1, int BN, int vec16) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int m0 = blockIdx.x * kTcBM, n0 = blockIdx.y * BN;
    const int bbytes = BN * kTcBK * 2;
    unsigned char* As = tc_smem;                           // [kTcStages][kTcABytes]
    unsigned char* Bs = tc_smem + kTcStages * kTcABytes;   // [kTcStages][bbytes]
    uint64_t* bar = reinterpret_cast<uint64_t*>(Bs + kTcStages * bbytes);
    unsigned* tslot = reinterpret_cast<unsigned*>(bar + kTcStages);
    const unsigned ncols = BN <= 32 ? 32u : BN <= 64 ? 64u : 128u;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kTcStages; s++) tc_mbar_init(&bar[s]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tslot;

    // This thread's 4 A rows (pixels) share one 8-wide k offset kc within each
    // 32-wide part of a slice: their (tap, channel) pair is tracked
    // incrementally as k advances by 32, so each chunk costs a bounds test and
    // an add (no division per chunk).
    const int kc = (tid & 3) * 8;
    const bf16* prow[4];
    int py[4], px[4], pn[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const Pix p = pixel_of(m0 + (tid >> 2) + 32 * i, M, H, W);
        py[i] = p.y;
        px[i] = p.x;
        pn[i] = p.y >= 0 ? p.base / (H * W) : 0;
        prow[i] = (!kUpCat && p.y >= 0) ? X + (int64_t)(p.base + p.y * W + p.x) * Cin : X;
    }
    int tap = kc / Cin, ci = kc - (kc / Cin) * Cin;  // k = k0 + kc at the next load
    // Byte offset of (row r, 8-element chunk c) of a stage in the core-matrix layout.
    auto cm = [](int r, int c) { return (r >> 3) * kTcSBO + c * 128 + (r & 7) * 16; };
    auto load = [&](int stage, int k0) {  // called with k0 = 0, kTcBK, 2*kTcBK, ... in order
#pragma unroll
        for (int half = 0; half < kTcBK / 32; half++) {
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
                cp_async16_ca(As + stage * kTcABytes + cm((tid >> 2) + 32 * i, half * 4 + (tid & 3)), src,
                              ok ? 16 : 0);
            }
            for (ci += 32; ci >= Cin; ci -= Cin) tap++;
        }
        for (int q = tid; q < BN * (kTcBK / 8); q += kThreads) {
            const int r = q / (kTcBK / 8), c = q % (kTcBK / 8), co = n0 + r;
            const bool ok = co < Cout && k0 + c * 8 < Kpad;
            cp_async16_ca(Bs + stage * bbytes + cm(r, c), ok ? Wt + (int64_t)co * Kpad + k0 + c * 8 : Wt, ok ? 16 : 0);
        }
    };

    const int KT = (Kpad + kTcBK - 1) / kTcBK;
    const uint32_t idesc = tc_idesc(BN);
    for (int s = 0; s < kTcPrefetch; s++) {
        if (s < KT) load(s, s * kTcBK);
        cp_commit();
    }
    bool fail = false;
    int last_commit = -1;  // thread 0: the last slice whose MMAs were committed
    for (int kt = 0; kt < KT; kt++) {
        const int nxt = kt + kTcPrefetch;
        if (nxt < KT) {
            // The stage last held slice nxt - kTcStages: its MMAs must be done reading it.
            const int st = nxt % kTcStages, prev = nxt - kTcStages;
            if (prev >= 0 && !fail) fail = !tc_mbar_wait(&bar[st], (prev / kTcStages) & 1);
            load(st, nxt * kTcBK);
        }
        cp_commit();
        cp_wait<kTcPrefetch>();  // this thread's copies of slice kt have landed
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (__syncthreads_or(fail)) {
            fail = true;
            break;
        }
        if (tid == 0) {
            tc_fence_after();
            const int s = kt % kTcStages;
            const unsigned a0 = smem_u32(As + s * kTcABytes), b0 = smem_u32(Bs + s * bbytes);
#pragma unroll
            for (int kk = 0; kk < kTcBK / 16; kk++)
                tc_mma(tmem, tc_desc(a0 + kk * 256), tc_desc(b0 + kk * 256), idesc, (kt | kk) != 0);
            tc_commit(&bar[s]);
            last_commit = kt;
        }
    }
    cp_wait<0>();
    // The last slice's commit completes after every earlier MMA.
    if (!fail && KT > 0) fail = !tc_mbar_wait(&bar[(KT - 1) % kTcStages], ((KT - 1) / kTcStages) & 1);
    fail = __syncthreads_or(fail);
    // Giving up: before the tensor memory is freed below, thread 0 waits once
    // more (bounded) for the last commit it issued, which arrives after all of
    // its MMAs, so that none is still writing the accumulator when it is freed.
    // If that wait runs out too the memory is freed regardless (the output is
    // not written and the status flag tells the host).
    if (fail && tid == 0 && last_commit >= 0)
        tc_mbar_wait(&bar[last_commit % kTcStages], (last_commit / kTcStages) & 1);
    tc_fence_after();
    if (!fail) {
        const int m = m0 + warp * 32 + lane;
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            tc_ld16(tmem + ((unsigned)(warp * 32) << 16) + (unsigned)c0, v);
            if (m >= M) continue;
#pragma unroll
            for (int g = 0; g < 16; g += 8) {
                const int co = n0 + c0 + g;
                if (co >= Cout) break;
                float o[8];
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const float b = (bias && co + e < Cout) ? bias[co + e] : 0.0f;
                    o[e] = __fadd_rn(v[g + e], b);
                    if (relu) o[e] = fmaxf(o[e], 0.0f);
                }
                bf16* dst = Y + (int64_t)m * Cout + co;
                if (vec16 && co + 8 <= Cout) {
                    __nv_bfloat162 h[4];
#pragma unroll
                    for (int e = 0; e < 4; e++) h[e] = __floats2bfloat162_rn(o[2 * e], o[2 * e + 1]);
                    *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(h);
                } else {
#pragma unroll
                    for (int e = 0; e < 8; e += 2)
                        if (co + e < Cout)
                            *reinterpret_cast<__nv_bfloat162*>(dst + e) = __floats2bfloat162_rn(o[e], o[e + 1]);
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(&g_conv_status, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
    }
}

// ---- halo-staged forward convolution on the tensor cores ---------------------
//
// An image is cut into column segments of Ws pixels (128 when the width is a
// multiple of 128 above it, else the whole width), and a segment's output
// pixels are numbered as slots of rows of pitch P = Ws + 2: slot s is pixel
// (s / P, x0 + s % P), and the two last slots of a row are junk whose outputs
// are discarded (2/P of the work).  A CTA computes nb blocks of 128
// consecutive slots of one segment (nb = 8 for Cout <= 32, 4 for Cout <= 128;
// its accumulators are nb x Cout tensor-memory columns) for all Cout channels,
// Cin and Cout multiples of 16.  K advances in groups of 16 input channels,
// each staged once in shared memory as
//   halo:    two planes of 8 channels holding the input rows the tile's slots
//            touch in the same pitch: plane slot (hr, hc) is input pixel
//            (R0 - 1 + hr, x0 - 1 + hc), the segment plus one column on each
//            side, zero outside the image; a pixel's 8 channels are one
//            16-byte row of a core matrix;
//   weights: for each of the 9 taps, the 16 channels' Cout x 16 slice in the
//            canonical K-major layout (8-row x 16-byte core matrices).
// The input of output slot s for tap (ky, kx) then sits at plane slot
// s - R0*P + ky*P + kx (R0 the tile's first row), so the MMA of block j and tap
// (ky, kx) reads its A operand in place: 128 consecutive plane slots, core
// matrices 128 bytes apart (stride byte offset), the second 8 channels one
// plane further (leading byte offset).  Each input pixel leaves L2 once per CTA
// (plus the two halo rows and columns) instead of once per tap as in the
// im2col gather above.
// kHaloStages groups are in flight; thread 0 issues a group's MMAs (nb blocks x
// 9 taps, K = 16 each) and commits them to the stage's mbarrier, which frees
// the stage for the group kHaloStages later.  Waits are bounded as in
// k_conv3x3.
constexpr int kHaloStages = 2;
constexpr int kSlotBlock = 128;

// Column segment width of an image width, and plane slots of a tile of nb
// blocks at row pitch P = Ws + 2: output slot s - S0 < nb*128 of a tile whose
// first slot sits at column soff <= P - 1 reads plane slot
// (s - S0) + soff + ky*P + kx <= 3P + nb*128 for tap (ky, kx), so the plane
// holds 3P + nb*128 + 1 slots.
__host__ __device__ constexpr int halo_seg(int W) { return (W > 128 && W % 128 == 0) ? 128 : W; }
__host__ __device__ constexpr int halo_slots(int P, int nb) { return 3 * P + nb * kSlotBlock + 1; }
__host__ __device__ constexpr int halo_plane(int P, int nb) { return halo_slots(P, nb) * 16; }
__host__ __device__ constexpr int halo_wbytes(int cout) { return 9 * 2 * cout * 16; }
__host__ __device__ constexpr int halo_stage_bytes(int P, int nb, int cout) {
    return (2 * halo_plane(P, nb) + halo_wbytes(cout) + 1023) / 1024 * 1024;
}
__host__ __device__ constexpr int halo_smem_bytes(int P, int nb, int cout) {
    return kHaloStages * halo_stage_bytes(P, nb, cout) + 1024 + 64;
}

// Descriptor with explicit byte offsets (16-byte units): no swizzle, version 1.
__device__ __forceinline__ uint64_t tc_desc2(unsigned saddr, unsigned lbo, unsigned sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

template <bool kUpCat>
__global__ void __launch_bounds__(kThreads) k_conv3x3_halo(const bf16* __restrict__ X, const bf16* __restrict__ Wt,
                                                           const float* __restrict__ bias, bf16* __restrict__ Y,
                                                           int H, int W, int Cin, int Cout, int Kpad, int relu,
                                                           const bf16* __restrict__ X2, int C1, int nb,
                                                           int tiles_per_seg) {
    extern __shared__ __align__(1024) unsigned char hsm_raw[];
    unsigned char* hsm = hsm_raw + ((1024 - (smem_u32(hsm_raw) & 1023)) & 1023);  // 1024-byte aligned stages
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int Ws = halo_seg(W), P = Ws + 2, segs = W / Ws;
    const int hslots = halo_slots(P, nb);
    const int plane = hslots * 16;
    const int sbytes = halo_stage_bytes(P, nb, Cout);
    uint64_t* bar = reinterpret_cast<uint64_t*>(hsm + kHaloStages * sbytes);
    unsigned* tslot = reinterpret_cast<unsigned*>(bar + kHaloStages);
    int bi = blockIdx.x;
    const int tile = bi % tiles_per_seg;
    bi /= tiles_per_seg;
    const int seg = bi % segs;
    const int n = bi / segs;
    const int x0 = seg * Ws;                     // the segment's first column
    const int S0 = tile * nb * kSlotBlock;       // first output slot of the tile
    const int R0 = S0 / P;                       // its row
    const int soff = S0 - R0 * P;                // its column (plane slot base)
    unsigned ncols = 32;
    while (ncols < (unsigned)(nb * Cout)) ncols <<= 1;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kHaloStages; s++) tc_mbar_init(&bar[s]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tslot;

    const int groups = Cin / 16;
    const int64_t img = (int64_t)n * H * W;
    // Stage group g into stage st: plane slot p is input (R0 - 1 + p / P,
    // x0 - 1 + p % P), zero outside the image.
    auto load = [&](int st, int g) {
        unsigned char* base = hsm + st * sbytes;
        const int c0 = 16 * g;
        for (int q = tid; q < 2 * hslots; q += kThreads) {
            const int pl = q >= hslots;
            const int p = q - pl * hslots;
            const int hr = p / P;
            const int iy = R0 - 1 + hr, ix = x0 - 1 + (p - hr * P);
            const int ci = c0 + 8 * pl;
            const bool ok = iy >= 0 && iy < H && ix >= 0 && ix < W;
            const bf16* src = X;
            if (ok) {
                if (!kUpCat)
                    src = X + ((img + (int64_t)iy * W + ix) * Cin + ci);
                else if (ci < C1)
                    src = X + (((int64_t)n * (H >> 1) + (iy >> 1)) * (W >> 1) + (ix >> 1)) * C1 + ci;
                else
                    src = X2 + ((img + (int64_t)iy * W + ix) * (Cin - C1) + (ci - C1));
            }
            cp_async16_ca(base + pl * plane + p * 16, src, ok ? 16 : 0);
        }
        unsigned char* wb = base + 2 * plane;
        for (int q = tid; q < 9 * 2 * Cout; q += kThreads) {
            const int co = q % Cout, tk = q / Cout;  // tk = tap * 2 + kc
            const int tap = tk >> 1, kc = tk & 1;
            cp_async16_ca(wb + (tk * Cout + co) * 16, Wt + (int64_t)co * Kpad + tap * Cin + c0 + 8 * kc, 16);
        }
    };

    const uint32_t idesc = tc_idesc(Cout);
    for (int s = 0; s < kHaloStages - 1; s++) {
        if (s < groups) load(s, s);
        cp_commit();
    }
    bool fail = false;
    int last_commit = -1;
    for (int g = 0; g < groups; g++) {
        const int nxt = g + kHaloStages - 1;
        if (nxt < groups) {
            // Stage nxt % kHaloStages last held group nxt - kHaloStages: its MMAs
            // must be done reading it.
            const int st = nxt % kHaloStages, prev = nxt - kHaloStages;
            if (prev >= 0 && !fail) fail = !tc_mbar_wait(&bar[st], (prev / kHaloStages) & 1);
            load(st, nxt);
        }
        cp_commit();
        cp_wait<kHaloStages - 1>();  // this thread's copies of group g have landed
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (__syncthreads_or(fail)) {
            fail = true;
            break;
        }
        if (tid == 0) {
            tc_fence_after();
            const int st = g % kHaloStages;
            const unsigned hb = smem_u32(hsm + st * sbytes), wb = hb + 2 * plane;
            for (int j = 0; j < nb; j++)
#pragma unroll
                for (int tap = 0; tap < 9; tap++) {
                    const int ky = tap / 3, kx = tap - 3 * (tap / 3);
                    const int p0 = soff + j * kSlotBlock + ky * P + kx;
                    const uint64_t da = tc_desc2(hb + (unsigned)(p0 * 16), (unsigned)plane, 128);
                    const uint64_t db = tc_desc2(wb + (unsigned)(tap * 2 * Cout * 16), (unsigned)(Cout * 16), 128);
                    tc_mma(tmem + (unsigned)(j * Cout), da, db, idesc, (g | tap) != 0);
                }
            tc_commit(&bar[st]);
            last_commit = g;
        }
    }
    cp_wait<0>();
    if (!fail && groups > 0) fail = !tc_mbar_wait(&bar[(groups - 1) % kHaloStages], ((groups - 1) / kHaloStages) & 1);
    fail = __syncthreads_or(fail);
    if (fail && tid == 0 && last_commit >= 0)
        tc_mbar_wait(&bar[last_commit % kHaloStages], (last_commit / kHaloStages) & 1);
    tc_fence_after();
    if (!fail) {
        for (int j = 0; j < nb; j++) {
            const int s = S0 + j * kSlotBlock + warp * 32 + lane;  // this thread's slot (TMEM lane)
            const int r = s / P, c = s - (s / P) * P;
            const bool store = r < H && c < Ws;
            bf16* dst = Y + ((img + (int64_t)r * W + x0 + c) * Cout);
            for (int c0 = 0; c0 < Cout; c0 += 16) {
                float v[16];
                tc_ld16(tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(j * Cout + c0), v);
                if (!store) continue;
                __nv_bfloat162 h[8];
#pragma unroll
                for (int e = 0; e < 16; e += 2) {
                    float o0 = __fadd_rn(v[e], bias ? bias[c0 + e] : 0.0f);
                    float o1 = __fadd_rn(v[e + 1], bias ? bias[c0 + e + 1] : 0.0f);
                    if (relu) {
                        o0 = fmaxf(o0, 0.0f);
                        o1 = fmaxf(o1, 0.0f);
                    }
                    h[e / 2] = __floats2bfloat162_rn(o0, o1);
                }
                uint4* d4 = reinterpret_cast<uint4*>(dst + c0);
                d4[0] = *reinterpret_cast<const uint4*>(&h[0]);
                d4[1] = *reinterpret_cast<const uint4*>(&h[4]);
            }
        }
    } else if (tid == 0) {
        atomicExch(&g_conv_status, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
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

// Forward-convolution kernel choice (ske_conv_select): 0 = the warp-specialised
// kernel where it applies, else the halo-staged one where it applies, else
// im2col; 1 = always the im2col kernel; 2 = halo-staged where it applies, else
// im2col.
int g_conv_path = 0;

// Launch of the tensor-core forward convolution: BN = Cout rounded up to 16,
// at most kTcMaxBN, and Cout / BN column tiles.  With 4 stages a CTA holds
// 36-64 KB of shared memory, so at most 6 (BN 16) down to 3 (BN 128) CTAs share
// an SM and their tensor-memory columns (32, 64 or 128 each) stay within the
// SM's 512.
// The halo-staged kernel applies when Cin, Cout (<= 256) and, for the upsampled
// concatenation, C1 are multiples of 16 and its stages fit shared memory.  Its
// shared memory is padded so that the CTAs an SM holds never ask for more than
// its 512 tensor-memory columns.
int halo_blocks(int cout) { return cout <= 32 ? 8 : cout <= 128 ? 4 : 2; }

// Cout above 128 (the 32 x 32, 256-channel bottleneck) measured faster on the
// im2col kernel (155-185 against 201-228 TFLOP/s): two 128-slot blocks per CTA
// leave too few MMAs per staged group.
bool halo_applies(int w_, int cin, int cout, int c1) {
    return cin % 16 == 0 && cout % 16 == 0 && cout >= 16 && cout <= 128 && c1 % 16 == 0 &&
           halo_smem_bytes(halo_seg(w_) + 2, halo_blocks(cout), cout) <= 227 * 1024;
}

template <bool kUpCat>
int launch_conv_halo(const bf16* x, const bf16* w, const float* bias, bf16* y, int n, int h, int w_, int cin,
                     int cout, int relu, const bf16* x2, int c1, cudaStream_t st) {
    const int kpad = (9 * cin + kTcBK - 1) / kTcBK * kTcBK;
    const int nb = halo_blocks(cout);
    unsigned ncols = 32;
    while (ncols < (unsigned)(nb * cout)) ncols <<= 1;
    const int ws = halo_seg(w_), pitch = ws + 2;
    int smem = halo_smem_bytes(pitch, nb, cout);
    const int max_ctas = 512 / (int)ncols;  // CTAs whose columns fit the SM's tensor memory
    const int floor_smem = 228 * 1024 / (max_ctas + 1) + 1;
    if (smem < floor_smem) smem = floor_smem;
    if (smem > 227 * 1024) return SKE_ERR_UNSUPPORTED;
    if (cudaFuncSetAttribute(k_conv3x3_halo<kUpCat>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
        cudaSuccess)
        return SKE_ERR_CUDA;
    const int64_t slots = (int64_t)h * pitch;  // of one segment
    const int64_t tiles = (slots + (int64_t)nb * kSlotBlock - 1) / ((int64_t)nb * kSlotBlock);
    const int64_t blocks = (int64_t)n * (w_ / ws) * tiles;
    if (blocks > 0x7fffffff || slots > 0x7fffffff / 2) return SKE_ERR_INVALID;
    k_conv3x3_halo<kUpCat><<<(unsigned)blocks, kThreads, smem, st>>>(x, w, bias, y, h, w_, cin, cout, kpad, relu, x2,
                                                                     c1, nb, (int)tiles);
    return cudaGetLastError() == cudaSuccess ? SKE_OK : SKE_ERR_CUDA;
}

// ---- warp-specialised persistent forward convolution -------------------------
//
// The halo-staged scheme above with the roles split across warps and each CTA
// resident for the whole launch (one CTA per SM, tiles taken round-robin).  A
// work item is one tile and one stage of 16*gs input channels (gs = 1, 2 or 4
// groups of 16), staged as 2*gs halo planes of 8 channels plus the groups'
// weights:
//   warps 4-7  producers: copy an item into a ring of S stages with 16-byte
//              cp.async.  Consecutive threads take consecutive 16-byte chunks
//              of one pixel's 16*gs channels (contiguous in NHWC), so a warp's
//              copies cover whole 32*gs-byte runs; the weights come from a copy
//              packed per call in the stage's own order (one contiguous block
//              per item).  Each producer thread's copies of an item arrive on
//              the stage's `full` barrier when they land
//              (cp.async.mbarrier.arrive.noinc, 128 arrivals), so the
//              producers never wait for their copies and all S stages can be
//              in flight.
//   warp 8     lane 0 waits for a stage's barrier, fences the producers' writes
//              for the async proxy and issues the item's gs x nb x 9 MMAs
//              (M 128, N Cout, K 16) into one of two tensor-memory
//              accumulators (columns 0 and 256),
//              commits them to the stage's `empty` barrier and, after a tile's
//              last item, to the accumulator's `acc_full` barrier.
//   warps 0-3  epilogue: warp w reads lanes 32w..32w+31 of the finished
//              accumulator (tcgen05.ld, 32 columns at a time), adds the bias,
//              applies ReLU, stores
//              bfloat16 and arrives on `acc_empty`, while the MMAs of the next
//              tile run into the other accumulator.
// Per output the MMAs run group by group and tap by tap, the order of the
// halo-staged kernel, so both give the same bits.  nb = 256 / Cout blocks of
// 128 slots (at most 8) so that the two accumulators fill the SM's 512
// tensor-memory columns.  Input channels past Cin (Cin a multiple of 8) read as
// zero, as do their weights.  kUpCat reads the channels below C1 (a multiple of
// 16*gs) from the half-resolution X at (y/2, x/2) and the others from X2.  Every
// wait is bounded and also gives up once another role has given up (the CTA's
// abort word); a producer then drains its own copies, the MMA thread waits for
// its last commit, and the CTA releases its tensor memory after a block
// barrier.  g_conv_status reports a give-up.
constexpr int kWsEpiWarps = 4, kWsProdWarps = 4;
constexpr int kWsProd = kWsProdWarps * 32;
constexpr int kWsThreads = (kWsEpiWarps + kWsProdWarps + 1) * 32;
constexpr int kWsMaxStages = 4;
constexpr int kWsExtra = 128 + 2 * kWsMaxStages * 8 + 4 * 8 + 16 + (2 * 256 + 4) * 4;  // alignment, barriers,
                                                                                        // words, bias, head
constexpr int kWsMinSmem = 116 * 1024;  // more than half an SM's shared memory: one CTA per SM
constexpr int kWsDevices = 64;          // devices whose SM count is cached

struct WsGeom {
    int H, W, Cin, Cout, C1, relu;
    int Ws, P, segs, tps, nb, hslots;
    int gs, lgs;      // 16-channel groups per item and log2(2 * gs)
    int items;        // items per tile
    int S;            // stages
    int plane, wbytes, sbytes;  // bytes: one 8-channel plane, an item's weights, one stage
    int total;        // tiles
};

__host__ __device__ constexpr int ws_blocks(int cout) { return 256 / cout > 8 ? 8 : 256 / cout; }

__device__ __forceinline__ void ws_bar_init(uint64_t* bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void ws_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool ws_try(uint64_t* bar, int parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait that also returns (false) once the CTA's abort word is set; a
// wait that runs out sets it.
__device__ __forceinline__ bool ws_wait(uint64_t* bar, int parity, volatile int* abort_word) {
    for (long long i = 0; i < kTcWaitLimit; i++) {
        if (ws_try(bar, parity)) return true;
        if ((i & 63) == 63 && *abort_word) return false;
    }
    *abort_word = 1;
    return false;
}

// Weights packed in the staged order: for each 16-channel group g, tap and
// 8-channel half, the Cout rows of 8 channels: Wp[((g*9 + tap)*2 + half)*Cout + co][0..7]
// = Wt[co][tap*Cin + 16g + 8half + 0..7], zero past Cin.  One thread per row.
__global__ void k_pack_weights(const bf16* __restrict__ Wt, bf16* __restrict__ Wp, int Cin, int Cout, int Kpad,
                               int rows) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= rows) return;
    const int co = e % Cout, r = e / Cout, half = r & 1, tap = (r >> 1) % 9, g = (r >> 1) / 9;
    const int ci = 16 * g + 8 * half;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (ci < Cin) v = *reinterpret_cast<const uint4*>(Wt + (int64_t)co * Kpad + tap * Cin + ci);
    reinterpret_cast<uint4*>(Wp)[e] = v;
}

// One 32-column chunk q of a finished accumulator (block q / cpb, columns
// 32 (q % cpb) ..): bias, ReLU, bfloat16; stored, or with a head folded into
// hsum (in channel order) and written at the block's last chunk.
__device__ __forceinline__ void ws_epi_chunk(int q, int cpb, const unsigned* r, int S0, int x0, int n, int64_t HW,
                                             int warp, int lane, const WsGeom& g, const float* sbias,
                                             const float* shead, bf16* __restrict__ Y, float* __restrict__ Yh,
                                             float& hsum) {
    const int j = q / cpb, c0 = (q - j * cpb) * 32;
    const int s = S0 + j * kSlotBlock + warp * 32 + lane;  // this thread's slot (lane)
    const int rr = s / g.P, c = s - rr * g.P;
    const bool store = rr < g.H && c < g.Ws;
    const int64_t pix = (int64_t)n * HW + (int64_t)rr * g.W + x0 + c;
    if (c0 == 0) hsum = 0.0f;
    if (store) {
#pragma unroll
        for (int e0 = 0; e0 < 32; e0 += 16) {
            __nv_bfloat162 h[8];
#pragma unroll
            for (int e = 0; e < 16; e += 2) {
                float o0 = __fadd_rn(__uint_as_float(r[e0 + e]), sbias[c0 + e0 + e]);
                float o1 = __fadd_rn(__uint_as_float(r[e0 + e + 1]), sbias[c0 + e0 + e + 1]);
                if (g.relu) {
                    o0 = fmaxf(o0, 0.0f);
                    o1 = fmaxf(o1, 0.0f);
                }
                h[e / 2] = __floats2bfloat162_rn(o0, o1);
            }
            if (Yh) {
#pragma unroll
                for (int e = 0; e < 16; e += 2) {
                    const float2 f = __bfloat1622float2(h[e / 2]);
                    hsum = __fmaf_rn(f.x, shead[c0 + e0 + e], hsum);
                    hsum = __fmaf_rn(f.y, shead[c0 + e0 + e + 1], hsum);
                }
            } else {
                uint4* d4 = reinterpret_cast<uint4*>(Y + pix * g.Cout + c0 + e0);
                d4[0] = *reinterpret_cast<const uint4*>(&h[0]);
                d4[1] = *reinterpret_cast<const uint4*>(&h[4]);
            }
        }
        if (Yh && c0 + 32 == g.Cout) Yh[pix] = __fadd_rn(hsum, shead[256]);
    }
}

template <bool kUpCat>
__global__ void __launch_bounds__(kWsThreads, 1)
    k_conv3x3_ws(const bf16* __restrict__ X, const bf16* __restrict__ Wp, const float* __restrict__ bias,
                 bf16* __restrict__ Y, const bf16* __restrict__ X2, const float* __restrict__ head_w,
                 const float* __restrict__ head_b, float* __restrict__ Yh, const WsGeom g) {
    extern __shared__ __align__(128) unsigned char ws_raw[];
    unsigned char* sm = ws_raw + ((128 - (smem_u32(ws_raw) & 127)) & 127);
    uint64_t* full = reinterpret_cast<uint64_t*>(sm + g.S * g.sbytes);
    uint64_t* empty = full + kWsMaxStages;
    uint64_t* accf = empty + kWsMaxStages;
    uint64_t* acce = accf + 2;
    unsigned* tslot = reinterpret_cast<unsigned*>(acce + 2);
    volatile int* abort_word = reinterpret_cast<volatile int*>(tslot + 1);
    float* sbias = reinterpret_cast<float*>(tslot + 4);
    float* shead = sbias + 256;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int s = 0; s < g.S; s++) {
            ws_bar_init(&full[s], kWsProd);
            ws_bar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            ws_bar_init(&accf[b], 1);
            ws_bar_init(&acce[b], kWsEpiWarps * 32);
        }
        *abort_word = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int c = tid; c < g.Cout; c += kWsThreads) {
        sbias[c] = bias ? bias[c] : 0.0f;
        shead[c] = head_w ? head_w[c] : 0.0f;
    }
    if (tid == 0) shead[256] = head_b ? *head_b : 0.0f;
    if (warp == 8) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tslot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tslot;
    const int64_t HW = (int64_t)g.H * g.W;
    const int tslots = g.nb * kSlotBlock;

    if (warp >= kWsEpiWarps && warp < kWsEpiWarps + kWsProdWarps) {
        // ---- producers ----
        const int pt = tid - kWsEpiWarps * 32;
        const int chunk = pt & ((1 << g.lgs) - 1);  // this thread's 8-channel plane of every item
        const int step = kWsProd >> g.lgs;          // slots per pass of all producer threads
        const int dq = step / g.P, dr = step - dq * g.P;
        const int slot0 = pt >> g.lgs, hr0 = slot0 / g.P, hc0 = slot0 - hr0 * g.P;
        const int c2 = g.Cin - g.C1;  // channels of X2 (kUpCat)
        const int wchunks = g.wbytes / 16;
        int k = 0;
        bool fail = false;
        for (int t = blockIdx.x; t < g.total && !fail; t += gridDim.x) {
            const int tile = t % g.tps, rest = t / g.tps, seg = rest % g.segs, n = rest / g.segs;
            const int x0 = seg * g.Ws, R0 = tile * tslots / g.P;
            for (int it = 0; it < g.items; it++, k++) {
                const int s = k % g.S, u = k / g.S;
                if (u > 0 && !ws_wait(&empty[s], (u - 1) & 1, abort_word)) {
                    fail = true;
                    break;
                }
                unsigned char* base = sm + s * g.sbytes;
                const int ci0 = 16 * g.gs * it, ci = ci0 + 8 * chunk;
                // Source of this thread's chunk: low-resolution X, X2 (kUpCat) or X,
                // its channel offset and channel count, or none past Cin.
                const bf16* src = X;
                int cs = g.Cin, cl = ci;
                bool lo = false;
                if (kUpCat) {
                    if (ci0 < g.C1) {
                        cs = g.C1;
                        lo = true;
                    } else {
                        src = X2;
                        cs = c2;
                        cl = ci - g.C1;
                    }
                }
                const bool chan_ok = cl < cs;
                unsigned char* dst = base + chunk * g.plane;
                int hr = hr0, hc = hc0;
                for (int p = slot0; p < g.hslots; p += step) {
                    const int iy = R0 - 1 + hr, ix = x0 - 1 + hc;
                    const bool ok = chan_ok && iy >= 0 && iy < g.H && ix >= 0 && ix < g.W;
                    const bf16* a = X;
                    if (ok) {
                        if (kUpCat && lo)
                            a = src + (((int64_t)n * (g.H >> 1) + (iy >> 1)) * (g.W >> 1) + (ix >> 1)) * cs + cl;
                        else
                            a = src + ((int64_t)n * HW + (int64_t)iy * g.W + ix) * cs + cl;
                    }
                    cp_async16(dst + p * 16, a, ok ? 16 : 0);
                    hc += dr;
                    hr += dq;
                    if (hc >= g.P) {
                        hc -= g.P;
                        hr++;
                    }
                }
                unsigned char* wb = base + 2 * g.gs * g.plane;
                const bf16* wsrc = Wp + (int64_t)it * (g.wbytes / 2);
                for (int q = pt; q < wchunks; q += kWsProd) cp_async16(wb + q * 16, wsrc + q * 8, 16);
                // The stage's barrier receives this thread's arrival once its copies have landed.
                asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(&full[s]))
                             : "memory");
            }
        }
        cp_wait_all();
    } else if (warp == kWsEpiWarps + kWsProdWarps) {
        // ---- MMA issuer ----
        if (lane == 0) {
            const uint32_t idesc = tc_idesc(g.Cout);
            uint64_t* last = nullptr;
            int last_par = 0, k = 0, i = 0;
            bool fail = false;
            for (int t = blockIdx.x; t < g.total && !fail; t += gridDim.x, i++) {
                const int b = i & 1, v = i >> 1;
                if (v > 0 && !ws_wait(&acce[b], (v - 1) & 1, abort_word)) break;
                tc_fence_after();
                const int S0 = (t % g.tps) * tslots, soff = S0 - (S0 / g.P) * g.P;
                const unsigned dcol = tmem + (unsigned)(b * 256);
                for (int it = 0; it < g.items; it++, k++) {
                    const int s = k % g.S, u = k / g.S;
                    if (!ws_wait(&full[s], u & 1, abort_word)) {
                        fail = true;
                        break;
                    }
                    // The producers' cp.async writes, now visible to this thread, before
                    // the tensor cores read them through the async proxy.
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    tc_fence_after();
                    const unsigned hb = smem_u32(sm + s * g.sbytes);
                    const unsigned wbs = hb + 2u * g.gs * g.plane;
                    for (int kk = 0; kk < g.gs; kk++) {
                        const uint64_t da0 = tc_desc2(hb + 2u * kk * g.plane, (unsigned)g.plane, 128);
                        const uint64_t db0 = tc_desc2(wbs + (unsigned)(kk * 18 * g.Cout * 16), (unsigned)(g.Cout * 16), 128);
                        for (int j = 0; j < g.nb; j++)
#pragma unroll
                            for (int tap = 0; tap < 9; tap++) {
                                const int ky = tap / 3, kx = tap - 3 * (tap / 3);
                                // start addresses advance in 16-byte units in the descriptors' low field
                                const uint64_t da = da0 + (uint64_t)(soff + j * kSlotBlock + ky * g.P + kx);
                                const uint64_t db = db0 + (uint64_t)(tap * 2 * g.Cout);
                                tc_mma(dcol + (unsigned)(j * g.Cout), da, db, idesc, (it | kk | tap) != 0);
                            }
                    }
                    tc_commit(&empty[s]);
                    last = &empty[s];
                    last_par = u & 1;
                }
                if (fail) break;
                tc_commit(&accf[b]);
                last = &accf[b];
                last_par = v & 1;
            }
            // Issued MMAs finish before the tensor memory is released.
            if (*abort_word && last) tc_mbar_wait(last, last_par);
        }
        __syncwarp();
    } else {
        // ---- epilogue ----
        int i = 0;
        for (int t = blockIdx.x; t < g.total; t += gridDim.x, i++) {
            const int b = i & 1, v = i >> 1;
            if (!ws_wait(&accf[b], v & 1, abort_word)) break;
            tc_fence_after();
            const int tile = t % g.tps, rest = t / g.tps, seg = rest % g.segs, n = rest / g.segs;
            const int x0 = seg * g.Ws, S0 = tile * tslots;
            const unsigned tbase = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(b * 256);
            if (g.Cout % 32 == 0) {
                // Chunks of 32 columns, double-buffered: the next chunk's load is in
                // flight while this one is converted and stored.
                const int cpb = g.Cout / 32, nq = g.nb * cpb;
                unsigned ra[32], rb[32];
                float hsum = 0.0f;
                tc_ld32_issue(tbase, ra);
                tc_ld32_wait(ra);
                for (int q = 0; q < nq; q += 2) {
                    if (q + 1 < nq) tc_ld32_issue(tbase + (unsigned)((q + 1) / cpb * g.Cout + (q + 1) % cpb * 32), rb);
                    ws_epi_chunk(q, cpb, ra, S0, x0, n, HW, warp, lane, g, sbias, shead, Y, Yh, hsum);
                    tc_ld32_wait(rb);
                    if (q + 1 < nq) {
                        if (q + 2 < nq) tc_ld32_issue(tbase + (unsigned)((q + 2) / cpb * g.Cout + (q + 2) % cpb * 32), ra);
                        ws_epi_chunk(q + 1, cpb, rb, S0, x0, n, HW, warp, lane, g, sbias, shead, Y, Yh, hsum);
                        tc_ld32_wait(ra);
                    }
                }
            } else
            for (int j = 0; j < g.nb; j++) {
                const int s = S0 + j * kSlotBlock + warp * 32 + lane;  // this thread's slot (lane)
                const int r = s / g.P, c = s - (s / g.P) * g.P;
                const bool store = r < g.H && c < g.Ws;
                const int64_t pix = (int64_t)n * HW + (int64_t)r * g.W + x0 + c;
                bf16* dst = Y + pix * g.Cout;
                const unsigned taddr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(b * 256 + j * g.Cout);
                float hsum = 0.0f;  // head: sum over channels of bf16(activation) * head_w, in channel order
                for (int c0 = 0; c0 < g.Cout; c0 += 32) {
                    float v[32];
                    const int nc = g.Cout - c0 >= 32 ? 32 : 16;
                    if (nc == 32)
                        tc_ld32(taddr + (unsigned)c0, v);
                    else
                        tc_ld16(taddr + (unsigned)c0, v);
                    if (!store) continue;
                    for (int e0 = 0; e0 < nc; e0 += 16) {
                        __nv_bfloat162 h[8];
#pragma unroll
                        for (int e = 0; e < 16; e += 2) {
                            float o0 = __fadd_rn(v[e0 + e], sbias[c0 + e0 + e]);
                            float o1 = __fadd_rn(v[e0 + e + 1], sbias[c0 + e0 + e + 1]);
                            if (g.relu) {
                                o0 = fmaxf(o0, 0.0f);
                                o1 = fmaxf(o1, 0.0f);
                            }
                            h[e / 2] = __floats2bfloat162_rn(o0, o1);
                        }
                        if (Yh) {
#pragma unroll
                            for (int e = 0; e < 16; e += 2) {
                                const float2 f = __bfloat1622float2(h[e / 2]);
                                hsum = __fmaf_rn(f.x, shead[c0 + e0 + e], hsum);
                                hsum = __fmaf_rn(f.y, shead[c0 + e0 + e + 1], hsum);
                            }
                        } else {
                            uint4* d4 = reinterpret_cast<uint4*>(dst + c0 + e0);
                            d4[0] = *reinterpret_cast<const uint4*>(&h[0]);
                            d4[1] = *reinterpret_cast<const uint4*>(&h[4]);
                        }
                    }
                }
                if (Yh && store) Yh[pix] = __fadd_rn(hsum, shead[256]);
            }
            tc_fence_before();
            ws_arrive(&acce[b]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (tid == 0 && *abort_word) atomicExch(&g_conv_status, 1);
    if (warp == kWsEpiWarps + kWsProdWarps) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
    }
}

// Channels per item for later launches (ske_conv_stage_channels): 0 = the most
// of 64, 32, 16 whose stages fit twice in shared memory.
int g_ws_stage = 0;

// The warp-specialised kernel applies for Cin a multiple of 8, Cout a multiple
// of 16 up to 256, C1 (upsampled channels) a multiple of 16, and at least two
// stages in shared memory.
bool ws_geometry(WsGeom* g, int n, int h, int w_, int cin, int cout, int c1, int relu) {
    if (cin % 8 || cout % 16 || cout < 16 || cout > 256 || c1 % 16) return false;
    g->H = h;
    g->W = w_;
    g->Cin = cin;
    g->Cout = cout;
    g->C1 = c1;
    g->relu = relu;
    g->Ws = halo_seg(w_);
    g->P = g->Ws + 2;
    g->segs = w_ / g->Ws;
    g->nb = ws_blocks(cout);
    g->hslots = halo_slots(g->P, g->nb);
    g->plane = (g->hslots * 16 + 127) / 128 * 128;
    const int groups = (cin + 15) / 16;
    g->S = 0;
    for (int gs = 4; gs >= 1; gs >>= 1) {
        if (g_ws_stage && g_ws_stage != 16 * gs) continue;
        if (gs > 1 && (cin % (16 * gs) || c1 % (16 * gs))) continue;
        const int wbytes = gs * 18 * cout * 16;
        const int sbytes = 2 * gs * g->plane + (wbytes + 127) / 128 * 128;
        const int stages = std::min(kWsMaxStages, (227 * 1024 - kWsExtra) / sbytes);
        if (stages < 2) continue;
        g->gs = gs;
        g->lgs = gs == 4 ? 3 : gs == 2 ? 2 : 1;
        g->items = groups / gs;
        g->wbytes = wbytes;
        g->sbytes = sbytes;
        g->S = stages;
        break;
    }
    if (g->S < 2) return false;
    const int64_t slots = (int64_t)h * g->P;
    const int64_t tps = (slots + g->nb * kSlotBlock - 1) / (g->nb * kSlotBlock);
    const int64_t total = (int64_t)n * g->segs * tps;
    if (total > 0x7fffffff || slots + 4 * g->P > 0x7fffffff / 2) return false;
    g->tps = (int)tps;
    g->total = (int)total;
    return true;
}

// Packs the weights into a stream-ordered temporary (freed after the launch)
// and launches one CTA per SM.  SKE_ERR_UNSUPPORTED if the temporary cannot be
// had (the caller then takes another kernel).
template <bool kUpCat>
int launch_conv_ws(const WsGeom& g, const bf16* x, const bf16* w, const float* bias, bf16* y, const bf16* x2,
                   cudaStream_t st, const float* head_w = nullptr, const float* head_b = nullptr,
                   float* yh = nullptr) {
    const int smem = std::max(kWsMinSmem, g.S * g.sbytes + kWsExtra);
    // Per device, once: the SM count and the kernel's shared-memory limit.
    static std::atomic<int> sm_count[kWsDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return SKE_ERR_CUDA;
    int sms = dev < kWsDevices ? sm_count[dev].load(std::memory_order_relaxed) : 0;
    if (sms < 1) {
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1 ||
            cudaFuncSetAttribute(k_conv3x3_ws<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_conv3x3_ws<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
                cudaSuccess)
            return SKE_ERR_CUDA;
        if (dev < kWsDevices) sm_count[dev].store(sms, std::memory_order_relaxed);
    }
    const int kpad = (9 * g.Cin + kTcBK - 1) / kTcBK * kTcBK;
    const int rows = g.items * g.gs * 18 * g.Cout;  // 16-byte rows of the packed weights
    bf16* wp = nullptr;
    if (cudaMallocAsync(reinterpret_cast<void**>(&wp), (size_t)rows * 16, st) != cudaSuccess) {
        cudaGetLastError();
        return SKE_ERR_UNSUPPORTED;
    }
    k_pack_weights<<<(rows + 255) / 256, 256, 0, st>>>(w, wp, g.Cin, g.Cout, kpad, rows);
    const int grid = std::min(g.total, sms);
    k_conv3x3_ws<kUpCat><<<grid, kWsThreads, smem, st>>>(x, wp, bias, y, x2, head_w, head_b, yh, g);
    const cudaError_t e = cudaGetLastError();
    cudaFreeAsync(wp, st);
    return e == cudaSuccess ? SKE_OK : SKE_ERR_CUDA;
}

// ---- weight gradient on the tensor cores (tcgen05) ---------------------------
//
// dW[co][tap*Cin + ci] = sum over output pixels p of dY[p][co] * X[p + off(tap)][ci].
// The output pixels of a column segment (kWgSeg wide where the width allows)
// are numbered as slots of rows of pitch P = Ws + 2 as in the halo-staged
// forward kernel; a tile is kWgSlots consecutive slots.  Per tile the CTA
// stages dY as 8-channel planes of the tile's slots (zero for the junk slots
// and outside the image) and X as 8-channel halo planes (the rows the tile
// touches, one column on each side, zero outside), and issues for each tap and
// each K step of 16 slots one MMA
//   D_tap (M = 128 output channels, N = 16 or 32 input channels) += dY^T X_tap
// with both operands read in place as MN-major matrices: a core matrix is 8
// consecutive slots of one plane (128 contiguous bytes), 8 channels along M or
// N by 8 slots along K.  Without swizzling the leading byte offset steps along
// K and the stride byte offset along M or N whatever the major-ness, so here
// the leading byte offset is 128 (the next 8 slots) and the stride byte offset
// one plane (the next 8 channels) -- the forward kernel's K-major operands have
// the same two offsets the other way round.  X_tap starts at plane slot
// k*16 + soff + ky*P + kx, the tap's shift.
// The 9 taps' accumulators sit side by side in tensor memory (9 N columns
// each) and sum over all the tiles of the CTA's chunk; the epilogue adds them
// to dW with float32 atomics (warp w: output channels 32w..32w+31 of the CTA's
// block of 128).  dY planes past Cout stay zero (zeroed once).  All threads
// stage a tile with cp.async into a ring of kWgStages stages; thread 0 issues
// its MMAs and commits them to the stage's mbarrier.  Waits are bounded as in
// k_conv3x3; a give-up skips the rest, drains the last commit, frees the tensor
// memory and sets g_conv_status.
constexpr int kWgSeg = 32;
constexpr int kWgSlots = 128;
constexpr int kWgStages = 3;
constexpr int kWgPlanesA = 16;  // 128 output channels

struct WgGeom {
    int H, W, Cin, Cout, Kpad;
    int Ws, P, segs, tps, hslots, total, chunk;
    int nblk;                  // N: input channels per CTA (16 or 32)
    int planeA, planeB, sbytes;  // bytes
};

__host__ __device__ constexpr int wg_seg(int W) { return (W > kWgSeg && W % kWgSeg == 0) ? kWgSeg : W; }

// Instruction descriptor of the weight-gradient MMA: as tc_idesc, with A and B
// MN-major (bits 15 and 16).
__host__ __device__ constexpr uint32_t wg_idesc(int n) { return tc_idesc(n) | (1u << 15) | (1u << 16); }

__global__ void __launch_bounds__(kThreads, 1)
    k_conv3x3_wgrad_tc(const bf16* __restrict__ X, const bf16* __restrict__ dY, float* __restrict__ dW,
                       const WgGeom g) {
    extern __shared__ __align__(128) unsigned char wg_raw[];
    unsigned char* sm = wg_raw + ((128 - (smem_u32(wg_raw) & 127)) & 127);
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + kWgStages * g.sbytes);
    unsigned* tslot = reinterpret_cast<unsigned*>(bar + kWgStages);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ci0 = blockIdx.x * g.nblk, co0 = blockIdx.y * 128;
    const int t0 = blockIdx.z * g.chunk, t1 = min(t0 + g.chunk, g.total);
    if (t0 >= t1) return;  // uniform over the block
    const int coPl = min(kWgPlanesA, (g.Cout - co0 + 7) / 8);  // dY planes with output channels
    const int xPl = g.nblk / 8;
    for (int s = 0; s < kWgStages; s++) {
        uint4* a = reinterpret_cast<uint4*>(sm + s * g.sbytes);
        for (int q = tid; q < kWgPlanesA * g.planeA / 16; q += kThreads) a[q] = make_uint4(0, 0, 0, 0);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tslot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kWgStages; s++) tc_mbar_init(&bar[s]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tslot;
    const int64_t HW = (int64_t)g.H * g.W;

    auto load = [&](int st, int t) {
        unsigned char* base = sm + st * g.sbytes;
        const int tile = t % g.tps, rest = t / g.tps, seg = rest % g.segs, n = rest / g.segs;
        const int x0 = seg * g.Ws, S0 = tile * kWgSlots, R0 = S0 / g.P;
        for (int q = tid; q < coPl * kWgSlots; q += kThreads) {
            const int pl = q / kWgSlots, sl = q - pl * kWgSlots;
            const int s = S0 + sl, r = s / g.P, c = s - r * g.P;
            const bool ok = r < g.H && c < g.Ws && co0 + 8 * pl < g.Cout;
            const bf16* src = ok ? dY + ((int64_t)n * HW + (int64_t)r * g.W + x0 + c) * g.Cout + co0 + 8 * pl : dY;
            cp_async16(base + pl * g.planeA + sl * 16, src, ok ? 16 : 0);
        }
        unsigned char* xb = base + kWgPlanesA * g.planeA;
        for (int q = tid; q < xPl * g.hslots; q += kThreads) {
            const int pl = q / g.hslots, p = q - pl * g.hslots;
            const int hr = p / g.P, iy = R0 - 1 + hr, ix = x0 - 1 + (p - hr * g.P);
            const int ci = ci0 + 8 * pl;
            const bool ok = iy >= 0 && iy < g.H && ix >= 0 && ix < g.W && ci < g.Cin;
            const bf16* src = ok ? X + ((int64_t)n * HW + (int64_t)iy * g.W + ix) * g.Cin + ci : X;
            cp_async16(xb + pl * g.planeB + p * 16, src, ok ? 16 : 0);
        }
    };

    const uint32_t idesc = wg_idesc(g.nblk);
    const int nt = t1 - t0;
    for (int s = 0; s < kWgStages - 1; s++) {
        if (s < nt) load(s, t0 + s);
        cp_commit();
    }
    bool fail = false;
    int last_commit = -1;
    for (int i = 0; i < nt; i++) {
        const int nxt = i + kWgStages - 1;
        if (nxt < nt) {
            const int st = nxt % kWgStages, prev = nxt - kWgStages;
            if (prev >= 0 && !fail) fail = !tc_mbar_wait(&bar[st], (prev / kWgStages) & 1);
            if (!fail) load(st, t0 + nxt);
        }
        cp_commit();
        cp_wait<kWgStages - 1>();
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (__syncthreads_or(fail)) {
            fail = true;
            break;
        }
        if (tid == 0) {
            tc_fence_after();
            const int st = i % kWgStages;
            const int S0 = ((t0 + i) % g.tps) * kWgSlots, soff = S0 - (S0 / g.P) * g.P;
            const unsigned ab = smem_u32(sm + st * g.sbytes), xb = ab + kWgPlanesA * g.planeA;
            const uint64_t da0 = tc_desc2(ab, 128, (unsigned)g.planeA);
            const uint64_t db0 = tc_desc2(xb, 128, (unsigned)g.planeB);
#pragma unroll 1
            for (int tap = 0; tap < 9; tap++) {
                const int ky = tap / 3, kx = tap - 3 * (tap / 3);
#pragma unroll
                for (int k = 0; k < kWgSlots / 16; k++) {
                    // start addresses advance in 16-byte units in the descriptors' low field
                    const uint64_t da = da0 + (uint64_t)(k * 16);
                    const uint64_t db = db0 + (uint64_t)(k * 16 + soff + ky * g.P + kx);
                    tc_mma(tmem + (unsigned)(tap * g.nblk), da, db, idesc, (i | k) != 0);
                }
            }
            tc_commit(&bar[st]);
            last_commit = i;
        }
    }
    cp_wait<0>();
    if (tid == 0 && last_commit >= 0 && !tc_mbar_wait(&bar[last_commit % kWgStages], (last_commit / kWgStages) & 1))
        fail = true;
    fail = __syncthreads_or(fail);
    tc_fence_after();
    if (!fail) {
        const int co = co0 + warp * 32 + lane;
        for (int tap = 0; tap < 9; tap++)
            for (int c0 = 0; c0 < g.nblk; c0 += 16) {
                float v[16];
                tc_ld16(tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(tap * g.nblk + c0), v);
                if (co >= g.Cout) continue;
                float* dst = dW + (int64_t)co * g.Kpad + tap * g.Cin + ci0 + c0;
#pragma unroll
                for (int e = 0; e < 16; e++)
                    if (ci0 + c0 + e < g.Cin) atomicAdd(dst + e, v[e]);
            }
    } else if (tid == 0) {
        atomicExch(&g_conv_status, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
    }
}

// The tensor-core weight gradient for Cout >= 8 (multiple of 8), Cin a
// multiple of 8; false where it does not apply.
bool wg_geometry(WgGeom* g, int n, int h, int w_, int cin, int cout, int sms) {
    g->H = h;
    g->W = w_;
    g->Cin = cin;
    g->Cout = cout;
    g->Kpad = (9 * cin + kTcBK - 1) / kTcBK * kTcBK;
    g->Ws = wg_seg(w_);
    g->P = g->Ws + 2;
    g->segs = w_ / g->Ws;
    g->nblk = cin <= 16 ? 16 : 32;
    g->hslots = 3 * g->P + kWgSlots + 1;
    g->planeA = kWgSlots * 16;
    g->planeB = (g->hslots * 16 + 127) / 128 * 128;
    g->sbytes = kWgPlanesA * g->planeA + (g->nblk / 8) * g->planeB;
    if (kWgStages * g->sbytes + 256 > 227 * 1024) return false;
    const int64_t slots = (int64_t)h * g->P;
    const int64_t tps = (slots + kWgSlots - 1) / kWgSlots;
    const int64_t total = (int64_t)n * g->segs * tps;
    if (total > 0x7fffffff || slots + 4 * g->P > 0x7fffffff / 2) return false;
    g->tps = (int)tps;
    g->total = (int)total;
    const int blocks = ((cin + g->nblk - 1) / g->nblk) * ((cout + 127) / 128);
    const int chunks = (int)std::max<int64_t>(1, std::min<int64_t>(total, (int64_t)2 * sms / std::max(blocks, 1)));
    g->chunk = (int)((total + chunks - 1) / chunks);
    return true;
}

// Weight-gradient kernel (ske_conv_wgrad_select): 0 = tcgen05 where it applies,
// 1 (default) = mma.sync, which measured faster for the surrogate's layers
// (3.22 against 3.75 ms for the 14 layers at batch 16; tcgen05 faster only on
// the 384-channel decoder input).
int g_wgrad_path = 1;

template <bool kUpCat>
int launch_conv_tc(const bf16* x, const bf16* w, const float* bias, bf16* y, int64_t m, int h, int w_, int cin,
                   int cout, int relu, const bf16* x2, int c1, cudaStream_t st) {
    const int n = (int)(m / ((int64_t)h * w_));
    WsGeom geo;
    if (g_conv_path == 0 && aligned(y, 16) && ws_geometry(&geo, n, h, w_, cin, cout, kUpCat ? c1 : 0, relu)) {
        const int r = launch_conv_ws<kUpCat>(geo, x, w, bias, y, x2, st);
        if (r != SKE_ERR_UNSUPPORTED) return r;
    }
    if (halo_applies(w_, cin, cout, kUpCat ? c1 : 0) && aligned(y, 16) && g_conv_path != 1)
        return launch_conv_halo<kUpCat>(x, w, bias, y, (int)(m / ((int64_t)h * w_)), h, w_, cin, cout, relu, x2, c1,
                                        st);
    const int kpad = (9 * cin + kTcBK - 1) / kTcBK * kTcBK;
    const int bn = std::min(kTcMaxBN, (cout + 15) / 16 * 16);
    const int smem = tc_smem_bytes(bn);
    if (cudaFuncSetAttribute(k_conv3x3<kUpCat>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             tc_smem_bytes(kTcMaxBN)) != cudaSuccess)
        return SKE_ERR_CUDA;
    const dim3 grid((unsigned)((m + kTcBM - 1) / kTcBM), (unsigned)((cout + bn - 1) / bn));
    const int vec16 = cout % 8 == 0 && aligned(y, 16);
    k_conv3x3<kUpCat><<<grid, kThreads, smem, st>>>(x, w, bias, y, (int)m, h, w_, cin, cout, kpad, relu, x2, c1, bn,
                                                     vec16);
    return cudaGetLastError() == cudaSuccess ? SKE_OK : SKE_ERR_CUDA;
}

}  // namespace

namespace ske {
int set_last_error(int code, const char* msg);  // engine.cu: the thread's ske_last_error
}  // namespace ske

// A conv entry point's failure: a reason for its status becomes the calling
// thread's last error (ske_last_error), so no earlier call's message is left.
static int conv_result(int rc, const char* fn) {
    if (rc == SKE_OK) return rc;
    const char* why = rc == SKE_ERR_INVALID       ? "invalid argument (a null pointer, a size outside the kernel's "
                                                   "limits or a misaligned tensor)"
                      : rc == SKE_ERR_UNSUPPORTED ? "shape not supported by this kernel"
                      : rc == SKE_ERR_CUDA        ? "a CUDA launch or call failed"
                                                  : "failed";
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", fn, why);
    return ske::set_last_error(rc, buf);
}

static int ske_conv3x3_bf16_impl(const void* x, const void* w, const float* bias, void* y, int n, int h, int w_,
                                int cin, int cout, int relu, void* stream) {
    if (!x || !w || !y || n < 1 || h < 1 || w_ < 1 || cin < 8 || cin % 8 || cout < 2 || cout % 2)
        return SKE_ERR_INVALID;
    if (!aligned(x, 16) || !aligned(w, 16) || !aligned(y, 4) || !aligned(bias, 4)) return SKE_ERR_INVALID;
    const int64_t m = (int64_t)n * h * w_;
    if (m > 0x7fffffff / 2 || (int64_t)cin * 9 > 0x7fffffff / 2) return SKE_ERR_INVALID;
    return launch_conv_tc<false>((const bf16*)x, (const bf16*)w, bias, (bf16*)y, m, h, w_, cin, cout, relu, nullptr,
                                 0, (cudaStream_t)stream);
}

extern "C" int ske_conv3x3_bf16(const void* x, const void* w, const float* bias, void* y, int n, int h, int w_,
                                int cin, int cout, int relu, void* stream) {
    return conv_result(ske_conv3x3_bf16_impl(x, w, bias, y, n, h, w_, cin, cout, relu, stream), "conv3x3_bf16");
}

static int ske_conv3x3_upcat_bf16_impl(const void* xlow, const void* xskip, const void* w, const float* bias, void* y,
                                      int n, int h, int w_, int c1, int c2, int cout, int relu, void* stream) {
    if (!xlow || !xskip || !w || !y || n < 1 || h < 2 || w_ < 2 || h % 2 || w_ % 2 || c1 < 8 || c1 % 8 ||
        c2 < 8 || c2 % 8 || cout < 2 || cout % 2)
        return SKE_ERR_INVALID;
    if (!aligned(xlow, 16) || !aligned(xskip, 16) || !aligned(w, 16) || !aligned(y, 4) || !aligned(bias, 4))
        return SKE_ERR_INVALID;
    const int64_t m = (int64_t)n * h * w_;
    const int cin = c1 + c2;
    if (m > 0x7fffffff / 2 || (int64_t)cin * 9 > 0x7fffffff / 2) return SKE_ERR_INVALID;
    return launch_conv_tc<true>((const bf16*)xlow, (const bf16*)w, bias, (bf16*)y, m, h, w_, cin, cout, relu,
                                (const bf16*)xskip, c1, (cudaStream_t)stream);
}

extern "C" int ske_conv3x3_upcat_bf16(const void* xlow, const void* xskip, const void* w, const float* bias, void* y,
                                      int n, int h, int w_, int c1, int c2, int cout, int relu, void* stream) {
    return conv_result(ske_conv3x3_upcat_bf16_impl(xlow, xskip, w, bias, y, n, h, w_, c1, c2, cout, relu, stream),
                       "conv3x3_upcat_bf16");
}

static int ske_conv3x3_head_bf16_impl(const void* x, const void* w, const float* bias, const float* head_w,
                                     const float* head_b, float* y, int n, int h, int w_, int cin, int cout,
                                     int relu, void* stream) {
    if (!x || !w || !head_w || !head_b || !y || n < 1 || h < 1 || w_ < 1 || cin < 8 || cin % 8 || cout < 16 || cout % 16)
        return SKE_ERR_INVALID;
    if (!aligned(x, 16) || !aligned(w, 16) || !aligned(y, 4) || !aligned(bias, 4) || !aligned(head_w, 4) ||
        !aligned(head_b, 4))
        return SKE_ERR_INVALID;
    const int64_t m = (int64_t)n * h * w_;
    if (m > 0x7fffffff / 2 || (int64_t)cin * 9 > 0x7fffffff / 2) return SKE_ERR_INVALID;
    WsGeom geo;
    if (g_conv_path != 0 || !ws_geometry(&geo, n, h, w_, cin, cout, 0, relu)) return SKE_ERR_UNSUPPORTED;
    return launch_conv_ws<false>(geo, (const bf16*)x, (const bf16*)w, bias, nullptr, nullptr, (cudaStream_t)stream,
                                 head_w, head_b, y);
}

extern "C" int ske_conv3x3_head_bf16(const void* x, const void* w, const float* bias, const float* head_w,
                                     const float* head_b, float* y, int n, int h, int w_, int cin, int cout,
                                     int relu, void* stream) {
    return conv_result(ske_conv3x3_head_bf16_impl(x, w, bias, head_w, head_b, y, n, h, w_, cin, cout, relu, stream),
                       "conv3x3_head_bf16");
}

// 2 x 2 max pooling of NHWC bfloat16 (H, W even, C a multiple of 8): one
// thread per output pixel and 8 channels, four 16-byte loads, NaN propagated
// (as torch.amax).
static __global__ void k_maxpool2(const bf16* __restrict__ X, bf16* __restrict__ Y, int64_t total, int H2, int W2,
                           int C8) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int c8 = (int)(i % C8);
    int64_t rest = i / C8;
    const int x = (int)(rest % W2);
    rest /= W2;
    const int y = (int)(rest % H2);
    const int64_t n = rest / H2;
    const int64_t W = 2 * (int64_t)W2, C = 8 * (int64_t)C8;
    const bf16* p = X + ((n * 2 * H2 + 2 * y) * W + 2 * x) * C + 8 * c8;
    const uint4 q[4] = {*reinterpret_cast<const uint4*>(p), *reinterpret_cast<const uint4*>(p + C),
                        *reinterpret_cast<const uint4*>(p + W * C), *reinterpret_cast<const uint4*>(p + W * C + C)};
    uint4 o;
    const __nv_bfloat162* a = reinterpret_cast<const __nv_bfloat162*>(&q[0]);
    const __nv_bfloat162* b = reinterpret_cast<const __nv_bfloat162*>(&q[1]);
    const __nv_bfloat162* c = reinterpret_cast<const __nv_bfloat162*>(&q[2]);
    const __nv_bfloat162* d = reinterpret_cast<const __nv_bfloat162*>(&q[3]);
    __nv_bfloat162* r = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
    for (int k = 0; k < 4; k++) r[k] = __hmax2_nan(__hmax2_nan(a[k], b[k]), __hmax2_nan(c[k], d[k]));
    reinterpret_cast<uint4*>(Y)[i] = o;
}

static int ske_maxpool2_bf16_impl(const void* x, void* y, int n, int h, int w_, int c, void* stream) {
    if (!x || !y || n < 1 || h < 2 || w_ < 2 || h % 2 || w_ % 2 || c < 8 || c % 8) return SKE_ERR_INVALID;
    if (!aligned(x, 16) || !aligned(y, 16)) return SKE_ERR_INVALID;
    const int64_t total = (int64_t)n * (h / 2) * (w_ / 2) * (c / 8);
    const int64_t blocks = (total + 255) / 256;
    if (blocks > 0x7fffffff) return SKE_ERR_INVALID;
    k_maxpool2<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>((const bf16*)x, (bf16*)y, total, h / 2, w_ / 2,
                                                                   c / 8);
    return cudaGetLastError() == cudaSuccess ? SKE_OK : SKE_ERR_CUDA;
}

extern "C" int ske_maxpool2_bf16(const void* x, void* y, int n, int h, int w_, int c, void* stream) {
    return conv_result(ske_maxpool2_bf16_impl(x, y, n, h, w_, c, stream), "maxpool2_bf16");
}

// Surrogate network input, one thread per cell: channel 0 = (h - mean) /
// (range, or 1 when 0), 1 = log1p(range), 2 = log1p(coarse area of the cell's
// coarse cell) / coarse_scale, 3..7 = 0, each rounded to bfloat16 (the same
// float32 operations as the element-wise tensor expressions).
static __global__ void k_encode(const float* __restrict__ T, const float* __restrict__ mean,
                                const float* __restrict__ range, const float* __restrict__ coarse, int factor,
                                float coarse_scale, bf16* __restrict__ X, int64_t total, int side) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int64_t n = i / ((int64_t)side * side);
    const int rem = (int)(i - n * side * side), y = rem / side, x = rem - (rem / side) * side;
    const float r = range[n];
    const int cs = side / factor;
    const float c = coarse[(n * cs + y / factor) * cs + x / factor];
    __nv_bfloat162 v[4];
    v[0] = __halves2bfloat162(__float2bfloat16_rn(__fdiv_rn(__fsub_rn(T[i], mean[n]), r > 0.0f ? r : 1.0f)),
                              __float2bfloat16_rn(log1pf(r)));
    v[1] = __halves2bfloat162(__float2bfloat16_rn(__fdiv_rn(log1pf(c), coarse_scale)), __float2bfloat16_rn(0.0f));
    v[2] = v[3] = __halves2bfloat162(__float2bfloat16_rn(0.0f), __float2bfloat16_rn(0.0f));
    reinterpret_cast<uint4*>(X)[i] = *reinterpret_cast<const uint4*>(v);
}

static int ske_surrogate_encode_bf16_impl(const float* tiles, const float* mean, const float* range,
                                         const float* coarse, int coarse_factor, float coarse_scale, void* x, int n,
                                         int side, void* stream) {
    // side * side must fit an int (the kernel's cell index within a tile).
    if (!tiles || !mean || !range || !coarse || !x || n < 1 || side < 1 || side > 46340 || coarse_factor < 1 ||
        side % coarse_factor || !(coarse_scale > 0.0f))
        return SKE_ERR_INVALID;
    if (!aligned(x, 16) || !aligned(tiles, 4) || !aligned(coarse, 4)) return SKE_ERR_INVALID;
    const int64_t total = (int64_t)n * side * side;
    const int64_t blocks = (total + 255) / 256;
    if (blocks > 0x7fffffff) return SKE_ERR_INVALID;
    k_encode<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(tiles, mean, range, coarse, coarse_factor,
                                                                 coarse_scale, (bf16*)x, total, side);
    return cudaGetLastError() == cudaSuccess ? SKE_OK : SKE_ERR_CUDA;
}

extern "C" int ske_surrogate_encode_bf16(const float* tiles, const float* mean, const float* range,
                                         const float* coarse, int coarse_factor, float coarse_scale, void* x, int n,
                                         int side, void* stream) {
    return conv_result(ske_surrogate_encode_bf16_impl(tiles, mean, range, coarse, coarse_factor, coarse_scale, x,
                                                      n, side, stream),
                       "surrogate_encode_bf16");
}

static int ske_conv_select_impl(int path) {
    if (path < 0 || path > 2) return SKE_ERR_INVALID;
    g_conv_path = path;
    return SKE_OK;
}

extern "C" int ske_conv_select(int path) {
    return conv_result(ske_conv_select_impl(path), "conv_select");
}

static int ske_conv_wgrad_select_impl(int path) {
    if (path != 0 && path != 1) return SKE_ERR_INVALID;
    g_wgrad_path = path;
    return SKE_OK;
}

extern "C" int ske_conv_wgrad_select(int path) {
    return conv_result(ske_conv_wgrad_select_impl(path), "conv_wgrad_select");
}

static int ske_conv_stage_channels_impl(int channels) {
    if (channels != 0 && channels != 16 && channels != 32 && channels != 64) return SKE_ERR_INVALID;
    g_ws_stage = channels;
    return SKE_OK;
}

extern "C" int ske_conv_stage_channels(int channels) {
    return conv_result(ske_conv_stage_channels_impl(channels), "conv_stage_channels");
}

static int ske_conv_status_impl(int* failed, void* stream) {
    if (!failed) return SKE_ERR_INVALID;
    if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) return SKE_ERR_CUDA;
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_conv_status, sizeof(int)) != cudaSuccess) return SKE_ERR_CUDA;
    if (v) {
        const int zero = 0;
        if (cudaMemcpyToSymbol(g_conv_status, &zero, sizeof(int)) != cudaSuccess) return SKE_ERR_CUDA;
    }
    *failed = v;
    return SKE_OK;
}

extern "C" int ske_conv_status(int* failed, void* stream) {
    return conv_result(ske_conv_status_impl(failed, stream), "conv_status");
}

static int ske_conv3x3_wgrad_bf16_impl(const void* x, const void* dy, float* dw, int n, int h, int w_, int cin,
                                      int cout, void* stream) {
    if (!x || !dy || !dw || n < 1 || h < 1 || w_ < 1 || cin < 8 || cin % 8 || cout < 8 || cout % 8)
        return SKE_ERR_INVALID;
    if (!aligned(x, 16) || !aligned(dy, 16) || !aligned(dw, 4)) return SKE_ERR_INVALID;
    const int64_t m = (int64_t)n * h * w_;
    if (m > 0x7fffffff / 2) return SKE_ERR_INVALID;
    const int kpad = (9 * cin + kBK - 1) / kBK * kBK;
    int dev = 0, sms = 0;
    WgGeom wg;
    if (g_wgrad_path == 0 && cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0 &&
        wg_geometry(&wg, n, h, w_, cin, cout, sms)) {
        const int smem = std::max(kWsMinSmem, kWgStages * wg.sbytes + 256);
        if (cudaFuncSetAttribute(k_conv3x3_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
            return SKE_ERR_CUDA;
        const dim3 g3((unsigned)((cin + wg.nblk - 1) / wg.nblk), (unsigned)((cout + 127) / 128),
                      (unsigned)((wg.total + wg.chunk - 1) / wg.chunk));
        k_conv3x3_wgrad_tc<<<g3, kThreads, smem, (cudaStream_t)stream>>>((const bf16*)x, (const bf16*)dy, dw, wg);
        return cudaGetLastError() == cudaSuccess ? SKE_OK : SKE_ERR_CUDA;
    }
    const dim3 grid((unsigned)((kpad + 63) / 64), (unsigned)((cout + 63) / 64),
                    (unsigned)((m + kWgChunk - 1) / kWgChunk));
    k_conv3x3_wgrad<<<grid, kThreads, 0, (cudaStream_t)stream>>>((const bf16*)x, (const bf16*)dy, dw, (int)m, h, w_,
                                                                 cin, cout, kpad);
    return cudaGetLastError() == cudaSuccess ? SKE_OK : SKE_ERR_CUDA;
}

extern "C" int ske_conv3x3_wgrad_bf16(const void* x, const void* dy, float* dw, int n, int h, int w_, int cin,
                                      int cout, void* stream) {
    return conv_result(ske_conv3x3_wgrad_bf16_impl(x, dy, dw, n, h, w_, cin, cout, stream), "conv3x3_wgrad_bf16");
}
