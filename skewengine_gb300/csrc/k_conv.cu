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
#include <cuda_bf16.h>

#include <algorithm>
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
// blocks at row pitch P = Ws + 2: enough rows for every tap of every output slot.
__host__ __device__ constexpr int halo_seg(int W) { return (W > 128 && W % 128 == 0) ? 128 : W; }
__host__ __device__ constexpr int halo_slots(int P, int nb) { return 3 * P + nb * kSlotBlock; }
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

// Forward-convolution kernel choice (ske_conv_select): 0 = halo-staged where it
// applies, 1 = always the im2col kernel.
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

template <bool kUpCat>
int launch_conv_tc(const bf16* x, const bf16* w, const float* bias, bf16* y, int64_t m, int h, int w_, int cin,
                   int cout, int relu, const bf16* x2, int c1, cudaStream_t st) {
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

extern "C" int ske_conv3x3_bf16(const void* x, const void* w, const float* bias, void* y, int n, int h, int w_,
                                int cin, int cout, int relu, void* stream) {
    if (!x || !w || !y || n < 1 || h < 1 || w_ < 1 || cin < 8 || cin % 8 || cout < 2 || cout % 2)
        return SKE_ERR_INVALID;
    if (!aligned(x, 16) || !aligned(w, 16) || !aligned(y, 4) || !aligned(bias, 4)) return SKE_ERR_INVALID;
    const int64_t m = (int64_t)n * h * w_;
    if (m > 0x7fffffff / 2 || (int64_t)cin * 9 > 0x7fffffff / 2) return SKE_ERR_INVALID;
    return launch_conv_tc<false>((const bf16*)x, (const bf16*)w, bias, (bf16*)y, m, h, w_, cin, cout, relu, nullptr,
                                 0, (cudaStream_t)stream);
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
    return launch_conv_tc<true>((const bf16*)xlow, (const bf16*)w, bias, (bf16*)y, m, h, w_, cin, cout, relu,
                                (const bf16*)xskip, c1, (cudaStream_t)stream);
}

extern "C" int ske_conv_select(int path) {
    if (path != 0 && path != 1) return SKE_ERR_INVALID;
    g_conv_path = path;
    return SKE_OK;
}

extern "C" int ske_conv_status(int* failed, void* stream) {
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
