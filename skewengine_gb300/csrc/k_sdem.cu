// Total-viewshed line-of-sight sweep (kernelSDEM, src/kernelSDEM.h:168-222).
//
// For every valid cell j of a skewed row (the observer) the reference scans the
// row forward (k = j+1 ..) and backward (k = j-1 ..), tracking the horizon slope
// max((S[k] - h)/d) with h = S[j] + POVh; each step is visible when its slope
// beats the horizon, and every visible run that closes before the row end adds
// d_close^2 - d_open^2 to cv.  The output is cv * (float)scale^2.
//
// GB300 mapping
//  * Persistent kernel; a warp takes one work item = (sector slot, skewed row,
//    chunk of 128 consecutive observers) from a global queue ordered longest row
//    first.  Every lane owns 4 consecutive observers.
//  * The row is staged in shared memory once per item; lanes read it through a
//    register sliding window refilled by one aligned 16-byte load per 4 steps,
//    so shared-memory traffic is 1 byte per observer-step.
//  * The step distance d is warp-uniform, so d, RN(1/d), 2d+1 and d+1 come from a
//    constant-memory table.
//  * Division: the quotient (S[k]-h)/d must be the correctly rounded one,
//    because visibility compares it strictly against the running maximum.
//    q0 = RN(a*y), r = fma(-q0, d, a), q = fma(r, y, q0) with y = RN(1/d)
//    (Markstein's correction step, P. Markstein, "Computation of elementary
//    functions on the IBM RISC System/6000 processor", IBM J. R&D 34(1), 1990).
//    It is applied only to rows whose values lie in a range where it is exact
//    for every d <= 4095 (checked exhaustively against IEEE division by the GPU
//    tests); other rows take the IEEE-division path.
//  * Accumulation: with v_t the visibility of step t (distance d_t = t+1) and the
//    last visible run starting at distance rs,
//        cv = 1 + sum_t v_t (2 d_t + 1) - v_end ((n+1)^2 - rs^2),
//    which equals the reference's sum of closed runs (each closed run
//    [o, c) contributes c^2 - o^2 = sum of its ring areas; the +1 and the last
//    term account for the initial run and the run still open at the row end).
//    Per step this needs one predicated add and one predicated move.  All terms
//    are integers below 2^24 for rows up to 4096 cells, so the float result is
//    exact and equal to the reference's.  Longer rows use the reference-order
//    path.
#include <algorithm>
#include <vector>

#include "kernels.h"

namespace ske {

namespace {

constexpr int kChunk = 128;       // observers per work item (4 per lane)
constexpr int kWarps = 8;         // warps per CTA
constexpr int kPadFront = 136;    // zero cells before the row (backward window overrun)
constexpr int kPadBack = 144;     // zero cells after the row (forward window overrun)
constexpr int kFastMaxRow = 4096; // exact float accumulation bound (see header)

// {d, RN(1/d), 2d+1, d+1} for d = 0..4095 (entry 0 unused).
__constant__ float4 c_step[kFastMaxRow];

__host__ __device__ inline int row_capacity(int max_row) {
    return kPadFront + ((max_row + 3) & ~3) + kPadBack;
}

// Values for which the Markstein quotient is exact: zero, or finite with
// magnitude in [2^-80, 2^90].  If S[k] and h both qualify, a = S[k]-h is zero or
// has magnitude in [2^-103, 2^91].
__device__ __forceinline__ bool div_safe(float v) {
    const float m = fabsf(v);
    return v == 0.0f || (m >= 8.271806125530277e-25f && m <= 1.2379400392853803e27f);
}

__device__ __forceinline__ float div_fast(float a, float d, float y) {
    const float q0 = __fmul_rn(a, y);
    const float r = __fmaf_rn(-q0, d, a);
    return __fmaf_rn(r, y, q0);
}

struct Item {
    int slot, row, chunk;
};

__device__ __forceinline__ Item decode(uint64_t it) {
    Item r;
    r.slot = (int)(it >> 48);
    r.row = (int)((it >> 16) & 0xffffffffu);
    r.chunk = (int)(it & 0xffffu);
    return r;
}

// Forward scan of observers x0..x0+3 over A[0..L) (A 16-byte aligned, x0 % 4 == 0),
// fast path.  Returns the four partial cv values.
__device__ __forceinline__ void scan_fwd_fast(const float* __restrict__ A, int x0, int L, float povh,
                                              float cv[4]) {
    int n[4];
    float h[4], mx[4], acc[4], rs[4];
    bool vis[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        n[q] = L - 1 - (x0 + q);
        h[q] = __fadd_rn(A[x0 + q], povh);
        mx[q] = -2000.0f;
        acc[q] = 0.0f;
        rs[q] = 0.0f;
        vis[q] = true;
    }
    const int dmax = __reduce_max_sync(0xffffffffu, max(n[0], 0));
    const float4* A4 = reinterpret_cast<const float4*>(A) + (x0 >> 2);
    float4 cur = A4[0];
    for (int m = 0; 4 * m <= dmax; m++) {
        const float4 nxt = A4[m + 1];
        const float w[8] = {cur.x, cur.y, cur.z, cur.w, nxt.x, nxt.y, nxt.z, nxt.w};
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int d = 4 * m + e;
            if (d == 0 || d > dmax) continue;
            const float4 st = c_step[d];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (d <= n[q]) {
                    const float sl = div_fast(__fsub_rn(w[e + q], h[q]), st.x, st.y);
                    const bool above = sl > mx[q];
                    if (above) {
                        mx[q] = sl;
                        acc[q] = __fadd_rn(acc[q], st.z);
                    } else {
                        rs[q] = st.w;
                    }
                    vis[q] = above;
                }
            }
        }
        cur = nxt;
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if (n[q] < 0) {
            cv[q] = 0.0f;
            continue;
        }
        const float e = (float)(n[q] + 1);
        const float tail = vis[q] ? __fsub_rn(__fmul_rn(e, e), __fmul_rn(rs[q], rs[q])) : 0.0f;
        cv[q] = __fsub_rn(__fadd_rn(1.0f, acc[q]), tail);
    }
}

// Backward scan of observers x0..x0+3 (targets k = x - d), fast path.
__device__ __forceinline__ void scan_bwd_fast(const float* __restrict__ A, int x0, int L, float povh,
                                              float cv[4]) {
    int n[4];
    float h[4], mx[4], acc[4], rs[4];
    bool vis[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        n[q] = (x0 + q < L) ? x0 + q : -1;
        h[q] = __fadd_rn(A[x0 + q], povh);
        mx[q] = -2000.0f;
        acc[q] = 0.0f;
        rs[q] = 0.0f;
        vis[q] = true;
    }
    const int dmax = __reduce_max_sync(0xffffffffu, max(max(n[3], n[2]), max(n[1], max(n[0], 0))));
    const float4* A4 = reinterpret_cast<const float4*>(A) + (x0 >> 2);
    float4 cur = A4[0];
    for (int m = 0; 4 * m <= dmax; m++) {
        const float4 prv = A4[-m - 1];
        const float w[8] = {prv.x, prv.y, prv.z, prv.w, cur.x, cur.y, cur.z, cur.w};
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int d = 4 * m + e;
            if (d == 0 || d > dmax) continue;
            const float4 st = c_step[d];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (d <= n[q]) {
                    const float sl = div_fast(__fsub_rn(w[q - e + 4], h[q]), st.x, st.y);
                    const bool above = sl > mx[q];
                    if (above) {
                        mx[q] = sl;
                        acc[q] = __fadd_rn(acc[q], st.z);
                    } else {
                        rs[q] = st.w;
                    }
                    vis[q] = above;
                }
            }
        }
        cur = prv;
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if (n[q] < 0) {
            cv[q] = 0.0f;
            continue;
        }
        const float e = (float)(n[q] + 1);
        const float tail = vis[q] ? __fsub_rn(__fmul_rn(e, e), __fmul_rn(rs[q], rs[q])) : 0.0f;
        cv[q] = __fsub_rn(__fadd_rn(1.0f, acc[q]), tail);
    }
}

// Reference-order path (kernelSDEM.h:180-218 step for step): IEEE division,
// std::max horizon update, cv accumulated in float forward then backward.
__device__ float scan_reference(const float* __restrict__ A, int x, int L, float povh) {
    const float h = __fadd_rn(A[x], povh);
    float cv = 0.0f;
    for (int dir = 1; dir >= -1; dir -= 2) {
        float mx = -2000.0f, opened = 0.0f;
        bool vis = true;
        const int n = dir > 0 ? L - 1 - x : x;
        for (int s = 1; s <= n; s++) {
            const float d = (float)s;
            const float sl = __fdiv_rn(__fsub_rn(A[x + dir * s], h), d);
            const bool above = sl > mx;
            const bool opening = above && !vis;
            const bool closing = !above && vis;
            vis = above;
            mx = (sl < mx) ? mx : sl;
            if (opening) opened = d;
            if (closing) cv = __fadd_rn(cv, __fsub_rn(__fmul_rn(d, d), __fmul_rn(opened, opened)));
        }
    }
    return cv;
}

__global__ void __launch_bounds__(kWarps * 32) k_sdem(SdemLaunch a) {
    extern __shared__ float4 smem4[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cap = row_capacity(a.max_row);
    float* buf = reinterpret_cast<float*>(smem4) + (size_t)warp * cap;
    float* A = buf + kPadFront;
    for (;;) {
        unsigned idx = 0;
        if (lane == 0) idx = atomicAdd(a.counter, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if ((int64_t)idx >= a.n_items) break;
        const Item it = decode(a.items[idx]);
        const SectorDesc& d = a.g.desc[a.b.angle[it.slot]];
        const int32_t* first = a.g.first + d.row_off;
        const int32_t* last = a.g.last + d.row_off;
        const int f = first[it.row];
        const int L = last[it.row] - f;
        if (L > a.max_row || L <= 0) {
            if (lane == 0) atomicExch(a.status, 1);
            continue;
        }
        const int64_t rowbase = (int64_t)it.row * d.dim_i + f;  // flat index of the row start
        const float* src = a.SI + it.slot * a.stride + rowbase;
        bool ok = true;
        for (int x = lane; x < L; x += 32) {
            const float v = src[x];
            A[x] = v;
            ok = ok && div_safe(v) && div_safe(__fadd_rn(v, a.povh));
        }
        for (int x = lane; x < kPadFront; x += 32) buf[x] = 0.0f;
        const int tail_end = ((L + 3) & ~3) + kPadBack;
        for (int x = L + lane; x < tail_end; x += 32) A[x] = 0.0f;
        const bool fast = __all_sync(0xffffffffu, ok) && L <= kFastMaxRow && div_safe(a.povh);
        __syncwarp();

        const int x0 = it.chunk * kChunk + 4 * lane;
        float cv[4];
        if (fast) {
            float cb[4];
            scan_fwd_fast(A, x0, L, a.povh, cv);
            scan_bwd_fast(A, x0, L, a.povh, cb);
#pragma unroll
            for (int q = 0; q < 4; q++) cv[q] = __fadd_rn(cv[q], cb[q]);
        } else {
#pragma unroll
            for (int q = 0; q < 4; q++) cv[q] = (x0 + q < L) ? scan_reference(A, x0 + q, L, a.povh) : 0.0f;
        }
        float* out = a.SO + it.slot * a.stride;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int x = x0 + q;
            if (x >= L) continue;
            const int64_t p = rowbase + x;
            if (owner_row(d, first, last, p) != it.row) continue;
            out[p] = a.counts_only ? cv[q] : __fmul_rn(cv[q], d.r2);
        }
        __syncwarp();
    }
}

// Exhaustive check of div_fast against IEEE division: every float bit pattern a
// with div_safe-compatible magnitude (zero or |a| in [2^-103, 2^91], the range
// of S[k]-h when both operands pass div_safe) and every d in [1, dmax].
__global__ void k_div_check(int dmax, unsigned long long* checked, unsigned long long* bad,
                            unsigned* first_bad) {
    unsigned long long n_ok = 0, n_bad = 0;
    for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < (1ull << 32);
         u += (uint64_t)gridDim.x * blockDim.x) {
        const float a = __uint_as_float((unsigned)u);
        const float m = fabsf(a);
        // 0x0c000000 = 2^-103, 0x6d000000 = 2^91; NaN fails both comparisons.
        if (!(a == 0.0f || (m >= __uint_as_float(0x0c000000u) && m <= __uint_as_float(0x6d000000u)))) continue;
        for (int d = 1; d <= dmax; d++) {
            const float4 st = c_step[d];
            const float q = div_fast(a, st.x, st.y);
            const float ref = __fdiv_rn(a, st.x);
            if (__float_as_uint(q) != __float_as_uint(ref) && !(q == 0.0f && ref == 0.0f)) {
                n_bad++;
                atomicCAS(first_bad, 0xffffffffu, (unsigned)u);
            }
            n_ok++;
        }
    }
    atomicAdd(checked, n_ok);
    if (n_bad) atomicAdd(bad, n_bad);
}

}  // namespace

cudaError_t sdem_division_selftest(int dmax, int num_sms, unsigned long long* h_checked,
                                   unsigned long long* h_bad, unsigned* h_first_bad) {
    if (dmax < 1 || dmax >= kFastMaxRow) return cudaErrorInvalidValue;
    unsigned long long* d_cnt = nullptr;
    unsigned* d_first = nullptr;
    cudaError_t e = cudaMalloc(&d_cnt, 2 * sizeof(unsigned long long));
    if (e != cudaSuccess) return e;
    e = cudaMalloc(&d_first, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(d_cnt, 0, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(d_first, 0xff, sizeof(unsigned));
    if (e == cudaSuccess) {
        k_div_check<<<num_sms * 8, 256>>>(dmax, d_cnt, d_cnt + 1, d_first);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    unsigned long long cnt[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(h_first_bad, d_first, sizeof(unsigned), cudaMemcpyDeviceToHost);
    *h_checked = cnt[0];
    *h_bad = cnt[1];
    cudaFree(d_cnt);
    cudaFree(d_first);
    return e;
}

int sdem_chunk() { return kChunk; }

cudaError_t sdem_init_tables() {
    std::vector<float4> tab(kFastMaxRow);
    for (int d = 0; d < kFastMaxRow; d++) {
        const float df = (float)d;
        tab[d] = make_float4(df, d ? 1.0f / df : 0.0f, 2.0f * df + 1.0f, df + 1.0f);
    }
    return cudaMemcpyToSymbol(c_step, tab.data(), sizeof(float4) * kFastMaxRow);
}

void sdem_items(const Geometry& geo, const Batch& b, std::vector<uint64_t>& items, int* max_row) {
    // Counting sort of rows by valid length, longest first: every chunk of a row
    // costs about L + 126 warp steps, so long rows go first.
    int lmax = 0;
    for (int s = 0; s < b.count; s++) {
        const SectorDesc& d = geo.desc[b.angle[s]];
        for (int r = 0; r < d.H; r++) lmax = std::max(lmax, geo.last[d.row_off + r] - geo.first[d.row_off + r]);
    }
    std::vector<int64_t> bucket(lmax + 2, 0);
    for (int s = 0; s < b.count; s++) {
        const SectorDesc& d = geo.desc[b.angle[s]];
        for (int r = 0; r < d.H; r++) {
            const int L = geo.last[d.row_off + r] - geo.first[d.row_off + r];
            if (L > 0) bucket[L] += (L + kChunk - 1) / kChunk;
        }
    }
    std::vector<int64_t> start(lmax + 2, 0);
    int64_t total = 0;
    for (int L = lmax; L >= 1; L--) {
        start[L] = total;
        total += bucket[L];
    }
    items.assign(total, 0);
    for (int s = 0; s < b.count; s++) {
        const SectorDesc& d = geo.desc[b.angle[s]];
        for (int r = 0; r < d.H; r++) {
            const int L = geo.last[d.row_off + r] - geo.first[d.row_off + r];
            if (L <= 0) continue;
            const int nc = (L + kChunk - 1) / kChunk;
            for (int c = 0; c < nc; c++)
                items[start[L]++] = ((uint64_t)s << 48) | ((uint64_t)(uint32_t)r << 16) | (uint64_t)c;
        }
    }
    *max_row = lmax;
}

cudaError_t launch_sdem(const SdemLaunch& a, int num_sms, cudaStream_t st) {
    if (a.n_items == 0) return cudaSuccess;
    const size_t smem = sizeof(float) * (size_t)row_capacity(a.max_row) * kWarps;
    cudaError_t e = cudaFuncSetAttribute(k_sdem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sdem, kWarps * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int64_t blocks = (int64_t)per_sm * num_sms;
    const int64_t need = (a.n_items + kWarps - 1) / kWarps;
    if (blocks > need) blocks = need;
    e = cudaMemsetAsync(a.counter, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    k_sdem<<<(int)blocks, kWarps * 32, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace ske
