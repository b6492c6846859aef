// Total-viewshed line-of-sight sweep (kernelSDEM, src/kernelSDEM.h:168-222).
//
// For every valid cell j of a skewed row (the observer) the reference scans the
// row forward (k = j+1 ..) and backward (k = j-1 ..), tracking the horizon slope
// max((S[k] - h)/d) with h = S[j] + POVh; each step is visible when its slope
// beats the horizon, and every visible run that closes before the row end adds
// d_close^2 - d_open^2 to cv.  The output is cv * (float)scale^2.
//
// Two sweeps share the arithmetic below.
//
// Compacting sweep (k_sdem, the engine's)
//  * Persistent kernel; a warp takes one skewed row (sector slot, row) from a
//    global queue ordered longest row first and scans it in both directions.
//  * Work proceeds in levels of kLevel steps.  Level 0 takes every observer of
//    the row; after each level an exact horizon test (below) retires the
//    observers that can see nothing further, and the survivors are appended to a
//    per-warp list (one per direction) in global scratch.  The next level
//    processes only those lists, in batches of 64 observers (2 per lane): full
//    batches of one direction, then the two lists' remainders paired (a forward
//    observer in slot 0, a backward one in slot 1).  An observer's work
//    therefore ends within kLevel steps of the test that retires it, instead of
//    with the slowest of a fixed group: on 2000x2000 fractal terrain this runs
//    about 22% of the line-of-sight steps (counting empty slots), against 68%
//    for the chunked sweep.  64-step levels measured faster than 32 or 128
//    (fewer list passes against more steps past an observer's end).
//  * All observers of a batch are at the same step distance d, so -d, RN(1/d)
//    and 2d+1 still come from the constant table; each lane reads its two
//    observers' targets with one shared-memory load per step each, and computes
//    both slopes with packed f32x2 instructions.
//  * Each direction's count of an observer goes to a per-warp scratch array;
//    after the last level the two are added (forward + backward, integers below
//    2^24) and scaled into the output cell.
//
// Chunked sweep (k_sdem_chunked, the allocation-free entry point's)
//  * Persistent kernel; a warp takes one work item = (sector slot, skewed row,
//    chunk of 128 consecutive observers) from a global queue ordered longest row
//    first.  Every lane owns 4 consecutive observers.
//  * The row is staged in shared memory once per item; lanes read it through a
//    register sliding window refilled by one aligned 16-byte load per 4 steps,
//    so shared-memory traffic is 1 byte per observer-step.
//  * The step distance d is warp-uniform, so -d, RN(1/d) and 2d+1 come from a
//    constant-memory table.  The slopes of two observers at a time use packed
//    f32x2 instructions.
//
// Common to both
//  * Division: the quotient (S[k]-h)/d must be the correctly rounded one,
//    because visibility compares it strictly against the running maximum.
//    q0 = RN(a*y), r = fma(q0, -d, a), q = fma(r, y, q0) with y = RN(1/d)
//    (Markstein's correction step, P. Markstein, "Computation of elementary
//    functions on the IBM RISC System/6000 processor", IBM J. R&D 34(1), 1990).
//    It is applied only to rows whose values lie in a range where it is exact
//    for every d <= 4095 (checked exhaustively against IEEE division by
//    ske_selftest_division); other rows take the IEEE-division path.
//  * Accumulation: a closed visible run [o, c) contributes c^2 - o^2 to the
//    reference's cv, which is the sum of the ring areas 2d+1 over its steps
//    d = o .. c-1.  So each visible step adds 2d+1 to a running sum acc, and
//    every invisible step (the one that closes a run, or any later one) copies
//    acc into cl, the sum over closed runs.  The initial run starts at distance
//    0 (ring 1 not swept), hence cl starts at -1 and cv = 1 + cl; a run still
//    open at the row end never reaches cl, exactly as the reference does not
//    count it.  All values are integers below 2^24 for rows up to 4096 cells,
//    so the float result is exact and equal to the reference's.  Longer rows
//    use the reference-order path.
//  * Horizon pruning (exact): after step d the remaining targets (distances
//    d+1 .. n) are all invisible when the bound b = fl(a/(d+1)) for a >= 0, or
//    b = fl(a/n) for a < 0, is at most the horizon, with a = fl(Smax - h) and
//    Smax an upper bound of the remaining heights.  Rounding is monotonic, so
//    every remaining slope fl(fl(S[k]-h)/d') is at most fl(a/d'), and a/d' is
//    largest at d' = d+1 when a >= 0 and at d' = n when a < 0.  An observer that
//    passes is finished: every later step would be invisible, so cv = 1 + sum
//    (its last run closes at the next step).  The chunked sweep takes Smax
//    from per-8-cell suffix (forward) and prefix (backward) maxima, tests every
//    kCheck steps with the a >= 0 bound and stops a warp when all its observers
//    are finished.  The compacting sweep tests each observer after every level
//    against 16-cell, 128-cell and suffix (prefix) maxima (see retire).
#include <algorithm>
#include <vector>

#include "kernels.h"

namespace ske {

namespace {

constexpr int kChunk = 128;        // observers per work item (4 per lane)
constexpr int kWarps = 8;          // warps per CTA
constexpr int kPadFront = 136;     // zero cells before the row (backward window overrun)
constexpr int kPadBack = 144;      // zero cells after the row (forward window overrun)
constexpr int kFastMaxRow = 4096;  // exact float accumulation bound (see header)
constexpr int kBlk = 8;            // cells per block of the pruning maxima
constexpr int kCheck = 32;         // steps between pruning tests (multiple of 4)

// {-d, RN(1/d), 2d+1, d+1} for d = 0..4095 (entry 0 unused).
__constant__ float4 c_step[kFastMaxRow];

__host__ __device__ inline int row_pad(int max_row) { return kPadFront + ((max_row + 3) & ~3) + kPadBack; }
__host__ __device__ inline int blocks_pad(int max_row) { return ((max_row + kBlk - 1) / kBlk + 3) & ~3; }
// Shared floats per warp: the padded row plus suffix and prefix block maxima.
__host__ __device__ inline int warp_floats(int max_row) { return row_pad(max_row) + 2 * blocks_pad(max_row); }

// Values for which the Markstein quotient is exact: zero, or finite with
// magnitude in [2^-80, 2^90].  If S[k] and h both qualify, a = S[k]-h is zero or
// has magnitude in [2^-103, 2^91].
__device__ __forceinline__ bool div_safe(float v) {
    const float m = fabsf(v);
    return v == 0.0f || (m >= 8.271806125530277e-25f && m <= 1.2379400392853803e27f);
}

__device__ __forceinline__ float div_fast(float a, float negd, float y) {
    const float q0 = __fmul_rn(a, y);
    const float r = __fmaf_rn(q0, negd, a);
    return __fmaf_rn(r, y, q0);
}

// Packed pairs of floats for the f32x2 instructions: two independent IEEE
// operations, round to nearest, no flush to zero.
typedef unsigned long long f2;
__device__ __forceinline__ f2 pk(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1,%2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk(f2 v, float& a, float& b) { asm("mov.b64 {%0,%1}, %2;" : "=f"(a), "=f"(b) : "l"(v)); }
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
// Both halves of a/d correctly rounded (div_fast on each half).
__device__ __forceinline__ f2 div2(f2 a, f2 negd, f2 y) {
    const f2 q0 = mul2(a, y);
    return fma2(fma2(q0, negd, a), y, q0);
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

// State of the 4 observers of a lane in one scan direction.  acc is the ring
// sum of all visible steps; cl is acc at the last invisible step, i.e. the ring
// sum of the closed runs (-1 before any: the initial run starts at distance 0).
struct Scan4 {
    float h[4], mx[4], acc[4], cl[4];
    int n[4];        // steps of each observer (-1: observer outside the row)
    bool done[4];    // finished by pruning
};

// One block of 4 steps d = d0 .. d0+3.  The window holds the 8 row values the
// block needs: forward w = A[x0+d0 .. x0+d0+7], step e of observer q reads
// w[e+q]; backward w = A[x0-d0-4 .. x0-d0+3], step e reads w[q-e+4].  Slopes of
// observer pairs (0,1) and (2,3) use packed f32x2 operations; the horizon test,
// the horizon update and the two sums are per observer.
template <bool kFwd, bool kTail>
__device__ __forceinline__ void block4(Scan4& s, const float w[8], int d0) {
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int d = d0 + e;
        if (d == 0) continue;  // only in the first block
        const float4 st = c_step[d];
        const f2 nd2 = pk(st.x, st.x), y2 = pk(st.y, st.y);
        const float ring = st.z;
        float qv[4];
#define SKE_W(q) (kFwd ? w[e + (q)] : w[(q)-e + 4])
        upk(div2(sub2(pk(SKE_W(0), SKE_W(1)), pk(s.h[0], s.h[1])), nd2, y2), qv[0], qv[1]);
        upk(div2(sub2(pk(SKE_W(2), SKE_W(3)), pk(s.h[2], s.h[3])), nd2, y2), qv[2], qv[3]);
#undef SKE_W
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (kTail && d > s.n[q]) continue;
            const bool above = qv[q] > s.mx[q];
            s.mx[q] = above ? qv[q] : s.mx[q];
            s.cl[q] = above ? s.cl[q] : s.acc[q];
            s.acc[q] = above ? __fadd_rn(s.acc[q], ring) : s.acc[q];
        }
    }
}

// Pruning test after step dc for the 4 observers: smax is an upper bound of
// every remaining target height of all four.
__device__ __forceinline__ void prune4(Scan4& s, float smax, int dc) {
    const float4 st = c_step[dc + 1];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const float a = __fsub_rn(smax, s.h[q]);
        const float b = div_fast(a, st.x, st.y);
        s.done[q] = s.done[q] || (dc < s.n[q] && a >= 0.0f && b <= s.mx[q]);
    }
}

// Scan of the lane's observers x0..x0+3 in one direction (fast path).
// A: the row (16-byte aligned, zero padded), bmax: suffix (forward) or prefix
// (backward) maxima of kBlk-cell blocks.
template <bool kFwd>
__device__ __forceinline__ void scan_fast(const float* __restrict__ A, const float* __restrict__ bmax, int x0, int L,
                                          float povh, float cv[4]) {
    Scan4 s;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int x = x0 + q;
        s.n[q] = x < L ? (kFwd ? L - 1 - x : x) : -1;
        s.h[q] = __fadd_rn(A[x], povh);
        s.mx[q] = -2000.0f;
        s.acc[q] = 0.0f;
        s.cl[q] = -1.0f;
        s.done[q] = false;
    }
    // Steps every observer of the warp takes (no bounds test) and the most any takes.
    const int lane_min = kFwd ? s.n[3] : s.n[0];
    const int lane_max = max(max(s.n[0], s.n[1]), max(max(s.n[2], s.n[3]), 0));
    const int dmain = __reduce_min_sync(0xffffffffu, lane_min < 0 ? 0 : lane_min);
    const int dall = __reduce_max_sync(0xffffffffu, lane_max);
    const float4* A4 = reinterpret_cast<const float4*>(A) + (x0 >> 2);
    float4 cur = A4[0];
    for (int m = 0; 4 * m <= dall; m++) {
        const float4 nx = kFwd ? A4[m + 1] : A4[-m - 1];
        const float4 lo = kFwd ? cur : nx, hi = kFwd ? nx : cur;
        const float w[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
        if (4 * m + 3 <= dmain) block4<kFwd, false>(s, w, 4 * m);
        else block4<kFwd, true>(s, w, 4 * m);
        cur = nx;
        const int dc = 4 * m + 3;
        if ((dc + 1) % kCheck == 0 && dc < dall) {
            // Remaining targets: forward x+dc+1 .., backward .. x-dc-1 (all four
            // observers' targets lie on the same side of the bound's block).
            // Backward: the lane's largest in-row observer bounds its targets.
            const int k = kFwd ? x0 + dc + 1 : min(x0 + 3, L - 1) - dc - 1;
            if (kFwd ? k < L : k >= 0) prune4(s, bmax[k / kBlk], dc);
            bool fin = true;
#pragma unroll
            for (int q = 0; q < 4; q++) fin = fin && (s.done[q] || dc >= s.n[q]);
            if (__all_sync(0xffffffffu, fin)) break;
        }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if (s.n[q] < 0) {
            cv[q] = 0.0f;
            continue;
        }
        // A pruned observer's open run closes at its next step: every run counts.
        cv[q] = __fadd_rn(1.0f, s.done[q] ? s.acc[q] : s.cl[q]);
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

// Block maxima for pruning: suf[b] = max A[kBlk*b ..] (to the row end),
// pre[b] = max A[.. kBlk*b + kBlk-1] (from the row start).  Rows on the fast
// path are finite.
__device__ void block_maxima(const float* __restrict__ A, int L, float* suf, float* pre, int lane) {
    const float ninf = __int_as_float(0xff800000);
    const int nb = (L + kBlk - 1) / kBlk;
    const int per = (nb + 31) / 32;
    const int b0 = lane * per, b1 = min(b0 + per, nb);
    float run = ninf;
    for (int b = b0; b < b1; b++) {  // block maxima, then lane-local prefix
        float m = ninf;
        for (int c = b * kBlk; c < min(b * kBlk + kBlk, L); c++) m = fmaxf(m, A[c]);
        suf[b] = m;
        run = fmaxf(run, m);
        pre[b] = run;
    }
    // Inclusive prefix / suffix max of the lane totals (Hillis-Steele), then
    // shift by one lane for the exclusive values.
    float inc_p = run, inc_s = run;
    for (int off = 1; off < 32; off <<= 1) {
        const float up = __shfl_up_sync(0xffffffffu, inc_p, off);
        const float dn = __shfl_down_sync(0xffffffffu, inc_s, off);
        if (lane >= off) inc_p = fmaxf(inc_p, up);
        if (lane + off < 32) inc_s = fmaxf(inc_s, dn);
    }
    float before = __shfl_up_sync(0xffffffffu, inc_p, 1);
    float after = __shfl_down_sync(0xffffffffu, inc_s, 1);
    if (lane == 0) before = ninf;
    if (lane == 31) after = ninf;
    float r = after;
    for (int b = b1 - 1; b >= b0; b--) {
        r = fmaxf(r, suf[b]);
        suf[b] = r;
    }
    for (int b = b0; b < b1; b++) pre[b] = fmaxf(pre[b], before);
}

__global__ void __launch_bounds__(kWarps * 32) k_sdem_chunked(SdemLaunch a) {
    extern __shared__ float4 smem4[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wf = warp_floats(a.max_row);
    float* buf = reinterpret_cast<float*>(smem4) + (size_t)warp * wf;
    float* A = buf + kPadFront;
    float* suf = buf + row_pad(a.max_row);
    float* pre = suf + blocks_pad(a.max_row);
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
        if (fast) {
            block_maxima(A, L, suf, pre, lane);
            __syncwarp();
        }

        const int x0 = it.chunk * kChunk + 4 * lane;
        float cv[4];
        if (fast) {
            float cb[4];
            scan_fast<true>(A, suf, x0, L, a.povh, cv);
            scan_fast<false>(A, pre, x0, L, a.povh, cb);
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

// ---- compacting sweep --------------------------------------------------------

constexpr int kLevel = 64;  // line-of-sight steps per level
constexpr int kUnroll = 8;  // steps per unrolled block of a level
constexpr int kSlots = 2;   // observers per lane in a batch (one packed pair)
static_assert(kLevel % kUnroll == 0, "a level is whole blocks");
constexpr int kLWarps = 4;  // warps per CTA
// Per-warp scratch, in units of max_row int4 entries: four survivor lists and
// the two directions' counts (2*max_row floats, within one more unit).
constexpr int kListsPerWarp = 5;
constexpr int kLPad = 64;   // NaN cells on both sides of the row (>= kLevel - 1)
// Longest row on the fast path: every step distance a level touches (at most
// the last survivor's n + kLevel) stays inside the constant table.
constexpr int kLFastMaxRow = kFastMaxRow - kLevel;
static_assert(kSlots == 2, "level_steps packs exactly one pair per lane");

// {-n, RN(1/n)} for n = 0..4095, for lane-divergent lookups (the a < 0 bound).
__device__ float2 g_recip[kFastMaxRow];

// Retirement bound terms: kT blocks of kB1 cells, then kT blocks of kB2 cells,
// then the suffix (prefix) maximum of everything beyond.
constexpr int kB1 = 16, kB1Log = 4;
constexpr int kB2 = 128, kB2Log = 7;
constexpr int kT = 4;
constexpr int kMPad = 8;  // -inf entries on both sides of the kB1 and kB2 maxima
// 1 - 2^-20: the factor that keeps fl(fl(mx * kShrink) * ds) below mx * ds.
constexpr float kShrink = 0.99999904632568359375f;

__host__ __device__ inline int lrow_pad(int max_row) { return kLPad + ((max_row + 3) & ~3) + kLPad; }
__host__ __device__ inline int nblk(int max_row, int size) { return (max_row + size - 1) / size; }

// Per-warp shared memory of the compacting sweep, in floats from the warp's base:
// the padded row; suffix maxima of kB2-cell blocks (one -inf entry after);
// prefix maxima of kB2-cell blocks (one -inf entry before); kB1-cell and
// kB2-cell block maxima (kMPad -inf entries on both sides).  About 1.17 floats
// per cell of the longest row: 2335 per warp at 2000 cells, so six 4-warp CTAs
// share an SM's 228 KB.
struct LLayout {
    int s128, p128, b16, b128, total;
    __host__ __device__ explicit LLayout(int max_row) {
        const int n16 = nblk(max_row, kB1), n128 = nblk(max_row, kB2);
        s128 = lrow_pad(max_row);
        p128 = s128 + n128 + 2;
        b16 = p128 + n128 + kMPad;
        b128 = b16 + n16 + 2 * kMPad;
        total = b128 + n128 + kMPad;
    }
};

// The block maxima of the row being swept.
struct RowMax {
    const float *s128, *p128, *b16, *b128;
    int n128;
};

// One lane's two observers of a batch.  Slot q scans forward when the batch's
// template flag for it is set, backward otherwise.
struct Slots {
    int x[kSlots];  // position in the row
    int n[kSlots];  // steps in the slot's direction
    bool valid[kSlots];  // false: empty slot (its steps run, its state is dropped)
    float h[kSlots], mx[kSlots], acc[kSlots], cl[kSlots];
};

// Visibility update.  The comparison is unordered (true for a NaN slope): a
// step past the observer's last target reads the row's NaN padding, counts as
// visible and so leaves cl, the only value a finished observer keeps, as it
// was.  For finite slopes it is the reference's sl > mx.
__device__ __forceinline__ void visit(Slots& s, int q, float sl, float ring) {
    const bool above = !(sl <= s.mx[q]);
    s.mx[q] = above ? sl : s.mx[q];
    s.cl[q] = above ? s.cl[q] : s.acc[q];
    s.acc[q] = above ? __fadd_rn(s.acc[q], ring) : s.acc[q];
}

// Steps d0 .. d0+kLevel-1 of the lane's two observers (directions kF0, kF1).
// An observer that ends inside the level reads at most kLevel-1 cells of the
// row's NaN padding (see visit).  The level runs as a loop over blocks of
// kUnroll steps: fully unrolled levels overflow the instruction cache.
// kLen > 0: a compile-time level length; kLen = 0: the run-time length len.
template <bool kF0, bool kF1, int kLen>
__device__ __forceinline__ void level_steps(Slots& s, const float* __restrict__ A, int d0, int len) {
    const float* p0 = A + (kF0 ? s.x[0] + d0 : s.x[0] - d0);
    const float* p1 = A + (kF1 ? s.x[1] + d0 : s.x[1] - d0);
    const f2 hh = pk(s.h[0], s.h[1]);
    const int steps = kLen > 0 ? kLen : len;
#pragma unroll 1
    for (int k0 = 0; k0 < steps; k0 += kUnroll) {
#pragma unroll
        for (int k = 0; k < kUnroll; k++) {
            const int d = d0 + k0 + k;
            const float4 st = c_step[d];
            const float z0 = kF0 ? p0[k] : p0[-k];
            const float z1 = kF1 ? p1[k] : p1[-k];
            float q0, q1;
            upk(div2(sub2(pk(z0, z1), hh), pk(st.x, st.x), pk(st.y, st.y)), q0, q1);
            visit(s, 0, q0, st.z);
            visit(s, 1, q1, st.z);
        }
        p0 += kF0 ? kUnroll : -kUnroll;
        p1 += kF1 ? kUnroll : -kUnroll;
    }
}

// Where a row's results go.
struct RowOut {
    float* out;           // the sector's output grid
    int64_t rowbase;      // flat index of the row's first valid cell
    int first;            // its column
    int row;
    const SectorDesc* sd;
    const int32_t* rfirst;
    const int32_t* rlast;
    int counts_only;
    bool compact;         // batched run: the row's cells are its own compact row
};

// Cells that lie in the row's own span of the flat grid (column < dim_i) are
// always the row's; cells past it may belong to a later row (owner_row).  A
// compact row (batched runs) owns all its cells.
__device__ __forceinline__ bool owns(const RowOut& o, int x) {
    return o.compact || o.first + x < o.sd->dim_i || owner_row(*o.sd, o.rfirst, o.rlast, o.rowbase + x) == o.row;
}

// The maxima arrays of a fast-path row (finite, at most 32 * kB2 cells, so one
// kB2 block per lane): kB1- and kB2-cell block maxima with their -inf padding,
// s128[b] = max A[kB2*b ..] to the row end (s128[n128] = -inf) and
// p128[b] = max A[.. kB2*b + kB2-1] from the row start (p128[-1] = -inf).
__device__ void row_maxima(const float* __restrict__ A, int L, float* s128, float* p128, float* b16, float* b128,
                           int lane) {
    const float ninf = __int_as_float(0xff800000);
    const int n16 = nblk(L, kB1), n128 = nblk(L, kB2);
    // kB1 = 16 cells: half a warp per block, a row segment of 32 cells per pass.
    for (int c0 = 0; c0 < n16 * kB1; c0 += 32) {
        float m = c0 + lane < L ? A[c0 + lane] : ninf;
#pragma unroll
        for (int off = kB1 / 2; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
        const int b = (c0 + lane) >> kB1Log;
        if ((lane & (kB1 - 1)) == 0 && b < n16) b16[b] = m;
    }
    if (lane < kMPad) {
        b16[-1 - lane] = ninf;
        b16[n16 + lane] = ninf;
        b128[-1 - lane] = ninf;
        b128[n128 + lane] = ninf;
    }
    __syncwarp();
    constexpr int kPer = kB2 / kB1;
    float m = ninf;  // this lane's kB2 block
    if (lane < n128) {
        for (int c = lane * kPer; c < min(lane * kPer + kPer, n16); c++) m = fmaxf(m, b16[c]);
        b128[lane] = m;
    }
    // Inclusive prefix and suffix maxima over the lanes (Hillis-Steele).
    float inc_p = m, inc_s = m;
    for (int off = 1; off < 32; off <<= 1) {
        const float up = __shfl_up_sync(0xffffffffu, inc_p, off);
        const float dn = __shfl_down_sync(0xffffffffu, inc_s, off);
        if (lane >= off) inc_p = fmaxf(inc_p, up);
        if (lane + off < 32) inc_s = fmaxf(inc_s, dn);
    }
    if (lane < n128) {
        s128[lane] = inc_s;
        p128[lane] = inc_p;
    }
    if (lane == 0) {
        s128[n128] = ninf;
        p128[-1] = ninf;
    }
}

// Retirement test after step dc: true when no target beyond distance dc can be
// visible from observer x (n steps in this direction, height h, horizon mx).
// The remaining targets are covered by kT blocks of kB1 cells from the one
// holding the nearest target, kT blocks of kB2 cells from the next uncovered
// cell, and the suffix (prefix) maximum beyond; blocks past the row end read
// -inf.  The first block may also hold up to kB1-1 passed targets, which only
// raises the bound.
//  * mx < 0: every remaining slope is at most fl(a/n), a = fl(Smax - h) < 0
//    with Smax the maximum over all those blocks, as in the header.
//  * mx >= 0: a block of remaining targets with maximum M and nearest
//    remaining distance ds holds no visible target when
//    M - h <= fl(fl(mx * kShrink) * ds): that product is below mx * ds, so
//    every target u = fl(z - h) <= M - h at distance d' >= ds has
//    u / d' <= mx (u >= 0) or u / d' < 0 <= mx (u < 0), and fl(u / d') <= mx.
template <bool kFwd>
__device__ __forceinline__ bool retire(const RowMax& rm, int x, int n, int dc, float h, float mx) {
    const int k = kFwd ? x + dc + 1 : x - dc - 1;  // nearest remaining target
    const int b = k >> kB1Log;
    float m1[kT], m2[kT];
#pragma unroll
    for (int j = 0; j < kT; j++) m1[j] = rm.b16[kFwd ? b + j : b - j];
    const int c = kFwd ? (b + kT) * kB1 : (b - kT + 1) * kB1 - 1;  // first uncovered cell
    const int b2 = c >> kB2Log;                                     // arithmetic shift: floor
#pragma unroll
    for (int j = 0; j < kT; j++) m2[j] = rm.b128[kFwd ? b2 + j : b2 - j];
    const float tail = kFwd ? rm.s128[min(b2 + kT, rm.n128)] : rm.p128[max(b2 - kT, -1)];
    if (mx < 0.0f) {
        float m = tail;
#pragma unroll
        for (int j = 0; j < kT; j++) m = fmaxf(m, fmaxf(m1[j], m2[j]));
        const float a = __fsub_rn(m, h);
        if (!(a < 0.0f)) return false;
        const float2 t = g_recip[n];
        return div_fast(a, t.x, t.y) <= mx;
    }
    const float mxc = __fmul_rn(mx, kShrink);
    bool ok = __fsub_rn(m1[0], h) <= __fmul_rn(mxc, __int2float_rn(dc + 1));
    float ds = __int2float_rn(kFwd ? (b + 1) * kB1 - x : x - (b * kB1 - 1));
#pragma unroll
    for (int j = 1; j < kT; j++) {
        ok &= __fsub_rn(m1[j], h) <= __fmul_rn(mxc, ds);
        ds = __fadd_rn(ds, (float)kB1);
    }
    ok &= __fsub_rn(m2[0], h) <= __fmul_rn(mxc, __int2float_rn(kFwd ? c - x : x - c));
    ds = __int2float_rn(kFwd ? (b2 + 1) * kB2 - x : x - (b2 * kB2 - 1));
#pragma unroll
    for (int j = 1; j < kT; j++) {
        ok &= __fsub_rn(m2[j], h) <= __fmul_rn(mxc, ds);
        ds = __fadd_rn(ds, (float)kB2);
    }
    ok &= __fsub_rn(tail, h) <= __fmul_rn(mxc, ds);
    return ok;
}

// The survivor lists and results of one row's sweep (per-warp global scratch).
struct RowLists {
    const int4* in[2];  // this level's survivors, forward / backward (null: level 0)
    int4* out[2];       // the next level's, forward / backward
    int n[2];           // entries of in[]
    int used[2];        // entries of in[] taken by this level's batches so far
    int made[2];        // entries appended to out[]
    float* cv[2];       // finished observers' counts by position, forward / backward
};

// One batch of a level: slot q takes entry used[dir] + lane + 32*qi of its
// direction's list, where qi counts the batch's earlier slots of that direction.
template <bool kF0, bool kF1, int kLen>
__device__ __forceinline__ void sweep_batch(const float* __restrict__ A, const RowMax& rm, int L, float povh,
                                            RowLists& rl, int d0, int len, int lane) {
    constexpr bool kDir[kSlots] = {kF0, kF1};
    const unsigned below = (1u << lane) - 1u;
    const int dc = d0 + (kLen > 0 ? kLen : len) - 1;  // last step of the level
    Slots s;
#pragma unroll
    for (int q = 0; q < kSlots; q++) {
        const int dir = kDir[q] ? 0 : 1;
        const int idx = rl.used[dir] + lane + (q == 1 && kF0 == kF1 ? 32 : 0);
        if (idx < rl.n[dir]) {
            if (rl.in[dir]) {
                const int4 e = rl.in[dir][idx];
                s.x[q] = e.x;
                s.mx[q] = __int_as_float(e.y);
                s.acc[q] = __int_as_float(e.z);
                s.cl[q] = __int_as_float(e.w);
            } else {
                s.x[q] = idx;
                s.mx[q] = -2000.0f;
                s.acc[q] = 0.0f;
                s.cl[q] = -1.0f;
            }
            s.n[q] = kDir[q] ? L - 1 - s.x[q] : s.x[q];
            s.valid[q] = true;
            s.h[q] = __fadd_rn(A[s.x[q]], povh);
        } else {
            // Empty: its reads stay in A[-(kLevel-1) .. kLevel-1].
            s.x[q] = kDir[q] ? -d0 : d0;
            s.n[q] = dc;
            s.valid[q] = false;
            s.h[q] = s.mx[q] = s.acc[q] = s.cl[q] = 0.0f;
        }
    }
    if (kF0 == kF1) rl.used[kF0 ? 0 : 1] += 64;
    else rl.used[0] += 32, rl.used[1] += 32;
    level_steps<kF0, kF1, kLen>(s, A, d0, len);

    // Retire finished observers, keep the others for the next level.
#pragma unroll
    for (int q = 0; q < kSlots; q++) {
        const int dir = kDir[q] ? 0 : 1;
        bool keep = false;
        if (s.valid[q]) {
            bool done = false;
            if (s.n[q] > dc) {
                done = kDir[q] ? retire<true>(rm, s.x[q], s.n[q], dc, s.h[q], s.mx[q])
                               : retire<false>(rm, s.x[q], s.n[q], dc, s.h[q], s.mx[q]);
                keep = !done;
            }
            if (!keep) rl.cv[dir][s.x[q]] = __fadd_rn(1.0f, done ? s.acc[q] : s.cl[q]);
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep)
            rl.out[dir][rl.made[dir] + __popc(m & below)] =
                make_int4(s.x[q], __float_as_int(s.mx[q]), __float_as_int(s.acc[q]), __float_as_int(s.cl[q]));
        rl.made[dir] += __popc(m);
    }
}

// Both scan directions of the row, level by level.  Level 0 takes every
// observer 0..L-1 in each direction; each later level takes the previous
// level's survivors.  A level runs full batches of one direction while a list
// has 64 entries left, then pairs what remains of the two (a forward observer
// in slot 0, a backward one in slot 1), so short lists share batches.
// lists: four lists of L_max entries (forward in/out, backward in/out);
// cvf, cvb: the two directions' counts, added and scaled at the end.
// One level over the current lists: full batches of one direction, then the
// remainders paired.  kLen > 0: every level kLen steps (compile time); kLen = 0:
// len steps.
template <int kLen>
__device__ __forceinline__ void run_level(const float* __restrict__ A, const RowMax& rm, int L, float povh,
                                          RowLists& rl, int d0, int len, int lane) {
    while (rl.n[0] - rl.used[0] >= 64) sweep_batch<true, true, kLen>(A, rm, L, povh, rl, d0, len, lane);
    while (rl.n[1] - rl.used[1] >= 64) sweep_batch<false, false, kLen>(A, rm, L, povh, rl, d0, len, lane);
    while (rl.used[0] < rl.n[0] || rl.used[1] < rl.n[1])
        sweep_batch<true, false, kLen>(A, rm, L, povh, rl, d0, len, lane);
}

// kFixed: every level kLevel steps, a compile-time length (the built-in
// schedule).  Otherwise lvl0, then lvl1 (skipped when 0), then kLevel each, each
// one of 16, 32, 48 or 64 steps, in one loop with run-time lengths.  The two are
// separate kernels: with both in one kernel the built-in schedule ran 7%
// slower (shared register allocation), and a loop compiled once per length ran
// the short schedules far slower still (a row then executes several compiled
// lengths and falls out of the instruction cache).
template <bool kFixed>
__device__ void sweep_row(const float* __restrict__ A, const RowMax& rm, int L, float povh, int4* lists,
                          int max_row, float* cvf, float* cvb, const RowOut& o, int lane, int lvl0, int lvl1) {
    RowLists rl;
    rl.in[0] = rl.in[1] = nullptr;
    rl.out[0] = lists;
    rl.out[1] = lists + 2 * (int64_t)max_row;
    rl.n[0] = rl.n[1] = L;
    rl.cv[0] = cvf;
    rl.cv[1] = cvb;
    int len = lvl0, level = 0;
    for (int d0 = 1; rl.n[0] > 0 || rl.n[1] > 0; d0 += len, level++) {
        len = level == 0 ? lvl0 : (level == 1 && lvl1 > 0) ? lvl1 : kLevel;
        rl.used[0] = rl.used[1] = 0;
        rl.made[0] = rl.made[1] = 0;
        if (kFixed) run_level<kLevel>(A, rm, L, povh, rl, d0, kLevel, lane);
        else run_level<0>(A, rm, L, povh, rl, d0, len, lane);
        __syncwarp();  // this level's lists and counts are visible to every lane
#pragma unroll
        for (int dir = 0; dir < 2; dir++) {
            int4* base = lists + 2 * (int64_t)max_row * dir;
            rl.in[dir] = rl.out[dir];
            rl.out[dir] = rl.out[dir] == base ? base + max_row : base;
            rl.n[dir] = rl.made[dir];
        }
    }
    for (int x = lane; x < L; x += 32) {
        if (!owns(o, x)) continue;
        const float t = __fadd_rn(cvf[x], cvb[x]);  // forward count, then backward
        o.out[o.rowbase + x] = o.counts_only ? t : __fmul_rn(t, o.sd->r2);
    }
}

// kBatch: the items are batch_item()s of a batched run over several grids,
// whose rows are compact rows of the pools SI/SO (kernels.h, BatchGrid).
// kFixed: the built-in level schedule (see sweep_row).
template <bool kBatch, bool kFixed>
__global__ void __launch_bounds__(kLWarps * 32) k_sdem(SdemLaunch a) {
    extern __shared__ float4 smem4[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const LLayout lay(a.max_row);
    float* buf = reinterpret_cast<float*>(smem4) + (size_t)warp * lay.total;
    float* A = buf + kLPad;
    float* s128 = buf + lay.s128;
    float* p128 = buf + lay.p128;
    float* b16 = buf + lay.b16;
    float* b128 = buf + lay.b128;
    const int64_t gwarp = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
    int4* lists = a.lists + gwarp * kListsPerWarp * (int64_t)a.max_row;
    float* cvf = reinterpret_cast<float*>(lists + 4 * (int64_t)a.max_row);
    float* cvb = cvf + a.max_row;
    for (;;) {
        unsigned idx = 0;
        if (lane == 0) idx = atomicAdd(a.counter, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if ((int64_t)idx >= a.n_items) break;
        const SectorDesc* dp;
        const int32_t *first = nullptr, *last = nullptr;
        int row, f, L;
        int64_t slot_off = 0;  // the sector's slot in SI/SO (per-engine runs)
        RowOut o;
        if (kBatch) {
            const uint64_t raw = a.items[idx];
            const BatchSector bs = a.bt.sectors[(int)(raw >> 32)];
            const BatchGrid& G = a.bt.grids[bs.grid];
            row = (int)(raw & 0xffffffffu);
            dp = &G.desc[bs.angle];
            const int4 m = G.rowtab[dp->row_off + row];  // {first, last, rowoff}
            f = m.x;
            L = m.y - m.x;
            o.out = a.SO;
            o.rowbase = bs.cells + m.z;
        } else {
            const Item it = decode(a.items[idx]);
            row = it.row;
            dp = &a.g.desc[a.b.angle[it.slot]];
            first = a.g.first + dp->row_off;
            last = a.g.last + dp->row_off;
            f = first[row];
            L = last[row] - f;
            slot_off = it.slot * a.stride;
            o.out = a.SO + slot_off;
            o.rowbase = (int64_t)row * dp->dim_i + f;
        }
        const SectorDesc& d = *dp;
        if (L > a.max_row || L <= 0) {
            if (lane == 0) atomicExch(a.status, 1);
            continue;
        }
        o.first = f;
        o.row = row;
        o.sd = &d;
        o.rfirst = first;
        o.rlast = last;
        o.counts_only = a.counts_only;
        o.compact = kBatch;
        const float* src = a.SI + slot_off + o.rowbase;
        bool ok = true;
        for (int x = lane; x < L; x += 32) {
            const float v = src[x];
            A[x] = v;
            ok = ok && div_safe(v) && div_safe(__fadd_rn(v, a.povh));
        }
        const float pad = __int_as_float(0x7fc00000);  // NaN (see visit)
        for (int x = lane; x < kLPad; x += 32) buf[x] = pad;
        const int tail_end = ((L + 3) & ~3) + kLPad;
        for (int x = L + lane; x < tail_end; x += 32) A[x] = pad;
        const bool fast = __all_sync(0xffffffffu, ok) && L <= kLFastMaxRow && div_safe(a.povh);
        __syncwarp();
        if (fast) {
            row_maxima(A, L, s128, p128, b16, b128, lane);
            __syncwarp();
            const RowMax rm{s128, p128, b16, b128, nblk(L, kB2)};
            sweep_row<kFixed>(A, rm, L, a.povh, lists, a.max_row, cvf, cvb, o, lane, a.lvl0, a.lvl1);
        } else {
            for (int x = lane; x < L; x += 32) {
                if (!owns(o, x)) continue;
                const float cv = scan_reference(A, x, L, a.povh);
                o.out[o.rowbase + x] = a.counts_only ? cv : __fmul_rn(cv, d.r2);
            }
        }
        __syncwarp();
    }
}

// ---- the built-in schedule, per-engine runs ---------------------------------
// The same sweep as k_sdem<false, true>, kept as its own copy: the built-in
// schedule's kernel ran 7% slower once the level-length and batch variants
// shared its source functions (the compiler allocates and schedules this hot
// loop differently; with a larger register budget it ran slower still), so the
// engine's per-grid runs launch this copy, whose code is the one measured in
// the sweep's tuning record.
__device__ __forceinline__ bool owns64(const RowOut& o, int x) {
    return o.first + x < o.sd->dim_i || owner_row(*o.sd, o.rfirst, o.rlast, o.rowbase + x) == o.row;
}

template <bool kF0, bool kF1>
__device__ __forceinline__ void level_steps64(Slots& s, const float* __restrict__ A, int d0) {
    const float* p0 = A + (kF0 ? s.x[0] + d0 : s.x[0] - d0);
    const float* p1 = A + (kF1 ? s.x[1] + d0 : s.x[1] - d0);
    const f2 hh = pk(s.h[0], s.h[1]);
#pragma unroll 1
    for (int k0 = 0; k0 < kLevel; k0 += kUnroll) {
#pragma unroll
        for (int k = 0; k < kUnroll; k++) {
            const int d = d0 + k0 + k;
            const float4 st = c_step[d];
            const float z0 = kF0 ? p0[k] : p0[-k];
            const float z1 = kF1 ? p1[k] : p1[-k];
            float q0, q1;
            upk(div2(sub2(pk(z0, z1), hh), pk(st.x, st.x), pk(st.y, st.y)), q0, q1);
            visit(s, 0, q0, st.z);
            visit(s, 1, q1, st.z);
        }
        p0 += kF0 ? kUnroll : -kUnroll;
        p1 += kF1 ? kUnroll : -kUnroll;
    }
}

// One batch of a level: slot q takes entry used[dir] + lane + 32*qi of its
// direction's list, where qi counts the batch's earlier slots of that direction.
template <bool kF0, bool kF1>
__device__ __forceinline__ void sweep_batch64(const float* __restrict__ A, const RowMax& rm, int L, float povh,
                                            RowLists& rl, int d0, int lane) {
    constexpr bool kDir[kSlots] = {kF0, kF1};
    const unsigned below = (1u << lane) - 1u;
    const int dc = d0 + kLevel - 1;  // last step of the level
    Slots s;
#pragma unroll
    for (int q = 0; q < kSlots; q++) {
        const int dir = kDir[q] ? 0 : 1;
        const int idx = rl.used[dir] + lane + (q == 1 && kF0 == kF1 ? 32 : 0);
        if (idx < rl.n[dir]) {
            if (rl.in[dir]) {
                const int4 e = rl.in[dir][idx];
                s.x[q] = e.x;
                s.mx[q] = __int_as_float(e.y);
                s.acc[q] = __int_as_float(e.z);
                s.cl[q] = __int_as_float(e.w);
            } else {
                s.x[q] = idx;
                s.mx[q] = -2000.0f;
                s.acc[q] = 0.0f;
                s.cl[q] = -1.0f;
            }
            s.n[q] = kDir[q] ? L - 1 - s.x[q] : s.x[q];
            s.valid[q] = true;
            s.h[q] = __fadd_rn(A[s.x[q]], povh);
        } else {
            // Empty: its reads stay in A[-(kLevel-1) .. kLevel-1].
            s.x[q] = kDir[q] ? -d0 : d0;
            s.n[q] = dc;
            s.valid[q] = false;
            s.h[q] = s.mx[q] = s.acc[q] = s.cl[q] = 0.0f;
        }
    }
    if (kF0 == kF1) rl.used[kF0 ? 0 : 1] += 64;
    else rl.used[0] += 32, rl.used[1] += 32;
    level_steps64<kF0, kF1>(s, A, d0);

    // Retire finished observers, keep the others for the next level.
#pragma unroll
    for (int q = 0; q < kSlots; q++) {
        const int dir = kDir[q] ? 0 : 1;
        bool keep = false;
        if (s.valid[q]) {
            bool done = false;
            if (s.n[q] > dc) {
                done = kDir[q] ? retire<true>(rm, s.x[q], s.n[q], dc, s.h[q], s.mx[q])
                               : retire<false>(rm, s.x[q], s.n[q], dc, s.h[q], s.mx[q]);
                keep = !done;
            }
            if (!keep) rl.cv[dir][s.x[q]] = __fadd_rn(1.0f, done ? s.acc[q] : s.cl[q]);
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep)
            rl.out[dir][rl.made[dir] + __popc(m & below)] =
                make_int4(s.x[q], __float_as_int(s.mx[q]), __float_as_int(s.acc[q]), __float_as_int(s.cl[q]));
        rl.made[dir] += __popc(m);
    }
}

// Both scan directions of the row, level by level.  Level 0 takes every
// observer 0..L-1 in each direction; each later level takes the previous
// level's survivors.  A level runs full batches of one direction while a list
// has 64 entries left, then pairs what remains of the two (a forward observer
// in slot 0, a backward one in slot 1), so short lists share batches.
// lists: four lists of L_max entries (forward in/out, backward in/out);
// cvf, cvb: the two directions' counts, added and scaled at the end.
__device__ void sweep_row64(const float* __restrict__ A, const RowMax& rm, int L, float povh, int4* lists,
                          int max_row, float* cvf, float* cvb, const RowOut& o, int lane) {
    RowLists rl;
    rl.in[0] = rl.in[1] = nullptr;
    rl.out[0] = lists;
    rl.out[1] = lists + 2 * (int64_t)max_row;
    rl.n[0] = rl.n[1] = L;
    rl.cv[0] = cvf;
    rl.cv[1] = cvb;
    for (int d0 = 1; rl.n[0] > 0 || rl.n[1] > 0; d0 += kLevel) {
        rl.used[0] = rl.used[1] = 0;
        rl.made[0] = rl.made[1] = 0;
        while (rl.n[0] - rl.used[0] >= 64) sweep_batch64<true, true>(A, rm, L, povh, rl, d0, lane);
        while (rl.n[1] - rl.used[1] >= 64) sweep_batch64<false, false>(A, rm, L, povh, rl, d0, lane);
        while (rl.used[0] < rl.n[0] || rl.used[1] < rl.n[1]) sweep_batch64<true, false>(A, rm, L, povh, rl, d0, lane);
        __syncwarp();  // this level's lists and counts are visible to every lane
#pragma unroll
        for (int dir = 0; dir < 2; dir++) {
            int4* base = lists + 2 * (int64_t)max_row * dir;
            rl.in[dir] = rl.out[dir];
            rl.out[dir] = rl.out[dir] == base ? base + max_row : base;
            rl.n[dir] = rl.made[dir];
        }
    }
    for (int x = lane; x < L; x += 32) {
        if (!owns64(o, x)) continue;
        const float t = __fadd_rn(cvf[x], cvb[x]);  // forward count, then backward
        o.out[o.rowbase + x] = o.counts_only ? t : __fmul_rn(t, o.sd->r2);
    }
}

__global__ void __launch_bounds__(kLWarps * 32) k_sdem_fixed(SdemLaunch a) {
    extern __shared__ float4 smem4[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const LLayout lay(a.max_row);
    float* buf = reinterpret_cast<float*>(smem4) + (size_t)warp * lay.total;
    float* A = buf + kLPad;
    float* s128 = buf + lay.s128;
    float* p128 = buf + lay.p128;
    float* b16 = buf + lay.b16;
    float* b128 = buf + lay.b128;
    const int64_t gwarp = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
    int4* lists = a.lists + gwarp * kListsPerWarp * (int64_t)a.max_row;
    float* cvf = reinterpret_cast<float*>(lists + 4 * (int64_t)a.max_row);
    float* cvb = cvf + a.max_row;
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
        RowOut o;
        o.out = a.SO + it.slot * a.stride;
        o.rowbase = (int64_t)it.row * d.dim_i + f;
        o.first = f;
        o.row = it.row;
        o.sd = &d;
        o.rfirst = first;
        o.rlast = last;
        o.counts_only = a.counts_only;
        const float* src = a.SI + it.slot * a.stride + o.rowbase;
        bool ok = true;
        for (int x = lane; x < L; x += 32) {
            const float v = src[x];
            A[x] = v;
            ok = ok && div_safe(v) && div_safe(__fadd_rn(v, a.povh));
        }
        const float pad = __int_as_float(0x7fc00000);  // NaN (see visit)
        for (int x = lane; x < kLPad; x += 32) buf[x] = pad;
        const int tail_end = ((L + 3) & ~3) + kLPad;
        for (int x = L + lane; x < tail_end; x += 32) A[x] = pad;
        const bool fast = __all_sync(0xffffffffu, ok) && L <= kLFastMaxRow && div_safe(a.povh);
        __syncwarp();
        if (fast) {
            row_maxima(A, L, s128, p128, b16, b128, lane);
            __syncwarp();
            const RowMax rm{s128, p128, b16, b128, nblk(L, kB2)};
            sweep_row64(A, rm, L, a.povh, lists, a.max_row, cvf, cvb, o, lane);
        } else {
            for (int x = lane; x < L; x += 32) {
                if (!owns64(o, x)) continue;
                const float cv = scan_reference(A, x, L, a.povh);
                o.out[o.rowbase + x] = a.counts_only ? cv : __fmul_rn(cv, d.r2);
            }
        }
        __syncwarp();
    }
}

// The built-in schedule for batched runs: the same sweep over compact rows
// (kernels.h, BatchGrid); only the work item's decode differs.
__global__ void __launch_bounds__(kLWarps * 32) k_sdem_fixed_batch(SdemLaunch a) {
    extern __shared__ float4 smem4[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const LLayout lay(a.max_row);
    float* buf = reinterpret_cast<float*>(smem4) + (size_t)warp * lay.total;
    float* A = buf + kLPad;
    float* s128 = buf + lay.s128;
    float* p128 = buf + lay.p128;
    float* b16 = buf + lay.b16;
    float* b128 = buf + lay.b128;
    const int64_t gwarp = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
    int4* lists = a.lists + gwarp * kListsPerWarp * (int64_t)a.max_row;
    float* cvf = reinterpret_cast<float*>(lists + 4 * (int64_t)a.max_row);
    float* cvb = cvf + a.max_row;
    for (;;) {
        unsigned idx = 0;
        if (lane == 0) idx = atomicAdd(a.counter, 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if ((int64_t)idx >= a.n_items) break;
        const uint64_t raw = a.items[idx];
        const BatchSector bs = a.bt.sectors[(int)(raw >> 32)];
        const BatchGrid& G = a.bt.grids[bs.grid];
        const int row = (int)(raw & 0xffffffffu);
        const SectorDesc& d = G.desc[bs.angle];
        const int4 m = G.rowtab[d.row_off + row];  // {first, last, rowoff}
        const int f = m.x;
        const int L = m.y - m.x;
        if (L > a.max_row || L <= 0) {
            if (lane == 0) atomicExch(a.status, 1);
            continue;
        }
        RowOut o;  // a compact row: its cells are its own (first + x < last <= dim_i)
        o.out = a.SO;
        o.rowbase = bs.cells + m.z;
        o.first = f;
        o.row = row;
        o.sd = &d;
        o.rfirst = nullptr;
        o.rlast = nullptr;
        o.counts_only = a.counts_only;
        const float* src = a.SI + o.rowbase;
        bool ok = true;
        for (int x = lane; x < L; x += 32) {
            const float v = src[x];
            A[x] = v;
            ok = ok && div_safe(v) && div_safe(__fadd_rn(v, a.povh));
        }
        const float pad = __int_as_float(0x7fc00000);  // NaN (see visit)
        for (int x = lane; x < kLPad; x += 32) buf[x] = pad;
        const int tail_end = ((L + 3) & ~3) + kLPad;
        for (int x = L + lane; x < tail_end; x += 32) A[x] = pad;
        const bool fast = __all_sync(0xffffffffu, ok) && L <= kLFastMaxRow && div_safe(a.povh);
        __syncwarp();
        if (fast) {
            row_maxima(A, L, s128, p128, b16, b128, lane);
            __syncwarp();
            const RowMax rm{s128, p128, b16, b128, nblk(L, kB2)};
            sweep_row64(A, rm, L, a.povh, lists, a.max_row, cvf, cvb, o, lane);
        } else {
            for (int x = lane; x < L; x += 32) {
                if (!owns64(o, x)) continue;
                const float cv = scan_reference(A, x, L, a.povh);
                o.out[o.rowbase + x] = a.counts_only ? cv : __fmul_rn(cv, d.r2);
            }
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
            const float ref = __fdiv_rn(a, -st.x);
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

namespace {
struct StepTable {
    float4 v[kFastMaxRow];
    StepTable() {
        for (int d = 0; d < kFastMaxRow; d++) {
            const float df = (float)d;
            v[d] = make_float4(-df, d ? 1.0f / df : 0.0f, 2.0f * df + 1.0f, df + 1.0f);
        }
    }
};
}  // namespace

cudaError_t sdem_init_tables() {
    static const StepTable tab;  // built once, thread-safe, no heap
    static float2 recip[kFastMaxRow];
    for (int n = 0; n < kFastMaxRow; n++) recip[n] = make_float2(tab.v[n].x, tab.v[n].y);
    cudaError_t e = cudaMemcpyToSymbol(c_step, tab.v, sizeof(tab.v));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_recip, recip, sizeof(recip));
    return e;
}

void sdem_items(const Geometry& geo, const Batch& b, std::vector<uint64_t>& items, int* max_row) {
    // Counting sort of rows by valid length, longest first: a row's work grows
    // about as L^2, so long rows go first.
    int lmax = 0;
    for (int s = 0; s < b.count; s++) {
        const SectorDesc& d = geo.desc[b.angle[s]];
        for (int r = 0; r < d.H; r++) lmax = std::max(lmax, geo.last[d.row_off + r] - geo.first[d.row_off + r]);
    }
    std::vector<int64_t> start(lmax + 2, 0);
    for (int s = 0; s < b.count; s++) {
        const SectorDesc& d = geo.desc[b.angle[s]];
        for (int r = 0; r < d.H; r++) {
            const int L = geo.last[d.row_off + r] - geo.first[d.row_off + r];
            if (L > 0) start[L]++;
        }
    }
    int64_t total = 0;
    for (int L = lmax; L >= 1; L--) {
        const int64_t cnt = start[L];
        start[L] = total;
        total += cnt;
    }
    items.assign(total, 0);
    for (int s = 0; s < b.count; s++) {
        const SectorDesc& d = geo.desc[b.angle[s]];
        for (int r = 0; r < d.H; r++) {
            const int L = geo.last[d.row_off + r] - geo.first[d.row_off + r];
            if (L > 0) items[start[L]++] = ((uint64_t)s << 48) | ((uint64_t)(uint32_t)r << 16);
        }
    }
    *max_row = lmax;
}

size_t sdem_list_bytes(int max_row, int num_sms) {
    // kListsPerWarp units of max_row entries per warp, for as many warps as an SM holds.
    int dev = 0, threads = 2048;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&threads, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
    return (size_t)num_sms * (size_t)(threads / 32) * kListsPerWarp * (size_t)std::max(max_row, 1) * sizeof(int4);
}

int sdem_max_ctas_per_sm(const SdemLaunch& a) {
    const size_t smem = sizeof(float) * (size_t)LLayout(std::max(a.max_row, 1)).total * kLWarps;
    const bool fixed = a.lvl0 == kLevel && a.lvl1 == 0;
    auto kern = a.batched ? (fixed ? k_sdem_fixed_batch : k_sdem<true, false>)
                          : (fixed ? k_sdem_fixed : k_sdem<false, false>);
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kLWarps * 32, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return per_sm;
}

cudaError_t launch_sdem(const SdemLaunch& a, int num_sms, cudaStream_t st) {
    if (a.n_items == 0) return cudaSuccess;
    auto level_ok = [](int v) { return v == 16 || v == 32 || v == 48 || v == 64; };
    if (!level_ok(a.lvl0) || (a.lvl1 != 0 && !level_ok(a.lvl1)) || a.ctas_per_sm < 0) return cudaErrorInvalidValue;
    const size_t smem = sizeof(float) * (size_t)LLayout(a.max_row).total * kLWarps;
    const bool fixed = a.lvl0 == kLevel && a.lvl1 == 0;
    auto kern = a.batched ? (fixed ? k_sdem_fixed_batch : k_sdem<true, false>)
                          : (fixed ? k_sdem_fixed : k_sdem<false, false>);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kLWarps * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    if (a.ctas_per_sm > 0 && per_sm > a.ctas_per_sm) per_sm = a.ctas_per_sm;
    int64_t blocks = (int64_t)per_sm * num_sms;
    const int64_t need = (a.n_items + kLWarps - 1) / kLWarps;
    if (blocks > need) blocks = need;
    // Every warp owns kListsPerWarp units of max_row entries in the scratch.
    const size_t list_per_block = (size_t)kLWarps * kListsPerWarp * (size_t)a.max_row * sizeof(int4);
    const int64_t fit = a.lists ? (int64_t)(a.list_bytes / list_per_block) : 0;
    if (fit < 1) return cudaErrorInvalidValue;
    if (blocks > fit) blocks = fit;
    e = cudaMemsetAsync(a.counter, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    kern<<<(int)blocks, kLWarps * 32, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_sdem_chunked(const SdemLaunch& a, int num_sms, cudaStream_t st) {
    if (a.n_items == 0) return cudaSuccess;
    const size_t smem = sizeof(float) * (size_t)warp_floats(a.max_row) * kWarps;
    cudaError_t e = cudaFuncSetAttribute(k_sdem_chunked, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sdem_chunked, kWarps * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int64_t blocks = (int64_t)per_sm * num_sms;
    const int64_t need = (a.n_items + kWarps - 1) / kWarps;
    if (blocks > need) blocks = need;
    e = cudaMemsetAsync(a.counter, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    k_sdem_chunked<<<(int)blocks, kWarps * 32, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace ske

