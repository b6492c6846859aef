// Data-layout kernels of the sector loop: the four input orientations, the skew
// gather, the identity operator, deskew/accumulate and the final fold.
//
// All are HBM/L2-bound integer-indexed copies with one or two fp32 multiply-adds
// per cell; the arithmetic that must match the reference uses explicit _rn
// intrinsics (no contraction).
#include <vector>

#include <cuda.h>

#include "kernels.h"

namespace ske {

namespace {

constexpr int kTile = 32;

// prepare (skewEngine.cuh:925-951): o0 = input, o1 = transpose + flip both,
// o2 = transpose + flip y, o3 = flip x.  32x32 tiles staged through shared
// memory so the transposed stores stay coalesced.
__global__ void k_prepare(const float* __restrict__ in, float* __restrict__ orient, int dimx, int dimy) {
    __shared__ float tile[kTile][kTile + 1];
    const int64_t n = (int64_t)dimx * dimy;
    float* o0 = orient;
    float* o1 = orient + n;
    float* o2 = orient + 2 * n;
    float* o3 = orient + 3 * n;
    const int j0 = blockIdx.x * kTile, i0 = blockIdx.y * kTile;
    for (int ty = threadIdx.y; ty < kTile; ty += blockDim.y) {
        const int i = i0 + ty, j = j0 + threadIdx.x;
        if (i < dimy && j < dimx) {
            const float v = in[(int64_t)i * dimx + j];
            tile[ty][threadIdx.x] = v;
            o0[(int64_t)i * dimx + j] = v;
            o3[(int64_t)i * dimx + (dimx - 1 - j)] = v;
        }
    }
    __syncthreads();
    // Transposed writes: thread x walks input rows (output columns).
    for (int ty = threadIdx.y; ty < kTile; ty += blockDim.y) {
        const int j = j0 + ty, i = i0 + threadIdx.x;
        if (i < dimy && j < dimx) {
            const float v = tile[threadIdx.x][ty];
            const int ci = dimy - 1 - i, cj = dimx - 1 - j;
            o1[(int64_t)dimy * cj + ci] = v;
            o2[(int64_t)dimy * j + ci] = v;
        }
    }
}

// Skewed input of every sector: thread = one column c of kSkewRows consecutive
// rows.  Cell (r, c) = 0 + w_c*x[r-t_c-1][c] + (1-w_c)*x[r-t_c][c] (skew_gather):
// the column's target and weight stay in registers, and the second source value
// of row r is the first of row r+1, so each cell loads one new value.  Then the
// slot's cells past H*dim_i are zeroed (all blocks share that work), unless the
// caller skips it for sectors whose rows stay within dim_i.
constexpr int kSkewRows = 32;
constexpr int kSkewCols = 256;

__global__ void __launch_bounds__(kSkewCols) k_skew(DevGeometry g, Batch b, const float* __restrict__ orient,
                                                    int64_t n_cells, float* __restrict__ SI, int64_t stride,
                                                    int64_t len, bool zero_tail) {
    const int slot = blockIdx.z;
    const SectorDesc d = g.desc[b.angle[slot]];
    float* out = SI + slot * stride;
    const int c = blockIdx.x * kSkewCols + threadIdx.x;
    const int r0 = blockIdx.y * kSkewRows;
    if (r0 < d.H && c < d.dim_i) {
        const float* src = orient + (int64_t)d.type * n_cells;
        const int t = g.target[d.col_off + c];
        const float w = g.weight[d.col_off + c], w1 = __fsub_rn(1.0f, w);
        int i0 = r0 - t - 1;  // source row of the w term
        const float* p = src + ((int64_t)i0 * d.dim_i + c);
        float* o = out + ((int64_t)r0 * d.dim_i + c);
        float a = (unsigned)i0 < (unsigned)d.dim_o ? p[0] : 0.0f;
        const int r1 = min(r0 + kSkewRows, d.H);
        for (int r = r0; r < r1; r++) {
            const bool v0 = (unsigned)i0 < (unsigned)d.dim_o, v1 = (unsigned)(i0 + 1) < (unsigned)d.dim_o;
            const float bv = v1 ? p[d.dim_i] : 0.0f;
            float acc = 0.0f;
            acc = v0 ? __fadd_rn(acc, __fmul_rn(w, a)) : acc;
            acc = v1 ? __fadd_rn(acc, __fmul_rn(w1, bv)) : acc;
            *o = acc;
            a = bv;
            i0++;
            p += d.dim_i;
            o += d.dim_i;
        }
    }
    if (!zero_tail && d.in_width) return;  // nothing reads past H*dim_i
    const int64_t z0 = (int64_t)d.H * d.dim_i;
    const int64_t nthreads = (int64_t)gridDim.x * gridDim.y * kSkewCols;
    for (int64_t q = z0 + ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * kSkewCols + threadIdx.x; q < len;
         q += nthreads)
        out[q] = 0.0f;
}

__global__ void k_identity(DevGeometry g, Batch b, const float* __restrict__ SI, float* __restrict__ SO,
                           int64_t stride, int64_t len) {
    const int slot = blockIdx.y;
    const SectorDesc d = g.desc[b.angle[slot]];
    const int32_t* first = g.first + d.row_off;
    const int32_t* last = g.last + d.row_off;
    const float* in = SI + slot * stride;
    float* out = SO + slot * stride;
    for (int64_t p = gtid(); p < len; p += gstride())
        out[p] = owner_row(d, first, last, p) >= 0 ? in[p] : 0.0f;
}

// Deskew + accumulate, tiled.  A CTA owns a kDeskewRows x 32 tile of one
// orientation's accumulator (blockIdx.z = sector type) and keeps it in registers
// while it walks that type's sectors of the batch in order.  For each sector
// the skewed rows the tile needs, [i0 + t(j0), i1 + t(j0+31)], are staged in
// shared memory with coalesced 128-byte row loads; every thread then combines
// its two cells (rows i+t_j and i+t_j+1 of its column) exactly as the reference
// does.  Accumulator traffic: one read and one write per batch instead of per
// sector.
constexpr int kDeskewRows = 64;
constexpr int kDeskewBand = kDeskewRows + 34;  // rows + 1 + max column drift over 32 columns (+1)
enum { kDeskewAdd = 0, kDeskewKahan = 1, kDeskewMax = 2 };

// Skewed output cell (r, c), c < dim_i, of a Radon sector read from its
// filtered row values q instead of SO: the back-projection writes
// 0.0f + q[r] (in binary64, then rounded) on every valid cell of row r
// (kernelRADN.h:251-257), and zero elsewhere.  Only for sectors whose rows stay
// within dim_i, where no two rows share a cell.
__device__ __forceinline__ float row_cell(const SectorDesc& d, const int32_t* __restrict__ first,
                                          const int32_t* __restrict__ last, const cd* __restrict__ q, int r, int c) {
    return (r < d.H && c >= first[r] && c < last[r]) ? __double2float_rn(__dadd_rn(0.0, q[r].re)) : 0.0f;
}

// kRows: the batch's skewed outputs are Radon sectors given as per-row values
// (Q: pstride complex doubles per slot, real part) rather than SO.
// kMasked: SO is defined only on its sectors' valid cells (rows within dim_i,
// not zeroed first): a staged row carries the mask of the tile's columns in
// its valid range and other cells read as zero.
template <int kMode, bool kRows = false, bool kMasked = false>
__global__ void __launch_bounds__(256, kMode == kDeskewKahan ? 2 : 4) k_deskew(DevGeometry g, TypeLists tl, const float* __restrict__ SO,
                                                int64_t stride, float* __restrict__ acc, float* __restrict__ comp,
                                                int dimx, int dimy, const cd* __restrict__ Q = nullptr,
                                                int64_t pstride = 0) {
    __shared__ float band[kRows ? 1 : kDeskewBand][kTile];
    __shared__ unsigned bmask[kMasked ? kDeskewBand : 1];
    // kRows: the band's rows as (value, mask of the tile's columns inside the
    // row's valid range); a cell is its row's value inside the range, else zero.
    __shared__ float2 rqm[kRows ? kDeskewBand : 1];
    // Thread (tx, ty) owns rows ty*kPer .. ty*kPer+kPer-1 of the tile in column
    // j0+tx: consecutive rows share a skewed cell (row k's upper cell is row
    // k+1's lower one), so kPer+1 cells per sector serve its kPer rows.
    constexpr int kPer = kDeskewRows / 8;
    const int t = blockIdx.z;
    const int cnt = tl.count[t];
    if (cnt == 0) return;
    const int64_t n = (int64_t)dimx * dimy;
    const int dim_i = (t == 1 || t == 2) ? dimy : dimx;
    const int dim_o = (t == 1 || t == 2) ? dimx : dimy;
    const int j0 = blockIdx.x * kTile, i0 = blockIdx.y * kDeskewRows;
    if (j0 >= dim_i || i0 >= dim_o) return;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int j = j0 + tx;
    const bool col_ok = j < dim_i;
    const int jlast = min(j0 + kTile, dim_i) - 1;
    const int i_end = min(i0 + kDeskewRows, dim_o);
    float* A = acc + t * n;
    const int ib = ty * kPer;
    const int nv = min(kPer, i_end - i0 - ib);  // this thread's rows inside the grid
    float s[kPer], c[kPer];
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        const int i = i0 + ib + k;
        s[k] = (col_ok && i < i_end) ? A[(int64_t)i * dim_i + j] : 0.0f;
        c[k] = (kMode == kDeskewKahan && col_ok && i < i_end) ? comp[t * n + (int64_t)i * dim_i + j] : 0.0f;
    }
    for (int q = 0; q < cnt; q++) {
        const SectorDesc& d = g.desc[tl.angle[t][q]];
        const int32_t* tg = g.target + d.col_off;
        const int tmin = tg[j0], tmax = tg[jlast];
        const int tj = col_ok ? tg[j] : tmin;
        const float w = col_ok ? g.weight[d.col_off + j] : 0.0f;
        // Rows r0 .. r0+nrows-1 hold every (i+t_j, i+t_j+1) of the tile.
        const int r0 = i0 + tmin;
        const int nrows = (i_end - i0) + 1 + (tmax - tmin);
        const float* so = SO + tl.slot[t][q] * stride;
        const cd* qv = kRows ? Q + tl.slot[t][q] * pstride : nullptr;
        const int32_t* rfirst = g.first + d.row_off;
        const int32_t* rlast = g.last + d.row_off;
        // Steep sectors of elongated grids (tan > 1) can drift more than the band
        // holds; those tiles read the skewed cells directly.
        const bool staged = nrows <= kDeskewBand;
        bool full = false;  // kMasked: every staged cell of the tile is valid
        if (staged && kRows) {
            __syncthreads();  // previous sector's rows fully consumed
            const int tid = ty * kTile + tx;
            if (tid < nrows) {
                const int r = r0 + tid;
                float v = 0.0f;
                unsigned m = 0;
                if (r < d.H) {
                    v = __double2float_rn(__dadd_rn(0.0, qv[r].re));
                    const int lo_c = max(rfirst[r] - j0, 0), hi_c = min(rlast[r] - j0, kTile);
                    if (hi_c > lo_c) m = (hi_c >= 32 ? 0xffffffffu : (1u << hi_c) - 1u) & ~((1u << lo_c) - 1u);
                }
                rqm[tid] = make_float2(v, __uint_as_float(m));
            }
            __syncthreads();
        } else if (staged) {
            // All of this thread's band loads are issued before any store.
            constexpr int kLoads = (kDeskewBand + 7) / 8;
            float v[kLoads];
#pragma unroll
            for (int u = 0; u < kLoads; u++) {
                const int rr = ty + 8 * u;
                v[u] = (rr < nrows && j0 + tx <= jlast) ? so[(int64_t)(r0 + rr) * dim_i + j0 + tx] : 0.0f;
            }
            unsigned m = 0;
            const int tid = ty * kTile + tx;
            if (kMasked && tid < nrows) {
                const int r = r0 + tid;
                if (r < d.H) {
                    const int lo_c = max(rfirst[r] - j0, 0), hi_c = min(rlast[r] - j0, kTile);
                    if (hi_c > lo_c) m = (hi_c >= 32 ? 0xffffffffu : (1u << hi_c) - 1u) & ~((1u << lo_c) - 1u);
                }
            }
            __syncthreads();  // previous sector's band fully consumed
#pragma unroll
            for (int u = 0; u < kLoads; u++)
                if (ty + 8 * u < nrows) band[ty + 8 * u][tx] = v[u];
            if (kMasked) {
                if (tid < nrows) bmask[tid] = m;
                // Tiles whose staged rows cover all 32 columns need no mask.
                full = __syncthreads_and(tid >= nrows || m == 0xffffffffu);
            } else {
                __syncthreads();
            }
        }
        if (!col_ok || nv <= 0) continue;
        const int off = tj - tmin;
        // Cells of skewed rows i0+ib+tj .. i0+ib+tj+nv (band rows ib+off ..).
        float cell[kPer + 1];
#pragma unroll
        for (int kk = 0; kk <= kPer; kk++) {
            cell[kk] = 0.0f;
            if (kk > nv) continue;
            const int br = ib + kk + off;
            const int r = i0 + ib + kk + tj;
            if (kRows && staged) {
                const float2 e = rqm[br];
                cell[kk] = ((__float_as_uint(e.y) >> tx) & 1u) ? e.x : 0.0f;
            } else if (kRows) {
                cell[kk] = row_cell(d, rfirst, rlast, qv, r, j);
            } else if (kMasked && !full) {
                const bool ok = staged ? ((bmask[br] >> tx) & 1u) != 0
                                       : (r < d.H && j >= rfirst[r] && j < rlast[r]);
                cell[kk] = ok ? (staged ? band[br][tx] : so[(int64_t)r * dim_i + j]) : 0.0f;
            } else {
                cell[kk] = staged ? band[br][tx] : so[(int64_t)r * dim_i + j];
            }
        }
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            if (k >= nv) continue;
            const float lo = cell[k], hi = cell[k + 1];
            if (kMode == kDeskewMax) {
                const float m = (lo < hi) ? hi : lo;  // std::max(lo, hi)
                float v = (s[k] < m) ? m : s[k];      // std::max(acc, m)
                // a + 1000*(int)(v/1000): the low decimal digits carry the angle.
                const int qq = __float2int_rz(__fdiv_rn(v, 1000.0f));
                s[k] = __int2float_rn(d.angle + 1000 * qq);
            } else {
                const float v = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, w), lo), __fmul_rn(w, hi));
                if (kMode == kDeskewKahan) {
                    const float y = __fsub_rn(v, c[k]);
                    const float tsum = __fadd_rn(s[k], y);
                    c[k] = __fsub_rn(__fsub_rn(tsum, s[k]), y);
                    s[k] = tsum;
                } else {
                    s[k] = __fadd_rn(s[k], v);
                }
            }
        }
    }
    if (!col_ok) return;
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        const int i = i0 + ib + k;
        if (i >= i_end) continue;
        A[(int64_t)i * dim_i + j] = s[k];
        if (kMode == kDeskewKahan) comp[t * n + (int64_t)i * dim_i + j] = c[k];
    }
}

// ---- TMA-staged deskew ------------------------------------------------------
// The same deskew (add / Kahan, plain or masked) with each sector's band of
// kDeskewBand skewed rows x 32 columns brought into shared memory by the tensor
// memory accelerator: the skewed output is a 3-D tensor (columns dim_i, rows,
// slots; row pitch dim_i*4 bytes, a multiple of 16), thread 0 issues one
// cp.async.bulk.tensor per sector (x = j0, a multiple of 32 floats) and the
// copies complete on mbarriers.  Two buffers: the next staged sector's band is
// in flight while the CTA accumulates the current one.  Columns past dim_i and
// rows past the tensor read as zero.  Every wait is bounded; a wait that runs
// out sets the engine's status word (the host reports SKE_ERR_DEVICE).
constexpr int kTmaBoxBytes = kDeskewBand * kTile * 4;
constexpr long long kTmaWaitLimit = 1ll << 20;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect(uint64_t* bar, int bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* bar, int parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the completion of phase `parity`; false if it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, int parity) {
    for (long long i = 0; i < kTmaWaitLimit; i++)
        if (mbar_try(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_band(float* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // earlier generic reads of dst come first
    mbar_expect(bar, kTmaBoxBytes);
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

template <int kMode, bool kMasked>
__global__ void __launch_bounds__(256, kMode == kDeskewKahan ? 2 : 4)
    k_deskew_tma(const __grid_constant__ CUtensorMap map_x, const __grid_constant__ CUtensorMap map_y, DevGeometry g,
                 TypeLists tl, const float* __restrict__ SO, int64_t stride, float* __restrict__ acc,
                 float* __restrict__ comp, int dimx, int dimy, int* __restrict__ status) {
    __shared__ __align__(128) float band[2][kDeskewBand][kTile];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ unsigned bmask[kMasked ? kDeskewBand : 1];
    __shared__ int s_abort;  // a band wait ran out: stop issuing and reading bands
    constexpr int kPer = kDeskewRows / 8;
    const int t = blockIdx.z;
    const int cnt = tl.count[t];
    if (cnt == 0) return;
    const int64_t n = (int64_t)dimx * dimy;
    const int dim_i = (t == 1 || t == 2) ? dimy : dimx;
    const int dim_o = (t == 1 || t == 2) ? dimx : dimy;
    const CUtensorMap* map = (t == 1 || t == 2) ? &map_y : &map_x;
    const int j0 = blockIdx.x * kTile, i0 = blockIdx.y * kDeskewRows;
    if (j0 >= dim_i || i0 >= dim_o) return;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTile + tx;
    const int j = j0 + tx;
    const bool col_ok = j < dim_i;
    const int jlast = min(j0 + kTile, dim_i) - 1;
    const int i_end = min(i0 + kDeskewRows, dim_o);
    const int ib = ty * kPer;
    const int nv = min(kPer, i_end - i0 - ib);
    float* A = acc + t * n;
    float s[kPer], c[kPer];
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        const int i = i0 + ib + k;
        s[k] = (col_ok && i < i_end) ? A[(int64_t)i * dim_i + j] : 0.0f;
        c[k] = (kMode == kDeskewKahan && col_ok && i < i_end) ? comp[t * n + (int64_t)i * dim_i + j] : 0.0f;
    }
    // Band origin of sector q and whether it fits the staged band.
    auto band_of = [&](int q, int* r0, int* nrows) {
        const SectorDesc& d = g.desc[tl.angle[t][q]];
        const int32_t* tg = g.target + d.col_off;
        *r0 = i0 + tg[j0];
        *nrows = (i_end - i0) + 1 + (tg[jlast] - tg[j0]);
        return *nrows <= kDeskewBand;
    };
    if (tid == 0) {
        mbar_init(&bar[0]);
        mbar_init(&bar[1]);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    int r0n, nrn;
    // uses[b]: phases of bar[b] this thread has seen complete; issued[b]: copies
    // thread 0 has started into buffer b.  issued - uses (thread 0) is what is
    // still in flight if the CTA has to give up.
    int uses[2] = {0, 0}, issued[2] = {0, 0};
    if (tid == 0 && band_of(0, &r0n, &nrn)) {
        tma_band(&band[0][0][0], map, j0, r0n, tl.slot[t][0], &bar[0]);
        issued[0]++;
    }
    volatile int* abort_flag = &s_abort;
    for (int q = 0; q < cnt; q++) {
        const int buf = q & 1;
        // Prefetch the next sector's band into the other buffer (freed by the
        // barrier that ended the previous sector), unless the CTA is giving up.
        if (tid == 0 && q + 1 < cnt && !*abort_flag && band_of(q + 1, &r0n, &nrn)) {
            tma_band(&band[buf ^ 1][0][0], map, j0, r0n, tl.slot[t][q + 1], &bar[buf ^ 1]);
            issued[buf ^ 1]++;
        }
        const SectorDesc& d = g.desc[tl.angle[t][q]];
        const int32_t* tg = g.target + d.col_off;
        const int tmin = tg[j0];
        const int tj = col_ok ? tg[j] : tmin;
        const float w = col_ok ? g.weight[d.col_off + j] : 0.0f;
        int r0, nrows;
        const bool staged = band_of(q, &r0, &nrows);
        const float* so = SO + tl.slot[t][q] * stride;
        const int32_t* rfirst = g.first + d.row_off;
        const int32_t* rlast = g.last + d.row_off;
        bool full = false;
        if (staged) {
            unsigned m = 0;
            if (kMasked && tid < nrows) {
                const int r = r0 + tid;
                if (r < d.H) {
                    const int lo_c = max(rfirst[r] - j0, 0), hi_c = min(rlast[r] - j0, kTile);
                    if (hi_c > lo_c) m = (hi_c >= 32 ? 0xffffffffu : (1u << hi_c) - 1u) & ~((1u << lo_c) - 1u);
                }
                bmask[tid] = m;
            }
            if (mbar_wait(&bar[buf], uses[buf] & 1)) uses[buf]++;
            else *abort_flag = 1;  // written before the barrier, read by every thread after it
            if (kMasked) full = __syncthreads_and(tid >= nrows || m == 0xffffffffu);
            else __syncthreads();
            if (*abort_flag) break;  // CTA-uniform: the band is not read
        }
        if (col_ok && nv > 0) {
            const int off = tj - tmin;
            float cell[kPer + 1];
#pragma unroll
            for (int kk = 0; kk <= kPer; kk++) {
                cell[kk] = 0.0f;
                if (kk > nv) continue;
                const int br = ib + kk + off;
                const int r = i0 + ib + kk + tj;
                if (kMasked && !full) {
                    const bool okc = staged ? ((bmask[br] >> tx) & 1u) != 0
                                            : (r < d.H && j >= rfirst[r] && j < rlast[r]);
                    cell[kk] = okc ? (staged ? band[buf][br][tx] : so[(int64_t)r * dim_i + j]) : 0.0f;
                } else {
                    cell[kk] = staged ? band[buf][br][tx] : so[(int64_t)r * dim_i + j];
                }
            }
#pragma unroll
            for (int k = 0; k < kPer; k++) {
                if (k >= nv) continue;
                const float v = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, w), cell[k]), __fmul_rn(w, cell[k + 1]));
                if (kMode == kDeskewKahan) {
                    const float y = __fsub_rn(v, c[k]);
                    const float ts = __fadd_rn(s[k], y);
                    c[k] = __fsub_rn(__fsub_rn(ts, s[k]), y);
                    s[k] = ts;
                } else {
                    s[k] = __fadd_rn(s[k], v);
                }
            }
        }
        __syncthreads();  // this buffer and the masks are free for the next sectors
    }
    if (*abort_flag) {
        // A band copy did not arrive in time.  Report it, leave the accumulators
        // as they were, and keep the CTA (and so its shared memory) alive until
        // every copy thread 0 started has landed, each wait again bounded.
        if (tid == 0) {
            atomicExch(status, 7);
            for (int b = 0; b < 2; b++)
                if (issued[b] > uses[b]) mbar_wait(&bar[b], uses[b] & 1);
        }
        return;
    }
    if (!col_ok) return;
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        const int i = i0 + ib + k;
        if (i >= i_end) continue;
        A[(int64_t)i * dim_i + j] = s[k];
        if (kMode == kDeskewKahan) comp[t * n + (int64_t)i * dim_i + j] = c[k];
    }
}

// ---- TMA-staged skew -------------------------------------------------------
// A block of 256 threads owns kSkTmaCols skewed columns c0.. and kSkTmaRows
// skewed rows r0.. of one sector.  Column c of row r reads orientation rows
// r - t_c - 1 and r - t_c (skew_gather), so the block needs rows
// [r0 - max t - 1, r0 + kSkTmaRows - min t] of its 32 columns: thread 0 loads
// them as one kSkTmaBox x 32 TMA box (128-byte rows, zero outside the grid) and
// every thread then reads its column from shared memory (one bank per column)
// and writes its rows coalesced.  The same operations and validity tests as
// k_skew, so the same bits.  Where the columns' shifts span more than
// kSkTmaSpan rows (strongly non-square grids) the block reads global memory
// directly.  The wait for the box is bounded: one that runs out sets the
// engine's status word (7), skips the block's rows and waits once more for the
// copy before the block exits.
constexpr int kSkTmaCols = 32, kSkTmaRows = 64, kSkTmaSpan = 64;
constexpr int kSkTmaBox = kSkTmaRows + kSkTmaSpan + 1;
constexpr int kSkTmaBytes = kSkTmaBox * kSkTmaCols * 4;

__global__ void __launch_bounds__(256) k_skew_tma(const __grid_constant__ SkewMaps maps, DevGeometry g, Batch b,
                                                  const float* __restrict__ orient, int64_t n_cells,
                                                  float* __restrict__ SI, int64_t stride, int64_t len,
                                                  bool zero_tail, int* __restrict__ status) {
    __shared__ __align__(128) float box[kSkTmaBox][kSkTmaCols];
    __shared__ __align__(8) uint64_t bar;
    __shared__ int s_tmax, s_tmin;
    const int slot = blockIdx.z;
    const SectorDesc d = g.desc[b.angle[slot]];
    float* out = SI + slot * stride;
    const int c0 = blockIdx.x * kSkTmaCols, r0 = blockIdx.y * kSkTmaRows;
    const int x = threadIdx.x & 31, y = threadIdx.x >> 5;
    if (r0 < d.H && c0 < d.dim_i) {  // uniform over the block
        const int c = c0 + x;
        const int cc = min(c, d.dim_i - 1);
        const int t = g.target[d.col_off + cc];
        if (y == 0) {
            int hi = t, lo = t;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
                lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            }
            if (x == 0) {
                s_tmax = hi;
                s_tmin = lo;
                mbar_init(&bar);
                asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            }
        }
        __syncthreads();
        const int tmax = s_tmax, rbase = r0 - tmax - 1;
        const bool staged = tmax - s_tmin <= kSkTmaSpan;
        bool ok = true;
        if (staged) {
            if (threadIdx.x == 0) {
                mbar_expect(&bar, kSkTmaBytes);
                asm volatile(
                    "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
                    "[%4];" ::"r"(smem_addr(&box[0][0])),
                    "l"(reinterpret_cast<uint64_t>(&maps.t[d.type])), "r"(c0), "r"(rbase), "r"(smem_addr(&bar))
                    : "memory");
            }
            ok = mbar_wait(&bar, 0);
        }
        if (!ok) {
            if (threadIdx.x == 0) {
                atomicExch(status, 7);
                mbar_wait(&bar, 0);  // the copy lands before the block's shared memory is released
            }
        } else if (c < d.dim_i) {
            const float* src = orient + (int64_t)d.type * n_cells;
            const float w = g.weight[d.col_off + c], w1 = __fsub_rn(1.0f, w);
            const int r1 = min(r0 + kSkTmaRows, d.H);
            for (int r = r0 + y; r < r1; r += 8) {
                const int i0 = r - t - 1;
                const bool v0 = (unsigned)i0 < (unsigned)d.dim_o, v1 = (unsigned)(i0 + 1) < (unsigned)d.dim_o;
                float a, bv;
                if (staged) {
                    a = box[i0 - rbase][x];
                    bv = box[i0 + 1 - rbase][x];
                } else {
                    a = v0 ? src[(int64_t)i0 * d.dim_i + c] : 0.0f;
                    bv = v1 ? src[(int64_t)(i0 + 1) * d.dim_i + c] : 0.0f;
                }
                float acc = 0.0f;
                acc = v0 ? __fadd_rn(acc, __fmul_rn(w, a)) : acc;
                acc = v1 ? __fadd_rn(acc, __fmul_rn(w1, bv)) : acc;
                out[(int64_t)r * d.dim_i + c] = acc;
            }
        }
    }
    if (!zero_tail && d.in_width) return;  // nothing reads past H*dim_i
    const int64_t z0 = (int64_t)d.H * d.dim_i;
    const int64_t nthreads = (int64_t)gridDim.x * gridDim.y * blockDim.x;
    for (int64_t q = z0 + ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x; q < len;
         q += nthreads)
        out[q] = 0.0f;
}

__global__ void k_reduce(const float* __restrict__ acc, const float* __restrict__ comp, unsigned used,
                         float* __restrict__ out, int dimx, int dimy, int is_max, int kahan) {
    const int64_t n = (int64_t)dimx * dimy;
    for (int64_t idx = gtid(); idx < n; idx += gstride()) {
        const int i = (int)(idx / dimx);
        const int j = (int)(idx - (int64_t)i * dimx);
        const int ci = dimy - 1 - i, cj = dimx - 1 - j;
        const int64_t at[4] = {idx, (int64_t)cj * dimy + ci, (int64_t)j * dimy + ci, (int64_t)i * dimx + cj};
        if (kahan && !is_max) {
            double s = 0.0;
            for (int t = 0; t < 4; t++)
                if (used & (1u << t)) s += (double)acc[t * n + at[t]] - (double)comp[t * n + at[t]];
            out[idx] = (float)s;
            continue;
        }
        float o = 0.0f;
        for (int t = 0; t < 4; t++) {
            if (!(used & (1u << t))) continue;
            const float v = acc[t * n + at[t]];
            if (is_max) o = o > v ? o : v;
            else o = __fadd_rn(o, v);
        }
        out[idx] = o;
    }
}

inline int blocks_for(int64_t work, int threads, int cap = 65535) {
    int64_t b = (work + threads - 1) / threads;
    if (b < 1) b = 1;
    return (int)(b > cap ? cap : b);
}

}  // namespace

cudaError_t launch_prepare(const float* in, float* orient, int dimx, int dimy, cudaStream_t st) {
    dim3 grid((dimx + kTile - 1) / kTile, (dimy + kTile - 1) / kTile);
    k_prepare<<<grid, dim3(kTile, 8), 0, st>>>(in, orient, dimx, dimy);
    return cudaGetLastError();
}

cudaError_t launch_skew(const DevGeometry& g, const Batch& b, const float* orient, int64_t n_cells, float* SI,
                        int64_t stride, int64_t len, int max_cols, int max_rows, cudaStream_t st, bool zero_tail) {
    dim3 grid((max_cols + kSkewCols - 1) / kSkewCols, (max_rows + kSkewRows - 1) / kSkewRows, b.count);
    k_skew<<<grid, kSkewCols, 0, st>>>(g, b, orient, n_cells, SI, stride, len, zero_tail);
    return cudaGetLastError();
}

int g_skew_path = 0;

int skew_select(int path) {
    if (path != 0 && path != 1) return -1;
    g_skew_path = path;
    return 0;
}

cudaError_t launch_skew_staged(const DevGeometry& g, const Batch& b, const float* orient, int64_t n_cells,
                               float* SI, int64_t stride, int64_t len, int max_cols, int max_rows, cudaStream_t st,
                               bool zero_tail, const SkewMaps* maps, int* status) {
    if (g_skew_path != 1 || !maps || !maps->ok || !status)
        return launch_skew(g, b, orient, n_cells, SI, stride, len, max_cols, max_rows, st, zero_tail);
    dim3 grid((max_cols + kSkTmaCols - 1) / kSkTmaCols, (max_rows + kSkTmaRows - 1) / kSkTmaRows, b.count);
    k_skew_tma<<<grid, 256, 0, st>>>(*maps, g, b, orient, n_cells, SI, stride, len, zero_tail, status);
    return cudaGetLastError();
}

cudaError_t launch_identity(const DevGeometry& g, const Batch& b, const float* SI, float* SO, int64_t stride,
                            int64_t len, cudaStream_t st) {
    dim3 grid(blocks_for(len, 256, 4096), b.count);
    k_identity<<<grid, 256, 0, st>>>(g, b, SI, SO, stride, len);
    return cudaGetLastError();
}

static dim3 deskew_grid(int dimx, int dimy) {
    const int dl = dimx > dimy ? dimx : dimy;  // covers both orientations
    return dim3((dl + kTile - 1) / kTile, (dl + kDeskewRows - 1) / kDeskewRows, 4);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

bool encode_band_maps(DeskewMaps* m, const float* SO, int64_t stride, int slots, int dimx, int dimy) {
    m->ok = false;
    const EncodeTiledFn fn = encode_fn();
    if (!fn || !SO || slots < 1 || stride % 4 || ((uintptr_t)SO & 15)) return false;
    const int widths[2] = {dimx, dimy};
    for (int k = 0; k < 2; k++) {
        const int w = widths[k];
        const int64_t rows = stride / w;
        // Row pitch a multiple of 16 bytes; box no wider or taller than the tensor.
        if (w % 4 || w < kTile || rows < kDeskewBand) return false;
        const cuuint64_t dims[3] = {(cuuint64_t)w, (cuuint64_t)rows, (cuuint64_t)slots};
        const cuuint64_t strides[2] = {(cuuint64_t)w * 4, (cuuint64_t)stride * 4};
        const cuuint32_t box[3] = {(cuuint32_t)kTile, (cuuint32_t)kDeskewBand, 1};
        const cuuint32_t estr[3] = {1, 1, 1};
        if (fn(k == 0 ? &m->x : &m->y, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)SO, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    }
    m->ok = true;
    return true;
}

bool encode_skew_maps(SkewMaps* m, const float* orient, int dimx, int dimy) {
    m->ok = false;
    const EncodeTiledFn fn = encode_fn();
    // Row pitch and orientation offsets multiples of 16 bytes; the box (32 x
    // kSkTmaBox) no wider or taller than an orientation.
    if (!fn || !orient || dimx % 4 || dimy % 4 || dimx < kSkTmaBox || dimy < kSkTmaBox ||
        ((uintptr_t)orient & 15))
        return false;
    const int64_t n = (int64_t)dimx * dimy;
    for (int t = 0; t < 4; t++) {
        const bool tr = t == 1 || t == 2;  // transposed orientations: rows of dimy cells
        const int di = tr ? dimy : dimx, dout = tr ? dimx : dimy;
        const cuuint64_t dims[2] = {(cuuint64_t)di, (cuuint64_t)dout};
        const cuuint64_t strides[1] = {(cuuint64_t)di * 4};
        const cuuint32_t box[2] = {(cuuint32_t)kSkTmaCols, (cuuint32_t)kSkTmaBox};
        const cuuint32_t estr[2] = {1, 1};
        if (fn(&m->t[t], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)(orient + t * n), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    }
    m->ok = true;
    return true;
}

cudaError_t launch_deskew_add(const DevGeometry& g, const TypeLists& tl, const float* SO, int64_t stride,
                              float* acc, float* comp, int dimx, int dimy, int accum_mode, cudaStream_t st,
                              const cd* Q, int64_t pstride, bool masked, const DeskewMaps* maps, int* status) {
    const dim3 grid = deskew_grid(dimx, dimy), block(kTile, 8);
    if (!Q && maps && maps->ok && status) {
        if (accum_mode == kAccumKahan) {
            if (masked)
                k_deskew_tma<kDeskewKahan, true><<<grid, block, 0, st>>>(maps->x, maps->y, g, tl, SO, stride, acc, comp,
                                                                        dimx, dimy, status);
            else
                k_deskew_tma<kDeskewKahan, false><<<grid, block, 0, st>>>(maps->x, maps->y, g, tl, SO, stride, acc,
                                                                         comp, dimx, dimy, status);
        } else {
            if (masked)
                k_deskew_tma<kDeskewAdd, true><<<grid, block, 0, st>>>(maps->x, maps->y, g, tl, SO, stride, acc,
                                                                      nullptr, dimx, dimy, status);
            else
                k_deskew_tma<kDeskewAdd, false><<<grid, block, 0, st>>>(maps->x, maps->y, g, tl, SO, stride, acc,
                                                                       nullptr, dimx, dimy, status);
        }
        return cudaGetLastError();
    }
    if (masked && !Q) {
        if (accum_mode == kAccumKahan)
            k_deskew<kDeskewKahan, false, true><<<grid, block, 0, st>>>(g, tl, SO, stride, acc, comp, dimx, dimy);
        else
            k_deskew<kDeskewAdd, false, true><<<grid, block, 0, st>>>(g, tl, SO, stride, acc, nullptr, dimx, dimy);
        return cudaGetLastError();
    }
    if (Q) {
        if (accum_mode == kAccumKahan)
            k_deskew<kDeskewKahan, true><<<grid, block, 0, st>>>(g, tl, SO, stride, acc, comp, dimx, dimy, Q, pstride);
        else
            k_deskew<kDeskewAdd, true><<<grid, block, 0, st>>>(g, tl, SO, stride, acc, nullptr, dimx, dimy, Q,
                                                              pstride);
    } else if (accum_mode == kAccumKahan) {
        k_deskew<kDeskewKahan><<<grid, block, 0, st>>>(g, tl, SO, stride, acc, comp, dimx, dimy);
    } else {
        k_deskew<kDeskewAdd><<<grid, block, 0, st>>>(g, tl, SO, stride, acc, nullptr, dimx, dimy);
    }
    return cudaGetLastError();
}

cudaError_t launch_deskew_max(const DevGeometry& g, const TypeLists& tl, const float* SO, int64_t stride,
                              float* acc, int dimx, int dimy, cudaStream_t st) {
    k_deskew<kDeskewMax><<<deskew_grid(dimx, dimy), dim3(kTile, 8), 0, st>>>(g, tl, SO, stride, acc, nullptr, dimx,
                                                                            dimy);
    return cudaGetLastError();
}

cudaError_t launch_reduce(const float* acc, const float* comp, unsigned used, float* out, int dimx, int dimy,
                          int is_max, int accum_mode, cudaStream_t st) {
    const int64_t n = (int64_t)dimx * dimy;
    k_reduce<<<blocks_for(n, 256, 8192), 256, 0, st>>>(acc, comp, used, out, dimx, dimy, is_max,
                                                        accum_mode == kAccumKahan);
    return cudaGetLastError();
}

}  // namespace ske
