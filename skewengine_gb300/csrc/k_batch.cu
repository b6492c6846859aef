// Batched runs over grids of uneven size: one launch each for the orientations,
// the skew, the deskew and the fold of every sector of every grid of a wave
// (the sweep runs in between, k_sdem.cu).  The reference runs one grid per
// program and its sectors one at a time per thread (src/main.cu:86-168); here
// a wave's sectors of all grids form one work list.
//
// Skewed grids are kept as compact rows (kernels.h, BatchGrid): only the valid
// cells [first[r], last[r]) of every skewed row, row after row.  A skewed grid
// of a square n x n grid has about 1.44 n^2 cells of which n^2 + n are valid,
// so a wave holds 2 x 4 bytes x (n^2 + n) per sector for its skewed input and
// output, instead of 2 x 4 x (2 n^2 + n) for the reference's skew buffers.
//
// All of these are HBM/L2-bound copies; the arithmetic that must match the
// reference uses explicit _rn intrinsics, as in k_layout.cu.
#include "kernels.h"

namespace ske {

namespace {

constexpr int kTile = 32;
constexpr int kRows = 32;              // deskew tile rows (8 warps x 4 rows)
enum { kAdd = 0, kKahan = 1 };

// Largest k in [0, n) with start[k] <= b (start[n] is the total, above b).
__device__ __forceinline__ int find_entry(const int64_t* __restrict__ start, int n, int64_t b) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (start[mid] <= b) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The four orientations of one 32 x 32 tile of a grid (skewEngine.cuh:925-951,
// as k_prepare), and zeros into the accumulator and compensation cells those
// four writes touch, so every accumulator cell is cleared exactly once.
__global__ void __launch_bounds__(256) k_prepare_batch(BatchTables T) {
    __shared__ float tile[kTile][kTile + 1];
    const int g = find_entry(T.prep_start, T.n_grids, blockIdx.x);
    const BatchGrid& G = T.grids[g];
    const int dimx = G.dimx, dimy = G.dimy;
    const int64_t n = G.n;
    const int64_t lb = blockIdx.x - T.prep_start[g];
    const int tiles_x = (dimx + kTile - 1) / kTile;
    const int j0 = (int)(lb % tiles_x) * kTile, i0 = (int)(lb / tiles_x) * kTile;
    float* o0 = G.orient;
    float* o1 = G.orient + n;
    float* o2 = G.orient + 2 * n;
    float* o3 = G.orient + 3 * n;
    for (int ty = threadIdx.y; ty < kTile; ty += blockDim.y) {
        const int i = i0 + ty, j = j0 + threadIdx.x;
        if (i < dimy && j < dimx) {
            const float v = G.in[(int64_t)i * dimx + j];
            tile[ty][threadIdx.x] = v;
            const int64_t p0 = (int64_t)i * dimx + j, p3 = (int64_t)i * dimx + (dimx - 1 - j);
            o0[p0] = v;
            o3[p3] = v;
            G.acc[p0] = 0.0f;
            G.acc[3 * n + p3] = 0.0f;
            if (G.comp) {
                G.comp[p0] = 0.0f;
                G.comp[3 * n + p3] = 0.0f;
            }
        }
    }
    __syncthreads();
    for (int ty = threadIdx.y; ty < kTile; ty += blockDim.y) {
        const int j = j0 + ty, i = i0 + threadIdx.x;
        if (i < dimy && j < dimx) {
            const float v = tile[threadIdx.x][ty];
            const int ci = dimy - 1 - i, cj = dimx - 1 - j;
            const int64_t p1 = (int64_t)dimy * cj + ci, p2 = (int64_t)dimy * j + ci;
            o1[p1] = v;
            o2[p2] = v;
            G.acc[n + p1] = 0.0f;
            G.acc[2 * n + p2] = 0.0f;
            if (G.comp) {
                G.comp[n + p1] = 0.0f;
                G.comp[2 * n + p2] = 0.0f;
            }
        }
    }
}

// Compact skewed rows, streamed by column as k_skew does: a thread owns column
// c of kSkewRows consecutive skewed rows of one sector.  Cell (r, c) is the
// reference scatter's two contributions gathered (skew_gather,
// skewEngine.cuh:615-620): w*x[r-t-1][c] + (1-w)*x[r-t][c] onto 0; the
// column's target and weight stay in registers and row r's second source value
// is row r+1's first, so a cell costs one load.  Row r's valid cells
// [first, last) go to the row's compact segment, so a block's stores to one row
// are consecutive.
constexpr int kSkewRows = 32;
constexpr int kSkewCols = 256;

__global__ void __launch_bounds__(kSkewCols) k_skew_batch(BatchTables T, float* __restrict__ SI) {
    __shared__ int4 meta[kSkewRows];
    const int sidx = find_entry(T.skew_start, T.n_sectors, blockIdx.x);
    const BatchSector bs = T.sectors[sidx];
    const BatchGrid& G = T.grids[bs.grid];
    const SectorDesc& d = G.desc[bs.angle];
    const int dim_i = d.dim_i, dim_o = d.dim_o, H = d.H;
    const int64_t lb = blockIdx.x - T.skew_start[sidx];
    const int bx_n = (dim_i + kSkewCols - 1) / kSkewCols;
    const int c = (int)(lb % bx_n) * kSkewCols + threadIdx.x;
    const int r0 = (int)(lb / bx_n) * kSkewRows;
    const int r1 = min(r0 + kSkewRows, H);
    if (threadIdx.x < r1 - r0) meta[threadIdx.x] = G.rowtab[d.row_off + r0 + threadIdx.x];
    __syncthreads();
    if (c >= dim_i) return;
    const float* src = G.orient + (int64_t)d.type * G.n;
    const int t = G.target[d.col_off + c];
    const float w = G.weight[d.col_off + c], w1 = __fsub_rn(1.0f, w);
    int i0 = r0 - t - 1;  // source row of the w term
    const float* p = src + ((int64_t)i0 * dim_i + c);
    float a = (unsigned)i0 < (unsigned)dim_o ? p[0] : 0.0f;
    float* out = SI + bs.cells;
    for (int r = r0; r < r1; r++) {
        const bool v0 = (unsigned)i0 < (unsigned)dim_o, v1 = (unsigned)(i0 + 1) < (unsigned)dim_o;
        const float bv = v1 ? p[dim_i] : 0.0f;
        const int4 m = meta[r - r0];
        if (c >= m.x && c < m.y) {
            float acc = 0.0f;
            acc = v0 ? __fadd_rn(acc, __fmul_rn(w, a)) : acc;
            acc = v1 ? __fadd_rn(acc, __fmul_rn(w1, bv)) : acc;
            out[m.z + (c - m.x)] = acc;
        }
        a = bv;
        i0++;
        p += dim_i;
    }
}

// A sector's kPer + 1 staged cells of this thread's column (zero outside the
// sector's rows and outside a row's valid range).
template <int kPer>
__device__ __forceinline__ void deskew_cells(const BatchGrid& G, const SectorRef& d, int tj, int ib, int j, int nv,
                                             const float* __restrict__ SO, float* cell) {
    const int4* rt = G.rowtab + d.row_off;
    const float* so = SO + d.cells;
#pragma unroll
    for (int kk = 0; kk <= kPer; kk++) {
        const int r = ib + kk + tj;
        cell[kk] = 0.0f;
        if (kk <= nv && r < d.H) {
            const int4 m = rt[r];
            if (j >= m.x && j < m.y) cell[kk] = so[m.z + (j - m.x)];
        }
    }
}

// Deskew + accumulate (skewEngine.cuh:772-792) of one kRows x 32 accumulator
// tile of one orientation of one grid over that type's sectors in accumulation
// order.  A thread owns kPer consecutive accumulator rows of one column, keeps
// them in registers, and per sector gathers the kPer+1 skewed cells they need
// (rows i+t_j .. i+t_j+kPer of column j; a cell outside its row's valid range
// is zero) straight from the compact rows: one row-table load and one value
// load per cell, lanes of a warp on consecutive columns.  There are no
// barriers, so warps advance independently and hide each other's latency; the
// next sector's cells are loaded before the current one is accumulated, and
// descriptors, targets and weights two sectors ahead.  The arithmetic is the
// reference's, in its order.
template <int kMode>
__global__ void __launch_bounds__(256, 4) k_deskew_batch(BatchTables T, const float* __restrict__ SO) {
    constexpr int kPer = kRows / 8;
    const int k = find_entry(T.tile_start, 4 * T.n_grids, blockIdx.x);
    const int gi = k >> 2, t = k & 3;
    const BatchGrid& G = T.grids[gi];
    const int cnt = G.ts_count[t];
    if (cnt == 0) return;
    const int64_t n = G.n;
    const int dim_i = (t == 1 || t == 2) ? G.dimy : G.dimx;
    const int dim_o = (t == 1 || t == 2) ? G.dimx : G.dimy;
    const int64_t lt = blockIdx.x - T.tile_start[k];
    const int tiles_x = (dim_i + kTile - 1) / kTile;
    const int j = (int)(lt % tiles_x) * kTile + (threadIdx.x & 31);
    const int ib = (int)(lt / tiles_x) * kRows + (threadIdx.x >> 5) * kPer;
    if (j >= dim_i || ib >= dim_o) return;
    const int nv = min(kPer, dim_o - ib);
    float* A = G.acc + t * n + (int64_t)ib * dim_i + j;
    float* Cc = G.comp + t * n + (int64_t)ib * dim_i + j;
    float s[kPer], c[kPer];
#pragma unroll
    for (int q = 0; q < kPer; q++) {
        s[q] = q < nv ? A[(int64_t)q * dim_i] : 0.0f;
        c[q] = (kMode == kKahan && q < nv) ? Cc[(int64_t)q * dim_i] : 0.0f;
    }
    // Software pipeline: the cells of sector q + 1 are loaded before sector q is
    // accumulated, and descriptors, targets and weights two sectors ahead.
    const SectorRef* refs = T.refs + G.ts_start[t];
    const SectorRef d0 = refs[0];
    float cell[kPer + 1], nxt[kPer + 1];
    deskew_cells<kPer>(G, d0, G.target[d0.col_off + j], ib, j, nv, SO, cell);
    float w = G.weight[d0.col_off + j];
    SectorRef d1 = d0;
    int t1 = 0;
    float w_1 = 0.0f;
    if (cnt > 1) {
        d1 = refs[1];
        t1 = G.target[d1.col_off + j];
        w_1 = G.weight[d1.col_off + j];
    }
    for (int q = 0; q < cnt; q++) {
        if (q + 1 < cnt) deskew_cells<kPer>(G, d1, t1, ib, j, nv, SO, nxt);
        SectorRef d2 = d1;
        int t2 = 0;
        float w_2 = 0.0f;
        if (q + 2 < cnt) {
            d2 = refs[q + 2];
            t2 = G.target[d2.col_off + j];
            w_2 = G.weight[d2.col_off + j];
        }
        const float w1 = __fsub_rn(1.0f, w);
#pragma unroll
        for (int q2 = 0; q2 < kPer; q2++) {
            if (q2 >= nv) continue;
            const float v = __fadd_rn(__fmul_rn(w1, cell[q2]), __fmul_rn(w, cell[q2 + 1]));
            if (kMode == kKahan) {
                const float y = __fsub_rn(v, c[q2]);
                const float ts = __fadd_rn(s[q2], y);
                c[q2] = __fsub_rn(__fsub_rn(ts, s[q2]), y);
                s[q2] = ts;
            } else {
                s[q2] = __fadd_rn(s[q2], v);
            }
        }
#pragma unroll
        for (int kk = 0; kk <= kPer; kk++) cell[kk] = nxt[kk];
        w = w_1;
        d1 = d2;
        t1 = t2;
        w_1 = w_2;
    }
#pragma unroll
    for (int q = 0; q < kPer; q++) {
        if (q >= nv) continue;
        A[(int64_t)q * dim_i] = s[q];
        if (kMode == kKahan) Cc[(int64_t)q * dim_i] = c[q];
    }
}

// Fold (skewEngine.cuh:862-914, as k_reduce) of one 32 x 32 output tile of a
// grid: the used types in type order, compensated sums in double for Kahan,
// the maximum for the cepstrum.
__global__ void __launch_bounds__(256) k_reduce_batch(BatchTables T, int kahan, int is_max) {
    const int g = find_entry(T.prep_start, T.n_grids, blockIdx.x);
    const BatchGrid& G = T.grids[g];
    const int dimx = G.dimx, dimy = G.dimy;
    const int64_t n = G.n;
    const int64_t lb = blockIdx.x - T.prep_start[g];
    const int tiles_x = (dimx + kTile - 1) / kTile;
    const int j = (int)(lb % tiles_x) * kTile + threadIdx.x;
    const int i0 = (int)(lb / tiles_x) * kTile;
    if (j >= dimx) return;
    const unsigned used = G.used;
    for (int i = i0 + threadIdx.y; i < min(i0 + kTile, dimy); i += blockDim.y) {
        const int ci = dimy - 1 - i, cj = dimx - 1 - j;
        const int64_t idx = (int64_t)i * dimx + j;
        const int64_t at[4] = {idx, (int64_t)cj * dimy + ci, (int64_t)j * dimy + ci, (int64_t)i * dimx + cj};
        if (is_max) {
            float o = 0.0f;
            for (int t = 0; t < 4; t++)
                if (used & (1u << t)) {
                    const float v = G.acc[t * n + at[t]];
                    o = o > v ? o : v;
                }
            G.out[idx] = o;
        } else if (kahan) {
            double sum = 0.0;
            for (int t = 0; t < 4; t++)
                if (used & (1u << t)) sum += (double)G.acc[t * n + at[t]] - (double)G.comp[t * n + at[t]];
            G.out[idx] = (float)sum;
        } else {
            float o = 0.0f;
            for (int t = 0; t < 4; t++)
                if (used & (1u << t)) o = __fadd_rn(o, G.acc[t * n + at[t]]);
            G.out[idx] = o;
        }
    }
}

}  // namespace

int64_t batch_prep_blocks(int dimx, int dimy) {
    return (int64_t)((dimx + kTile - 1) / kTile) * ((dimy + kTile - 1) / kTile);
}

int64_t batch_deskew_tiles(int dimx, int dimy, int t) {
    const int dim_i = (t == 1 || t == 2) ? dimy : dimx;
    const int dim_o = (t == 1 || t == 2) ? dimx : dimy;
    return (int64_t)((dim_i + kTile - 1) / kTile) * ((dim_o + kRows - 1) / kRows);
}

cudaError_t launch_prepare_batch(const BatchTables& t, int64_t blocks, cudaStream_t st) {
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffff) return cudaErrorInvalidValue;
    k_prepare_batch<<<(unsigned)blocks, dim3(kTile, 8), 0, st>>>(t);
    return cudaGetLastError();
}

int64_t batch_skew_blocks(int dim_i, int H) {
    return (int64_t)((dim_i + kSkewCols - 1) / kSkewCols) * ((H + kSkewRows - 1) / kSkewRows);
}

cudaError_t launch_skew_batch(const BatchTables& t, int64_t blocks, float* SI, cudaStream_t st) {
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffff) return cudaErrorInvalidValue;
    k_skew_batch<<<(unsigned)blocks, kSkewCols, 0, st>>>(t, SI);
    return cudaGetLastError();
}

cudaError_t launch_deskew_batch(const BatchTables& t, int64_t tiles, const float* SO, int accum_mode,
                                cudaStream_t st) {
    if (tiles <= 0) return cudaSuccess;
    if (tiles > 0x7fffffff) return cudaErrorInvalidValue;
    if (accum_mode == kAccumKahan) k_deskew_batch<kKahan><<<(unsigned)tiles, 256, 0, st>>>(t, SO);
    else k_deskew_batch<kAdd><<<(unsigned)tiles, 256, 0, st>>>(t, SO);
    return cudaGetLastError();
}

cudaError_t launch_reduce_batch(const BatchTables& t, int64_t blocks, int accum_mode, cudaStream_t st, int is_max) {
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffff) return cudaErrorInvalidValue;
    k_reduce_batch<<<(unsigned)blocks, dim3(kTile, 8), 0, st>>>(t, accum_mode == kAccumKahan, is_max);
    return cudaGetLastError();
}

}  // namespace ske
