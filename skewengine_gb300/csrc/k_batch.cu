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
constexpr int kRows = 64;              // deskew tile rows
constexpr int kBand = kRows + 34;      // rows + 1 + max column drift over 32 columns (+1)
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

// Compact skewed rows: a warp per work item (sector, row) writes the row's
// valid cells, each the reference scatter's two contributions gathered
// (skew_gather, skewEngine.cuh:615-620).
__global__ void __launch_bounds__(256) k_skew_batch(BatchTables T, const uint64_t* __restrict__ items,
                                                    int64_t n_items, float* __restrict__ SI) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < n_items; w += nwarps) {
        const uint64_t it = items[w];
        const int sidx = (int)(it >> 32), row = (int)(it & 0xffffffffu);
        const BatchSector bs = T.sectors[sidx];
        const BatchGrid& G = T.grids[bs.grid];
        const SectorDesc d = G.desc[bs.angle];
        const int f = G.first[d.row_off + row];
        const int L = G.last[d.row_off + row] - f;
        const int32_t* tg = G.target + d.col_off;
        const float* wg = G.weight + d.col_off;
        const float* src = G.orient + (int64_t)d.type * G.n;
        float* o = SI + bs.cells + G.rowoff[d.row_off + row];
        for (int x = lane; x < L; x += 32) o[x] = skew_gather(d, tg, wg, src, row, f + x);
    }
}

// Skewed output cell (r, c) of a sector in compact rows; zero outside the rows.
__device__ __forceinline__ float compact_cell(const SectorDesc& d, const int32_t* __restrict__ first,
                                              const int32_t* __restrict__ last, const int32_t* __restrict__ rowoff,
                                              const float* __restrict__ so, int r, int c) {
    if (r >= d.H) return 0.0f;
    const int f = first[r];
    return (c >= f && c < last[r]) ? so[rowoff[r] + (c - f)] : 0.0f;
}

// Deskew + accumulate (skewEngine.cuh:772-792) of one 64 x 32 accumulator tile
// of one orientation of one grid over that type's sectors in accumulation
// order, as k_deskew: the tile's accumulators stay in registers; per sector the
// band of skewed rows it needs is staged in shared memory (zeros outside the
// rows), and every thread combines its two cells exactly as the reference.
template <int kMode>
__global__ void __launch_bounds__(256, kMode == kKahan ? 2 : 4)
    k_deskew_batch(BatchTables T, const float* __restrict__ SO) {
    __shared__ float band[kBand][kTile];
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
    const int j0 = (int)(lt % tiles_x) * kTile, i0 = (int)(lt / tiles_x) * kRows;
    if (j0 >= dim_i || i0 >= dim_o) return;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int j = j0 + tx;
    const bool col_ok = j < dim_i;
    const int jlast = min(j0 + kTile, dim_i) - 1;
    const int i_end = min(i0 + kRows, dim_o);
    const int ib = ty * kPer;
    const int nv = min(kPer, i_end - i0 - ib);
    float* A = G.acc + t * n;
    float* Cc = G.comp + t * n;
    float s[kPer], c[kPer];
#pragma unroll
    for (int q = 0; q < kPer; q++) {
        const int i = i0 + ib + q;
        s[q] = (col_ok && i < i_end) ? A[(int64_t)i * dim_i + j] : 0.0f;
        c[q] = (kMode == kKahan && col_ok && i < i_end) ? Cc[(int64_t)i * dim_i + j] : 0.0f;
    }
    const int* ord = T.order + G.ts_start[t];
    for (int q = 0; q < cnt; q++) {
        const BatchSector bs = T.sectors[ord[q]];
        const SectorDesc& d = G.desc[bs.angle];
        const int32_t* tg = G.target + d.col_off;
        const int32_t* rfirst = G.first + d.row_off;
        const int32_t* rlast = G.last + d.row_off;
        const int32_t* roff = G.rowoff + d.row_off;
        const float* so = SO + bs.cells;
        const int tmin = tg[j0], tmax = tg[jlast];
        const int tj = col_ok ? tg[j] : tmin;
        const float w = col_ok ? G.weight[d.col_off + j] : 0.0f;
        const int r0 = i0 + tmin;
        const int nrows = (i_end - i0) + 1 + (tmax - tmin);
        const bool staged = nrows <= kBand;  // always for square grids (drift <= 32 over 32 columns)
        if (staged) {
            constexpr int kLoads = (kBand + 7) / 8;
            float v[kLoads];
#pragma unroll
            for (int u = 0; u < kLoads; u++) {
                const int rr = ty + 8 * u;
                v[u] = (rr < nrows && j0 + tx <= jlast) ? compact_cell(d, rfirst, rlast, roff, so, r0 + rr, j0 + tx)
                                                        : 0.0f;
            }
            __syncthreads();  // previous sector's band fully consumed
#pragma unroll
            for (int u = 0; u < kLoads; u++)
                if (ty + 8 * u < nrows) band[ty + 8 * u][tx] = v[u];
            __syncthreads();
        }
        if (!col_ok || nv <= 0) continue;
        const int off = tj - tmin;
        float cell[kPer + 1];
#pragma unroll
        for (int kk = 0; kk <= kPer; kk++) {
            cell[kk] = 0.0f;
            if (kk > nv) continue;
            cell[kk] = staged ? band[ib + kk + off][tx]
                              : compact_cell(d, rfirst, rlast, roff, so, i0 + ib + kk + tj, j);
        }
#pragma unroll
        for (int q2 = 0; q2 < kPer; q2++) {
            if (q2 >= nv) continue;
            const float v = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, w), cell[q2]), __fmul_rn(w, cell[q2 + 1]));
            if (kMode == kKahan) {
                const float y = __fsub_rn(v, c[q2]);
                const float ts = __fadd_rn(s[q2], y);
                c[q2] = __fsub_rn(__fsub_rn(ts, s[q2]), y);
                s[q2] = ts;
            } else {
                s[q2] = __fadd_rn(s[q2], v);
            }
        }
    }
    if (!col_ok) return;
#pragma unroll
    for (int q = 0; q < kPer; q++) {
        const int i = i0 + ib + q;
        if (i >= i_end) continue;
        A[(int64_t)i * dim_i + j] = s[q];
        if (kMode == kKahan) Cc[(int64_t)i * dim_i + j] = c[q];
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

cudaError_t launch_skew_batch(const BatchTables& t, const uint64_t* items, int64_t n_items, float* SI, int num_sms,
                              cudaStream_t st) {
    if (n_items <= 0) return cudaSuccess;
    int64_t blocks = (n_items + 7) / 8;
    if (blocks > (int64_t)num_sms * 16) blocks = (int64_t)num_sms * 16;
    k_skew_batch<<<(unsigned)blocks, 256, 0, st>>>(t, items, n_items, SI);
    return cudaGetLastError();
}

cudaError_t launch_deskew_batch(const BatchTables& t, int64_t tiles, const float* SO, int accum_mode,
                                cudaStream_t st) {
    if (tiles <= 0) return cudaSuccess;
    if (tiles > 0x7fffffff) return cudaErrorInvalidValue;
    if (accum_mode == kAccumKahan) k_deskew_batch<kKahan><<<(unsigned)tiles, dim3(kTile, 8), 0, st>>>(t, SO);
    else k_deskew_batch<kAdd><<<(unsigned)tiles, dim3(kTile, 8), 0, st>>>(t, SO);
    return cudaGetLastError();
}

cudaError_t launch_reduce_batch(const BatchTables& t, int64_t blocks, int accum_mode, cudaStream_t st, int is_max) {
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffff) return cudaErrorInvalidValue;
    k_reduce_batch<<<(unsigned)blocks, dim3(kTile, 8), 0, st>>>(t, accum_mode == kAccumKahan, is_max);
    return cudaGetLastError();
}

}  // namespace ske
