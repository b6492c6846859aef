// Host-side launchers of the engine's CUDA kernels.  Each returns the launch's
// cudaError_t (cudaGetLastError after the launch).
#pragma once

#include <cstdint>

#include <cuda.h>

#include "ske_device.cuh"

namespace ske {

// Per-type ordered lists of batch slots, for the deskew kernels: slots of type t
// in the order their sectors must be accumulated.
struct TypeLists {
    int count[4];
    int slot[4][kMaxBatch];
    int angle[4][kMaxBatch];
};

// Kahan mode keeps a compensation buffer beside every accumulator.
enum AccumMode { kAccumReference = 0, kAccumKahan = 1 };

// --- layout (k_layout.cu) -------------------------------------------------
// The four orientations of a dimy x dimx input (skewEngine.cuh:925-951):
// orient[t*N ...], t = 0..3.
cudaError_t launch_prepare(const float* in, float* orient, int dimx, int dimy, cudaStream_t st);

// Skewed input of every sector of the batch into slot s of SI (stride floats per
// slot, `len` = 2N + dim_l cells each, zero past H*dim_i).
// zero_tail false: sectors whose rows stay within dim_i leave the cells past
// H*dim_i as they were.
// max_cols / max_rows: the largest dim_i / H of any sector (the grid's extent).
cudaError_t launch_skew(const DevGeometry& g, const Batch& b, const float* orient, int64_t n_cells,
                        float* SI, int64_t stride, int64_t len, int max_cols, int max_rows, cudaStream_t st,
                        bool zero_tail = true);

// Tensor maps of the four input orientations for the TMA-staged skew: 2-D
// float32 views (dim_i columns, dim_o rows) of orient + t*N.
struct SkewMaps {
    CUtensorMap t[4];
    bool ok = false;
};
// Encodes the four maps; false (maps unusable, the gather kernel runs) unless
// both sides are multiples of 4 and at least 129 cells.
bool encode_skew_maps(SkewMaps* m, const float* orient, int dimx, int dimy);
// The same skew as launch_skew with each block's input rows staged by one TMA
// box load when that path is selected (skew_select(1)) and `maps` is usable
// (status: the engine's status word, set when a bounded wait gives up).  The
// column-gather kernel is the default: it measured faster (0.94 against 1.31 ms
// per 2000x2000 step of 180 sectors).
int skew_select(int path);  // 0 = column gather, 1 = TMA-staged; -1 for another value
cudaError_t launch_skew_staged(const DevGeometry& g, const Batch& b, const float* orient, int64_t n_cells,
                               float* SI, int64_t stride, int64_t len, int max_cols, int max_rows, cudaStream_t st,
                               bool zero_tail, const SkewMaps* maps, int* status);

// Identity operator (kernelUNIT.h:16-23): SO = SI on covered cells, 0 elsewhere.
cudaError_t launch_identity(const DevGeometry& g, const Batch& b, const float* SI, float* SO,
                            int64_t stride, int64_t len, cudaStream_t st);

// Deskew + accumulate (skewEngine.cuh:772-792) of every slot of the batch into
// the per-type accumulators acc[t*N ...] (and comp[] in Kahan mode).
// With Q set, the slots are Radon sectors whose rows stay within dim_i, read
// from their filtered row values (Q: pstride complex doubles per slot) instead
// of SO: what the back-projection would write, without writing it.
// Tensor maps of the skewed-output buffer for the TMA-staged deskew: 3-D
// (columns, rows, slots) float32 views with rows of dimx (x) and dimy (y) cells.
struct DeskewMaps {
    CUtensorMap x, y;
    bool ok = false;
};
// Encodes both maps; false (and maps unusable) where the layout does not allow
// TMA (a row width not a multiple of 4 cells or under 32, no driver entry point).
bool encode_band_maps(DeskewMaps* m, const float* SO, int64_t stride, int slots, int dimx, int dimy);

// masked: SO holds defined values only on its sectors' valid cells (rows within
// dim_i, SO not zeroed first); every other cell is read as zero.  With maps
// (ok) and a status word, the bands are staged by TMA (k_deskew_tma); a copy
// that never completes sets *status.
cudaError_t launch_deskew_add(const DevGeometry& g, const TypeLists& tl, const float* SO,
                              int64_t stride, float* acc, float* comp, int dimx, int dimy,
                              int accum_mode, cudaStream_t st, const cd* Q = nullptr, int64_t pstride = 0,
                              bool masked = false, const DeskewMaps* maps = nullptr, int* status = nullptr);
// Max mode with angle encoding (skewEngine.cuh:774-785).
cudaError_t launch_deskew_max(const DevGeometry& g, const TypeLists& tl, const float* SO,
                              int64_t stride, float* acc, int dimx, int dimy, cudaStream_t st);

// Fold the four accumulators back (skewEngine.cuh:862-914) into out (N floats);
// `used` bit t set when type t received at least one sector.
cudaError_t launch_reduce(const float* acc, const float* comp, unsigned used, float* out, int dimx,
                          int dimy, int is_max, int accum_mode, cudaStream_t st);

// --- batched runs over grids of uneven size (k_batch.cu) -------------------
// Every sector of every grid of a batch keeps only its skewed rows' valid
// cells, row after row ("compact rows"): row r of a sector starts at
// cells + rowoff[row_off + r] of the batch's skewed pools and holds
// last[r] - first[r] cells.  A batch applies only to sectors whose rows stay
// within dim_i (every sector of a square grid), where a skewed cell belongs to
// one row and the cells outside the rows are the zeros the reference's deskew
// reads.
struct BatchGrid {
    int dimx, dimy;
    int64_t n;                 // dimx * dimy
    const float* in;           // the caller's input (device)
    float* out;                // the caller's output (device)
    float* orient;             // 4n: the four orientations
    float* acc;                // 4n per-type accumulators
    float* comp;               // 4n Kahan compensations
    const SectorDesc* desc;    // the grid's 180 sector descriptors
    const int32_t* target;
    const float* weight;
    const int32_t* first;
    const int32_t* last;
    const int32_t* rowoff;     // per angle, row r's start within the sector's compact rows
    const int4* rowtab;        // per row (rowoff's layout): {first, last, rowoff, 0}
    unsigned used;             // types that receive a sector
    int ts_start[4];           // sectors of type t: refs[ts_start[t] .. + ts_count[t]]
    int ts_count[4];
};
struct BatchSector {
    int grid, angle;
    int64_t cells;  // start of the sector's compact rows in the skewed pools
};
// What the deskew needs of a sector, in the (grid, type) accumulation order.
struct SectorRef {
    int64_t cells;    // start of its compact rows
    int64_t col_off;  // its target/weight entries
    int64_t row_off;  // its rows in the grid's row tables
    int32_t H, angle;
};
// Tables of one wave of a batched run (device pointers).
struct BatchTables {
    const BatchGrid* grids;
    const BatchSector* sectors;
    const SectorRef* refs;       // sectors grouped by (grid, type), accumulation order inside
    const int64_t* prep_start;   // per grid, its first block of the prepare and fold launches (+ total)
    const int64_t* tile_start;   // per (grid, type), its first deskew tile (+ total)
    const int64_t* skew_start;   // per sector, its first skew block (+ total)
    int n_grids;
    int n_sectors;
};
// Work items of a batch's skew and sweep: (sector index << 32) | row, longest
// row first.
__host__ __device__ inline uint64_t batch_item(int sector, int row) {
    return ((uint64_t)(uint32_t)sector << 32) | (uint32_t)row;
}

// Orientations of every grid of the wave, zeroing their accumulators (and
// compensations, where comp is set).  blocks: prep_start[n_grids].
cudaError_t launch_prepare_batch(const BatchTables& t, int64_t blocks, cudaStream_t st);
// Compact skewed rows of every sector.  blocks: skew_start[n_sectors].
cudaError_t launch_skew_batch(const BatchTables& t, int64_t blocks, float* SI, cudaStream_t st);
// Blocks of the skew launch for one sector of dim_i columns and H rows.
int64_t batch_skew_blocks(int dim_i, int H);
// Deskew + accumulate of every sector of the wave in (grid, type) order;
// tiles: tile_start[4 * n_grids].
cudaError_t launch_deskew_batch(const BatchTables& t, int64_t tiles, const float* SO, int accum_mode,
                                cudaStream_t st);
// Fold of every grid into its output (the maximum with is_max).  blocks:
// prep_start[n_grids].
cudaError_t launch_reduce_batch(const BatchTables& t, int64_t blocks, int accum_mode, cudaStream_t st,
                                int is_max = 0);
// Blocks of the prepare and fold launches for one grid.
int64_t batch_prep_blocks(int dimx, int dimy);
// Deskew tiles of one orientation of a grid (type t: 0..3).
int64_t batch_deskew_tiles(int dimx, int dimy, int t);

// --- operators ------------------------------------------------------------
// Total viewshed sweep (k_sdem.cu).  items: sorted work list (see sdem_items).
struct SdemLaunch {
    DevGeometry g;
    Batch b;
    const float* SI;
    float* SO;
    int64_t stride;
    const uint64_t* items;
    int64_t n_items;
    unsigned* counter;  // work-queue head, zeroed by the launcher
    float povh;
    int max_row;        // longest valid row length of the batch
    int counts_only;    // 1: write integer cv instead of cv*r2
    int* status;        // device error word (0 = ok)
    int4* lists;        // survivor-list scratch (compacting sweep only)
    size_t list_bytes;  // its size; at least sdem_list_bytes(max_row, num_sms)
    // Compacting sweep's level lengths: lvl0 steps, then lvl1 (none when 0),
    // then 64 each; each 16, 32, 48 or 64 (lvl1 also 0).
    int lvl0 = 64, lvl1 = 0;
    int ctas_per_sm = 0;  // compacting sweep: resident CTAs per SM (0 = as many as fit)
    // Batched runs (compacting sweep only): items are batch_item()s whose rows
    // are read from and written to the compact pools SI/SO; g, b and stride
    // are unused.
    int batched = 0;
    BatchTables bt{};
};
// Compacting sweep (the engine's): items are (slot, row), one per valid row.
cudaError_t launch_sdem(const SdemLaunch& a, int num_sms, cudaStream_t st);
// Resident CTAs per SM launch_sdem uses for this launch when ctas_per_sm is 0.
int sdem_max_ctas_per_sm(const SdemLaunch& a);
// Bytes of survivor-list scratch launch_sdem needs for rows up to max_row cells.
size_t sdem_list_bytes(int max_row, int num_sms);
// Work items of a batch for launch_sdem, longest row first: (slot, row).
void sdem_items(const struct Geometry& geo, const Batch& b, std::vector<uint64_t>& items,
                int* max_row);
// Chunked sweep (the allocation-free entry point's): items are (slot, row,
// chunk of sdem_chunk() observers); needs no scratch beyond the item list.
cudaError_t launch_sdem_chunked(const SdemLaunch& a, int num_sms, cudaStream_t st);
int sdem_chunk();

// Radon / filtered back-projection (k_radon.cu).  P: per-slot complex scratch
// of pstride complex doubles; re: per-slot max_H doubles.
// backproject = false leaves SO untouched (the deskew reads P instead).  With
// orient set (only with backproject = false, for sectors whose rows stay within
// dim_i) the row sums gather the skewed cells from the oriented input (n_cells
// per orientation) and SI is not read: the batch needs no skew launch.
cudaError_t launch_radon(const DevGeometry& g, const Batch& b, const float* SI, float* SO,
                         int64_t stride, int64_t len, double* P, int64_t pstride, const double* twiddles,
                         const int64_t* tw_off, int max_H2, cudaStream_t st, bool backproject = true,
                         const float* orient = nullptr, int64_t n_cells = 0, bool f32 = false);

// Kernel launches launch_radon makes (rows_only: gathered sums, no back-projection;
// f32: the float32 mode).
int radon_launches(bool rows_only, int max_H2, bool f32 = false);
// Radon path for later launches: 0 = fused sector kernel where it applies, 1 =
// separate sums and transform; -1 for another value.
int radon_select(int path);

// Local Radon transform (k_lradon.cu): tiles of every sector up to max_H rows
// and max_cols columns; gauss: 180 x 64 weights, taper: the kept bins' factors.
cudaError_t launch_local_radon(const DevGeometry& g, const Batch& b, const float* SI, float* SO, int64_t stride,
                               int max_H, int max_cols, const double* gauss, const double* taper, const double* tw64,
                               cudaStream_t st);

// Cepstrum blur estimation in float32, fused over the sector loop, for a batch
// of square images of side dim (k_cepstrum_f32.cu): orientations from
// t.grids[b].orient, max-accumulators into t.grids[b].acc (initial values
// read), every sector of tl in its type's order.
cudaError_t launch_cepstrum_f32(const BatchTables& t, int images, const DevGeometry& g, const TypeLists& tl, int dim,
                                cudaStream_t st);
cudaError_t cepstrum_f32_init_tables();
// Local Radon in float32 (SKE_FLAG_LOCAL_RADON_F32, k_lradon_f32.cu): the
// twiddle tables (once per device) and the launch (same grid as k_lradon).
int lradon_f32_init_tables();
cudaError_t launch_local_radon_f32(const DevGeometry& g, const Batch& b, const float* SI, float* SO, int64_t stride,
                                   int max_H, int max_cols, const double* gauss, const double* taper,
                                   cudaStream_t st);

// Cepstrum blur estimation (k_cepstrum.cu).
cudaError_t launch_cepstrum(const DevGeometry& g, const Batch& b, const float* SI, float* SO,
                            int64_t stride, int64_t len, const double* tw64, const double* tw32,
                            cudaStream_t st);

// Constant tables used by the SDEM sweep, uploaded once per device.
cudaError_t sdem_init_tables();

// Record `msg` as the calling thread's last error (ske_last_error) and return code.
int set_last_error(int code, const char* msg);

// Exhaustive comparison of the sweep's division with IEEE division over every
// float numerator in the sweep's fast-path range and every d in [1, dmax]
// (synchronous, on the current device).
cudaError_t measure_fp32_peak(int num_sms, int reps, double* scalar_ops, double* packed_ops);
cudaError_t measure_fp64_peak(int num_sms, int reps, double* dfma_ops);

cudaError_t sdem_division_selftest(int dmax, int num_sms, unsigned long long* checked,
                                   unsigned long long* bad, unsigned* first_bad);

}  // namespace ske
