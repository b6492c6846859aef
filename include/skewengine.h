/*
 * skewengine.h -- C ABI of the GB300-native skewed-data-mapping engine.
 *
 * The engine runs the sector loop of luisfromero/skewEngine on one GPU:
 * for every integer angle a in [0, max_sector) it skews the 2-D input so that
 * lines at angle a become memory rows, runs a per-row operator over the valid
 * part [first, last) of every skewed row, deskews the result and accumulates it
 * into one of four orientation buffers, and finally folds those back into the
 * input orientation.  All compute is hand-written sm_103a CUDA; there is no CPU
 * fallback: without a usable GPU every compute entry point returns an error.
 *
 * Conventions
 *  - Every entry point returns an int status (SKE_OK == 0).  On failure the
 *    message of the calling thread's last error is available from
 *    ske_last_error().  Nothing in the library calls exit() or traps on device,
 *    and no C++ exception leaves it: a request too large for host memory
 *    returns SKE_ERR_INVALID with a "host:" message.
 *  - Arrays are row-major float32, dimy rows of dimx cells, like the reference's
 *    inputD / outD (src/global.cpp:24).
 *  - "on_device" arguments say whether a pointer is a device pointer (1) or a
 *    host pointer (0).  Host buffers are staged through the engine's pinned
 *    buffers.
 *  - An engine is bound to one device and one CUDA stream; calls on one engine
 *    are not thread-safe (as one reference skewEngine object per OpenMP thread,
 *    src/main.cu:91).  Different engines may be used from different threads.
 *  - Device buffers are read and written in the engine's stream order: a caller
 *    that produces an input (or still reads an output buffer) on another stream
 *    makes the engine's stream wait for that work first (an event, or the
 *    engine created on the caller's stream).  A call that runs sectors has
 *    finished its device work when it returns.
 */
#ifndef SKEWENGINE_H
#define SKEWENGINE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SKE_ABI_VERSION 1

/* Status codes. */
#define SKE_OK 0
#define SKE_ERR_INVALID 1     /* bad argument (null pointer, size, angle ...)  */
#define SKE_ERR_CUDA 2        /* a CUDA runtime call failed                     */
#define SKE_ERR_NO_DEVICE 3   /* no usable CUDA device                          */
#define SKE_ERR_STATE 4       /* call out of order (e.g. kernel() before skew())*/
#define SKE_ERR_UNSUPPORTED 5 /* valid request the library does not support     */
#define SKE_ERR_DEVICE 6      /* a kernel reported an error through its status  */

/* Operators: values of the reference KERNELS enum (src/global.h:77). */
#define SKE_KERNEL_SDEM 0        /* total viewshed, kernelV3 (src/kernelSDEM.h:168)   */
#define SKE_KERNEL_IDENTITYDEM 1 /* identity, kernelUNIT.h:16                         */
#define SKE_KERNEL_RADON 2       /* Radon + filtered back-projection, kernelRADN.h:213*/
#define SKE_KERNEL_IDENTITYIMG 3 /* identity, kernelUNIT.h:16                         */
#define SKE_KERNEL_CEPSTRUM 4    /* cepstrum blur estimation, kernelBLUR.h:267        */
/* The reference's Radon operator with its LRT switch set (kernelRADN.h:212-220):
   the local Radon transform pointRadon (kernelRADN.h:114-182) of every skewed
   cell, added back like the global transform.  The reference has no operator id
   for it; 5 follows its enum. */
#define SKE_KERNEL_LOCAL_RADON 5

/* Cross-sector accumulation of the additive operators. */
#define SKE_ACCUM_REFERENCE 0 /* float adds in sector order, bit-identical to the
                                 reference run on one thread (skewEngine.cuh:786-792) */
#define SKE_ACCUM_KAHAN 1     /* compensated (Kahan) float sums per orientation,
                                 folded in double at the end                       */

/* Run parameters (reference: compile-time globals of src/global.cpp and
 * src/kernelSDEM.h). */
typedef struct ske_params {
    int32_t max_sector; /* angles 0..max_sector-1, 1..180 (global.cpp:69, default 180) */
    float povh;         /* observer height in cell units (kernelSDEM.h:159, 1.5/10)    */
    int32_t accum;      /* SKE_ACCUM_*                                                  */
    int32_t flags;      /* SKE_FLAG_* bits, 0 by default                                */
} ske_params;

/* ske_params.flags (no counterpart in the reference). */
#define SKE_FLAG_NO_TUNE 1  /* keep the viewshed sweep's built-in shape: skip the
                               autotuner that times a few level schedules and CTA
                               counts on the first run (results are identical)   */
#define SKE_FLAG_NO_GRAPH 2 /* batched runs: launch the kernels of every call
                               directly instead of replaying a captured CUDA graph */
#define SKE_FLAG_CEPSTRUM_F32 4 /* cepstrum of square images in float32 on the FP32
                               pipes, skew + operator + max-deskew fused in one
                               launch per batch: outputs may fall in another
                               1000-wide bin than the reference's binary64 where a
                               value sits at a bin edge (a measured, stated rate);
                               without the flag the cepstrum is the reference's,
                               bit for bit                                         */
#define SKE_FLAG_RADON_F32 16 /* Radon ray sums, transform and ramp filter in
                               float32 on the FP32 pipes (sectors up to 8192
                               rows); values differ from the reference's binary64
                               in their low bits (a measured, stated error);
                               without the flag the operator is the reference's,
                               bit for bit                                         */
#define SKE_FLAG_LOCAL_RADON_F32 8 /* local Radon transform in float32 on the
                               FP32 pipes (direct sums over the transform bins the
                               reference reads); values differ in their last bits
                               and, where two successive |Z|^2 nearly tie, the
                               first ascent can fall on another bin (a measured,
                               stated rate); without the flag it is the
                               reference's binary64, bit for bit                   */

/* Geometry of one sector, computeParams + skewShape (skewEngine.cuh:504-596). */
typedef struct ske_sector_geometry {
    int32_t angle;       /* a                                   */
    int32_t sector_type; /* 0..3: plain, transposed, transposed+mirrored, mirrored */
    int32_t new_angle;   /* angle folded into [0, 45]            */
    int32_t dim_i;       /* inner (row) length = skewWidth        */
    int32_t dim_o;       /* outer dimension                      */
    int32_t offset;      /* (int)(skewness*(dim_i-1))            */
    int32_t skew_height; /* rows of the skewed grid              */
    int32_t dim_l;       /* max(dimx, dimy)                      */
    double scale;        /* 1/cos(new_angle)                     */
    double skewness;     /* tan(new_angle)                       */
} ske_sector_geometry;

/* Device view of the current sector handed to a custom operator: the fields the
 * reference passes to kernelcuda (skewEngine.cuh:369, :709) plus geometry.
 * skew_in/skew_out hold 2*dimx*dimy + dim_l floats, row stride dim_i. */
typedef struct ske_sector_view {
    ske_sector_geometry geom;
    float* skew_out;       /* d_skewOutput (zeroed before the operator runs) */
    const float* skew_in;  /* d_skewInput                                     */
    const int32_t* first;  /* d_first[skew_height]                            */
    const int32_t* last;   /* d_last[skew_height]                             */
    const int32_t* target; /* d_target[dim_i]                                 */
    const float* weight;   /* d_weight[dim_i]                                 */
    float povh;
    void* stream;          /* cudaStream_t the operator must launch on       */
} ske_sector_view;

/* A custom device operator: launches its own kernels on view->stream, reading
 * skew_in and writing skew_out over [first[r], last[r]) of every row r.
 * Replaces the reference's kernelcuda function pointer (skewEngine.cuh:369).
 * Return 0 on success. */
typedef int (*ske_operator_fn)(void* user, const ske_sector_view* view);

typedef struct ske_engine_s* ske_engine;

/* Library / device ---------------------------------------------------------*/

/* ABI version (SKE_ABI_VERSION). */
int ske_abi_version(void);

/* Message of the calling thread's last failed call ("" if none). */
const char* ske_last_error(void);

/* Fill *p with the reference defaults: 180 sectors, povh = 1.5/10,
 * accumulation in reference order. */
int ske_params_default(ske_params* p);

/* Number of CUDA devices visible (0 on a machine without a GPU). */
int ske_device_count(int* count);

/* Host-only geometry of one sector (no GPU needed): replaces
 * skewEngine::computeParams/skewShape (skewEngine.cuh:504-596).  first/last
 * (skew_height entries each) and target/weight (dim_i entries each) may be NULL;
 * size them with a first call that passes NULL. */
int ske_geometry(int dimx, int dimy, int angle, ske_sector_geometry* geom, int32_t* first,
                 int32_t* last, int32_t* target, float* weight);

/* Engine lifetime ----------------------------------------------------------*/

/* Create an engine for dimx x dimy grids on `device`, launching on `stream`
 * (a cudaStream_t; NULL = the engine creates its own).  Replaces the skewEngine
 * constructor + skewAlloc (skewEngine.cuh:462, :419) and the per-thread
 * cudaSetDevice/cudaStreamCreate of skewCudaMalloc (skewEngine.cuh:1030-1031). */
int ske_create(ske_engine* out, int dimx, int dimy, int device, void* stream);

/* Release every device and host resource of the engine (skewEngine::~skewEngine,
 * skewEngine.cuh:484-501). */
int ske_destroy(ske_engine e);

/* The CUDA stream the engine launches on. */
int ske_stream(ske_engine e, void** stream);

/* Whole run ----------------------------------------------------------------*/

/* Full sector loop for one operator: prepare the four orientations, run every
 * sector 0..p->max_sector-1 (skew -> operator -> deskew/accumulate), fold the
 * orientations back, and write dimx*dimy floats to `output`.  Replaces
 * skewEngine::allocate + execute() + reduce (skewEngine.cuh:389, main.cu:71-172,
 * skewEngine.cuh:862).  Results equal the reference run on one OpenMP thread
 * (bit for bit for SDEM/identity/Radon in SKE_ACCUM_REFERENCE mode).
 * The total-viewshed sweep stages each skewed row in shared memory: rows of up
 * to 13,224 cells fit a GB300's 227 KB per CTA (grids whose longer side is at
 * most that); a longer row fails the launch and the call returns
 * SKE_ERR_CUDA. */
int ske_run(ske_engine e, int kernel, const float* input, int input_on_device, float* output,
            int output_on_device, const ske_params* p);

/* Same with a caller-supplied list of angles (each in [0,180)), processed and
 * accumulated in list order. */
int ske_run_angles(ske_engine e, int kernel, const float* input, int input_on_device,
                   float* output, int output_on_device, const int32_t* angles, int nangles,
                   const ske_params* p);

/* Run the listed sectors and return, instead of the folded output, the four
 * per-type accumulators (4*dimx*dimy floats, type-major, each in its sector
 * type's orientation) and the mask of types that received a sector: the state a
 * reference engine thread holds before its critical-section reduce
 * (skewEngine.cuh:270-273, main.cu:160-164).  Used to shard sectors across
 * GPUs; fold with the reduce order of skewEngine.cuh:885-912. */
int ske_accumulate(ske_engine e, int kernel, const float* input, int input_on_device,
                   const int32_t* angles, int nangles, const ske_params* p, float* acc,
                   int acc_on_device, uint32_t* used_mask);

/* Test hook (no reference counterpart): the device or pinned-host allocation
 * `after` allocations from now fails as if out of memory (0 = the next one);
 * negative turns injection off.  Calls that hit it return SKE_ERR_CUDA with
 * nothing leaked; used to test failure handling without faulting a GPU. */
int ske_inject_alloc_failure(int64_t after);

/* Checkpoint / resume at sector granularity.  Like ske_accumulate, but the
 * per-type accumulators start from the state in acc (4*N floats), comp (4*N
 * Kahan compensations; Kahan mode only, else may be null) and *used_mask
 * instead of from zero, and return the state after the listed sectors in the
 * same buffers (host or device, state_on_device).  Accumulating angles [0,k)
 * and then [k,180) this way leaves the same bits as one pass over [0,180):
 * the additions continue in the same order.  The reference has no such call;
 * its sector loop (main.cu:147-164) keeps this state in the engine. */
int ske_accumulate_resume(ske_engine e, int kernel, const float* input, int input_on_device,
                          const int32_t* angles, int nangles, const ske_params* p, float* acc,
                          float* comp, int state_on_device, uint32_t* used_mask);

/* Fold a saved accumulator state into the output grid exactly as ske_run's
 * final reduce does (skewEngine.cuh:862-914): max for the cepstrum, sums
 * otherwise (compensated in Kahan mode). */
int ske_fold(ske_engine e, int kernel, const float* acc, const float* comp, int state_on_device,
             uint32_t used_mask, int accum, float* output, int output_on_device);

/* Batched total viewshed (SDEM) over `count` square or rectangular DEMs of
 * uneven sizes: inputs[i]/outputs[i] are dimx[i] x dimy[i] host or device
 * arrays.  All DEMs and all their sectors are scheduled together.  Engines are
 * created for the largest grid internally; `e` supplies device and stream. */
int ske_run_batch(ske_engine e, int kernel, int count, const int32_t* dimx, const int32_t* dimy,
                  const float* const* inputs, int inputs_on_device, float* const* outputs,
                  int outputs_on_device, const ske_params* p);

/* ske_run_batch over the listed angles (each in [0,180), accumulated in list
 * order) for every DEM, as ske_run_angles is ske_run over a list.
 *
 * Total viewshed (SKE_KERNEL_SDEM): the grids whose sectors' rows stay within
 * their width (every square grid) run together.  The engine keeps a plan of
 * the batch (geometry per grid size, buffers, work lists) while later calls
 * bring the same grid sizes and angles; its memory budget splits the batch into
 * waves, and each wave is five kernel launches over all of its grids and
 * sectors (orientations, skew, viewshed sweep, deskew, fold; the main loop of
 * src/main.cu:86-168 for every grid at once), replayed as a captured CUDA graph
 * from the second call on (SKE_FLAG_NO_GRAPH: plain launches).  Results are the
 * same as ske_run_angles on each grid, bit for bit in both accumulation modes.
 * Float32 cepstrum (SKE_KERNEL_CEPSTRUM with SKE_FLAG_CEPSTRUM_F32): each run of
 * consecutive square images of one side shares one launch sequence.  Other
 * grids and other operators run one grid at a time. */
int ske_run_batch_angles(ske_engine e, int kernel, int count, const int32_t* dimx, const int32_t* dimy,
                         const float* const* inputs, int inputs_on_device, float* const* outputs,
                         int outputs_on_device, const int32_t* angles, int nangles, const ske_params* p);

/* Radon operator's kernels for sectors whose rows stay within their width:
 * 0 = one fused sector kernel (a thread-block cluster per sector: row sums into
 * the leader's shared memory, then the filtered transform), 1 (default) = row
 * sums and transform as two launches, which measured faster on GB300.  Same
 * results.  No reference counterpart. */
int ske_radon_select(int path);

/* Skew kernel for later runs of every engine: 0 (default) = column gather (each
 * thread streams one skewed column from the L2-resident orientations), 1 = each
 * 32-column x 64-row block's source rows staged by one TMA box load (grids whose
 * sides are multiples of 4 and at least 129 cells; others keep the gather).
 * Both give the same bits; the gather measured faster (0.94 against 1.31 ms per
 * 2000x2000 step of 180 sectors).  Replaces no reference call (cudaSkew,
 * skewEngine.cuh:56-88, is one kernel). */
int ske_skew_select(int path);

/* Shape of the last viewshed sweep the engine launched: level schedule (lvl0
 * steps, then lvl1 when non-zero, then 64-step levels) and resident CTAs per SM
 * (0 = as many as fit), as chosen by the autotuner.  No reference counterpart. */
int ske_sweep_shape(ske_engine e, int* lvl0, int* lvl1, int* ctas_per_sm);

/* Fix the viewshed sweep's shape for this engine's later runs instead of the
 * autotuner's choice: lvl0 and lvl1 of 16, 32, 48 or 64 steps (lvl1 0: none),
 * ctas_per_sm 0 = as many as fit.  lvl0 = 0 returns the choice to the
 * autotuner.  Results do not depend on the shape.  No reference counterpart. */
int ske_set_sweep_shape(ske_engine e, int lvl0, int lvl1, int ctas_per_sm);

/* Per-sector API (drop-in for the reference's skew/kernel/deskew/reduce
 * methods driven from main.cu:147-164) ----------------------------------------*/

/* Upload `input` and build the four orientations (skewEngine::prepare,
 * skewEngine.cuh:925-987 + the H2D copies of skewCudaMalloc :1041-1044); clears
 * the four orientation accumulators (d_output, :1040). */
int ske_prepare(ske_engine e, const float* input, int on_device);

/* skewEngine::skew(angle) (skewEngine.cuh:606): geometry of `angle`, reset and
 * fill the skewed input. */
int ske_skew(ske_engine e, int angle);

/* skewEngine::kernel() (skewEngine.cuh:695): run a built-in operator over the
 * current skewed grid. */
int ske_kernel(ske_engine e, int kernel, float povh);

/* Run a custom device operator over the current skewed grid. */
int ske_kernel_custom(ske_engine e, ske_operator_fn fn, void* user, float povh);

/* skewEngine::deskew(isMax) (skewEngine.cuh:756): deskew the current skewed
 * output into the accumulator of the current sector type.  is_max = 1 for the
 * cepstrum max/angle encoding, 0 to add.  accum = SKE_ACCUM_*. */
int ske_deskew(ske_engine e, int is_max, int accum);

/* skewEngine::reduce(out, isMax) (skewEngine.cuh:862): fold the four
 * accumulators into `output` (dimx*dimy).  `output` is overwritten (the
 * reference adds into a caller-zeroed outD). */
int ske_reduce(ske_engine e, float* output, int on_device, int is_max);

/* Geometry and device buffers of the current sector. */
int ske_sector(ske_engine e, ske_sector_view* view);

/* Copy the current skewed input / output (2*dimx*dimy + dim_l floats). */
int ske_copy_skewed(ske_engine e, float* skew_in, float* skew_out, int on_device);

/* Total-viewshed visibility counts of one sector: for every skewed cell in
 * [first,last) the integer-valued sum cv of kernelSDEM.h:182-218 before the
 * scale factor; other cells 0.  counts: 2*dimx*dimy + dim_l floats. */
int ske_sdem_counts(ske_engine e, int angle, float povh, float* counts, int on_device);

/* Total-viewshed sweep of ONE skewed sector that allocates nothing.  No
 * counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc -- code that runs under a fixed GPU
 * memory budget, inside another framework's allocator, or on a path where
 * allocation is forbidden -- this runs the viewshed sweep (its chunked form,
 * whose only scratch is its work list) over a skewed sector the caller already
 * holds in device memory: `skew_in` (row stride dim_i), `first`/`last`
 * (skew_height int32 entries, device, every row with 0 <= first <= last <=
 * dim_l like the engine's own geometry; any other row is rejected with
 * SKE_ERR_INVALID), and writes cv*scale2 to every valid cell of `skew_out`
 * (other cells are left as they are: zero the buffer first, as resetSkew
 * does, skewEngine.cuh:542-570).  `skew_in` and `skew_out` must each hold at
 * least (skew_height-1)*dim_i + dim_l floats, the last cell a row can reach;
 * the engine's own skew buffers hold 2*dimx*dimy + dim_l (skewEngine.cuh:425-426).
 * Results equal the built-in SDEM operator's on the same sector bit for bit.
 *
 * Its scratch (sector descriptor, work-queue head, status word, work items) is
 * a file-scope device array of about 8 MiB that every GPU loading this library
 * holds until the process exits; limits: dim_l <= 4096, skew_height <= 131072,
 * at most 2^20 work items of 128 observers.  Larger sectors are rejected with
 * SKE_ERR_INVALID and a message.  No cudaMalloc, cudaFree or allocating library
 * routine is called.  The first call on a device takes the array's device
 * address and uploads the sweep's constant table; make that first call before
 * any stream capture.  Every call shares the array and keeps the last call's
 * contents (the queue head and status are cleared on each call); calls that
 * overlap on the GPU race, calls from several host threads are serialised.
 * Every call copies the row limits and, at the end, a status word to the host
 * and waits for `stream` (a cudaStream_t, NULL = default) each time, so it
 * returns with the sweep finished.  The calling thread's current device is
 * restored before the call returns. */
int ske_sdem_sector_noalloc(int device, const float* skew_in, float* skew_out, int dim_i,
                            int skew_height, int dim_l, const int32_t* first, const int32_t* last,
                            float scale2, float povh, void* stream);

/* Profiling ----------------------------------------------------------------*/

/* Enable (1) / disable (0) CUDA-event timing of every kernel launch. */
int ske_profile_enable(ske_engine e, int enable);

/* Accumulated device time (ms) and launch count of kernel family `name`
 * ("prepare", "skew", "sdem_sweep", "radon_sums", "radon_fft", "cepstrum",
 *  "identity", "deskew", "reduce") since profiling was enabled; synchronises the
 * engine's stream. */
int ske_profile_get(ske_engine e, const char* name, double* ms, int64_t* launches);

/* Number of this library's kernels launched by the engine since creation. */
int ske_launch_count(ske_engine e, int64_t* launches);

/* Self-test of the total-viewshed sweep's division: compares its
 * multiply-and-correct quotient with IEEE division for every float numerator
 * in the sweep's fast-path range and every distance d in [1, dmax] (dmax <=
 * 4095) on `device`.  No reference counterpart (the reference divides
 * directly, kernelSDEM.h:191).  Synchronous. */
int ske_selftest_division(int device, int dmax, int64_t* checked, int64_t* mismatches,
                          uint32_t* first_bad_bits);

/* FP32 pipe throughput of `device` in lane operations per second (one fused
 * multiply-add = one operation), scalar and packed two-wide: the roofline
 * denominator of the total-viewshed sweep.  No reference counterpart. */
int ske_measure_fp32_peak(int device, double* scalar_ops, double* packed_ops);

/* Binary64 fused multiply-add throughput of `device` in lane operations per
 * second: the roofline denominator of the Radon transform and cepstrum, which
 * compute in double precision like the reference.  No reference counterpart. */
int ske_measure_fp64_peak(int device, double* dfma_ops);

/* ---- Image input/output (host only; no GPU) ------------------------------
 * The reference's image operators read their input with helper::read_png
 * (src/helper.h:167-184: decode to 8-bit RGBA, then R + G + B per pixel) and
 * write results as PNG images coloured by showResults / showResultsRADN /
 * showResultsCEPS (src/main.h:124-141, src/kernelRADN.h:384-400,
 * src/kernelBLUR.h:396-410) with HSVtoRGB (src/color.cpp:80-115).
 * Every function returns SKE_OK or SKE_ERR_INVALID (unreadable or malformed
 * file, buffer too small, bad argument). */

/* Width and height of a PNG file; images of more than 2^31 pixels (the
 * decoder's limit) are refused. */
int ske_png_size(const char* path, int* width, int* height);
/* Decode a PNG (any colour type, bit depth, interlacing) to 8-bit RGBA, as the
 * reference's PNG library does; capacity in bytes (>= 4 * width * height). */
int ske_png_read_rgba(const char* path, uint8_t* rgba, size_t capacity);
/* The reference's image input: one float per pixel, R + G + B of the decoded
 * RGBA (replaces read_png + configureRADN/configureCEPS, src/kernelRADN.h:77-87);
 * capacity in floats (>= width * height). */
int ske_png_read_image(const char* path, float* image, size_t capacity);
/* Write 8-bit grey (channels 1) or RGB (channels 3) pixels as a PNG file
 * (replaces lodepng::encode(..., LCT_GREY / LCT_RGB) in the result writers). */
int ske_png_write(const char* path, const uint8_t* pixels, int width, int height, int channels);
/* HSVtoRGB (src/color.cpp:80-115) with the reference's float arithmetic. */
void ske_hsv_to_rgb(float h, float s, float v, uint8_t* rgb);
/* The reference's colouring of an operator's output grid into 3 * dimx * dimy
 * RGB bytes: Radon (and local Radon) grey with the automatic scale
 * 255 / (max - min) shifted by min, image identity grey / 540, cepstrum and DEM
 * identity as HSV (hue = output mod 360).  SKE_KERNEL_SDEM has no colouring in
 * the reference (it writes raw floats) and returns SKE_ERR_INVALID. */
int ske_render(int kernel, const float* output, int dimx, int dimy, uint8_t* rgb);
/* The grey image the result writers store beside it: (R + G + B) / 3 of the
 * input image given as ske_png_read_image returns it. */
int ske_render_input(const float* image, int count, uint8_t* grey);

/* ---- Learned total-viewshed surrogate (no reference counterpart) ----------
 * The convolutions of a U-Net that approximates the engine's total-viewshed
 * output on DEM tiles.  3x3, stride 1, zero padding 1, NHWC bfloat16 tensors
 * on the device, ordered on `stream`: y = relu?(conv(x, w) + bias).
 * w: cout x kpad bfloat16, kpad = 9*cin rounded up to a multiple of 32, entry
 * [co][(ky*3 + kx)*cin + ci], zero past 9*cin; bias: cout floats or null.
 * cin a multiple of 8, cout even.  In every function below the bfloat16
 * inputs and weights, and the outputs of ske_maxpool2_bf16 and
 * ske_surrogate_encode_bf16, start on 16-byte boundaries; the other outputs
 * and the float32 arrays on 4-byte ones (SKE_ERR_INVALID otherwise). */
int ske_conv3x3_bf16(const void* x, const void* w, const float* bias, void* y, int n, int h, int w_,
                     int cin, int cout, int relu, void* stream);
/* ske_conv3x3_bf16 of the channel concatenation [nearest-upsampled xlow, xskip]
 * without materialising it: xlow is n x h/2 x w/2 x c1, xskip n x h x w x c2
 * (h, w even; c1, c2 multiples of 8); w has cin = c1 + c2.  Same results as the
 * convolution of the concatenated tensor. */
int ske_conv3x3_upcat_bf16(const void* xlow, const void* xskip, const void* w, const float* bias, void* y,
                           int n, int h, int w_, int c1, int c2, int cout, int relu, void* stream);
/* Weight gradient of ske_conv3x3_bf16, added into dw (cout x kpad float32):
 * dw[co][k] += sum over pixels of dy[pixel][co] * (im2col x)[pixel][k],
 * kpad = 9*cin rounded up to a multiple of 32 (the padding columns are left as
 * they are).  cin and cout multiples of 8. */
int ske_conv3x3_wgrad_bf16(const void* x, const void* dy, float* dw, int n, int h, int w_, int cin,
                           int cout, void* stream);
/* The same 3x3 convolution (+ bias, ReLU when relu != 0) followed by a 1x1
 * convolution to one channel, fused: y[pixel] = head_b + sum over c in order of
 * bf16(act[pixel][c]) * head_w[c] in float32, y float32 (n x h x w), head_w
 * (cout floats) and head_b (one float) on the device.  The activations are not
 * written.  Cout a multiple of 16; SKE_ERR_UNSUPPORTED where the
 * warp-specialised kernel does not apply (or another kernel is selected).  No
 * reference counterpart. */
int ske_conv3x3_head_bf16(const void* x, const void* w, const float* bias, const float* head_w,
                          const float* head_b, float* y, int n, int h, int w_, int cin, int cout, int relu,
                          void* stream);

/* The surrogate's network input on the device: x (n x side x side x 8,
 * bfloat16) from float32 tiles (n x side x side), their per-tile mean and
 * height range (n floats each) and coarse areas (n x side/f x side/f, f =
 * coarse_factor): x[...,0] = (h - mean) / (range, or 1 for 0), x[...,1] =
 * log1p(range), x[...,2] = log1p(coarse area of the cell's coarse cell) /
 * coarse_scale, channels 3-7 zero.  side at most 46340.  No reference
 * counterpart. */
int ske_surrogate_encode_bf16(const float* tiles, const float* mean, const float* range, const float* coarse,
                              int coarse_factor, float coarse_scale, void* x, int n, int side, void* stream);

/* 2 x 2 max pooling of an NHWC bfloat16 tensor on the device (h, w even, c a
 * multiple of 8): y[n][i][j][c] = max of x[n][2i..2i+1][2j..2j+1][c], NaN
 * propagated.  No reference counterpart. */
int ske_maxpool2_bf16(const void* x, void* y, int n, int h, int w_, int c, void* stream);

/* Forward-convolution kernel choice for later calls: 0 (default) = the
 * warp-specialised persistent kernel wherever it applies (Cin a multiple of 8,
 * Cout a multiple of 16 up to 256, C1 a multiple of 16, two pipeline stages
 * within shared memory), else the halo-staged kernel where it applies (Cin,
 * Cout and C1 multiples of 16, Cout <= 128), else the im2col kernel; 1 = always
 * the im2col kernel; 2 = the halo-staged kernel where it applies, else im2col.
 * No reference counterpart. */
int ske_conv_select(int path);

/* Input channels the warp-specialised forward kernel stages per pipeline step
 * for later calls: 16, 32 or 64 (wider steps copy longer contiguous runs of
 * each pixel but fit fewer steps in shared memory), or 0 (default) = the most
 * of 64, 32, 16 that divides Cin and C1 with two steps fitting.  A tuning
 * knob; no reference counterpart. */
int ske_conv_stage_channels(int channels);

/* Weight-gradient kernel for later calls of ske_conv3x3_wgrad_bf16: 1 (default)
 * = ldmatrix + mma.sync; 0 = tcgen05 (dY and X staged once per tile as
 * 8-channel planes and read in place as MN-major operands, the 9 taps'
 * accumulators in tensor memory, float32 atomics into dw), measured slower on
 * the surrogate's layers except the widest.  Same sums in other orders.  No
 * reference counterpart. */
int ske_conv_wgrad_select(int path);

/* Synchronises `stream`, then sets *failed to 1 if a forward convolution or
 * the tcgen05 weight gradient since the previous call gave up waiting for its
 * tensor-core operations (a forward convolution's output is then not written;
 * the weight gradient adds none of its CTA's sums to dw), else 0, and clears
 * the flag. */
int ske_conv_status(int* failed, void* stream);

/* The reference's grid input (readBilData, parse_hdr and check_dem,
 * src/kernelSDEM.h:31-142; read_png, src/helper.h:167-184): an ESRI .bil int16
 * DEM divided by 10 in binary64 (cell units of a 10 m grid), a raw float32 grid,
 * or a .png image as R + G + B per pixel.  dimx/dimy give the file's grid; 0
 * takes the .hdr's NCOLS/NROWS (else a square from the file size) or the
 * image's size.  crop_x/crop_y drop columns/rows from the right/bottom as
 * readBilData's crop does: the top-left (dimx - crop_x) x (dimy - crop_y)
 * window, rows read at the file's pitch.  Writes the window's size to
 * *out_dimx and *out_dimy and, when `grid` is not NULL, its cells (row-major;
 * `capacity` in floats).  SKE_OK, or SKE_ERR_INVALID for an unreadable, short
 * or malformed file, an empty window or a small buffer.  Host only. */
int ske_read_grid(const char* path, int dimx, int dimy, int crop_x, int crop_y, float* grid, size_t capacity,
                  int* out_dimx, int* out_dimy);

/* Reference command-line entry point (src/main.cu:200-202): runs one operator on
 * an input file and writes the result.
 *   argv: run <kernel> <input> <dimx> <dimy> <output> [max_sector] [povh] [accum]
 *         [crop_x] [crop_y]
 *   kernel: sdem | identitydem | radon | identityimg | cepstrum | localradon, or
 *           0..5 (the reference's KERNELS enum, src/global.h:77; 5 = radon with
 *           its local-transform switch set);
 *   input:  raw float32 grid, ESRI .bil int16 DEM (with its .hdr; dimx/dimy 0
 *           take NCOLS/NROWS) or .png image, read and cropped as ske_read_grid;
 *   output: raw float32 grid (.flt) or, for a name ending in .png, the
 *           reference's coloured result image.
 * Returns 0 or a SKE_* status; messages go to stderr. */
int run(int argc, char** argv);

#ifdef __cplusplus
}
#endif

#endif /* SKEWENGINE_H */
