// Test oracle (CPU restatement of the reference skewEngine CPU path).
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg may load the library built from this file, and only as a
// checker or as the timed CPU baseline; the product never links or calls it.
//
// Parity: pinned against the reference's own CPU code (oracle/ref_harness.cu
// compiled from the reference sources) through the golden fixtures in
// tests/golden, which tests/test_oracle_golden.py checks bit for bit.
#ifndef SKEWPORT_H
#define SKEWPORT_H

#ifdef __cplusplus
extern "C" {
#endif

// Operator ids follow the reference KERNELS enum (src/global.h:77); 5 is the
// reference's Radon operator with LRT set (kernelRADN.h:212-220), the local Radon
// transform.
enum { PORT_SDEM = 0, PORT_IDENTITYDEM = 1, PORT_RADON = 2, PORT_IDENTITYIMG = 3, PORT_CEPSTRUM = 4,
       PORT_LOCAL_RADON = 5 };

// Per-sector geometry, restating skewEngine::computeParams (skewEngine.cuh:504-539)
// and skewEngine::skewShape (skewEngine.cuh:573-596).
//   iinfo[0..6] = sectorType, newAngle, dim_i, dim_o, offset, skewHeight, dim_l
//   dinfo[0..1] = scale, skewness
//   first/last: 2*dim_l+1 entries (rows >= skewHeight are left as zero)
//   target/weight: dim_l entries (columns >= dim_i are left as zero)
int port_geometry(int dimx, int dimy, int angle, int* iinfo, double* dinfo,
                  unsigned short* first, unsigned short* last, int* target, float* weight);

// Whole run over the given angles (in the given order when nthreads == 1),
// restating the reference driver loop (src/main.cu:86-168).  output: dimx*dimy.
int port_run_angles(int op, const float* input, float* output, int dimx, int dimy,
                    const int* angles, int nangles, float povh, int nthreads);

// The result port_run_angles gives with one thread (the reference's
// single-thread accumulation order, in list order), computed on nthreads: each
// sector's deskewed values are formed in parallel, then folded into the
// per-type accumulators in list order.  Bit-identical to nthreads == 1.
int port_run_angles_ordered(int op, const float* input, float* output, int dimx, int dimy,
                            const int* angles, int nangles, float povh, int nthreads);

// Whole run over angles 0..nsect-1.
int port_run(int op, const float* input, float* output, int dimx, int dimy, int nsect,
             float povh, int nthreads);

// One sector: skewed input, operator output (2*N + dim_l floats each) and this
// sector's contribution folded back to the input orientation (N floats).
int port_sector(int op, const float* input, int dimx, int dimy, int angle, float povh,
                float* skew_in, float* skew_out, float* acc);

// kernelSDEM visibility counts of one sector: for every skewed cell of every row
// in [first,last) the integer-valued `cv` before the scale factor
// (kernelSDEM.h:182-218); other cells 0.  counts: 2*N + dim_l floats.
int port_sdem_counts(const float* input, int dimx, int dimy, int angle, float povh,
                     float* counts);

// Per-type accumulators (4*N floats, type-major, each in its orientation's
// layout) after deskewing the given angles in order on one thread, and the
// bit mask of types that received a sector: the state one reference engine
// thread holds before its reduce (skewEngine.cuh:270-273, :759-770).
int port_accumulate(int op, const float* input, int dimx, int dimy, const int* angles, int nangles,
                    float povh, float* acc, int* used_mask);

// The same sector loop carried out entirely in binary64 (skew weights, skewed
// grids, operator, deskew and fold), for the Radon transform and the cepstrum:
// the FP64 reference against which the float pipeline's error is stated.
// output: dimx*dimy doubles.
int port_run_f64(int op, const float* input, double* output, int dimx, int dimy, int nsect, float povh);

// Sum over sectors 0..nsect-1 and rows of L*(L-1), L = last-first: the number of
// line-of-sight steps kernelSDEM performs (both directions).
double port_los_steps(int dimx, int dimy, int nsect);

#ifdef __cplusplus
}
#endif

#endif
