// Internal declarations shared by the host runtime and the CUDA kernels of the
// skew engine.  Not part of the public ABI (include/skewengine.h).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace ske {

constexpr int kMaxSectors = 180;  // integer angles 0..179 (src/global.cpp:69)
constexpr int kBlurWindow = 64;   // effective cepstrum window (src/kernelRADN.h:19)

// Geometry of one sector as the kernels see it (computeParams + skewShape,
// skewEngine.cuh:504-596).  Plain data, uploaded once per engine.
struct SectorDesc {
    int32_t angle;      // a
    int32_t type;       // sectorType 0..3
    int32_t new_angle;  // newAngle
    int32_t dim_i;      // skewWidth (row stride of the skewed grid)
    int32_t dim_o;
    int32_t offset;
    int32_t H;          // skewHeight
    int32_t diml;       // max(dimx, dimy)
    float r2;           // (float)(scale*scale), kernelSDEM.h:171
    int32_t in_width;   // 1: every row's last <= dim_i (no row reaches into the next row's span)
    double scale;       // 1/cos(newAngle)
    double skewness;    // tan(newAngle)
    int64_t col_off;    // first entry of this sector in target/weight tables
    int64_t row_off;    // first entry of this sector in first/last tables
};

// Host tables for a grid: one SectorDesc per angle 0..179 and the concatenated
// per-angle target/weight (dim_i entries) and first/last (H entries).
struct Geometry {
    int dimx = 0, dimy = 0;
    std::vector<SectorDesc> desc;
    std::vector<int32_t> target, first, last;
    std::vector<float> weight;
    int64_t max_cells = 0;  // max over angles of H*dim_i
    int max_H = 0;
};

// Geometry of one angle.  first/last get H entries, target/weight dim_i.
void sector_geometry(int dimx, int dimy, int angle, SectorDesc& d, std::vector<int32_t>& first,
                     std::vector<int32_t>& last, std::vector<int32_t>& target, std::vector<float>& weight);

// Geometry of all 180 angles.
// The bounds every kernel relies on (checked on the host once per table build):
// empty string when they hold, else which one fails.
std::string check_sector(const SectorDesc& d, const int32_t* first, const int32_t* last, const int32_t* target,
                         int dimx, int dimy);
// All 180 sectors' tables; returns check_sector's complaint about the first
// sector that fails it (empty string: every table is within bounds).
std::string build_geometry(int dimx, int dimy, Geometry& g);

// Twiddles of the reference radix-2 DIF FFT (helper.h:59-82) for size n (a power
// of two): the stage with half-span h uses entries [n-2h, n-h), entry l being the
// twiddle after l sequential complex multiplications, exactly as the reference
// advances it.  n-1 entries in total (none for n == 1).
void fft_twiddles(unsigned n, std::vector<double>& re_im);

// Constants of the local Radon transform (pointRadon, kernelRADN.h:114-182),
// computed on the host with the reference's expressions: gauss[64*a + m] =
// exp(-(m-32)^2 / (2 sigma^2)), sigma = (64/5)/scale of angle a, for a < 180;
// taper[k] = sin(k/(25.6-1) * pi/2) for k <= 25 (the bins the filter keeps).
constexpr int kLocalRadonWindow = 64;  // winSize (kernelRADN.h:19)
constexpr int kLocalRadonKeep = 26;    // bins k <= 0.4 * 64
void local_radon_tables(const Geometry& g, std::vector<double>& gauss, std::vector<double>& taper);

// Size of the skewed buffers of a grid: 2*N + dim_l floats
// (skewEngine.cuh:425-426, the CPU path's buffer size).
inline int64_t skew_buffer_len(int dimx, int dimy) {
    return 2 * (int64_t)dimx * dimy + (dimx > dimy ? dimx : dimy);
}

}  // namespace ske
