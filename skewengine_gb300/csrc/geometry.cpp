// Host-side sector geometry and FFT twiddle tables.
//
// The per-sector tables are computed on the host in double precision with the
// platform libm, exactly as the reference computes them on its host
// (skewEngine.cuh:504-539 computeParams, :573-596 skewShape), and uploaded once
// per engine.  Keeping them on the host keeps tan/cos bit-identical to the
// reference's own CPU run on the same machine.
//
// Compiled with -ffp-contract=off so no multiply-add is fused.
#include <cmath>
#include <cstdio>
#include <complex>

#include "ske_internal.h"

namespace ske {

void sector_geometry(int dimx, int dimy, int angle, SectorDesc& d, std::vector<int32_t>& first,
                     std::vector<int32_t>& last, std::vector<int32_t>& target, std::vector<float>& weight) {
    const double deg = M_PI / 180.0;                                   // skewEngine.cuh:258
    const float frontier = (float)(atan2((double)dimy, (double)dimx) * 180 / M_PI);  // :465
    const int fa = (int)frontier;
    const bool tr = angle > fa && angle < 180 - fa;
    const bool mi = angle > 90;
    d = SectorDesc();
    d.angle = angle;
    d.type = tr ? (mi ? 2 : 1) : (mi ? 3 : 0);
    d.new_angle = d.type == 0 ? angle : d.type == 1 ? 90 - angle : d.type == 2 ? angle - 90 : 180 - angle;
    d.scale = 1 / cos(deg * d.new_angle);
    d.skewness = tan(d.new_angle * deg);
    d.r2 = (float)(d.scale * d.scale);
    d.dim_i = tr ? dimy : dimx;
    d.dim_o = tr ? dimx : dimy;
    d.diml = dimx > dimy ? dimx : dimy;
    d.offset = (int)(d.skewness * (d.dim_i - 1));
    d.H = d.new_angle ? d.dim_o + d.offset + 1 : d.dim_o;

    target.assign(d.dim_i, 0);
    weight.assign(d.dim_i, 0.0f);
    for (int j = 0; j < d.dim_i; j++) {
        const double drift = d.skewness * j;
        target[j] = (int32_t)drift;
        weight[j] = (float)(drift - target[j]);
    }

    // Valid column range [first, last) of every skewed row.  The reference keeps
    // these in 2*dim_l+1 entries and only reads rows < H; rows H and H+1 can be
    // touched by the edge updates below, so work on H+2 rows and keep H.
    const int rows = d.H + 2;
    std::vector<int32_t> f(rows, 0), l(rows, 0);
    for (int r = 0; r < d.dim_o && r < rows; r++) f[r] = 0;
    for (int r = d.offset; r < d.H; r++) l[r] = d.diml;
    for (int r = 0; r < d.offset && r < rows; r++) l[r] = 0;
    for (int r = d.dim_o; r < d.H; r++) f[r] = d.diml;
    for (int j = 0; j < d.dim_i; j++) {
        const int top = target[j];
        if (j > l[top]) l[top] = j + 1;
        if (j > l[top + 1]) l[top + 1] = j + 1;
        const int bot = target[j] + d.dim_o - 1;
        if (bot < rows && j < f[bot]) f[bot] = j;
        if (bot + 1 < rows && j < f[bot + 1]) f[bot + 1] = j;
    }
    first.assign(f.begin(), f.begin() + d.H);
    last.assign(l.begin(), l.begin() + d.H);
}

// The skew, the operators and the deskew index the skewed grid of a sector as
// rows r < H of stride dim_i whose valid cells are [first[r], last[r]) (a row
// with first >= last is empty).  They rely on: 0 <= first and last <= dim_l;
// the farthest cell a row reaches, (H-1)*dim_i + last, inside the skew buffer
// of 2*dimx*dimy + dim_l floats (skewEngine.cuh:425-426); and every column's
// source rows target[j] .. target[j] + dim_o inside rows 0 .. H.  The tables
// follow the reference's formulas, which keep all three; checking them here
// turns any table that did not into an error before a kernel runs.
std::string check_sector(const SectorDesc& d, const int32_t* first, const int32_t* last, const int32_t* target,
                         int dimx, int dimy) {
    char msg[160];
    if (d.H < 1 || d.dim_i < 1 || d.dim_o < 1 || d.diml != (dimx > dimy ? dimx : dimy)) {
        snprintf(msg, sizeof msg, "angle %d: skewed grid %d rows x %d (outer %d)", d.angle, d.H, d.dim_i, d.dim_o);
        return msg;
    }
    const int64_t len = skew_buffer_len(dimx, dimy);
    for (int r = 0; r < d.H; r++) {
        if (first[r] < 0 || last[r] > d.diml || (int64_t)r * d.dim_i + last[r] > len) {
            snprintf(msg, sizeof msg, "angle %d: row %d spans [%d, %d) of %d x %d, buffer %lld", d.angle, r,
                     first[r], last[r], d.H, d.dim_i, (long long)len);
            return msg;
        }
    }
    for (int j = 0; j < d.dim_i; j++) {
        if (target[j] < 0 || target[j] + d.dim_o > d.H) {
            snprintf(msg, sizeof msg, "angle %d: column %d shifts %d rows in a skewed grid of %d", d.angle, j,
                     target[j], d.H);
            return msg;
        }
    }
    return std::string();
}

std::string build_geometry(int dimx, int dimy, Geometry& g) {
    g.dimx = dimx;
    g.dimy = dimy;
    g.desc.resize(kMaxSectors);
    g.target.clear();
    g.weight.clear();
    g.first.clear();
    g.last.clear();
    g.max_cells = 0;
    g.max_H = 0;
    std::vector<int32_t> f, l, t;
    std::vector<float> w;
    for (int a = 0; a < kMaxSectors; a++) {
        SectorDesc& d = g.desc[a];
        sector_geometry(dimx, dimy, a, d, f, l, t, w);
        std::string why = check_sector(d, f.data(), l.data(), t.data(), dimx, dimy);
        if (!why.empty()) return why;
        d.col_off = (int64_t)g.target.size();
        d.row_off = (int64_t)g.first.size();
        g.target.insert(g.target.end(), t.begin(), t.end());
        g.weight.insert(g.weight.end(), w.begin(), w.end());
        g.first.insert(g.first.end(), f.begin(), f.end());
        g.last.insert(g.last.end(), l.begin(), l.end());
        const int64_t cells = (int64_t)d.H * d.dim_i;
        if (cells > g.max_cells) g.max_cells = cells;
        if (d.H > g.max_H) g.max_H = d.H;
    }
    return std::string();
}

void fft_twiddles(unsigned n, std::vector<double>& re_im) {
    re_im.assign(n > 1 ? 2 * (size_t)(n - 1) : 0, 0.0);
    if (n <= 1) return;
    typedef std::complex<double> cplx;
    const double theta = (double)(3.14159265358979323846264338328L / n);  // helper.h:63
    cplx step(cos(theta), -sin(theta));
    for (unsigned h = n / 2; h >= 1; h /= 2) {
        step = step * step;
        cplx w = 1.0;
        const size_t base = n - 2 * (size_t)h;
        for (unsigned l = 0; l < h; l++) {
            re_im[2 * (base + l)] = w.real();
            re_im[2 * (base + l) + 1] = w.imag();
            w *= step;
        }
    }
}

void local_radon_tables(const Geometry& g, std::vector<double>& gauss, std::vector<double>& taper) {
    const int w2 = kLocalRadonWindow / 2;
    gauss.assign((size_t)kLocalRadonWindow * g.desc.size(), 0.0);
    for (size_t a = 0; a < g.desc.size(); a++) {
        double sigma = kLocalRadonWindow / 5.0;  // kernelRADN.h:123-126
        sigma = sigma / g.desc[a].scale;
        for (int kk = 0; kk < kLocalRadonWindow; kk++)  // kernelRADN.h:138
            gauss[a * kLocalRadonWindow + kk] = exp(-(kk - w2) * (kk - w2) / (2 * sigma * sigma));
    }
    const double dws = kLocalRadonWindow, cutoff = 0.4;  // kernelRADN.h:157-161
    taper.assign(kLocalRadonKeep, 0.0);
    for (int k = 0; k < kLocalRadonKeep; k++) taper[k] = sin((k / (cutoff * dws - 1)) * M_PI_2);
}

}  // namespace ske
