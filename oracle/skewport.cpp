// Test oracle: CPU restatement of the reference skewEngine CPU path.
//
// TEST INFRASTRUCTURE ONLY (see skewport.h).  Every function below restates one
// piece of the reference and cites it.  The arithmetic is kept in the same
// precision and order as the reference so results are bit-identical to it when
// both are built without floating-point contraction (oracle/Makefile).
//
// Parity pinned against the reference's own CPU code through tests/golden.

#include "skewport.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#include <omp.h>

namespace {

typedef std::complex<double> cplx;

const double kDegToRad = M_PI / 180.0;  // skewEngine.cuh:258

struct Sector {
    int a = 0, type = 0, newAngle = 0, dim_i = 0, dim_o = 0, offset = 0, H = 0, diml = 0;
    double scale = 0, skewness = 0;
    std::vector<int> target;
    std::vector<float> weight;
    std::vector<unsigned short> first, last;
};

// skewEngine ctor (skewEngine.cuh:465): frontier angle between plain and transposed
// sectors, in degrees, stored as float.
float frontier_angle(int dimx, int dimy) { return (float)(atan2((double)dimy, (double)dimx) * 180 / M_PI); }

// computeParams (skewEngine.cuh:504-539) + skewShape (skewEngine.cuh:573-596).
void make_sector(int dimx, int dimy, int angle, Sector& s) {
    const float fAngle = frontier_angle(dimx, dimy);
    s.diml = std::max(dimx, dimy);
    s.a = angle;
    const bool transposed = angle > (int)fAngle && angle < 180 - (int)fAngle;
    const bool mirrored = angle > 90;
    if (!transposed && !mirrored) { s.type = 0; s.newAngle = angle; }
    if (transposed && !mirrored) { s.type = 1; s.newAngle = 90 - angle; }
    if (transposed && mirrored) { s.type = 2; s.newAngle = angle - 90; }
    if (!transposed && mirrored) { s.type = 3; s.newAngle = 180 - angle; }
    s.scale = 1 / cos(kDegToRad * s.newAngle);
    s.skewness = tan(s.newAngle * kDegToRad);
    s.dim_i = transposed ? dimy : dimx;
    s.dim_o = transposed ? dimx : dimy;
    s.offset = (int)(s.skewness * (s.dim_i - 1));
    s.H = s.newAngle ? s.dim_o + s.offset + 1 : s.dim_o;
    s.target.assign(s.diml, 0);
    s.weight.assign(s.diml, 0.0f);
    for (int j = 0; j < s.dim_i; j++) {
        const double drift = s.skewness * j;
        s.target[j] = (int)drift;
        s.weight[j] = (float)(drift - s.target[j]);
    }
    // Row limits [first, last) of the valid part of every skewed row.
    s.first.assign(2 * s.diml + 1, 0);
    s.last.assign(2 * s.diml + 1, 0);
    for (int r = 0; r < s.dim_o; r++) s.first[r] = 0;
    for (int r = s.offset; r < s.H; r++) s.last[r] = (unsigned short)s.diml;
    for (int r = 0; r < s.offset; r++) s.last[r] = 0;
    for (int r = s.dim_o; r < s.H; r++) s.first[r] = (unsigned short)s.diml;
    for (int j = 0; j < s.dim_i; j++) {
        const int top = s.target[j];
        for (int r = top; r <= top + 1; r++)
            if (j > s.last[r]) s.last[r] = (unsigned short)(j + 1);
        const int bottom = s.target[j] + s.dim_o - 1;
        for (int r = bottom; r <= bottom + 1; r++)
            if (j < s.first[r]) s.first[r] = (unsigned short)j;
    }
}

// prepare (skewEngine.cuh:925-951): the four orientations of the input.
void orientations(const float* in, int dimx, int dimy, std::vector<float> o[4]) {
    const size_t n = (size_t)dimx * dimy;
    for (int t = 0; t < 4; t++) o[t].resize(n);
    for (int i = 0; i < dimy; i++) {
        const int ci = dimy - 1 - i;
        for (int j = 0; j < dimx; j++) {
            const int cj = dimx - 1 - j;
            const float v = in[(size_t)dimx * i + j];
            o[0][(size_t)dimx * i + j] = v;
            o[1][(size_t)dimy * cj + ci] = v;
            o[2][(size_t)dimy * j + ci] = v;
            o[3][(size_t)dimx * i + cj] = v;
        }
    }
}

// skew (skewEngine.cuh:612-621): scatter every source cell onto two skewed rows.
void skew_rows(const Sector& s, const float* src, float* S) {
    for (int i = 0; i < s.dim_o; i++)
        for (int j = 0; j < s.dim_i; j++) {
            const float v = src[(size_t)s.dim_i * i + j];
            S[(size_t)(i + s.target[j]) * s.dim_i + j] += (1.0f - s.weight[j]) * v;
            S[(size_t)(i + s.target[j] + 1) * s.dim_i + j] += s.weight[j] * v;
        }
}

// helper::fft (helper.h:59-106): in-place radix-2 decimation in frequency, the
// twiddle advanced by repeated complex multiplication, then bit reversal and an
// optional 1/sqrt(n) scaling.
void fft_dif(cplx* x, unsigned n, bool normalize) {
    const double theta = (double)(3.14159265358979323846264338328L / n);
    cplx step(cos(theta), -sin(theta));
    for (unsigned half = n; half > 1;) {
        const unsigned span = half;
        half >>= 1;
        step = step * step;
        cplx w = 1.0L;
        for (unsigned l = 0; l < half; l++) {
            for (unsigned a = l; a < n; a += span) {
                const unsigned b = a + half;
                const cplx d = x[a] - x[b];
                x[a] += x[b];
                x[b] = d * w;
            }
            w *= step;
        }
    }
    const unsigned bits = (unsigned)log2(n);
    for (unsigned a = 0; a < n && bits > 0; a++) {
        unsigned b = a, rev = 0;
        for (unsigned k = 0; k < bits; k++) { rev = (rev << 1) | (b & 1u); b >>= 1; }
        if (rev > a) std::swap(x[a], x[rev]);
    }
    if (!normalize) return;
    const cplx f = 1.0 / sqrt(n);
    for (unsigned i = 0; i < n; i++) x[i] *= f;
}

// helper::ifft (helper.h:108-114).
void ifft(cplx* x, unsigned n) {
    for (unsigned i = 0; i < n; i++) x[i] = std::conj(x[i]);
    fft_dif(x, n, false);
    for (unsigned i = 0; i < n; i++) x[i] = std::conj(x[i]);
    for (unsigned i = 0; i < n; i++) x[i] /= cplx((double)n);
}

// kernelV3 (kernelSDEM.h:168-222): total-viewshed line-of-sight sweep.  When
// `counts` is given, the integer-valued cv is stored instead of cv*r.
void op_sdem(const Sector& s, const float* S, float* O, float povh, bool counts) {
    const float r2 = (float)pow(s.scale, 2);
    for (int row = 0; row < s.H; row++) {
        const int lo = s.first[row], hi = s.last[row];
        const float* v = S + (size_t)s.dim_i * row;
        float* out = O + (size_t)s.dim_i * row;
        for (int j = lo; j < hi; j++) {
            float cv = 0;
            const float h = v[j] + povh;
            for (int dir = 1; dir >= -1; dir -= 2) {
                float horizon = -2000;
                bool seen = true;
                float opened = 0;
                for (int k = j + dir; k >= lo && k < hi; k += dir) {
                    const float d = (float)(dir > 0 ? k - j : j - k);
                    const float slope = (v[k] - h) / d;
                    const bool above = slope > horizon;
                    if (above && !seen) opened = d;
                    if (!above && seen) cv += (d * d - opened * opened);
                    seen = above;
                    horizon = std::max(slope, horizon);
                }
            }
            out[j] = counts ? cv : cv * r2;
        }
    }
}

// radon, global mode (kernelRADN.h:221-258): ray sums, ramp filter in the
// frequency domain, filtered back-projection along the row.
void op_radon(const Sector& s, const float* S, float* O) {
    const int H = s.H;
    const int H2 = (int)pow(2, ceil(log2(H)));
    std::vector<cplx> p(H2, cplx(0, 0));
    for (int i = 0; i < H; i++) {
        const float* v = S + (size_t)s.dim_i * i;
        for (int j = s.first[i]; j < s.last[i]; j++) p[i] = cplx(p[i].real() + v[j], 0);
    }
    fft_dif(p.data(), (unsigned)H2, false);
    for (int i = 0; i < H2; i++) p[i] = i > H / 2 ? cplx(0) : ((double)i / H) * p[i];
    ifft(p.data(), (unsigned)H2);
    for (int i = 0; i < H; i++) {
        float* out = O + (size_t)s.dim_i * i;
        for (int j = s.first[i]; j < s.last[i]; j++) out[j] += p[i].real();
    }
}

// getBlurParameter2 (kernelBLUR.h:88-110): skip the descending head from index 5,
// then the largest sample (the first ascending sample itself is not visited).
double blur_peak(const double* v, int n) {
    int i = 5;
    while (i < n && !(v[i] > v[i - 1])) i++;
    if (i == n) return 0;
    double best = v[i - 1];
    int at = i;
    for (i = i + 1; i < n; i++)
        if (v[i] > best) { best = v[i]; at = i; }
    return at == 0 ? 0 : best;
}

// cepstrum + lineCepstrum + select_subarray (kernelBLUR.h:267-302, :153-228,
// :69-85) with the effective window of 64 (kernelRADN.h:19 wins the shared
// KERNELCOMMONS guard).
const int kWin = 64;
void op_cepstrum(const Sector& s, const float* S, float* O) {
    cplx w1[kWin], w2[kWin / 2];
    double samples[kWin / 4];
    for (int row = 0; row < s.H; row++) {
        const int lo = s.first[row], hi = s.last[row];
        const float* v = S + (size_t)s.dim_i * row;
        for (int j = lo; j < hi; j++) {
            for (int m = 0; m < kWin; m++) {
                const int idx = j - kWin / 2 + m;
                w1[m] = (idx < lo || idx >= hi) ? cplx(0, 0) : cplx(v[idx], 0);
            }
            fft_dif(w1, kWin, true);
            for (int k = 0; k < kWin / 2; k++) {
                const double ps = pow(w1[k].real(), 2) + pow(w1[k].imag(), 2);
                w2[k] = cplx(log(ps), 0);
            }
            fft_dif(w2, kWin / 2, true);
            for (int k = 0; k < kWin / 4; k++) samples[k] = -std::min(0.0, w2[k].real());
            O[(size_t)s.dim_i * row + j] = (float)(blur_peak(samples, kWin / 4) * 10000);
        }
    }
}

// identity (kernelUNIT.h:16-23).
// pointRadon (kernelRADN.h:114-182), the local Radon transform of one skewed
// cell (i, j), called for every valid cell when LRT is set (kernelRADN.h:215-220):
// 64 rows k = i-32 .. i+31, each summed in binary64 over the 65 columns
// j-32 .. j+32 that lie in the row's valid range (rows outside the grid give 0),
// weighted by exp(-(k-i)^2 / (2 sigma^2)), sigma = (64/5)/scale; a normalised
// FFT; the real parts tapered by sin(k/(25.6-1) * pi/2) for k <= 25.6 and zeroed
// above; a second normalised FFT; and getParameter (kernelRADN.h:89-102): from
// index 5 the first |v_i|^2 > |v_{i-1}|^2 gives |v_{i-1}|^2, none gives 0.
const int kLrWin = 64;  // winSize (kernelRADN.h:19)
float local_radon_cell(const Sector& s, const float* S, int i, int j) {
    const int w2 = kLrWin / 2;
    const double dws = kLrWin;
    double sigma = kLrWin / 5.0;
    sigma = sigma / s.scale;
    cplx in1[kLrWin];
    for (int k = i - w2; k < i + w2; k++) {
        double accum = 0;
        if (k >= 0 && k < s.H) {
            const int fi = s.first[k], la = s.last[k];
            for (int l = j - w2; l <= j + w2; l++)
                accum += (l < fi || l >= la) ? 0 : S[(size_t)k * s.dim_i + l];
        }
        const int kk = k - (i - w2);
        const double gauss = exp(-(kk - w2) * (kk - w2) / (2 * sigma * sigma));
        in1[kk] = {accum * gauss, 0};
    }
    fft_dif(in1, kLrWin, true);
    const double cutoff = 0.4;
    cplx in2[kLrWin];
    for (int k = 0; k < kLrWin; k++)
        in2[k] = k > cutoff * dws ? 0 : sin((k / (cutoff * dws - 1)) * M_PI_2) * in1[k].real();
    fft_dif(in2, kLrWin, true);
    double v = 0;
    int m;
    for (m = 5; m < w2; m++)
        if (std::norm(in2[m]) > std::norm(in2[m - 1])) break;
    if (m < w2) v = std::norm(in2[m - 1]);
    return (float)v;
}

void op_local_radon(const Sector& s, const float* S, float* O) {
    for (int i = 0; i < s.H; i++)
        for (int j = s.first[i]; j < s.last[i]; j++) O[(size_t)s.dim_i * i + j] = local_radon_cell(s, S, i, j);
}

void op_identity(const Sector& s, const float* S, float* O) {
    for (int row = 0; row < s.H; row++)
        for (int j = s.first[row]; j < s.last[row]; j++)
            O[(size_t)s.dim_i * row + j] = S[(size_t)s.dim_i * row + j];
}

void run_operator(int op, const Sector& s, const float* S, float* O, float povh) {
    switch (op) {
        case PORT_SDEM: op_sdem(s, S, O, povh, false); break;
        case PORT_RADON: op_radon(s, S, O); break;
        case PORT_CEPSTRUM: op_cepstrum(s, S, O); break;
        case PORT_LOCAL_RADON: op_local_radon(s, S, O); break;
        default: op_identity(s, S, O); break;
    }
}

// deskew (skewEngine.cuh:772-793): gather the two skewed cells of every source
// cell back.  Add mode accumulates; max mode keeps the maximum and re-encodes the
// low three decimal digits with the current angle.
void deskew_rows(const Sector& s, const float* O, float* acc, bool max_mode) {
    for (int i = 0; i < s.dim_o; i++)
        for (int j = 0; j < s.dim_i; j++) {
            const float lo = O[(size_t)(i + s.target[j]) * s.dim_i + j];
            const float hi = O[(size_t)(i + s.target[j] + 1) * s.dim_i + j];
            float& cell = acc[(size_t)i * s.dim_i + j];
            if (max_mode) {
                cell = std::max(cell, std::max(lo, hi));
                cell = s.a + 1000 * (int)(cell / 1000);
            } else {
                cell += (1.0f - s.weight[j]) * lo + s.weight[j] * hi;
            }
        }
}

// reduce (skewEngine.cuh:862-914): fold the four per-type accumulators back into
// the input orientation, in type order 0..3, skipping types never used.
void reduce_types(float* out, int dimx, int dimy, const std::vector<float> acc[4], bool max_mode) {
    for (int i = 0; i < dimy; i++) {
        const int ci = dimy - 1 - i;
        for (int j = 0; j < dimx; j++) {
            const int cj = dimx - 1 - j;
            const size_t idx[4] = {(size_t)i * dimx + j, (size_t)cj * dimy + ci,
                                   (size_t)j * dimy + ci, (size_t)i * dimx + cj};
            float& o = out[(size_t)i * dimx + j];
            for (int t = 0; t < 4; t++) {
                if (acc[t].empty()) continue;
                const float v = acc[t][idx[t]];
                if (max_mode) o = o > v ? o : v;
                else o += v;
            }
        }
    }
}

struct Worker {
    std::vector<float> S, O;
    std::vector<float> acc[4];
};

// ---- binary64 restatement (error reference for Radon and cepstrum) ----------

void op_radon_f64(const Sector& s, const double* S, double* O) {
    const int H = s.H;
    const int H2 = (int)pow(2, ceil(log2(H)));
    std::vector<cplx> p(H2, cplx(0, 0));
    for (int i = 0; i < H; i++)
        for (int j = s.first[i]; j < s.last[i]; j++) p[i] = cplx(p[i].real() + S[(size_t)s.dim_i * i + j], 0);
    fft_dif(p.data(), (unsigned)H2, false);
    for (int i = 0; i < H2; i++) p[i] = i > H / 2 ? cplx(0) : ((double)i / H) * p[i];
    ifft(p.data(), (unsigned)H2);
    for (int i = 0; i < H; i++)
        for (int j = s.first[i]; j < s.last[i]; j++) O[(size_t)s.dim_i * i + j] += p[i].real();
}

void op_cepstrum_f64(const Sector& s, const double* S, double* O) {
    cplx w1[kWin], w2[kWin / 2];
    double samples[kWin / 4];
    for (int row = 0; row < s.H; row++) {
        const int lo = s.first[row], hi = s.last[row];
        const double* v = S + (size_t)s.dim_i * row;
        for (int j = lo; j < hi; j++) {
            for (int m = 0; m < kWin; m++) {
                const int idx = j - kWin / 2 + m;
                w1[m] = (idx < lo || idx >= hi) ? cplx(0, 0) : cplx(v[idx], 0);
            }
            fft_dif(w1, kWin, true);
            for (int k = 0; k < kWin / 2; k++)
                w2[k] = cplx(log(pow(w1[k].real(), 2) + pow(w1[k].imag(), 2)), 0);
            fft_dif(w2, kWin / 2, true);
            for (int k = 0; k < kWin / 4; k++) samples[k] = -std::min(0.0, w2[k].real());
            O[(size_t)s.dim_i * row + j] = blur_peak(samples, kWin / 4) * 10000;
        }
    }
}

void run_sector(int op, int dimx, int dimy, const std::vector<float> src[4], int angle, float povh,
                Worker& w) {
    Sector s;
    make_sector(dimx, dimy, angle, s);
    std::fill(w.S.begin(), w.S.end(), 0.0f);
    std::fill(w.O.begin(), w.O.end(), 0.0f);
    skew_rows(s, src[s.type].data(), w.S.data());
    run_operator(op, s, w.S.data(), w.O.data(), povh);
    if (w.acc[s.type].empty()) w.acc[s.type].assign((size_t)dimx * dimy, 0.0f);
    deskew_rows(s, w.O.data(), w.acc[s.type].data(), op == PORT_CEPSTRUM);
}

}  // namespace

extern "C" {

int port_geometry(int dimx, int dimy, int angle, int* iinfo, double* dinfo, unsigned short* first,
                  unsigned short* last, int* target, float* weight) {
    if (dimx <= 0 || dimy <= 0 || angle < 0 || angle >= 180) return 1;
    Sector s;
    make_sector(dimx, dimy, angle, s);
    const int ints[7] = {s.type, s.newAngle, s.dim_i, s.dim_o, s.offset, s.H, s.diml};
    memcpy(iinfo, ints, sizeof(ints));
    dinfo[0] = s.scale;
    dinfo[1] = s.skewness;
    if (first) {
        memset(first, 0, sizeof(unsigned short) * (2 * s.diml + 1));
        std::copy(s.first.begin(), s.first.begin() + s.H, first);
    }
    if (last) {
        memset(last, 0, sizeof(unsigned short) * (2 * s.diml + 1));
        std::copy(s.last.begin(), s.last.begin() + s.H, last);
    }
    if (target) std::copy(s.target.begin(), s.target.end(), target);
    if (weight) std::copy(s.weight.begin(), s.weight.end(), weight);
    return 0;
}

int port_run_angles(int op, const float* input, float* output, int dimx, int dimy, const int* angles,
                    int nangles, float povh, int nthreads) {
    if (dimx <= 0 || dimy <= 0 || nangles <= 0) return 1;
    for (int i = 0; i < nangles; i++)
        if (angles[i] < 0 || angles[i] >= 180) return 1;
    std::vector<float> src[4];
    orientations(input, dimx, dimy, src);
    const size_t n = (size_t)dimx * dimy;
    const int diml = std::max(dimx, dimy);
    const int nt = nthreads > 0 ? nthreads : 1;
    std::vector<Worker> workers(nt);
    memset(output, 0, sizeof(float) * n);
#pragma omp parallel num_threads(nt)
    {
        Worker& w = workers[omp_get_thread_num()];
        w.S.assign(2 * n + diml, 0.0f);
        w.O.assign(2 * n + diml, 0.0f);
#pragma omp for schedule(dynamic)
        for (int i = 0; i < nangles; i++) run_sector(op, dimx, dimy, src, angles[i], povh, w);
    }
    // Deterministic stand-in for the reference's critical-section reduce
    // (main.cu:160-164): threads fold in id order.
    for (int t = 0; t < nt; t++) reduce_types(output, dimx, dimy, workers[t].acc, op == PORT_CEPSTRUM);
    return 0;
}

int port_run_angles_ordered(int op, const float* input, float* output, int dimx, int dimy, const int* angles,
                            int nangles, float povh, int nthreads) {
    if (dimx <= 0 || dimy <= 0 || nangles <= 0) return 1;
    for (int i = 0; i < nangles; i++)
        if (angles[i] < 0 || angles[i] >= 180) return 1;
    std::vector<float> src[4];
    orientations(input, dimx, dimy, src);
    const size_t n = (size_t)dimx * dimy;
    const int diml = std::max(dimx, dimy);
    const int nt = nthreads > 0 ? nthreads : 1;
    const bool max_mode = op == PORT_CEPSTRUM;
    // Per sector of a chunk: its geometry and the value its deskew folds into
    // every accumulator cell, (1-w)*lo + w*hi (add) or max(lo, hi) (max), the
    // same float expressions deskew_rows evaluates.
    const int chunk = 2 * nt;
    std::vector<Sector> sec(chunk);
    std::vector<std::vector<float>> val(chunk, std::vector<float>(n));
    std::vector<std::vector<float>> S(nt, std::vector<float>(2 * n + diml)), O(nt, std::vector<float>(2 * n + diml));
    std::vector<float> acc[4];
    for (int c0 = 0; c0 < nangles; c0 += chunk) {
        const int cn = std::min(chunk, nangles - c0);
#pragma omp parallel for num_threads(nt) schedule(dynamic)
        for (int k = 0; k < cn; k++) {
            const int th = omp_get_thread_num();
            Sector& s = sec[k];
            make_sector(dimx, dimy, angles[c0 + k], s);
            std::fill(S[th].begin(), S[th].end(), 0.0f);
            std::fill(O[th].begin(), O[th].end(), 0.0f);
            skew_rows(s, src[s.type].data(), S[th].data());
            run_operator(op, s, S[th].data(), O[th].data(), povh);
            const float* Ot = O[th].data();
            for (int i = 0; i < s.dim_o; i++)
                for (int j = 0; j < s.dim_i; j++) {
                    const float lo = Ot[(size_t)(i + s.target[j]) * s.dim_i + j];
                    const float hi = Ot[(size_t)(i + s.target[j] + 1) * s.dim_i + j];
                    val[k][(size_t)i * s.dim_i + j] =
                        max_mode ? std::max(lo, hi) : (1.0f - s.weight[j]) * lo + s.weight[j] * hi;
                }
        }
        for (int k = 0; k < cn; k++) {  // fold in list order, as one reference thread does
            const Sector& s = sec[k];
            std::vector<float>& a = acc[s.type];
            if (a.empty()) a.assign(n, 0.0f);
            const float* v = val[k].data();
            for (size_t q = 0; q < (size_t)s.dim_o * s.dim_i; q++) {
                if (max_mode) {
                    a[q] = std::max(a[q], v[q]);
                    a[q] = s.a + 1000 * (int)(a[q] / 1000);
                } else {
                    a[q] += v[q];
                }
            }
        }
    }
    memset(output, 0, sizeof(float) * n);
    reduce_types(output, dimx, dimy, acc, max_mode);
    return 0;
}

int port_run(int op, const float* input, float* output, int dimx, int dimy, int nsect, float povh,
             int nthreads) {
    if (nsect <= 0 || nsect > 180) return 1;
    std::vector<int> angles(nsect);
    for (int i = 0; i < nsect; i++) angles[i] = i;
    return port_run_angles(op, input, output, dimx, dimy, angles.data(), nsect, povh, nthreads);
}

int port_sector(int op, const float* input, int dimx, int dimy, int angle, float povh, float* skew_in,
                float* skew_out, float* acc) {
    if (dimx <= 0 || dimy <= 0 || angle < 0 || angle >= 180) return 1;
    std::vector<float> src[4];
    orientations(input, dimx, dimy, src);
    const size_t n = (size_t)dimx * dimy;
    Worker w;
    w.S.assign(2 * n + std::max(dimx, dimy), 0.0f);
    w.O.assign(w.S.size(), 0.0f);
    run_sector(op, dimx, dimy, src, angle, povh, w);
    if (skew_in) std::copy(w.S.begin(), w.S.end(), skew_in);
    if (skew_out) std::copy(w.O.begin(), w.O.end(), skew_out);
    if (acc) {
        memset(acc, 0, sizeof(float) * n);
        reduce_types(acc, dimx, dimy, w.acc, op == PORT_CEPSTRUM);
    }
    return 0;
}

int port_sdem_counts(const float* input, int dimx, int dimy, int angle, float povh, float* counts) {
    if (dimx <= 0 || dimy <= 0 || angle < 0 || angle >= 180) return 1;
    std::vector<float> src[4];
    orientations(input, dimx, dimy, src);
    const size_t n = (size_t)dimx * dimy;
    Sector s;
    make_sector(dimx, dimy, angle, s);
    std::vector<float> S(2 * n + s.diml, 0.0f);
    skew_rows(s, src[s.type].data(), S.data());
    memset(counts, 0, sizeof(float) * S.size());
    op_sdem(s, S.data(), counts, povh, true);
    return 0;
}

int port_accumulate(int op, const float* input, int dimx, int dimy, const int* angles, int nangles, float povh,
                    float* acc, int* used_mask) {
    if (dimx <= 0 || dimy <= 0 || nangles < 0) return 1;
    for (int i = 0; i < nangles; i++)
        if (angles[i] < 0 || angles[i] >= 180) return 1;
    std::vector<float> src[4];
    orientations(input, dimx, dimy, src);
    const size_t n = (size_t)dimx * dimy;
    Worker w;
    w.S.assign(2 * n + std::max(dimx, dimy), 0.0f);
    w.O.assign(w.S.size(), 0.0f);
    for (int i = 0; i < nangles; i++) run_sector(op, dimx, dimy, src, angles[i], povh, w);
    int mask = 0;
    for (int t = 0; t < 4; t++) {
        if (w.acc[t].empty()) {
            memset(acc + t * n, 0, sizeof(float) * n);
        } else {
            std::copy(w.acc[t].begin(), w.acc[t].end(), acc + t * n);
            mask |= 1 << t;
        }
    }
    *used_mask = mask;
    return 0;
}

int port_run_f64(int op, const float* input, double* output, int dimx, int dimy, int nsect, float povh) {
    (void)povh;
    if (dimx <= 0 || dimy <= 0 || nsect <= 0 || nsect > 180) return 1;
    if (op != PORT_RADON && op != PORT_CEPSTRUM && op != PORT_IDENTITYDEM && op != PORT_IDENTITYIMG) return 1;
    std::vector<float> srcf[4];
    orientations(input, dimx, dimy, srcf);
    const size_t n = (size_t)dimx * dimy;
    const bool max_mode = op == PORT_CEPSTRUM;
    std::vector<double> S(2 * n + std::max(dimx, dimy)), O(S.size());
    std::vector<double> acc[4];
    for (int a = 0; a < nsect; a++) {
        Sector s;
        make_sector(dimx, dimy, a, s);
        std::fill(S.begin(), S.end(), 0.0);
        std::fill(O.begin(), O.end(), 0.0);
        const float* src = srcf[s.type].data();
        for (int i = 0; i < s.dim_o; i++)  // skew with the exact drift fraction
            for (int j = 0; j < s.dim_i; j++) {
                const double w = s.skewness * j - s.target[j];
                const double v = src[(size_t)s.dim_i * i + j];
                S[(size_t)(i + s.target[j]) * s.dim_i + j] += (1.0 - w) * v;
                S[(size_t)(i + s.target[j] + 1) * s.dim_i + j] += w * v;
            }
        if (op == PORT_RADON) op_radon_f64(s, S.data(), O.data());
        else if (op == PORT_CEPSTRUM) op_cepstrum_f64(s, S.data(), O.data());
        else
            for (int r = 0; r < s.H; r++)
                for (int j = s.first[r]; j < s.last[r]; j++) O[(size_t)s.dim_i * r + j] = S[(size_t)s.dim_i * r + j];
        if (acc[s.type].empty()) acc[s.type].assign(n, 0.0);
        for (int i = 0; i < s.dim_o; i++)
            for (int j = 0; j < s.dim_i; j++) {
                const double w = s.skewness * j - s.target[j];
                const double lo = O[(size_t)(i + s.target[j]) * s.dim_i + j];
                const double hi = O[(size_t)(i + s.target[j] + 1) * s.dim_i + j];
                double& cell = acc[s.type][(size_t)i * s.dim_i + j];
                if (max_mode) cell = s.a + 1000.0 * std::floor(std::max(cell, std::max(lo, hi)) / 1000.0);
                else cell += (1.0 - w) * lo + w * hi;
            }
    }
    for (int i = 0; i < dimy; i++)
        for (int j = 0; j < dimx; j++) {
            const int ci = dimy - 1 - i, cj = dimx - 1 - j;
            const size_t idx[4] = {(size_t)i * dimx + j, (size_t)cj * dimy + ci, (size_t)j * dimy + ci,
                                   (size_t)i * dimx + cj};
            double o = 0.0;
            for (int t = 0; t < 4; t++) {
                if (acc[t].empty()) continue;
                o = max_mode ? std::max(o, acc[t][idx[t]]) : o + acc[t][idx[t]];
            }
            output[(size_t)i * dimx + j] = o;
        }
    return 0;
}

double port_los_steps(int dimx, int dimy, int nsect) {
    double total = 0;
    for (int a = 0; a < nsect; a++) {
        Sector s;
        make_sector(dimx, dimy, a, s);
        for (int r = 0; r < s.H; r++) {
            const double L = (double)s.last[r] - (double)s.first[r];
            if (L > 0) total += L * (L - 1);
        }
    }
    return total;
}

}  // extern "C"
