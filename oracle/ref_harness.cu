// Test oracle: drives the reference skewEngine CPU path, compiled from the
// reference's own unmodified sources (src/skewEngine.cuh, src/kernelSDEM.h,
// src/kernelRADN.h, src/kernelBLUR.h, src/kernelUNIT.h, src/helper.h).
//
// This file is test infrastructure only.  It is compiled by oracle/Makefile into
// oracle/_ref/libskewref.so, which exists only where the reference sources are
// present; it is used to generate and re-check the golden fixtures in
// tests/golden and as a CPU timing baseline.  Nothing in the product links it.
//
// The sector loop below restates the reference driver `execute()`
// (src/main.cu:86-168): one engine per OpenMP thread, operator bound through
// `kernelcpu`, `skew(i); kernel(); deskew(isMax)` per sector with a dynamic
// schedule, then `reduce(outD, isMax)` inside a critical section.  main.cu itself
// does not compile with GCC 13, so it is not built.
//
// One harness-side choice: before each sector the full skew buffers are cleared
// (the reference only clears skewHeight*dim_i cells, skewEngine.cuh:567-568).
// For non-square inputs the reference reads past that region
// (last[] is initialised with dim_l, skewEngine.cuh:581), which would otherwise
// read values left behind by earlier sectors; clearing makes those reads zero
// and the run deterministic.  Square inputs never read past the region.

#include <cstdio>
#include <cstring>
#include <fstream>
#include <omp.h>
#include <unistd.h>
#include <vector>

#include "helper.h"

// The reference writes its result images under the compile-time O_DIR
// (src/defaults.h:21-28), a directory of its author's machine; the harness
// renders into the current directory instead (skref_render changes into a
// directory the caller gives).
#undef O_DIR
#define O_DIR ""

// Globals that src/main.cu defines (main.cu:59-60) and the kernel headers use.
int skewAlgorithm;
bool timing = true;

#include "kernelSDEM.h"
#include "kernelRADN.h"
#include "kernelBLUR.h"
#include "kernelUNIT.h"

static void bind_operator(skewEngine<float>* sk, int alg) {
    switch (alg) {
        case KERNEL_SDEM: sk->kernelcpu = kernelV3; break;
        case KERNEL_RADON: sk->kernelcpu = radon; break;
        case KERNEL_CEPSTRUM: sk->kernelcpu = cepstrum; break;
        default: sk->kernelcpu = identity; break;  // KERNEL_IDENTITYDEM / KERNEL_IDENTITYIMG
    }
}

static void clear_full(skewEngine<float>* sk, int n, int diml) {
    memset(sk->skewInput, 0, sizeof(float) * (size_t)(2 * n + diml));
    memset(sk->skewOutput, 0, sizeof(float) * (size_t)(2 * n + diml));
}

extern "C" {

int skref_run_angles(int alg, const float* input, float* output, int dx, int dy, const int* angles,
                     int nangles, float povh, int nthreads);

// Whole run: output (dimx*dimy floats) = reference result for `alg`
// (KERNELS enum, global.h:77) over sectors [0, nsect).
int skref_run(int alg, const float* input, float* output, int dx, int dy, int nsect,
              float povh, int nthreads) {
    if (nsect <= 0 || nsect > 180) return 1;
    int angles[180];
    for (int i = 0; i < nsect; i++) angles[i] = i;
    return skref_run_angles(alg, input, output, dx, dy, angles, nsect, povh, nthreads);
}

// Same over an explicit list of angles (the loop index i of main.cu:147 maps to
// angles[i]).
int skref_run_angles(int alg, const float* input, float* output, int dx, int dy, const int* angles,
                     int nsect, float povh, int nthreads) {
    if (dx <= 0 || dy <= 0 || nsect <= 0 || nsect > 180) return 1;
    for (int i = 0; i < nsect; i++)
        if (angles[i] < 0 || angles[i] >= 180) return 1;
    dimx = dx;
    dimy = dy;
    N = dim = dx * dy;
    maxSector = nsect;
    POVh = povh;
    skewAlgorithm = alg;
    float* inputD = new float[N];
    memcpy(inputD, input, sizeof(float) * (size_t)N);
    inputData<float> in = skewEngine<float>::prepare(inputD, dimx, dimy);
    memset(output, 0, sizeof(float) * (size_t)N);
    const int diml = dx > dy ? dx : dy;
    const int isMax = alg == KERNEL_CEPSTRUM ? 1 : 0;
    omp_set_num_threads(nthreads > 0 ? nthreads : 1);
#pragma omp parallel default(shared)
    {
        int id = omp_get_thread_num();
        skewEngine<float>* sk = new skewEngine<float>(dimx, dimy, in, false, id);
        bind_operator(sk, alg);
        sk->skewAlloc();
#pragma omp barrier
#pragma omp for schedule(dynamic) nowait
        for (int i = 0; i < nsect; i++) {
            clear_full(sk, N, diml);
            sk->skew(angles[i]);
            sk->kernel();
            sk->deskew(isMax);
        }
#pragma omp critical
        { sk->reduce(output, isMax); }
        delete sk;
    }
    delete[] in.input1;
    delete[] in.input2;
    delete[] in.input3;
    delete[] inputD;
    return 0;
}

// One sector in isolation, exposing the engine's intermediate state.
//   iinfo[0..6] = sectorType, newAngle, dim_i, dim_o, offset, skewHeight, dim_l
//   dinfo[0..1] = scale, skewness
//   skewIn/skewOut: 2*N + dim_l floats (the engine's whole skew buffers)
//   first/last: 2*dim_l+1 entries; target/weight: dim_l entries
//   acc: N floats, the per-type accumulator after deskew of this one sector
int skref_sector(int alg, const float* input, int dx, int dy, int angle, float povh,
                 int* iinfo, double* dinfo, float* skewIn, float* skewOut,
                 unsigned short* first, unsigned short* last, int* target, float* weight,
                 float* acc) {
    if (dx <= 0 || dy <= 0 || angle < 0 || angle >= 180) return 1;
    dimx = dx;
    dimy = dy;
    N = dim = dx * dy;
    maxSector = 180;
    POVh = povh;
    skewAlgorithm = alg;
    float* inputD = new float[N];
    memcpy(inputD, input, sizeof(float) * (size_t)N);
    inputData<float> in = skewEngine<float>::prepare(inputD, dimx, dimy);
    const int diml = dx > dy ? dx : dy;
    skewEngine<float>* sk = new skewEngine<float>(dimx, dimy, in, false, 0);
    bind_operator(sk, alg);
    sk->skewAlloc();
    memset(sk->first, 0, sizeof(unsigned short) * (size_t)(2 * diml + 1));
    memset(sk->last, 0, sizeof(unsigned short) * (size_t)(2 * diml + 1));
    clear_full(sk, N, diml);
    sk->skew(angle);
    if (skewIn) memcpy(skewIn, sk->skewInput, sizeof(float) * (size_t)(2 * N + diml));
    sk->kernel();
    if (skewOut) memcpy(skewOut, sk->skewOutput, sizeof(float) * (size_t)(2 * N + diml));
    sk->deskew(alg == KERNEL_CEPSTRUM ? 1 : 0);
    iinfo[0] = sk->sectorType;
    iinfo[1] = sk->newAngle;
    iinfo[2] = sk->dim_i;
    iinfo[3] = sk->dim_o;
    iinfo[4] = sk->offset;
    iinfo[5] = sk->skewHeight;
    iinfo[6] = diml;
    dinfo[0] = sk->scale;
    dinfo[1] = sk->skewness;
    if (first) memcpy(first, sk->first, sizeof(unsigned short) * (size_t)(2 * diml + 1));
    if (last) memcpy(last, sk->last, sizeof(unsigned short) * (size_t)(2 * diml + 1));
    if (target) memcpy(target, sk->target, sizeof(int) * (size_t)diml);
    if (weight) memcpy(weight, sk->weight, sizeof(float) * (size_t)diml);
    if (acc) {
        // Per-type accumulator of this sector: reduce() folds it back into the
        // input orientation, so expose it through a zeroed output.
        memset(acc, 0, sizeof(float) * (size_t)N);
        sk->reduce(acc, alg == KERNEL_CEPSTRUM ? 1 : 0);
    }
    delete sk;
    delete[] in.input1;
    delete[] in.input2;
    delete[] in.input3;
    delete[] inputD;
    return 0;
}

// The reference's Radon operator switch (kernelRADN.h:212, `bool LRT`): false =
// global Radon / filtered back-projection (the reference default), true = the
// local Radon transform pointRadon (kernelRADN.h:114-182) per skewed cell.
int skref_set_local_radon(int on) {
    LRT = on != 0;
    return 0;
}

// The reference's DEM reader readBilData (src/kernelSDEM.h:31-52) on a .bil of
// file_dx x file_dy int16 cells with its crop: `out` receives the
// (file_dx - crop_x) x (file_dy - crop_y) grid it builds (int16 / 10.0, rows
// read at the file's pitch).  Used only to generate golden fixtures.
int skref_read_bil(const char* path, int file_dx, int file_dy, int crop_x, int crop_y, float* out) {
    if (crop_x < 0 || crop_y < 0 || file_dx <= crop_x || file_dy <= crop_y) return 1;
    dimx = file_dx;
    dimy = file_dy;
    float* data = new float[(size_t)file_dx * file_dy];
    std::vector<char> name(path, path + strlen(path) + 1);
    readBilData<float>(name.data(), data, crop_x, crop_y);
    const int ok = dimx == file_dx - crop_x && dimy == file_dy - crop_y;
    if (ok) memcpy(out, data, sizeof(float) * (size_t)dimx * dimy);
    delete[] data;
    return ok ? 0 : 2;
}

// The reference's result colourings, run in `dir`: for the Radon operator and
// the image identity showResultsRADN (src/kernelRADN.h:384-400) with the scale
// and shift showResults picks (src/main.h:124-141, restated: 255 / (max - min)
// and min for alg 2, 1/540 for alg 3); for the cepstrum and the DEM identity
// showResultsCEPS (src/kernelBLUR.h:306-410, after execute()'s sample-point
// set-up, whose sample dumps it writes too).  `rgb` receives salida2.png, the
// coloured result, decoded by the reference's PNG library.  Used only to
// generate golden fixtures.
int skref_render(int alg, const float* out, int dx, int dy, const char* dir, unsigned char* rgb) {
    if (dx <= 0 || dy <= 0 || !dir) return 1;
    dimx = dx;
    dimy = dy;
    N = dim = dx * dy;
    skewAlgorithm = alg;
    std::vector<float> o(out, out + (size_t)dim);
    outD = o.data();
    pixels.assign((size_t)dim, 0);
    saveSampleData = false;
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd) || chdir(dir) != 0) return 2;
    if (alg == KERNEL_RADON || alg == KERNEL_IDENTITYIMG) {
        const pair_t mm = helper::getMinMax(outD);
        const float autoScale = 255 / (mm.max - mm.min);
        float escala = (float)(1.0 / 540);
        if (alg == KERNEL_RADON) escala = autoScale;
        if (alg == KERNEL_RADON)
            showResultsRADN(escala, mm.min);
        else
            showResultsRADN(escala);
    } else {
        if (samplePoints.empty()) {  // execute()'s set-up of the sample points (src/main.cu:79-83)
            samplePoints.push_back(punto1);
            samplePoints.push_back(punto2);
            samplePoints.push_back(punto3);
        }
        for (int i = 0; i < 180; i++)
            if (sampleData1[i].empty()) allocSampleData(i);
        showResultsCEPS();
    }
    std::vector<unsigned char> img;
    unsigned w = 0, h = 0;
    const unsigned err = lodepng::decode(img, w, h, "salida2.png", LCT_RGB);
    const int back = chdir(cwd);
    outD = nullptr;
    if (err || back != 0 || w != (unsigned)dx || h != (unsigned)dy) return 3;
    memcpy(rgb, img.data(), img.size());
    return 0;
}

// Result rendering and PNG coding as the reference does them: HSVtoRGB from
// src/color.cpp:80-115, helper::getMinMax (src/helper.h:190-201) and the
// reference's vendored lodepng (src/third-party/Lodepng.cpp), which its
// read_png (src/helper.h:167-184) and result writers (kernelRADN.h:384-400,
// kernelBLUR.h:396-410) call.  Used only to generate golden fixtures.
int skref_hsv_to_rgb(float h, float s, float v, unsigned char* rgb) {
    const rgbColor c = HSVtoRGB({h, s, v});
    rgb[0] = c.R;
    rgb[1] = c.G;
    rgb[2] = c.B;
    return 0;
}

int skref_min_max(float* data, int n, float* mn, float* mx) {
    dimx = n;
    dimy = 1;
    const pair_t p = helper::getMinMax(data);
    *mn = p.min;
    *mx = p.max;
    return 0;
}

// Encode 8-bit RGBA pixels as a PNG of the given colour type and bit depth
// (lodepng's own conversion), optionally Adam7-interlaced.
int skref_png_encode(const char* path, const unsigned char* rgba, unsigned w, unsigned h, int colortype,
                     int bitdepth, int interlace) {
    lodepng::State st;
    st.info_raw.colortype = LCT_RGBA;
    st.info_raw.bitdepth = 8;
    st.info_png.color.colortype = (LodePNGColorType)colortype;
    st.info_png.color.bitdepth = (unsigned)bitdepth;
    st.info_png.interlace_method = (unsigned)interlace;
    st.encoder.auto_convert = LAC_NO;
    std::vector<unsigned char> img(rgba, rgba + (size_t)w * h * 4), png;
    const unsigned err = lodepng::encode(png, img, w, h, st);
    if (err) return (int)err;
    return (int)lodepng_save_file(png.data(), png.size(), path);
}

// Encode with lodepng's automatic choice of the smallest lossless colour type
// (palette, grey, low bit depths), optionally interlaced.
int skref_png_encode_auto(const char* path, const unsigned char* rgba, unsigned w, unsigned h, int interlace) {
    lodepng::State st;
    st.info_raw.colortype = LCT_RGBA;
    st.info_raw.bitdepth = 8;
    st.info_png.interlace_method = (unsigned)interlace;
    st.encoder.auto_convert = LAC_AUTO;
    std::vector<unsigned char> img(rgba, rgba + (size_t)w * h * 4), png;
    const unsigned err = lodepng::encode(png, img, w, h, st);
    if (err) return (int)err;
    return (int)lodepng_save_file(png.data(), png.size(), path);
}

// Decode to 8-bit RGBA as read_png does (lodepng::decode's default).
int skref_png_decode(const char* path, unsigned char* rgba, size_t cap, unsigned* w, unsigned* h) {
    std::vector<unsigned char> img;
    const unsigned err = lodepng::decode(img, *w, *h, path);
    if (err) return (int)err;
    if (img.size() > cap) return -1;
    memcpy(rgba, img.data(), img.size());
    return 0;
}

}  // extern "C"
