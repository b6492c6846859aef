// Command-line entry point `run(argc, argv)`, the reference's only C export
// (src/main.cu:200-202), plus the DEM file formats it reads and writes.
//
//   run <kernel> <input> <dimx> <dimy> <output> [max_sector] [povh] [accum]
//       [crop_x] [crop_y]
//
//   kernel     sdem | identitydem | radon | identityimg | cepstrum | localradon,
//              or 0..5 (KERNELS enum, src/global.h:77; 5 = radon with LRT set)
//   input      raw little-endian float32 grid (dimy rows of dimx), or an ESRI
//              .bil int16 grid whose values are divided by 10 as readBilData does
//              (src/kernelSDEM.h:43-50); dimx/dimy 0 take NCOLS/NROWS from the
//              .hdr beside it, else a square grid from the file size
//              (check_dem, src/kernelSDEM.h:98-142)
//              A .png input is an image read as the reference's image operators
//              read theirs (helper::read_png, src/helper.h:167-184: R + G + B per
//              pixel); dimx/dimy 0 take its size.
//   output     raw float32 grid (the .flt dump of showResultsSDEM,
//              src/kernelSDEM.h:433-439), or, for a name ending in .png, the
//              reference's coloured result image (showResults, src/main.h:124-141)
//              and, for an image input, its grey copy as <stem>_input.png (the
//              reference's salida2.png and salida1.png)
//   max_sector angles 0..max_sector-1 (default 180), povh observer height in cell
//              units (default 0.15), accum 0 reference order / 1 Kahan.
//   crop_x/y   columns / rows dropped from the right / bottom of the input grid
//              (readBilData's crop, src/kernelSDEM.h:31-52): the run takes the
//              top-left (dimx - crop_x) x (dimy - crop_y) window.
//
// Returns 0 on success, a SKE_* status otherwise; messages go to stderr.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "../../include/skewengine.h"
#include "image_io.h"

namespace {

// An input error: the message becomes the calling thread's last error
// (ske_last_error); run() also prints it.
int input_error(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return ske::set_last_error(SKE_ERR_INVALID, buf);
}

int parse_kernel(const char* s) {
    static const char* names[] = {"sdem", "identitydem", "radon", "identityimg", "cepstrum", "localradon"};
    for (int i = 0; i < 6; i++)
        if (!strcmp(s, names[i])) return i;
    char* end = nullptr;
    long v = strtol(s, &end, 10);
    if (end && *end == 0 && v >= SKE_KERNEL_SDEM && v <= SKE_KERNEL_LOCAL_RADON) return (int)v;
    return -1;
}

bool ends_with(const std::string& s, const char* suf) {
    const size_t n = strlen(suf);
    return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

// NROWS / NCOLS from an ESRI header next to `bil` (same stem, .hdr).
void read_hdr(const std::string& bil, int* ncols, int* nrows) {
    const std::string hdr = bil.substr(0, bil.find_last_of('.')) + ".hdr";
    FILE* f = fopen(hdr.c_str(), "r");
    if (!f) return;
    char line[256];
    while (fgets(line, sizeof(line), f)) {
        char key[64];
        int v = 0;
        if (sscanf(line, "%63s %d", key, &v) != 2) continue;
        for (char* k = key; *k; k++) *k = (char)toupper((unsigned char)*k);
        if (!strcmp(key, "NCOLS")) *ncols = v;
        if (!strcmp(key, "NROWS")) *nrows = v;
    }
    fclose(f);
}

long file_size(const char* path) {
    FILE* f = fopen(path, "rb");
    if (!f) return -1;
    fseek(f, 0, SEEK_END);
    const long n = ftell(f);
    fclose(f);
    return n;
}

// The input grid of a run: the file's grid (dimx x dimy; 0 = from the .hdr,
// the image or the file size), then readBilData's crop (src/kernelSDEM.h:31-52):
// the top-left (dimx - crop_x) x (dimy - crop_y) window, rows at the file's
// pitch.  On success *dimx/*dimy hold the window's size.
int load_input(const std::string& path, int* dimx, int* dimy, int crop_x, int crop_y, std::vector<float>& out) {
    if (crop_x < 0 || crop_y < 0) return input_error("negative crop %d, %d", crop_x, crop_y);
    int fdx = *dimx, fdy = *dimy;
    std::vector<float> full;
    if (ends_with(path, ".png")) {
        int w = 0, h = 0;
        const int rc = ske::png_read_grid(path.c_str(), &w, &h, full);
        if (rc != SKE_OK) return input_error("cannot read image %s", path.c_str());
        if ((fdx > 0 && fdx != w) || (fdy > 0 && fdy != h))
            return input_error("%s is %dx%d, not %dx%d", path.c_str(), w, h, fdx, fdy);
        fdx = w;
        fdy = h;
    } else {
        const bool bil = ends_with(path, ".bil");
        const long bytes = file_size(path.c_str());
        if (bytes < 0) return input_error("cannot open %s", path.c_str());
        const int cell = bil ? 2 : 4;
        if (fdx <= 0 || fdy <= 0) {
            int nc = 0, nr = 0;
            if (bil) read_hdr(path, &nc, &nr);
            if (nc <= 0 || nr <= 0) nc = nr = (int)std::sqrt((double)(bytes / cell));
            fdx = nc;
            fdy = nr;
        }
        if (fdx <= 0 || fdy <= 0 || crop_x >= fdx || crop_y >= fdy)
            return input_error("%s: a %dx%d grid cropped by %d, %d is empty", path.c_str(), fdx, fdy, crop_x, crop_y);
        // The rows the window reads, at the file's pitch (the last one only up
        // to the window's width, as readBilData reads it).
        const size_t rows = (size_t)(fdy - crop_y);
        const size_t n = (rows - 1) * (size_t)fdx + (size_t)(fdx - crop_x);
        if ((size_t)bytes < n * cell) return input_error("%s holds %ld bytes, need %zu", path.c_str(), bytes, n * cell);
        full.resize(n);
        FILE* f = fopen(path.c_str(), "rb");
        if (!f) return input_error("cannot open %s", path.c_str());
        if (bil) {
            std::vector<int16_t> raw(n);
            const size_t got = fread(raw.data(), 2, n, f);
            fclose(f);
            if (got != n) return input_error("cannot read %s", path.c_str());
            for (size_t i = 0; i < n; i++) full[i] = (float)(((float)raw[i]) / 10.0);
        } else {
            const size_t got = fread(full.data(), 4, n, f);
            fclose(f);
            if (got != n) return input_error("cannot read %s", path.c_str());
        }
    }
    if (crop_x >= fdx || crop_y >= fdy)
        return input_error("a %dx%d grid cropped by %d, %d is empty", fdx, fdy, crop_x, crop_y);
    const int wx = fdx - crop_x, wy = fdy - crop_y;
    if (crop_x == 0 && crop_y == 0 && full.size() == (size_t)wx * wy) {
        out.swap(full);
    } else {
        out.resize((size_t)wx * wy);
        for (int i = 0; i < wy; i++)
            std::copy(full.begin() + (size_t)i * fdx, full.begin() + (size_t)i * fdx + wx, out.begin() + (size_t)i * wx);
    }
    *dimx = wx;
    *dimy = wy;
    return SKE_OK;
}

int run_main(int argc, char** argv) {
    if (argc < 6) {
        fprintf(stderr,
                "usage: run <kernel> <input> <dimx> <dimy> <output> [max_sector] [povh] [accum] [crop_x] [crop_y]\n");
        return SKE_ERR_INVALID;
    }
    const int kernel = parse_kernel(argv[1]);
    if (kernel < 0) {
        fprintf(stderr, "run: unknown kernel '%s'\n", argv[1]);
        return SKE_ERR_INVALID;
    }
    int dimx = atoi(argv[3]), dimy = atoi(argv[4]);
    const int crop_x = argc > 9 ? atoi(argv[9]) : 0, crop_y = argc > 10 ? atoi(argv[10]) : 0;
    std::vector<float> in;
    int rc = load_input(argv[2], &dimx, &dimy, crop_x, crop_y, in);
    if (rc != SKE_OK) {
        fprintf(stderr, "run: %s\n", ske_last_error());
        return rc;
    }
    ske_params p;
    ske_params_default(&p);
    if (argc > 6) p.max_sector = atoi(argv[6]);
    if (argc > 7) p.povh = (float)atof(argv[7]);
    if (argc > 8) p.accum = atoi(argv[8]);
    ske_engine e = nullptr;
    rc = ske_create(&e, dimx, dimy, 0, nullptr);
    if (rc != SKE_OK) {
        fprintf(stderr, "run: %s\n", ske_last_error());
        return rc;
    }
    std::vector<float> out((size_t)dimx * dimy);
    rc = ske_run(e, kernel, in.data(), 0, out.data(), 0, &p);
    if (rc != SKE_OK) fprintf(stderr, "run: %s\n", ske_last_error());
    ske_destroy(e);
    if (rc != SKE_OK) return rc;
    const std::string dst = argv[5];
    if (ends_with(dst, ".png")) {
        std::vector<uint8_t> rgb(out.size() * 3);
        rc = ske_render(kernel, out.data(), dimx, dimy, rgb.data());
        if (rc == SKE_OK) rc = ske_png_write(dst.c_str(), rgb.data(), dimx, dimy, 3);
        if (rc == SKE_OK && ends_with(argv[2], ".png")) {
            std::vector<uint8_t> grey(in.size());
            rc = ske_render_input(in.data(), (int)in.size(), grey.data());
            if (rc == SKE_OK)
                rc = ske_png_write((dst.substr(0, dst.size() - 4) + "_input.png").c_str(), grey.data(), dimx, dimy, 1);
        }
        if (rc != SKE_OK) fprintf(stderr, "run: cannot render or write %s\n", dst.c_str());
        return rc;
    }
    FILE* f = fopen(dst.c_str(), "wb");
    if (!f) {
        fprintf(stderr, "run: cannot write %s\n", dst.c_str());
        return SKE_ERR_INVALID;
    }
    fwrite(out.data(), sizeof(float), out.size(), f);
    fclose(f);
    return SKE_OK;
}

}  // namespace

extern "C" int run(int argc, char** argv) {
    try {
        return run_main(argc, argv);
    } catch (const std::exception& ex) {  // e.g. a grid too large to allocate: no exception crosses the C ABI
        fprintf(stderr, "run: %s\n", ex.what());
        return SKE_ERR_INVALID;
    }
}

extern "C" int ske_read_grid(const char* path, int dimx, int dimy, int crop_x, int crop_y, float* grid,
                             size_t capacity, int* out_dimx, int* out_dimy) {
    if (!path || !out_dimx || !out_dimy) return SKE_ERR_INVALID;
    try {
        std::vector<float> g;
        int dx = dimx, dy = dimy;
        const int rc = load_input(path, &dx, &dy, crop_x, crop_y, g);
        if (rc != SKE_OK) return rc;
        *out_dimx = dx;
        *out_dimy = dy;
        if (!grid) return SKE_OK;
        if (g.size() > capacity) return SKE_ERR_INVALID;
        std::copy(g.begin(), g.end(), grid);
        return SKE_OK;
    } catch (const std::exception&) {  // allocation failure: no exception crosses the C ABI
        return SKE_ERR_INVALID;
    }
}
