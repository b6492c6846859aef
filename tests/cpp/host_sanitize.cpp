// Host code of the library under AddressSanitizer and UBSan, run by
// tests/test_host_sanitizers.py (compiled there from the library's own host
// sources: image_io.cpp, cli.cpp, geometry.cpp).
//
//   host_sanitize png <file>...   PNG size query, RGBA and grid reads of each file
//   host_sanitize grid <dir>      ske_read_grid and run()'s argument handling on
//                                 random .bil/raw files, headers, sizes and crops
//   host_sanitize geometry        every sector's tables of random square, flat
//                                 and tall grids, checked against the kernels' bounds
//
// The engine entry points run() reaches after reading its input are stood in
// for below (they report no device), so no GPU code is built.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "skewengine.h"
#include "ske_internal.h"

namespace ske {
static std::string g_last;
int set_last_error(int code, const char* msg) {
    g_last = msg;
    return code;
}
}  // namespace ske

extern "C" {
const char* ske_last_error(void) { return ske::g_last.c_str(); }
int ske_params_default(ske_params* p) {
    p->max_sector = 180;
    p->povh = 0.15f;
    p->accum = 0;
    p->flags = 0;
    return SKE_OK;
}
int ske_create(ske_engine*, int, int, int, void*) { return SKE_ERR_NO_DEVICE; }
int ske_run(ske_engine, int, const float*, int, float*, int, const ske_params*) { return SKE_ERR_NO_DEVICE; }
int ske_destroy(ske_engine) { return SKE_OK; }
}

namespace {

unsigned g_seed = 2024;
unsigned rnd() {
    g_seed = g_seed * 1103515245u + 12345u;
    return g_seed >> 8;
}

int png_files(int n, char** files) {
    int decoded = 0;
    for (int i = 0; i < n; i++) {
        int w = 0, h = 0;
        if (ske_png_size(files[i], &w, &h) != SKE_OK || (size_t)w * h > ((size_t)1 << 24)) continue;
        std::vector<uint8_t> px((size_t)w * h * 4);
        std::vector<float> grid((size_t)w * h);
        decoded += ske_png_read_rgba(files[i], px.data(), px.size()) == SKE_OK;
        ske_png_read_image(files[i], grid.data(), grid.size());
    }
    printf("png %d files, %d decoded\n", n, decoded);
    return 0;
}

int grids(const std::string& dir) {
    const std::string bil = dir + "/g.bil", hdr = dir + "/g.hdr", raw = dir + "/g.raw", out = dir + "/o.flt";
    int read = 0;
    for (int it = 0; it < 3000; it++) {
        std::vector<int16_t> v(rnd() % 3000);
        for (int16_t& x : v) x = (int16_t)rnd();
        for (const std::string* p : {&bil, &raw}) {
            FILE* f = fopen(p->c_str(), "wb");
            if (!v.empty()) fwrite(v.data(), 2, v.size(), f);
            fclose(f);
        }
        if (rnd() % 2) {
            FILE* f = fopen(hdr.c_str(), "w");
            fprintf(f, "NROWS %d\nncols %d\nJUNK\n%s\n", (int)(rnd() % 80) - 5, (int)(rnd() % 80) - 5,
                    rnd() % 2 ? "NCOLS 2147483647" : "x");
            fclose(f);
        } else {
            remove(hdr.c_str());
        }
        const int dx = rnd() % 3 ? 0 : (int)(rnd() % 90) - 5, dy = rnd() % 3 ? 0 : (int)(rnd() % 90) - 5;
        const int cx = (int)(rnd() % 70) - 3, cy = (int)(rnd() % 70) - 3;
        const std::string& path = rnd() % 2 ? bil : raw;
        int ox = 0, oy = 0;
        if (ske_read_grid(path.c_str(), dx, dy, cx, cy, nullptr, 0, &ox, &oy) == SKE_OK) {
            std::vector<float> g((size_t)ox * oy);
            read += ske_read_grid(path.c_str(), dx, dy, cx, cy, g.data(), g.size(), &ox, &oy) == SKE_OK;
        }
        std::string a[] = {"run", "sdem", path, std::to_string(dx), std::to_string(dy), out, "180", "0.15", "0",
                           std::to_string(cx), std::to_string(cy)};
        std::vector<char*> av;
        for (std::string& s : a) av.push_back(&s[0]);
        run((int)av.size(), av.data());
    }
    printf("grid 3000 cases, %d read\n", read);
    return 0;
}

int geometry() {
    long sectors = 0, refused = 0;
    for (int it = 0; it < 240; it++) {
        int dx, dy;
        switch (it % 4) {
            case 0: dx = 1 + rnd() % 64, dy = 1 + rnd() % 64; break;
            case 1: dx = 1 + rnd() % 3000, dy = 1 + rnd() % 8; break;
            case 2: dx = 1 + rnd() % 8, dy = 1 + rnd() % 3000; break;
            default: dx = 1 + rnd() % 1500, dy = 1 + rnd() % 1500; break;
        }
        ske::SectorDesc d;
        std::vector<int32_t> f, l, t;
        std::vector<float> w;
        for (int a = 0; a < 180; a++, sectors++) {
            ske::sector_geometry(dx, dy, a, d, f, l, t, w);
            refused += !ske::check_sector(d, f.data(), l.data(), t.data(), dx, dy).empty();
        }
    }
    printf("geometry %ld sectors, %ld refused\n", sectors, refused);
    return refused ? 1 : 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc >= 2 && !strcmp(argv[1], "png")) return png_files(argc - 2, argv + 2);
    if (argc >= 3 && !strcmp(argv[1], "grid")) return grids(argv[2]);
    if (argc >= 2 && !strcmp(argv[1], "geometry")) return geometry();
    fprintf(stderr, "usage: host_sanitize png <file>... | grid <dir> | geometry\n");
    return 2;
}
