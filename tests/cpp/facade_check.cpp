// Checks of the C++ facade (include/skewengine.hpp), run by
// tests/test_z_cpp_facade.py.
//
//   facade_check host   no device needed: operator ids, host geometry (printed
//                       for the test to compare with the C ABI through Python),
//                       the refusals of a CPU engine and of a missing device
//   facade_check gpu    on device 0: the reference's per-sector loop through the
//                       facade equals execute() bit for bit (total viewshed),
//                       the cepstrum's max loop equals the same C ABI calls,
//                       and a kernelcuda operator receives the reference's
//                       arguments in its order
#include <cstdio>
#include <cstring>
#include <vector>

#include "skewengine.hpp"

static_assert(ske::KERNEL_SDEM == 0 && ske::KERNEL_IDENTITYDEM == 1 && ske::KERNEL_RADON == 2 &&
                  ske::KERNEL_IDENTITYIMG == 3 && ske::KERNEL_CEPSTRUM == 4,
              "the reference's KERNELS order (src/global.h:77)");

namespace {

int failures = 0;

void expect(bool ok, const char* what) {
    if (!ok) {
        std::printf("FAIL %s\n", what);
        failures++;
    }
}

int host_checks() {
    const int shapes[][2] = {{37, 23}, {23, 37}, {16, 16}, {1, 9}};
    const int angles[] = {0, 1, 30, 45, 46, 89, 90, 91, 135, 179};
    for (const auto& s : shapes)
        for (int a : angles) {
            const ske::sector_tables t = ske::sector_geometry(s[0], s[1], a);
            long long sf = 0, sl = 0, st = 0;
            double sw = 0.0;
            for (int32_t v : t.first) sf += v;
            for (int32_t v : t.last) sl += v;
            for (int32_t v : t.target) st += v;
            for (float v : t.weight) sw += v;
            std::printf("geom %d %d %d %d %d %d %d %d %d %d %.17g %lld %lld %lld %.17g\n", s[0], s[1], a,
                        t.geom.sector_type, t.geom.new_angle, t.geom.dim_i, t.geom.dim_o, t.geom.offset,
                        t.geom.skew_height, t.geom.dim_l, t.geom.scale, sf, sl, st, sw);
        }
    std::vector<float> grid(8 * 8, 1.0f);
    const ske::inputData<float> in = ske::skewEngine<float>::prepare(grid.data(), 8, 8);
    try {
        ske::skewEngine<float> cpu(8, 8, in, false);
        expect(false, "a CPU engine is refused");
    } catch (const ske::error& e) {
        expect(e.status == SKE_ERR_UNSUPPORTED, "a CPU engine is refused as unsupported");
    }
    try {
        ske::skewEngine<float> nodev(8, 8, in, true, 4096);
        expect(false, "device 4096 is refused");
    } catch (const ske::error& e) {
        expect(e.status == SKE_ERR_NO_DEVICE || e.status == SKE_ERR_INVALID, "device 4096 is refused");
    }
    try {
        ske::sector_geometry(8, 8, 180);
        expect(false, "angle 180 is refused");
    } catch (const ske::error& e) {
        expect(e.status == SKE_ERR_INVALID && std::strlen(e.what()) > 0, "angle 180 is refused with a message");
    }
    try {
        std::vector<float> out(64, 0.0f);
        ske::execute(ske::KERNEL_SDEM, grid.data(), out.data(), 8, 8, 180, 0.15f, 4096);
        expect(false, "execute on device 4096 is refused");
    } catch (const ske::error& e) {
        expect(e.status == SKE_ERR_NO_DEVICE || e.status == SKE_ERR_INVALID, "execute on device 4096 is refused");
    }
    float* outD = nullptr;
    ske::inputData<float> in2;
    ske::skewEngine<float>::allocate(in2, grid.data(), &outD, 8, 8);
    bool zeroed = in2.grid == grid.data();
    for (int i = 0; i < 64; i++) zeroed = zeroed && outD[i] == 0.0f;
    expect(zeroed, "allocate gives the input and a zeroed output");
    ske::skewEngine<float>::deallocate(in2, grid.data(), outD);
    return failures;
}

// Seeded heights in [0, 150) cell units.
std::vector<float> heights(int n, unsigned seed) {
    std::vector<float> v((size_t)n);
    for (float& x : v) {
        seed = seed * 1664525u + 1013904223u;
        x = (float)(seed >> 8) * (150.0f / 16777216.0f);
    }
    return v;
}

struct Seen {
    const ske::skewEngine<float>* eng = nullptr;
    int calls = 0, bad = 0;
};
Seen seen;

int probe(float* out, const float* in, int dim_i, int skewHeight, const int32_t* last, const int32_t* first,
          float val, int angle, void* stream) {
    const ske::skewEngine<float>& e = *seen.eng;
    seen.calls++;
    if (out != e.d_skewOutput || in != e.d_skewInput || dim_i != e.dim_i || skewHeight != e.skewHeight ||
        last != e.d_last || first != e.d_first || val != e.val || angle != e.newAngle || !stream)
        seen.bad++;
    return 0;  // launches nothing: the skewed output stays zero
}

bool same_bits(const std::vector<float>& a, const std::vector<float>& b) {
    return a.size() == b.size() && std::memcmp(a.data(), b.data(), a.size() * sizeof(float)) == 0;
}

// The reference's sector loop (src/main.cu:147-164) through the facade.
std::vector<float> facade_loop(const std::vector<float>& x, int dimx, int dimy, int alg) {
    const int is_max = alg == ske::KERNEL_CEPSTRUM;
    std::vector<float> out((size_t)dimx * dimy, 0.0f);
    ske::skewEngine<float> eng(dimx, dimy, ske::skewEngine<float>::prepare(x.data(), dimx, dimy));
    eng.algorithm = alg;
    eng.skewAlloc();
    for (int i = 0; i < 180; i++) {
        eng.skew(i);
        eng.kernel();
        eng.deskew(is_max);
    }
    eng.reduce(out.data(), is_max);
    return out;
}

// The same loop through the C ABI's per-sector calls.
std::vector<float> abi_loop(const std::vector<float>& x, int dimx, int dimy, int alg) {
    const int is_max = alg == ske::KERNEL_CEPSTRUM;
    std::vector<float> out((size_t)dimx * dimy, 0.0f);
    ske_engine e = nullptr;
    ske::check(ske_create(&e, dimx, dimy, 0, nullptr));
    ske::check(ske_prepare(e, x.data(), 0));
    for (int i = 0; i < 180; i++) {
        ske::check(ske_skew(e, i));
        ske::check(ske_kernel(e, alg, 0.15f));
        ske::check(ske_deskew(e, is_max, SKE_ACCUM_REFERENCE));
    }
    ske::check(ske_reduce(e, out.data(), 0, is_max));
    ske_destroy(e);
    return out;
}

bool any_nonzero(const std::vector<float>& v) {
    for (float f : v)
        if (f != 0.0f) return true;
    return false;
}

int gpu_checks() {
    // Total viewshed on a 64 x 64 grid: the loop equals the whole run
    // (ske_run), as the per-sector API does through ctypes.
    const std::vector<float> dem = heights(64 * 64, 77u);
    const std::vector<float> loop = facade_loop(dem, 64, 64, ske::KERNEL_SDEM);
    std::vector<float> whole((size_t)64 * 64, 0.0f);
    ske::execute(ske::KERNEL_SDEM, dem.data(), whole.data(), 64, 64);
    expect(same_bits(loop, whole) && any_nonzero(whole), "per-sector loop equals execute (total viewshed)");
    const int dimx = 48, dimy = 40, n = dimx * dimy;
    const std::vector<float> x = heights(n, 2024u);
    {
        // The row-pointer reduce(T**) adds the same fold as reduce(T*).
        ske::skewEngine<float> eng(dimx, dimy, ske::skewEngine<float>::prepare(x.data(), dimx, dimy));
        for (int i = 0; i < 180; i += 7) {
            eng.skew(i);
            eng.kernel();
            eng.deskew(0);
        }
        std::vector<float> flat((size_t)n, 0.0f), rows((size_t)n, 0.0f);
        std::vector<float*> ptr((size_t)dimy);
        for (int i = 0; i < dimy; i++) ptr[(size_t)i] = rows.data() + (size_t)i * dimx;
        eng.reduce(flat.data(), 0);
        eng.reduce(ptr.data());
        expect(same_bits(flat, rows) && any_nonzero(flat), "reduce(T**) equals reduce(T*)");
    }
    // Cepstrum (max deskew and fold): the facade's loop equals the same calls
    // made on the C ABI directly.
    const std::vector<float> ceps = facade_loop(x, dimx, dimy, ske::KERNEL_CEPSTRUM);
    expect(same_bits(ceps, abi_loop(x, dimx, dimy, ske::KERNEL_CEPSTRUM)) && any_nonzero(ceps),
           "per-sector loop equals the C ABI's (cepstrum)");
    {
        ske::skewEngine<float> eng(dimx, dimy, ske::skewEngine<float>::prepare(x.data(), dimx, dimy));
        seen.eng = &eng;
        eng.kernelcuda = probe;
        eng.val = 0.25f;
        for (int i : {0, 30, 60, 90, 120, 150}) {
            eng.skew(i);
            eng.kernel();
            eng.deskew(0);
        }
        std::vector<float> out((size_t)n, 0.0f);
        eng.reduce(out.data(), 0);
        bool zero = true;
        for (float v : out) zero = zero && v == 0.0f;
        expect(seen.calls == 6 && seen.bad == 0, "kernelcuda receives the reference's arguments in its order");
        expect(zero, "an operator that writes nothing leaves a zero result");
    }
    return failures;
}

}  // namespace

int main(int argc, char** argv) {
    const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
    try {
        const int f = gpu ? gpu_checks() : host_checks();
        std::printf(f ? "facade checks: %d failed\n" : "facade checks passed\n", f);
        return f ? 1 : 0;
    } catch (const ske::error& e) {
        std::printf("FAIL unexpected error %d: %s\n", e.status, e.what());
        return 1;
    }
}
