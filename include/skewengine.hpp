/*
 * skewengine.hpp -- C++ facade of the C ABI (skewengine.h) with the interface
 * of the reference's skewEngine<T> class (src/skewEngine.cuh:141-372) and its
 * execute() driver (src/main.cu:71-172), for C++ callers of that class.
 *
 * Header only; it calls nothing but the C ABI, so it links against
 * libskewengine.so alone.  Errors throw ske::error (status + message) where the
 * reference either printed, exited or carried on.
 *
 * Where it differs from the reference, and why:
 *  - float only: the engine's kernels are float32 (the reference instantiates
 *    skewEngine<float> only, src/main.cu:91).
 *  - The GPU is the only path: isGPU = false (the reference's CPU loop) throws
 *    SKE_ERR_UNSUPPORTED.  There is no OpenCL mode.
 *  - inputData<float> holds the input grid, not the four orientations: the
 *    engine builds those on the device (prepare, src/skewEngine.cuh:925-987).
 *  - kernelcuda is a host function that launches its own kernels on the
 *    engine's stream (the last argument), where the reference launches the
 *    pointer as a kernel on a 16x16 grid (src/skewEngine.cuh:695-746).  Its
 *    other arguments are the reference's, in its order (last before first);
 *    row limits are int32 instead of unsigned short.
 *  - The operator value (the observer height POVh of kernelSDEM) is the member
 *    `val`, where the reference passes the literal 0.15f.
 */
#ifndef SKEWENGINE_HPP
#define SKEWENGINE_HPP

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "skewengine.h"

namespace ske {

/* The reference's operators (enum KERNELS, src/global.h:77), plus its Radon
 * operator with LRT set (src/kernelRADN.h:212-220) as an id of its own. */
enum KERNELS : int {
    KERNEL_SDEM = SKE_KERNEL_SDEM,
    KERNEL_IDENTITYDEM = SKE_KERNEL_IDENTITYDEM,
    KERNEL_RADON = SKE_KERNEL_RADON,
    KERNEL_IDENTITYIMG = SKE_KERNEL_IDENTITYIMG,
    KERNEL_CEPSTRUM = SKE_KERNEL_CEPSTRUM,
    KERNEL_LOCAL_RADON = SKE_KERNEL_LOCAL_RADON
};

/* A failed C ABI call: its status (SKE_ERR_*) and message. */
class error : public std::runtime_error {
public:
    error(int code, const std::string& what) : std::runtime_error(what), status(code) {}
    int status;
};

inline void check(int rc) {
    if (rc != SKE_OK) throw error(rc, ske_last_error());
}

/* The input of an engine (inputData<T>, src/global.h:37): the dimy x dimx
 * grid, on the host (on_device 0) or the device (1). */
template <typename T>
struct inputData;

template <>
struct inputData<float> {
    const float* grid = nullptr;
    int on_device = 0;
};

template <typename T>
class skewEngine;

template <>
class skewEngine<float> {
public:
    /* kernelcuda (src/skewEngine.cuh:369): the reference's kernel arguments,
     * then the stream to launch on; returns 0 on success. */
    typedef int (*cuda_operator)(float* d_skewOutput, const float* d_skewInput, int dim_i, int skewHeight,
                                 const int32_t* d_last, const int32_t* d_first, float val, int angle, void* stream);

    /* src/skewEngine.cuh:462-477 (+ skewAlloc, :419-456): an engine for
     * dx x dy grids on `device`, its orientations built from inData (the
     * reference's arguments dimx, dimy, inData, isGPU, deviceId).
     * stream: a cudaStream_t to run on (NULL: the engine makes its own). */
    skewEngine(int dx, int dy, inputData<float> inData, bool gpu = true, int device = 0, void* stream = nullptr)
        : dimx(dx), dimy(dy), N(dx * dy), dim_l(dx > dy ? dx : dy), isGPU(gpu), deviceId(device) {
        if (!gpu) throw error(SKE_ERR_UNSUPPORTED, "skewEngine: no CPU path, the engine runs on the GPU");
        check(ske_create(&e_, dx, dy, device, stream));
        const int rc = ske_prepare(e_, inData.grid, inData.on_device);
        if (rc != SKE_OK) {
            const std::string msg = ske_last_error();
            ske_destroy(e_);
            throw error(rc, msg);
        }
    }
    virtual ~skewEngine() { ske_destroy(e_); }
    skewEngine(const skewEngine&) = delete;
    skewEngine& operator=(const skewEngine&) = delete;

    /* prepare(inputD, dimx, dimy) (src/skewEngine.cuh:925): the input of an
     * engine (the orientations themselves are built by the engine). */
    static inputData<float> prepare(const float* inputD, int /*dimx*/, int /*dimy*/, int on_device = 0) {
        inputData<float> d;
        d.grid = inputD;
        d.on_device = on_device;
        return d;
    }
    /* allocate / deallocate (src/skewEngine.cuh:379-411): the input and a
     * zeroed host output grid outD. */
    static void allocate(inputData<float>& inData, float* inputD, float** outD, int dimx, int dimy) {
        inData = prepare(inputD, dimx, dimy);
        *outD = new float[(size_t)dimx * dimy]();
    }
    static void deallocate(inputData<float> /*inData*/, float* /*inputD*/, float* outD) { delete[] outD; }

    /* Buffers are allocated by the constructor; kept for callers of the
     * reference's skewAlloc(). */
    void skewAlloc() {}

    /* skew(angle) (src/skewEngine.cuh:606-639) with resetSkew of the output:
     * the skewed input of sector `angle`; the public sector fields below
     * describe it afterwards. */
    void skew(int angle) {
        check(ske_skew(e_, angle));
        ske_sector_view v;
        check(ske_sector(e_, &v));
        a = v.geom.angle;
        sectorType = v.geom.sector_type;
        newAngle = v.geom.new_angle;
        dim_i = skewWidth = v.geom.dim_i;
        dim_o = v.geom.dim_o;
        offset = v.geom.offset;
        skewHeight = v.geom.skew_height;
        scale = v.geom.scale;
        skewness = v.geom.skewness;
        d_skewInput = const_cast<float*>(v.skew_in);
        d_skewOutput = v.skew_out;
        d_first = v.first;
        d_last = v.last;
        d_target = v.target;
        d_weight = v.weight;
    }

    /* kernel() (src/skewEngine.cuh:695-746): kernelcuda when set, else the
     * built-in operator `algorithm`, over the current skewed grid. */
    void kernel() {
        if (kernelcuda)
            check(ske_kernel_custom(e_, &skewEngine::trampoline, this, val));
        else
            check(ske_kernel(e_, algorithm, val));
    }

    /* deskew(isMax) (src/skewEngine.cuh:756-833) into the accumulator of the
     * current sector type, in accumulation mode `accum` (SKE_ACCUM_*). */
    void deskew(int isMax = 0) { check(ske_deskew(e_, isMax, accum)); }

    /* reduce(output, isMax) (src/skewEngine.cuh:862-914): the engine's fold
     * added into (isMax: maxed into) the host grid `output`, as the reference
     * adds into the caller's outD; a zeroed outD receives the fold itself. */
    void reduce(float* output, int isMax = 0) {
        std::vector<float> fold((size_t)N);
        check(ske_reduce(e_, fold.data(), 0, isMax));
        for (size_t i = 0; i < fold.size(); i++) {
            if (isMax)
                output[i] = output[i] > fold[i] ? output[i] : fold[i];
            else
                output[i] = output[i] + fold[i];
        }
    }
    /* The deprecated row-pointer form reduce(T** output) (src/skewEngine.cuh:
     * 842-854): the fold added into output[i][j], rows i < dimy. */
    void reduce(float** output) {
        std::vector<float> fold((size_t)N);
        check(ske_reduce(e_, fold.data(), 0, 0));
        for (int i = 0; i < dimy; i++)
            for (int j = 0; j < dimx; j++) output[i][j] = output[i][j] + fold[(size_t)i * dimx + j];
    }
    /* The fold written to a device grid (overwritten, not added). */
    void reduce_device(float* d_output, int isMax = 0) { check(ske_reduce(e_, d_output, 1, isMax)); }

    /* The C ABI handle, for calls the reference class has no method for. */
    ske_engine handle() const { return e_; }

    /* Grid (src/skewEngine.cuh:222-247). */
    int dimx, dimy, N, dim_l;
    bool isGPU;
    int deviceId;
    /* The current sector (src/skewEngine.cuh:307-366), set by skew(). */
    int a = -1, sectorType = 0, newAngle = 0, offset = 0, skewHeight = 0, skewWidth = 0, dim_i = 0, dim_o = 0;
    double scale = 0.0, skewness = 0.0;
    float* d_skewInput = nullptr;
    float* d_skewOutput = nullptr;
    const int32_t* d_first = nullptr;
    const int32_t* d_last = nullptr;
    const int32_t* d_target = nullptr;
    const float* d_weight = nullptr;
    /* The operator: kernelcuda if set, else the built-in `algorithm`; `val` is
     * handed to it (POVh for kernelSDEM); `accum` is the deskew's mode. */
    cuda_operator kernelcuda = nullptr;
    int algorithm = KERNEL_SDEM;
    float val = 0.15f;
    int accum = SKE_ACCUM_REFERENCE;

private:
    static int trampoline(void* user, const ske_sector_view* v) {
        const skewEngine* self = static_cast<const skewEngine*>(user);
        return self->kernelcuda(v->skew_out, v->skew_in, v->geom.dim_i, v->geom.skew_height, v->last, v->first,
                                v->povh, v->geom.new_angle, v->stream);
    }
    ske_engine e_ = nullptr;
};

/* execute(skewAlgorithm) (src/main.cu:71-172) on one GPU: every sector of
 * [0, maxSector) through skew, the operator and deskew (the cepstrum with the
 * max encoding), then reduce into the host grid outD (added, as the
 * reference's threads add into it).  The whole loop runs as batched launches
 * (ske_run); the result is the reference's single-thread one. */
inline void execute(int skewAlgorithm, const float* inputD, float* outD, int dimx, int dimy, int maxSector = 180,
                    float val = 0.15f, int deviceId = 0) {
    ske_engine e = nullptr;
    check(ske_create(&e, dimx, dimy, deviceId, nullptr));
    ske_params p;
    ske_params_default(&p);
    p.max_sector = maxSector;
    p.povh = val;
    std::vector<float> fold((size_t)dimx * dimy);
    const int rc = ske_run(e, skewAlgorithm, inputD, 0, fold.data(), 0, &p);
    const std::string msg = rc == SKE_OK ? std::string() : std::string(ske_last_error());
    ske_destroy(e);
    if (rc != SKE_OK) throw error(rc, msg);
    const bool is_max = skewAlgorithm == KERNEL_CEPSTRUM;
    for (size_t i = 0; i < fold.size(); i++) {
        if (is_max)
            outD[i] = outD[i] > fold[i] ? outD[i] : fold[i];
        else
            outD[i] = outD[i] + fold[i];
    }
}

/* computeParams + skewShape (src/skewEngine.cuh:504-596) of one sector, on the
 * host: geometry, and first/last (skew_height entries each), target and
 * weight (dim_i entries each). */
struct sector_tables {
    ske_sector_geometry geom;
    std::vector<int32_t> first, last, target;
    std::vector<float> weight;
};

inline sector_tables sector_geometry(int dimx, int dimy, int angle) {
    sector_tables t;
    check(ske_geometry(dimx, dimy, angle, &t.geom, nullptr, nullptr, nullptr, nullptr));
    t.first.resize((size_t)t.geom.skew_height);
    t.last.resize((size_t)t.geom.skew_height);
    t.target.resize((size_t)t.geom.dim_i);
    t.weight.resize((size_t)t.geom.dim_i);
    check(ske_geometry(dimx, dimy, angle, &t.geom, t.first.data(), t.last.data(), t.target.data(), t.weight.data()));
    return t;
}

}  // namespace ske

#endif  // SKEWENGINE_HPP
