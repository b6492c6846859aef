// C ABI of the skew engine (include/skewengine.h): engine object, device
// buffers, the batched sector loop and the per-sector drop-in API.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <exception>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/skewengine.h"
#include "kernels.h"

using namespace ske;

namespace {

thread_local std::string t_last_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_last_error = buf;
    return code;
}

// A C++ exception from host code (std::bad_alloc when a request is too large
// for host memory) becomes an error status: none crosses the C ABI.
int host_failure(const std::exception& ex) { return fail(SKE_ERR_INVALID, "host: %s", ex.what()); }

#define SKE_CK(call)                                                                              \
    do {                                                                                          \
        cudaError_t _e = (call);                                                                  \
        if (_e != cudaSuccess) return fail(SKE_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(_e)); \
    } while (0)

#define SKE_TRY(expr)            \
    do {                         \
        int _rc = (expr);        \
        if (_rc != SKE_OK) return _rc; \
    } while (0)

std::mutex g_init_mutex;
std::vector<int> g_tables_ready;  // per device: SDEM constant tables uploaded

int ensure_device_tables(int device) {
    std::lock_guard<std::mutex> lock(g_init_mutex);
    if ((int)g_tables_ready.size() <= device) g_tables_ready.resize(device + 1, 0);
    if (g_tables_ready[device]) return SKE_OK;
    SKE_CK(sdem_init_tables());
    SKE_CK(cepstrum_f32_init_tables());
    if (lradon_f32_init_tables() != 0) return fail(SKE_ERR_CUDA, "local Radon float32 tables");
    g_tables_ready[device] = 1;
    return SKE_OK;
}

bool valid_kernel(int k) { return k >= SKE_KERNEL_SDEM && k <= SKE_KERNEL_LOCAL_RADON; }

// Allocation fault injection for tests (ske_inject_alloc_failure): the
// allocation this many allocations from now fails; negative = off.
std::atomic<int64_t> g_alloc_fail_in{-1};

bool injected_alloc_failure() {
    int64_t n = g_alloc_fail_in.load();
    while (n >= 0 && !g_alloc_fail_in.compare_exchange_weak(n, n - 1)) {
    }
    return n == 0;
}

template <typename T>
int dev_alloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) return SKE_OK;
    if (injected_alloc_failure()) return fail(SKE_ERR_CUDA, "injected device allocation failure");
    SKE_CK(cudaMalloc((void**)p, sizeof(T) * count));
    return SKE_OK;
}

int pinned_alloc(float** p, size_t count) {
    *p = nullptr;
    if (injected_alloc_failure()) return fail(SKE_ERR_CUDA, "injected pinned allocation failure");
    SKE_CK(cudaHostAlloc((void**)p, sizeof(float) * count, cudaHostAllocPortable));
    return SKE_OK;
}

struct ItemPlan {
    uint64_t* d_items = nullptr;
    int64_t n_items = 0;
    int max_row = 0;
    std::vector<uint64_t> h_items;  // host copy: the autotuner samples it
};

// Shape of the compacting sweep the autotuner chooses: level schedule
// (lvl0, then lvl1, then 64-step levels) and resident CTAs per SM (0 = all
// that fit).  Every shape gives the same results bit for bit; only the time
// differs.
struct SweepShape {
    int lvl0 = 64, lvl1 = 0, ctas = 0;
};

struct BatchPlan;
void destroy_batch_plan(BatchPlan* p);
struct ImagePlan;
void destroy_image_plan(ImagePlan* p);

struct ProfEntry {
    double ms = 0;
    int64_t launches = 0;
};

}  // namespace

int ske::set_last_error(int code, const char* msg) { return fail(code, "%s", msg); }

struct ske_engine_s {
    int dimx = 0, dimy = 0, device = 0, num_sms = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int64_t N = 0, len = 0, stride = 0;
    Geometry geo;
    DevGeometry dg{};
    SectorDesc* d_desc = nullptr;
    int32_t *d_target = nullptr, *d_first = nullptr, *d_last = nullptr;
    float* d_weight = nullptr;
    float *d_in = nullptr, *d_orient = nullptr, *d_acc = nullptr, *d_comp = nullptr, *d_out = nullptr;
    float *d_SI = nullptr, *d_SO = nullptr;
    int slots = 0;  // capacity of d_SI/d_SO in sectors
    double* d_P = nullptr;
    int64_t pstride = 0;  // complex doubles per slot
    int max_H2 = 1;
    double* d_tw = nullptr;
    int64_t* d_tw_off = nullptr;
    int64_t tw_off_host[32] = {0};
    int64_t lr_gauss_off = 0, lr_taper_off = 0;  // local Radon tables inside d_tw
    unsigned* d_counter = nullptr;
    int* d_status = nullptr;
    // Tensor maps of d_SO for the TMA-staged deskew, for the buffer they were
    // encoded for.
    DeskewMaps maps;
    const float* maps_so = nullptr;
    int maps_slots = 0;
    // Tensor maps of d_orient for the TMA-staged skew (encoded with the buffer).
    SkewMaps skew_maps;
    int4* d_lists = nullptr;  // survivor lists of the viewshed sweep
    size_t list_bytes = 0;
    float* h_pin = nullptr;
    std::map<std::vector<int>, ItemPlan> item_plans;
    // Per angle: every skewed row's valid range lies within dim_i (no row
    // overruns into the next, so each skewed cell belongs to one row at most).
    std::vector<char> rows_in_width;
    // per-sector API state
    bool prepared = false;
    int cur_angle = -1;
    bool kernel_ran = false;
    unsigned used = 0;
    int accum_mode = SKE_ACCUM_REFERENCE;
    // profiling
    bool prof = false;
    std::map<std::string, ProfEntry> prof_tot;
    struct Pending {
        std::string name;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> event_pool;
    int64_t launches = 0;
    // Batches of uneven grids: one cached child engine per other grid size.
    // A child borrows the parent's skew-buffer slots, Radon scratch and sweep
    // lists (the parent's stride holds the child's skewed grids) and owns the rest.
    ske_engine parent = nullptr;
    std::map<std::pair<int, int>, ske_engine> children;
    // Batched total-viewshed runs: the plan of the last batch (grids, angles,
    // waves, work lists, captured graphs), reused while the batch keeps its shape.
    BatchPlan* batch_plan = nullptr;
    ImagePlan* image_plan = nullptr;  // float32 cepstrum over batches of square images
    int flags = 0;           // ske_params.flags of the current run
    SweepShape last_shape;   // shape of the last compacting sweep launched
    SweepShape fixed_shape{0, 0, 0};  // ske_set_sweep_shape (lvl0 0: the autotuner decides)
    uint64_t* d_tune_items = nullptr;  // the autotuner's sample of a work list
    size_t tune_items_cap = 0;
};

namespace {

// Brackets a group of kernel launches for the profiler.
struct LaunchScope {
    ske_engine e;
    const char* name;
    cudaEvent_t a = nullptr, b = nullptr;
    int kernels;
    LaunchScope(ske_engine e_, const char* n, int k) : e(e_), name(n), kernels(k) {
        if (e->prof) {
            a = take();
            b = take();
            cudaEventRecord(a, e->stream);
        }
    }
    cudaEvent_t take() {
        if (!e->event_pool.empty()) {
            cudaEvent_t ev = e->event_pool.back();
            e->event_pool.pop_back();
            return ev;
        }
        cudaEvent_t ev;
        cudaEventCreate(&ev);
        return ev;
    }
    int done(cudaError_t err) {
        if (err != cudaSuccess) return fail(SKE_ERR_CUDA, "%s launch failed: %s", name, cudaGetErrorString(err));
        e->launches += kernels;
        if (e->prof) {
            cudaEventRecord(b, e->stream);
            e->pending.push_back({name, a, b});
            a = b = nullptr;
        }
        return SKE_OK;
    }
};

int flush_profile(ske_engine e) {
    if (e->pending.empty()) return SKE_OK;
    SKE_CK(cudaStreamSynchronize(e->stream));
    for (auto& p : e->pending) {
        float ms = 0;
        cudaEventElapsedTime(&ms, p.a, p.b);
        ProfEntry& t = e->prof_tot[p.name];
        t.ms += ms;
        t.launches += 1;
        e->event_pool.push_back(p.a);
        e->event_pool.push_back(p.b);
    }
    e->pending.clear();
    return SKE_OK;
}

int set_device(ske_engine e) {
    SKE_CK(cudaSetDevice(e->device));
    return SKE_OK;
}

bool is_pinned_host(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

// Host -> device copy of n floats, through the engine's pinned buffer unless the
// source is already page-locked.
int upload(ske_engine e, float* dst, const float* src, int64_t n) {
    if (is_pinned_host(src)) {
        SKE_CK(cudaMemcpyAsync(dst, src, sizeof(float) * n, cudaMemcpyHostToDevice, e->stream));
        return SKE_OK;
    }
    SKE_CK(cudaStreamSynchronize(e->stream));  // pinned buffer may still be in use
    memcpy(e->h_pin, src, sizeof(float) * n);
    SKE_CK(cudaMemcpyAsync(dst, e->h_pin, sizeof(float) * n, cudaMemcpyHostToDevice, e->stream));
    return SKE_OK;
}

int download(ske_engine e, float* dst, const float* src, int64_t n) {
    if (is_pinned_host(dst)) {
        SKE_CK(cudaMemcpyAsync(dst, src, sizeof(float) * n, cudaMemcpyDeviceToHost, e->stream));
        SKE_CK(cudaStreamSynchronize(e->stream));
        return SKE_OK;
    }
    SKE_CK(cudaMemcpyAsync(e->h_pin, src, sizeof(float) * n, cudaMemcpyDeviceToHost, e->stream));
    SKE_CK(cudaStreamSynchronize(e->stream));
    memcpy(dst, e->h_pin, sizeof(float) * n);
    return SKE_OK;
}

int check_status(ske_engine e) {
    int st = 0;
    SKE_CK(cudaMemcpyAsync(&st, e->d_status, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    SKE_CK(cudaStreamSynchronize(e->stream));
    if (st != 0) {
        cudaMemsetAsync(e->d_status, 0, sizeof(int), e->stream);
        return fail(SKE_ERR_DEVICE, "device status %d reported by a kernel", st);
    }
    return SKE_OK;
}

// Make room for `want` sector slots of skewed buffers (and Radon scratch).
int ensure_slots(ske_engine e, int want) {
    if (e->parent) {  // borrowed from the parent, which may grow them
        SKE_TRY(ensure_slots(e->parent, want));
        e->d_SI = e->parent->d_SI;
        e->d_SO = e->parent->d_SO;
        e->d_P = e->parent->d_P;
        e->slots = e->parent->slots;
        return SKE_OK;
    }
    if (want <= e->slots) return SKE_OK;
    SKE_CK(cudaStreamSynchronize(e->stream));
    cudaFree(e->d_SI);
    cudaFree(e->d_SO);
    cudaFree(e->d_P);
    e->d_SI = e->d_SO = nullptr;
    e->d_P = nullptr;
    e->slots = 0;
    SKE_TRY(dev_alloc(&e->d_SI, (size_t)e->stride * want));
    SKE_TRY(dev_alloc(&e->d_SO, (size_t)e->stride * want));
    SKE_TRY(dev_alloc(&e->d_P, (size_t)e->pstride * 2 * want));
    e->slots = want;
    return SKE_OK;
}

// Make room for `bytes` of survivor-list scratch for the viewshed sweep.
int ensure_lists(ske_engine e, size_t bytes) {
    if (e->parent) {
        SKE_TRY(ensure_lists(e->parent, bytes));
        e->d_lists = e->parent->d_lists;
        e->list_bytes = e->parent->list_bytes;
        return SKE_OK;
    }
    if (bytes <= e->list_bytes) return SKE_OK;
    SKE_CK(cudaStreamSynchronize(e->stream));
    cudaFree(e->d_lists);
    e->d_lists = nullptr;
    e->list_bytes = 0;
    SKE_TRY(dev_alloc(&e->d_lists, (bytes + sizeof(int4) - 1) / sizeof(int4)));
    e->list_bytes = bytes;
    return SKE_OK;
}

// Sectors per launch: as many as fit in a quarter of free memory (at most 180).
int batch_capacity(ske_engine e, int nangles) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        free_b = (size_t)1 << 30;
    }
    const size_t per_slot = sizeof(float) * 2 * (size_t)e->stride + sizeof(double) * 2 * (size_t)e->pstride;
    size_t budget = free_b / 4 + (size_t)e->slots * per_slot;
    int cap = (int)std::min<size_t>(budget / std::max<size_t>(per_slot, 1), (size_t)kMaxBatch);
    cap = std::max(cap, 1);
    return std::min(cap, nangles);
}

int get_items(ske_engine e, const Batch& b, ItemPlan** out) {
    std::vector<int> key(b.angle, b.angle + b.count);
    auto it = e->item_plans.find(key);
    if (it != e->item_plans.end()) {
        *out = &it->second;
        return SKE_OK;
    }
    ItemPlan plan;
    sdem_items(e->geo, b, plan.h_items, &plan.max_row);
    plan.n_items = (int64_t)plan.h_items.size();
    SKE_TRY(dev_alloc(&plan.d_items, plan.h_items.size()));
    if (!plan.h_items.empty())
        SKE_CK(cudaMemcpy(plan.d_items, plan.h_items.data(), sizeof(uint64_t) * plan.h_items.size(),
                          cudaMemcpyHostToDevice));
    auto ins = e->item_plans.emplace(key, std::move(plan));
    *out = &ins.first->second;
    return SKE_OK;
}

// ---- sweep autotuner --------------------------------------------------------
// The compacting sweep's speed depends on its level schedule (a short first
// level retires the many observers that see nothing far away sooner, for more
// retirement tests) and on how many CTAs share an SM (more warps hide latency,
// fewer leave each warp more L1).  The tuner times a few shapes on the actual
// work list (a strided sample of it beyond 2^20 rows) the first time a device
// meets rows of a given length class, and keeps the fastest for the process.
// Every shape writes the same bits.
std::mutex g_tune_mutex;
std::map<std::pair<int, int>, SweepShape> g_tuned;  // (device, max_row / 256) -> shape

int tune_sweep(ske_engine e, const SdemLaunch& base, const std::vector<uint64_t>& items, SweepShape* out) {
    *out = SweepShape();
    if (e->fixed_shape.lvl0 > 0) {
        *out = e->fixed_shape;
        return SKE_OK;
    }
    if (e->flags & SKE_FLAG_NO_TUNE) return SKE_OK;
    const auto key = std::make_pair(e->device, (base.max_row + 255) / 256);
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
        *out = it->second;
        return SKE_OK;
    }
    if (items.size() < (size_t)64 * e->num_sms) return SKE_OK;  // too little work to time; keep the default
    // The whole list up to 2^20 rows, else every stride-th row (which keeps the
    // longest-first length distribution).
    const size_t stride = std::max<size_t>(1, items.size() >> 20);
    std::vector<uint64_t> sample;
    sample.reserve(items.size() / stride + 1);
    for (size_t i = 0; i < items.size(); i += stride) sample.push_back(items[i]);
    if (sample.size() > e->tune_items_cap) {
        cudaFree(e->d_tune_items);
        e->d_tune_items = nullptr;
        e->tune_items_cap = 0;
        SKE_TRY(dev_alloc(&e->d_tune_items, sample.size()));
        e->tune_items_cap = sample.size();
    }
    SKE_CK(cudaMemcpyAsync(e->d_tune_items, sample.data(), sizeof(uint64_t) * sample.size(), cudaMemcpyHostToDevice,
                           e->stream));
    const int max_ctas = sdem_max_ctas_per_sm(base);
    const SweepShape sched[] = {{64, 0, 0}, {16, 48, 0}, {32, 0, 0}, {48, 0, 0}};
    std::vector<SweepShape> cands;
    for (const SweepShape& c : sched) {
        cands.push_back(c);
        if (max_ctas > 1) cands.push_back({c.lvl0, c.lvl1, max_ctas - 1});
    }
    if (max_ctas > 2) cands.push_back({32, 0, max_ctas - 2});
    cudaEvent_t ev[2];
    SKE_CK(cudaEventCreate(&ev[0]));
    SKE_CK(cudaEventCreate(&ev[1]));
    float best = 0.0f;
    SweepShape pick;
    int rc = SKE_OK;
    for (int rep = 0; rep < 2 && rc == SKE_OK; rep++) {  // the second pass is the one compared
        for (const SweepShape& c : cands) {
            SdemLaunch a = base;
            a.items = e->d_tune_items;
            a.n_items = (int64_t)sample.size();
            a.lvl0 = c.lvl0;
            a.lvl1 = c.lvl1;
            a.ctas_per_sm = c.ctas;
            cudaError_t err = cudaEventRecord(ev[0], e->stream);
            if (err == cudaSuccess) err = launch_sdem(a, e->num_sms, e->stream);
            if (err == cudaSuccess) err = cudaEventRecord(ev[1], e->stream);
            if (err == cudaSuccess) err = cudaEventSynchronize(ev[1]);
            float ms = 0.0f;
            if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, ev[0], ev[1]);
            if (err != cudaSuccess) {
                rc = fail(SKE_ERR_CUDA, "sweep autotuner: %s", cudaGetErrorString(err));
                break;
            }
            e->launches += 1;
            if (rep == 1 && (best == 0.0f || ms < best)) {
                best = ms;
                pick = c;
            }
        }
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    if (rc != SKE_OK) return rc;
    g_tuned[key] = pick;
    *out = pick;
    return SKE_OK;
}

// rows_only (Radon, sectors whose rows stay within dim_i): the row sums gather
// the skewed cells from the oriented input (no skew needed) and the
// back-projection into SO is skipped.
// so_masked (batched total viewshed, every sector's rows within dim_i): SO is
// not zeroed first; the sweep writes every valid cell and the deskew reads the
// others as zero.
int run_operator(ske_engine e, int kernel, const Batch& b, float povh, int counts_only, bool rows_only = false,
                 bool so_masked = false) {
    switch (kernel) {
        case SKE_KERNEL_SDEM: {
            ItemPlan* plan = nullptr;
            SKE_TRY(get_items(e, b, &plan));
            if (!so_masked) SKE_CK(cudaMemsetAsync(e->d_SO, 0, sizeof(float) * e->stride * b.count, e->stream));
            SKE_TRY(ensure_lists(e, sdem_list_bytes(std::max(plan->max_row, 1), e->num_sms)));
            SdemLaunch a;
            a.g = e->dg;
            a.b = b;
            a.SI = e->d_SI;
            a.SO = e->d_SO;
            a.stride = e->stride;
            a.items = plan->d_items;
            a.n_items = plan->n_items;
            a.counter = e->d_counter;
            a.povh = povh;
            a.max_row = std::max(plan->max_row, 1);
            a.counts_only = counts_only;
            a.status = e->d_status;
            a.lists = e->d_lists;
            a.list_bytes = e->list_bytes;
            SweepShape shape;
            SKE_TRY(tune_sweep(e, a, plan->h_items, &shape));
            a.lvl0 = shape.lvl0;
            a.lvl1 = shape.lvl1;
            a.ctas_per_sm = shape.ctas;
            e->last_shape = shape;
            LaunchScope ls(e, "sdem_sweep", plan->n_items > 0 ? 1 : 0);
            return ls.done(launch_sdem(a, e->num_sms, e->stream));
        }
        case SKE_KERNEL_RADON: {
            const bool f32 = (e->flags & SKE_FLAG_RADON_F32) != 0;
            LaunchScope ls(e, "radon", radon_launches(rows_only, e->max_H2, f32));
            return ls.done(launch_radon(e->dg, b, e->d_SI, e->d_SO, e->stride, e->len, e->d_P, e->pstride, e->d_tw,
                                        e->d_tw_off, e->max_H2, e->stream, !rows_only,
                                        rows_only ? e->d_orient : nullptr, e->N, f32));
        }
        case SKE_KERNEL_LOCAL_RADON: {
            SKE_CK(cudaMemsetAsync(e->d_SO, 0, sizeof(float) * e->stride * b.count, e->stream));
            LaunchScope ls(e, "local_radon", 1);
            if (e->flags & SKE_FLAG_LOCAL_RADON_F32)
                return ls.done(launch_local_radon_f32(e->dg, b, e->d_SI, e->d_SO, e->stride, e->geo.max_H,
                                                      std::max(e->dimx, e->dimy), e->d_tw + e->lr_gauss_off,
                                                      e->d_tw + e->lr_taper_off, e->stream));
            return ls.done(launch_local_radon(e->dg, b, e->d_SI, e->d_SO, e->stride, e->geo.max_H,
                                              std::max(e->dimx, e->dimy), e->d_tw + e->lr_gauss_off,
                                              e->d_tw + e->lr_taper_off, e->d_tw + e->tw_off_host[6], e->stream));
        }
        case SKE_KERNEL_CEPSTRUM: {
            LaunchScope ls(e, "cepstrum", 1);
            return ls.done(launch_cepstrum(e->dg, b, e->d_SI, e->d_SO, e->stride, e->len, e->d_tw + e->tw_off_host[6],
                                           e->d_tw + e->tw_off_host[5], e->stream));
        }
        default: {
            LaunchScope ls(e, "identity", 1);
            return ls.done(launch_identity(e->dg, b, e->d_SI, e->d_SO, e->stride, e->len, e->stream));
        }
    }
}

// zero_tail false (batched runs): sectors whose rows stay within dim_i leave
// the slot past H*dim_i unwritten, since no operator of the batch reads it.
int run_skew(ske_engine e, const Batch& b, bool zero_tail = true) {
    LaunchScope ls(e, "skew", 1);
    return ls.done(launch_skew_staged(e->dg, b, e->d_orient, e->N, e->d_SI, e->stride, e->len,
                                      std::max(e->dimx, e->dimy), e->geo.max_H, e->stream, zero_tail, &e->skew_maps,
                                      e->d_status));
}

// rows_from_p: the batch is Radon sectors whose back-projection was skipped;
// the deskew reads their filtered row values from the Radon scratch.
int run_deskew(ske_engine e, const Batch& b, int is_max, int accum, bool rows_from_p = false, bool so_masked = false) {
    TypeLists tl;
    memset(&tl, 0, sizeof(tl));
    for (int s = 0; s < b.count; s++) {
        const int t = e->geo.desc[b.angle[s]].type;
        tl.slot[t][tl.count[t]] = s;
        tl.angle[t][tl.count[t]] = b.angle[s];
        tl.count[t]++;
        e->used |= 1u << t;
    }
    if (e->maps_so != e->d_SO || e->maps_slots != e->slots) {
        encode_band_maps(&e->maps, e->d_SO, e->stride, e->slots, e->dimx, e->dimy);  // ok = false: plain staging
        e->maps_so = e->d_SO;
        e->maps_slots = e->slots;
    }
    LaunchScope ls(e, "deskew", 1);
    if (is_max) return ls.done(launch_deskew_max(e->dg, tl, e->d_SO, e->stride, e->d_acc, e->dimx, e->dimy, e->stream));
    return ls.done(launch_deskew_add(e->dg, tl, e->d_SO, e->stride, e->d_acc, e->d_comp, e->dimx, e->dimy, accum,
                                     e->stream, rows_from_p ? reinterpret_cast<const cd*>(e->d_P) : nullptr,
                                     e->pstride, so_masked, &e->maps, e->d_status));
}

int run_prepare(ske_engine e, const float* input, int on_device) {
    const float* src = input;
    if (!on_device) {
        SKE_TRY(upload(e, e->d_in, input, e->N));
        src = e->d_in;
    }
    {
        LaunchScope ls(e, "prepare", 1);
        SKE_TRY(ls.done(launch_prepare(src, e->d_orient, e->dimx, e->dimy, e->stream)));
    }
    SKE_CK(cudaMemsetAsync(e->d_acc, 0, sizeof(float) * 4 * e->N, e->stream));
    SKE_CK(cudaMemsetAsync(e->d_comp, 0, sizeof(float) * 4 * e->N, e->stream));
    e->used = 0;
    e->prepared = true;
    e->cur_angle = -1;
    e->kernel_ran = false;
    return SKE_OK;
}

int run_reduce(ske_engine e, float* output, int on_device, int is_max, int accum) {
    float* dst = on_device ? output : e->d_out;
    {
        LaunchScope ls(e, "reduce", 1);
        SKE_TRY(ls.done(launch_reduce(e->d_acc, e->d_comp, e->used, dst, e->dimx, e->dimy, is_max, accum, e->stream)));
    }
    if (!on_device) SKE_TRY(download(e, output, e->d_out, e->N));
    return check_status(e);
}

int validate_params(const ske_params* p, ske_params* out) {
    ske_params_default(out);
    if (p) *out = *p;
    if (out->max_sector < 1 || out->max_sector > kMaxSectors)
        return fail(SKE_ERR_INVALID, "max_sector %d outside [1,180]", out->max_sector);
    if (out->accum != SKE_ACCUM_REFERENCE && out->accum != SKE_ACCUM_KAHAN)
        return fail(SKE_ERR_INVALID, "unknown accumulation mode %d", out->accum);
    return SKE_OK;
}

// Accumulator state a run starts from instead of zero (checkpoint/resume).
struct StartState {
    const float* acc;   // 4 x N per-type accumulators
    const float* comp;  // 4 x N Kahan compensations (Kahan mode only)
    uint32_t used;      // types that already received a sector
    int on_device;
};

int load_state(ske_engine e, const StartState& st, int accum) {
    for (int t = 0; t < 4; t++) {
        const int64_t off = (int64_t)t * e->N;
        if (st.on_device) {
            SKE_CK(cudaMemcpyAsync(e->d_acc + off, st.acc + off, sizeof(float) * e->N, cudaMemcpyDeviceToDevice,
                                   e->stream));
            if (accum == SKE_ACCUM_KAHAN)
                SKE_CK(cudaMemcpyAsync(e->d_comp + off, st.comp + off, sizeof(float) * e->N,
                                       cudaMemcpyDeviceToDevice, e->stream));
        } else {
            SKE_TRY(upload(e, e->d_acc + off, st.acc + off, e->N));
            if (accum == SKE_ACCUM_KAHAN) SKE_TRY(upload(e, e->d_comp + off, st.comp + off, e->N));
        }
    }
    e->used = st.used & 0xfu;
    return SKE_OK;
}

// Prepare + every listed sector (skew, operator, deskew) into the accumulators,
// which start from zero or, with `start`, from a saved state.
int accumulate_angles(ske_engine e, int kernel, const float* input, int input_on_device, const int32_t* angles,
                      int nangles, const ske_params* p, ske_params* prm, const StartState* start = nullptr) {
    if (!e) return fail(SKE_ERR_INVALID, "null engine");
    if (!valid_kernel(kernel)) return fail(SKE_ERR_INVALID, "unknown kernel %d", kernel);
    if (!input) return fail(SKE_ERR_INVALID, "null input");
    if (nangles < 0 || (nangles > 0 && !angles)) return fail(SKE_ERR_INVALID, "bad angle list");
    for (int i = 0; i < nangles; i++)
        if (angles[i] < 0 || angles[i] >= kMaxSectors) return fail(SKE_ERR_INVALID, "angle %d outside [0,180)", angles[i]);
    SKE_TRY(validate_params(p, prm));
    SKE_TRY(set_device(e));
    e->flags = prm->flags;
    const int is_max = kernel == SKE_KERNEL_CEPSTRUM;
    SKE_TRY(run_prepare(e, input, input_on_device));
    if (start) {
        if (!start->acc || (prm->accum == SKE_ACCUM_KAHAN && !start->comp))
            return fail(SKE_ERR_INVALID, "null accumulator state");
        SKE_TRY(load_state(e, *start, prm->accum));
    }
    e->accum_mode = prm->accum;
    if (nangles == 0) return SKE_OK;
    const int cap = batch_capacity(e, nangles);
    SKE_TRY(ensure_slots(e, cap));
    for (int s0 = 0; s0 < nangles; s0 += cap) {
        Batch b;
        b.count = std::min(cap, nangles - s0);
        for (int s = 0; s < b.count; s++) b.angle[s] = angles[s0 + s];
        // Radon sectors whose rows stay within their width: the row sums gather
        // the skewed cells themselves and the deskew reads the filtered row
        // values, so neither the skew nor the back-projection runs.
        bool in_width = true;
        for (int s = 0; s < b.count; s++) in_width = in_width && e->rows_in_width[b.angle[s]] != 0;
        const bool rows_only = kernel == SKE_KERNEL_RADON && in_width;
        const bool so_masked = kernel == SKE_KERNEL_SDEM && in_width;
        if (!rows_only) SKE_TRY(run_skew(e, b, false));
        SKE_TRY(run_operator(e, kernel, b, prm->povh, 0, rows_only, so_masked));
        SKE_TRY(run_deskew(e, b, is_max, prm->accum, rows_only, so_masked));
    }
    e->accum_mode = prm->accum;
    return SKE_OK;
}

int run_images_f32(ske_engine e, int count, int dim, const float* const* inputs, int in_dev, float* const* outputs,
                   int out_dev, const int32_t* angles, int nangles);

int run_angle_list(ske_engine e, int kernel, const float* input, int input_on_device, float* output,
                   int output_on_device, const int32_t* angles, int nangles, const ske_params* p) {
    if (!output) return fail(SKE_ERR_INVALID, "null output");
    if (nangles < 1) return fail(SKE_ERR_INVALID, "empty angle list");
    if (e && kernel == SKE_KERNEL_CEPSTRUM && p && (p->flags & SKE_FLAG_CEPSTRUM_F32) && e->dimx == e->dimy) {
        if (!input) return fail(SKE_ERR_INVALID, "null input");
        for (int i = 0; i < nangles; i++)
            if (!angles || angles[i] < 0 || angles[i] >= kMaxSectors) return fail(SKE_ERR_INVALID, "bad angle list");
        ske_params chk;
        SKE_TRY(validate_params(p, &chk));
        SKE_TRY(set_device(e));
        e->flags = chk.flags;
        return run_images_f32(e, 1, e->dimx, &input, input_on_device, &output, output_on_device, angles, nangles);
    }
    ske_params prm;
    SKE_TRY(accumulate_angles(e, kernel, input, input_on_device, angles, nangles, p, &prm));
    SKE_TRY(run_reduce(e, output, output_on_device, kernel == SKE_KERNEL_CEPSTRUM, prm.accum));
    e->prepared = false;  // the accumulators now hold this run
    return SKE_OK;
}

// ---- batched total viewshed over grids of uneven size -------------------------
// A batch plan holds, per grid size, the device geometry and the compact-row
// offsets; per grid, its orientation, accumulator and staging buffers; and the
// batch split into waves whose skewed rows (compact) fit the device memory
// budget.  Each wave runs as five launches over all of its grids and sectors:
// orientations, skew, sweep, deskew, fold (captured as a CUDA graph after its
// first run).  Grids too large for a wave of their own, or with sectors whose
// rows leave dim_i, run through the per-grid engine path instead.

struct GridGeo {
    int dimx = 0, dimy = 0;
    Geometry geo;
    std::vector<int32_t> rowoff;  // per skewed row: start within its sector's compact rows
    std::vector<int4> rowtab;     // per skewed row: {first, last, rowoff, 0}
    std::vector<int64_t> cells;   // per angle: valid cells (compact size)
    SectorDesc* d_desc = nullptr;
    int32_t *d_target = nullptr, *d_first = nullptr, *d_last = nullptr, *d_rowoff = nullptr;
    float* d_weight = nullptr;
    int4* d_rowtab = nullptr;
};

struct BatchWave {
    std::vector<int> grids;         // plan grid indices
    std::vector<BatchGrid> h_grids; // host copies of the wave's grid table (in/out set per call)
    BatchGrid* d_grids = nullptr;
    BatchSector* d_sectors = nullptr;
    SectorRef* d_refs = nullptr;
    int64_t* d_prep = nullptr;
    int64_t* d_tiles = nullptr;
    int64_t* d_skew = nullptr;
    uint64_t* d_items = nullptr;
    std::vector<uint64_t> items;
    int64_t n_items = 0, prep_blocks = 0, tiles = 0, cells = 0, skew_blocks = 0;
    int max_row = 0;
    BatchTables tables{};
    cudaGraphExec_t graph = nullptr;
    bool graph_failed = false;
    const void* graph_lists = nullptr;  // survivor-list scratch the graph was captured with
};

struct BatchPlan {
    std::vector<int> dimx, dimy, angles;
    int accum = 0;
    std::map<std::pair<int, int>, GridGeo*> geos;
    std::vector<GridGeo*> grid_geo;
    std::vector<int64_t> grid_off, io_off;  // per grid: offsets in d_grid_pool (12 n) and d_io_pool (2 n)
    float* d_grid_pool = nullptr;
    float* d_io_pool = nullptr;
    float *d_SI = nullptr, *d_SO = nullptr;
    std::vector<BatchWave> waves;
    std::vector<int> fallback;  // grids run through the per-grid engine path
    bool tuned = false;
    SweepShape shape;
};

void free_wave(BatchWave& w) {
    if (w.graph) cudaGraphExecDestroy(w.graph);
    void* bufs[] = {w.d_grids, w.d_sectors, w.d_refs, w.d_prep, w.d_tiles, w.d_skew, w.d_items};
    for (void* b : bufs) cudaFree(b);
    w = BatchWave();
}

void destroy_batch_plan(BatchPlan* p) {
    if (!p) return;
    for (BatchWave& w : p->waves) free_wave(w);
    for (auto& kv : p->geos) {
        GridGeo* g = kv.second;
        void* bufs[] = {g->d_desc, g->d_target, g->d_first, g->d_last, g->d_rowoff, g->d_weight, g->d_rowtab};
        for (void* b : bufs) cudaFree(b);
        delete g;
    }
    cudaFree(p->d_grid_pool);
    cudaFree(p->d_io_pool);
    cudaFree(p->d_SI);
    cudaFree(p->d_SO);
    delete p;
}

template <typename T>
int upload_vec(T** d, const std::vector<T>& h) {
    SKE_TRY(dev_alloc(d, h.size()));
    if (!h.empty()) SKE_CK(cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
    return SKE_OK;
}

int make_grid_geo(int dimx, int dimy, GridGeo** out) {
    GridGeo* g = new GridGeo();
    *out = g;
    g->dimx = dimx;
    g->dimy = dimy;
    const std::string why = build_geometry(dimx, dimy, g->geo);
    if (!why.empty()) return fail(SKE_ERR_INVALID, "sector geometry of %dx%d: %s", dimx, dimy, why.c_str());
    g->rowoff.assign(g->geo.first.size(), 0);
    g->rowtab.assign(g->geo.first.size(), make_int4(0, 0, 0, 0));
    g->cells.assign(g->geo.desc.size(), 0);
    for (size_t a = 0; a < g->geo.desc.size(); a++) {
        SectorDesc& d = g->geo.desc[a];
        int64_t c = 0;
        d.in_width = 1;
        for (int r = 0; r < d.H; r++) {
            const int64_t k = d.row_off + r;
            g->rowoff[k] = (int32_t)c;
            g->rowtab[k] = make_int4(g->geo.first[k], g->geo.last[k], (int)c, 0);
            const int L = g->geo.last[k] - g->geo.first[k];
            if (L > 0) c += L;
            if (g->geo.last[k] > d.dim_i) d.in_width = 0;
        }
        g->cells[a] = c;
    }
    SKE_TRY(upload_vec(&g->d_desc, g->geo.desc));
    SKE_TRY(upload_vec(&g->d_target, g->geo.target));
    SKE_TRY(upload_vec(&g->d_weight, g->geo.weight));
    SKE_TRY(upload_vec(&g->d_first, g->geo.first));
    SKE_TRY(upload_vec(&g->d_last, g->geo.last));
    SKE_TRY(upload_vec(&g->d_rowoff, g->rowoff));
    SKE_TRY(upload_vec(&g->d_rowtab, g->rowtab));
    return SKE_OK;
}

// Tables of one wave: its sectors in (grid, angle-list) order, the per-(grid,
// type) accumulation order, the prepare/fold and deskew block ranges, and the
// work list (every valid row, longest first).
int build_wave(BatchPlan* p, BatchWave& w) {
    std::vector<BatchSector> secs;
    std::vector<SectorRef> refs;
    std::vector<int64_t> prep(1, 0), tiles(1, 0), skew(1, 0);
    int64_t cells = 0;
    int lmax = 0;
    w.h_grids.clear();
    for (size_t li = 0; li < w.grids.size(); li++) {
        const int gi = w.grids[li];
        const GridGeo* gg = p->grid_geo[gi];
        BatchGrid G{};
        G.dimx = gg->dimx;
        G.dimy = gg->dimy;
        G.n = (int64_t)gg->dimx * gg->dimy;
        float* base = p->d_grid_pool + p->grid_off[gi];
        G.orient = base;
        G.acc = base + 4 * G.n;
        G.comp = base + 8 * G.n;
        G.desc = gg->d_desc;
        G.target = gg->d_target;
        G.weight = gg->d_weight;
        G.first = gg->d_first;
        G.last = gg->d_last;
        G.rowoff = gg->d_rowoff;
        G.rowtab = gg->d_rowtab;
        const int s0 = (int)secs.size();
        for (int a : p->angles) {
            secs.push_back(BatchSector{(int)li, a, cells});
            cells += gg->cells[a];
            const SectorDesc& d = gg->geo.desc[a];
            skew.push_back(skew.back() + batch_skew_blocks(d.dim_i, d.H));
            for (int r = 0; r < d.H; r++)
                lmax = std::max(lmax, gg->geo.last[d.row_off + r] - gg->geo.first[d.row_off + r]);
        }
        for (int t = 0; t < 4; t++) {
            G.ts_start[t] = (int)refs.size();
            for (int s = s0; s < (int)secs.size(); s++) {
                const SectorDesc& d = gg->geo.desc[secs[s].angle];
                if (d.type == t) refs.push_back(SectorRef{secs[s].cells, d.col_off, d.row_off, d.H, d.angle});
            }
            G.ts_count[t] = (int)refs.size() - G.ts_start[t];
            if (G.ts_count[t] > 0) G.used |= 1u << t;
            tiles.push_back(tiles.back() + (G.ts_count[t] > 0 ? batch_deskew_tiles(G.dimx, G.dimy, t) : 0));
        }
        prep.push_back(prep.back() + batch_prep_blocks(G.dimx, G.dimy));
        w.h_grids.push_back(G);
    }
    // Work list: counting sort of rows by length, longest first.
    std::vector<int64_t> start(lmax + 2, 0);
    for (const BatchSector& bs : secs) {
        const GridGeo* gg = p->grid_geo[w.grids[bs.grid]];
        const SectorDesc& d = gg->geo.desc[bs.angle];
        for (int r = 0; r < d.H; r++) {
            const int L = gg->geo.last[d.row_off + r] - gg->geo.first[d.row_off + r];
            if (L > 0) start[L]++;
        }
    }
    int64_t total = 0;
    for (int L = lmax; L >= 1; L--) {
        const int64_t c = start[L];
        start[L] = total;
        total += c;
    }
    w.items.assign(total, 0);
    for (size_t si = 0; si < secs.size(); si++) {
        const GridGeo* gg = p->grid_geo[w.grids[secs[si].grid]];
        const SectorDesc& d = gg->geo.desc[secs[si].angle];
        for (int r = 0; r < d.H; r++) {
            const int L = gg->geo.last[d.row_off + r] - gg->geo.first[d.row_off + r];
            if (L > 0) w.items[start[L]++] = batch_item((int)si, r);
        }
    }
    w.n_items = total;
    w.max_row = lmax;
    w.cells = cells;
    w.prep_blocks = prep.back();
    w.tiles = tiles.back();
    w.skew_blocks = skew.back();
    SKE_TRY(upload_vec(&w.d_grids, w.h_grids));
    SKE_TRY(upload_vec(&w.d_sectors, secs));
    SKE_TRY(upload_vec(&w.d_refs, refs));
    SKE_TRY(upload_vec(&w.d_prep, prep));
    SKE_TRY(upload_vec(&w.d_tiles, tiles));
    SKE_TRY(upload_vec(&w.d_skew, skew));
    SKE_TRY(upload_vec(&w.d_items, w.items));
    w.tables = BatchTables{w.d_grids, w.d_sectors, w.d_refs,  w.d_prep, w.d_tiles,
                           w.d_skew,  (int)w.grids.size(), (int)secs.size()};
    return SKE_OK;
}

bool same_plan(const BatchPlan* p, int count, const int32_t* dimx, const int32_t* dimy, const int32_t* angles,
               int nangles, int accum) {
    if (!p || (int)p->dimx.size() != count || (int)p->angles.size() != nangles || p->accum != accum) return false;
    for (int i = 0; i < count; i++)
        if (p->dimx[i] != dimx[i] || p->dimy[i] != dimy[i]) return false;
    for (int i = 0; i < nangles; i++)
        if (p->angles[i] != angles[i]) return false;
    return true;
}

int build_batch_plan(ske_engine e, int count, const int32_t* dimx, const int32_t* dimy, const int32_t* angles,
                     int nangles, int accum, BatchPlan** out) {
    BatchPlan* p = new BatchPlan();
    *out = p;
    p->dimx.assign(dimx, dimx + count);
    p->dimy.assign(dimy, dimy + count);
    p->angles.assign(angles, angles + nangles);
    p->accum = accum;
    int64_t grid_floats = 0, io_floats = 0;
    std::vector<char> eligible(count, 1);
    for (int i = 0; i < count; i++) {
        const auto key = std::make_pair((int)dimx[i], (int)dimy[i]);
        auto it = p->geos.find(key);
        GridGeo* gg = nullptr;
        if (it == p->geos.end()) {
            const int rc = make_grid_geo(dimx[i], dimy[i], &gg);
            p->geos[key] = gg;
            if (rc != SKE_OK) return rc;
        } else {
            gg = it->second;
        }
        p->grid_geo.push_back(gg);
        for (int k = 0; k < nangles; k++)
            if (!gg->geo.desc[angles[k]].in_width) eligible[i] = 0;
        const int64_t n = (int64_t)dimx[i] * dimy[i];
        p->grid_off.push_back(grid_floats);
        p->io_off.push_back(io_floats);
        if (eligible[i]) {
            grid_floats += 12 * n;
            io_floats += 2 * n;
        }
    }
    SKE_TRY(dev_alloc(&p->d_grid_pool, (size_t)grid_floats));
    SKE_TRY(dev_alloc(&p->d_io_pool, (size_t)io_floats));
    // Memory budget of a wave's compact skewed input and output (8 bytes per
    // valid cell), after the plan's buffers, the sweep's survivor lists and a
    // reserve for work lists and tables.
    int lmax_all = 1;
    for (int i = 0; i < count; i++) lmax_all = std::max(lmax_all, std::max((int)dimx[i], (int)dimy[i]));
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        free_b = (size_t)4 << 30;
    }
    const size_t lists = sdem_list_bytes(lmax_all, e->num_sms);
    const size_t have_lists = e->parent ? 0 : e->list_bytes;
    const size_t reserve = (lists > have_lists ? lists - have_lists : 0) + ((size_t)2 << 30);
    const int64_t budget = free_b > reserve ? (int64_t)((free_b - reserve) * 0.8) : 0;
    const int64_t cap_cells = budget / 8;
    int64_t wave_cells = 0;
    BatchWave cur;
    for (int i = 0; i < count; i++) {
        if (!eligible[i]) {
            p->fallback.push_back(i);
            continue;
        }
        int64_t c = 0;
        for (int k = 0; k < nangles; k++) c += p->grid_geo[i]->cells[angles[k]];
        if (c > cap_cells) {  // not even alone: the per-grid path batches its sectors itself
            p->fallback.push_back(i);
            continue;
        }
        if (!cur.grids.empty() && wave_cells + c > cap_cells) {
            p->waves.push_back(std::move(cur));
            cur = BatchWave();
            wave_cells = 0;
        }
        cur.grids.push_back(i);
        wave_cells += c;
    }
    if (!cur.grids.empty()) p->waves.push_back(std::move(cur));
    int64_t pool = 0;
    for (BatchWave& w : p->waves) {
        SKE_TRY(build_wave(p, w));
        pool = std::max(pool, w.cells);
    }
    SKE_TRY(dev_alloc(&p->d_SI, (size_t)pool));
    SKE_TRY(dev_alloc(&p->d_SO, (size_t)pool));
    return SKE_OK;
}

// The five launches of one wave, in stream order.
int launch_wave(ske_engine e, BatchPlan* p, BatchWave& w, float povh) {
    const BatchTables& t = w.tables;
    {
        LaunchScope ls(e, "prepare", 1);
        SKE_TRY(ls.done(launch_prepare_batch(t, w.prep_blocks, e->stream)));
    }
    {
        LaunchScope ls(e, "skew", 1);
        SKE_TRY(ls.done(launch_skew_batch(t, w.skew_blocks, p->d_SI, e->stream)));
    }
    SdemLaunch a;
    memset(&a.g, 0, sizeof(a.g));
    a.b.count = 0;
    a.SI = p->d_SI;
    a.SO = p->d_SO;
    a.stride = 0;
    a.items = w.d_items;
    a.n_items = w.n_items;
    a.counter = e->d_counter;
    a.povh = povh;
    a.max_row = std::max(w.max_row, 1);
    a.counts_only = 0;
    a.status = e->d_status;
    a.lists = e->d_lists;
    a.list_bytes = e->list_bytes;
    a.batched = 1;
    a.bt = t;
    a.lvl0 = p->shape.lvl0;
    a.lvl1 = p->shape.lvl1;
    a.ctas_per_sm = p->shape.ctas;
    {
        LaunchScope ls(e, "sdem_sweep", w.n_items > 0 ? 1 : 0);
        SKE_TRY(ls.done(launch_sdem(a, e->num_sms, e->stream)));
    }
    {
        LaunchScope ls(e, "deskew", 1);
        SKE_TRY(ls.done(launch_deskew_batch(t, w.tiles, p->d_SO, p->accum, e->stream)));
    }
    LaunchScope ls(e, "reduce", 1);
    return ls.done(launch_reduce_batch(t, w.prep_blocks, p->accum, e->stream));
}

// Tunes the sweep on the first wave (after its skew), once per plan.
int tune_batch(ske_engine e, BatchPlan* p, BatchWave& w, float povh) {
    if (p->tuned) return SKE_OK;
    SdemLaunch a;
    memset(&a.g, 0, sizeof(a.g));
    a.b.count = 0;
    a.SI = p->d_SI;
    a.SO = p->d_SO;
    a.stride = 0;
    a.counter = e->d_counter;
    a.povh = povh;
    a.max_row = std::max(w.max_row, 1);
    a.counts_only = 0;
    a.status = e->d_status;
    a.lists = e->d_lists;
    a.list_bytes = e->list_bytes;
    a.batched = 1;
    a.bt = w.tables;
    SKE_TRY(tune_sweep(e, a, w.items, &p->shape));
    p->tuned = true;
    e->last_shape = p->shape;
    return SKE_OK;
}

int run_wave(ske_engine e, BatchPlan* p, BatchWave& w, float povh, const float* const* inputs, int in_dev,
             float* const* outputs, int out_dev) {
    for (size_t li = 0; li < w.grids.size(); li++) {
        const int gi = w.grids[li];
        BatchGrid& G = w.h_grids[li];
        float* io = p->d_io_pool + p->io_off[gi];
        if (in_dev) {
            G.in = inputs[gi];
        } else {
            SKE_CK(cudaMemcpyAsync(io, inputs[gi], sizeof(float) * G.n, cudaMemcpyHostToDevice, e->stream));
            G.in = io;
        }
        G.out = out_dev ? outputs[gi] : io + G.n;
    }
    SKE_CK(cudaMemcpyAsync(w.d_grids, w.h_grids.data(), sizeof(BatchGrid) * w.h_grids.size(), cudaMemcpyHostToDevice,
                           e->stream));
    SKE_TRY(ensure_lists(e, sdem_list_bytes(std::max(w.max_row, 1), e->num_sms)));
    if (w.graph && w.graph_lists != (const void*)e->d_lists) {  // the lists moved: capture again
        cudaGraphExecDestroy(w.graph);
        w.graph = nullptr;
    }
    if (w.graph && !e->prof) {
        SKE_CK(cudaGraphLaunch(w.graph, e->stream));
        e->launches += 5;
    } else if (!p->tuned && !(e->flags & SKE_FLAG_NO_TUNE)) {
        // First run: orientations and skew, tune the sweep on them, then the rest.
        const BatchTables& t = w.tables;
        {
            LaunchScope ls(e, "prepare", 1);
            SKE_TRY(ls.done(launch_prepare_batch(t, w.prep_blocks, e->stream)));
        }
        {
            LaunchScope ls(e, "skew", 1);
            SKE_TRY(ls.done(launch_skew_batch(t, w.skew_blocks, p->d_SI, e->stream)));
        }
        SKE_TRY(tune_batch(e, p, w, povh));
        SKE_TRY(launch_wave(e, p, w, povh));  // again from the orientations (the tuner wrote parts of SO)
    } else {
        p->tuned = true;
        SKE_TRY(launch_wave(e, p, w, povh));
    }
    if (!w.graph && !w.graph_failed && !(e->flags & SKE_FLAG_NO_GRAPH) && !e->prof) {
        // Capture the wave's launches for the next calls (nothing runs now).
        cudaGraph_t g = nullptr;
        const int64_t before = e->launches;
        cudaError_t err = cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeRelaxed);
        int rc = SKE_OK;
        if (err == cudaSuccess) {
            rc = launch_wave(e, p, w, povh);
            err = cudaStreamEndCapture(e->stream, &g);
        }
        e->launches = before;
        if (err == cudaSuccess && rc == SKE_OK && g) err = cudaGraphInstantiate(&w.graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (err != cudaSuccess || rc != SKE_OK || !w.graph) {
            cudaGetLastError();
            if (w.graph) cudaGraphExecDestroy(w.graph);
            w.graph = nullptr;
            w.graph_failed = true;
        } else {
            w.graph_lists = e->d_lists;
        }
    }
    if (!out_dev)
        for (size_t li = 0; li < w.grids.size(); li++) {
            const BatchGrid& G = w.h_grids[li];
            SKE_CK(cudaMemcpyAsync(outputs[w.grids[li]], G.out, sizeof(float) * G.n, cudaMemcpyDeviceToHost,
                                   e->stream));
        }
    return SKE_OK;
}

// ---- float32 cepstrum over batches of square images --------------------------
// Every image of a batch has the same side; per wave of images (as many as the
// memory budget holds) three launches: orientations, the fused float32
// cepstrum sector loop (k_cepstrum_f32.cu) and the max fold.

struct ImagePlan {
    int dim = 0, count = 0, wave = 0;
    std::vector<int> angles;
    GridGeo* geo = nullptr;
    TypeLists tl;
    unsigned used = 0;
    float* d_pool = nullptr;  // per wave slot: orientations 4n + accumulators 4n
    float* d_io = nullptr;    // per wave slot: input n + output n (host buffers)
    std::vector<BatchGrid> h_grids;
    BatchGrid* d_grids = nullptr;
    int64_t* d_prep = nullptr;
};

void destroy_image_plan(ImagePlan* p) {
    if (!p) return;
    if (p->geo) {
        GridGeo* g = p->geo;
        void* bufs[] = {g->d_desc, g->d_target, g->d_first, g->d_last, g->d_rowoff, g->d_weight, g->d_rowtab};
        for (void* b : bufs) cudaFree(b);
        delete g;
    }
    void* bufs[] = {p->d_pool, p->d_io, p->d_grids, p->d_prep};
    for (void* b : bufs) cudaFree(b);
    delete p;
}

int build_image_plan(int dim, int count, const int32_t* angles, int nangles, ImagePlan** out) {
    ImagePlan* p = new ImagePlan();
    *out = p;
    p->dim = dim;
    p->count = count;
    p->angles.assign(angles, angles + nangles);
    SKE_TRY(make_grid_geo(dim, dim, &p->geo));
    memset(&p->tl, 0, sizeof(p->tl));
    for (int k = 0; k < nangles; k++) {
        const int t = p->geo->geo.desc[angles[k]].type;
        p->tl.angle[t][p->tl.count[t]] = angles[k];
        p->tl.slot[t][p->tl.count[t]] = k;
        p->tl.count[t]++;
        p->used |= 1u << t;
    }
    const int64_t n = (int64_t)dim * dim;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        free_b = (size_t)4 << 30;
    }
    const int64_t per = 10 * n * (int64_t)sizeof(float);
    const int64_t budget = free_b > ((size_t)1 << 30) ? (int64_t)((free_b - ((size_t)1 << 30)) / 2) : per;
    p->wave = (int)std::max<int64_t>(1, std::min<int64_t>(count, budget / per));
    SKE_TRY(dev_alloc(&p->d_pool, (size_t)(8 * n) * p->wave));
    SKE_TRY(dev_alloc(&p->d_io, (size_t)(2 * n) * p->wave));
    SKE_TRY(dev_alloc(&p->d_grids, (size_t)p->wave));
    std::vector<int64_t> prep(p->wave + 1);
    for (int k = 0; k <= p->wave; k++) prep[k] = k * batch_prep_blocks(dim, dim);
    SKE_TRY(upload_vec(&p->d_prep, prep));
    p->h_grids.resize(p->wave);
    for (int k = 0; k < p->wave; k++) {
        BatchGrid& G = p->h_grids[k];
        memset(&G, 0, sizeof(G));
        G.dimx = G.dimy = dim;
        G.n = n;
        G.orient = p->d_pool + (int64_t)k * 8 * n;
        G.acc = G.orient + 4 * n;
        G.comp = nullptr;
        G.used = p->used;
    }
    return SKE_OK;
}

int run_images_f32(ske_engine e, int count, int dim, const float* const* inputs, int in_dev, float* const* outputs,
                   int out_dev, const int32_t* angles, int nangles) {
    ImagePlan* p = e->image_plan;
    if (!p || p->dim != dim || p->count != count || p->angles != std::vector<int>(angles, angles + nangles)) {
        SKE_CK(cudaStreamSynchronize(e->stream));
        destroy_image_plan(p);
        e->image_plan = nullptr;
        ImagePlan* np = nullptr;
        int rc;
        try {
            rc = build_image_plan(dim, count, angles, nangles, &np);
        } catch (const std::exception& ex) {
            rc = host_failure(ex);
        }
        if (rc != SKE_OK) {
            destroy_image_plan(np);
            return rc;
        }
        e->image_plan = p = np;
    }
    const int64_t n = (int64_t)dim * dim;
    const DevGeometry g{p->geo->d_desc, p->geo->d_target, p->geo->d_weight, p->geo->d_first, p->geo->d_last};
    for (int w0 = 0; w0 < count; w0 += p->wave) {
        const int nw = std::min(p->wave, count - w0);
        for (int k = 0; k < nw; k++) {
            BatchGrid& G = p->h_grids[k];
            float* io = p->d_io + (int64_t)k * 2 * n;
            if (in_dev) {
                G.in = inputs[w0 + k];
            } else {
                SKE_CK(cudaMemcpyAsync(io, inputs[w0 + k], sizeof(float) * n, cudaMemcpyHostToDevice, e->stream));
                G.in = io;
            }
            G.out = out_dev ? outputs[w0 + k] : io + n;
        }
        SKE_CK(cudaMemcpyAsync(p->d_grids, p->h_grids.data(), sizeof(BatchGrid) * nw, cudaMemcpyHostToDevice,
                               e->stream));
        const BatchTables t{p->d_grids, nullptr, nullptr, p->d_prep, nullptr, nullptr, nw, 0};
        const int64_t blocks = (int64_t)nw * batch_prep_blocks(dim, dim);
        {
            LaunchScope ls(e, "prepare", 1);
            SKE_TRY(ls.done(launch_prepare_batch(t, blocks, e->stream)));
        }
        {
            LaunchScope ls(e, "cepstrum", 1);
            SKE_TRY(ls.done(launch_cepstrum_f32(t, nw, g, p->tl, dim, e->stream)));
        }
        {
            LaunchScope ls(e, "reduce", 1);
            SKE_TRY(ls.done(launch_reduce_batch(t, blocks, SKE_ACCUM_REFERENCE, e->stream, 1)));
        }
        if (!out_dev)
            for (int k = 0; k < nw; k++)
                SKE_CK(cudaMemcpyAsync(outputs[w0 + k], p->h_grids[k].out, sizeof(float) * n, cudaMemcpyDeviceToHost,
                                       e->stream));
    }
    return check_status(e);
}

}  // namespace

extern "C" {

int ske_abi_version(void) { return SKE_ABI_VERSION; }

const char* ske_last_error(void) { return t_last_error.c_str(); }

int ske_params_default(ske_params* p) {
    if (!p) return fail(SKE_ERR_INVALID, "null params");
    p->max_sector = 180;
    p->povh = (float)(1.5 / 10.0);  // obsheight / step (kernelSDEM.h:159)
    p->accum = SKE_ACCUM_REFERENCE;
    p->flags = 0;
    return SKE_OK;
}

int ske_device_count(int* count) {
    if (!count) return fail(SKE_ERR_INVALID, "null count");
    *count = 0;
    int n = 0;
    cudaError_t err = cudaGetDeviceCount(&n);
    if (err != cudaSuccess) {
        cudaGetLastError();
        return SKE_OK;
    }
    *count = n;
    return SKE_OK;
}

int ske_geometry(int dimx, int dimy, int angle, ske_sector_geometry* geom, int32_t* first, int32_t* last,
                 int32_t* target, float* weight) try {
    if (dimx < 1 || dimy < 1 || dimx > 65535 || dimy > 65535)
        return fail(SKE_ERR_INVALID, "grid %dx%d outside [1,65535]", dimx, dimy);
    if (angle < 0 || angle >= kMaxSectors) return fail(SKE_ERR_INVALID, "angle %d outside [0,180)", angle);
    if (!geom) return fail(SKE_ERR_INVALID, "null geometry");
    SectorDesc d;
    std::vector<int32_t> f, l, t;
    std::vector<float> w;
    sector_geometry(dimx, dimy, angle, d, f, l, t, w);
    const std::string why = check_sector(d, f.data(), l.data(), t.data(), dimx, dimy);
    if (!why.empty()) return fail(SKE_ERR_INVALID, "sector geometry of %dx%d: %s", dimx, dimy, why.c_str());
    geom->angle = d.angle;
    geom->sector_type = d.type;
    geom->new_angle = d.new_angle;
    geom->dim_i = d.dim_i;
    geom->dim_o = d.dim_o;
    geom->offset = d.offset;
    geom->skew_height = d.H;
    geom->dim_l = d.diml;
    geom->scale = d.scale;
    geom->skewness = d.skewness;
    if (first) std::copy(f.begin(), f.end(), first);
    if (last) std::copy(l.begin(), l.end(), last);
    if (target) std::copy(t.begin(), t.end(), target);
    if (weight) std::copy(w.begin(), w.end(), weight);
    return SKE_OK;
} catch (const std::exception& ex) {
    return host_failure(ex);
}

namespace {
int create_engine(ske_engine* out, int dimx, int dimy, int device, void* stream, ske_engine parent);
int init_engine(ske_engine e, int dimx, int dimy, int device, void* stream, ske_engine parent);
}

int ske_create(ske_engine* out, int dimx, int dimy, int device, void* stream) try {
    return create_engine(out, dimx, dimy, device, stream, nullptr);
} catch (const std::exception& ex) {
    return host_failure(ex);
}

namespace {
int create_engine(ske_engine* out, int dimx, int dimy, int device, void* stream, ske_engine parent) {
    if (!out) return fail(SKE_ERR_INVALID, "null engine pointer");
    *out = nullptr;
    if (dimx < 1 || dimy < 1 || dimx > 65535 || dimy > 65535)
        return fail(SKE_ERR_INVALID, "grid %dx%d outside [1,65535]", dimx, dimy);
    int ndev = 0;
    cudaError_t err = cudaGetDeviceCount(&ndev);
    if (err != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SKE_ERR_NO_DEVICE, "no CUDA device available (%s)",
                    err != cudaSuccess ? cudaGetErrorString(err) : "0 devices");
    }
    if (device < 0 || device >= ndev) return fail(SKE_ERR_INVALID, "device %d outside [0,%d)", device, ndev);
    ske_engine e = new ske_engine_s();
    int rc;
    try {
        rc = init_engine(e, dimx, dimy, device, stream, parent);
    } catch (const std::exception& ex) {
        rc = host_failure(ex);
    }
    if (rc != SKE_OK) {
        ske_destroy(e);  // frees whatever was allocated before the failure
        return rc;
    }
    *out = e;
    return SKE_OK;
}

int init_engine(ske_engine e, int dimx, int dimy, int device, void* stream, ske_engine parent) {
    e->dimx = dimx;
    e->dimy = dimy;
    e->device = device;
    SKE_CK(cudaSetDevice(device));
    SKE_CK(cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, device));
    SKE_TRY(ensure_device_tables(device));
    if (stream) {
        e->stream = (cudaStream_t)stream;
    } else {
        SKE_CK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
        e->own_stream = true;
    }
    e->N = (int64_t)dimx * dimy;
    e->len = skew_buffer_len(dimx, dimy);
    e->stride = (e->len + 63) & ~(int64_t)63;
    const std::string why = build_geometry(dimx, dimy, e->geo);
    if (!why.empty()) return fail(SKE_ERR_INVALID, "sector geometry of %dx%d: %s", dimx, dimy, why.c_str());
    e->rows_in_width.assign(e->geo.desc.size(), 1);
    for (size_t a = 0; a < e->geo.desc.size(); a++) {
        SectorDesc& d = e->geo.desc[a];
        for (int r = 0; r < d.H; r++)
            if (e->geo.last[d.row_off + r] > d.dim_i) e->rows_in_width[a] = 0;
        d.in_width = e->rows_in_width[a];
    }
    while (e->max_H2 < e->geo.max_H) e->max_H2 <<= 1;
    e->pstride = e->max_H2;
    if (parent && parent->stride >= e->len && parent->pstride >= e->max_H2) {
        e->parent = parent;  // skewed grids fit the parent's slots: borrow them
        e->stride = parent->stride;
        e->pstride = parent->pstride;
    }
    // Geometry tables.
    SKE_TRY(dev_alloc(&e->d_desc, e->geo.desc.size()));
    SKE_TRY(dev_alloc(&e->d_target, e->geo.target.size()));
    SKE_TRY(dev_alloc(&e->d_weight, e->geo.weight.size()));
    SKE_TRY(dev_alloc(&e->d_first, e->geo.first.size()));
    SKE_TRY(dev_alloc(&e->d_last, e->geo.last.size()));
    SKE_CK(cudaMemcpy(e->d_desc, e->geo.desc.data(), sizeof(SectorDesc) * e->geo.desc.size(), cudaMemcpyHostToDevice));
    SKE_CK(cudaMemcpy(e->d_target, e->geo.target.data(), sizeof(int32_t) * e->geo.target.size(), cudaMemcpyHostToDevice));
    SKE_CK(cudaMemcpy(e->d_weight, e->geo.weight.data(), sizeof(float) * e->geo.weight.size(), cudaMemcpyHostToDevice));
    SKE_CK(cudaMemcpy(e->d_first, e->geo.first.data(), sizeof(int32_t) * e->geo.first.size(), cudaMemcpyHostToDevice));
    SKE_CK(cudaMemcpy(e->d_last, e->geo.last.data(), sizeof(int32_t) * e->geo.last.size(), cudaMemcpyHostToDevice));
    e->dg = DevGeometry{e->d_desc, e->d_target, e->d_weight, e->d_first, e->d_last};
    // FFT twiddles for every power of two up to max(64, max_H2).
    std::vector<double> all, tw;
    const int top = std::max(6, 31 - __builtin_clz((unsigned)e->max_H2));
    for (int k = 0; k <= top; k++) {
        e->tw_off_host[k] = (int64_t)all.size();
        fft_twiddles(1u << k, tw);
        all.insert(all.end(), tw.begin(), tw.end());
    }
    // Local Radon weights (180 x 64) and taper.
    std::vector<double> gauss, taper;
    local_radon_tables(e->geo, gauss, taper);
    e->lr_gauss_off = (int64_t)all.size();
    all.insert(all.end(), gauss.begin(), gauss.end());
    e->lr_taper_off = (int64_t)all.size();
    all.insert(all.end(), taper.begin(), taper.end());
    all.push_back(0.0);
    SKE_TRY(dev_alloc(&e->d_tw, all.size()));
    SKE_TRY(dev_alloc(&e->d_tw_off, 32));
    SKE_CK(cudaMemcpy(e->d_tw, all.data(), sizeof(double) * all.size(), cudaMemcpyHostToDevice));
    SKE_CK(cudaMemcpy(e->d_tw_off, e->tw_off_host, sizeof(int64_t) * 32, cudaMemcpyHostToDevice));
    // Grids and accumulators.
    SKE_TRY(dev_alloc(&e->d_in, e->N));
    SKE_TRY(dev_alloc(&e->d_orient, 4 * e->N));
    encode_skew_maps(&e->skew_maps, e->d_orient, e->dimx, e->dimy);  // ok = false: the gather kernel runs
    SKE_TRY(dev_alloc(&e->d_acc, 4 * e->N));
    SKE_TRY(dev_alloc(&e->d_comp, 4 * e->N));
    SKE_TRY(dev_alloc(&e->d_out, e->N));
    SKE_TRY(dev_alloc(&e->d_counter, 1));
    SKE_TRY(dev_alloc(&e->d_status, 1));
    SKE_CK(cudaMemset(e->d_status, 0, sizeof(int)));
    SKE_TRY(pinned_alloc(&e->h_pin, (size_t)std::max<int64_t>(e->N, e->len)));
    return ensure_slots(e, 1);
}
}  // namespace

int ske_destroy(ske_engine e) {
    if (!e) return SKE_OK;
    for (auto& kv : e->children) ske_destroy(kv.second);
    e->children.clear();
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    destroy_batch_plan(e->batch_plan);
    e->batch_plan = nullptr;
    destroy_image_plan(e->image_plan);
    e->image_plan = nullptr;
    cudaFree(e->d_tune_items);
    if (e->parent) e->d_SI = e->d_SO = nullptr, e->d_P = nullptr, e->d_lists = nullptr;  // borrowed
    for (auto& kv : e->item_plans) cudaFree(kv.second.d_items);
    for (auto& p : e->pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (cudaEvent_t ev : e->event_pool) cudaEventDestroy(ev);
    void* bufs[] = {e->d_desc, e->d_target, e->d_first, e->d_last, e->d_weight, e->d_in, e->d_orient, e->d_acc,
                    e->d_comp, e->d_out, e->d_SI, e->d_SO, e->d_P, e->d_tw, e->d_tw_off, e->d_counter, e->d_status,
                    e->d_lists};
    for (void* b : bufs) cudaFree(b);
    if (e->h_pin) cudaFreeHost(e->h_pin);
    if (e->own_stream) cudaStreamDestroy(e->stream);
    delete e;
    return SKE_OK;
}

int ske_inject_alloc_failure(int64_t after) {
    g_alloc_fail_in.store(after < 0 ? -1 : after);
    return SKE_OK;
}

int ske_stream(ske_engine e, void** stream) {
    if (!e || !stream) return fail(SKE_ERR_INVALID, "null argument");
    *stream = (void*)e->stream;
    return SKE_OK;
}

int ske_run(ske_engine e, int kernel, const float* input, int input_on_device, float* output, int output_on_device,
            const ske_params* p) try {
    ske_params prm;
    SKE_TRY(validate_params(p, &prm));
    std::vector<int32_t> angles(prm.max_sector);
    for (int i = 0; i < prm.max_sector; i++) angles[i] = i;
    return run_angle_list(e, kernel, input, input_on_device, output, output_on_device, angles.data(),
                          prm.max_sector, &prm);
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_run_angles(ske_engine e, int kernel, const float* input, int input_on_device, float* output,
                   int output_on_device, const int32_t* angles, int nangles, const ske_params* p) try {
    return run_angle_list(e, kernel, input, input_on_device, output, output_on_device, angles, nangles, p);
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_accumulate(ske_engine e, int kernel, const float* input, int input_on_device, const int32_t* angles,
                   int nangles, const ske_params* p, float* acc, int acc_on_device, uint32_t* used_mask) try {
    if (!acc || !used_mask) return fail(SKE_ERR_INVALID, "null output");
    ske_params prm;
    SKE_TRY(accumulate_angles(e, kernel, input, input_on_device, angles, nangles, p, &prm));
    if (prm.accum == SKE_ACCUM_KAHAN)
        return fail(SKE_ERR_UNSUPPORTED, "accumulators are exported in reference accumulation mode only");
    if (acc_on_device) {
        SKE_CK(cudaMemcpyAsync(acc, e->d_acc, sizeof(float) * 4 * e->N, cudaMemcpyDeviceToDevice, e->stream));
        SKE_CK(cudaStreamSynchronize(e->stream));
    } else {
        for (int t = 0; t < 4; t++) SKE_TRY(download(e, acc + t * e->N, e->d_acc + t * e->N, e->N));
    }
    *used_mask = e->used;
    e->prepared = false;
    return check_status(e);
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_accumulate_resume(ske_engine e, int kernel, const float* input, int input_on_device, const int32_t* angles,
                          int nangles, const ske_params* p, float* acc, float* comp, int state_on_device,
                          uint32_t* used_mask) try {
    if (!acc || !used_mask) return fail(SKE_ERR_INVALID, "null accumulator state");
    const StartState st{acc, comp, *used_mask, state_on_device};
    ske_params prm;
    SKE_TRY(accumulate_angles(e, kernel, input, input_on_device, angles, nangles, p, &prm, &st));
    for (int t = 0; t < 4; t++) {
        const int64_t off = (int64_t)t * e->N;
        if (state_on_device) {
            SKE_CK(cudaMemcpyAsync(acc + off, e->d_acc + off, sizeof(float) * e->N, cudaMemcpyDeviceToDevice,
                                   e->stream));
            if (prm.accum == SKE_ACCUM_KAHAN)
                SKE_CK(cudaMemcpyAsync(comp + off, e->d_comp + off, sizeof(float) * e->N, cudaMemcpyDeviceToDevice,
                                       e->stream));
        } else {
            SKE_TRY(download(e, acc + off, e->d_acc + off, e->N));
            if (prm.accum == SKE_ACCUM_KAHAN) SKE_TRY(download(e, comp + off, e->d_comp + off, e->N));
        }
    }
    SKE_CK(cudaStreamSynchronize(e->stream));
    *used_mask = e->used;
    e->prepared = false;
    return check_status(e);
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_fold(ske_engine e, int kernel, const float* acc, const float* comp, int state_on_device, uint32_t used_mask,
             int accum, float* output, int output_on_device) try {
    if (!e) return fail(SKE_ERR_INVALID, "null engine");
    if (!valid_kernel(kernel)) return fail(SKE_ERR_INVALID, "unknown kernel %d", kernel);
    if (accum != SKE_ACCUM_REFERENCE && accum != SKE_ACCUM_KAHAN)
        return fail(SKE_ERR_INVALID, "unknown accumulation mode %d", accum);
    if (!acc || !output || (accum == SKE_ACCUM_KAHAN && !comp)) return fail(SKE_ERR_INVALID, "null argument");
    SKE_TRY(set_device(e));
    SKE_TRY(load_state(e, StartState{acc, comp, used_mask, state_on_device}, accum));
    SKE_TRY(run_reduce(e, output, output_on_device, kernel == SKE_KERNEL_CEPSTRUM, accum));
    SKE_CK(cudaStreamSynchronize(e->stream));
    return SKE_OK;
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_run_batch(ske_engine e, int kernel, int count, const int32_t* dimx, const int32_t* dimy,
                  const float* const* inputs, int inputs_on_device, float* const* outputs, int outputs_on_device,
                  const ske_params* p) try {
    ske_params prm;
    SKE_TRY(validate_params(p, &prm));
    std::vector<int32_t> angles(prm.max_sector);
    for (int i = 0; i < prm.max_sector; i++) angles[i] = i;
    return ske_run_batch_angles(e, kernel, count, dimx, dimy, inputs, inputs_on_device, outputs, outputs_on_device,
                                angles.data(), prm.max_sector, &prm);
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_run_batch_angles(ske_engine e, int kernel, int count, const int32_t* dimx, const int32_t* dimy,
                         const float* const* inputs, int inputs_on_device, float* const* outputs,
                         int outputs_on_device, const int32_t* angles, int nangles, const ske_params* p) try {
    if (!e) return fail(SKE_ERR_INVALID, "null engine");
    if (!valid_kernel(kernel)) return fail(SKE_ERR_INVALID, "unknown kernel %d", kernel);
    if (count < 0 || (count > 0 && (!dimx || !dimy || !inputs || !outputs)))
        return fail(SKE_ERR_INVALID, "bad batch arguments");
    if (nangles < 1 || !angles) return fail(SKE_ERR_INVALID, "empty angle list");
    for (int i = 0; i < nangles; i++)
        if (angles[i] < 0 || angles[i] >= kMaxSectors) return fail(SKE_ERR_INVALID, "angle %d outside [0,180)", angles[i]);
    for (int i = 0; i < count; i++) {
        if (dimx[i] < 1 || dimy[i] < 1 || dimx[i] > 65535 || dimy[i] > 65535)
            return fail(SKE_ERR_INVALID, "grid %d: %dx%d outside [1,65535]", i, dimx[i], dimy[i]);
        if (!inputs[i] || !outputs[i]) return fail(SKE_ERR_INVALID, "grid %d: null input or output", i);
    }
    ske_params prm;
    SKE_TRY(validate_params(p, &prm));
    SKE_TRY(set_device(e));
    e->flags = prm.flags;
    std::vector<int> per_grid;  // grids run one at a time through an engine of their size
    if (kernel == SKE_KERNEL_CEPSTRUM && (prm.flags & SKE_FLAG_CEPSTRUM_F32) && count > 0) {
        // Runs of consecutive square images of one side share a launch sequence.
        int i = 0;
        while (i < count) {
            if (dimx[i] != dimy[i]) {
                per_grid.push_back(i++);
                continue;
            }
            int k = i + 1;
            while (k < count && dimx[k] == dimx[i] && dimy[k] == dimx[i]) k++;
            SKE_TRY(run_images_f32(e, k - i, dimx[i], inputs + i, inputs_on_device, outputs + i, outputs_on_device,
                                   angles, nangles));
            i = k;
        }
    } else if (kernel == SKE_KERNEL_SDEM && count > 0) {
        if (!same_plan(e->batch_plan, count, dimx, dimy, angles, nangles, prm.accum)) {
            SKE_CK(cudaStreamSynchronize(e->stream));
            destroy_batch_plan(e->batch_plan);
            e->batch_plan = nullptr;
            BatchPlan* np = nullptr;
            int rc;
            try {
                rc = build_batch_plan(e, count, dimx, dimy, angles, nangles, prm.accum, &np);
            } catch (const std::exception& ex) {
                rc = host_failure(ex);
            }
            if (rc != SKE_OK) {
                destroy_batch_plan(np);
                return rc;
            }
            e->batch_plan = np;
        }
        BatchPlan* bp = e->batch_plan;
        for (BatchWave& w : bp->waves)
            SKE_TRY(run_wave(e, bp, w, prm.povh, inputs, inputs_on_device, outputs, outputs_on_device));
        SKE_TRY(check_status(e));
        per_grid = bp->fallback;
    } else {
        for (int i = 0; i < count; i++) per_grid.push_back(i);
    }
    // One child engine per other grid size, created on first use and kept with
    // the parent (geometry, work lists and buffers are reused by later batches).
    for (int i : per_grid) {
        ske_engine sub = e;
        if (dimx[i] != e->dimx || dimy[i] != e->dimy) {
            const auto key = std::make_pair((int)dimx[i], (int)dimy[i]);
            auto it = e->children.find(key);
            if (it == e->children.end()) {
                SKE_TRY(create_engine(&sub, dimx[i], dimy[i], e->device, (void*)e->stream, e));
                e->children[key] = sub;
            } else {
                sub = it->second;
            }
        }
        const int64_t before = sub->launches;
        const int rc = ske_run_angles(sub, kernel, inputs[i], inputs_on_device, outputs[i], outputs_on_device, angles,
                                      nangles, &prm);
        if (sub != e) e->launches += sub->launches - before;
        if (rc != SKE_OK) return rc;
    }
    return SKE_OK;
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_skew_select(int path) {
    if (skew_select(path) != 0) return fail(SKE_ERR_INVALID, "skew path must be 0 or 1");
    return SKE_OK;
}

int ske_set_sweep_shape(ske_engine e, int lvl0, int lvl1, int ctas_per_sm) try {
    if (!e) return fail(SKE_ERR_INVALID, "null engine");
    auto ok = [](int v) { return v == 16 || v == 32 || v == 48 || v == 64; };
    if (lvl0 != 0 && (!ok(lvl0) || (lvl1 != 0 && !ok(lvl1)) || ctas_per_sm < 0))
        return fail(SKE_ERR_INVALID, "sweep shape: levels of 16, 32, 48 or 64 steps (lvl1 also 0), CTAs >= 0");
    e->fixed_shape = lvl0 == 0 ? SweepShape{0, 0, 0} : SweepShape{lvl0, lvl1, ctas_per_sm};
    if (e->batch_plan) e->batch_plan->tuned = false;  // the next batch call applies it (and captures again)
    if (e->batch_plan)
        for (BatchWave& w : e->batch_plan->waves)
            if (w.graph) {
                cudaGraphExecDestroy(w.graph);
                w.graph = nullptr;
            }
    return SKE_OK;
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_radon_select(int path) {
    if (radon_select(path) != 0) return fail(SKE_ERR_INVALID, "radon path %d: 0 (fused) or 1 (two launches)", path);
    return SKE_OK;
}

int ske_sweep_shape(ske_engine e, int* lvl0, int* lvl1, int* ctas_per_sm) {
    if (!e || !lvl0 || !lvl1 || !ctas_per_sm) return fail(SKE_ERR_INVALID, "null argument");
    *lvl0 = e->last_shape.lvl0;
    *lvl1 = e->last_shape.lvl1;
    *ctas_per_sm = e->last_shape.ctas;
    return SKE_OK;
}

int ske_prepare(ske_engine e, const float* input, int on_device) try {
    if (!e || !input) return fail(SKE_ERR_INVALID, "null argument");
    SKE_TRY(set_device(e));
    e->flags = 0;  // the per-sector calls take no parameters: the reference's operators, no modes
    return run_prepare(e, input, on_device);
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_skew(ske_engine e, int angle) try {
    if (!e) return fail(SKE_ERR_INVALID, "null engine");
    if (!e->prepared) return fail(SKE_ERR_STATE, "skew() before prepare()");
    if (angle < 0 || angle >= kMaxSectors) return fail(SKE_ERR_INVALID, "angle %d outside [0,180)", angle);
    SKE_TRY(set_device(e));
    Batch b;
    b.count = 1;
    b.angle[0] = angle;
    SKE_TRY(run_skew(e, b));
    SKE_CK(cudaMemsetAsync(e->d_SO, 0, sizeof(float) * e->stride, e->stream));  // resetSkew
    e->cur_angle = angle;
    e->kernel_ran = false;
    return SKE_OK;
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_kernel(ske_engine e, int kernel, float povh) try {
    if (!e) return fail(SKE_ERR_INVALID, "null engine");
    if (!valid_kernel(kernel)) return fail(SKE_ERR_INVALID, "unknown kernel %d", kernel);
    if (e->cur_angle < 0) return fail(SKE_ERR_STATE, "kernel() before skew()");
    SKE_TRY(set_device(e));
    Batch b;
    b.count = 1;
    b.angle[0] = e->cur_angle;
    SKE_TRY(run_operator(e, kernel, b, povh, 0));
    e->kernel_ran = true;
    return SKE_OK;
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_sector(ske_engine e, ske_sector_view* v) {
    if (!e || !v) return fail(SKE_ERR_INVALID, "null argument");
    if (e->cur_angle < 0) return fail(SKE_ERR_STATE, "no current sector: call skew() first");
    const SectorDesc& d = e->geo.desc[e->cur_angle];
    memset(v, 0, sizeof(*v));
    v->geom.angle = d.angle;
    v->geom.sector_type = d.type;
    v->geom.new_angle = d.new_angle;
    v->geom.dim_i = d.dim_i;
    v->geom.dim_o = d.dim_o;
    v->geom.offset = d.offset;
    v->geom.skew_height = d.H;
    v->geom.dim_l = d.diml;
    v->geom.scale = d.scale;
    v->geom.skewness = d.skewness;
    v->skew_out = e->d_SO;
    v->skew_in = e->d_SI;
    v->first = e->d_first + d.row_off;
    v->last = e->d_last + d.row_off;
    v->target = e->d_target + d.col_off;
    v->weight = e->d_weight + d.col_off;
    v->stream = (void*)e->stream;
    return SKE_OK;
}

int ske_kernel_custom(ske_engine e, ske_operator_fn fn, void* user, float povh) {
    if (!e || !fn) return fail(SKE_ERR_INVALID, "null argument");
    ske_sector_view v;
    SKE_TRY(ske_sector(e, &v));
    v.povh = povh;
    SKE_TRY(set_device(e));
    const int rc = fn(user, &v);
    if (rc != 0) return fail(SKE_ERR_DEVICE, "custom operator returned %d", rc);
    SKE_CK(cudaGetLastError());
    e->kernel_ran = true;
    return SKE_OK;
}

int ske_deskew(ske_engine e, int is_max, int accum) try {
    if (!e) return fail(SKE_ERR_INVALID, "null engine");
    if (!e->kernel_ran) return fail(SKE_ERR_STATE, "deskew() before kernel()");
    if (accum != SKE_ACCUM_REFERENCE && accum != SKE_ACCUM_KAHAN)
        return fail(SKE_ERR_INVALID, "unknown accumulation mode %d", accum);
    SKE_TRY(set_device(e));
    Batch b;
    b.count = 1;
    b.angle[0] = e->cur_angle;
    e->accum_mode = accum;
    return run_deskew(e, b, is_max, accum);
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_reduce(ske_engine e, float* output, int on_device, int is_max) try {
    if (!e || !output) return fail(SKE_ERR_INVALID, "null argument");
    if (!e->prepared) return fail(SKE_ERR_STATE, "reduce() before prepare()");
    SKE_TRY(set_device(e));
    return run_reduce(e, output, on_device, is_max, e->accum_mode);
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_copy_skewed(ske_engine e, float* skew_in, float* skew_out, int on_device) try {
    if (!e) return fail(SKE_ERR_INVALID, "null engine");
    if (e->cur_angle < 0) return fail(SKE_ERR_STATE, "no current sector: call skew() first");
    SKE_TRY(set_device(e));
    if (on_device) {
        if (skew_in) SKE_CK(cudaMemcpyAsync(skew_in, e->d_SI, sizeof(float) * e->len, cudaMemcpyDeviceToDevice, e->stream));
        if (skew_out)
            SKE_CK(cudaMemcpyAsync(skew_out, e->d_SO, sizeof(float) * e->len, cudaMemcpyDeviceToDevice, e->stream));
        SKE_CK(cudaStreamSynchronize(e->stream));
        return SKE_OK;
    }
    if (skew_in) SKE_TRY(download(e, skew_in, e->d_SI, e->len));
    if (skew_out) SKE_TRY(download(e, skew_out, e->d_SO, e->len));
    return SKE_OK;
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_sdem_counts(ske_engine e, int angle, float povh, float* counts, int on_device) try {
    if (!e || !counts) return fail(SKE_ERR_INVALID, "null argument");
    if (!e->prepared) return fail(SKE_ERR_STATE, "sdem_counts() before prepare()");
    if (angle < 0 || angle >= kMaxSectors) return fail(SKE_ERR_INVALID, "angle %d outside [0,180)", angle);
    SKE_TRY(set_device(e));
    Batch b;
    b.count = 1;
    b.angle[0] = angle;
    SKE_TRY(run_skew(e, b));
    SKE_TRY(run_operator(e, SKE_KERNEL_SDEM, b, povh, 1));
    e->cur_angle = angle;
    e->kernel_ran = true;
    if (on_device) {
        SKE_CK(cudaMemcpyAsync(counts, e->d_SO, sizeof(float) * e->len, cudaMemcpyDeviceToDevice, e->stream));
        SKE_CK(cudaStreamSynchronize(e->stream));
    } else {
        SKE_TRY(download(e, counts, e->d_SO, e->len));
    }
    return check_status(e);
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_profile_enable(ske_engine e, int enable) try {
    if (!e) return fail(SKE_ERR_INVALID, "null engine");
    SKE_TRY(set_device(e));
    SKE_TRY(flush_profile(e));
    e->prof = enable != 0;
    e->prof_tot.clear();
    return SKE_OK;
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_profile_get(ske_engine e, const char* name, double* ms, int64_t* launches) try {
    if (!e || !name) return fail(SKE_ERR_INVALID, "null argument");
    SKE_TRY(set_device(e));
    SKE_TRY(flush_profile(e));
    auto it = e->prof_tot.find(name);
    if (ms) *ms = it == e->prof_tot.end() ? 0.0 : it->second.ms;
    if (launches) *launches = it == e->prof_tot.end() ? 0 : it->second.launches;
    return SKE_OK;
} catch (const std::exception& ex) {
    return host_failure(ex);
}

int ske_selftest_division(int device, int dmax, int64_t* checked, int64_t* mismatches, uint32_t* first_bad_bits) {
    if (!checked || !mismatches || !first_bad_bits) return fail(SKE_ERR_INVALID, "null argument");
    if (dmax < 1 || dmax > 4095) return fail(SKE_ERR_INVALID, "dmax %d outside [1,4095]", dmax);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return fail(SKE_ERR_NO_DEVICE, "device %d not available", device);
    }
    SKE_CK(cudaSetDevice(device));
    SKE_TRY(ensure_device_tables(device));
    int sms = 0;
    SKE_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    unsigned long long c = 0, b = 0;
    unsigned fb = 0;
    SKE_CK(sdem_division_selftest(dmax, sms, &c, &b, &fb));
    *checked = (int64_t)c;
    *mismatches = (int64_t)b;
    *first_bad_bits = fb;
    return SKE_OK;
}

int ske_measure_fp32_peak(int device, double* scalar_ops, double* packed_ops) {
    if (!scalar_ops || !packed_ops) return fail(SKE_ERR_INVALID, "null argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return fail(SKE_ERR_NO_DEVICE, "device %d not available", device);
    }
    SKE_CK(cudaSetDevice(device));
    int sms = 0;
    SKE_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    SKE_CK(measure_fp32_peak(sms, 5, scalar_ops, packed_ops));
    return SKE_OK;
}

int ske_measure_fp64_peak(int device, double* dfma_ops) {
    if (!dfma_ops) return fail(SKE_ERR_INVALID, "null argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return fail(SKE_ERR_NO_DEVICE, "device %d not available", device);
    }
    SKE_CK(cudaSetDevice(device));
    int sms = 0;
    SKE_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    SKE_CK(measure_fp64_peak(sms, 3, dfma_ops));
    return SKE_OK;
}

int ske_launch_count(ske_engine e, int64_t* launches) {
    if (!e || !launches) return fail(SKE_ERR_INVALID, "null argument");
    *launches = e->launches;
    return SKE_OK;
}

}  // extern "C"
