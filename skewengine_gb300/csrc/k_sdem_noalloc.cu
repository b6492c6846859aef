// Allocation-free total-viewshed sweep of one skewed sector
// (ske_sdem_sector_noalloc in include/skewengine.h).
//
// Some callers cannot call cudaMalloc: code that must not grow GPU memory while
// it runs (a service with a fixed memory budget, another framework's
// allocator-owned context, or a driver layer that forbids allocation on its
// call path).  For them this entry point runs the chunked viewshed sweep (the
// one whose only scratch is its work list; the engine's compacting sweep needs
// survivor lists that grow with the grid) over a skewed sector the caller
// already holds in device memory, with every piece of the sweep's scratch in
// static storage: the sector descriptor, the work-queue
// head, the status word and the sorted work-item list in one file-scope device
// array, the row limits and the item list being built in file-scope host
// arrays.  No cudaMalloc, cudaFree or other allocating routine is called.
//
// The device array (kScratchBytes, about 8 MiB) is created by the CUDA module
// on every GPU that loads this library and held until the process exits.  Its
// device address is taken once per device, with that device current
// (cudaGetSymbolAddress), by the first call on the device; that first call also
// uploads the sweep's constant table, so it should come before any stream
// capture.  All calls share the array (and the host arrays), which keep the
// last call's contents: the queue head and status are cleared on every call,
// the item list and descriptor are rewritten.  Calls that overlap on the GPU
// race; calls from several host threads are serialised by a mutex.  Each call
// reads the row limits and, at the end, a status word back to the host and
// waits for `stream` to drain both times; the calling thread's current device
// is restored before it returns.
#include <algorithm>
#include <mutex>

#include "../../include/skewengine.h"
#include "kernels.h"

namespace ske {
namespace {

constexpr int kMaxRowCells = 4096;         // longest row the sweep's fast path takes
constexpr int kMaxItems = 1 << 20;         // work items: 8 MiB
constexpr int kMaxRows = 1 << 17;          // skewed rows
constexpr int kMaxDevices = 64;
constexpr size_t kHeaderBytes = 256;       // descriptor at 0, queue head at 128, status at 192
constexpr size_t kScratchBytes = kHeaderBytes + sizeof(uint64_t) * (size_t)kMaxItems;

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_mutex;
unsigned char* g_addr[kMaxDevices];  // device address of g_scratch on each device
int32_t h_first[kMaxRows], h_last[kMaxRows];
int64_t h_bucket[kMaxRowCells + 2];
uint64_t h_items[kMaxItems];
SectorDesc h_desc;
int h_status;

// Per-device set-up, with the device current.
int setup(int device) {
    if (g_addr[device]) return SKE_OK;
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return set_last_error(SKE_ERR_CUDA, cudaGetErrorString(e));
    e = sdem_init_tables();
    if (e != cudaSuccess) return set_last_error(SKE_ERR_CUDA, cudaGetErrorString(e));
    g_addr[device] = static_cast<unsigned char*>(p);
    return SKE_OK;
}

int cuda_fail(cudaError_t e) { return set_last_error(SKE_ERR_CUDA, cudaGetErrorString(e)); }

// Restores the calling thread's current device on every return path, so a
// caller working on another device keeps it.
struct DeviceGuard {
    int saved = -1;
    DeviceGuard() {
        if (cudaGetDevice(&saved) != cudaSuccess) {
            cudaGetLastError();
            saved = -1;
        }
    }
    ~DeviceGuard() {
        if (saved >= 0) cudaSetDevice(saved);
    }
};

}  // namespace
}  // namespace ske

extern "C" int ske_sdem_sector_noalloc(int device, const float* skew_in, float* skew_out, int dim_i,
                                       int skew_height, int dim_l, const int32_t* first, const int32_t* last,
                                       float scale2, float povh, void* stream) {
    using namespace ske;
    if (!skew_in || !skew_out || !first || !last)
        return set_last_error(SKE_ERR_INVALID, "sdem_sector_noalloc: null pointer");
    if (dim_i < 1 || skew_height < 1 || dim_l < dim_i)
        return set_last_error(SKE_ERR_INVALID, "sdem_sector_noalloc: bad sector shape");
    if (dim_l > kMaxRowCells)
        return set_last_error(SKE_ERR_INVALID,
                              "sdem_sector_noalloc: dim_l above 4096 exceeds the static scratch limits");
    if (skew_height > kMaxRows)
        return set_last_error(SKE_ERR_INVALID,
                              "sdem_sector_noalloc: more than 131072 skewed rows exceed the static scratch limits");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev || device >= kMaxDevices) {
        cudaGetLastError();
        return set_last_error(SKE_ERR_NO_DEVICE, "sdem_sector_noalloc: device not available");
    }
    std::lock_guard<std::mutex> lock(g_mutex);
    DeviceGuard restore;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_fail(e);
    const int rc = setup(device);
    if (rc != SKE_OK) return rc;

    // Row limits to the host, then the chunked sweep's work items (row, chunk
    // of 128 observers) sorted longest row first.
    e = cudaMemcpyAsync(h_first, first, sizeof(int32_t) * skew_height, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_last, last, sizeof(int32_t) * skew_height, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e);
    // Every row must satisfy 0 <= first <= last <= dim_l, as the engine's own
    // geometry does (skewShape, skewEngine.cuh:573-596): the sweep then reads
    // and writes flat cells r*dim_i + [first, last) only, all below
    // (skew_height-1)*dim_i + dim_l, and owner_row's early exit stays exact.
    const int chunk = sdem_chunk();
    int lmax = 0;
    for (int r = 0; r < skew_height; r++) {
        if (h_first[r] < 0 || h_last[r] > dim_l || h_first[r] > h_last[r])
            return set_last_error(SKE_ERR_INVALID,
                                  "sdem_sector_noalloc: a row's first/last is outside 0 <= first <= last <= dim_l");
        lmax = std::max(lmax, h_last[r] - h_first[r]);
    }
    std::fill(h_bucket, h_bucket + lmax + 2, (int64_t)0);
    int64_t total = 0;
    for (int r = 0; r < skew_height; r++) {
        const int L = h_last[r] - h_first[r];
        if (L > 0) {
            h_bucket[L] += (L + chunk - 1) / chunk;
            total += (L + chunk - 1) / chunk;
        }
    }
    if (total > kMaxItems)
        return set_last_error(SKE_ERR_INVALID,
                              "sdem_sector_noalloc: more than 2^20 work items exceed the static scratch limits");
    int64_t next = 0;
    for (int L = lmax; L >= 1; L--) {
        const int64_t cnt = h_bucket[L];
        h_bucket[L] = next;
        next += cnt;
    }
    for (int r = 0; r < skew_height; r++) {
        const int L = h_last[r] - h_first[r];
        for (int c = 0; L > 0 && c < (L + chunk - 1) / chunk; c++)
            h_items[h_bucket[L]++] = ((uint64_t)(uint32_t)r << 16) | (uint64_t)c;
    }

    // Descriptor fields the sweep reads; the rest stay zero.
    h_desc = SectorDesc();
    h_desc.dim_i = dim_i;
    h_desc.H = skew_height;
    h_desc.diml = dim_l;
    h_desc.r2 = scale2;
    unsigned char* base = g_addr[device];
    SectorDesc* d_desc = reinterpret_cast<SectorDesc*>(base);
    unsigned* d_counter = reinterpret_cast<unsigned*>(base + 128);
    int* d_status = reinterpret_cast<int*>(base + 192);
    uint64_t* d_items = reinterpret_cast<uint64_t*>(base + kHeaderBytes);
    e = cudaMemcpyAsync(d_desc, &h_desc, sizeof(SectorDesc), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_status, 0, sizeof(int), st);
    if (e == cudaSuccess && total > 0)
        e = cudaMemcpyAsync(d_items, h_items, sizeof(uint64_t) * total, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host arrays are reused by the next call
    if (e != cudaSuccess) return cuda_fail(e);

    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return cuda_fail(e);
    SdemLaunch a;
    a.g = DevGeometry{d_desc, nullptr, nullptr, first, last};
    a.b.count = 1;
    a.b.angle[0] = 0;
    a.SI = skew_in;
    a.SO = skew_out;
    a.stride = 0;
    a.items = d_items;
    a.n_items = total;
    a.counter = d_counter;  // cleared by launch_sdem_chunked
    a.povh = povh;
    a.max_row = std::max(lmax, 1);
    a.counts_only = 0;
    a.status = d_status;
    a.lists = nullptr;
    a.list_bytes = 0;
    e = launch_sdem_chunked(a, sms, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_status, d_status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e);
    if (h_status != 0) return set_last_error(SKE_ERR_DEVICE, "sdem_sector_noalloc: the sweep rejected a work item");
    return SKE_OK;
}
