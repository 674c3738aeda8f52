// batch_static.cu -- mcd_price_batch_static: batched GBM pricing that
// allocates no memory.
//
// Some callers cannot call cudaMalloc: a service that reserves all of its
// device memory up front and accounts for every byte, code running where an
// allocation's implicit device synchronisation is not acceptable, or a host
// process that is only allowed to use memory that already exists when it
// starts.  For them this entry point runs the same persistent path kernel and
// merge kernel as mcd_price_batch, but keeps every byte of scratch they need
// (contract records, the slab prefix, slab partials, device results, the
// ticket and error word) in one file-scope __device__ array of fixed size,
// which the CUDA module reserves when it is loaded and keeps until the process
// exits.  The caller passes inputs and outputs as host arrays.
//
// Limits: at most kStaticMaxContracts contracts and kStaticMaxSlabs slabs of
// 4096 paths per call (about 1.07e9 paths in total); the array is about 7 MB.
// Contracts are processed in the order given (no longest-first sort), which
// changes load balance but not results: slab partials and their merge order
// depend only on the slab index, so results are bitwise identical to
// mcd_price_batch's.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "engine.hpp"
#include "mcd_gpu.h"

namespace {

using mcdg::DevContract;
using mcdg::Welford;

constexpr size_t kStaticMaxContracts = 4096;
constexpr size_t kStaticMaxSlabs = 262144;
constexpr int kStaticMaxDevices = 64;

constexpr size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }
constexpr size_t kOffContracts = 0;
constexpr size_t kOffPrefix = align256(kOffContracts + sizeof(DevContract) * kStaticMaxContracts);
constexpr size_t kOffPartials = align256(kOffPrefix + sizeof(uint32_t) * (kStaticMaxContracts + 1));
constexpr size_t kOffResults = align256(kOffPartials + sizeof(Welford) * kStaticMaxSlabs);
constexpr size_t kOffFlags = align256(kOffResults + sizeof(mcd_mc_result) * kStaticMaxContracts);
constexpr size_t kStaticScratchBytes = align256(kOffFlags + 256);

// The scratch array.  Host code must not use this name as an address (on the
// host it is a stand-in object); the device address comes from
// cudaGetSymbolAddress, resolved once per device in static_setup().
static __device__ __align__(256) unsigned char g_batch_scratch[kStaticScratchBytes];

// Host-side state, all static: resolved device addresses and launch shapes per
// device, and a staging area for the converted contracts.  One lock serialises
// calls (the device array is shared by all of them).
std::mutex g_static_lock;
unsigned char* g_scratch_addr[kStaticMaxDevices] = {};
int g_grid[kStaticMaxDevices][2] = {};  // persistent grid per device and precision
DevContract g_stage_contracts[kStaticMaxContracts];
uint32_t g_stage_prefix[kStaticMaxContracts + 1];

int report(char* msg, size_t cap, int code, const char* text) {
    if (msg && cap) std::snprintf(msg, cap, "%s", text);
    return code;
}

int report_cuda(char* msg, size_t cap, cudaError_t e, const char* where) {
    if (msg && cap) std::snprintf(msg, cap, "%s: %s", where, cudaGetErrorString(e));
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? MCD_ERR_OUT_OF_MEMORY : MCD_ERR_CUDA;
}

// First call on a device: resolve the array's device address with that
// device current and size the grids.  Must happen outside any stream capture.
// With CUDA's lazy module loading (the runtime's default) this is also when
// the module is loaded on the device and the array's memory is reserved.
int static_setup(int device, char* msg, size_t cap) {
    if (g_scratch_addr[device]) return MCD_OK;
    void* addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_batch_scratch);
    if (e != cudaSuccess) return report_cuda(msg, cap, e, "cudaGetSymbolAddress(scratch)");
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return report_cuda(msg, cap, e, "SM count");
    for (int precision = 0; precision < 2; ++precision) {
        int blocks = 0;
        e = mcdg::path_kernel_occupancy(precision, 1, &blocks);
        if (e != cudaSuccess) return report_cuda(msg, cap, e, "occupancy");
        g_grid[device][precision] = sms * (blocks > 0 ? blocks : 1);
    }
    g_scratch_addr[device] = static_cast<unsigned char*>(addr);
    return MCD_OK;
}

}  // namespace

extern "C" int mcd_price_batch_static(const mcd_contract* contracts, size_t n, int precision,
                                      mcd_mc_result* results, void* stream, char* error_message,
                                      size_t error_capacity) {
    std::lock_guard<std::mutex> lock(g_static_lock);
    if (error_message && error_capacity) error_message[0] = '\0';
    if (precision != MCD_PRECISION_FP64 && precision != MCD_PRECISION_FP32)
        return report(error_message, error_capacity, MCD_ERR_INVALID_ARGUMENT,
                      "precision must be 0 (FP64) or 1 (FP32)");
    if (n > kStaticMaxContracts)
        return report(error_message, error_capacity, MCD_ERR_INVALID_ARGUMENT,
                      "mcd_price_batch_static: at most 4096 contracts per call");
    if (n > 0 && (!contracts || !results))
        return report(error_message, error_capacity, MCD_ERR_INVALID_ARGUMENT, "null array");
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return report_cuda(error_message, error_capacity, e, "cudaGetDevice");
    if (device < 0 || device >= kStaticMaxDevices)
        return report(error_message, error_capacity, MCD_ERR_UNSUPPORTED, "device index too large");
    // A call with n = 0 does the device's set-up only: a caller that reserves
    // the rest of device memory afterwards makes this call first.
    int rc = static_setup(device, error_message, error_capacity);
    if (rc != MCD_OK || n == 0) return rc;

    uint64_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        const char* why = mcdg::convert_contract(contracts[i], static_cast<uint32_t>(i), g_stage_contracts[i]);
        if (why) {
            char text[160];
            std::snprintf(text, sizeof text, "contract %zu: %s", i, why);
            return report(error_message, error_capacity, MCD_ERR_INVALID_ARGUMENT, text);
        }
        g_stage_prefix[i] = static_cast<uint32_t>(total);
        total += g_stage_contracts[i].n_slabs;
        if (total > kStaticMaxSlabs)
            return report(error_message, error_capacity, MCD_ERR_INVALID_ARGUMENT,
                          "mcd_price_batch_static: at most 262144 slabs of 4096 paths per call");
    }
    g_stage_prefix[n] = static_cast<uint32_t>(total);

    unsigned char* base = g_scratch_addr[device];
    DevContract* d_contracts = reinterpret_cast<DevContract*>(base + kOffContracts);
    uint32_t* d_prefix = reinterpret_cast<uint32_t*>(base + kOffPrefix);
    Welford* d_partials = reinterpret_cast<Welford*>(base + kOffPartials);
    mcd_mc_result* d_results = reinterpret_cast<mcd_mc_result*>(base + kOffResults);
    uint32_t* d_flags = reinterpret_cast<uint32_t*>(base + kOffFlags);
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // The array keeps the previous call's contents: the ticket and the error
    // word must start at zero; contracts, prefix, partials and results are
    // overwritten in full for the items of this call.
    e = cudaMemcpyAsync(d_contracts, g_stage_contracts, sizeof(DevContract) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_prefix, g_stage_prefix, sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_flags, 0, 2 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return report_cuda(error_message, error_capacity, e, "stage contracts");
    if (total > 0) {
        e = mcdg::launch_path_kernel(precision, 1, g_grid[device][precision], d_contracts, static_cast<int>(n),
                                     d_prefix, d_flags, d_partials, d_flags + 1, s);
        if (e != cudaSuccess) return report_cuda(error_message, error_capacity, e, "path kernel");
    }
    e = mcdg::launch_merge_kernel(d_contracts, static_cast<int>(n), d_prefix, d_partials, d_results, s);
    if (e != cudaSuccess) return report_cuda(error_message, error_capacity, e, "merge kernel");
    uint32_t flags[2] = {0, 0};
    e = cudaMemcpyAsync(results, d_results, sizeof(mcd_mc_result) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(flags, d_flags, sizeof flags, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return report_cuda(error_message, error_capacity, e, "batch execution");
    if (flags[1] != 0)
        return report(error_message, error_capacity, MCD_ERR_CUDA, "path kernel reported an inconsistent work item");
    return MCD_OK;
}
