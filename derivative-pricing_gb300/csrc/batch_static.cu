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

// The control-variate anchor (analytic_host.cpp), declared in context.hpp.
double mcd_host_kemna_vorst(double spot, double strike, double rate, double carry_yield,
                            double vol, double time, int type);

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
int g_grid[kStaticMaxDevices] = {};
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
// device current and size the grid.  Must happen outside any stream capture.
int static_setup(int device, char* msg, size_t cap) {
    if (g_scratch_addr[device]) return MCD_OK;
    void* addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_batch_scratch);
    if (e != cudaSuccess) return report_cuda(msg, cap, e, "cudaGetSymbolAddress(scratch)");
    int sms = 0, blocks = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return report_cuda(msg, cap, e, "SM count");
    e = mcdg::path_kernel_occupancy(1, 1, &blocks);
    if (e != cudaSuccess) return report_cuda(msg, cap, e, "occupancy");
    g_grid[device] = sms * (blocks > 0 ? blocks : 1);
    g_scratch_addr[device] = static_cast<unsigned char*>(addr);
    return MCD_OK;
}

bool finite_params(const mcd_contract& c) {
    const double v[] = {c.spot, c.strike, c.barrier, c.rebate, c.rate, c.carry_yield, c.vol,
                        c.time, c.cash_amount};
    for (double x : v)
        if (!std::isfinite(x)) return false;
    return true;
}

// Same validation and FP64 constants as mcd_price_batch's planner (operation
// order of src/models/gbm.cpp:8-10 and src/pricers/monte_carlo.cpp:159-193).
const char* convert(const mcd_contract& in, uint32_t index, DevContract& out) {
    if (in.product < 0 || in.product > 4) return "unknown product";
    if (in.type != 0 && in.type != 1) return "type must be 0 (call) or 1 (put)";
    if (!finite_params(in)) return "non-finite parameter";
    if (!(in.spot > 0.0) || !(in.vol > 0.0) || !(in.time > 0.0)) return "spot, vol and time must be > 0";
    if (in.path_count > (1ull << 53)) return "path_count must be <= 2^53";
    const bool path_dependent = in.product >= MCD_PRODUCT_ASIAN;
    if (path_dependent && in.monitoring_points < 1) return "monitoring_points must be >= 1";
    if (in.product == MCD_PRODUCT_BARRIER &&
        (!(in.barrier > 0.0) || (in.direction != 0 && in.direction != 1) || (in.knock != 0 && in.knock != 1)))
        return "barrier needs barrier > 0, direction 0/1 and knock 0/1";
    if ((in.product == MCD_PRODUCT_ASIAN || in.product == MCD_PRODUCT_LOOKBACK) &&
        in.strike_style != 0 && in.strike_style != 1)
        return "strike_style must be 0 or 1";
    if (in.product == MCD_PRODUCT_ASIAN && in.average_style != 0 && in.average_style != 1)
        return "average_style must be 0 or 1";
    if (in.product == MCD_PRODUCT_DIGITAL && in.digital_style != 0 && in.digital_style != 1)
        return "digital_style must be 0 or 1";
    std::memset(&out, 0, sizeof out);
    out.type = in.type;
    out.up = in.direction == MCD_UP;
    out.out = in.knock == MCD_OUT;
    out.floating = in.strike_style == MCD_FLOATING;
    out.asset = in.digital_style == MCD_ASSET_OR_NOTHING;
    out.antithetic = in.antithetic ? 1 : 0;
    out.spot = in.spot;
    out.strike = in.strike;
    out.barrier = in.barrier;
    out.rebate = in.rebate;
    out.cash = in.cash_amount;
    out.discount = std::exp(-in.rate * in.time);
    out.path_count = in.path_count;
    out.seed = in.seed;
    out.orig_index = index;
    double dt = in.time;
    if (path_dependent) {
        dt = in.time / static_cast<double>(in.monitoring_points);
        out.n_steps = in.monitoring_points;
    } else {
        out.n_steps = 1;
    }
    switch (in.product) {
        case MCD_PRODUCT_EUROPEAN: out.kind = mcdg::kEuropean; break;
        case MCD_PRODUCT_DIGITAL: out.kind = mcdg::kDigital; break;
        case MCD_PRODUCT_ASIAN:
            if (in.average_style == MCD_GEOMETRIC) {
                out.kind = mcdg::kAsianGeo;
            } else if (in.control_variate && in.strike_style == MCD_FIXED) {
                out.kind = mcdg::kAsianCv;
                out.kv_anchor = mcd_host_kemna_vorst(in.spot, in.strike, in.rate, in.carry_yield,
                                                     in.vol, in.time, in.type);
            } else {
                out.kind = mcdg::kAsianArith;
            }
            break;
        case MCD_PRODUCT_BARRIER:
            out.kind = in.brownian_bridge ? mcdg::kBarrierBridge : mcdg::kBarrier;
            out.log_barrier = std::log(in.barrier);
            out.log_h_rel = std::log(in.barrier / in.spot);
            out.bb_denom = in.vol * in.vol * dt;
            break;
        default:
            out.kind = in.strike_style == MCD_FIXED ? mcdg::kLookbackFixed : mcdg::kLookbackFloating;
            break;
    }
    out.drift = (in.rate - in.carry_yield - 0.5 * in.vol * in.vol) * dt;
    out.vs = in.vol * std::sqrt(dt);
    out.n_slabs = static_cast<uint32_t>((in.path_count + mcdg::kSlabPaths - 1) / mcdg::kSlabPaths);
    return nullptr;
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
    if (n == 0) return MCD_OK;
    if (!contracts || !results)
        return report(error_message, error_capacity, MCD_ERR_INVALID_ARGUMENT, "null array");
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return report_cuda(error_message, error_capacity, e, "cudaGetDevice");
    if (device < 0 || device >= kStaticMaxDevices)
        return report(error_message, error_capacity, MCD_ERR_UNSUPPORTED, "device index too large");
    int rc = static_setup(device, error_message, error_capacity);
    if (rc != MCD_OK) return rc;

    uint64_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        const char* why = convert(contracts[i], static_cast<uint32_t>(i), g_stage_contracts[i]);
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
        e = mcdg::launch_path_kernel(precision, 1, g_grid[device], d_contracts, static_cast<int>(n),
                                     d_prefix, static_cast<uint32_t>(total), d_flags, d_partials,
                                     d_flags + 1, s);
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
