// context.hpp -- the state behind an mcd_ctx handle (private).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "engine.hpp"
#include "mcd_gpu.h"

namespace mcdg {

struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
};

struct HostBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
};

struct BatchPlan {
    std::vector<DevContract> dev;    // longest-first
    std::vector<uint32_t> prefix;    // n + 1 running slab counts
    uint32_t total_items = 0;
    size_t n = 0;
};

struct LaunchShape {
    int variant = 1;      // __launch_bounds__ min-blocks 8
    int ctas_per_sm = 0;  // 0: occupancy limit
};

// Key of a captured graph.  items: the work items the captured launch was
// given; 0 for the path engine, whose kernel reads its item count from the
// uploaded prefix (one graph serves every path count; the partials buffer's
// address changes whenever it has to grow).
struct GraphKey {
    int precision, variant, grid;
    size_t n;
    uint32_t items;
    const void *contracts, *prefix, *partials, *results;
    bool operator==(const GraphKey& o) const {
        return precision == o.precision && variant == o.variant && grid == o.grid && n == o.n && items == o.items &&
               contracts == o.contracts && prefix == o.prefix && partials == o.partials && results == o.results;
    }
};

struct CachedGraph {
    GraphKey key;
    cudaGraphExec_t exec;
};

// Key of the device-resident plan: the caller's array, its length, the
// precision and a digest of the records' content (launch_words_digest).
struct DevicePlanKey {
    const void* contracts;
    size_t n;
    int precision;
    uint64_t digest;
    bool operator==(const DevicePlanKey& o) const {
        return contracts == o.contracts && n == o.n && precision == o.precision && digest == o.digest;
    }
};

struct Ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    std::string error;

    DeviceBuffer d_contracts, d_prefix, d_partials, d_results, d_scratch, d_scratch2;
    uint32_t* d_flags = nullptr;  // [0] ticket, [1] error word, [4..5] contract digest, rest spare
    HostBuffer h_stage;

    BatchPlan host_plan, device_plan;
    DevicePlanKey device_plan_key{nullptr, 0, 0, 0};
    bool device_plan_valid = false;

    LaunchShape shape[2];
    std::vector<CachedGraph> graphs;

    // Extra streams and events for graphs captured as concurrent chains
    // (fork from and join to `stream`); created on first use.
    static constexpr int kAuxStreams = 3;
    cudaStream_t aux_stream[kAuxStreams] = {};
    cudaEvent_t ev_fork = nullptr, ev_join[kAuxStreams] = {}, ev_stage[kAuxStreams] = {}, ev_train[kAuxStreams] = {};
    int ensure_aux();

    // Per-launch timing: a ring of (start, stop) event pairs recorded around
    // each graph launch on the launching stream; completed pairs are folded
    // into kernel_ms_sum by collect_timing().
    static constexpr int kEventPairs = 64;
    cudaEvent_t ev_start[kEventPairs] = {}, ev_stop[kEventPairs] = {};
    int ev_pending[kEventPairs] = {};  // ring of pending pair indices
    int ev_head = 0, ev_count = 0;
    double kernel_ms_sum = 0.0;
    uint64_t kernel_launches = 0;
    double last_ms = 0.0;
    int record_start(cudaStream_t s, int* pair);
    int record_stop(cudaStream_t s, int pair);
    void collect_timing(bool block);

    // State owned by the other modules (Heston, LSM, QMC, Greeks); freed by
    // release_extensions().
    DeviceBuffer ext[48];

    // Sensitivity engine (greeks_api.cpp): launch shape and the last graph.
    LaunchShape greeks_shape[2];
    cudaGraphExec_t greeks_graph = nullptr;
    GraphKey greeks_key{};

    // Training schedule of the learned LSM regression (mcd_lsm_set_mlp_config).
    int mlp_steps_first = 100;
    int mlp_steps = 0;
    float mlp_lr_first = 3e-3f;
    float mlp_lr = 1e-3f;
    // Networks of the last learned-LSM run (for mcd_lsm_mlp_policy).
    std::vector<uint32_t> mlp_reg_offset;
    std::vector<int32_t> mlp_steps_of;

    int fail(int code, const std::string& msg);
    int cuda_fail(cudaError_t e, const char* where);
    int reserve(DeviceBuffer& b, size_t bytes, const char* what);
    int reserve_host(HostBuffer& b, size_t bytes, const char* what);
    void release_extensions();
    ~Ctx();
};

// Batch planning and execution of the path engine (context.cpp).
int plan_contract(Ctx& ctx, const mcd_contract& in, uint32_t index, DevContract& out);
int plan_batch(Ctx& ctx, const mcd_contract* contracts, size_t n, BatchPlan& plan);
int price_batch_host(Ctx& ctx, const mcd_contract* contracts, size_t n, int precision,
                     mcd_mc_result* results);

}  // namespace mcdg

// Host analytic anchors used by the pricers themselves (analytic_host.cpp).
double mcd_host_normal_cdf(double x);
double mcd_host_bsm(double spot, double strike, double rate, double carry_yield, double vol,
                    double time, int type);
double mcd_host_kemna_vorst(double spot, double strike, double rate, double carry_yield,
                            double vol, double time, int type);

// Status for an exception caught at the C ABI (nothing may unwind through
// it): host out of memory, or an internal failure; the message goes to the
// context when there is one.  Called from the entry points' catch handlers.
int abi_exception(mcd_ctx* handle) noexcept;

#define MCD_CTX_OR_FAIL(handle, var)                              \
    if (!(handle)) return MCD_ERR_INVALID_ARGUMENT;               \
    ::mcdg::Ctx* var = reinterpret_cast<::mcdg::Ctx*>(handle);    \
    cudaSetDevice(var->device)
