// context.cpp -- the C ABI (include/mcd_gpu.h): context, validation, batch
// planning, CUDA-graph capture of the persistent path kernel, autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "context.hpp"
#include "engine.hpp"
#include "mcd_gpu.h"

using namespace mcdg;

namespace {

thread_local std::string g_create_error;

}  // namespace

// ---------------------------------------------------------------------------
// context helpers (context.hpp)
// ---------------------------------------------------------------------------
namespace mcdg {

int Ctx::fail(int code, const std::string& msg) {
    error = msg;
    return code;
}

int Ctx::cuda_fail(cudaError_t e, const char* where) {
    error = std::string(where) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return e == cudaErrorMemoryAllocation ? MCD_ERR_OUT_OF_MEMORY : MCD_ERR_CUDA;
}

int Ctx::reserve(DeviceBuffer& b, size_t bytes, const char* what) {
    if (b.bytes >= bytes && b.ptr != nullptr) return MCD_OK;
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
    // At least 1 MiB: small and medium calls then never reallocate (a
    // cudaFree/cudaMalloc pair waits for the whole device).
    size_t want = std::max<size_t>(bytes, size_t(1) << 20);
    want = want + want / 4;  // grow with headroom
    cudaError_t e = cudaMalloc(&b.ptr, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_fail(e, what);
    }
    b.bytes = want;
    return MCD_OK;
}

int Ctx::reserve_host(HostBuffer& b, size_t bytes, const char* what) {
    if (b.bytes >= bytes && b.ptr != nullptr) return MCD_OK;
    if (b.ptr) cudaFreeHost(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
    size_t want = std::max<size_t>(bytes, size_t(64) << 10);
    want = want + want / 4;
    cudaError_t e = cudaMallocHost(&b.ptr, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_fail(e, what);
    }
    b.bytes = want;
    return MCD_OK;
}

Ctx::~Ctx() {
    for (auto& g : graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
    }
    if (greeks_graph) cudaGraphExecDestroy(greeks_graph);
    for (DeviceBuffer* b : {&d_contracts, &d_prefix, &d_partials, &d_results, &d_scratch, &d_scratch2}) {
        if (b->ptr) cudaFree(b->ptr);
    }
    if (d_flags) cudaFree(d_flags);
    if (h_stage.ptr) cudaFreeHost(h_stage.ptr);
    for (int i = 0; i < kEventPairs; ++i) {
        if (ev_start[i]) cudaEventDestroy(ev_start[i]);
        if (ev_stop[i]) cudaEventDestroy(ev_stop[i]);
    }
    for (int i = 0; i < kAuxStreams; ++i) {
        if (aux_stream[i]) cudaStreamDestroy(aux_stream[i]);
        if (ev_join[i]) cudaEventDestroy(ev_join[i]);
        if (ev_stage[i]) cudaEventDestroy(ev_stage[i]);
        if (ev_train[i]) cudaEventDestroy(ev_train[i]);
    }
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (stream) cudaStreamDestroy(stream);
    release_extensions();
}

}  // namespace mcdg

// Planning and graph helpers, shared with the other modules through
// context.hpp (greeks_api.cpp builds its batches with them).
namespace mcdg {

bool finite_all(std::initializer_list<double> xs) {
    for (double x : xs)
        if (!std::isfinite(x)) return false;
    return true;
}

// Validates one contract and converts it to the kernel layout; returns null
// or the reason the contract is rejected.  No context: mcd_price_batch's
// planner and the allocation-free entry point (batch_static.cu) share it, so
// their checks and constants cannot drift apart.  The derived constants use
// the reference's operation order (gbm.cpp:8-10, monte_carlo.cpp:159-160,
// :191-193, :219, :277-280) so FP64 paths see the same values the reference
// computes per step.
const char* convert_contract(const mcd_contract& in, uint32_t index, DevContract& out) {
    if (in.product < 0 || in.product > 4) return "unknown product";
    if (in.type != 0 && in.type != 1) return "type must be 0 (call) or 1 (put)";
    if (!finite_all({in.spot, in.strike, in.barrier, in.rebate, in.rate, in.carry_yield, in.vol,
                     in.time, in.cash_amount}))
        return "non-finite parameter";
    if (!(in.spot > 0.0)) return "spot must be > 0";
    if (!(in.vol > 0.0)) return "vol must be > 0";
    if (!(in.time > 0.0)) return "time must be > 0";
    if (in.path_count > (1ull << 53)) return "path_count must be <= 2^53";
    const bool path_dependent = in.product >= MCD_PRODUCT_ASIAN;
    if (path_dependent && in.monitoring_points < 1) return "monitoring_points must be >= 1";
    if (in.product == MCD_PRODUCT_BARRIER) {
        if (!(in.barrier > 0.0)) return "barrier must be > 0";
        if (in.direction != 0 && in.direction != 1) return "direction must be 0 (up) or 1 (down)";
        if (in.knock != 0 && in.knock != 1) return "knock must be 0 (in) or 1 (out)";
    }
    if ((in.product == MCD_PRODUCT_ASIAN || in.product == MCD_PRODUCT_LOOKBACK) &&
        in.strike_style != 0 && in.strike_style != 1)
        return "strike_style must be 0 (fixed) or 1 (floating)";
    if (in.product == MCD_PRODUCT_ASIAN && in.average_style != 0 && in.average_style != 1)
        return "average_style must be 0 (arithmetic) or 1 (geometric)";
    if (in.product == MCD_PRODUCT_DIGITAL && in.digital_style != 0 && in.digital_style != 1)
        return "digital_style must be 0 (cash) or 1 (asset)";
    // Slab count in 64 bits before it is narrowed: path counts up to 2^53 are
    // accepted above, and from 2^44 paths on the count no longer fits 32 bits.
    const uint64_t slabs = (in.path_count + kSlabPaths - 1) / kSlabPaths;
    if (slabs > 0xFFFFFFFFull) return "too many paths";

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
    const double vol = in.vol;
    double dt = in.time;
    switch (in.product) {
        case MCD_PRODUCT_EUROPEAN: out.kind = kEuropean; out.n_steps = 1; break;
        case MCD_PRODUCT_DIGITAL: out.kind = kDigital; out.n_steps = 1; break;
        case MCD_PRODUCT_ASIAN:
            dt = in.time / static_cast<double>(in.monitoring_points);
            out.n_steps = in.monitoring_points;
            if (in.average_style == MCD_GEOMETRIC) {
                out.kind = kAsianGeo;
            } else if (in.control_variate && in.strike_style == MCD_FIXED) {
                out.kind = kAsianCv;
                out.kv_anchor = mcd_host_kemna_vorst(in.spot, in.strike, in.rate, in.carry_yield,
                                                     in.vol, in.time, in.type);
            } else {
                out.kind = kAsianArith;
            }
            break;
        case MCD_PRODUCT_BARRIER:
            dt = in.time / static_cast<double>(in.monitoring_points);
            out.n_steps = in.monitoring_points;
            out.kind = in.brownian_bridge ? kBarrierBridge : kBarrier;
            out.log_barrier = std::log(in.barrier);
            out.log_h_rel = std::log(in.barrier / in.spot);
            out.bb_denom = vol * vol * dt;
            break;
        default:
            dt = in.time / static_cast<double>(in.monitoring_points);
            out.n_steps = in.monitoring_points;
            out.kind = in.strike_style == MCD_FIXED ? kLookbackFixed : kLookbackFloating;
            break;
    }
    out.drift = (in.rate - in.carry_yield - 0.5 * vol * vol) * dt;
    out.vs = vol * std::sqrt(dt);
    out.n_slabs = static_cast<uint32_t>(slabs);
    return nullptr;
}

int plan_contract(Ctx& ctx, const mcd_contract& in, uint32_t index, DevContract& out) {
    const char* why = convert_contract(in, index, out);
    if (!why) return MCD_OK;
    char msg[256];
    std::snprintf(msg, sizeof msg, "contract %u: %s", index, why);
    return ctx.fail(MCD_ERR_INVALID_ARGUMENT, msg);
}

// Cost of one slab of a contract, used for longest-first ordering.
double slab_cost(const DevContract& c) {
    double per_step = c.kind == kBarrierBridge ? 2.0 : 1.0;
    if (c.kind == kAsianCv) per_step = 1.2;
    return static_cast<double>(c.n_steps) * per_step * (c.antithetic ? 2.0 : 1.0);
}

int plan_batch(Ctx& ctx, const mcd_contract* contracts, size_t n, BatchPlan& plan) {
    if (n > 0x7FFFFFFF) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "too many contracts");
    plan.dev.resize(n);
    for (size_t i = 0; i < n; ++i) {
        const int rc = plan_contract(ctx, contracts[i], static_cast<uint32_t>(i), plan.dev[i]);
        if (rc != MCD_OK) return rc;
    }
    std::stable_sort(plan.dev.begin(), plan.dev.end(), [](const DevContract& a, const DevContract& b) {
        return slab_cost(a) > slab_cost(b);
    });
    plan.prefix.resize(n + 1);
    uint64_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        plan.prefix[i] = static_cast<uint32_t>(total);
        total += plan.dev[i].n_slabs;
        if (total > 0xFFFFFFF0ull) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "batch too large");
    }
    plan.prefix[n] = static_cast<uint32_t>(total);
    plan.total_items = static_cast<uint32_t>(total);
    plan.n = n;
    return MCD_OK;
}

int launch_shape(Ctx& ctx, int precision, int& variant, int& grid) {
    LaunchShape& s = ctx.shape[precision];
    variant = s.variant;
    int blocks = 0;
    cudaError_t e = path_kernel_occupancy(precision, variant, &blocks);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "occupancy query");
    int per_sm = s.ctas_per_sm > 0 ? s.ctas_per_sm : blocks;
    if (per_sm < 1) per_sm = 1;
    grid = ctx.sm_count * per_sm;
    return MCD_OK;
}

// Uploads a plan into the context's device buffers (async on ctx.stream).
int upload_plan(Ctx& ctx, const BatchPlan& plan) {
    // The device-resident plan shares these buffers; any upload retires it.
    ctx.device_plan_valid = false;
    const size_t n = plan.n;
    int rc = ctx.reserve(ctx.d_contracts, sizeof(DevContract) * std::max<size_t>(n, 1), "contracts");
    if (rc) return rc;
    rc = ctx.reserve(ctx.d_prefix, sizeof(uint32_t) * (n + 1), "prefix");
    if (rc) return rc;
    rc = ctx.reserve(ctx.d_partials, sizeof(Welford) * std::max<uint32_t>(plan.total_items, 1), "partials");
    if (rc) return rc;
    rc = ctx.reserve(ctx.d_results, sizeof(mcd_mc_result) * std::max<size_t>(n, 1), "results");
    if (rc) return rc;
    // Stage through pinned memory so the copies are truly asynchronous.
    const size_t cbytes = sizeof(DevContract) * n, pbytes = sizeof(uint32_t) * (n + 1);
    rc = ctx.reserve_host(ctx.h_stage, cbytes + pbytes, "pinned staging");
    if (rc) return rc;
    cudaError_t e = cudaStreamSynchronize(ctx.stream);  // staging buffer reuse
    if (e != cudaSuccess) return ctx.cuda_fail(e, "stream sync");
    char* stage = static_cast<char*>(ctx.h_stage.ptr);
    if (n) std::memcpy(stage, plan.dev.data(), cbytes);
    std::memcpy(stage + cbytes, plan.prefix.data(), pbytes);
    if (n) {
        e = cudaMemcpyAsync(ctx.d_contracts.ptr, stage, cbytes, cudaMemcpyHostToDevice, ctx.stream);
        if (e != cudaSuccess) return ctx.cuda_fail(e, "copy contracts");
    }
    e = cudaMemcpyAsync(ctx.d_prefix.ptr, stage + cbytes, pbytes, cudaMemcpyHostToDevice, ctx.stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "copy prefix");
    return MCD_OK;
}

// Captures (or reuses) the graph: reset ticket and error word, persistent
// path kernel, merge kernel.  Timing events are recorded around the graph
// launch on the launching stream (run_graph), not inside the graph.
int get_graph(Ctx& ctx, int precision, const BatchPlan& plan, void* results, cudaGraphExec_t* out) {
    int variant = 0, grid = 0;
    int rc = launch_shape(ctx, precision, variant, grid);
    if (rc) return rc;
    GraphKey key{precision, variant, grid, plan.n, 0u, ctx.d_contracts.ptr,
                 ctx.d_prefix.ptr, ctx.d_partials.ptr, results};
    for (auto& g : ctx.graphs) {
        if (g.key == key && g.exec) {
            *out = g.exec;
            return MCD_OK;
        }
    }
    cudaGetLastError();  // launches below report their own status only
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "begin capture");
    uint32_t* ticket = ctx.d_flags;
    uint32_t* err = ctx.d_flags + 1;
    cudaError_t e1 = cudaMemsetAsync(ctx.d_flags, 0, 2 * sizeof(uint32_t), ctx.stream);
    cudaError_t e2 = launch_path_kernel(precision, variant, grid,
                                        static_cast<const DevContract*>(ctx.d_contracts.ptr),
                                        static_cast<int>(plan.n),
                                        static_cast<const uint32_t*>(ctx.d_prefix.ptr), ticket,
                                        static_cast<Welford*>(ctx.d_partials.ptr), err, ctx.stream);
    cudaError_t e3 = launch_merge_kernel(static_cast<const DevContract*>(ctx.d_contracts.ptr),
                                         static_cast<int>(plan.n),
                                         static_cast<const uint32_t*>(ctx.d_prefix.ptr),
                                         static_cast<const Welford*>(ctx.d_partials.ptr), results,
                                         ctx.stream);
    e = cudaStreamEndCapture(ctx.stream, &graph);
    const char* stage[3] = {"capture: reset flags", "capture: path kernel", "capture: merge kernel"};
    const cudaError_t es[3] = {e1, e2, e3};
    for (int i = 0; i < 3; ++i) {
        if (es[i] != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            return ctx.cuda_fail(es[i], stage[i]);
        }
    }
    if (e != cudaSuccess) return ctx.cuda_fail(e, "end capture");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "instantiate graph");
    // Keep a small cache; evict the oldest.
    if (ctx.graphs.size() >= 8) {
        cudaGraphExecDestroy(ctx.graphs.front().exec);
        ctx.graphs.erase(ctx.graphs.begin());
    }
    ctx.graphs.push_back(CachedGraph{key, exec});
    *out = exec;
    return MCD_OK;
}

int run_graph(Ctx& ctx, cudaGraphExec_t exec, cudaStream_t stream) {
    int pair = -1;
    int rc = ctx.record_start(stream, &pair);
    if (rc) return rc;
    cudaError_t e = cudaGraphLaunch(exec, stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "graph launch");
    return ctx.record_stop(stream, pair);
}

// Folds completed launch intervals into the running kernel time and checks
// the device error word.  Requires the stream to be idle.
int collect_after_sync(Ctx& ctx) {
    ctx.collect_timing(false);
    uint32_t flags[2] = {0, 0};
    cudaError_t e = cudaMemcpy(flags, ctx.d_flags, sizeof flags, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "read error word");
    if (flags[1] != 0) return ctx.fail(MCD_ERR_CUDA, "path kernel reported an inconsistent work item");
    return MCD_OK;
}

int price_batch_host(Ctx& ctx, const mcd_contract* contracts, size_t n, int precision,
                     mcd_mc_result* results) {
    BatchPlan& plan = ctx.host_plan;
    int rc = plan_batch(ctx, contracts, n, plan);
    if (rc) return rc;
    if (n == 0) return MCD_OK;
    rc = upload_plan(ctx, plan);
    if (rc) return rc;
    cudaGraphExec_t exec = nullptr;
    rc = get_graph(ctx, precision, plan, ctx.d_results.ptr, &exec);
    if (rc) return rc;
    rc = run_graph(ctx, exec, ctx.stream);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(results, ctx.d_results.ptr, sizeof(mcd_mc_result) * n,
                                    cudaMemcpyDeviceToHost, ctx.stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "copy results");
    e = cudaStreamSynchronize(ctx.stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "batch execution");
    return collect_after_sync(ctx);
}

}  // namespace mcdg

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
int abi_exception(mcd_ctx* handle) noexcept {
    int code = MCD_ERR_INVALID_ARGUMENT;
    const char* msg = "internal error";
    try {
        throw;
    } catch (const std::bad_alloc&) {
        code = MCD_ERR_OUT_OF_MEMORY;
        msg = "host out of memory";
    } catch (const std::exception& e) {
        msg = e.what();
    } catch (...) {
    }
    try {
        if (handle) reinterpret_cast<Ctx*>(handle)->error = std::string("internal error: ") + msg;
        else g_create_error = std::string("internal error: ") + msg;
    } catch (...) {
    }
    return code;
}

extern "C" {

int mcd_abi_version(void) { return MCD_GPU_ABI_VERSION; }

int mcd_create(int device, mcd_ctx** out) try {
    if (!out) {
        g_create_error = "out must not be NULL";
        return MCD_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        g_create_error = std::string("no CUDA device: ") + cudaGetErrorString(e);
        return MCD_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) {
        g_create_error = "device index out of range";
        return MCD_ERR_INVALID_ARGUMENT;
    }
    Ctx* ctx = new Ctx();
    ctx->device = device;
    auto init_fail = [&](cudaError_t err, const char* where) {
        g_create_error = std::string(where) + ": " + cudaGetErrorString(err);
        delete ctx;
        return err == cudaErrorMemoryAllocation ? MCD_ERR_OUT_OF_MEMORY : MCD_ERR_CUDA;
    };
    if ((e = cudaSetDevice(device)) != cudaSuccess) return init_fail(e, "cudaSetDevice");
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, device)) != cudaSuccess) return init_fail(e, "properties");
    if (prop.major < 10) {
        g_create_error = "this library is built for sm_103a (GB300); device is sm_" +
                         std::to_string(prop.major) + std::to_string(prop.minor);
        delete ctx;
        return MCD_ERR_UNSUPPORTED;
    }
    ctx->sm_count = prop.multiProcessorCount;
    if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return init_fail(e, "stream");
    for (int i = 0; i < Ctx::kEventPairs; ++i) {
        if ((e = cudaEventCreate(&ctx->ev_start[i])) != cudaSuccess) return init_fail(e, "event");
        if ((e = cudaEventCreate(&ctx->ev_stop[i])) != cudaSuccess) return init_fail(e, "event");
    }
    if ((e = cudaMalloc(reinterpret_cast<void**>(&ctx->d_flags), 64)) != cudaSuccess)
        return init_fail(e, "flags");
    cudaMemset(ctx->d_flags, 0, 64);
    *out = reinterpret_cast<mcd_ctx*>(ctx);
    return MCD_OK;
} catch (...) {
    return abi_exception(nullptr);
}

void mcd_destroy(mcd_ctx* handle) {
    if (!handle) return;
    Ctx* ctx = reinterpret_cast<Ctx*>(handle);
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    delete ctx;
}

const char* mcd_last_error(const mcd_ctx* handle) {
    if (!handle) return g_create_error.c_str();
    return reinterpret_cast<const Ctx*>(handle)->error.c_str();
}

int mcd_synchronize(mcd_ctx* handle) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "synchronize");
    return collect_after_sync(*ctx);
} catch (...) {
    return abi_exception(handle);
}

int mcd_price_batch(mcd_ctx* handle, const mcd_contract* contracts, size_t n, int precision,
                    mcd_mc_result* results) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (n > 0 && (!contracts || !results)) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "null array");
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    return price_batch_host(*ctx, contracts, n, precision, results);
} catch (...) {
    return abi_exception(handle);
}

int mcd_price_batch_device(mcd_ctx* handle, const mcd_contract* contracts, size_t n, int precision,
                           mcd_mc_result* results, void* stream) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (n > 0 && (!contracts || !results)) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "null array");
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    if (n == 0) return MCD_OK;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    // The plan is keyed on the contract array's content, not only its
    // address: a digest of the caller's records is computed on the caller's
    // stream (after whatever the caller queued there, e.g. an in-place rewrite
    // of the contracts) and read back; a changed digest re-plans.  Waiting for
    // it also retires this context's previous launches on that stream, so a
    // new plan never overwrites buffers a running graph still reads.
    static_assert(sizeof(mcd_contract) % sizeof(uint64_t) == 0, "contract records are whole words");
    uint64_t* d_digest = reinterpret_cast<uint64_t*>(ctx->d_flags + 4);
    cudaError_t e = launch_words_digest(reinterpret_cast<const uint64_t*>(contracts),
                                        n * (sizeof(mcd_contract) / sizeof(uint64_t)), d_digest, s);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "contract digest");
    uint64_t digest = 0;
    e = cudaMemcpyAsync(&digest, d_digest, sizeof digest, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "read contract digest");
    DevicePlanKey key{contracts, n, precision, digest};
    if (!(ctx->device_plan_valid && ctx->device_plan_key == key)) {
        std::vector<mcd_contract> host(n);
        e = cudaMemcpyAsync(host.data(), contracts, sizeof(mcd_contract) * n, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "read device contracts");
        int rc = plan_batch(*ctx, host.data(), n, ctx->device_plan);
        if (rc) return rc;
        rc = upload_plan(*ctx, ctx->device_plan);
        if (rc) return rc;
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "upload plan");
        ctx->device_plan_key = key;
        ctx->device_plan_valid = true;
    }
    cudaGraphExec_t exec = nullptr;
    int rc = get_graph(*ctx, precision, ctx->device_plan, results, &exec);
    if (rc) return rc;
    return run_graph(*ctx, exec, s);
} catch (...) {
    return abi_exception(handle);
}

int mcd_batch_invalidate(mcd_ctx* handle) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    ctx->device_plan_valid = false;
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_set_launch_shape(mcd_ctx* handle, int precision, int variant, int ctas_per_sm) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "bad precision");
    if (variant < 0 || variant >= kNumVariants) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "variant must be 0..4");
    if (ctas_per_sm < 0 || ctas_per_sm > 64) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "ctas_per_sm must be 0..64");
    ctx->shape[precision].variant = variant;
    ctx->shape[precision].ctas_per_sm = ctas_per_sm;
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_get_launch_shape(mcd_ctx* handle, int precision, int* variant, int* ctas_per_sm) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "bad precision");
    int v = 0, grid = 0;
    int rc = launch_shape(*ctx, precision, v, grid);
    if (rc) return rc;
    if (variant) *variant = v;
    if (ctas_per_sm) *ctas_per_sm = grid / ctx->sm_count;
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_autotune(mcd_ctx* handle, const mcd_contract* contracts, size_t n, int precision,
                 int* variant_out, int* ctas_out, double* best_ms_out) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "bad precision");
    if (n == 0 || !contracts) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "empty tuning batch");
    BatchPlan plan;
    int rc = plan_batch(*ctx, contracts, n, plan);
    if (rc) return rc;
    rc = upload_plan(*ctx, plan);
    if (rc) return rc;
    const LaunchShape saved = ctx->shape[precision];
    double best = 1e300;
    LaunchShape best_shape = saved;
    for (int v = 0; v < kNumVariants; ++v) {
        int occ = 0;
        cudaError_t e = path_kernel_occupancy(precision, v, &occ);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "occupancy");
        if (occ < 1) continue;
        std::vector<int> cands;
        for (int c : {occ, (3 * occ + 3) / 4, (occ + 1) / 2, 2 * occ})
            if (c >= 1 && std::find(cands.begin(), cands.end(), c) == cands.end()) cands.push_back(c);
        for (int c : cands) {
            ctx->shape[precision] = LaunchShape{v, c};
            cudaGraphExec_t exec = nullptr;
            rc = get_graph(*ctx, precision, plan, ctx->d_results.ptr, &exec);
            if (rc) { ctx->shape[precision] = saved; return rc; }
            double total = 0.0;
            for (int rep = 0; rep < 3; ++rep) {
                rc = run_graph(*ctx, exec, ctx->stream);
                if (rc) { ctx->shape[precision] = saved; return rc; }
                e = cudaStreamSynchronize(ctx->stream);
                if (e != cudaSuccess) { ctx->shape[precision] = saved; return ctx->cuda_fail(e, "tuning run"); }
                ctx->collect_timing(true);
                if (rep > 0) total += ctx->last_ms;  // first run warms up
            }
            const double avg = total / 2.0;
            if (avg < best) {
                best = avg;
                best_shape = LaunchShape{v, c};
            }
        }
    }
    ctx->shape[precision] = best_shape;
    if (variant_out) *variant_out = best_shape.variant;
    if (ctas_out) *ctas_out = best_shape.ctas_per_sm;
    if (best_ms_out) *best_ms_out = best;
    return collect_after_sync(*ctx);
} catch (...) {
    return abi_exception(handle);
}

int mcd_kernel_timing(mcd_ctx* handle, int reset, double* avg_ms, uint64_t* launches) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    ctx->collect_timing(true);
    if (avg_ms) *avg_ms = ctx->kernel_launches ? ctx->kernel_ms_sum / ctx->kernel_launches : 0.0;
    if (launches) *launches = ctx->kernel_launches;
    if (reset) {
        ctx->kernel_ms_sum = 0.0;
        ctx->kernel_launches = 0;
    }
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

// ---- single-contract entry points --------------------------------------------
static int price_one(mcd_ctx* handle, const mcd_contract& c, int precision, mcd_mc_result* out) {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (!out) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "out must not be NULL");
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    return price_batch_host(*ctx, &c, 1, precision, out);
}

static mcd_contract base_contract(int product, double spot, double strike, double rate,
                                  double carry_yield, double vol, double time, int type,
                                  uint64_t path_count, uint64_t seed, const mcd_mc_options* o) {
    mcd_contract c;
    std::memset(&c, 0, sizeof c);
    c.product = product;
    c.type = type;
    c.spot = spot;
    c.strike = strike;
    c.rate = rate;
    c.carry_yield = carry_yield;
    c.vol = vol;
    c.time = time;
    c.cash_amount = 1.0;
    c.path_count = path_count;
    c.seed = seed;
    c.monitoring_points = 1;
    if (o) {
        c.antithetic = o->antithetic ? 1 : 0;
        c.control_variate = o->control_variate ? 1 : 0;
        c.brownian_bridge = o->brownian_bridge ? 1 : 0;
    }
    return c;
}

int mcd_price_european(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                       double vol, double time, int type, uint64_t path_count, uint64_t seed,
                       const mcd_mc_options* options, int precision, mcd_mc_result* out) try {
    const mcd_contract c = base_contract(MCD_PRODUCT_EUROPEAN, spot, strike, rate, carry_yield, vol,
                                         time, type, path_count, seed, options);
    return price_one(ctx, c, precision, out);
} catch (...) {
    return abi_exception(ctx);
}

int mcd_price_digital(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                      double vol, double time, int type, int digital_style, double cash_amount,
                      uint64_t path_count, uint64_t seed, const mcd_mc_options* options,
                      int precision, mcd_mc_result* out) try {
    mcd_contract c = base_contract(MCD_PRODUCT_DIGITAL, spot, strike, rate, carry_yield, vol, time,
                                   type, path_count, seed, options);
    c.digital_style = digital_style;
    c.cash_amount = cash_amount;
    return price_one(ctx, c, precision, out);
} catch (...) {
    return abi_exception(ctx);
}

int mcd_price_asian(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                    double vol, double time, int type, int strike_style, int average_style,
                    int monitoring_points, uint64_t path_count, uint64_t seed,
                    const mcd_mc_options* options, int precision, mcd_mc_result* out) try {
    mcd_contract c = base_contract(MCD_PRODUCT_ASIAN, spot, strike, rate, carry_yield, vol, time,
                                   type, path_count, seed, options);
    c.strike_style = strike_style;
    c.average_style = average_style;
    c.monitoring_points = monitoring_points;
    return price_one(ctx, c, precision, out);
} catch (...) {
    return abi_exception(ctx);
}

int mcd_price_barrier(mcd_ctx* ctx, double spot, double strike, double barrier, double rate,
                      double carry_yield, double vol, double time, int type, int direction,
                      int knock, double rebate, int monitoring_points, uint64_t path_count,
                      uint64_t seed, const mcd_mc_options* options, int precision,
                      mcd_mc_result* out) try {
    mcd_contract c = base_contract(MCD_PRODUCT_BARRIER, spot, strike, rate, carry_yield, vol, time,
                                   type, path_count, seed, options);
    c.barrier = barrier;
    c.direction = direction;
    c.knock = knock;
    c.rebate = rebate;
    c.monitoring_points = monitoring_points;
    return price_one(ctx, c, precision, out);
} catch (...) {
    return abi_exception(ctx);
}

int mcd_price_lookback(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                       double vol, double time, int type, int strike_style, int monitoring_points,
                       uint64_t path_count, uint64_t seed, const mcd_mc_options* options,
                       int precision, mcd_mc_result* out) try {
    mcd_contract c = base_contract(MCD_PRODUCT_LOOKBACK, spot, strike, rate, carry_yield, vol, time,
                                   type, path_count, seed, options);
    c.strike_style = strike_style;
    c.monitoring_points = monitoring_points;
    return price_one(ctx, c, precision, out);
} catch (...) {
    return abi_exception(ctx);
}

// ---- draws ---------------------------------------------------------------------
int mcd_philox(mcd_ctx* handle, const uint32_t* counters, const uint32_t* keys, size_t n,
               uint32_t* out) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (n == 0) return MCD_OK;
    if (!counters || !keys || !out) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "null array");
    // counters and outputs are read/written as uint4, keys as uint2: every
    // sub-buffer starts on a 256-byte boundary.
    auto align256 = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
    const size_t cb = 16 * n, kb = 8 * n;
    const size_t off_keys = align256(cb), off_out = align256(off_keys + kb);
    int rc = ctx->reserve(ctx->d_scratch, off_out + cb, "philox buffers");
    if (rc) return rc;
    char* base = static_cast<char*>(ctx->d_scratch.ptr);
    cudaError_t e = cudaMemcpyAsync(base, counters, cb, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + off_keys, keys, kb, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = launch_philox_kernel(reinterpret_cast<const uint32_t*>(base),
                                 reinterpret_cast<const uint32_t*>(base + off_keys), n,
                                 reinterpret_cast<uint32_t*>(base + off_out), ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, base + off_out, cb, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "philox");
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_draws(mcd_ctx* handle, uint64_t seed, uint64_t path_begin, uint64_t n_paths,
              uint32_t draw_begin, uint32_t n_draws, int stream_id, int precision, double* out) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (stream_id != 0 && stream_id != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "stream_id must be 0 or 1");
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "bad precision");
    const uint64_t total = n_paths * n_draws;
    if (total == 0) return MCD_OK;
    if (!out) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "null output");
    if (n_draws != 0 && total / n_draws != n_paths) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "size overflow");
    if (total > (1ull << 31)) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "at most 2^31 draws per call");
    int rc = ctx->reserve(ctx->d_scratch, sizeof(double) * total, "draw buffer");
    if (rc) return rc;
    cudaError_t e = launch_draws_kernel(seed, path_begin, n_paths, draw_begin, n_draws, stream_id,
                                        precision, static_cast<double*>(ctx->d_scratch.ptr), ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, ctx->d_scratch.ptr, sizeof(double) * total, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "draws");
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

}  // extern "C"

namespace mcdg {

int Ctx::record_start(cudaStream_t s, int* pair) {
    if (ev_count == kEventPairs) collect_timing(true);  // ring full: retire the oldest
    if (ev_count == kEventPairs) return fail(MCD_ERR_CUDA, "timing ring exhausted");
    // Free pair: the one after the newest pending entry.
    const int idx = (ev_head + ev_count) % kEventPairs;
    cudaError_t e = cudaEventRecord(ev_start[idx], s);
    if (e != cudaSuccess) return cuda_fail(e, "record start event");
    *pair = idx;
    return MCD_OK;
}

int Ctx::record_stop(cudaStream_t s, int pair) {
    cudaError_t e = cudaEventRecord(ev_stop[pair], s);
    if (e != cudaSuccess) return cuda_fail(e, "record stop event");
    ev_pending[(ev_head + ev_count) % kEventPairs] = pair;
    ++ev_count;
    return MCD_OK;
}

void Ctx::collect_timing(bool block) {
    while (ev_count > 0) {
        const int pair = ev_pending[ev_head];
        if (block) {
            if (cudaEventSynchronize(ev_stop[pair]) != cudaSuccess) { cudaGetLastError(); break; }
        } else if (cudaEventQuery(ev_stop[pair]) != cudaSuccess) {
            cudaGetLastError();
            break;
        }
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ev_start[pair], ev_stop[pair]) == cudaSuccess) {
            kernel_ms_sum += ms;
            kernel_launches += 1;
            last_ms = ms;
        } else {
            cudaGetLastError();
        }
        ev_head = (ev_head + 1) % kEventPairs;
        --ev_count;
    }
}

int Ctx::ensure_aux() {
    if (ev_fork) return MCD_OK;
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < kAuxStreams && e == cudaSuccess; ++i) {
        e = cudaStreamCreateWithFlags(&aux_stream[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_join[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_stage[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_train[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(e, "auxiliary streams");
    return MCD_OK;
}

void Ctx::release_extensions() {
    for (DeviceBuffer& b : ext) {
        if (b.ptr) cudaFree(b.ptr);
        b.ptr = nullptr;
        b.bytes = 0;
    }
}
}  // namespace mcdg
