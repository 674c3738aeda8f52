// qmc_api.cpp -- C ABI of the Sobol quasi-Monte Carlo engine (include/mcd_gpu.h):
// direction numbers, bridge programs, batch planning and the graph launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "context.hpp"
#include "engine.hpp"
#include "mcd_gpu.h"
#include "qmc.hpp"

using namespace mcdg;

namespace {

enum { kQDirs = 27, kQProg = 28, kQConst = 29, kQDev = 30, kQPrefix = 31, kQPart = 32, kQOut = 33, kQFlags = 34 };

// ---- Sobol direction numbers ---------------------------------------------
// Dimensions 0..6 use the reference's primitive polynomials
// (src/core/sobol.cpp:22-30: degree, interior coefficients a_1..a_{s-1} as
// bits 0..s-2); further dimensions continue with every remaining primitive
// polynomial in ascending (degree, interior bits) order.  All use the
// reference's initial direction numbers m_1..m_s = 1 and the Bratley-Fox
// recurrence (sobol.cpp:40-65): m_k = m_{k-s} ^ (m_{k-s} << s)
// ^ sum_j a_j (m_{k-j} << j).
constexpr unsigned kRefDegree[7] = {0, 1, 2, 3, 4, 5, 6};
constexpr uint32_t kRefInterior[7] = {0u, 0u, 1u, 1u, 1u, 2u, 1u};

// The multiplicative order of x modulo the polynomial is 2^s - 1.
bool primitive(unsigned s, uint32_t interior) {
    uint32_t poly = (1u << s) | 1u;
    for (unsigned j = 1; j < s; ++j)
        if ((interior >> (j - 1)) & 1u) poly |= 1u << (s - j);
    const uint32_t period = (1u << s) - 1u;
    uint32_t r = 1u;
    for (uint32_t k = 1; k <= period; ++k) {
        r <<= 1;
        if (r & (1u << s)) r ^= poly;
        if (r == 1u) return k == period;
    }
    return false;
}

// Direction numbers (kSobolDims x 32, dims-major) followed by the warp
// decomposition's Y table (kSobolDims x 32 lanes).
std::vector<uint32_t> sobol_directions() {
    std::vector<std::pair<unsigned, uint32_t>> polys;
    for (int d = 0; d < 7; ++d) polys.emplace_back(kRefDegree[d], kRefInterior[d]);
    for (unsigned s = 1; polys.size() < static_cast<size_t>(kSobolDims) && s < 20; ++s) {
        const uint32_t masks = s > 1 ? (1u << (s - 1)) : 1u;
        for (uint32_t m = 0; m < masks && polys.size() < static_cast<size_t>(kSobolDims); ++m) {
            bool in_table = false;
            for (int k = 1; k < 7; ++k)
                if (kRefDegree[k] == s && kRefInterior[k] == m) in_table = true;
            if (!in_table && primitive(s, m)) polys.emplace_back(s, m);
        }
    }
    std::vector<uint32_t> dirs(static_cast<size_t>(kSobolDims) * kSobolBits, 0u);
    for (int d = 0; d < kSobolDims; ++d) {
        const unsigned s = polys[d].first;
        const uint32_t mask = polys[d].second;
        uint32_t m[kSobolBits + 1] = {};
        for (unsigned k = 1; k <= kSobolBits; ++k) {
            if (s == 0 || k <= s) {
                m[k] = 1u;
            } else {
                uint32_t mk = m[k - s] ^ (m[k - s] << s);
                for (unsigned j = 1; j < s; ++j)
                    if ((mask >> (j - 1)) & 1u) mk ^= m[k - j] << j;
                m[k] = mk;
            }
            dirs[static_cast<size_t>(d) * kSobolBits + (k - 1)] = m[k] << (kSobolBits - k);
        }
    }
    // Y table of the warp decomposition (qmc.cu, SobolLane): for lane l the
    // low index part is (l + 1) mod 32; Y[d][l] = the coordinate bits of its
    // Gray code in dimension d.
    dirs.resize(static_cast<size_t>(kSobolDims) * kSobolBits * 2);
    uint32_t* y = dirs.data() + static_cast<size_t>(kSobolDims) * kSobolBits;
    for (int d = 0; d < kSobolDims; ++d)
        for (uint32_t l = 0; l < 32; ++l) {
            const uint32_t low = (l + 1) & 31u, g = low ^ (low >> 1);
            uint32_t x = 0;
            for (int b = 0; b < 5; ++b)
                if ((g >> b) & 1u) x ^= dirs[static_cast<size_t>(d) * kSobolBits + b];
            y[static_cast<size_t>(d) * 32 + l] = x;
        }
    return dirs;
}

// ---- bridge programs --------------------------------------------------------
// brownian_bridge_path.cpp:33-66: breadth-first bisection gives each point its
// draw number; the program lists the points in depth-first pre-order.
void build_program(int n, std::vector<BridgeNode>& out) {
    std::vector<int> draw_of(n, -1), depth_of(n, 0);
    std::vector<std::pair<int, int>> interval(n, {-1, -1});
    draw_of[n - 1] = 0;
    std::deque<std::pair<int, int>> queue{{-1, n - 1}};
    int draw = 1;
    while (!queue.empty() && draw < n) {
        const auto [l, r] = queue.front();
        queue.pop_front();
        if (r - l <= 1) continue;
        const int mid = (l + r) / 2;
        draw_of[mid] = draw++;
        interval[mid] = {l, r};
        queue.push_back({l, mid});
        queue.push_back({mid, r});
    }
    auto slot = [&](int t) { return t < 0 ? 0 : depth_of[t] + 1; };
    auto emit = [&](int m, int l, int r, int depth) {
        depth_of[m] = depth;
        BridgeNode b;
        std::memset(&b, 0, sizeof b);
        b.t_left = static_cast<int16_t>(l);
        b.t_mid = static_cast<int16_t>(m);
        b.t_right = static_cast<int16_t>(r);
        b.dim = static_cast<uint16_t>(draw_of[m]);
        b.slot_left = static_cast<uint8_t>(slot(l));
        b.slot_right = static_cast<uint8_t>(slot(r));
        b.slot_out = static_cast<uint8_t>(depth + 1);
        out.push_back(b);
    };
    // iterative pre-order over (node, interval, depth)
    struct Frame { int m, l, r, depth; };
    emit(n - 1, -1, -1, 0);
    std::vector<Frame> stack;
    if (n >= 2) stack.push_back({(n - 2) / 2, -1, n - 1, 1});
    while (!stack.empty()) {
        const Frame f = stack.back();
        stack.pop_back();
        emit(f.m, f.l, f.r, f.depth);
        // push right first so the left subtree is visited first
        if (f.r - f.m > 1) stack.push_back({(f.m + f.r) / 2, f.m, f.r, f.depth + 1});
        if (f.m - f.l > 1) stack.push_back({(f.l + f.m) / 2, f.l, f.m, f.depth + 1});
    }
}

int plan_qmc(Ctx& ctx, const mcd_contract* cs, size_t n, BatchPlan& plan, std::vector<DevQmc>& consts,
             std::vector<BridgeNode>& programs) {
    for (size_t i = 0; i < n; ++i) {
        const mcd_contract& c = cs[i];
        const std::string who = "contract " + std::to_string(i) + ": ";
        if (c.antithetic) return ctx.fail(MCD_ERR_UNSUPPORTED, who + "quasi-Monte Carlo takes no antithetic pairing");
        if (c.product == MCD_PRODUCT_ASIAN && c.control_variate && c.strike_style == MCD_FIXED &&
            c.average_style == MCD_ARITHMETIC)
            return ctx.fail(MCD_ERR_UNSUPPORTED, who + "no control variate under quasi-Monte Carlo");
        if (c.product == MCD_PRODUCT_BARRIER && c.brownian_bridge)
            return ctx.fail(MCD_ERR_UNSUPPORTED, who + "no Brownian-bridge crossing correction under quasi-Monte Carlo");
        if (c.product >= MCD_PRODUCT_ASIAN && c.monitoring_points > kSobolDims)
            return ctx.fail(MCD_ERR_INVALID_ARGUMENT, who + "monitoring_points must be <= MCD_SOBOL_MAX_DIMS (256)");
    }
    int rc = plan_batch(ctx, cs, n, plan);
    if (rc) return rc;
    std::map<int, uint32_t> offset_of;
    programs.clear();
    consts.resize(n);
    for (size_t j = 0; j < n; ++j) {
        const DevContract& d = plan.dev[j];
        const mcd_contract& in = cs[d.orig_index];
        DevQmc& q = consts[j];
        std::memset(&q, 0, sizeof q);
        q.time = in.time;
        q.vol = in.vol;
        q.drift_rate = in.rate - in.carry_yield - 0.5 * in.vol * in.vol;  // brownian_bridge_path.cpp:70
        if (d.kind == kEuropean || d.kind == kDigital) continue;
        auto it = offset_of.find(d.n_steps);
        if (it == offset_of.end()) {
            it = offset_of.emplace(d.n_steps, static_cast<uint32_t>(programs.size())).first;
            build_program(d.n_steps, programs);
        }
        q.prog_offset = it->second;
    }
    if (programs.empty()) programs.resize(1);
    return MCD_OK;
}

int qmc_batch(Ctx& ctx, const mcd_contract* cs, size_t n, int precision, mcd_mc_result* results) {
    if (precision != 0 && precision != 1) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    if (n == 0) return MCD_OK;
    if (!cs || !results) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "null array");
    BatchPlan plan;
    std::vector<DevQmc> consts;
    std::vector<BridgeNode> programs;
    int rc = plan_qmc(ctx, cs, n, plan, consts, programs);
    if (rc) return rc;
    if (!ctx.ext[kQDirs].ptr) {
        const std::vector<uint32_t> dirs = sobol_directions();
        rc = ctx.reserve(ctx.ext[kQDirs], sizeof(uint32_t) * dirs.size(), "sobol directions");
        if (rc) return rc;
        cudaError_t e = cudaMemcpy(ctx.ext[kQDirs].ptr, dirs.data(), sizeof(uint32_t) * dirs.size(),
                                   cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return ctx.cuda_fail(e, "sobol directions upload");
    }
    rc = ctx.reserve(ctx.ext[kQProg], sizeof(BridgeNode) * programs.size(), "bridge programs");
    if (!rc) rc = ctx.reserve(ctx.ext[kQConst], sizeof(DevQmc) * n, "qmc constants");
    if (!rc) rc = ctx.reserve(ctx.ext[kQDev], sizeof(DevContract) * n, "qmc contracts");
    if (!rc) rc = ctx.reserve(ctx.ext[kQPrefix], sizeof(uint32_t) * (n + 1), "qmc prefix");
    if (!rc) rc = ctx.reserve(ctx.ext[kQPart], sizeof(Welford) * std::max<uint32_t>(plan.total_items, 1), "qmc partials");
    if (!rc) rc = ctx.reserve(ctx.ext[kQOut], sizeof(mcd_mc_result) * n, "qmc results");
    if (!rc) rc = ctx.reserve(ctx.ext[kQFlags], 256, "qmc flags");
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(ctx.ext[kQProg].ptr, programs.data(), sizeof(BridgeNode) * programs.size(),
                                    cudaMemcpyHostToDevice, ctx.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx.ext[kQConst].ptr, consts.data(), sizeof(DevQmc) * n, cudaMemcpyHostToDevice, ctx.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx.ext[kQDev].ptr, plan.dev.data(), sizeof(DevContract) * n, cudaMemcpyHostToDevice,
                            ctx.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx.ext[kQPrefix].ptr, plan.prefix.data(), sizeof(uint32_t) * (n + 1),
                            cudaMemcpyHostToDevice, ctx.stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "qmc upload");
    int blocks = 0;
    e = qmc_kernel_occupancy(precision, &blocks);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "qmc occupancy");
    const int grid = ctx.sm_count * std::max(blocks, 1);
    // one graph: reset flags, persistent QMC kernel, the path engine's merge
    cudaGetLastError();
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "qmc begin capture");
    uint32_t* flags = static_cast<uint32_t*>(ctx.ext[kQFlags].ptr);
    cudaError_t e1 = cudaMemsetAsync(flags, 0, 2 * sizeof(uint32_t), ctx.stream);
    cudaError_t e2 = launch_qmc_kernel(precision, grid, static_cast<const DevContract*>(ctx.ext[kQDev].ptr),
                                       static_cast<const DevQmc*>(ctx.ext[kQConst].ptr), static_cast<int>(n),
                                       static_cast<const uint32_t*>(ctx.ext[kQPrefix].ptr), plan.total_items,
                                       static_cast<const BridgeNode*>(ctx.ext[kQProg].ptr),
                                       static_cast<const uint32_t*>(ctx.ext[kQDirs].ptr), flags,
                                       static_cast<Welford*>(ctx.ext[kQPart].ptr), flags + 1, ctx.stream);
    cudaError_t e3 = launch_merge_kernel(static_cast<const DevContract*>(ctx.ext[kQDev].ptr), static_cast<int>(n),
                                         static_cast<const uint32_t*>(ctx.ext[kQPrefix].ptr),
                                         static_cast<const Welford*>(ctx.ext[kQPart].ptr), ctx.ext[kQOut].ptr,
                                         ctx.stream);
    e = cudaStreamEndCapture(ctx.stream, &graph);
    for (cudaError_t ei : {e1, e2, e3}) {
        if (ei != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            return ctx.cuda_fail(ei, "qmc capture");
        }
    }
    if (e != cudaSuccess) return ctx.cuda_fail(e, "qmc end capture");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "qmc instantiate");
    int pair = -1;
    rc = ctx.record_start(ctx.stream, &pair);
    if (!rc) {
        e = cudaGraphLaunch(exec, ctx.stream);
        if (e != cudaSuccess) rc = ctx.cuda_fail(e, "qmc graph launch");
    }
    if (!rc) rc = ctx.record_stop(ctx.stream, pair);
    uint32_t hflags[2] = {0, 0};
    if (!rc) {
        e = cudaMemcpyAsync(results, ctx.ext[kQOut].ptr, sizeof(mcd_mc_result) * n, cudaMemcpyDeviceToHost, ctx.stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hflags, flags, sizeof hflags, cudaMemcpyDeviceToHost, ctx.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx.stream);
        if (e != cudaSuccess) rc = ctx.cuda_fail(e, "qmc execution");
    }
    cudaGraphExecDestroy(exec);
    ctx.collect_timing(false);
    if (rc) return rc;
    if (hflags[1] != 0) return ctx.fail(MCD_ERR_CUDA, "qmc kernel reported an inconsistent work item");
    for (size_t i = 0; i < n; ++i) results[i].standard_error = 0.0;  // qmc.hpp:9-15: no standard error
    return MCD_OK;
}

mcd_contract qmc_contract(int product, double spot, double strike, double rate, double carry_yield, double vol,
                          double time, int type, uint64_t path_count) {
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
    c.monitoring_points = 1;
    c.path_count = path_count;
    return c;
}

}  // namespace

extern "C" {

int mcd_qmc_batch(mcd_ctx* handle, const mcd_contract* contracts, size_t n, int precision, mcd_mc_result* results) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    return qmc_batch(*ctx, contracts, n, precision, results);
} catch (...) {
    return abi_exception(handle);
}

int mcd_qmc_sobol_european(mcd_ctx* handle, double spot, double strike, double rate, double carry_yield, double vol,
                           double time, int type, uint64_t path_count, int precision, double* price) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (!price) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "price must not be NULL");
    const mcd_contract c = qmc_contract(MCD_PRODUCT_EUROPEAN, spot, strike, rate, carry_yield, vol, time, type,
                                        path_count);
    mcd_mc_result r;
    const int rc = qmc_batch(*ctx, &c, 1, precision, &r);
    if (!rc) *price = r.price;
    return rc;
} catch (...) {
    return abi_exception(handle);
}

int mcd_qmc_sobol_asian(mcd_ctx* handle, double spot, double strike, double rate, double carry_yield, double vol,
                        double time, int type, int strike_style, int monitoring_points, uint64_t path_count,
                        int precision, double* price) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (!price) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "price must not be NULL");
    mcd_contract c = qmc_contract(MCD_PRODUCT_ASIAN, spot, strike, rate, carry_yield, vol, time, type, path_count);
    c.strike_style = strike_style;
    c.average_style = MCD_ARITHMETIC;
    c.monitoring_points = monitoring_points;
    mcd_mc_result r;
    const int rc = qmc_batch(*ctx, &c, 1, precision, &r);
    if (!rc) *price = r.price;
    return rc;
} catch (...) {
    return abi_exception(handle);
}

int mcd_sobol_points(mcd_ctx* handle, unsigned dim_begin, unsigned n_dims, uint64_t index_begin, uint64_t n_indices,
                     double* out) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (!out) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "out must not be NULL");
    if (dim_begin + static_cast<uint64_t>(n_dims) > static_cast<uint64_t>(kSobolDims))
        return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "dimensions must be < MCD_SOBOL_MAX_DIMS (256)");
    if (n_indices * n_dims > (1ull << 28)) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "at most 2^28 points per call");
    if (n_indices == 0 || n_dims == 0) return MCD_OK;
    if (!ctx->ext[kQDirs].ptr) {
        const std::vector<uint32_t> dirs = sobol_directions();
        int rc = ctx->reserve(ctx->ext[kQDirs], sizeof(uint32_t) * dirs.size(), "sobol directions");
        if (rc) return rc;
        cudaError_t e = cudaMemcpy(ctx->ext[kQDirs].ptr, dirs.data(), sizeof(uint32_t) * dirs.size(),
                                   cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "sobol directions upload");
    }
    const size_t bytes = sizeof(double) * n_indices * n_dims;
    int rc = ctx->reserve(ctx->d_scratch, bytes, "sobol output");
    if (rc) return rc;
    cudaError_t e = launch_sobol_points(static_cast<const uint32_t*>(ctx->ext[kQDirs].ptr), dim_begin, n_dims,
                                        index_begin, n_indices, static_cast<double*>(ctx->d_scratch.ptr), ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, ctx->d_scratch.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "sobol points");
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

}  // extern "C"
