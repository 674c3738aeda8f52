// greeks_api.cpp -- C ABI of the sensitivity engine (include/mcd_gpu.h):
// batched risk in one graph launch, and the reference's Greeks entry points
// (src/greeks/{finite_difference,likelihood_ratio,pathwise}.cpp) on top of it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <string>
#include <vector>

#include "context.hpp"
#include "engine.hpp"
#include "greeks.hpp"
#include "mcd_gpu.h"

using namespace mcdg;

namespace {

enum { kGDev = 21, kGConst = 22, kGPrefix = 23, kGPart = 24, kGOut = 25, kGFlags = 26 };

// Bits of mcd_greeks_result::defined.
uint32_t defined_bits(int kind) {
    uint32_t bits = 0xFu | (0xFu << kGLrDelta);  // price, finite differences, LR delta..rho
    if (kind == kEuropean || kind == kAsianArith || kind == kAsianGeo) bits |= 0x7u << kGPwDelta;
    if (kind == kEuropean || kind == kDigital) bits |= 1u << kGLrTheta;
    return bits;
}

int plan_greeks(Ctx& ctx, const mcd_contract* cs, size_t n, double spot_rel, double vol_rel, BatchPlan& plan,
                std::vector<DevGreeks>& consts) {
    if (!(spot_rel > 0.0 && spot_rel < 1.0) || !(vol_rel > 0.0 && vol_rel < 1.0))
        return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "bump sizes must be in (0, 1) relative to spot and vol");
    for (size_t i = 0; i < n; ++i) {
        const mcd_contract& c = cs[i];
        if (c.antithetic)
            return ctx.fail(MCD_ERR_UNSUPPORTED, "contract " + std::to_string(i) + ": Greeks take no antithetic pairing");
        if (c.product == MCD_PRODUCT_ASIAN && c.control_variate && c.strike_style == MCD_FIXED &&
            c.average_style == MCD_ARITHMETIC)
            return ctx.fail(MCD_ERR_UNSUPPORTED, "contract " + std::to_string(i) + ": no Greeks for the control-variate Asian");
        if (c.product == MCD_PRODUCT_BARRIER && c.brownian_bridge)
            return ctx.fail(MCD_ERR_UNSUPPORTED, "contract " + std::to_string(i) + ": no Greeks for the Brownian-bridge barrier");
    }
    int rc = plan_batch(ctx, cs, n, plan);
    if (rc) return rc;
    consts.resize(n);
    for (size_t j = 0; j < n; ++j) {
        const DevContract& d = plan.dev[j];
        const mcd_contract& in = cs[d.orig_index];
        DevGreeks& g = consts[j];
        std::memset(&g, 0, sizeof g);
        const bool terminal = d.kind == kEuropean || d.kind == kDigital;
        g.vol = in.vol;
        g.time = in.time;
        g.rate = in.rate;
        g.dt = terminal ? in.time : in.time / static_cast<double>(in.monitoring_points);
        g.sqrt_dt = std::sqrt(g.dt);
        g.mu = in.rate - in.carry_yield - 0.5 * in.vol * in.vol;
        g.h_spot = spot_rel * in.spot;
        g.h_vol = vol_rel * in.vol;
        const double vu = in.vol + g.h_vol, vd = in.vol - g.h_vol;
        g.drift_up = (in.rate - in.carry_yield - 0.5 * vu * vu) * g.dt;
        g.vs_up = vu * std::sqrt(g.dt);
        g.drift_dn = (in.rate - in.carry_yield - 0.5 * vd * vd) * g.dt;
        g.vs_dn = vd * std::sqrt(g.dt);
        if (in.product == MCD_PRODUCT_BARRIER) {
            g.log_h_rel_up = std::log(in.barrier / (in.spot + g.h_spot));
            g.log_h_rel_dn = std::log(in.barrier / (in.spot - g.h_spot));
        }
        g.inv_2hs = 1.0 / (2.0 * g.h_spot);
        g.inv_hs2 = 1.0 / (g.h_spot * g.h_spot);
        g.inv_2hv = 1.0 / (2.0 * g.h_vol);
        g.lr_delta_scale = 1.0 / (in.spot * in.vol * g.sqrt_dt);
        g.lr_gamma_scale = 1.0 / (in.spot * in.spot * in.vol * in.vol * g.dt);
        g.sqrt_dt_over_vol = g.sqrt_dt / in.vol;
        g.inv_vol = 1.0 / in.vol;
        g.inv_n = 1.0 / static_cast<double>(d.n_steps);
        g.inv_spot = 1.0 / in.spot;
        g.inv_2t = 1.0 / (2.0 * in.time);
        g.mu_over_vol_sqrt_t = g.mu / (in.vol * g.sqrt_dt);
        // The vol-bump exponent is h_vol D - h_vol^2 i dt / 2 with |D| below
        // 8 sqrt(T) + vol T on all but > 8-sigma paths.
        g.vol_series = g.h_vol * (8.0 * std::sqrt(in.time) + in.vol * in.time) <= 1e-2 ? 1 : 0;
    }
    return MCD_OK;
}

int greeks_grid(Ctx& ctx, int precision, int& variant, int& grid) {
    const LaunchShape& s = ctx.greeks_shape[precision];
    variant = s.variant;
    int blocks = 0;
    cudaError_t e = greeks_kernel_occupancy(precision, variant, &blocks);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "greeks occupancy");
    int per_sm = s.ctas_per_sm > 0 ? s.ctas_per_sm : blocks;
    grid = ctx.sm_count * std::max(per_sm, 1);
    return MCD_OK;
}

// Uploads the plan and captures (or reuses) the graph: reset ticket and
// error word, sensitivity kernel, merge.
int prepare_greeks(Ctx& ctx, int precision, const BatchPlan& plan, const std::vector<DevGreeks>& consts,
                   cudaGraphExec_t* out) {
    const size_t n = plan.n;
    int rc = ctx.reserve(ctx.ext[kGDev], sizeof(DevContract) * n, "greeks contracts");
    if (!rc) rc = ctx.reserve(ctx.ext[kGConst], sizeof(DevGreeks) * n, "greeks constants");
    if (!rc) rc = ctx.reserve(ctx.ext[kGPrefix], sizeof(uint32_t) * (n + 1), "greeks prefix");
    if (!rc) rc = ctx.reserve(ctx.ext[kGPart], sizeof(Welford) * kNumGreeks * std::max<uint32_t>(plan.total_items, 1),
                              "greeks partials");
    if (!rc) rc = ctx.reserve(ctx.ext[kGOut], sizeof(double) * kGreeksOutStride * n, "greeks results");
    if (!rc) rc = ctx.reserve(ctx.ext[kGFlags], 256, "greeks flags");
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(ctx.ext[kGDev].ptr, plan.dev.data(), sizeof(DevContract) * n,
                                    cudaMemcpyHostToDevice, ctx.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx.ext[kGConst].ptr, consts.data(), sizeof(DevGreeks) * n, cudaMemcpyHostToDevice,
                            ctx.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx.ext[kGPrefix].ptr, plan.prefix.data(), sizeof(uint32_t) * (n + 1),
                            cudaMemcpyHostToDevice, ctx.stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "greeks upload");
    int variant = 0, grid = 0;
    rc = greeks_grid(ctx, precision, variant, grid);
    if (rc) return rc;
    const GraphKey key{precision, variant, grid, n, plan.total_items, ctx.ext[kGDev].ptr, ctx.ext[kGPrefix].ptr,
                       ctx.ext[kGPart].ptr, ctx.ext[kGOut].ptr};
    if (ctx.greeks_graph && ctx.greeks_key == key) {
        *out = ctx.greeks_graph;
        return MCD_OK;
    }
    if (ctx.greeks_graph) {
        cudaGraphExecDestroy(ctx.greeks_graph);
        ctx.greeks_graph = nullptr;
    }
    cudaGetLastError();
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "greeks begin capture");
    uint32_t* flags = static_cast<uint32_t*>(ctx.ext[kGFlags].ptr);
    cudaError_t e1 = cudaMemsetAsync(flags, 0, 2 * sizeof(uint32_t), ctx.stream);
    cudaError_t e2 = launch_greeks_kernel(precision, variant, grid, static_cast<const DevContract*>(ctx.ext[kGDev].ptr),
                                          static_cast<const DevGreeks*>(ctx.ext[kGConst].ptr), static_cast<int>(n),
                                          static_cast<const uint32_t*>(ctx.ext[kGPrefix].ptr), plan.total_items,
                                          flags, static_cast<Welford*>(ctx.ext[kGPart].ptr), flags + 1, ctx.stream);
    cudaError_t e3 = launch_greeks_merge(static_cast<const DevContract*>(ctx.ext[kGDev].ptr), static_cast<int>(n),
                                         static_cast<const uint32_t*>(ctx.ext[kGPrefix].ptr),
                                         static_cast<const Welford*>(ctx.ext[kGPart].ptr),
                                         static_cast<double*>(ctx.ext[kGOut].ptr), ctx.stream);
    e = cudaStreamEndCapture(ctx.stream, &graph);
    for (cudaError_t ei : {e1, e2, e3}) {
        if (ei != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            return ctx.cuda_fail(ei, "greeks capture");
        }
    }
    if (e != cudaSuccess) return ctx.cuda_fail(e, "greeks end capture");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "greeks instantiate");
    ctx.greeks_graph = exec;
    ctx.greeks_key = key;
    *out = exec;
    return MCD_OK;
}

int run_greeks(Ctx& ctx, cudaGraphExec_t exec, size_t n, std::vector<double>& out) {
    int pair = -1;
    int rc = ctx.record_start(ctx.stream, &pair);
    if (rc) return rc;
    cudaError_t e = cudaGraphLaunch(exec, ctx.stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "greeks graph launch");
    rc = ctx.record_stop(ctx.stream, pair);
    if (rc) return rc;
    out.assign(kGreeksOutStride * n, 0.0);
    uint32_t flags[2] = {0, 0};
    e = cudaMemcpyAsync(out.data(), ctx.ext[kGOut].ptr, sizeof(double) * out.size(), cudaMemcpyDeviceToHost,
                        ctx.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(flags, ctx.ext[kGFlags].ptr, sizeof flags, cudaMemcpyDeviceToHost, ctx.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx.stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "greeks execution");
    ctx.collect_timing(false);
    if (flags[1] != 0) return ctx.fail(MCD_ERR_CUDA, "greeks kernel reported an inconsistent work item");
    return MCD_OK;
}

int greeks_batch(Ctx& ctx, const mcd_contract* cs, size_t n, double spot_rel, double vol_rel, int precision,
                 mcd_greeks_result* results) {
    if (precision != 0 && precision != 1) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    if (n == 0) return MCD_OK;
    if (!cs || !results) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "null array");
    BatchPlan plan;
    std::vector<DevGreeks> consts;
    int rc = plan_greeks(ctx, cs, n, spot_rel, vol_rel, plan, consts);
    if (rc) return rc;
    cudaGraphExec_t exec = nullptr;
    rc = prepare_greeks(ctx, precision, plan, consts, &exec);
    if (rc) return rc;
    std::vector<double> out;
    rc = run_greeks(ctx, exec, n, out);
    if (rc) return rc;
    std::vector<int> kind_of(n, 0);
    for (const DevContract& d : plan.dev) kind_of[d.orig_index] = d.kind;
    for (size_t i = 0; i < n; ++i) {
        const double* o = out.data() + kGreeksOutStride * i;
        mcd_greeks_result& r = results[i];
        std::memset(&r, 0, sizeof r);
        mcd_greek* g = &r.price;  // the twelve mcd_greek fields are consecutive
        r.defined = defined_bits(kind_of[i]);
        for (int q = 0; q < kNumGreeks; ++q) {
            if (r.defined & (1u << q)) {
                g[q].value = o[2 * q];
                g[q].standard_error = o[2 * q + 1];
            }
        }
        r.path_count = static_cast<uint64_t>(o[2 * kNumGreeks]);
    }
    return MCD_OK;
}

static_assert(offsetof(mcd_greeks_result, lr_theta) == sizeof(mcd_greek) * kGLrTheta,
              "mcd_greeks_result fields follow the kernel's output order");

mcd_contract make_contract(int product, double spot, double strike, double rate, double carry_yield, double vol,
                           double time, int type, uint64_t path_count, uint64_t seed) {
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
    c.seed = seed;
    return c;
}

// One contract through the batch engine; the FD bumps are irrelevant here.
int greeks_one(mcd_ctx* handle, const mcd_contract& c, int precision, mcd_greeks_result* r) {
    MCD_CTX_OR_FAIL(handle, ctx);
    return greeks_batch(*ctx, &c, 1, 1e-4, 1e-4, precision, r);
}

void to_lr(const mcd_greeks_result& r, bool has_theta, mcd_lr_greeks* out) {
    std::memset(out, 0, sizeof *out);
    out->delta = r.lr_delta;
    out->gamma = r.lr_gamma;
    out->vega = r.lr_vega;
    out->rho = r.lr_rho;
    if (has_theta) out->theta = r.lr_theta;
    out->has_theta = has_theta ? 1 : 0;
}

void to_pw(const mcd_greeks_result& r, mcd_pathwise_greeks* out) {
    out->delta = r.pathwise_delta;
    out->vega = r.pathwise_vega;
    out->rho = r.pathwise_rho;
}

}  // namespace

extern "C" {

int mcd_greeks_batch(mcd_ctx* handle, const mcd_contract* contracts, size_t n, double spot_bump_rel,
                     double vol_bump_rel, int precision, mcd_greeks_result* results) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    return greeks_batch(*ctx, contracts, n, spot_bump_rel, vol_bump_rel, precision, results);
} catch (...) {
    return abi_exception(handle);
}

int mcd_greeks_set_launch_shape(mcd_ctx* handle, int precision, int variant, int ctas_per_sm) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "bad precision");
    if (variant < 0 || variant >= kGreeksVariants) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "variant must be 0..3");
    if (ctas_per_sm < 0 || ctas_per_sm > 64) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "ctas_per_sm must be 0..64");
    ctx->greeks_shape[precision] = LaunchShape{variant, ctas_per_sm};
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_greeks_autotune(mcd_ctx* handle, const mcd_contract* contracts, size_t n, double spot_bump_rel,
                        double vol_bump_rel, int precision, int* variant_out, int* ctas_out, double* best_ms_out) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "bad precision");
    if (n == 0 || !contracts) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "empty tuning batch");
    BatchPlan plan;
    std::vector<DevGreeks> consts;
    int rc = plan_greeks(*ctx, contracts, n, spot_bump_rel, vol_bump_rel, plan, consts);
    if (rc) return rc;
    const LaunchShape saved = ctx->greeks_shape[precision];
    double best = 1e300;
    LaunchShape best_shape = saved;
    std::vector<double> out;
    for (int v = 0; v < kGreeksVariants; ++v) {
        int occ = 0;
        cudaError_t e = greeks_kernel_occupancy(precision, v, &occ);
        if (e != cudaSuccess) return ctx->cuda_fail(e, "greeks occupancy");
        if (occ < 1) continue;
        std::vector<int> cands;
        for (int c : {occ, (occ + 1) / 2, 2 * occ})
            if (c >= 1 && std::find(cands.begin(), cands.end(), c) == cands.end()) cands.push_back(c);
        for (int c : cands) {
            ctx->greeks_shape[precision] = LaunchShape{v, c};
            cudaGraphExec_t exec = nullptr;
            rc = prepare_greeks(*ctx, precision, plan, consts, &exec);
            double total = 0.0;
            for (int rep = 0; rep < 3 && !rc; ++rep) {
                rc = run_greeks(*ctx, exec, n, out);
                ctx->collect_timing(true);
                if (rep > 0) total += ctx->last_ms;
            }
            if (rc) {
                ctx->greeks_shape[precision] = saved;
                return rc;
            }
            if (total / 2.0 < best) {
                best = total / 2.0;
                best_shape = LaunchShape{v, c};
            }
        }
    }
    ctx->greeks_shape[precision] = best_shape;
    if (variant_out) *variant_out = best_shape.variant;
    if (ctas_out) *ctas_out = best_shape.ctas_per_sm;
    if (best_ms_out) *best_ms_out = best;
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

mcd_bump_sizes mcd_default_bump_sizes(double spot, double vol, double time) {
    mcd_bump_sizes b;
    b.spot = std::max(spot * 0.01, 1e-4);
    b.vol = std::max(vol * 0.01, 1e-4);
    b.rate = 0.01;
    b.time = std::max(time * 0.01, 1e-4);
    return b;
}

int mcd_fd_european(mcd_ctx* handle, double spot, double strike, double rate, double carry_yield, double vol,
                    double time, int type, uint64_t path_count, uint64_t seed, mcd_bump_sizes bumps, int precision,
                    mcd_european_greeks* out) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (!out) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "out must not be NULL");
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    // finite_difference.cpp:46-57: the nine scenarios, same seed and paths
    const double s[9][5] = {
        {spot, rate, carry_yield, vol, time},
        {spot + bumps.spot, rate, carry_yield, vol, time},
        {spot - bumps.spot, rate, carry_yield, vol, time},
        {spot, rate, carry_yield, vol + bumps.vol, time},
        {spot, rate, carry_yield, vol - bumps.vol, time},
        {spot, rate + bumps.rate, carry_yield, vol, time},
        {spot, rate - bumps.rate, carry_yield, vol, time},
        {spot, rate, carry_yield, vol, time + bumps.time},
        {spot, rate, carry_yield, vol, time - bumps.time},
    };
    mcd_contract cs[9];
    for (int i = 0; i < 9; ++i)
        cs[i] = make_contract(MCD_PRODUCT_EUROPEAN, s[i][0], strike, s[i][1], s[i][2], s[i][3], s[i][4], type,
                              path_count, seed);
    mcd_mc_result r[9];
    const int rc = price_batch_host(*ctx, cs, 9, precision, r);
    if (rc) return rc;
    // finite_difference.cpp:59-64
    out->delta = (r[1].price - r[2].price) / (2.0 * bumps.spot);
    out->gamma = (r[1].price - 2.0 * r[0].price + r[2].price) / (bumps.spot * bumps.spot);
    out->vega = (r[3].price - r[4].price) / (2.0 * bumps.vol);
    out->theta = -(r[7].price - r[8].price) / (2.0 * bumps.time);
    out->rho = (r[5].price - r[6].price) / (2.0 * bumps.rate);
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_lr_european(mcd_ctx* handle, double spot, double strike, double rate, double carry_yield, double vol,
                    double time, int type, uint64_t path_count, uint64_t seed, int precision, mcd_lr_greeks* out) try {
    if (!out) return MCD_ERR_INVALID_ARGUMENT;
    mcd_greeks_result r;
    const int rc = greeks_one(handle, make_contract(MCD_PRODUCT_EUROPEAN, spot, strike, rate, carry_yield, vol, time,
                                                    type, path_count, seed),
                              precision, &r);
    if (!rc) to_lr(r, true, out);
    return rc;
} catch (...) {
    return abi_exception(handle);
}

int mcd_lr_digital(mcd_ctx* handle, double spot, double strike, double rate, double carry_yield, double vol,
                   double time, int type, int digital_style, double cash_amount, uint64_t path_count, uint64_t seed,
                   int precision, mcd_lr_greeks* out) try {
    if (!out) return MCD_ERR_INVALID_ARGUMENT;
    mcd_contract c = make_contract(MCD_PRODUCT_DIGITAL, spot, strike, rate, carry_yield, vol, time, type, path_count,
                                   seed);
    c.digital_style = digital_style;
    c.cash_amount = cash_amount;
    mcd_greeks_result r;
    const int rc = greeks_one(handle, c, precision, &r);
    if (!rc) to_lr(r, true, out);
    return rc;
} catch (...) {
    return abi_exception(handle);
}

int mcd_lr_barrier(mcd_ctx* handle, double spot, double strike, double barrier, double rate, double carry_yield,
                   double vol, double time, int type, int direction, int knock, double rebate,
                   int monitoring_points, uint64_t path_count, uint64_t seed, int precision, mcd_lr_greeks* out) try {
    if (!out) return MCD_ERR_INVALID_ARGUMENT;
    mcd_contract c = make_contract(MCD_PRODUCT_BARRIER, spot, strike, rate, carry_yield, vol, time, type, path_count,
                                   seed);
    c.barrier = barrier;
    c.direction = direction;
    c.knock = knock;
    c.rebate = rebate;
    c.monitoring_points = monitoring_points;
    mcd_greeks_result r;
    const int rc = greeks_one(handle, c, precision, &r);
    if (!rc) to_lr(r, false, out);
    return rc;
} catch (...) {
    return abi_exception(handle);
}

int mcd_pathwise_european(mcd_ctx* handle, double spot, double strike, double rate, double carry_yield, double vol,
                          double time, int type, uint64_t path_count, uint64_t seed, int precision,
                          mcd_pathwise_greeks* out) try {
    if (!out) return MCD_ERR_INVALID_ARGUMENT;
    mcd_greeks_result r;
    const int rc = greeks_one(handle, make_contract(MCD_PRODUCT_EUROPEAN, spot, strike, rate, carry_yield, vol, time,
                                                    type, path_count, seed),
                              precision, &r);
    if (!rc) to_pw(r, out);
    return rc;
} catch (...) {
    return abi_exception(handle);
}

int mcd_pathwise_asian(mcd_ctx* handle, double spot, double strike, double rate, double carry_yield, double vol,
                       double time, int type, int strike_style, int average_style, int monitoring_points,
                       uint64_t path_count, uint64_t seed, int precision, mcd_pathwise_greeks* out) try {
    if (!out) return MCD_ERR_INVALID_ARGUMENT;
    mcd_contract c = make_contract(MCD_PRODUCT_ASIAN, spot, strike, rate, carry_yield, vol, time, type, path_count,
                                   seed);
    c.strike_style = strike_style;
    c.average_style = average_style;
    c.monitoring_points = monitoring_points;
    mcd_greeks_result r;
    const int rc = greeks_one(handle, c, precision, &r);
    if (!rc) to_pw(r, out);
    return rc;
} catch (...) {
    return abi_exception(handle);
}

}  // extern "C"
