// lsm_api.cpp -- C ABI for the batched Longstaff-Schwartz engine (lsm.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "context.hpp"
#include "lsm.hpp"
#include "lsm_mlp.hpp"
#include "mcd_gpu.h"

using namespace mcdg;

namespace {

// Extension slots of Ctx::ext used by this module (Heston uses 0..3).
enum { kDev = 4, kChunkMap = 5, kStore = 6, kCf = 7, kReg = 8, kPartA = 9, kPartB = 10,
       kFinal = 11, kOut = 12 };

struct LsmPlan {
    std::vector<LsmDev> dev;
    std::vector<uint32_t> chunk_contract;
    uint64_t store_elems = 0, cf_elems = 0, reg_rows = 0;
    uint32_t total_chunks = 0;
    int max_steps = 0;
};

int plan_lsm(Ctx& ctx, const mcd_lsm_contract* cs, size_t n, LsmPlan& p) {
    p = LsmPlan{};
    p.dev.resize(n);
    for (size_t i = 0; i < n; ++i) {
        const mcd_lsm_contract& c = cs[i];
        const double v[] = {c.spot, c.strike, c.rate, c.carry_yield, c.vol, c.time};
        for (double x : v)
            if (!std::isfinite(x)) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "lsm contract " + std::to_string(i) + ": non-finite parameter");
        if (!(c.spot > 0) || !(c.strike > 0) || !(c.vol > 0) || !(c.time > 0))
            return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "lsm contract " + std::to_string(i) + ": spot, strike, vol, time must be > 0");
        if (c.type != 0 && c.type != 1) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "type must be 0 (call) or 1 (put)");
        if (c.monitoring_points < 1 || c.monitoring_points > 100000)
            return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "monitoring_points must be 1..100000");
        if (c.path_count > (1ull << 40)) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "path_count too large");
        LsmDev& d = p.dev[i];
        std::memset(&d, 0, sizeof d);
        const double dt = c.time / static_cast<double>(c.monitoring_points);
        d.spot = c.spot;
        d.strike = c.strike;
        d.disc = std::exp(-c.rate * dt);
        d.drift = (c.rate - c.carry_yield - 0.5 * c.vol * c.vol) * dt;
        d.vs = c.vol * std::sqrt(dt);
        const double phi = c.type == 0 ? 1.0 : -1.0;
        const double x = phi * (c.spot - c.strike);
        d.inception = x > 0.0 ? x : 0.0;
        d.seed = c.seed;
        d.path_count = c.path_count;
        d.n_steps = c.monitoring_points;
        d.type = c.type;
        d.s_offset = p.store_elems;
        d.cf_offset = p.cf_elems;
        d.reg_offset = static_cast<uint32_t>(p.reg_rows);
        const uint64_t chunks = (c.path_count + kLsmChunk - 1) / kLsmChunk;
        if (p.total_chunks + chunks > 0x7FFFFFFFull) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "batch too large");
        d.chunk_begin = p.total_chunks;
        d.n_chunks = static_cast<uint32_t>(chunks);
        for (uint64_t q = 0; q < chunks; ++q) p.chunk_contract.push_back(static_cast<uint32_t>(i));
        p.total_chunks += static_cast<uint32_t>(chunks);
        p.store_elems += static_cast<uint64_t>(c.monitoring_points) * c.path_count;
        p.cf_elems += c.path_count;
        p.reg_rows += static_cast<uint64_t>(c.monitoring_points) + 1;
        p.max_steps = std::max(p.max_steps, c.monitoring_points);
    }
    return MCD_OK;
}

int upload_and_run(Ctx& ctx, const LsmPlan& p, int precision, bool frozen,
                   const std::vector<LsmReg>* frozen_reg, std::vector<double>& out) {
    const size_t n = p.dev.size();
    const size_t elem = precision == 0 ? sizeof(double) : sizeof(float);
    int rc = ctx.reserve(ctx.ext[kDev], sizeof(LsmDev) * n, "lsm contracts");
    if (!rc) rc = ctx.reserve(ctx.ext[kChunkMap], sizeof(uint32_t) * std::max<size_t>(p.total_chunks, 1), "lsm chunk map");
    if (!rc) rc = ctx.reserve(ctx.ext[kStore], elem * std::max<uint64_t>(p.store_elems, 1), "lsm path store");
    if (!rc) rc = ctx.reserve(ctx.ext[kCf], sizeof(double) * std::max<uint64_t>(p.cf_elems, 1), "lsm cash flows");
    if (!rc) rc = ctx.reserve(ctx.ext[kReg], sizeof(LsmReg) * p.reg_rows, "lsm regression table");
    if (!rc) rc = ctx.reserve(ctx.ext[kPartA], sizeof(LsmPartial) * std::max<size_t>(p.total_chunks, 1), "lsm partials");
    if (!rc) rc = ctx.reserve(ctx.ext[kPartB], sizeof(LsmPartial) * std::max<size_t>(p.total_chunks, 1), "lsm partials");
    if (!rc) rc = ctx.reserve(ctx.ext[kFinal], sizeof(Welford) * std::max<size_t>(p.total_chunks, 1), "lsm final partials");
    if (!rc) rc = ctx.reserve(ctx.ext[kOut], sizeof(double) * 6 * n, "lsm results");
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(ctx.ext[kDev].ptr, p.dev.data(), sizeof(LsmDev) * n, cudaMemcpyHostToDevice, ctx.stream);
    if (e == cudaSuccess && p.total_chunks)
        e = cudaMemcpyAsync(ctx.ext[kChunkMap].ptr, p.chunk_contract.data(), sizeof(uint32_t) * p.total_chunks,
                            cudaMemcpyHostToDevice, ctx.stream);
    if (e == cudaSuccess) {
        if (frozen_reg)
            e = cudaMemcpyAsync(ctx.ext[kReg].ptr, frozen_reg->data(), sizeof(LsmReg) * p.reg_rows,
                                cudaMemcpyHostToDevice, ctx.stream);
        else
            e = cudaMemsetAsync(ctx.ext[kReg].ptr, 0, sizeof(LsmReg) * p.reg_rows, ctx.stream);
    }
    if (e != cudaSuccess) return ctx.cuda_fail(e, "lsm upload");

    // Capture forward pass + every backward iteration + finish into one graph.
    cudaGetLastError();
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "lsm begin capture");
    const LsmDev* d_dev = static_cast<const LsmDev*>(ctx.ext[kDev].ptr);
    const uint32_t* d_map = static_cast<const uint32_t*>(ctx.ext[kChunkMap].ptr);
    cudaError_t le = launch_lsm_forward(precision, d_dev, static_cast<int>(n), d_map, p.total_chunks,
                                        ctx.ext[kStore].ptr, ctx.stream);
    for (int k = 0; k < p.max_steps && le == cudaSuccess; ++k)
        le = launch_lsm_iteration(precision, k, frozen, d_dev, static_cast<int>(n), d_map, p.total_chunks,
                                  ctx.ext[kStore].ptr, static_cast<double*>(ctx.ext[kCf].ptr),
                                  static_cast<LsmReg*>(ctx.ext[kReg].ptr),
                                  static_cast<LsmPartial*>(ctx.ext[kPartA].ptr),
                                  static_cast<LsmPartial*>(ctx.ext[kPartB].ptr),
                                  static_cast<Welford*>(ctx.ext[kFinal].ptr), ctx.stream);
    if (le == cudaSuccess)
        le = launch_lsm_finish(d_dev, static_cast<int>(n), static_cast<const Welford*>(ctx.ext[kFinal].ptr),
                               static_cast<double*>(ctx.ext[kOut].ptr), ctx.stream);
    e = cudaStreamEndCapture(ctx.stream, &graph);
    if (le != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return ctx.cuda_fail(le, "lsm capture");
    }
    if (e != cudaSuccess) return ctx.cuda_fail(e, "lsm end capture");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "lsm instantiate");
    int pair = -1;
    rc = ctx.record_start(ctx.stream, &pair);
    if (!rc) {
        e = cudaGraphLaunch(exec, ctx.stream);
        if (e != cudaSuccess) rc = ctx.cuda_fail(e, "lsm graph launch");
    }
    if (!rc) rc = ctx.record_stop(ctx.stream, pair);
    out.assign(6 * n, 0.0);
    if (!rc) {
        e = cudaMemcpyAsync(out.data(), ctx.ext[kOut].ptr, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, ctx.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx.stream);
        if (e != cudaSuccess) rc = ctx.cuda_fail(e, "lsm execution");
    }
    cudaGraphExecDestroy(exec);
    ctx.collect_timing(false);
    return rc;
}

int lsm_batch(Ctx& ctx, const mcd_lsm_contract* cs, size_t n, int precision, int regression,
              mcd_lsm_result* results, std::vector<LsmReg>* reg_out) {
    if (precision != 0 && precision != 1) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    if (regression == MCD_LSM_MLP) return lsm_mlp_batch(ctx, cs, n, precision, results);
    if (regression != MCD_LSM_QR) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "regression must be MCD_LSM_QR or MCD_LSM_MLP");
    if (n == 0) return MCD_OK;
    if (!cs || !results) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "null array");
    LsmPlan p;
    int rc = plan_lsm(ctx, cs, n, p);
    if (rc) return rc;
    std::vector<double> out;
    rc = upload_and_run(ctx, p, precision, false, nullptr, out);
    if (rc) return rc;
    for (size_t i = 0; i < n; ++i) {
        results[i].price = out[6 * i];
        results[i].standard_error = out[6 * i + 1];
        results[i].path_count = static_cast<uint64_t>(out[6 * i + 2]);
        results[i].exercise_at_inception = out[6 * i + 3] != 0.0 ? 1 : 0;
        results[i].reserved = 0;
    }
    if (reg_out) {
        reg_out->resize(p.reg_rows);
        cudaError_t e = cudaMemcpy(reg_out->data(), ctx.ext[kReg].ptr, sizeof(LsmReg) * p.reg_rows,
                                   cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return ctx.cuda_fail(e, "lsm policy copy");
    }
    return MCD_OK;
}

}  // namespace

extern "C" {

int mcd_lsm_american(mcd_ctx* handle, double spot, double strike, double rate, double carry_yield,
                     double vol, double time, int type, int monitoring_points,
                     uint64_t path_count, uint64_t seed, int precision, int regression,
                     mcd_lsm_result* out, double* coefficients, uint8_t* has_coefficients) {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (!out) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "out must not be NULL");
    const mcd_lsm_contract c{spot, strike, rate, carry_yield, vol, time, type, monitoring_points,
                             path_count, seed};
    std::vector<LsmReg> reg;
    const bool want_policy = coefficients || has_coefficients;
    const int rc = lsm_batch(*ctx, &c, 1, precision, regression, out,
                             (want_policy && regression == MCD_LSM_QR) ? &reg : nullptr);
    if (rc) return rc;
    if (want_policy && regression == MCD_LSM_QR) {
        for (int d = 0; d <= monitoring_points; ++d) {
            const bool has = reg[d].has == 1;
            if (has_coefficients) has_coefficients[d] = has ? 1 : 0;
            if (coefficients)
                for (int b = 0; b < 4; ++b) coefficients[4 * d + b] = has ? reg[d].gamma[b] : 0.0;
        }
    }
    return MCD_OK;
}

int mcd_lsm_reprice_frozen(mcd_ctx* handle, double spot, double strike, double rate,
                           double carry_yield, double vol, double time, int type,
                           int monitoring_points, uint64_t path_count, uint64_t seed,
                           const double* coefficients, const uint8_t* has_coefficients,
                           int exercise_at_inception, int precision, double* price) {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (!coefficients || !has_coefficients || !price) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "null argument");
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    const mcd_lsm_contract c{spot, strike, rate, carry_yield, vol, time, type, monitoring_points,
                             path_count, seed};
    LsmPlan p;
    int rc = plan_lsm(*ctx, &c, 1, p);
    if (rc) return rc;
    std::vector<LsmReg> reg(p.reg_rows);
    std::memset(reg.data(), 0, sizeof(LsmReg) * reg.size());
    for (int d = 1; d < monitoring_points; ++d) {
        if (!has_coefficients[d]) continue;
        reg[d].has = 1;
        for (int b = 0; b < 4; ++b) reg[d].gamma[b] = coefficients[4 * d + b];
    }
    std::vector<double> out;
    rc = upload_and_run(*ctx, p, precision, true, &reg, out);
    if (rc) return rc;
    // Frozen inception decision (src/pricers/lsm.cpp:206-212): the base run's
    // choice is replayed; otherwise the price is the path average itself.
    if (exercise_at_inception) {
        const double phi = type == 0 ? 1.0 : -1.0;
        const double x = phi * (spot - strike);
        *price = x > 0.0 ? x : 0.0;
    } else {
        *price = out[4];
    }
    return MCD_OK;
}

int mcd_lsm_batch(mcd_ctx* handle, const mcd_lsm_contract* contracts, size_t n, int precision,
                  int regression, mcd_lsm_result* results) {
    MCD_CTX_OR_FAIL(handle, ctx);
    return lsm_batch(*ctx, contracts, n, precision, regression, results, nullptr);
}

}  // extern "C"
