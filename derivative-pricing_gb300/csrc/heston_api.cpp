// heston_api.cpp -- C ABI for the Heston QE engine (heston.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "context.hpp"
#include "heston.hpp"
#include "mcd_gpu.h"

using namespace mcdg;

namespace {

// Extension slots of Ctx::ext used by this module.
enum { kSets = 0, kStrikes = 1, kPartials = 2, kOut = 3 };

bool finite(double x) { return std::isfinite(x); }

// Per-set constants in the reference's operation order
// (src/pricers/heston.cpp:95-99 for e and the constant part of s2,
// :123-132 for dt, drift, K0..K4, discount and ln S0).
int make_set(Ctx& ctx, const mcd_heston_params& p, int steps, uint64_t paths, uint64_t seed,
             size_t index, HestonSet& h) {
    const double v[] = {p.spot, p.rate, p.carry_yield, p.v0, p.kappa, p.theta, p.xi, p.rho, p.time};
    for (double x : v)
        if (!finite(x)) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "heston set " + std::to_string(index) + ": non-finite parameter");
    if (!(p.spot > 0) || !(p.kappa > 0) || !(p.theta > 0) || !(p.xi > 0) || !(p.v0 >= 0) ||
        !(p.time > 0) || p.rho < -1.0 || p.rho > 1.0)
        return ctx.fail(MCD_ERR_INVALID_ARGUMENT,
                        "heston set " + std::to_string(index) +
                            ": need spot, kappa, theta, xi, time > 0, v0 >= 0, |rho| <= 1");
    std::memset(&h, 0, sizeof h);
    const double dt = p.time / static_cast<double>(steps);
    h.spot = p.spot;
    h.v0 = p.v0;
    h.theta = p.theta;
    h.kappa = p.kappa;
    h.xi = p.xi;
    h.e = std::exp(-p.kappa * dt);
    h.s2_const = p.theta * p.xi * p.xi / (2.0 * p.kappa) * (1.0 - h.e) * (1.0 - h.e);
    h.s2_lin = p.xi * p.xi * h.e / p.kappa * (1.0 - h.e);
    h.drift = (p.rate - p.carry_yield) * dt;
    h.k0 = -p.rho * p.kappa * p.theta * dt / p.xi;
    h.k1 = 0.5 * dt * (p.kappa * p.rho / p.xi - 0.5) - p.rho / p.xi;
    h.k2 = 0.5 * dt * (p.kappa * p.rho / p.xi - 0.5) + p.rho / p.xi;
    h.k3 = 0.5 * dt * (1.0 - p.rho * p.rho);
    h.k4 = h.k3;
    h.discount = std::exp(-p.rate * p.time);
    h.log_s0 = std::log(p.spot);
    h.seed = seed;
    h.path_count = paths;
    h.n_slabs = static_cast<uint32_t>((paths + kSlabPaths - 1) / kSlabPaths);
    h.n_steps = steps;
    return MCD_OK;
}

int heston_run(Ctx& ctx, const mcd_heston_params* sets, size_t n_sets, const double* strikes,
               size_t n_strikes, int type, int steps, uint64_t paths, uint64_t seed,
               int precision, mcd_mc_result* results) {
    if (precision != 0 && precision != 1) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    if (type != 0 && type != 1) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "type must be 0 (call) or 1 (put)");
    if (steps < 1) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "monitoring_points must be >= 1");
    if (n_strikes < 1 || n_strikes > 256) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "n_strikes must be 1..256");
    if (paths > (1ull << 53)) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "path_count must be <= 2^53");
    if (n_sets == 0) return MCD_OK;
    if (!sets || !strikes || !results) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "null array");
    for (size_t k = 0; k < n_strikes; ++k)
        if (!finite(strikes[k])) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "non-finite strike");
    std::vector<HestonSet> hs(n_sets);
    for (size_t i = 0; i < n_sets; ++i) {
        const int rc = make_set(ctx, sets[i], steps, paths, seed, i, hs[i]);
        if (rc) return rc;
    }
    const uint32_t items_per_set = hs[0].n_slabs;
    const uint64_t total_items = static_cast<uint64_t>(items_per_set) * n_sets;
    if (total_items > 0xFFFFFFF0ull) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "batch too large");
    int rc = ctx.reserve(ctx.ext[kSets], sizeof(HestonSet) * n_sets, "heston sets");
    if (!rc) rc = ctx.reserve(ctx.ext[kStrikes], sizeof(double) * n_strikes, "strikes");
    if (!rc) rc = ctx.reserve(ctx.ext[kPartials], sizeof(Welford) * std::max<uint64_t>(total_items, 1) * n_strikes, "heston partials");
    if (!rc) rc = ctx.reserve(ctx.ext[kOut], sizeof(mcd_mc_result) * n_sets * n_strikes, "heston results");
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(ctx.ext[kSets].ptr, hs.data(), sizeof(HestonSet) * n_sets, cudaMemcpyHostToDevice, ctx.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctx.ext[kStrikes].ptr, strikes, sizeof(double) * n_strikes, cudaMemcpyHostToDevice, ctx.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx.d_flags, 0, sizeof(uint32_t), ctx.stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "heston upload");
    int blocks = 0;
    e = heston_occupancy(precision, &blocks);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "heston occupancy");
    const int grid = ctx.sm_count * std::max(blocks, 1);
    int pair = -1;
    rc = ctx.record_start(ctx.stream, &pair);
    if (rc) return rc;
    e = launch_heston(precision, grid, static_cast<const HestonSet*>(ctx.ext[kSets].ptr),
                      static_cast<int>(n_sets), static_cast<const double*>(ctx.ext[kStrikes].ptr),
                      static_cast<int>(n_strikes), type, items_per_set, ctx.d_flags,
                      static_cast<Welford*>(ctx.ext[kPartials].ptr),
                      static_cast<double*>(ctx.ext[kOut].ptr), ctx.stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "heston launch");
    rc = ctx.record_stop(ctx.stream, pair);
    if (rc) return rc;
    e = cudaMemcpyAsync(results, ctx.ext[kOut].ptr, sizeof(mcd_mc_result) * n_sets * n_strikes,
                        cudaMemcpyDeviceToHost, ctx.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx.stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "heston execution");
    ctx.collect_timing(false);
    return MCD_OK;
}

}  // namespace

extern "C" {

int mcd_heston_qe_european(mcd_ctx* handle, const mcd_heston_params* params, double strike,
                           int type, int monitoring_points, uint64_t path_count, uint64_t seed,
                           int precision, mcd_mc_result* out) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (!params || !out) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "null argument");
    return heston_run(*ctx, params, 1, &strike, 1, type, monitoring_points, path_count, seed,
                      precision, out);
} catch (...) {
    return abi_exception(handle);
}

int mcd_heston_qe_batch(mcd_ctx* handle, const mcd_heston_params* sets, size_t n_sets,
                        const double* strikes, size_t n_strikes, int type, int monitoring_points,
                        uint64_t path_count, uint64_t seed, int precision, mcd_mc_result* results) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    return heston_run(*ctx, sets, n_sets, strikes, n_strikes, type, monitoring_points, path_count,
                      seed, precision, results);
} catch (...) {
    return abi_exception(handle);
}

}  // extern "C"
