// pricers.cpp -- mcd::pricers / mcd::greeks (mcd_shim.hpp) over the C ABI.
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>

#include "mcd_gpu.h"
#include "mcd_shim.hpp"

namespace mcd {

std::string_view version() noexcept { return "gb300-gpu"; }

namespace gpu {
namespace {

thread_local Precision t_precision = Precision::FP64;

struct CtxHolder {
    mcd_ctx* ctx = nullptr;
    ~CtxHolder() {
        if (ctx) mcd_destroy(ctx);
    }
};

thread_local CtxHolder t_ctx;

}  // namespace

void set_precision(Precision p) { t_precision = p; }
Precision precision() { return t_precision; }

// The calling thread's context, created on first use.
mcd_ctx* context() {
    if (!t_ctx.ctx) {
        const char* dev = std::getenv("MCD_GPU_DEVICE");
        const int device = dev ? std::atoi(dev) : 0;
        mcd_ctx* c = nullptr;
        if (mcd_create(device, &c) != MCD_OK) throw Error(std::string("mcd_create: ") + mcd_last_error(nullptr));
        t_ctx.ctx = c;
    }
    return t_ctx.ctx;
}

void check(int status, const char* what) {
    if (status != MCD_OK) throw Error(std::string(what) + ": " + mcd_last_error(t_ctx.ctx));
}

}  // namespace gpu

namespace {

int prec() { return static_cast<int>(gpu::precision()); }
int ot(OptionType t) { return t == OptionType::Call ? MCD_CALL : MCD_PUT; }

mcd_mc_options opts(const pricers::McOptions& o) {
    mcd_mc_options r;
    std::memset(&r, 0, sizeof r);
    r.antithetic = o.antithetic ? 1 : 0;
    r.control_variate = o.control_variate ? 1 : 0;
    r.brownian_bridge = o.brownian_bridge ? 1 : 0;
    r.num_threads = o.num_threads;
    return r;
}

pricers::McResult mc(const mcd_mc_result& r) { return pricers::McResult{r.price, r.standard_error, r.path_count}; }

greeks::LrGreeksResult lr(const mcd_greek& g) { return greeks::LrGreeksResult{g.value, g.standard_error}; }
greeks::PathwiseGreeksResult pw(const mcd_greek& g) { return greeks::PathwiseGreeksResult{g.value, g.standard_error}; }

greeks::LrGreeks lr_out(const mcd_lr_greeks& g) {
    greeks::LrGreeks r;
    r.delta = lr(g.delta);
    r.gamma = lr(g.gamma);
    r.vega = lr(g.vega);
    r.rho = lr(g.rho);
    if (g.has_theta) r.theta = lr(g.theta);
    return r;
}

greeks::PathwiseGreeks pw_out(const mcd_pathwise_greeks& g) { return greeks::PathwiseGreeks{pw(g.delta), pw(g.vega), pw(g.rho)}; }

}  // namespace

namespace pricers {

McResult monte_carlo_european(double spot, double strike, double rate, double carry_yield, double vol, double time,
                              OptionType type, std::uint64_t path_count, std::uint64_t seed) {
    return monte_carlo_european(spot, strike, rate, carry_yield, vol, time, type, path_count, seed, McOptions{});
}

McResult monte_carlo_european(double spot, double strike, double rate, double carry_yield, double vol, double time,
                              OptionType type, std::uint64_t path_count, std::uint64_t seed, McOptions options) {
    const mcd_mc_options o = opts(options);
    mcd_mc_result r;
    gpu::check(mcd_price_european(gpu::context(), spot, strike, rate, carry_yield, vol, time, ot(type), path_count,
                                  seed, &o, prec(), &r),
               "monte_carlo_european");
    return mc(r);
}

McResult monte_carlo_digital(double spot, double strike, double rate, double carry_yield, double vol, double time,
                             OptionType type, DigitalStyle style, double cash_amount, std::uint64_t path_count,
                             std::uint64_t seed, McOptions options) {
    const mcd_mc_options o = opts(options);
    mcd_mc_result r;
    gpu::check(mcd_price_digital(gpu::context(), spot, strike, rate, carry_yield, vol, time, ot(type),
                                 style == DigitalStyle::CashOrNothing ? MCD_CASH_OR_NOTHING : MCD_ASSET_OR_NOTHING,
                                 cash_amount, path_count, seed, &o, prec(), &r),
               "monte_carlo_digital");
    return mc(r);
}

McResult monte_carlo_asian(double spot, double strike, double rate, double carry_yield, double vol, double time,
                           OptionType type, StrikeStyle strike_style, AverageStyle average_style,
                           int monitoring_points, std::uint64_t path_count, std::uint64_t seed, McOptions options) {
    const mcd_mc_options o = opts(options);
    mcd_mc_result r;
    gpu::check(mcd_price_asian(gpu::context(), spot, strike, rate, carry_yield, vol, time, ot(type),
                               strike_style == StrikeStyle::Fixed ? MCD_FIXED : MCD_FLOATING,
                               average_style == AverageStyle::Arithmetic ? MCD_ARITHMETIC : MCD_GEOMETRIC,
                               monitoring_points, path_count, seed, &o, prec(), &r),
               "monte_carlo_asian");
    return mc(r);
}

McResult monte_carlo_barrier(double spot, double strike, double barrier, double rate, double carry_yield, double vol,
                             double time, OptionType type, BarrierDirection direction, BarrierKnock knock,
                             double rebate, int monitoring_points, std::uint64_t path_count, std::uint64_t seed,
                             McOptions options) {
    const mcd_mc_options o = opts(options);
    mcd_mc_result r;
    gpu::check(mcd_price_barrier(gpu::context(), spot, strike, barrier, rate, carry_yield, vol, time, ot(type),
                                 direction == BarrierDirection::Up ? MCD_UP : MCD_DOWN,
                                 knock == BarrierKnock::In ? MCD_IN : MCD_OUT, rebate, monitoring_points, path_count,
                                 seed, &o, prec(), &r),
               "monte_carlo_barrier");
    return mc(r);
}

McResult monte_carlo_lookback(double spot, double strike, double rate, double carry_yield, double vol, double time,
                              OptionType type, StrikeStyle style, int monitoring_points, std::uint64_t path_count,
                              std::uint64_t seed, McOptions options) {
    const mcd_mc_options o = opts(options);
    mcd_mc_result r;
    gpu::check(mcd_price_lookback(gpu::context(), spot, strike, rate, carry_yield, vol, time, ot(type),
                                  style == StrikeStyle::Fixed ? MCD_FIXED : MCD_FLOATING, monitoring_points,
                                  path_count, seed, &o, prec(), &r),
               "monte_carlo_lookback");
    return mc(r);
}

QmcResult qmc_sobol_european(double spot, double strike, double rate, double carry_yield, double vol, double time,
                             OptionType type, std::uint64_t path_count) {
    QmcResult r;
    gpu::check(mcd_qmc_sobol_european(gpu::context(), spot, strike, rate, carry_yield, vol, time, ot(type),
                                      path_count, prec(), &r.price),
               "qmc_sobol_european");
    return r;
}

QmcResult qmc_sobol_asian(double spot, double strike, double rate, double carry_yield, double vol, double time,
                          OptionType type, StrikeStyle strike_style, int monitoring_points,
                          std::uint64_t path_count) {
    QmcResult r;
    gpu::check(mcd_qmc_sobol_asian(gpu::context(), spot, strike, rate, carry_yield, vol, time, ot(type),
                                   strike_style == StrikeStyle::Fixed ? MCD_FIXED : MCD_FLOATING, monitoring_points,
                                   path_count, prec(), &r.price),
               "qmc_sobol_asian");
    return r;
}

LsmResult monte_carlo_lsm_american(double spot, double strike, double rate, double carry_yield, double vol,
                                   double time, OptionType type, int monitoring_points, std::uint64_t path_count,
                                   std::uint64_t seed) {
    const size_t n1 = monitoring_points > 0 ? static_cast<size_t>(monitoring_points) + 1 : 1;
    std::vector<double> co(n1 * 4, 0.0);
    std::vector<uint8_t> has(n1, 0);
    mcd_lsm_result r;
    gpu::check(mcd_lsm_american(gpu::context(), spot, strike, rate, carry_yield, vol, time, ot(type),
                                monitoring_points, path_count, seed, prec(), MCD_LSM_QR, &r, co.data(), has.data()),
               "monte_carlo_lsm_american");
    LsmResult out;
    out.price = r.price;
    out.standard_error = r.standard_error;
    out.policy.exercise_at_inception = r.exercise_at_inception != 0;
    out.policy.coefficients_by_date.resize(n1);  // lsm.cpp:74; dates without a fit stay empty
    for (size_t d = 0; d < n1; ++d)
        if (has[d]) out.policy.coefficients_by_date[d].assign(co.begin() + 4 * d, co.begin() + 4 * d + 4);
    return out;
}

double reprice_against_frozen_policy(double spot, double strike, double rate, double carry_yield, double vol,
                                     double time, OptionType type, int monitoring_points, std::uint64_t path_count,
                                     std::uint64_t seed, const LsmPolicy& policy) {
    const size_t n1 = monitoring_points > 0 ? static_cast<size_t>(monitoring_points) + 1 : 1;
    std::vector<double> co(n1 * 4, 0.0);
    std::vector<uint8_t> has(n1, 0);
    for (size_t d = 0; d < n1 && d < policy.coefficients_by_date.size(); ++d) {
        const auto& c = policy.coefficients_by_date[d];
        if (c.size() == 4) {
            has[d] = 1;
            for (int k = 0; k < 4; ++k) co[4 * d + k] = c[k];
        }
    }
    double price = 0.0;
    gpu::check(mcd_lsm_reprice_frozen(gpu::context(), spot, strike, rate, carry_yield, vol, time, ot(type),
                                      monitoring_points, path_count, seed, co.data(), has.data(),
                                      policy.exercise_at_inception ? 1 : 0, prec(), &price),
               "reprice_against_frozen_policy");
    return price;
}

HestonMcResult heston_qe_european(const models::HestonParams& p, double strike, OptionType type,
                                  int monitoring_points, std::uint64_t path_count, std::uint64_t seed) {
    const mcd_heston_params hp{p.spot, p.rate, p.carry_yield, p.v0, p.kappa, p.theta, p.xi, p.rho, p.time};
    mcd_mc_result r;
    gpu::check(mcd_heston_qe_european(gpu::context(), &hp, strike, ot(type), monitoring_points, path_count, seed,
                                      prec(), &r),
               "heston_qe_european");
    return HestonMcResult{r.price, r.standard_error, r.path_count};
}

}  // namespace pricers

namespace greeks {

BumpSizes default_bump_sizes(double spot, double vol, double time) noexcept {
    const mcd_bump_sizes b = mcd_default_bump_sizes(spot, vol, time);
    return BumpSizes{b.spot, b.vol, b.rate, b.time};
}

EuropeanGreeks finite_difference_european(double spot, double strike, double rate, double carry_yield, double vol,
                                          double time, OptionType type, std::uint64_t path_count, std::uint64_t seed,
                                          BumpSizes bumps) {
    mcd_european_greeks g;
    gpu::check(mcd_fd_european(gpu::context(), spot, strike, rate, carry_yield, vol, time, ot(type), path_count, seed,
                               mcd_bump_sizes{bumps.spot, bumps.vol, bumps.rate, bumps.time}, prec(), &g),
               "finite_difference_european");
    return EuropeanGreeks{g.delta, g.gamma, g.vega, g.theta, g.rho};
}

LrGreeks likelihood_ratio_european(double spot, double strike, double rate, double carry_yield, double vol,
                                   double time, OptionType type, std::uint64_t path_count, std::uint64_t seed) {
    mcd_lr_greeks g;
    gpu::check(mcd_lr_european(gpu::context(), spot, strike, rate, carry_yield, vol, time, ot(type), path_count, seed,
                               prec(), &g),
               "likelihood_ratio_european");
    return lr_out(g);
}

LrGreeks likelihood_ratio_digital(double spot, double strike, double rate, double carry_yield, double vol,
                                  double time, OptionType type, DigitalStyle style, double cash_amount,
                                  std::uint64_t path_count, std::uint64_t seed) {
    mcd_lr_greeks g;
    gpu::check(mcd_lr_digital(gpu::context(), spot, strike, rate, carry_yield, vol, time, ot(type),
                              style == DigitalStyle::CashOrNothing ? MCD_CASH_OR_NOTHING : MCD_ASSET_OR_NOTHING,
                              cash_amount, path_count, seed, prec(), &g),
               "likelihood_ratio_digital");
    return lr_out(g);
}

LrGreeks likelihood_ratio_barrier(double spot, double strike, double barrier, double rate, double carry_yield,
                                  double vol, double time, OptionType type, BarrierDirection direction,
                                  BarrierKnock knock, double rebate, int monitoring_points, std::uint64_t path_count,
                                  std::uint64_t seed) {
    mcd_lr_greeks g;
    gpu::check(mcd_lr_barrier(gpu::context(), spot, strike, barrier, rate, carry_yield, vol, time, ot(type),
                              direction == BarrierDirection::Up ? MCD_UP : MCD_DOWN,
                              knock == BarrierKnock::In ? MCD_IN : MCD_OUT, rebate, monitoring_points, path_count,
                              seed, prec(), &g),
               "likelihood_ratio_barrier");
    return lr_out(g);
}

PathwiseGreeks pathwise_european(double spot, double strike, double rate, double carry_yield, double vol,
                                 double time, OptionType type, std::uint64_t path_count, std::uint64_t seed) {
    mcd_pathwise_greeks g;
    gpu::check(mcd_pathwise_european(gpu::context(), spot, strike, rate, carry_yield, vol, time, ot(type), path_count,
                                     seed, prec(), &g),
               "pathwise_european");
    return pw_out(g);
}

PathwiseGreeks pathwise_asian(double spot, double strike, double rate, double carry_yield, double vol, double time,
                              OptionType type, StrikeStyle strike_style, AverageStyle average_style,
                              int monitoring_points, std::uint64_t path_count, std::uint64_t seed) {
    mcd_pathwise_greeks g;
    gpu::check(mcd_pathwise_asian(gpu::context(), spot, strike, rate, carry_yield, vol, time, ot(type),
                                  strike_style == StrikeStyle::Fixed ? MCD_FIXED : MCD_FLOATING,
                                  average_style == AverageStyle::Arithmetic ? MCD_ARITHMETIC : MCD_GEOMETRIC,
                                  monitoring_points, path_count, seed, prec(), &g),
               "pathwise_asian");
    return pw_out(g);
}

}  // namespace greeks

}  // namespace mcd
