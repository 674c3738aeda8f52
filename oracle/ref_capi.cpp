// ref_capi.cpp -- C entry points over the reference library (mcd), compiled
// together with the reference's own sources by oracle/Makefile (target `ref`)
// into oracle/_ref/libmcd_ref.so.  TEST INFRASTRUCTURE ONLY: used to pin the C
// restatement in mcd_oracle.c and to generate tests/golden fixtures.  The
// reference sources are read where they lie; nothing of them is copied here.
//
// Argument lists mirror mcd_oracle.h so the two can be compared call for call.
#include "mcd/core/normal.hpp"
#include "mcd/core/rng.hpp"
#include "mcd/core/sobol.hpp"
#include "mcd/core/thread_pool.hpp"
#include "mcd/greeks/finite_difference.hpp"
#include "mcd/greeks/likelihood_ratio.hpp"
#include "mcd/greeks/pathwise.hpp"
#include "mcd/models/brownian_bridge_path.hpp"
#include "mcd/pricers/analytic.hpp"
#include "mcd/pricers/binomial.hpp"
#include "mcd/pricers/heston.hpp"
#include "mcd/pricers/lsm.hpp"
#include "mcd/pricers/monte_carlo.hpp"
#include "mcd/pricers/qmc.hpp"

#include <cstdint>
#include <cstring>
#include <span>

using namespace mcd;

namespace {
OptionType ot(int t) { return t == 0 ? OptionType::Call : OptionType::Put; }
BarrierDirection bd(int d) { return d == 0 ? BarrierDirection::Up : BarrierDirection::Down; }
BarrierKnock bk(int k) { return k == 0 ? BarrierKnock::In : BarrierKnock::Out; }
StrikeStyle ss(int s) { return s == 0 ? StrikeStyle::Fixed : StrikeStyle::Floating; }
AverageStyle as(int s) { return s == 0 ? AverageStyle::Arithmetic : AverageStyle::Geometric; }
DigitalStyle ds(int s) { return s == 0 ? DigitalStyle::CashOrNothing : DigitalStyle::AssetOrNothing; }
pricers::McOptions opts(int anti, int cv, int bb, unsigned threads) {
    pricers::McOptions o;
    o.antithetic = anti != 0;
    o.control_variate = cv != 0;
    o.brownian_bridge = bb != 0;
    o.num_threads = threads;
    return o;
}
void put(const pricers::McResult& r, double* out) {
    out[0] = r.price;
    out[1] = r.standard_error;
    out[2] = static_cast<double>(r.path_count);
}
void put_greek(const greeks::LrGreeksResult& g, double* out) {
    out[0] = g.value;
    out[1] = g.standard_error;
}
} // namespace

extern "C" {

unsigned ref_logical_chunk_count() { return ThreadPool::logical_chunk_count(); }

void ref_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    const auto r = philox4x32_10({ctr[0], ctr[1], ctr[2], ctr[3]}, {key[0], key[1]});
    for (int i = 0; i < 4; ++i) out[i] = r[static_cast<std::size_t>(i)];
}
double ref_normal_variate(uint64_t seed, uint64_t path, uint32_t draw) {
    return standard_normal_variate(seed, path, draw);
}
double ref_uniform_variate(uint64_t seed, uint64_t path, uint32_t draw) {
    return uniform_variate(seed, path, draw);
}
double ref_inv_normal_cdf(double u) { return inverse_standard_normal_cdf(u); }
double ref_normal_cdf(double x) { return standard_normal_cdf(x); }
double ref_sobol_point(unsigned dim, uint64_t index) { return sobol_point(dim, index); }

void ref_brownian_bridge_gbm_path(double spot, double rate, double q, double vol, double time,
                                  int n, const double* normals, double* spots) {
    const models::GbmParams p{.spot = spot, .rate = rate, .carry_yield = q, .vol = vol, .time = time};
    const auto s = models::brownian_bridge_gbm_path(p, n, std::span<const double>(normals, static_cast<std::size_t>(n)));
    for (int i = 0; i < n; ++i) spots[i] = s[static_cast<std::size_t>(i)];
}

void ref_mc_european(double s, double k, double r, double q, double v, double t, int type,
                     uint64_t n, uint64_t seed, int anti, unsigned threads, double* out) {
    put(pricers::monte_carlo_european(s, k, r, q, v, t, ot(type), n, seed, opts(anti, 0, 0, threads)), out);
}
void ref_mc_digital(double s, double k, double r, double q, double v, double t, int type,
                    int style, double cash, uint64_t n, uint64_t seed, int anti, unsigned threads,
                    double* out) {
    put(pricers::monte_carlo_digital(s, k, r, q, v, t, ot(type), ds(style), cash, n, seed,
                                     opts(anti, 0, 0, threads)), out);
}
void ref_mc_asian(double s, double k, double r, double q, double v, double t, int type,
                  int strike_style, int avg_style, int steps, uint64_t n, uint64_t seed, int anti,
                  int cv, unsigned threads, double* out) {
    put(pricers::monte_carlo_asian(s, k, r, q, v, t, ot(type), ss(strike_style), as(avg_style),
                                   steps, n, seed, opts(anti, cv, 0, threads)), out);
}
void ref_mc_barrier(double s, double k, double h, double r, double q, double v, double t,
                    int type, int dir, int knock, double rebate, int steps, uint64_t n,
                    uint64_t seed, int anti, int bb, unsigned threads, double* out) {
    put(pricers::monte_carlo_barrier(s, k, h, r, q, v, t, ot(type), bd(dir), bk(knock), rebate,
                                     steps, n, seed, opts(anti, 0, bb, threads)), out);
}
void ref_mc_lookback(double s, double k, double r, double q, double v, double t, int type,
                     int style, int steps, uint64_t n, uint64_t seed, int anti, unsigned threads,
                     double* out) {
    put(pricers::monte_carlo_lookback(s, k, r, q, v, t, ot(type), ss(style), steps, n, seed,
                                      opts(anti, 0, 0, threads)), out);
}

// out: price, se; coeffs (steps+1)*4; has (steps+1); inception flag.
void ref_lsm_american(double s, double k, double r, double q, double v, double t, int type,
                      int steps, uint64_t n, uint64_t seed, double* out, double* coeffs,
                      uint8_t* has, int* inception) {
    const auto res = pricers::monte_carlo_lsm_american(s, k, r, q, v, t, ot(type), steps, n, seed);
    out[0] = res.price;
    out[1] = res.standard_error;
    for (int d = 0; d <= steps; ++d) {
        const auto& c = res.policy.coefficients_by_date[static_cast<std::size_t>(d)];
        has[d] = c.empty() ? 0 : 1;
        for (int b = 0; b < 4; ++b) coeffs[d * 4 + b] = c.empty() ? 0.0 : c[static_cast<std::size_t>(b)];
    }
    *inception = res.policy.exercise_at_inception ? 1 : 0;
}
double ref_lsm_reprice_frozen(double s, double k, double r, double q, double v, double t, int type,
                              int steps, uint64_t n, uint64_t seed, const double* coeffs,
                              const uint8_t* has, int inception) {
    pricers::LsmPolicy policy;
    policy.coefficients_by_date.resize(static_cast<std::size_t>(steps) + 1);
    for (int d = 0; d <= steps; ++d)
        if (has[d]) policy.coefficients_by_date[static_cast<std::size_t>(d)].assign(coeffs + d * 4, coeffs + d * 4 + 4);
    policy.exercise_at_inception = inception != 0;
    return pricers::reprice_against_frozen_policy(s, k, r, q, v, t, ot(type), steps, n, seed, policy);
}

void ref_heston_qe(const double* p9, double strike, int type, int steps, uint64_t n, uint64_t seed,
                   double* out) {
    const models::HestonParams p{.spot = p9[0], .rate = p9[1], .carry_yield = p9[2], .v0 = p9[3],
                                 .kappa = p9[4], .theta = p9[5], .xi = p9[6], .rho = p9[7], .time = p9[8]};
    const auto r = pricers::heston_qe_european(p, strike, ot(type), steps, n, seed);
    out[0] = r.price;
    out[1] = r.standard_error;
    out[2] = static_cast<double>(r.path_count);
}
double ref_heston_semi_analytic(const double* p9, double strike, int type) {
    const models::HestonParams p{.spot = p9[0], .rate = p9[1], .carry_yield = p9[2], .v0 = p9[3],
                                 .kappa = p9[4], .theta = p9[5], .xi = p9[6], .rho = p9[7], .time = p9[8]};
    return pricers::heston_semi_analytic(p, strike, ot(type));
}

double ref_qmc_european(double s, double k, double r, double q, double v, double t, int type, uint64_t n) {
    return pricers::qmc_sobol_european(s, k, r, q, v, t, ot(type), n).price;
}
double ref_qmc_asian(double s, double k, double r, double q, double v, double t, int type,
                     int strike_style, int steps, uint64_t n) {
    return pricers::qmc_sobol_asian(s, k, r, q, v, t, ot(type), ss(strike_style), steps, n).price;
}

// out: delta gamma vega theta rho
void ref_fd_european(double s, double k, double r, double q, double v, double t, int type,
                     uint64_t n, uint64_t seed, const double* bumps4, double* out) {
    const greeks::BumpSizes b{.spot = bumps4[0], .vol = bumps4[1], .rate = bumps4[2], .time = bumps4[3]};
    const auto g = greeks::finite_difference_european(s, k, r, q, v, t, ot(type), n, seed, b);
    out[0] = g.delta;
    out[1] = g.gamma;
    out[2] = g.vega;
    out[3] = g.theta;
    out[4] = g.rho;
}
void ref_default_bumps(double s, double v, double t, double* out4) {
    const auto b = greeks::default_bump_sizes(s, v, t);
    out4[0] = b.spot;
    out4[1] = b.vol;
    out4[2] = b.rate;
    out4[3] = b.time;
}
// out: delta(v,se) gamma vega rho theta (10 doubles); returns has_theta
int ref_lr_european(double s, double k, double r, double q, double v, double t, int type,
                    uint64_t n, uint64_t seed, double* out) {
    const auto g = greeks::likelihood_ratio_european(s, k, r, q, v, t, ot(type), n, seed);
    put_greek(g.delta, out); put_greek(g.gamma, out + 2); put_greek(g.vega, out + 4);
    put_greek(g.rho, out + 6); put_greek(*g.theta, out + 8);
    return 1;
}
int ref_lr_digital(double s, double k, double r, double q, double v, double t, int type, int style,
                   double cash, uint64_t n, uint64_t seed, double* out) {
    const auto g = greeks::likelihood_ratio_digital(s, k, r, q, v, t, ot(type), ds(style), cash, n, seed);
    put_greek(g.delta, out); put_greek(g.gamma, out + 2); put_greek(g.vega, out + 4);
    put_greek(g.rho, out + 6); put_greek(*g.theta, out + 8);
    return 1;
}
int ref_lr_barrier(double s, double k, double h, double r, double q, double v, double t, int type,
                   int dir, int knock, double rebate, int steps, uint64_t n, uint64_t seed, double* out) {
    const auto g = greeks::likelihood_ratio_barrier(s, k, h, r, q, v, t, ot(type), bd(dir), bk(knock),
                                                    rebate, steps, n, seed);
    put_greek(g.delta, out); put_greek(g.gamma, out + 2); put_greek(g.vega, out + 4);
    put_greek(g.rho, out + 6);
    out[8] = out[9] = 0.0;
    return g.theta.has_value() ? 1 : 0;
}
// out: delta vega rho (value, se) = 6 doubles
void ref_pathwise_european(double s, double k, double r, double q, double v, double t, int type,
                           uint64_t n, uint64_t seed, double* out) {
    const auto g = greeks::pathwise_european(s, k, r, q, v, t, ot(type), n, seed);
    out[0] = g.delta.value; out[1] = g.delta.standard_error;
    out[2] = g.vega.value; out[3] = g.vega.standard_error;
    out[4] = g.rho.value; out[5] = g.rho.standard_error;
}
void ref_pathwise_asian(double s, double k, double r, double q, double v, double t, int type,
                        int strike_style, int avg_style, int steps, uint64_t n, uint64_t seed,
                        double* out) {
    const auto g = greeks::pathwise_asian(s, k, r, q, v, t, ot(type), ss(strike_style), as(avg_style),
                                          steps, n, seed);
    out[0] = g.delta.value; out[1] = g.delta.standard_error;
    out[2] = g.vega.value; out[3] = g.vega.standard_error;
    out[4] = g.rho.value; out[5] = g.rho.standard_error;
}

double ref_bsm(double s, double k, double r, double q, double v, double t, int type) {
    return pricers::black_scholes_merton(s, k, r, q, v, t, ot(type));
}
double ref_kemna_vorst(double s, double k, double r, double q, double v, double t, int type) {
    return pricers::kemna_vorst(s, k, r, q, v, t, ot(type));
}
double ref_reiner_rubinstein(double s, double k, double h, double r, double q, double v, double t,
                             int type, int dir, int knock, double rebate) {
    return pricers::reiner_rubinstein(s, k, h, r, q, v, t, ot(type), bd(dir), bk(knock), rebate);
}
double ref_lookback_fixed(double s, double k, double r, double q, double v, double t, int type) {
    return pricers::lookback_fixed_strike(s, k, r, q, v, t, ot(type));
}
double ref_lookback_floating(double s, double r, double q, double v, double t, int type) {
    return pricers::lookback_floating_strike(s, r, q, v, t, ot(type));
}
double ref_digital_analytic(double s, double k, double r, double q, double v, double t, int type,
                            int style, double cash) {
    return pricers::digital(s, k, r, q, v, t, ot(type), ds(style), cash);
}
double ref_crr_american(double s, double k, double r, double q, double v, double t, int steps, int type) {
    return pricers::crr_binomial_american(s, k, r, q, v, t, steps, ot(type));
}
void ref_crr_european(double s, double k, double r, double q, double v, double t, int steps, int type,
                      double* out4) {
    const auto b = pricers::crr_binomial(s, k, r, q, v, t, steps, ot(type));
    out4[0] = b.price;
    out4[1] = b.risk_neutral_probability;
    out4[2] = b.up_factor;
    out4[3] = b.down_factor;
}
double ref_black76(double f, double k, double r, double v, double t, int type) {
    return pricers::black76(f, k, r, v, t, ot(type));
}
double ref_forward_price(double s, double r, double q, double t) { return pricers::forward_price(s, r, q, t); }
double ref_forward_value(double fn, double f0, double r, double t) { return pricers::forward_value(fn, f0, r, t); }
double ref_futures_mtm(double a, double b) { return pricers::futures_mark_to_market(a, b); }

} // extern "C"
