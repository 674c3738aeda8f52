// analytic_host.cpp -- closed forms the pricers need on the host.
//
// The control-variate Asian anchors its geometric leg at the Kemna-Vorst price
// (src/pricers/monte_carlo.cpp:279-280 -> src/pricers/analytic.cpp:51-59):
// the continuous geometric average of GBM is lognormal with volatility
// sigma/sqrt(3) and cost of carry b_g = (r - q - sigma^2/6)/2, priced by
// Black-Scholes-Merton with carry yield r - b_g.  The operation order below is
// the reference's, so the anchor is the same double.
#include <algorithm>
#include <cmath>
#include <vector>

#include "context.hpp"

double mcd_host_normal_cdf(double x) { return 0.5 * std::erfc(-x / 1.41421356237309504880); }

double mcd_host_bsm(double spot, double strike, double rate, double carry_yield, double vol,
                    double time, int type) {
    const double b = rate - carry_yield;
    const double sqrt_t = std::sqrt(time);
    const double d1 = (std::log(spot / strike) + (b + 0.5 * vol * vol) * time) / (vol * sqrt_t);
    const double d2 = d1 - vol * sqrt_t;
    const double phi = type == 0 ? 1.0 : -1.0;
    const double df_carry = std::exp(-carry_yield * time);
    const double df_rate = std::exp(-rate * time);
    return phi * spot * df_carry * mcd_host_normal_cdf(phi * d1) -
           phi * strike * df_rate * mcd_host_normal_cdf(phi * d2);
}

double mcd_host_kemna_vorst(double spot, double strike, double rate, double carry_yield,
                            double vol, double time, int type) {
    const double sigma_g = vol / 1.73205080756887729353;
    const double b_g = 0.5 * (rate - carry_yield - vol * vol / 6.0);
    const double q_eff = rate - b_g;
    return mcd_host_bsm(spot, strike, rate, q_eff, sigma_g, time, type);
}

// Cox-Ross-Rubinstein American price (src/pricers/binomial.cpp), the
// reference's accuracy yardstick for Longstaff-Schwartz (tests/lsm_test.cpp).
// Host code: exported as mcd_crr_binomial_american for benchmarks and callers
// that want the lattice price next to a Monte Carlo one.
extern "C" double mcd_crr_binomial_american(double spot, double strike, double rate, double carry_yield,
                                            double vol, double time, int steps, int type) {
    if (steps < 1) return std::nan("");
    const double dt = time / static_cast<double>(steps);
    const double u = std::exp(vol * std::sqrt(dt));
    const double d = 1.0 / u;
    const double p = (std::exp((rate - carry_yield) * dt) - d) / (u - d);
    const double disc = std::exp(-rate * dt);
    const double phi = type == 0 ? 1.0 : -1.0;
    std::vector<double> v(static_cast<size_t>(steps) + 1);
    auto node = [&](int level, int i) {
        return spot * std::pow(u, static_cast<double>(i)) * std::pow(d, static_cast<double>(level - i));
    };
    for (int i = 0; i <= steps; ++i) v[i] = std::max(phi * (node(steps, i) - strike), 0.0);
    for (int level = steps - 1; level >= 0; --level)
        for (int i = 0; i <= level; ++i)
            v[i] = std::max(disc * (p * v[i + 1] + (1.0 - p) * v[i]), std::max(phi * (node(level, i) - strike), 0.0));
    return v[0];
}
