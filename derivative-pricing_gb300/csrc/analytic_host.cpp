// analytic_host.cpp -- closed forms the pricers need on the host.
//
// The control-variate Asian anchors its geometric leg at the Kemna-Vorst price
// (src/pricers/monte_carlo.cpp:279-280 -> src/pricers/analytic.cpp:51-59):
// the continuous geometric average of GBM is lognormal with volatility
// sigma/sqrt(3) and cost of carry b_g = (r - q - sigma^2/6)/2, priced by
// Black-Scholes-Merton with carry yield r - b_g.  The operation order below is
// the reference's, so the anchor is the same double.
#include <cmath>

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
