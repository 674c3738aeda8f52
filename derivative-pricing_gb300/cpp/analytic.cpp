// analytic.cpp -- the reference's closed forms, lattices and semi-analytic
// Heston price (include/mcd/pricers/analytic.hpp, binomial.hpp, heston.hpp)
// over the host FP64 functions of libmcd_gpu.so, so the C ABI, the Python
// module and this API share one implementation.
#include "mcd_gpu.h"
#include "mcd_shim.hpp"

namespace mcd::pricers {

namespace {

int t(OptionType type) { return type == OptionType::Call ? MCD_CALL : MCD_PUT; }

}  // namespace

double black_scholes_merton(double spot, double strike, double rate, double carry_yield, double vol, double time,
                            OptionType type) {
    return mcd_black_scholes_merton(spot, strike, rate, carry_yield, vol, time, t(type));
}

double black76(double forward, double strike, double rate, double vol, double time, OptionType type) {
    return mcd_black76(forward, strike, rate, vol, time, t(type));
}

double kemna_vorst(double spot, double strike, double rate, double carry_yield, double vol, double time,
                   OptionType type) {
    return mcd_kemna_vorst(spot, strike, rate, carry_yield, vol, time, t(type));
}

double reiner_rubinstein(double spot, double strike, double barrier, double rate, double carry_yield, double vol,
                         double time, OptionType type, BarrierDirection direction, BarrierKnock knock,
                         double rebate) {
    return mcd_reiner_rubinstein(spot, strike, barrier, rate, carry_yield, vol, time, t(type),
                                 direction == BarrierDirection::Down ? MCD_DOWN : MCD_UP,
                                 knock == BarrierKnock::In ? MCD_IN : MCD_OUT, rebate);
}

double lookback_fixed_strike(double spot, double strike, double rate, double carry_yield, double vol, double time,
                             OptionType type) {
    return mcd_lookback_fixed_strike(spot, strike, rate, carry_yield, vol, time, t(type));
}

double lookback_floating_strike(double spot, double rate, double carry_yield, double vol, double time,
                                OptionType type) {
    return mcd_lookback_floating_strike(spot, rate, carry_yield, vol, time, t(type));
}

double digital(double spot, double strike, double rate, double carry_yield, double vol, double time,
               OptionType type, DigitalStyle style, double cash_amount) {
    return mcd_digital_analytic(spot, strike, rate, carry_yield, vol, time, t(type),
                                style == DigitalStyle::CashOrNothing ? MCD_CASH_OR_NOTHING : MCD_ASSET_OR_NOTHING,
                                cash_amount);
}

double forward_price(double spot, double rate, double carry_yield, double time) {
    return mcd_forward_price(spot, rate, carry_yield, time);
}

double forward_value(double forward_now, double forward_at_inception, double rate, double time_to_expiry) {
    return mcd_forward_value(forward_now, forward_at_inception, rate, time_to_expiry);
}

double futures_mark_to_market(double futures_price_new, double futures_price_old) {
    return mcd_futures_mark_to_market(futures_price_new, futures_price_old);
}

BinomialResult crr_binomial(double spot, double strike, double rate, double carry_yield, double vol, double time,
                            int steps, OptionType type) {
    double out[4] = {0.0, 0.0, 0.0, 0.0};
    mcd_crr_binomial(spot, strike, rate, carry_yield, vol, time, steps, t(type), out);
    return BinomialResult{out[0], out[1], out[2], out[3]};
}

double crr_binomial_american(double spot, double strike, double rate, double carry_yield, double vol, double time,
                             int steps, OptionType type) {
    return mcd_crr_binomial_american(spot, strike, rate, carry_yield, vol, time, steps, t(type));
}

double heston_semi_analytic(const models::HestonParams& p, double strike, OptionType type) {
    const mcd_heston_params q{p.spot, p.rate, p.carry_yield, p.v0, p.kappa, p.theta, p.xi, p.rho, p.time};
    return mcd_heston_semi_analytic(&q, strike, t(type));
}

}  // namespace mcd::pricers
