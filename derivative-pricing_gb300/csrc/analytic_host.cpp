// analytic_host.cpp -- the reference's closed forms and lattices, host FP64
// (src/pricers/analytic.cpp, src/pricers/binomial.cpp, src/pricers/heston.cpp
// :26-82).  The Monte Carlo pricers need two of them (the Kemna-Vorst anchor of
// the control-variate Asian, monte_carlo.cpp:279-280); the rest are exported
// through the C ABI so that callers of the reference's module (its Python
// bindings, its CLI) find every function they use.  Each formula keeps the
// reference's operation order, so results agree to the last few bits.
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "context.hpp"
#include "mcd_gpu.h"

namespace {

double sgn(int type) { return type == 0 ? 1.0 : -1.0; }

}  // namespace

// src/core/normal.cpp: Phi(x) = erfc(-x / sqrt 2) / 2
double mcd_host_normal_cdf(double x) { return 0.5 * std::erfc(-x / 1.41421356237309504880); }

// analytic.cpp:20-38 (generalised Black-Scholes with cost of carry b = r - q)
double mcd_host_bsm(double spot, double strike, double rate, double carry_yield, double vol,
                    double time, int type) {
    const double b = rate - carry_yield;
    const double sqrt_t = std::sqrt(time);
    const double d1 = (std::log(spot / strike) + (b + 0.5 * vol * vol) * time) / (vol * sqrt_t);
    const double d2 = d1 - vol * sqrt_t;
    const double phi = sgn(type);
    const double df_carry = std::exp(-carry_yield * time);
    const double df_rate = std::exp(-rate * time);
    return phi * spot * df_carry * mcd_host_normal_cdf(phi * d1) -
           phi * strike * df_rate * mcd_host_normal_cdf(phi * d2);
}

// analytic.cpp:51-59: the continuous geometric average of GBM is lognormal
// with volatility sigma/sqrt(3) and carry b_g = (r - q - sigma^2/6)/2.
double mcd_host_kemna_vorst(double spot, double strike, double rate, double carry_yield,
                            double vol, double time, int type) {
    const double sigma_g = vol / 1.73205080756887729353;
    const double b_g = 0.5 * (rate - carry_yield - vol * vol / 6.0);
    const double q_eff = rate - b_g;
    return mcd_host_bsm(spot, strike, rate, q_eff, sigma_g, time, type);
}

extern "C" {

double mcd_black_scholes_merton(double spot, double strike, double rate, double carry_yield, double vol,
                                double time, int type) {
    return mcd_host_bsm(spot, strike, rate, carry_yield, vol, time, type);
}

// analytic.cpp:40-49 (Black 1976 on a forward)
double mcd_black76(double forward, double strike, double rate, double vol, double time, int type) {
    const double sqrt_t = std::sqrt(time);
    const double d1 = (std::log(forward / strike) + 0.5 * vol * vol * time) / (vol * sqrt_t);
    const double d2 = d1 - vol * sqrt_t;
    const double phi = sgn(type);
    const double df = std::exp(-rate * time);
    return phi * df * (forward * mcd_host_normal_cdf(phi * d1) - strike * mcd_host_normal_cdf(phi * d2));
}

double mcd_kemna_vorst(double spot, double strike, double rate, double carry_yield, double vol, double time,
                       int type) {
    return mcd_host_kemna_vorst(spot, strike, rate, carry_yield, vol, time, type);
}

// analytic.cpp:61-132: Reiner-Rubinstein (1991) single-barrier options with a
// rebate, in Haug's A..F notation (eta = +1 down, -1 up; phi = +1 call).
double mcd_reiner_rubinstein(double spot, double strike, double barrier, double rate, double carry_yield,
                             double vol, double time, int type, int direction, int knock, double rebate) {
    const double b = rate - carry_yield;
    const double sqrt_t = std::sqrt(time);
    const double mu = (b - 0.5 * vol * vol) / (vol * vol);
    const double lambda = std::sqrt(mu * mu + 2.0 * rate / (vol * vol));
    const double phi = sgn(type);
    const double eta = direction == MCD_DOWN ? 1.0 : -1.0;
    const double x1 = std::log(spot / strike) / (vol * sqrt_t) + (1.0 + mu) * vol * sqrt_t;
    const double x2 = std::log(spot / barrier) / (vol * sqrt_t) + (1.0 + mu) * vol * sqrt_t;
    const double y1 = std::log(barrier * barrier / (spot * strike)) / (vol * sqrt_t) + (1.0 + mu) * vol * sqrt_t;
    const double y2 = std::log(barrier / spot) / (vol * sqrt_t) + (1.0 + mu) * vol * sqrt_t;
    const double z = std::log(barrier / spot) / (vol * sqrt_t) + lambda * vol * sqrt_t;
    const double dfc = std::exp((b - rate) * time);
    const double dfr = std::exp(-rate * time);
    const double h2m1 = std::pow(barrier / spot, 2.0 * (mu + 1.0));
    const double h2m = std::pow(barrier / spot, 2.0 * mu);
    const auto N = mcd_host_normal_cdf;
    const double A = phi * spot * dfc * N(phi * x1) - phi * strike * dfr * N(phi * x1 - phi * vol * sqrt_t);
    const double B = phi * spot * dfc * N(phi * x2) - phi * strike * dfr * N(phi * x2 - phi * vol * sqrt_t);
    const double C =
        phi * spot * dfc * h2m1 * N(eta * y1) - phi * strike * dfr * h2m * N(eta * y1 - eta * vol * sqrt_t);
    const double D =
        phi * spot * dfc * h2m1 * N(eta * y2) - phi * strike * dfr * h2m * N(eta * y2 - eta * vol * sqrt_t);
    const double E = rebate * dfr * (N(eta * x2 - eta * vol * sqrt_t) - h2m * N(eta * y2 - eta * vol * sqrt_t));
    const double F = rebate * (std::pow(barrier / spot, mu + lambda) * N(eta * z) +
                               std::pow(barrier / spot, mu - lambda) * N(eta * z - 2.0 * eta * lambda * vol * sqrt_t));
    const bool k_above = strike > barrier;
    const bool call = type == MCD_CALL, down = direction == MCD_DOWN;
    if (knock == MCD_IN) {
        if (down) {
            if (call) return k_above ? (C + E) : (A - B + D + E);
            return k_above ? (B - C + D + E) : (A + E);
        }
        if (call) return k_above ? (A + E) : (B - C + D + E);
        return k_above ? (A - B + D + E) : (C + E);
    }
    if (down) {
        if (call) return k_above ? (A - C + F) : (B - D + F);
        return k_above ? (A - B + C - D + F) : F;
    }
    if (call) return k_above ? F : (A - B + C - D + F);
    return k_above ? (B - D + F) : (A - C + F);
}

}  // extern "C"

namespace {

// analytic.cpp:145-190: Goldman-Sosin-Gatto / Conze-Viswanathan lookback
// terms with lambda = 2 (r - q) / sigma^2 and the running extreme = S0.
double lookback_terms(double spot, double reference, double rate, double q, double vol, double time, double eta,
                      bool floating) {
    const double lambda = 2.0 * (rate - q) / (vol * vol);
    const double sd = vol * std::sqrt(time);
    const double d1 = std::log(spot / reference) / sd + 0.5 * (lambda + 1.0) * sd;
    const auto N = mcd_host_normal_cdf;
    const double pw = std::pow(spot / reference, -lambda);
    const double dfc = std::exp(-q * time);
    const double dfr = std::exp(-rate * time);
    if (!floating) {
        const double n1 = N(eta * d1), n2 = N(eta * (d1 - sd)), n3 = N(eta * (d1 - lambda * sd)), n4 = N(eta * d1);
        return eta * (spot * dfc * n1 - reference * dfr * n2 - spot * dfr * (pw * n3 - dfc * n4 / dfr) / lambda);
    }
    const double n1 = N(eta * d1), n2 = N(eta * (d1 - sd)), n3 = N(eta * (-d1 + lambda * sd)), n4 = N(eta * -d1);
    return eta * ((spot * dfc * n1 - reference * dfr * n2) + spot * dfr * (pw * n3 - dfc * n4 / dfr) / lambda);
}

}  // namespace

extern "C" {

double mcd_lookback_fixed_strike(double spot, double strike, double rate, double carry_yield, double vol,
                                 double time, int type) {
    const double eta = sgn(type);
    const bool in_the_money = type == MCD_CALL ? strike <= spot : strike >= spot;
    if (in_the_money)
        return lookback_terms(spot, spot, rate, carry_yield, vol, time, eta, false) +
               eta * std::exp(-rate * time) * (spot - strike);
    return lookback_terms(spot, strike, rate, carry_yield, vol, time, eta, false);
}

double mcd_lookback_floating_strike(double spot, double rate, double carry_yield, double vol, double time,
                                    int type) {
    return lookback_terms(spot, spot, rate, carry_yield, vol, time, sgn(type), true);
}

// analytic.cpp:210-218 (cash- or asset-or-nothing)
double mcd_digital_analytic(double spot, double strike, double rate, double carry_yield, double vol, double time,
                            int type, int style, double cash_amount) {
    const double b = rate - carry_yield;
    const double sqrt_t = std::sqrt(time);
    const double d1 = (std::log(spot / strike) + (b + 0.5 * vol * vol) * time) / (vol * sqrt_t);
    const double d2 = d1 - vol * sqrt_t;
    const double phi = sgn(type);
    if (style == MCD_CASH_OR_NOTHING) return cash_amount * std::exp(-rate * time) * mcd_host_normal_cdf(phi * d2);
    return spot * std::exp(-carry_yield * time) * mcd_host_normal_cdf(phi * d1);
}

// analytic.cpp:224-235
double mcd_forward_price(double spot, double rate, double carry_yield, double time) {
    return spot * std::exp((rate - carry_yield) * time);
}
double mcd_forward_value(double forward_now, double forward_at_inception, double rate, double time_to_expiry) {
    return (forward_now - forward_at_inception) * std::exp(-rate * time_to_expiry);
}
double mcd_futures_mark_to_market(double futures_price_new, double futures_price_old) {
    return futures_price_new - futures_price_old;
}

}  // extern "C"

namespace {

// Cox-Ross-Rubinstein lattice (binomial.cpp): u = e^{sigma sqrt(dt)}, d = 1/u,
// p = (e^{(r-q) dt} - d)/(u - d), backward induction with the one-step
// discount; american adds the early-exercise max at every node.
double lattice(double spot, double strike, double rate, double carry_yield, double vol, double time, int steps,
               int type, bool american, double* p_out, double* u_out, double* d_out) {
    const double dt = time / static_cast<double>(steps);
    const double u = std::exp(vol * std::sqrt(dt));
    const double d = 1.0 / u;
    const double p = (std::exp((rate - carry_yield) * dt) - d) / (u - d);
    const double disc = std::exp(-rate * dt);
    const double phi = sgn(type);
    auto node = [&](int level, int i) {
        return spot * std::pow(u, static_cast<double>(i)) * std::pow(d, static_cast<double>(level - i));
    };
    std::vector<double> v(static_cast<size_t>(steps) + 1);
    for (int i = 0; i <= steps; ++i) v[i] = std::max(phi * (node(steps, i) - strike), 0.0);
    for (int level = steps - 1; level >= 0; --level)
        for (int i = 0; i <= level; ++i) {
            const double cont = disc * (p * v[i + 1] + (1.0 - p) * v[i]);
            v[i] = american ? std::max(cont, std::max(phi * (node(level, i) - strike), 0.0)) : cont;
        }
    if (p_out) *p_out = p;
    if (u_out) *u_out = u;
    if (d_out) *d_out = d;
    return v[0];
}

// heston.cpp:26-40: characteristic function of ln S_T in the "little trap"
// form (Albrecher, Mayer, Schoutens and Tistaert 2007).
std::complex<double> heston_cf(const mcd_heston_params& p, std::complex<double> u) {
    const std::complex<double> i(0.0, 1.0);
    const std::complex<double> bmr = p.kappa - p.rho * p.xi * i * u;
    const std::complex<double> d = std::sqrt(bmr * bmr + p.xi * p.xi * (i * u + u * u));
    const std::complex<double> g = (bmr - d) / (bmr + d);
    const std::complex<double> e = std::exp(-d * p.time);
    const std::complex<double> c = i * u * (p.rate - p.carry_yield) * p.time +
                                   (p.kappa * p.theta / (p.xi * p.xi)) *
                                       ((bmr - d) * p.time - 2.0 * std::log((1.0 - g * e) / (1.0 - g)));
    const std::complex<double> dd = (bmr - d) / (p.xi * p.xi) * (1.0 - e) / (1.0 - g * e);
    return std::exp(c + dd * p.v0);
}

// Gauss-Legendre nodes and weights on [-1, 1] (Newton on P_n).
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    const double pi = 3.14159265358979323846;
    for (int k = 0; k < (n + 1) / 2; ++k) {
        double z = std::cos(pi * (k + 0.75) / (n + 0.5)), dp = 1.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int j = 2; j <= n; ++j) {
                const double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            const double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-15) break;
        }
        x[k] = -z;
        x[n - 1 - k] = z;
        w[k] = w[n - 1 - k] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

}  // namespace

extern "C" {

double mcd_crr_binomial_american(double spot, double strike, double rate, double carry_yield, double vol,
                                 double time, int steps, int type) try {
    if (steps < 1) return std::nan("");
    return lattice(spot, strike, rate, carry_yield, vol, time, steps, type, true, nullptr, nullptr, nullptr);
} catch (...) {
    return std::nan("");
}

int mcd_crr_binomial(double spot, double strike, double rate, double carry_yield, double vol, double time, int steps,
                     int type, double* price_p_u_d) try {
    if (steps < 1 || !price_p_u_d) return MCD_ERR_INVALID_ARGUMENT;
    price_p_u_d[0] = lattice(spot, strike, rate, carry_yield, vol, time, steps, type, false, &price_p_u_d[1],
                             &price_p_u_d[2], &price_p_u_d[3]);
    return MCD_OK;
} catch (...) {  // a lattice too large for host memory
    return MCD_ERR_OUT_OF_MEMORY;
}

// Bermudan CRR lattice (no reference counterpart): exercise only at the
// levels steps_per_date * j, j = 0..dates-1 (t = 0 included, as the
// reference's LSM decides at inception), the European payoff at maturity.
// Node values come from a table of powers of u (one pow per level offset).
double mcd_crr_binomial_bermudan(double spot, double strike, double rate, double carry_yield, double vol,
                                 double time, int exercise_dates, int steps_per_date, int type) try {
    if (exercise_dates < 1 || steps_per_date < 1 || exercise_dates > (1 << 20) / steps_per_date)
        return std::nan("");
    const int steps = exercise_dates * steps_per_date;
    const double dt = time / static_cast<double>(steps);
    const double u = std::exp(vol * std::sqrt(dt));
    const double d = 1.0 / u;
    const double p = (std::exp((rate - carry_yield) * dt) - d) / (u - d);
    const double disc = std::exp(-rate * dt);
    const double phi = sgn(type);
    std::vector<double> upow(2 * static_cast<size_t>(steps) + 1);
    for (int k = -steps; k <= steps; ++k) upow[static_cast<size_t>(k + steps)] = std::pow(u, static_cast<double>(k));
    auto node = [&](int level, int i) { return spot * upow[static_cast<size_t>(2 * i - level + steps)]; };
    std::vector<double> v(static_cast<size_t>(steps) + 1);
    for (int i = 0; i <= steps; ++i) v[i] = std::max(phi * (node(steps, i) - strike), 0.0);
    for (int level = steps - 1; level >= 0; --level) {
        const bool exercise = level % steps_per_date == 0;
        for (int i = 0; i <= level; ++i) {
            const double cont = disc * (p * v[i + 1] + (1.0 - p) * v[i]);
            v[i] = exercise ? std::max(cont, std::max(phi * (node(level, i) - strike), 0.0)) : cont;
        }
    }
    return v[0];
} catch (...) {
    return std::nan("");
}

// heston.cpp:48-82: Heston (1993) P1/P2 as integrals over [0, 200] by
// 128-point Gauss-Legendre; the put from parity.
double mcd_heston_semi_analytic(const mcd_heston_params* params, double strike, int type) try {
    if (!params) return std::nan("");
    static const auto rule = [] {
        std::vector<double> x, w;
        gauss_legendre(128, x, w);
        return std::make_pair(x, w);
    }();
    const mcd_heston_params& p = *params;
    const std::complex<double> i(0.0, 1.0);
    const double k = std::log(strike / p.spot);
    const std::complex<double> phi_minus_i = heston_cf(p, std::complex<double>(0.0, -1.0));
    const double half = 100.0, mid = 100.0;
    double s1 = 0.0, s2 = 0.0;
    for (size_t j = 0; j < rule.first.size(); ++j) {
        const double u = mid + half * rule.first[j];
        const std::complex<double> kernel = std::exp(-i * u * k);
        s1 += rule.second[j] * std::real(kernel * (heston_cf(p, std::complex<double>(u, -1.0)) / phi_minus_i) / (i * u));
        s2 += rule.second[j] * std::real(kernel * heston_cf(p, std::complex<double>(u, 0.0)) / (i * u));
    }
    const double pi = 3.14159265358979323846;
    const double p1 = 0.5 + half * s1 / pi, p2 = 0.5 + half * s2 / pi;
    const double dq = std::exp(-p.carry_yield * p.time), dr = std::exp(-p.rate * p.time);
    const double call = p.spot * dq * p1 - strike * dr * p2;
    return type == MCD_CALL ? call : call - p.spot * dq + strike * dr;
} catch (...) {
    return std::nan("");
}

}  // extern "C"
