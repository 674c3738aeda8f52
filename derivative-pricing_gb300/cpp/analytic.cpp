// analytic.cpp -- the closed forms and lattices the JSON CLI also serves
// (host FP64; no GPU): forward price, Cox-Ross-Rubinstein trees and the
// semi-analytic Heston price.  Restated from the published methods the
// reference implements (src/pricers/analytic.cpp:224-226,
// src/pricers/binomial.cpp, src/pricers/heston.cpp:26-82).
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "mcd_shim.hpp"

namespace mcd::pricers {

namespace {

double payoff(double s, double k, OptionType type) {
    const double phi = type == OptionType::Call ? 1.0 : -1.0;
    return std::max(phi * (s - k), 0.0);
}

struct Tree {
    double u, d, p, disc;
};

// Cox-Ross-Rubinstein: u = e^{vol sqrt(dt)}, d = 1/u, risk-neutral
// p = (e^{(r-q) dt} - d)/(u - d), one-step discount e^{-r dt}.
Tree crr(double rate, double carry_yield, double vol, double time, int steps) {
    const double dt = time / static_cast<double>(steps);
    Tree t;
    t.u = std::exp(vol * std::sqrt(dt));
    t.d = 1.0 / t.u;
    t.p = (std::exp((rate - carry_yield) * dt) - t.d) / (t.u - t.d);
    t.disc = std::exp(-rate * dt);
    return t;
}

// Spot at node (level, i up-moves): S0 u^i d^(level-i).
double node_spot(double spot, const Tree& t, int level, int i) {
    return spot * std::pow(t.u, static_cast<double>(i)) * std::pow(t.d, static_cast<double>(level - i));
}

double lattice(double spot, double strike, const Tree& t, int steps, OptionType type, bool american) {
    std::vector<double> v(static_cast<size_t>(steps) + 1);
    for (int i = 0; i <= steps; ++i) v[i] = payoff(node_spot(spot, t, steps, i), strike, type);
    for (int level = steps - 1; level >= 0; --level) {
        for (int i = 0; i <= level; ++i) {
            const double cont = t.disc * (t.p * v[i + 1] + (1.0 - t.p) * v[i]);
            v[i] = american ? std::max(cont, payoff(node_spot(spot, t, level, i), strike, type)) : cont;
        }
    }
    return v[0];
}

// Gauss-Legendre nodes and weights on [-1, 1] by Newton iteration on P_n.
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < (n + 1) / 2; ++i) {
        double z = std::cos(pi * (i + 0.75) / (n + 0.5));
        double dp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; ++k) {
                const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            const double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-15) break;
        }
        x[i] = -z;
        x[n - 1 - i] = z;
        w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

// Heston characteristic function of ln S_T, "little trap" form (Albrecher,
// Mayer, Schoutens and Tistaert 2007).
std::complex<double> heston_cf(const models::HestonParams& p, std::complex<double> u) {
    const std::complex<double> i(0.0, 1.0);
    const std::complex<double> b = p.kappa - p.rho * p.xi * i * u;
    const std::complex<double> d = std::sqrt(b * b + p.xi * p.xi * (i * u + u * u));
    const std::complex<double> g = (b - d) / (b + d);
    const std::complex<double> e = std::exp(-d * p.time);
    const std::complex<double> c = i * u * (p.rate - p.carry_yield) * p.time +
                                   (p.kappa * p.theta / (p.xi * p.xi)) *
                                       ((b - d) * p.time - 2.0 * std::log((1.0 - g * e) / (1.0 - g)));
    const std::complex<double> dd = (b - d) / (p.xi * p.xi) * (1.0 - e) / (1.0 - g * e);
    return std::exp(c + dd * p.v0);
}

}  // namespace

double forward_price(double spot, double rate, double carry_yield, double time) {
    return spot * std::exp((rate - carry_yield) * time);
}

BinomialResult crr_binomial(double spot, double strike, double rate, double carry_yield, double vol, double time,
                            int steps, OptionType type) {
    const Tree t = crr(rate, carry_yield, vol, time, steps);
    return BinomialResult{lattice(spot, strike, t, steps, type, false), t.p, t.u, t.d};
}

double crr_binomial_american(double spot, double strike, double rate, double carry_yield, double vol, double time,
                             int steps, OptionType type) {
    return lattice(spot, strike, crr(rate, carry_yield, vol, time, steps), steps, type, true);
}

// Heston (1993) P1/P2 probabilities, each an integral over [0, 200] by
// 128-point Gauss-Legendre (the reference's rule, heston.cpp:48-82).
double heston_semi_analytic(const models::HestonParams& p, double strike, OptionType type) {
    static const auto rule = [] {
        std::vector<double> x, w;
        gauss_legendre(128, x, w);
        return std::make_pair(x, w);
    }();
    const std::complex<double> i(0.0, 1.0);
    const double k = std::log(strike / p.spot);
    const std::complex<double> phi_minus_i = heston_cf(p, std::complex<double>(0.0, -1.0));
    const double half = 100.0, mid = 100.0;
    double s1 = 0.0, s2 = 0.0;
    for (size_t j = 0; j < rule.first.size(); ++j) {
        const double u = mid + half * rule.first[j];
        const std::complex<double> kernel = std::exp(-i * u * k) / (i * u);
        s1 += rule.second[j] * std::real(kernel * heston_cf(p, std::complex<double>(u, -1.0)) / phi_minus_i);
        s2 += rule.second[j] * std::real(kernel * heston_cf(p, std::complex<double>(u, 0.0)));
    }
    const double pi = 3.14159265358979323846;
    const double p1 = 0.5 + half * s1 / pi, p2 = 0.5 + half * s2 / pi;
    const double call = p.spot * std::exp(-p.carry_yield * p.time) * p1 - strike * std::exp(-p.rate * p.time) * p2;
    if (type == OptionType::Call) return call;
    return call - p.spot * std::exp(-p.carry_yield * p.time) + strike * std::exp(-p.rate * p.time);
}

}  // namespace mcd::pricers
