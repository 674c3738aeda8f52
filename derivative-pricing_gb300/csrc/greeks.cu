// greeks.cu -- Monte Carlo sensitivities of a batch of GBM contracts in one
// persistent launch: common-random-number finite differences (spot and vol
// bumps), pathwise and likelihood-ratio estimators, all from one pass over
// each path's draws.
//
// The work items, slab layout, reduction trees and merge are those of the
// path engine (gbm_paths.cu), so the price output of this kernel is bitwise
// the price of mcd_price_batch for the same contract and precision.
//
// Reference semantics:
//   finite differences  src/greeks/finite_difference.cpp:40-65 (central
//                       differences of CRN re-prices; here per path, so the
//                       estimate comes with its standard error)
//   likelihood ratio    src/greeks/likelihood_ratio.cpp:33-73 (terminal) and
//                       :105-154 (barrier: first-step score for delta and
//                       gamma, per-step sums for vega and rho); the same
//                       first-step score is applied to Asian and lookback
//                       payoffs, which the reference does not cover
//   pathwise            src/greeks/pathwise.cpp:28-55 (European), :64-147
//                       (Asian)
//
// FP64 evaluates every bumped state literally (the arithmetic of five
// separate re-prices).  FP32 shares one log-path between the spot states
// (only the FP64 payoff is rescaled) and carries the vol-bumped states as
// differentials: with D_i = dx_i/dvol = sqrt(dt) W_i - vol i dt, the bumped
// log-spot is x_i +/- h D_i - h^2 i dt / 2 exactly, and its effect on a sum
// of spots is sum S_i expm1(+/- h D_i - h^2 i dt / 2), which FP32 resolves to
// full relative precision even for bumps of 1e-4 (a plain FP32 re-price
// would lose the difference in rounding noise).
//
// nvcc-flags: --fmad=false
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "engine.hpp"
#include "greeks.hpp"

namespace mcdg {

namespace {

__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }

// expm1 for the vol-bump exponents: a short Taylor series where |a| < 1/64
// (relative error below 2e-12 there; bumps of 1e-4 give |a| ~ 1e-4), else
// __expf(a) - 1 (relative error ~1e-7 / |a|, used for bumps above ~1 %).
__device__ __forceinline__ float expm1_small(float a) {
    if (fabsf(a) < 0.015625f) {
        const float p = __fmaf_rn(__fmaf_rn(__fmaf_rn(a, 1.0f / 120.0f, 1.0f / 24.0f), a, 1.0f / 6.0f), a, 0.5f);
        return __fmaf_rn(p * a, a, a);
    }
    return __expf(a) - 1.0f;
}

// expm1 by its cubic Taylor polynomial, for exponents the host bounds by
// 1e-2 (DevGreeks::vol_series): the first omitted term is below a^3 / 24 <
// 5e-8 of the result, under an FP32 rounding, in three instructions and
// without the range test of expm1_small.
__device__ __forceinline__ float expm1_series(float a) {
    return __fmaf_rn(__fmaf_rn(a, 1.0f / 6.0f, 0.5f) * a, a, a);
}

// Likelihood-ratio scores of the first step (likelihood_ratio.cpp:45-49,
// :140-142), with sqrt_t = sqrt(dt) of that step.
__device__ __forceinline__ void lr_first_step(double h, double z1, double spot, double vol, double sqrt_t, double t,
                                              double (&o)[kNumGreeks]) {
    const double delta_score = z1 / (spot * vol * sqrt_t);
    const double gamma_score = (z1 * z1 - vol * sqrt_t * z1 - 1.0) / (spot * spot * vol * vol * t);
    o[kGLrDelta] = h * delta_score;
    o[kGLrGamma] = h * gamma_score;
}

// ===========================================================================
// FP64: five literal states (base, spot up/down, vol up/down)
// ===========================================================================
template <int KIND>
__device__ void greeks64(const DevContract& c, const DevGreeks& g, const PhiloxKeys& k, uint64_t path,
                         double (&o)[kNumGreeks]) {
#pragma unroll
    for (int i = 0; i < kNumGreeks; ++i) o[i] = 0.0;
    const double phi = c.type == 0 ? 1.0 : -1.0;
    const PhiloxPath pp = philox_path(path, 0u, k);
    double v[5];
    if constexpr (KIND == kEuropean || KIND == kDigital) {
        const double z = normal_from_bits_f64(philox_word0(pp, 0u, k));
        const double m = exp(c.drift + c.vs * z);
        const double st[5] = {c.spot * m, (c.spot + g.h_spot) * m, (c.spot - g.h_spot) * m,
                              c.spot * exp(g.drift_up + g.vs_up * z), c.spot * exp(g.drift_dn + g.vs_dn * z)};
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            if constexpr (KIND == kEuropean) {
                v[j] = c.discount * dmax(phi * (st[j] - c.strike), 0.0);
            } else {
                const bool itm = phi * (st[j] - c.strike) > 0.0;
                v[j] = c.discount * (itm ? (c.asset ? st[j] : c.cash) : 0.0);
            }
        }
        const double h = v[0];
        // likelihood_ratio.cpp:40-64
        const double sqrt_t = g.sqrt_dt;
        lr_first_step(h, z, c.spot, g.vol, sqrt_t, g.time, o);
        const double vega_score = (z * z - 1.0) / g.vol - sqrt_t * z;
        const double rho_raw = sqrt_t * z / g.vol;
        const double theta_raw = (z * z - 1.0) / (2.0 * g.time) + g.mu * z / (g.vol * sqrt_t);
        o[kGLrVega] = h * vega_score;
        o[kGLrRho] = h * (rho_raw - g.time);
        o[kGLrTheta] = h * (g.rate - theta_raw);
        if constexpr (KIND == kEuropean) {  // pathwise.cpp:37-50
            const double s_t = st[0];
            const bool itm = phi * (s_t - c.strike) > 0.0;
            const double slope = itm ? phi : 0.0;
            const double ds_dspot = s_t / c.spot;
            const double ds_dvol = s_t * (sqrt_t * z - g.vol * g.time);
            const double ds_drate = s_t * g.time;
            o[kGPwDelta] = c.discount * slope * ds_dspot;
            o[kGPwVega] = c.discount * slope * ds_dvol;
            o[kGPwRho] = c.discount * slope * ds_drate - g.time * h;
        }
    } else {
        double s[5] = {c.spot, c.spot + g.h_spot, c.spot - g.h_spot, c.spot, c.spot};
        double sum[5] = {0.0, 0.0, 0.0, 0.0, 0.0}, lsum[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        double hi[5], lo[5];
        bool br[5] = {false, false, false, false, false};
#pragma unroll
        for (int j = 0; j < 5; ++j) hi[j] = lo[j] = s[j];
        double z1 = 0.0, vega_sum = 0.0, rho_sum = 0.0, cum_z = 0.0;
        double sum_s_dvol = 0.0, sum_dlns_dvol = 0.0, sum_s_drate = 0.0, sum_dlns_drate = 0.0;
        double last_s_dvol = 0.0, last_s_drate = 0.0;
        for (int step = 0; step < c.n_steps; ++step) {
            const double z = normal_from_bits_f64(philox_word0(pp, static_cast<uint32_t>(step), k));
            if (step == 0) z1 = z;
            vega_sum += (z * z - 1.0) / g.vol - g.sqrt_dt * z;
            rho_sum += g.sqrt_dt * z / g.vol;
            const double m = exp(c.drift + c.vs * z);
            s[0] = s[0] * m;
            s[1] = s[1] * m;
            s[2] = s[2] * m;
            s[3] = s[3] * exp(g.drift_up + g.vs_up * z);
            s[4] = s[4] * exp(g.drift_dn + g.vs_dn * z);
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                if constexpr (KIND == kAsianArith) {
                    sum[j] += s[j];
                } else if constexpr (KIND == kAsianGeo) {
                    lsum[j] += log(s[j]);
                } else if constexpr (KIND == kBarrier) {
                    const bool crossed = c.up ? s[j] >= c.barrier : s[j] <= c.barrier;
                    br[j] = br[j] || crossed;
                } else {
                    hi[j] = dmax(hi[j], s[j]);
                    lo[j] = dmin(lo[j], s[j]);
                }
            }
            if constexpr (KIND == kAsianArith || KIND == kAsianGeo) {  // pathwise.cpp:81-98
                cum_z += z;
                const double i = static_cast<double>(step + 1);
                const double dlns_dvol = -g.vol * i * g.dt + g.sqrt_dt * cum_z;
                const double dlns_drate = i * g.dt;
                const double ds_dvol = s[0] * dlns_dvol;
                const double ds_drate = s[0] * dlns_drate;
                sum_s_dvol += ds_dvol;
                sum_dlns_dvol += dlns_dvol;
                sum_s_drate += ds_drate;
                sum_dlns_drate += dlns_drate;
                last_s_dvol = ds_dvol;
                last_s_drate = ds_drate;
            }
        }
        const double n = static_cast<double>(c.n_steps);
        double avg0 = 0.0;
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            if constexpr (KIND == kAsianArith || KIND == kAsianGeo) {
                const double avg = KIND == kAsianArith ? sum[j] / n : exp(lsum[j] / n);
                if (j == 0) avg0 = avg;
                const double ref = c.floating ? (s[j] - avg) : (avg - c.strike);
                v[j] = c.discount * dmax(phi * ref, 0.0);
            } else if constexpr (KIND == kBarrier) {
                const double vanilla = dmax(phi * (s[j] - c.strike), 0.0);
                const bool pays = c.out ? !br[j] : br[j];
                v[j] = c.discount * (pays ? vanilla : c.rebate);
            } else if constexpr (KIND == kLookbackFixed) {
                v[j] = c.discount * (c.type == 0 ? dmax(hi[j] - c.strike, 0.0) : dmax(c.strike - lo[j], 0.0));
            } else {
                v[j] = c.discount * (c.type == 0 ? (s[j] - lo[j]) : (hi[j] - s[j]));
            }
        }
        const double h = v[0];
        lr_first_step(h, z1, c.spot, g.vol, g.sqrt_dt, g.dt, o);
        o[kGLrVega] = h * vega_sum;
        o[kGLrRho] = h * (rho_sum - g.time);
        if constexpr (KIND == kAsianArith || KIND == kAsianGeo) {  // pathwise.cpp:100-140
            const bool arith = KIND == kAsianArith;
            const double d_avg_dspot = avg0 / c.spot;
            const double d_avg_dvol = arith ? sum_s_dvol / n : avg0 * (sum_dlns_dvol / n);
            const double d_avg_drate = arith ? sum_s_drate / n : avg0 * (sum_dlns_drate / n);
            const double d_slast_dspot = s[0] / c.spot;
            const double ref = c.floating ? (s[0] - avg0) : (avg0 - c.strike);
            const bool itm = phi * ref > 0.0;
            const double slope = itm ? phi : 0.0;
            double delta_raw, vega_raw, rate_raw;
            if (!c.floating) {
                delta_raw = slope * d_avg_dspot;
                vega_raw = slope * d_avg_dvol;
                rate_raw = slope * d_avg_drate;
            } else {
                delta_raw = slope * (d_slast_dspot - d_avg_dspot);
                vega_raw = slope * (last_s_dvol - d_avg_dvol);
                rate_raw = slope * (last_s_drate - d_avg_drate);
            }
            o[kGPwDelta] = c.discount * delta_raw;
            o[kGPwVega] = c.discount * vega_raw;
            o[kGPwRho] = c.discount * rate_raw - g.time * h;
        }
    }
    o[kGPrice] = v[0];
    o[kGFdDelta] = (v[1] - v[2]) / (2.0 * g.h_spot);
    o[kGFdGamma] = (v[1] - 2.0 * v[0] + v[2]) / (g.h_spot * g.h_spot);
    o[kGFdVega] = (v[3] - v[4]) / (2.0 * g.h_vol);
}

// ===========================================================================
// FP32: one log-path, differential vol states, FP64 payoffs of the states
// ===========================================================================
template <int KIND, bool SER>
__device__ void greeks32(const DevContract& c, const DevGreeks& g, const PhiloxKeys& k, uint64_t path,
                         double (&o)[kNumGreeks]) {
#pragma unroll
    for (int i = 0; i < kNumGreeks; ++i) o[i] = 0.0;
    const float phi = c.type == 0 ? 1.0f : -1.0f;
    const double phid = c.type == 0 ? 1.0 : -1.0;
    const float mu = static_cast<float>(c.drift);
    const float sg = static_cast<float>(c.vs);
    const float s0 = static_cast<float>(c.spot);
    const float strike = static_cast<float>(c.strike);
    const double S0 = c.spot, K = c.strike, disc = c.discount, hs = g.h_spot, hv = g.h_vol;
    const float hvf = static_cast<float>(hv);
    const float cq = static_cast<float>(0.5 * hv * hv * g.dt);
    const PhiloxPath pp = philox_path(path, 0u, k);
    double v[5];
    if constexpr (KIND == kEuropean || KIND == kDigital) {
        const float z = normal_from_bits_f32(philox_word0(pp, 0u, k));
        const float ef = __expf(__fmaf_rn(sg, z, mu));
        const float s = s0 * ef;  // as the path engine
        float payoff;
        if constexpr (KIND == kEuropean) {
            payoff = fmaxf(phi * (s - strike), 0.0f);
        } else {
            const bool itm = phi * (s - strike) > 0.0f;
            payoff = itm ? (c.asset ? s : static_cast<float>(c.cash)) : 0.0f;
        }
        o[kGPrice] = c.discount * static_cast<double>(payoff);
        const float D = __fmaf_rn(static_cast<float>(g.sqrt_dt), z, -static_cast<float>(g.vol * g.time));
        const double em_up = static_cast<double>(expm1_small(__fmaf_rn(hvf, D, -cq)));
        const double em_dn = static_cast<double>(expm1_small(__fmaf_rn(-hvf, D, -cq)));
        const double st0 = S0 * static_cast<double>(ef);
        const double st[5] = {st0, (S0 + hs) * static_cast<double>(ef), (S0 - hs) * static_cast<double>(ef),
                              st0 + st0 * em_up, st0 + st0 * em_dn};
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            if constexpr (KIND == kEuropean) {
                v[j] = disc * dmax(phid * (st[j] - K), 0.0);
            } else {
                const bool itm = phid * (st[j] - K) > 0.0;
                v[j] = disc * (itm ? (c.asset ? st[j] : c.cash) : 0.0);
            }
        }
        const double h = v[0];
        const double zd = static_cast<double>(z);
        const double sqrt_t = g.sqrt_dt;
        o[kGLrDelta] = h * (zd * g.lr_delta_scale);
        o[kGLrGamma] = h * ((zd * zd - g.vol * sqrt_t * zd - 1.0) * g.lr_gamma_scale);
        o[kGLrVega] = h * ((zd * zd - 1.0) * g.inv_vol - sqrt_t * zd);
        o[kGLrRho] = h * (g.sqrt_dt_over_vol * zd - g.time);
        o[kGLrTheta] = h * (g.rate - ((zd * zd - 1.0) * g.inv_2t + g.mu_over_vol_sqrt_t * zd));
        if constexpr (KIND == kEuropean) {
            const bool itm = phid * (st0 - K) > 0.0;
            const double slope = itm ? phid : 0.0;
            o[kGPwDelta] = disc * slope * static_cast<double>(ef);
            o[kGPwVega] = disc * slope * st0 * static_cast<double>(D);
            o[kGPwRho] = disc * slope * st0 * g.time - g.time * h;
        }
    } else {
        const float lnh = static_cast<float>(c.log_h_rel);
        const float lnh_su = static_cast<float>(g.log_h_rel_up);
        const float lnh_sd = static_cast<float>(g.log_h_rel_dn);
        const float sqdt = static_cast<float>(g.sqrt_dt);
        const float vdt = static_cast<float>(g.vol * g.dt);
        const float inv_vol = static_cast<float>(1.0 / g.vol);
        // Per step: the log-spot x (as the path engine), the running sums of
        // the draws and of their squares (the likelihood-ratio vega and rho
        // scores follow from them), D = dx/dvol = sqrt(dt) sum z - vol i dt,
        // and the vol-bump exponents +/- h D - h^2 i dt / 2.  A barrier or
        // lookback state needs only the running extremes of x, x + e_up and
        // x + e_dn: a barrier is touched on some date exactly when the extreme
        // over the dates reaches it.
        float x = 0.0f, D = 0.0f, z1 = 0.0f, zsum = 0.0f, zsq = 0.0f, fi = 0.0f;
        float acc = 0.0f, acc2 = 0.0f, xmax = 0.0f, xmin = 0.0f;  // as the path engine
        float a_d = 0.0f, a_r = 0.0f, a_up = 0.0f, a_dn = 0.0f, sd = 0.0f;
        float xmax_up = 0.0f, xmin_up = 0.0f, xmax_dn = 0.0f, xmin_dn = 0.0f;
        float e_up = 0.0f, e_dn = 0.0f;  // bump exponents of the last step
        if constexpr (KIND == kBarrier) {  // extremes over the monitoring dates only
            const float start = c.up ? -3.0e38f : 3.0e38f;
            xmax = xmin = xmax_up = xmin_up = xmax_dn = xmin_dn = start;
        }
        for (int step = 0; step < c.n_steps; ++step) {
            const float z = normal_from_bits_f32(philox_word0(pp, static_cast<uint32_t>(step), k));
            if (step == 0) z1 = z;
            x = __fmaf_rn(sg, z, x + mu);
            zsum += z;
            zsq = __fmaf_rn(z, z, zsq);
            fi += 1.0f;
            D = __fmaf_rn(sqdt, zsum, -vdt * fi);
            const float q = cq * fi;
            e_up = __fmaf_rn(hvf, D, -q);
            e_dn = __fmaf_rn(-hvf, D, -q);
            if constexpr (KIND == kAsianArith) {
                const float e = __expf(x);
                acc += e;
                a_d = __fmaf_rn(e, D, a_d);
                a_r = __fmaf_rn(e, fi, a_r);
                a_up = __fmaf_rn(e, SER ? expm1_series(e_up) : expm1_small(e_up), a_up);
                a_dn = __fmaf_rn(e, SER ? expm1_series(e_dn) : expm1_small(e_dn), a_dn);
            } else if constexpr (KIND == kAsianGeo) {
                acc2 += x;
                sd += D;
            } else if constexpr (KIND == kBarrier) {
                if (c.up) {
                    xmax = fmaxf(xmax, x);
                    xmax_up = fmaxf(xmax_up, x + e_up);
                    xmax_dn = fmaxf(xmax_dn, x + e_dn);
                } else {
                    xmin = fminf(xmin, x);
                    xmin_up = fminf(xmin_up, x + e_up);
                    xmin_dn = fminf(xmin_dn, x + e_dn);
                }
            } else {
                xmax = fmaxf(xmax, x);
                xmin = fminf(xmin, x);
                xmax_up = fmaxf(xmax_up, x + e_up);
                xmin_up = fminf(xmin_up, x + e_up);
                xmax_dn = fmaxf(xmax_dn, x + e_dn);
                xmin_dn = fminf(xmin_dn, x + e_dn);
            }
        }
        // sum over steps of (z^2 - 1) / vol - sqrt(dt) z
        const float lr_vega = __fmaf_rn(zsq - fi, inv_vol, -sqdt * zsum);
        bool br = false, br_su = false, br_sd = false, br_vu = false, br_vd = false;
        if constexpr (KIND == kBarrier) {
            if (c.up) {
                br = xmax >= lnh;
                br_su = xmax >= lnh_su;
                br_sd = xmax >= lnh_sd;
                br_vu = xmax_up >= lnh;
                br_vd = xmax_dn >= lnh;
            } else {
                br = xmin <= lnh;
                br_su = xmin <= lnh_su;
                br_sd = xmin <= lnh_sd;
                br_vu = xmin_up <= lnh;
                br_vd = xmin_dn <= lnh;
            }
        }
        // price: the path engine's FP32 payoff
        const float inv_n = 1.0f / static_cast<float>(c.n_steps);
        const float lastf = s0 * __expf(x);
        if constexpr (KIND == kAsianArith || KIND == kAsianGeo) {
            const float avg = KIND == kAsianArith ? s0 * (acc * inv_n) : s0 * __expf(acc2 * inv_n);
            const float ref = c.floating ? (lastf - avg) : (avg - strike);
            o[kGPrice] = c.discount * static_cast<double>(fmaxf(phi * ref, 0.0f));
        } else if constexpr (KIND == kBarrier) {
            const float vanilla = fmaxf(phi * (lastf - strike), 0.0f);
            const bool pays = c.out ? !br : br;
            o[kGPrice] = c.discount * static_cast<double>(pays ? vanilla : static_cast<float>(c.rebate));
        } else if constexpr (KIND == kLookbackFixed) {
            const float val = c.type == 0 ? fmaxf(s0 * __expf(xmax) - strike, 0.0f)
                                          : fmaxf(strike - s0 * __expf(xmin), 0.0f);
            o[kGPrice] = c.discount * static_cast<double>(val);
        } else {
            const float val = c.type == 0 ? (lastf - s0 * __expf(xmin)) : (s0 * __expf(xmax) - lastf);
            o[kGPrice] = c.discount * static_cast<double>(val);
        }
        // the five states in FP64
        const double n = static_cast<double>(c.n_steps);
        const double le = static_cast<double>(__expf(x));  // S_n / S0
        const double em_up_n = static_cast<double>(expm1_small(e_up));
        const double em_dn_n = static_cast<double>(expm1_small(e_dn));
        const double last0 = S0 * le;
        const double last[5] = {last0, (S0 + hs) * le, (S0 - hs) * le, last0 + last0 * em_up_n,
                                last0 + last0 * em_dn_n};
        double avg0 = 0.0;
        if constexpr (KIND == kAsianArith || KIND == kAsianGeo) {
            double avg[5];
            if constexpr (KIND == kAsianArith) {
                const double a = static_cast<double>(acc) * g.inv_n;
                avg[0] = S0 * a;
                avg[1] = (S0 + hs) * a;
                avg[2] = (S0 - hs) * a;
                avg[3] = avg[0] + S0 * (static_cast<double>(a_up) * g.inv_n);
                avg[4] = avg[0] + S0 * (static_cast<double>(a_dn) * g.inv_n);
            } else {
                const double gm = exp(static_cast<double>(acc2) * g.inv_n);
                const double dbar = static_cast<double>(sd) * g.inv_n;
                const double ibar = 0.5 * (n + 1.0) * g.dt;  // mean of i dt
                avg[0] = S0 * gm;
                avg[1] = (S0 + hs) * gm;
                avg[2] = (S0 - hs) * gm;
                avg[3] = avg[0] + avg[0] * expm1(hv * dbar - 0.5 * hv * hv * ibar);
                avg[4] = avg[0] + avg[0] * expm1(-hv * dbar - 0.5 * hv * hv * ibar);
            }
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                const double ref = c.floating ? (last[j] - avg[j]) : (avg[j] - K);
                v[j] = disc * dmax(phid * ref, 0.0);
            }
            avg0 = avg[0];
        } else if constexpr (KIND == kBarrier) {
            const bool b[5] = {br, br_su, br_sd, br_vu, br_vd};
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                const double vanilla = dmax(phid * (last[j] - K), 0.0);
                const bool pays = c.out ? !b[j] : b[j];
                v[j] = disc * (pays ? vanilla : c.rebate);
            }
        } else {
            const double hi[5] = {S0 * exp(static_cast<double>(xmax)), (S0 + hs) * exp(static_cast<double>(xmax)),
                                  (S0 - hs) * exp(static_cast<double>(xmax)), S0 * exp(static_cast<double>(xmax_up)),
                                  S0 * exp(static_cast<double>(xmax_dn))};
            const double lo[5] = {S0 * exp(static_cast<double>(xmin)), (S0 + hs) * exp(static_cast<double>(xmin)),
                                  (S0 - hs) * exp(static_cast<double>(xmin)), S0 * exp(static_cast<double>(xmin_up)),
                                  S0 * exp(static_cast<double>(xmin_dn))};
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                if constexpr (KIND == kLookbackFixed)
                    v[j] = disc * (c.type == 0 ? dmax(hi[j] - K, 0.0) : dmax(K - lo[j], 0.0));
                else
                    v[j] = disc * (c.type == 0 ? (last[j] - lo[j]) : (hi[j] - last[j]));
            }
        }
        const double h = v[0];
        const double z1d = static_cast<double>(z1);
        o[kGLrDelta] = h * (z1d * g.lr_delta_scale);
        o[kGLrGamma] = h * ((z1d * z1d - g.vol * g.sqrt_dt * z1d - 1.0) * g.lr_gamma_scale);
        o[kGLrVega] = h * static_cast<double>(lr_vega);
        o[kGLrRho] = h * (g.sqrt_dt_over_vol * static_cast<double>(zsum) - g.time);
        if constexpr (KIND == kAsianArith || KIND == kAsianGeo) {
            const bool arith = KIND == kAsianArith;
            const double d_avg_dspot = avg0 * g.inv_spot;
            const double d_avg_dvol =
                arith ? S0 * static_cast<double>(a_d) * g.inv_n : avg0 * (static_cast<double>(sd) * g.inv_n);
            const double d_avg_drate =
                arith ? S0 * static_cast<double>(a_r) * g.dt * g.inv_n : avg0 * (0.5 * (n + 1.0) * g.dt);
            const double ref = c.floating ? (last0 - avg0) : (avg0 - K);
            const double slope = phid * ref > 0.0 ? phid : 0.0;
            double delta_raw, vega_raw, rate_raw;
            if (!c.floating) {
                delta_raw = slope * d_avg_dspot;
                vega_raw = slope * d_avg_dvol;
                rate_raw = slope * d_avg_drate;
            } else {
                delta_raw = slope * (le - d_avg_dspot);
                vega_raw = slope * (last0 * static_cast<double>(D) - d_avg_dvol);
                rate_raw = slope * (last0 * n * g.dt - d_avg_drate);
            }
            o[kGPwDelta] = disc * delta_raw;
            o[kGPwVega] = disc * vega_raw;
            o[kGPwRho] = disc * rate_raw - g.time * h;
        }
    }
    o[kGFdDelta] = (v[1] - v[2]) * g.inv_2hs;
    o[kGFdGamma] = (v[1] - 2.0 * v[0] + v[2]) * g.inv_hs2;
    o[kGFdVega] = (v[3] - v[4]) * g.inv_2hv;
}

// One slab: per-thread accumulation in path order (FP64: Welford per sample;
// FP32: count and FP64 sums), as the path engine.  The twelve accumulator
// pairs live in shared memory (acc[0][i][t], acc[1][i][t]) rather than
// registers: they are touched once per path, and the registers go to the
// path state instead.
template <int PREC, int KIND, bool SER = false>
__device__ void slab_greeks(const DevContract& c, const DevGreeks& g, const PhiloxKeys& k, uint64_t base,
                            double (*acc)[kNumGreeks][kSlabThreads], Welford (&w)[kNumGreeks]) {
    const int t = threadIdx.x;
    double o[kNumGreeks];
#pragma unroll
    for (int i = 0; i < kNumGreeks; ++i) acc[0][i][t] = acc[1][i][t] = 0.0;
    unsigned count = 0;
    for (int j = 0; j < kPathsPerThread; ++j) {
        const uint64_t path = base + static_cast<uint64_t>(j * kSlabThreads) + t;
        if (path >= c.path_count) break;
        ++count;
        if constexpr (PREC == 0) {
            greeks64<KIND>(c, g, k, path, o);
            const double inv = 1.0 / static_cast<double>(count);  // welford_add, one count for all outputs
#pragma unroll
            for (int i = 0; i < kNumGreeks; ++i) {
                const double mean = acc[0][i][t];
                const double delta = o[i] - mean;
                const double m = mean + delta * inv;
                acc[0][i][t] = m;
                acc[1][i][t] += delta * (o[i] - m);
            }
        } else {
            greeks32<KIND, SER>(c, g, k, path, o);
#pragma unroll
            for (int i = 0; i < kNumGreeks; ++i) {
                acc[0][i][t] += o[i];
                acc[1][i][t] = fma(o[i], o[i], acc[1][i][t]);
            }
        }
    }
#pragma unroll
    for (int i = 0; i < kNumGreeks; ++i) {
        if constexpr (PREC == 0)
            w[i] = Welford{count, count ? acc[0][i][t] : 0.0, count ? acc[1][i][t] : 0.0};
        else
            w[i] = welford_from_sums(count, acc[0][i][t], acc[1][i][t]);
    }
}

template <int PREC>
__device__ void run_greeks_slab(const DevContract& c, const DevGreeks& g, uint64_t base,
                                double (*acc)[kNumGreeks][kSlabThreads], Welford (&w)[kNumGreeks]) {
    const PhiloxKeys k = philox_keys(c.seed);
    switch (c.kind) {
        case kEuropean: slab_greeks<PREC, kEuropean>(c, g, k, base, acc, w); break;
        case kDigital: slab_greeks<PREC, kDigital>(c, g, k, base, acc, w); break;
        case kAsianArith:
            if (g.vol_series) slab_greeks<PREC, kAsianArith, true>(c, g, k, base, acc, w);
            else slab_greeks<PREC, kAsianArith, false>(c, g, k, base, acc, w);
            break;
        case kAsianGeo: slab_greeks<PREC, kAsianGeo>(c, g, k, base, acc, w); break;
        case kBarrier: slab_greeks<PREC, kBarrier>(c, g, k, base, acc, w); break;
        case kLookbackFixed: slab_greeks<PREC, kLookbackFixed>(c, g, k, base, acc, w); break;
        default: slab_greeks<PREC, kLookbackFloating>(c, g, k, base, acc, w); break;
    }
}

template <int PREC, int MINB>
__global__ void __launch_bounds__(kSlabThreads, MINB)
    greeks_kernel(const DevContract* __restrict__ contracts, const DevGreeks* __restrict__ greeks, int n_contracts,
                  const uint32_t* __restrict__ item_prefix, uint32_t total_items, uint32_t* __restrict__ ticket,
                  Welford* __restrict__ partials, uint32_t* __restrict__ error_flag) {
    __shared__ uint32_t s_item;
    __shared__ Welford s_warp[kSlabThreads / 32][kNumGreeks];
    __shared__ DevContract s_contract;
    __shared__ DevGreeks s_greeks;
    __shared__ double s_acc[2][kNumGreeks][kSlabThreads];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    static_assert(sizeof(DevContract) % 4 == 0 && sizeof(DevGreeks) % 4 == 0 &&
                      (sizeof(DevContract) + sizeof(DevGreeks)) / 4 <= 2 * kSlabThreads,
                  "contract staging assumes at most two words per thread");
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(ticket, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= total_items) return;
        int lo = 0, hi = n_contracts;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (item_prefix[mid] <= item) lo = mid; else hi = mid;
        }
        for (int i = threadIdx.x; i < static_cast<int>(sizeof(DevContract) / 4); i += kSlabThreads)
            reinterpret_cast<uint32_t*>(&s_contract)[i] = reinterpret_cast<const uint32_t*>(&contracts[lo])[i];
        for (int i = threadIdx.x; i < static_cast<int>(sizeof(DevGreeks) / 4); i += kSlabThreads)
            reinterpret_cast<uint32_t*>(&s_greeks)[i] = reinterpret_cast<const uint32_t*>(&greeks[lo])[i];
        __syncthreads();
        const uint32_t slab = item - item_prefix[lo];
        if (slab >= s_contract.n_slabs) {
            if (threadIdx.x == 0) atomicOr(error_flag, 1u);
            __syncthreads();
            continue;
        }
        Welford w[kNumGreeks];
        run_greeks_slab<PREC>(s_contract, s_greeks, static_cast<uint64_t>(slab) * kSlabPaths, s_acc, w);
#pragma unroll
        for (int i = 0; i < kNumGreeks; ++i) {
            const Welford r = welford_warp_reduce(w[i]);
            if (lane == 0) s_warp[warp][i] = r;
        }
        __syncthreads();
        if (threadIdx.x < kNumGreeks) {
            const int i = threadIdx.x;
            partials[static_cast<size_t>(item) * kNumGreeks + i] =
                welford_merge(welford_merge(s_warp[0][i], s_warp[1][i]), welford_merge(s_warp[2][i], s_warp[3][i]));
        }
        __syncthreads();
    }
}

// One warp per (contract, output): the path engine's merge.
__global__ void greeks_merge_kernel(const DevContract* __restrict__ contracts, int n_contracts,
                                    const uint32_t* __restrict__ item_prefix, const Welford* __restrict__ partials,
                                    double* __restrict__ out) {
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp_global >= n_contracts * kNumGreeks) return;
    const int ci = warp_global / kNumGreeks, gi = warp_global % kNumGreeks;
    const uint32_t begin = item_prefix[ci];
    const uint32_t count = contracts[ci].n_slabs;
    Welford w{0ull, 0.0, 0.0};
    for (uint32_t s = lane; s < count; s += 32)
        w = welford_merge(w, partials[(static_cast<size_t>(begin) + s) * kNumGreeks + gi]);
    w = welford_warp_reduce(w);
    if (lane == 0) {
        double* o = out + static_cast<size_t>(contracts[ci].orig_index) * kGreeksOutStride;
        const double var = w.count < 2 ? 0.0 : w.m2 / static_cast<double>(w.count - 1);
        o[2 * gi] = w.mean;
        o[2 * gi + 1] = w.count == 0 ? 0.0 : sqrt(var / static_cast<double>(w.count));
        if (gi == 0) o[2 * kNumGreeks] = static_cast<double>(w.count);
    }
}

template <int PREC, int MINB>
cudaError_t launch_one(int grid, const DevContract* c, const DevGreeks* g, int n, const uint32_t* prefix,
                       uint32_t total, uint32_t* ticket, Welford* partials, uint32_t* err, cudaStream_t stream) {
    cudaGetLastError();
    greeks_kernel<PREC, MINB><<<grid, kSlabThreads, 0, stream>>>(c, g, n, prefix, total, ticket, partials, err);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_greeks_kernel(int precision, int variant, int grid, const DevContract* contracts,
                                 const DevGreeks* greeks, int n_contracts, const uint32_t* item_prefix,
                                 uint32_t total_items, uint32_t* ticket, Welford* partials,
                                 uint32_t* error_flag, cudaStream_t stream) {
#define MCD_GREEKS_ARGS grid, contracts, greeks, n_contracts, item_prefix, total_items, ticket, partials, error_flag, stream
    if (precision == 0) {
        switch (variant) {
            case 0: return launch_one<0, 2>(MCD_GREEKS_ARGS);
            case 1: return launch_one<0, 4>(MCD_GREEKS_ARGS);
            case 2: return launch_one<0, 6>(MCD_GREEKS_ARGS);
            default: return launch_one<0, 8>(MCD_GREEKS_ARGS);
        }
    }
    switch (variant) {
        case 0: return launch_one<1, 2>(MCD_GREEKS_ARGS);
        case 1: return launch_one<1, 4>(MCD_GREEKS_ARGS);
        case 2: return launch_one<1, 6>(MCD_GREEKS_ARGS);
        default: return launch_one<1, 8>(MCD_GREEKS_ARGS);
    }
#undef MCD_GREEKS_ARGS
}

cudaError_t launch_greeks_merge(const DevContract* contracts, int n_contracts, const uint32_t* item_prefix,
                                const Welford* partials, double* out, cudaStream_t stream) {
    cudaGetLastError();
    const long long warps = static_cast<long long>(n_contracts) * kNumGreeks;
    const int threads = 256;
    const long long blocks = (warps * 32 + threads - 1) / threads;
    if (blocks > 0)
        greeks_merge_kernel<<<static_cast<unsigned>(blocks), threads, 0, stream>>>(contracts, n_contracts, item_prefix,
                                                                                  partials, out);
    return cudaGetLastError();
}

cudaError_t greeks_kernel_occupancy(int precision, int variant, int* blocks) {
    if (precision == 0) {
        switch (variant) {
            case 0: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, greeks_kernel<0, 2>, kSlabThreads, 0);
            case 1: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, greeks_kernel<0, 4>, kSlabThreads, 0);
            case 2: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, greeks_kernel<0, 6>, kSlabThreads, 0);
            default: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, greeks_kernel<0, 8>, kSlabThreads, 0);
        }
    }
    switch (variant) {
        case 0: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, greeks_kernel<1, 2>, kSlabThreads, 0);
        case 1: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, greeks_kernel<1, 4>, kSlabThreads, 0);
        case 2: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, greeks_kernel<1, 6>, kSlabThreads, 0);
        default: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, greeks_kernel<1, 8>, kSlabThreads, 0);
    }
}

}  // namespace mcdg
