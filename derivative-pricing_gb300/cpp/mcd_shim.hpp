// mcd_shim.hpp -- the reference's C++ pricing API (namespace mcd::pricers /
// mcd::greeks, include/mcd/{core/types,models/heston,pricers/*,greeks/*}.hpp)
// re-declared over the GPU engine's C ABI (include/mcd_gpu.h).
//
// Same names, argument order, enums and result structs, so code written
// against the reference (its JSON CLI apps/mcd_cli/main.cpp, its Python
// bindings) compiles against this header and links libmcd_shim.so instead of
// libmcd_core.a.  Two differences, both forced by a device underneath:
//   * functions are not noexcept: a failed GPU call throws mcd::gpu::Error
//     (the reference has no error channel and "trusts the caller");
//   * the arithmetic precision is a per-thread setting (mcd::gpu::set_precision,
//     default FP64 = the reference's arithmetic on the GPU).
// Every call of a thread goes to one mcd_ctx created on first use (device
// from MCD_GPU_DEVICE, default 0).
#pragma once

#include <cstdint>
#include <optional>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

namespace mcd {

// include/mcd/core/types.hpp:12-17
enum class OptionType : std::uint8_t { Call, Put };
enum class BarrierDirection : std::uint8_t { Up, Down };
enum class BarrierKnock : std::uint8_t { In, Out };
enum class StrikeStyle : std::uint8_t { Fixed, Floating };
enum class DigitalStyle : std::uint8_t { CashOrNothing, AssetOrNothing };
enum class AverageStyle : std::uint8_t { Arithmetic, Geometric };

[[nodiscard]] std::string_view version() noexcept;

// include/mcd/core/sobol.hpp:14 (this engine: 256 dimensions)
constexpr unsigned kSobolMaxDimensions = 256;

// include/mcd/core/rng_simd.hpp:14-18: whether the reference's NEON batch
// draw path is compiled in.  The draws here come from the GPU on any host, so
// the flag is false (the Python module's HAS_NEON and the JSON CLI's
// simd_enabled say the same).
inline constexpr bool kHasNeon = false;

namespace gpu {

enum class Precision : int { FP64 = 0, FP32 = 1 };

struct Error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

void set_precision(Precision p);
[[nodiscard]] Precision precision();

}  // namespace gpu

namespace models {
// include/mcd/models/heston.hpp:8-18
struct HestonParams {
    double spot;
    double rate;
    double carry_yield;
    double v0;
    double kappa;
    double theta;
    double xi;
    double rho;
    double time;
};
}  // namespace models

namespace pricers {

// include/mcd/pricers/monte_carlo.hpp:9-33
struct McResult {
    double price;
    double standard_error;
    std::uint64_t path_count;
};

struct McOptions {
    bool antithetic = false;
    bool control_variate = false;
    bool brownian_bridge = false;
    unsigned num_threads = 1;
};

McResult monte_carlo_european(double spot, double strike, double rate, double carry_yield, double vol, double time,
                              OptionType type, std::uint64_t path_count, std::uint64_t seed);
McResult monte_carlo_european(double spot, double strike, double rate, double carry_yield, double vol, double time,
                              OptionType type, std::uint64_t path_count, std::uint64_t seed, McOptions options);
McResult monte_carlo_digital(double spot, double strike, double rate, double carry_yield, double vol, double time,
                             OptionType type, DigitalStyle style, double cash_amount, std::uint64_t path_count,
                             std::uint64_t seed, McOptions options = {});
McResult monte_carlo_asian(double spot, double strike, double rate, double carry_yield, double vol, double time,
                           OptionType type, StrikeStyle strike_style, AverageStyle average_style,
                           int monitoring_points, std::uint64_t path_count, std::uint64_t seed,
                           McOptions options = {});
McResult monte_carlo_barrier(double spot, double strike, double barrier, double rate, double carry_yield, double vol,
                             double time, OptionType type, BarrierDirection direction, BarrierKnock knock,
                             double rebate, int monitoring_points, std::uint64_t path_count, std::uint64_t seed,
                             McOptions options = {});
McResult monte_carlo_lookback(double spot, double strike, double rate, double carry_yield, double vol, double time,
                              OptionType type, StrikeStyle style, int monitoring_points, std::uint64_t path_count,
                              std::uint64_t seed, McOptions options = {});

// include/mcd/pricers/qmc.hpp
struct QmcResult {
    double price = 0.0;
};
QmcResult qmc_sobol_european(double spot, double strike, double rate, double carry_yield, double vol, double time,
                             OptionType type, std::uint64_t path_count);
QmcResult qmc_sobol_asian(double spot, double strike, double rate, double carry_yield, double vol, double time,
                          OptionType type, StrikeStyle strike_style, int monitoring_points,
                          std::uint64_t path_count);

// include/mcd/pricers/lsm.hpp
struct LsmPolicy {
    std::vector<std::vector<double>> coefficients_by_date;
    bool exercise_at_inception = false;
};
struct LsmResult {
    double price = 0.0;
    double standard_error = 0.0;
    LsmPolicy policy;
};
LsmResult monte_carlo_lsm_american(double spot, double strike, double rate, double carry_yield, double vol,
                                   double time, OptionType type, int monitoring_points, std::uint64_t path_count,
                                   std::uint64_t seed);
double reprice_against_frozen_policy(double spot, double strike, double rate, double carry_yield, double vol,
                                     double time, OptionType type, int monitoring_points, std::uint64_t path_count,
                                     std::uint64_t seed, const LsmPolicy& policy);

// include/mcd/pricers/heston.hpp
struct HestonMcResult {
    double price = 0.0;
    double standard_error = 0.0;
    std::uint64_t path_count = 0;
};
HestonMcResult heston_qe_european(const models::HestonParams& params, double strike, OptionType type,
                                  int monitoring_points, std::uint64_t path_count, std::uint64_t seed);
double heston_semi_analytic(const models::HestonParams& params, double strike, OptionType type);

// include/mcd/pricers/analytic.hpp, binomial.hpp: closed forms and trees
// (host code, no GPU)
double black_scholes_merton(double spot, double strike, double rate, double carry_yield, double vol, double time,
                            OptionType type);
double black76(double forward, double strike, double rate, double vol, double time, OptionType type);
double kemna_vorst(double spot, double strike, double rate, double carry_yield, double vol, double time,
                   OptionType type);
double reiner_rubinstein(double spot, double strike, double barrier, double rate, double carry_yield, double vol,
                         double time, OptionType type, BarrierDirection direction, BarrierKnock knock,
                         double rebate = 0.0);
double lookback_fixed_strike(double spot, double strike, double rate, double carry_yield, double vol, double time,
                             OptionType type);
double lookback_floating_strike(double spot, double rate, double carry_yield, double vol, double time,
                                OptionType type);
double digital(double spot, double strike, double rate, double carry_yield, double vol, double time,
               OptionType type, DigitalStyle style, double cash_amount = 1.0);
double forward_price(double spot, double rate, double carry_yield, double time);
double forward_value(double forward_now, double forward_at_inception, double rate, double time_to_expiry);
double futures_mark_to_market(double futures_price_new, double futures_price_old);
struct BinomialResult {
    double price;
    double risk_neutral_probability;
    double up_factor;
    double down_factor;
};
BinomialResult crr_binomial(double spot, double strike, double rate, double carry_yield, double vol, double time,
                            int steps, OptionType type);
double crr_binomial_american(double spot, double strike, double rate, double carry_yield, double vol, double time,
                             int steps, OptionType type);

}  // namespace pricers

namespace greeks {

// include/mcd/greeks/finite_difference.hpp
struct EuropeanGreeks {
    double delta;
    double gamma;
    double vega;
    double theta;
    double rho;
};
struct BumpSizes {
    double spot;
    double vol;
    double rate;
    double time;
};
BumpSizes default_bump_sizes(double spot, double vol, double time) noexcept;
EuropeanGreeks finite_difference_european(double spot, double strike, double rate, double carry_yield, double vol,
                                          double time, OptionType type, std::uint64_t path_count, std::uint64_t seed,
                                          BumpSizes bumps);

// include/mcd/greeks/likelihood_ratio.hpp
struct LrGreeksResult {
    double value = 0.0;
    double standard_error = 0.0;
};
struct LrGreeks {
    LrGreeksResult delta, gamma, vega, rho;
    std::optional<LrGreeksResult> theta;
};
LrGreeks likelihood_ratio_european(double spot, double strike, double rate, double carry_yield, double vol,
                                   double time, OptionType type, std::uint64_t path_count, std::uint64_t seed);
LrGreeks likelihood_ratio_digital(double spot, double strike, double rate, double carry_yield, double vol,
                                  double time, OptionType type, DigitalStyle style, double cash_amount,
                                  std::uint64_t path_count, std::uint64_t seed);
LrGreeks likelihood_ratio_barrier(double spot, double strike, double barrier, double rate, double carry_yield,
                                  double vol, double time, OptionType type, BarrierDirection direction,
                                  BarrierKnock knock, double rebate, int monitoring_points, std::uint64_t path_count,
                                  std::uint64_t seed);

// include/mcd/greeks/pathwise.hpp
struct PathwiseGreeksResult {
    double value = 0.0;
    double standard_error = 0.0;
};
struct PathwiseGreeks {
    PathwiseGreeksResult delta, vega, rho;
};
PathwiseGreeks pathwise_european(double spot, double strike, double rate, double carry_yield, double vol,
                                 double time, OptionType type, std::uint64_t path_count, std::uint64_t seed);
PathwiseGreeks pathwise_asian(double spot, double strike, double rate, double carry_yield, double vol, double time,
                              OptionType type, StrikeStyle strike_style, AverageStyle average_style,
                              int monitoring_points, std::uint64_t path_count, std::uint64_t seed);

}  // namespace greeks

}  // namespace mcd

// ---- the JSON request handler (request.cpp), C linkage -------------------
// One JSON request object in, one JSON object out (the result, or
// {"error": message}); the returned string is released with mcd_shim_free.
// dialect: MCD_SHIM_DIALECT_CLI (the reference CLI's messages) or
// MCD_SHIM_DIALECT_LAMBDA (the reference Lambda layer's messages, its
// variance-reduction toggles and max_path_count, 0 = no cap).
// status: MCD_SHIM_OK, MCD_SHIM_REQUEST_ERROR (bad request) or
// MCD_SHIM_INTERNAL_ERROR (the device failed).
extern "C" {
enum { MCD_SHIM_DIALECT_CLI = 0, MCD_SHIM_DIALECT_LAMBDA = 1 };
enum { MCD_SHIM_OK = 0, MCD_SHIM_REQUEST_ERROR = 1, MCD_SHIM_INTERNAL_ERROR = 2 };
char* mcd_shim_handle_request(const char* request, int dialect, uint64_t max_path_count, int* status);
void mcd_shim_free(char* response);
}
