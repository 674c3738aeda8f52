/*
 * mcd_oracle.h -- CPU oracle for the mcd Monte Carlo hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * library's CPU algorithms (FredTheMay/derivative-pricing, "mcd"), used as the
 * checker for the CUDA implementation and as the timed CPU baseline.  Only the
 * tests, the smoke check and the benchmark's CPU-baseline leg may load it; the
 * product library never links or calls it.
 *
 * Parity status: pinned.  Every function cites the reference file:line it
 * restates; the restatement is checked bit-for-bit against the reference
 * compiled from its own sources (oracle/Makefile, target `ref`) and against the
 * known-answer vectors the reference's own tests carry (Philox KATs,
 * tests/rng_test.cpp:17-39; Lewis Heston prices, tests/heston_test.cpp:45-51).
 *
 * Enum values follow include/mcd/core/types.hpp:12-17 (underlying uint8_t):
 *   OptionType {Call=0, Put=1}, BarrierDirection {Up=0, Down=1},
 *   BarrierKnock {In=0, Out=1}, StrikeStyle {Fixed=0, Floating=1},
 *   DigitalStyle {CashOrNothing=0, AssetOrNothing=1},
 *   AverageStyle {Arithmetic=0, Geometric=1}.
 */
#ifndef MCD_ORACLE_H
#define MCD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double price;
    double standard_error;
    uint64_t path_count;
} orc_mc_result;

typedef struct {
    uint64_t count;
    double mean;
    double m2;
} orc_welford;

/* McOptions (include/mcd/pricers/monte_carlo.hpp:18-33) plus the logical chunk
 * count, which the reference fixes to std::thread::hardware_concurrency()
 * (src/core/thread_pool.cpp:41-44); chunk_count == 0 means "use nproc". */
typedef struct {
    int antithetic;
    int control_variate;
    int brownian_bridge;
    unsigned num_threads;
    unsigned chunk_count;
} orc_options;

/* ---- L1 numerics core -------------------------------------------------- */
void orc_philox4x32_10(const uint32_t counter[4], const uint32_t key[2], uint32_t out[4]);
double orc_uniform_open01(uint32_t bits);
double orc_normal_pdf(double x);
double orc_normal_cdf(double x);
double orc_inv_normal_cdf(double u);
double orc_normal_variate(uint64_t seed, uint64_t path, uint32_t draw);
double orc_uniform_variate(uint64_t seed, uint64_t path, uint32_t draw);

void orc_welford_add(orc_welford* w, double value);
void orc_welford_merge(orc_welford* w, const orc_welford* other);
double orc_welford_variance(const orc_welford* w);
double orc_welford_se(const orc_welford* w);
void orc_chunk_bounds(unsigned chunk, uint64_t total, unsigned chunk_count, uint64_t* begin,
                      uint64_t* end);
unsigned orc_default_chunk_count(void);

/* Sobol: dimensions 0..6 restate src/core/sobol.cpp; dimensions 7.. extend the
 * table with further primitive polynomials (see orc_sobol_polynomial). */
#define ORC_SOBOL_MAX_DIMS 256
int orc_sobol_polynomial(unsigned dimension, unsigned* degree, uint32_t* interior);
void orc_sobol_directions(unsigned dimension, uint32_t v[33]);
uint32_t orc_sobol_bits(unsigned dimension, uint64_t index);
double orc_sobol_point(unsigned dimension, uint64_t index);

/* Brownian-bridge GBM path (src/models/brownian_bridge_path.cpp:20-77). */
void orc_brownian_bridge_gbm_path(double spot, double rate, double carry_yield, double vol,
                                  double time, int n, const double* normals, double* spots);

/* ---- Monte Carlo pricers (src/pricers/monte_carlo.cpp:233-338) --------- */
orc_mc_result orc_mc_european(double spot, double strike, double rate, double carry_yield,
                              double vol, double time, int type, uint64_t path_count,
                              uint64_t seed, const orc_options* options);
orc_mc_result orc_mc_digital(double spot, double strike, double rate, double carry_yield,
                             double vol, double time, int type, int digital_style,
                             double cash_amount, uint64_t path_count, uint64_t seed,
                             const orc_options* options);
orc_mc_result orc_mc_asian(double spot, double strike, double rate, double carry_yield,
                           double vol, double time, int type, int strike_style,
                           int average_style, int monitoring_points, uint64_t path_count,
                           uint64_t seed, const orc_options* options);
orc_mc_result orc_mc_barrier(double spot, double strike, double barrier, double rate,
                             double carry_yield, double vol, double time, int type,
                             int direction, int knock, double rebate, int monitoring_points,
                             uint64_t path_count, uint64_t seed, const orc_options* options);
orc_mc_result orc_mc_lookback(double spot, double strike, double rate, double carry_yield,
                              double vol, double time, int type, int strike_style,
                              int monitoring_points, uint64_t path_count, uint64_t seed,
                              const orc_options* options);

/* ---- Longstaff-Schwartz (src/pricers/lsm.cpp) -------------------------- */
/* coefficients: (monitoring_points+1) x 4, row k valid iff has_coeffs[k]. */
orc_mc_result orc_lsm_american(double spot, double strike, double rate, double carry_yield,
                               double vol, double time, int type, int monitoring_points,
                               uint64_t path_count, uint64_t seed, double* coefficients,
                               uint8_t* has_coeffs, int* exercise_at_inception);
double orc_lsm_reprice_frozen(double spot, double strike, double rate, double carry_yield,
                              double vol, double time, int type, int monitoring_points,
                              uint64_t path_count, uint64_t seed, const double* coefficients,
                              const uint8_t* has_coeffs, int exercise_at_inception);
/* Householder least squares on a row-major rows x cols matrix (modified). */
void orc_householder_least_squares(double* a, int rows, int cols, double* y, double* beta);
void orc_laguerre_basis(double x, double out[4]);

/* ---- Heston (src/pricers/heston.cpp) ------------------------------------ */
typedef struct {
    double spot, rate, carry_yield, v0, kappa, theta, xi, rho, time;
} orc_heston_params;
orc_mc_result orc_heston_qe_european(const orc_heston_params* p, double strike, int type,
                                     int monitoring_points, uint64_t path_count, uint64_t seed);
double orc_heston_semi_analytic(const orc_heston_params* p, double strike, int type);

/* ---- Sobol QMC (src/pricers/qmc.cpp) ------------------------------------ */
double orc_qmc_sobol_european(double spot, double strike, double rate, double carry_yield,
                              double vol, double time, int type, uint64_t path_count);
double orc_qmc_sobol_asian(double spot, double strike, double rate, double carry_yield,
                           double vol, double time, int type, int strike_style,
                           int monitoring_points, uint64_t path_count);

/* ---- Greeks (src/greeks/*.cpp) ------------------------------------------ */
typedef struct { double delta, gamma, vega, theta, rho; } orc_european_greeks;
typedef struct { double spot, vol, rate, time; } orc_bumps;
typedef struct { double value, standard_error; } orc_greek;
typedef struct { orc_greek delta, gamma, vega, rho, theta; int has_theta; } orc_lr_greeks;
typedef struct { orc_greek delta, vega, rho; } orc_pathwise_greeks;

orc_bumps orc_default_bump_sizes(double spot, double vol, double time);
orc_european_greeks orc_fd_european(double spot, double strike, double rate, double carry_yield,
                                    double vol, double time, int type, uint64_t path_count,
                                    uint64_t seed, orc_bumps bumps, unsigned chunk_count);
orc_lr_greeks orc_lr_european(double spot, double strike, double rate, double carry_yield,
                              double vol, double time, int type, uint64_t path_count,
                              uint64_t seed);
orc_lr_greeks orc_lr_digital(double spot, double strike, double rate, double carry_yield,
                             double vol, double time, int type, int digital_style,
                             double cash_amount, uint64_t path_count, uint64_t seed);
orc_lr_greeks orc_lr_barrier(double spot, double strike, double barrier, double rate,
                             double carry_yield, double vol, double time, int type,
                             int direction, int knock, double rebate, int monitoring_points,
                             uint64_t path_count, uint64_t seed);
orc_pathwise_greeks orc_pathwise_european(double spot, double strike, double rate,
                                          double carry_yield, double vol, double time, int type,
                                          uint64_t path_count, uint64_t seed);
orc_pathwise_greeks orc_pathwise_asian(double spot, double strike, double rate,
                                       double carry_yield, double vol, double time, int type,
                                       int strike_style, int average_style,
                                       int monitoring_points, uint64_t path_count,
                                       uint64_t seed);

/* ---- Analytic / tree oracles (src/pricers/analytic.cpp, binomial.cpp) --- */
double orc_bsm(double spot, double strike, double rate, double carry_yield, double vol,
               double time, int type);
double orc_kemna_vorst(double spot, double strike, double rate, double carry_yield, double vol,
                       double time, int type);
double orc_reiner_rubinstein(double spot, double strike, double barrier, double rate,
                             double carry_yield, double vol, double time, int type,
                             int direction, int knock, double rebate);
double orc_lookback_fixed(double spot, double strike, double rate, double carry_yield,
                          double vol, double time, int type);
double orc_lookback_floating(double spot, double rate, double carry_yield, double vol,
                             double time, int type);
double orc_digital_analytic(double spot, double strike, double rate, double carry_yield,
                            double vol, double time, int type, int style, double cash_amount);
double orc_crr_binomial_american(double spot, double strike, double rate, double carry_yield,
                                 double vol, double time, int steps, int type);

/* ---- Batch helpers for the CPU baseline --------------------------------- */
/* Flat contract record shared with the CUDA library's mcd_contract layout
 * (include/mcd_gpu.h); product codes: 0 european, 1 digital, 2 asian,
 * 3 barrier, 4 lookback. */
typedef struct {
    int32_t product, type, direction, knock, strike_style, average_style, digital_style,
        monitoring_points;
    double spot, strike, barrier, rebate, rate, carry_yield, vol, time, cash_amount;
    uint64_t path_count, seed;
    uint8_t antithetic, control_variate, brownian_bridge, reserved0;
    uint32_t reserved1;
} orc_contract;

/* Prices contracts one after another, each on `num_threads` threads over the
 * reference's fixed chunk partition (the reference's own multithreaded path). */
void orc_price_batch(const orc_contract* contracts, int n, unsigned num_threads,
                     unsigned chunk_count, orc_mc_result* out);

/* Runs single-threaded reference pricers as independent items over threads
 * (contract-level parallelism); kind 0 = Heston QE (items = param sets x
 * strikes), kind 1 = LSM American. */
void orc_heston_batch(const orc_heston_params* sets, int n_sets, const double* strikes,
                      int n_strikes, int type, int monitoring_points, uint64_t path_count,
                      uint64_t seed, unsigned num_threads, orc_mc_result* out);
void orc_lsm_batch(const double* params /* n x 7: spot strike rate q vol time type */, int n,
                   int monitoring_points, uint64_t path_count, uint64_t seed,
                   unsigned num_threads, orc_mc_result* out);

#ifdef __cplusplus
}
#endif

#endif /* MCD_ORACLE_H */
