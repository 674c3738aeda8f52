/*
 * mcd_gpu.h -- C ABI of the GB300 (sm_103a) Monte Carlo engine for mcd.
 *
 * One shared library (libmcd_gpu.so) with plain C types: no C++ or torch types
 * cross this boundary.  Every entry point returns an mcd_status (0 = success,
 * negative = error); mcd_last_error() gives the message.  The caller owns every
 * host array passed in or out; an mcd_ctx owns its device memory, stream and
 * captured CUDA graphs.  Use one context per host thread (calls on a context
 * are stream-ordered and not thread-safe).
 *
 * Each pricing entry point replaces one reference function (cited per
 * declaration; paths are within FredTheMay/derivative-pricing).  The reference
 * functions are noexcept and "trust the caller"; this ABI validates arguments
 * instead and reports MCD_ERR_INVALID_ARGUMENT.
 *
 * Precision (mcd_precision):
 *   MCD_PRECISION_FP64  the reference's arithmetic in FP64 on the GPU (Acklam
 *                       inverse CDF with its Halley step, multiplicative GBM
 *                       steps); identical draws; prices agree with the CPU
 *                       reference to ~1e-12 relative.
 *   MCD_PRECISION_FP32  the same Philox draws (same counters, word 0) turned
 *                       into FP32 normals; paths evolve in FP32 (log space);
 *                       payoffs are accumulated and merged in FP64.
 *
 * Results are bitwise identical for a given precision regardless of launch
 * configuration (grid size, kernel variant): paths are grouped into fixed
 * slabs of MCD_SLAB_PATHS and every reduction tree is fixed by slab index.
 */
#ifndef MCD_GPU_H
#define MCD_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCD_GPU_ABI_VERSION 1
#define MCD_SLAB_PATHS 4096

typedef struct mcd_ctx mcd_ctx;

typedef enum {
    MCD_OK = 0,
    MCD_ERR_INVALID_ARGUMENT = -1,
    MCD_ERR_CUDA = -2,
    MCD_ERR_OUT_OF_MEMORY = -3,
    MCD_ERR_TIMEOUT = -4,
    MCD_ERR_UNSUPPORTED = -5,
    MCD_ERR_NO_DEVICE = -6
} mcd_status;

typedef enum { MCD_PRECISION_FP64 = 0, MCD_PRECISION_FP32 = 1 } mcd_precision;

/* Same values as mcd's enums (include/mcd/core/types.hpp:12-17). */
typedef enum { MCD_CALL = 0, MCD_PUT = 1 } mcd_option_type;
typedef enum { MCD_UP = 0, MCD_DOWN = 1 } mcd_barrier_direction;
typedef enum { MCD_IN = 0, MCD_OUT = 1 } mcd_barrier_knock;
typedef enum { MCD_FIXED = 0, MCD_FLOATING = 1 } mcd_strike_style;
typedef enum { MCD_CASH_OR_NOTHING = 0, MCD_ASSET_OR_NOTHING = 1 } mcd_digital_style;
typedef enum { MCD_ARITHMETIC = 0, MCD_GEOMETRIC = 1 } mcd_average_style;

typedef enum {
    MCD_PRODUCT_EUROPEAN = 0,
    MCD_PRODUCT_DIGITAL = 1,
    MCD_PRODUCT_ASIAN = 2,
    MCD_PRODUCT_BARRIER = 3,
    MCD_PRODUCT_LOOKBACK = 4
} mcd_product;

/* mcd::pricers::McResult (include/mcd/pricers/monte_carlo.hpp:9-13). */
typedef struct {
    double price;
    double standard_error;
    uint64_t path_count;
} mcd_mc_result;

/* mcd::pricers::McOptions (include/mcd/pricers/monte_carlo.hpp:18-33).
 * num_threads is accepted and ignored: the GPU result does not depend on it,
 * just as the reference's does not. */
typedef struct {
    uint8_t antithetic;
    uint8_t control_variate;
    uint8_t brownian_bridge;
    uint8_t reserved;
    uint32_t num_threads;
} mcd_mc_options;

/* One contract of a batch: the argument list of the reference pricer for
 * `product` (monte_carlo.hpp:38-80) flattened into one record.  Fields a
 * product does not use are ignored.  Draws are keyed on (seed, path, step)
 * exactly as in the reference, so a contract priced alone and inside a batch
 * gives the same result. */
typedef struct {
    int32_t product;           /* mcd_product */
    int32_t type;              /* mcd_option_type */
    int32_t direction;         /* barrier: mcd_barrier_direction */
    int32_t knock;             /* barrier: mcd_barrier_knock */
    int32_t strike_style;      /* asian, lookback: mcd_strike_style */
    int32_t average_style;     /* asian: mcd_average_style */
    int32_t digital_style;     /* digital: mcd_digital_style */
    int32_t monitoring_points; /* asian, barrier, lookback (>= 1) */
    double spot, strike, barrier, rebate, rate, carry_yield, vol, time, cash_amount;
    uint64_t path_count;
    uint64_t seed;
    uint8_t antithetic, control_variate, brownian_bridge, reserved0;
    uint32_t reserved1;
} mcd_contract;

/* ---- context ------------------------------------------------------------ */
int mcd_abi_version(void);
/* Creates a context on CUDA device `device` (its own non-blocking stream). */
int mcd_create(int device, mcd_ctx** out);
void mcd_destroy(mcd_ctx* ctx);
/* Message of the last failed call on ctx (or of the last failed mcd_create
 * when ctx is NULL).  Valid until the next call on the same context. */
const char* mcd_last_error(const mcd_ctx* ctx);
/* Blocks until all work queued on the context's stream has finished. */
int mcd_synchronize(mcd_ctx* ctx);

/* ---- single-contract pricers (one GPU launch each) ---------------------- */
/* replaces mcd::pricers::monte_carlo_european (src/pricers/monte_carlo.cpp:233-249) */
int mcd_price_european(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                       double vol, double time, int type, uint64_t path_count, uint64_t seed,
                       const mcd_mc_options* options, int precision, mcd_mc_result* out);
/* replaces mcd::pricers::monte_carlo_digital (src/pricers/monte_carlo.cpp:251-260) */
int mcd_price_digital(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                      double vol, double time, int type, int digital_style, double cash_amount,
                      uint64_t path_count, uint64_t seed, const mcd_mc_options* options,
                      int precision, mcd_mc_result* out);
/* replaces mcd::pricers::monte_carlo_asian (src/pricers/monte_carlo.cpp:262-308) */
int mcd_price_asian(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                    double vol, double time, int type, int strike_style, int average_style,
                    int monitoring_points, uint64_t path_count, uint64_t seed,
                    const mcd_mc_options* options, int precision, mcd_mc_result* out);
/* replaces mcd::pricers::monte_carlo_barrier (src/pricers/monte_carlo.cpp:310-324) */
int mcd_price_barrier(mcd_ctx* ctx, double spot, double strike, double barrier, double rate,
                      double carry_yield, double vol, double time, int type, int direction,
                      int knock, double rebate, int monitoring_points, uint64_t path_count,
                      uint64_t seed, const mcd_mc_options* options, int precision,
                      mcd_mc_result* out);
/* replaces mcd::pricers::monte_carlo_lookback (src/pricers/monte_carlo.cpp:326-338) */
int mcd_price_lookback(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                       double vol, double time, int type, int strike_style, int monitoring_points,
                       uint64_t path_count, uint64_t seed, const mcd_mc_options* options,
                       int precision, mcd_mc_result* out);

/* ---- batched pricing: one persistent-kernel launch in a CUDA graph ------ */
/* Host arrays in and out (copies included).  Equivalent to calling the
 * reference pricer once per contract (monte_carlo.cpp:233-338). */
int mcd_price_batch(mcd_ctx* ctx, const mcd_contract* contracts, size_t n, int precision,
                    mcd_mc_result* results);
/* Device-resident variant: `contracts` and `results` are device pointers; the
 * pricing is queued on `stream` (a cudaStream_t, or NULL for the context's
 * stream) and the call returns without waiting for it.  Each call first
 * computes an 8-byte digest of the contract records on `stream` and waits for
 * it (so everything the caller queued there before, such as an in-place
 * rewrite of the contracts, is seen); the launch plan is rebuilt whenever the
 * pointer, count, precision or digest changes (mcd_batch_invalidate forces
 * it), reading the records on `stream` as well. */
int mcd_price_batch_device(mcd_ctx* ctx, const mcd_contract* contracts, size_t n, int precision,
                           mcd_mc_result* results, void* stream);
int mcd_batch_invalidate(mcd_ctx* ctx);

/* Batched pricing that allocates no memory.  No counterpart in the reference
 * (the reference has no GPU and no device memory).
 *
 * For callers that cannot call cudaMalloc: services that reserve all device
 * memory when they start and must not allocate afterwards, and code where an
 * allocation's implicit device synchronisation is not acceptable.  It needs
 * no mcd_ctx.  It runs the same kernels as mcd_price_batch and returns bitwise
 * the same results; its scratch (contract records, slab partials, device
 * results, ticket and error word) lives in one fixed __device__ array of
 * about 7 MB.  Every GPU that loads the library holds that array until the
 * process exits.  Under CUDA's lazy module loading (the runtime's default)
 * the array is reserved on a device by the first call there, not when the
 * library is loaded: a caller that then reserves the rest of device memory
 * makes that first call (n = 0 will do) before doing so.
 *
 * Limits: at most 4096 contracts and 262144 slabs of MCD_SLAB_PATHS paths
 * (about 1.07e9 paths in total) per call.  Larger requests fail with
 * MCD_ERR_INVALID_ARGUMENT and a message saying which limit was hit.
 * Inputs and outputs are host arrays; `stream` is a cudaStream_t (NULL: the
 * legacy default stream) on the current device.  The call returns when the
 * results are in `results`.  On failure, a message is written to
 * error_message (if error_capacity > 0).
 *
 * The first call on a device does the set-up for that device (a call with
 * n = 0 does only that): it resolves the array's device address with that
 * device current.  Make that first call before any stream capture.  All calls share the one array, and it keeps
 * the last call's contents.  Calls that overlapped on the GPU would race on
 * it; this entry point serialises its calls with a process-wide lock and
 * waits for its GPU work before returning, so its own calls never overlap. */
int mcd_price_batch_static(const mcd_contract* contracts, size_t n, int precision,
                           mcd_mc_result* results, void* stream, char* error_message,
                           size_t error_capacity);

/* Launch shape of the persistent path kernel.  variant 0..4 selects the
 * register budget (__launch_bounds__ min blocks 4/8/12/16/6), ctas_per_sm the
 * grid (SM count x ctas_per_sm).  0 restores the autotuned/default choice.
 * Results do not depend on either. */
int mcd_set_launch_shape(mcd_ctx* ctx, int precision, int variant, int ctas_per_sm);
int mcd_get_launch_shape(mcd_ctx* ctx, int precision, int* variant, int* ctas_per_sm);
/* Autotuner: times every launch shape on `contracts` (host array) and keeps
 * the fastest for `precision`.  Writes the chosen shape and its time. */
int mcd_autotune(mcd_ctx* ctx, const mcd_contract* contracts, size_t n, int precision,
                 int* variant, int* ctas_per_sm, double* best_ms);

/* ---- Heston QE ------------------------------------------------------------ */
/* mcd::models::HestonParams (include/mcd/models/heston.hpp:8-18). */
typedef struct {
    double spot, rate, carry_yield, v0, kappa, theta, xi, rho, time;
} mcd_heston_params;

/* replaces mcd::pricers::heston_qe_european (src/pricers/heston.cpp:120-156):
 * Andersen QE variance step (psi_c = 1.5) and the K0..K4 log-spot update;
 * stream-0 normal for the spot and stream-1 uniform for the variance per
 * (path, step). */
int mcd_heston_qe_european(mcd_ctx* ctx, const mcd_heston_params* params, double strike, int type,
                           int monitoring_points, uint64_t path_count, uint64_t seed,
                           int precision, mcd_mc_result* out);
/* Many parameter sets x many strikes in one launch.  Equivalent to calling
 * heston_qe_european (src/pricers/heston.cpp:120-156) once per (set, strike)
 * with the same seed, path count and steps: each set's paths are simulated
 * once and paid out against every strike.  results: n_sets x n_strikes,
 * row-major.  1 <= n_strikes <= 256. */
int mcd_heston_qe_batch(mcd_ctx* ctx, const mcd_heston_params* sets, size_t n_sets,
                        const double* strikes, size_t n_strikes, int type, int monitoring_points,
                        uint64_t path_count, uint64_t seed, int precision, mcd_mc_result* results);

/* ---- Longstaff-Schwartz American options ---------------------------------- */
typedef enum { MCD_LSM_QR = 0, MCD_LSM_MLP = 1 } mcd_lsm_regression;

/* mcd::pricers::LsmResult (include/mcd/pricers/lsm.hpp:26-30) without the
 * policy vectors (returned separately), plus LsmPolicy::exercise_at_inception. */
typedef struct {
    double price;
    double standard_error;
    uint64_t path_count;
    int32_t exercise_at_inception;
    int32_t reserved;
} mcd_lsm_result;

/* One contract of an LSM batch: monte_carlo_lsm_american's argument list. */
typedef struct {
    double spot, strike, rate, carry_yield, vol, time;
    int32_t type;
    int32_t monitoring_points;
    uint64_t path_count;
    uint64_t seed;
} mcd_lsm_contract;

/* replaces mcd::pricers::monte_carlo_lsm_american (src/pricers/lsm.cpp:62-149):
 * weighted Laguerre basis of degree 3 on S/K, in-the-money regression (skipped
 * below 4 paths), exercise where intrinsic > continuation, inception check.
 * The regression is solved by two FP64 Gram passes (Cholesky-QR2) and a 4x4
 * Householder solve.  coefficients ((monitoring_points+1) x 4) and
 * has_coefficients (monitoring_points+1) receive the policy
 * (LsmPolicy::coefficients_by_date, lsm.hpp:16-24); either may be NULL.
 * regression selects MCD_LSM_QR or the learned MCD_LSM_MLP. */
int mcd_lsm_american(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                     double vol, double time, int type, int monitoring_points,
                     uint64_t path_count, uint64_t seed, int precision, int regression,
                     mcd_lsm_result* out, double* coefficients, uint8_t* has_coefficients);
/* replaces mcd::pricers::reprice_against_frozen_policy (src/pricers/lsm.cpp:151-213). */
int mcd_lsm_reprice_frozen(mcd_ctx* ctx, double spot, double strike, double rate,
                           double carry_yield, double vol, double time, int type,
                           int monitoring_points, uint64_t path_count, uint64_t seed,
                           const double* coefficients, const uint8_t* has_coefficients,
                           int exercise_at_inception, int precision, double* price);
/* Many American contracts (uneven date counts allowed) in one graph launch:
 * all paths stay resident and the contracts step back in lockstep. */
int mcd_lsm_batch(mcd_ctx* ctx, const mcd_lsm_contract* contracts, size_t n, int precision,
                  int regression, mcd_lsm_result* results);

/* Learned regression (MCD_LSM_MLP).  No counterpart in the reference: it
 * replaces the Laguerre least-squares fit of src/pricers/lsm.cpp:88-108 by a
 * 2 -> 64 -> 64 -> 1 GELU network of (4 (S/K - 1), tau/T).  The network is
 * trained on the GPU (Adam on 128-sample tiles of in-the-money paths,
 * BF16 tensor-core forward/backward with FP32 accumulation) at the latest
 * exercise date; its 64 hidden features plus a bias are then the regression
 * basis at every date, whose output layer is fitted by ridge least squares
 * over all in-the-money paths of that date (ridge 1e-3 in unit-diagonal
 * scaling).  At a date the features are functions of ln(S/K) alone, so the
 * network is evaluated on the tensor core at 512 values of ln(S/K) spanning
 * the date's in-the-money paths and each path uses the linear interpolation
 * (Gram matrix exact for the interpolated features, from integer bin
 * moments; the price depends on no launch or batch detail).  Target and
 * decision: the time value (continuation - exercise)/K; exercise where it is
 * predicted negative.  The learned regression takes 1 <= path_count <= 2^31.  A
 * date with fewer than 4 in-the-money paths has no exercise; a contract whose
 * fit produced non-finite weights is priced by the QR regression instead
 * (mcd_lsm_result.reserved = 1).  Schedule: steps_first Adam steps at the
 * latest date (default 100, learning rate lr_first; their samples take 2 KB
 * of device memory per step and contract), steps at each earlier date
 * (default 0: features fixed, learning rate lr). */
int mcd_lsm_set_mlp_config(mcd_ctx* ctx, int steps_first, int steps, double lr_first, double lr);
/* Networks of contract `contract` of the last learned run:
 * weights (monitoring_points+1) x 4417 floats (layout: W1[64][2], b1[64],
 * W2[64][64], b2[64], W3[64], b3), has (monitoring_points+1). */
int mcd_lsm_mlp_policy(mcd_ctx* ctx, size_t contract, float* weights, uint8_t* has);
/* Frozen learned policy replayed on the paths of `seed` (out-of-sample
 * evaluation); counterpart of reprice_against_frozen_policy for networks. */
int mcd_lsm_reprice_mlp(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                        double vol, double time, int type, int monitoring_points, uint64_t path_count,
                        uint64_t seed, const float* weights, const uint8_t* has, int precision,
                        mcd_lsm_result* out);
/* Checks of the tensor-core kernels (no counterpart in the reference):
 * D (128x64) = A (128x64) B^T (B 64x64) with BF16 inputs and FP32
 * accumulation; one forward/backward pass of the network on n <= 128 samples
 * (gradient of sum_i w_i (f(x_i) - y_i)^2 / #{w_i > 0}, parameter layout as
 * above); inference on n inputs. */
int mcd_umma_selftest(mcd_ctx* ctx, const float* a, const float* b, float* d);
int mcd_mlp_gradients(mcd_ctx* ctx, const float* params, const float* x0, const float* x1,
                      const float* y, const float* w, int n, float* grad, float* loss);
int mcd_mlp_forward(mcd_ctx* ctx, const float* params, const float* x0, const float* x1, size_t n,
                    float* out);

/* ---- Greeks --------------------------------------------------------------- */
/* mcd::greeks::LrGreeksResult / PathwiseGreeksResult
 * (include/mcd/greeks/likelihood_ratio.hpp:15-18, pathwise.hpp:14-17). */
typedef struct {
    double value;
    double standard_error;
} mcd_greek;

/* Sensitivities of one contract from mcd_greeks_batch.  Bit i of `defined`
 * is set when field i (in declaration order, price = bit 0) is defined for
 * the product: price and the finite differences always; pathwise for European
 * and Asian (src/greeks/pathwise.cpp); likelihood ratio delta/gamma/vega/rho
 * always (European and digital as likelihood_ratio.cpp:33-73, every
 * path-dependent product with the barrier's first-step score :105-154, which
 * the reference applies to barriers only); likelihood-ratio theta for European
 * and digital. */
typedef struct {
    mcd_greek price;
    mcd_greek fd_delta, fd_gamma, fd_vega;
    mcd_greek pathwise_delta, pathwise_vega, pathwise_rho;
    mcd_greek lr_delta, lr_gamma, lr_vega, lr_rho, lr_theta;
    uint64_t path_count;
    uint32_t defined;
    uint32_t reserved;
} mcd_greeks_result;

/* Batched risk: price, common-random-number finite-difference delta, gamma
 * and vega (central differences with bumps spot_bump_rel * spot and
 * vol_bump_rel * vol, as finite_difference.cpp:40-65 re-prices with the same
 * seed), pathwise and likelihood-ratio Greeks of every contract, in one
 * persistent launch (a CUDA graph of the sensitivity kernel and its merge).
 * Every estimate is the mean of a per-path quantity and comes with its
 * standard error.  The price equals mcd_price_batch's bit for bit.
 * Unsupported: antithetic pairing, the control-variate Asian and the
 * Brownian-bridge barrier (MCD_ERR_UNSUPPORTED).  The spot-down and vol-down
 * states must stay positive (bumps < 1). */
int mcd_greeks_batch(mcd_ctx* ctx, const mcd_contract* contracts, size_t n, double spot_bump_rel,
                     double vol_bump_rel, int precision, mcd_greeks_result* results);
/* Launch shape of the sensitivity kernel (variant 0..3: register budget for
 * 2, 4, 6 or 8 resident CTAs; ctas_per_sm 0 = occupancy limit) and its tuner, which
 * times every candidate on the given batch and keeps the fastest. */
int mcd_greeks_set_launch_shape(mcd_ctx* ctx, int precision, int variant, int ctas_per_sm);
int mcd_greeks_autotune(mcd_ctx* ctx, const mcd_contract* contracts, size_t n, double spot_bump_rel,
                        double vol_bump_rel, int precision, int* variant, int* ctas_per_sm,
                        double* best_ms);

/* mcd::greeks::EuropeanGreeks and BumpSizes (finite_difference.hpp:9-22). */
typedef struct {
    double delta, gamma, vega, theta, rho;
} mcd_european_greeks;
typedef struct {
    double spot, vol, rate, time;
} mcd_bump_sizes;
/* replaces mcd::greeks::default_bump_sizes (src/greeks/finite_difference.cpp:23-38) */
mcd_bump_sizes mcd_default_bump_sizes(double spot, double vol, double time);
/* replaces mcd::greeks::finite_difference_european (finite_difference.cpp:40-65):
 * the nine common-random-number re-prices run as one batch launch. */
int mcd_fd_european(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                    double vol, double time, int type, uint64_t path_count, uint64_t seed,
                    mcd_bump_sizes bumps, int precision, mcd_european_greeks* out);

/* mcd::greeks::LrGreeks (likelihood_ratio.hpp:20-29); has_theta = 0 where
 * the reference leaves theta empty (barrier). */
typedef struct {
    mcd_greek delta, gamma, vega, rho, theta;
    int32_t has_theta;
    int32_t reserved;
} mcd_lr_greeks;
/* replace mcd::greeks::likelihood_ratio_european / _digital / _barrier
 * (src/greeks/likelihood_ratio.cpp:75-154) */
int mcd_lr_european(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                    double vol, double time, int type, uint64_t path_count, uint64_t seed,
                    int precision, mcd_lr_greeks* out);
int mcd_lr_digital(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                   double vol, double time, int type, int digital_style, double cash_amount,
                   uint64_t path_count, uint64_t seed, int precision, mcd_lr_greeks* out);
int mcd_lr_barrier(mcd_ctx* ctx, double spot, double strike, double barrier, double rate,
                   double carry_yield, double vol, double time, int type, int direction, int knock,
                   double rebate, int monitoring_points, uint64_t path_count, uint64_t seed,
                   int precision, mcd_lr_greeks* out);

/* mcd::greeks::PathwiseGreeks (pathwise.hpp:23-25). */
typedef struct {
    mcd_greek delta, vega, rho;
} mcd_pathwise_greeks;
/* replace mcd::greeks::pathwise_european / pathwise_asian (src/greeks/pathwise.cpp:28-147) */
int mcd_pathwise_european(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                          double vol, double time, int type, uint64_t path_count, uint64_t seed,
                          int precision, mcd_pathwise_greeks* out);
int mcd_pathwise_asian(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                       double vol, double time, int type, int strike_style, int average_style,
                       int monitoring_points, uint64_t path_count, uint64_t seed, int precision,
                       mcd_pathwise_greeks* out);

/* ---- frozen-boundary American Greeks --------------------------------------- */
/* The reference's recipe for American sensitivities (tests/lsm_test.cpp:138-185):
 * fit the Longstaff-Schwartz policy once, then reprice against that frozen
 * policy (src/pricers/lsm.cpp:151-213) at bumped inputs on the same paths, so
 * the exercise boundary does not jump between the bumped prices.  Here every
 * scenario runs in one streaming pass (no path storage): each path carries
 * the base state and the states at spot +/- spot_bump and vol +/- vol_bump.
 * Values are central differences of the scenario prices, exactly as calling
 * the replay once per scenario; standard errors are those of the per-path
 * differences (common random numbers).  With exercise at inception every
 * scenario price is the intrinsic value at its spot (the frozen decision). */
typedef struct {
    mcd_greek price;           /* frozen replay at the inputs (= the fitted price) */
    mcd_greek delta, gamma, vega;
    double scenario[4];        /* frozen prices at spot+h, spot-h, vol+h_v, vol-h_v */
    double spot_bump, vol_bump;
    uint64_t path_count;
    int32_t exercise_at_inception;
    int32_t reserved;
} mcd_american_greeks;
/* Against a given QR policy (as returned by mcd_lsm_american).  Bumps are
 * absolute: 0 < spot_bump < spot, 0 < vol_bump < vol. */
int mcd_lsm_frozen_greeks(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                          double vol, double time, int type, int monitoring_points, uint64_t path_count,
                          uint64_t seed, const double* coefficients, const uint8_t* has_coefficients,
                          int exercise_at_inception, double spot_bump, double vol_bump, int precision,
                          mcd_american_greeks* out);
/* Many contracts: fits every policy by the QR regression (as mcd_lsm_batch),
 * then replays all scenarios of all contracts against the device-resident
 * policies in one launch.  Bumps relative: h = spot_bump_rel * spot,
 * h_v = vol_bump_rel * vol, each in (0, 1). */
int mcd_lsm_greeks_batch(mcd_ctx* ctx, const mcd_lsm_contract* contracts, size_t n, double spot_bump_rel,
                         double vol_bump_rel, int precision, mcd_american_greeks* results);

/* ---- Sobol quasi-Monte Carlo ----------------------------------------------- */
/* Dimensions of the Sobol generator: the reference's seven
 * (src/core/sobol.cpp:22-30) followed by every further primitive polynomial
 * in ascending (degree, coefficient bits) order, same initial direction
 * numbers (m_i = 1) and recurrence.  Path-dependent contracts need
 * monitoring_points <= this. */
#define MCD_SOBOL_MAX_DIMS 256
/* Quasi-Monte Carlo prices of a batch in one persistent launch: Sobol points
 * at indices 1..path_count, Brownian-bridge paths with dimension k on the
 * k-th breadth-first bisection point (src/models/brownian_bridge_path.cpp
 * :20-77), mean of the discounted payoffs (src/pricers/qmc.cpp:15-57).  Every
 * batch product is accepted (the reference covers the European and the
 * arithmetic Asian); antithetic pairing, the control-variate Asian and the
 * Brownian-bridge barrier are not (MCD_ERR_UNSUPPORTED).  standard_error is
 * 0: a low-discrepancy sequence has none (include/mcd/pricers/qmc.hpp:9-15). */
int mcd_qmc_batch(mcd_ctx* ctx, const mcd_contract* contracts, size_t n, int precision,
                  mcd_mc_result* results);
/* replaces mcd::pricers::qmc_sobol_european (src/pricers/qmc.cpp:15-30) */
int mcd_qmc_sobol_european(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                           double vol, double time, int type, uint64_t path_count, int precision,
                           double* price);
/* replaces mcd::pricers::qmc_sobol_asian (src/pricers/qmc.cpp:32-57); the
 * reference caps monitoring_points at 7, this at MCD_SOBOL_MAX_DIMS. */
int mcd_qmc_sobol_asian(mcd_ctx* ctx, double spot, double strike, double rate, double carry_yield,
                        double vol, double time, int type, int strike_style, int monitoring_points,
                        uint64_t path_count, int precision, double* price);
/* Sobol coordinates of dims [dim_begin, dim_begin + n_dims) at indices
 * [index_begin, index_begin + n_indices) from the device generator, row-major
 * by index; mcd::sobol_point (src/core/sobol.cpp:83-97) for each. */
int mcd_sobol_points(mcd_ctx* ctx, unsigned dim_begin, unsigned n_dims, uint64_t index_begin,
                     uint64_t n_indices, double* out);

/* ---- draws (parity and diagnostics) ------------------------------------- */
/* Philox4x32-10 of n (counter, key) pairs; replaces mcd::philox4x32_10
 * (src/core/rng.cpp:41-47).  counters: n x 4, keys: n x 2, out: n x 4. */
int mcd_philox(mcd_ctx* ctx, const uint32_t* counters, const uint32_t* keys, size_t n,
               uint32_t* out);
/* Draws for paths [path_begin, path_begin+n_paths) x draws
 * [draw_begin, draw_begin+n_draws), row-major by path.  stream_id 0 gives the
 * standard normal of mcd::standard_normal_variate (src/core/rng.cpp:59-66),
 * stream_id 1 the uniform of mcd::uniform_variate (:68-74); precision picks the
 * FP64 or FP32 transform (FP32 values are widened to double). */
int mcd_draws(mcd_ctx* ctx, uint64_t seed, uint64_t path_begin, uint64_t n_paths,
              uint32_t draw_begin, uint32_t n_draws, int stream_id, int precision, double* out);

/* ---- closed forms and lattices (host FP64, no GPU, no context) ------------ */
/* The reference module exports these beside the Monte Carlo pricers
 * (bindings/python/src/module.cpp); each keeps the reference's operation
 * order.  type: mcd_option_type; direction/knock/style: the enums above. */
/* replaces mcd::pricers::crr_binomial_american (src/pricers/binomial.cpp:39-72): the
 * Cox-Ross-Rubinstein American price, the yardstick for Longstaff-Schwartz.
 * NaN when steps < 1. */
double mcd_crr_binomial_american(double spot, double strike, double rate, double carry_yield, double vol,
                                 double time, int steps, int type);
/* No counterpart in the reference.  The Bermudan CRR price with exercise only
 * at t = j T / exercise_dates, j = 0 .. exercise_dates - 1 (the dates at which
 * Longstaff-Schwartz with that many monitoring points decides), steps_per_date
 * tree steps between dates: the exact value that LSM's in-sample estimate
 * approximates.  NaN for non-positive counts or more than 2^20 steps. */
double mcd_crr_binomial_bermudan(double spot, double strike, double rate, double carry_yield, double vol,
                                 double time, int exercise_dates, int steps_per_date, int type);
/* replaces mcd::pricers::crr_binomial (src/pricers/binomial.cpp:9-37): European
 * CRR tree; writes {price, risk-neutral probability, up factor, down factor}. */
int mcd_crr_binomial(double spot, double strike, double rate, double carry_yield, double vol, double time,
                     int steps, int type, double* price_p_u_d);
/* replaces mcd::pricers::black_scholes_merton (src/pricers/analytic.cpp:30-38) */
double mcd_black_scholes_merton(double spot, double strike, double rate, double carry_yield, double vol,
                                double time, int type);
/* replaces mcd::pricers::black76 (src/pricers/analytic.cpp:40-49) */
double mcd_black76(double forward, double strike, double rate, double vol, double time, int type);
/* replaces mcd::pricers::kemna_vorst (src/pricers/analytic.cpp:51-59) */
double mcd_kemna_vorst(double spot, double strike, double rate, double carry_yield, double vol, double time,
                       int type);
/* replaces mcd::pricers::reiner_rubinstein (src/pricers/analytic.cpp:61-132) */
double mcd_reiner_rubinstein(double spot, double strike, double barrier, double rate, double carry_yield,
                             double vol, double time, int type, int direction, int knock, double rebate);
/* replaces mcd::pricers::lookback_fixed_strike (src/pricers/analytic.cpp:184-195) */
double mcd_lookback_fixed_strike(double spot, double strike, double rate, double carry_yield, double vol,
                                 double time, int type);
/* replaces mcd::pricers::lookback_floating_strike (src/pricers/analytic.cpp:197-212) */
double mcd_lookback_floating_strike(double spot, double rate, double carry_yield, double vol, double time,
                                    int type);
/* replaces mcd::pricers::digital (src/pricers/analytic.cpp:214-222) */
double mcd_digital_analytic(double spot, double strike, double rate, double carry_yield, double vol, double time,
                            int type, int style, double cash_amount);
/* replace mcd::pricers::forward_price, forward_value, futures_mark_to_market
 * (src/pricers/analytic.cpp:224-235) */
double mcd_forward_price(double spot, double rate, double carry_yield, double time);
double mcd_forward_value(double forward_now, double forward_at_inception, double rate, double time_to_expiry);
double mcd_futures_mark_to_market(double futures_price_new, double futures_price_old);
/* replaces mcd::pricers::heston_semi_analytic (src/pricers/heston.cpp:48-82):
 * P1/P2 by 128-point Gauss-Legendre over [0, 200]. NaN for a null params. */
double mcd_heston_semi_analytic(const mcd_heston_params* params, double strike, int type);

/* ---- timing helper for benchmarks ---------------------------------------- */
/* Average device time (ms) of the persistent path kernel over the calls made
 * since the last reset, measured with CUDA events on the launching stream. */
int mcd_kernel_timing(mcd_ctx* ctx, int reset, double* avg_ms, uint64_t* launches);

#ifdef __cplusplus
}
#endif

#endif /* MCD_GPU_H */
