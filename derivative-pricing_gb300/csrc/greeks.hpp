// greeks.hpp -- batched sensitivities: layouts shared by host and kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "engine.hpp"

namespace mcdg {

// Per-path outputs, in this order (mcd_greeks_result lists the same).
enum GreekIndex : int {
    kGPrice = 0,
    kGFdDelta = 1,
    kGFdGamma = 2,
    kGFdVega = 3,
    kGPwDelta = 4,
    kGPwVega = 5,
    kGPwRho = 6,
    kGLrDelta = 7,
    kGLrGamma = 8,
    kGLrVega = 9,
    kGLrRho = 10,
    kGLrTheta = 11,
    kNumGreeks = 12,
};

// Constants of one contract beyond DevContract (same sorted position).
struct DevGreeks {
    double vol, time, rate;
    double dt, sqrt_dt;        // dt = T / monitoring points (T for terminal products)
    double mu;                 // r - q - vol^2 / 2   (likelihood_ratio.cpp:44)
    double h_spot, h_vol;      // absolute finite-difference bumps
    double drift_up, vs_up;    // per-step constants at vol + h_vol (gbm.cpp:8-10 order)
    double drift_dn, vs_dn;    // ... at vol - h_vol
    double log_h_rel_up;       // ln(H / (S0 + h_spot))  FP32 barrier test of the spot-up state
    double log_h_rel_dn;       // ln(H / (S0 - h_spot))
    // reciprocals for the FP32 kernel (FP64 divisions are costly on this GPU;
    // the FP64 kernel keeps the reference's divisions)
    double inv_2hs, inv_hs2, inv_2hv;
    double lr_delta_scale;     // 1 / (S0 vol sqrt(dt1)), dt1 = first-step length
    double lr_gamma_scale;     // 1 / (S0^2 vol^2 dt1)
    double sqrt_dt_over_vol, inv_vol, inv_n, inv_spot, inv_2t, mu_over_vol_sqrt_t;
    int32_t vol_series;        // |vol-bump exponent| <= 1e-2 on all but > 8-sigma paths: cubic expm1
    int32_t pad;
};

cudaError_t launch_greeks_kernel(int precision, int variant, int grid, const DevContract* contracts,
                                 const DevGreeks* greeks, int n_contracts, const uint32_t* item_prefix,
                                 uint32_t total_items, uint32_t* ticket, Welford* partials,
                                 uint32_t* error_flag, cudaStream_t stream);
// out: per contract (caller order) kNumGreeks x {mean, standard error}, then
// the path count as a double.
cudaError_t launch_greeks_merge(const DevContract* contracts, int n_contracts, const uint32_t* item_prefix,
                                const Welford* partials, double* out, cudaStream_t stream);
cudaError_t greeks_kernel_occupancy(int precision, int variant, int* blocks_per_sm);
constexpr int kGreeksVariants = 4;  // __launch_bounds__ min-blocks 2, 4, 6, 8
constexpr int kGreeksOutStride = 2 * kNumGreeks + 1;

}  // namespace mcdg
