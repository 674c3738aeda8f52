// lsm.hpp -- batched Longstaff-Schwartz: layouts shared by host and kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "engine.hpp"

namespace mcdg {

constexpr int kLsmChunk = 1024;      // paths per chunk (fixed reduction unit)
constexpr int kLsmThreads = 128;     // 8 paths per thread per chunk
constexpr unsigned kRefineGrid = 1216;  // CTAs of the second regression pass (8 per SM)
constexpr int kLsmBasis = 4;         // weighted Laguerre, degree 3 (src/pricers/lsm.cpp:16-25)

// One American contract.  Paths are stored date-major: S[d-1][i] for dates
// d = 1..n at s_offset + (d-1)*path_count + i (elements of the path
// precision); cashflows are FP64 at cf_offset + i.
struct LsmDev {
    double spot, strike;
    double disc;          // exp(-r dt) (src/pricers/lsm.cpp:67)
    double drift;         // (r - q - vol^2/2) dt  (src/models/gbm.cpp:8-9)
    double vs;            // vol sqrt(dt)          (src/models/gbm.cpp:10)
    double inception;     // intrinsic at t = 0    (src/pricers/lsm.cpp:141)
    uint64_t seed, path_count;
    uint64_t s_offset, cf_offset;
    uint32_t chunk_begin, n_chunks;
    uint32_t reg_offset;  // row of date 0 in the per-date regression table
    int32_t n_steps, type;
    uint32_t group_begin, n_groups;  // learned regression: CTAs of group_chunks chunks each
    uint32_t group_chunks;
    uint32_t fold_begin, n_folds;    // QR regression: second level of the chunk-sum tree,
    uint32_t fold_chunks;            // groups of fold_chunks chunks
    float strike_f, inv_strike_f, disc_f, phi_f;  // FP32 copies for the FP32-path kernels
};

constexpr int kLsmMaxGroups = 256;  // learned-regression CTAs per contract at most
constexpr int kLsmMinGroupChunks = 16;  // chunks per learned-regression CTA at least (amortises its set-up)
constexpr int kLsmMaxFolds = 256;       // QR: fold groups per contract at most
constexpr int kLsmMinFoldChunks = 32;   // QR: chunks per fold group at least
constexpr int kGramPacked = 66 * 67 / 2;  // upper triangle of the 66 x 66 Gram matrix, row-major

// Regression state of one (contract, date): T, the date's preconditioner
// (upper triangular, T^T X^T X T = I for its in-the-money basis matrix X;
// packed row-major: (0,0) (0,1) (0,2) (0,3) (1,1) (1,2) (1,3) (2,2) (2,3) (3,3)),
// the Laguerre coefficients gamma, and flags.
struct LsmReg {
    double T[10];
    double gamma[4];
    int32_t has;          // 1 coefficients valid (>= 4 ITM paths), -1 no regression, 2 second pass pending
    int32_t degenerate;   // Cholesky of the lagged Gram matrix: 0 plain, 2 with a diagonal shift, 1 failed
    float T_f[10];        // FP32 copies for the FP32-path kernels (written with T and gamma)
    float gamma_f[4];
    float poly_f[4];      // FP32 path: the continuation value e^{-x/2} (p0 + p1 x + p2 x^2 + p3 x^3),
                          // x = S/K, the Laguerre combination gamma expanded in FP64 (laguerre_poly)
};

// Per-chunk partial sums of one date's regression: count + 10 Gram entries +
// 4 right-hand side entries in a preconditioned basis.
struct LsmPartial {
    double v[16];
};

// Frozen-policy replay (lsm_frozen.cu).  One scenario = the inputs of one
// reprice_against_frozen_policy call (src/pricers/lsm.cpp:151-213) on the
// contract's paths (same seed): spot and the per-step GBM constants of its
// volatility, in FP64 and as the FP32 kernel's copies.
struct FrozenScenario {
    double spot, drift, vs;
    float spot_f, mu_f, sg_f, pad;
};
constexpr int kFrozenScenarios = 5;  // base, spot+h, spot-h, vol+h, vol-h
constexpr int kFrozenOutputs = 8;    // five scenario averages, then the CRN delta, gamma, vega
struct FrozenDev {
    FrozenScenario sc[kFrozenScenarios];
    double inv_2hs, inv_hs2, inv_2hv;  // 1/(2h_S), 1/h_S^2, 1/(2h_vol)
    float inv_2hs_f, inv_hs2_f, inv_2hv_f, pad;
};

// Forward simulation of chunks [chunk_first, chunk_first + chunk_count).
// Monomial coefficients of gamma_0 L_0 + ... + gamma_3 L_3 (the weighted
// Laguerre polynomials of src/pricers/lsm.cpp:21-25 without their common
// factor e^{-x/2}), computed in FP64 and rounded once.
__host__ __device__ inline void laguerre_poly(const double gamma[4], float poly[4]) {
    poly[0] = static_cast<float>(gamma[0] + gamma[1] + gamma[2] + gamma[3]);
    poly[1] = static_cast<float>(-gamma[1] - 2.0 * gamma[2] - 3.0 * gamma[3]);
    poly[2] = static_cast<float>(0.5 * gamma[2] + 1.5 * gamma[3]);
    poly[3] = static_cast<float>(-gamma[3] / 6.0);
}

#ifdef __CUDACC__
// One date of a stored GBM path: FP32 paths step ln(S/S0) and store
// S0 exp(x); FP64 paths multiply S by exp(drift + vs z).  Every kernel that
// regenerates stored path values uses these, so they agree bit for bit.
__device__ __forceinline__ float gbm_log_step_f32(float x, float z, float mu, float sg) { return __fmaf_rn(sg, z, x + mu); }
__device__ __forceinline__ float gbm_spot_f32(float s0, float x) { return s0 * __expf(x); }
__device__ __forceinline__ double gbm_step_f64(double s, double z, double drift, double vs) { return s * exp(drift + vs * z); }
// FP32 continuation value at S from poly (the FP32 backward pass and the
// FP32 frozen replay both use this, so their decisions coincide).
__device__ __forceinline__ float continuation_poly32(float s, float inv_strike, const float p[4]) {
    const float x = s * inv_strike;
    const float e = __expf(-0.5f * x);
    return e * __fmaf_rn(__fmaf_rn(__fmaf_rn(p[3], x, p[2]), x, p[1]), x, p[0]);
}
#endif

cudaError_t launch_lsm_forward(int precision, const LsmDev* c, int n_contracts,
                               const uint32_t* chunk_contract, uint32_t chunk_first, uint32_t chunk_count,
                               void* s_store, cudaStream_t stream);
// One backward iteration k (see lsm.cu) of the contracts whose chunks are
// [chunk_first, chunk_first + chunk_count) -- whole contracts.  part: one
// partial per chunk, gpart: one per fold group (LsmDev::fold_begin/n_folds),
// counters zeroed before the first iteration: 2 per contract, 2 per fold group,
// then one word per iteration.  Launches for disjoint sets of contracts may
// run concurrently on different streams.
cudaError_t launch_lsm_iteration(int precision, int k, const LsmDev* c, int n_contracts,
                                 const uint32_t* chunk_contract, uint32_t chunk_first, uint32_t chunk_count,
                                 uint32_t total_folds, const void* s_store, double* cf, LsmReg* reg,
                                 LsmPartial* part, LsmPartial* gpart, Welford* final_part, uint32_t* counters,
                                 cudaStream_t stream);
cudaError_t launch_lsm_finish(const LsmDev* c, int n_contracts, const Welford* final_part,
                              double* out /* n x 6: price, se, count, inception, mean, se */,
                              cudaStream_t stream);
// Streams every chunk's paths forward once against the regression table
// `reg` (rows per contract at LsmDev::reg_offset), in n_scenarios (1 or
// kFrozenScenarios) scenarios, and writes per contract and output the path
// average, its standard error and the path count (out: n x outputs x 3;
// outputs = 1 for one scenario, kFrozenOutputs for five).
cudaError_t launch_lsm_frozen(int precision, int n_scenarios, const LsmDev* c, const FrozenDev* f,
                              int n_contracts, const uint32_t* chunk_contract, uint32_t total_chunks,
                              const LsmReg* reg, Welford* partials, double* out, cudaStream_t stream);

}  // namespace mcdg
