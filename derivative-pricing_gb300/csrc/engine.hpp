// engine.hpp -- private interface between the C-ABI host code and the kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "mcd_gpu.h"

namespace mcdg {

// One accumulator (include/mcd/core/stats.hpp:21-71): count, mean, M2.
struct Welford {
    unsigned long long count;
    double mean;
    double m2;
};

constexpr int kSlabPaths = 4096;       // MCD_SLAB_PATHS
constexpr int kSlabThreads = 128;      // one CTA = one slab lane group
constexpr int kPathsPerThread = kSlabPaths / kSlabThreads;
constexpr int kNumVariants = 5;        // __launch_bounds__ min-blocks 4, 8, 12, 16, 6

// Internal product kinds: one loop body per kind (the switch is outside the
// step loop and uniform over a CTA).
enum Kind : int32_t {
    kEuropean = 0,
    kDigital = 1,
    kAsianArith = 2,
    kAsianGeo = 3,
    kAsianCv = 4,          // arithmetic fixed-strike with geometric control variate
    kBarrier = 5,
    kBarrierBridge = 6,    // Brownian-bridge crossing correction (stream 1 uniforms)
    kLookbackFixed = 7,
    kLookbackFloating = 8,
};

// A contract as the kernels see it: host-precomputed FP64 constants, laid out
// once per batch.  Terminal products use dt = T (one step).
struct DevContract {
    int32_t kind;
    int32_t type;          // 0 call, 1 put
    int32_t up;            // barrier direction is up
    int32_t out;           // barrier knock-out
    int32_t floating;      // floating strike (asian, lookback)
    int32_t asset;         // asset-or-nothing digital
    int32_t n_steps;
    int32_t antithetic;
    double spot, strike, barrier, rebate, cash;
    double discount;       // exp(-r T)                   (monte_carlo.cpp:160)
    double drift;          // (r - q - 0.5 vol^2) * dt    (gbm.cpp:8-9)
    double vs;             // vol * sqrt(dt)              (gbm.cpp:10)
    double log_barrier;    // ln H                        (monte_carlo.cpp:193)
    double log_h_rel;      // ln(H / S0)  (FP32 log-space barrier)
    double bb_denom;       // vol * vol * dt              (monte_carlo.cpp:219)
    double kv_anchor;      // kemna_vorst                 (monte_carlo.cpp:279-280)
    uint64_t path_count;
    uint64_t seed;
    uint32_t n_slabs;
    uint32_t orig_index;   // position in the caller's array
};

// Validates one contract and converts it to the kernel layout; null on
// success, else the reason it is rejected (context.cpp).  Shared by
// mcd_price_batch's planner and the allocation-free entry point.
const char* convert_contract(const mcd_contract& in, uint32_t index, DevContract& out);

// Launches (all asynchronous on `stream`).
// The persistent path kernel over items [0, item_prefix[n_contracts]) (the
// item count is read on the device, so one captured launch serves every path
// count of the same number of contracts).
cudaError_t launch_path_kernel(int precision, int variant, int grid, const DevContract* contracts,
                               int n_contracts, const uint32_t* item_prefix, uint32_t* ticket,
                               Welford* partials, uint32_t* error_flag, cudaStream_t stream);
cudaError_t launch_merge_kernel(const DevContract* contracts, int n_contracts,
                                const uint32_t* item_prefix, const Welford* partials,
                                void* results /* mcd_mc_result[] */, cudaStream_t stream);
cudaError_t path_kernel_occupancy(int precision, int variant, int* blocks_per_sm);
// Order-independent 64-bit digest of n_words 64-bit words (one CTA): the sum
// over i of mix(word_i, i), written to *out.
cudaError_t launch_words_digest(const uint64_t* words, size_t n_words, uint64_t* out,
                                cudaStream_t stream);

cudaError_t launch_philox_kernel(const uint32_t* counters, const uint32_t* keys, size_t n,
                                 uint32_t* out, cudaStream_t stream);
cudaError_t launch_draws_kernel(uint64_t seed, uint64_t path_begin, uint64_t n_paths,
                                uint32_t draw_begin, uint32_t n_draws, int stream_id,
                                int precision, double* out, cudaStream_t stream);

}  // namespace mcdg
