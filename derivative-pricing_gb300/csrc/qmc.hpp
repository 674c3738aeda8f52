// qmc.hpp -- Sobol quasi-Monte Carlo with Brownian-bridge paths: layouts
// shared by host and kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "engine.hpp"

namespace mcdg {

constexpr int kSobolDims = 256;  // MCD_SOBOL_MAX_DIMS
constexpr int kSobolBits = 32;
constexpr int kBridgeSlots = 12;  // bridge values kept per path (one per tree depth, plus the origin)

// One node of a bridge program (src/models/brownian_bridge_path.cpp:20-77
// rearranged).  The reference fills w[] in breadth-first bisection order,
// node k taking Sobol dimension k; a program lists the same nodes in
// depth-first pre-order, so every node's interval end points are its
// ancestors and a path needs one stored value per tree depth instead of all
// n.  t_* are time indices (point i sits at t = (i+1) T / n; -1 is the
// origin); slot 0 always holds the origin's w = 0.
struct BridgeNode {
    int16_t t_left, t_mid, t_right;  // t_left = t_right = -1 marks the terminal (root) node
    uint16_t dim;                    // Sobol dimension = breadth-first draw number
    uint8_t slot_left, slot_right, slot_out, pad;
    uint8_t pad2[4];
};
static_assert(sizeof(BridgeNode) == 16, "bridge node layout");

// Per contract (same sorted position as DevContract): its bridge program and
// the constants of brownian_bridge_path.cpp:70-76.
struct DevQmc {
    double time, vol;
    double drift_rate;  // r - q - vol^2 / 2
    uint32_t prog_offset;
    uint32_t pad;
};

cudaError_t launch_qmc_kernel(int precision, int grid, const DevContract* contracts, const DevQmc* qmc,
                              int n_contracts, const uint32_t* item_prefix, uint32_t total_items,
                              const BridgeNode* programs, const uint32_t* directions, uint32_t* ticket,
                              Welford* partials, uint32_t* error_flag, cudaStream_t stream);
cudaError_t qmc_kernel_occupancy(int precision, int* blocks_per_sm);
// Sobol coordinates x / 2^32 of dims [dim0, dim0 + n_dims) at indices
// [index0, index0 + n_idx), row-major by index (index 0 gives 0).
cudaError_t launch_sobol_points(const uint32_t* directions, uint32_t dim0, uint32_t n_dims, uint64_t index0,
                                uint64_t n_idx, double* out, cudaStream_t stream);

}  // namespace mcdg
