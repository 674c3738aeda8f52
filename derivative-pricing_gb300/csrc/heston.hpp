// heston.hpp -- Heston QE batch: per-set constants shared by host and device.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "engine.hpp"

namespace mcdg {

// One parameter set, with the reference's per-step constants precomputed on
// the host in its operation order (src/pricers/heston.cpp:95-99, :123-132).
struct HestonSet {
    double spot, v0, theta, kappa, xi;
    double e;          // exp(-kappa dt)
    double s2_const;   // theta xi^2 / (2 kappa) (1-e)^2
    double drift;      // (r - q) dt
    double k0, k1, k2, k3, k4;
    double discount;   // exp(-r T)
    double log_s0;     // ln S0
    double s2_lin;     // xi^2 e / kappa (1-e)   (FP32 path: s2 = v s2_lin + s2_const)
    uint64_t seed;
    uint64_t path_count;
    uint32_t n_slabs;
    int32_t n_steps;
};

// FP32 view used inside the FP32 kernel.
struct HestonSet32 {
    float s0, v0, theta, e, s2_lin, s2_const, c0, k1, k2, k3, k4;
};

__host__ __device__ inline HestonSet32 make_set32(const HestonSet& h) {
    HestonSet32 r;
    r.s0 = static_cast<float>(h.spot);
    r.v0 = static_cast<float>(h.v0);
    r.theta = static_cast<float>(h.theta);
    r.e = static_cast<float>(h.e);
    r.s2_lin = static_cast<float>(h.s2_lin);
    r.s2_const = static_cast<float>(h.s2_const);
    r.c0 = static_cast<float>(h.drift + h.k0);
    r.k1 = static_cast<float>(h.k1);
    r.k2 = static_cast<float>(h.k2);
    r.k3 = static_cast<float>(h.k3);
    r.k4 = static_cast<float>(h.k4);
    return r;
}

cudaError_t launch_heston(int precision, int grid, const HestonSet* sets, int n_sets,
                          const double* strikes, int n_strikes, int type, uint32_t items_per_set,
                          uint32_t* ticket, Welford* partials, double* out, cudaStream_t stream);
cudaError_t heston_occupancy(int precision, int* blocks);

}  // namespace mcdg
