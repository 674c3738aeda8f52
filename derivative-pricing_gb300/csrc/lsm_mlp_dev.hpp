// lsm_mlp_dev.hpp -- launch interface of the learned-regression kernels.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "engine.hpp"
#include "lsm.hpp"

namespace mcdg {

// Training schedule of the continuation network (per contract, per date).
struct MlpConfig {
    int steps_first;  // Adam steps at the first (latest) exercise date, from the initial weights
    int steps;        // Adam steps at every earlier date (feature fine-tuning; 0 = features fixed)
    float lr_first;
    float lr;
};

// Pass modes: kStep = exercise, discount and cash-flow update at date n-k;
// kGram = regression data of date n-k-1.
enum PassMode { kStep = 1, kGram = 2 };

// Node tables.  The network's inputs are x0 = 4 (S/K - 1) and the date's time
// input, which is one value per date, so at a date every learned feature is a
// function of u = ln(S/K) alone.  The features are evaluated (tcgen05) at
// kNodes equally spaced values of u covering the in-the-money side of the
// date's distribution, and every path uses their linear interpolation: as its
// regression basis (the fit is exact least squares on the interpolated
// features, built from per-bin moments of the paths) and for its exercise
// decision (an interpolated continuation table).
constexpr int kNodes = 512;
constexpr int kNodeSlices = kNodes / 64;            // Gram CTAs per contract (64 bins each)
constexpr int kMoments = 4;                          // per bin: n 2^40 + sum t, sum t^2, sum y, sum t y
constexpr int kCountShift = 40;                      // n above sum t (< 2^39 for <= 2^23 paths per CTA)
constexpr double kTScale = 65536.0;                  // t in [0, 1] as an integer of 16 bits
constexpr double kYScale = 16777216.0;               // |y| / y_bound as an integer of 24 bits
constexpr double kGridSd = 7.0;                      // the grid covers the mean +/- 7 standard deviations

struct NodeGrid {
    float lo, h, inv_h;  // node i at u = lo + i h
    float y_bound;       // |(cash flow - exercise value) / K| is at most this on the grid's paths
};

// ln(S_d/K) of the stored GBM paths is normal with mean ln(S0/K) + d drift and
// standard deviation vs sqrt(d); the grid takes the in-the-money side of
// +/- kGridSd of it (paths beyond use the end bins).  Every kernel derives
// the grid from this function, so they agree on it bit for bit.
__host__ __device__ inline NodeGrid node_grid(const LsmDev& c, int date) {
    const double m = log(c.spot / c.strike) + static_cast<double>(date) * c.drift;
    const double s = c.vs * sqrt(static_cast<double>(date));
    double lo, hi;
    if (c.type == 1) {  // put: in the money below the strike
        lo = fmin(m - kGridSd * s, -1e-6);
        hi = 0.0;
    } else {
        lo = 0.0;
        hi = fmax(m + kGridSd * s, 1e-6);
    }
    const double h = (hi - lo) / static_cast<double>(kNodes - 1);
    // cash flows and exercise values are at most max(S)/K over the remaining dates
    const double n = static_cast<double>(c.n_steps);
    const double top = log(c.spot / c.strike) + n * fmax(c.drift, 0.0) + kGridSd * c.vs * sqrt(n);
    NodeGrid g;
    g.lo = static_cast<float>(lo);
    g.h = static_cast<float>(h);
    g.inv_h = static_cast<float>(1.0 / h);
    g.y_bound = static_cast<float>(c.type == 1 ? 1.0 : 2.0 * fmax(exp(top), 1.0));
    return g;
}

// Feature tables: the network's 64 last-layer features at the kNodes nodes of
// a date, for contracts [c_first, c_end), at feats + (reg_offset + d) x
// kNodes x 64 floats.  all_dates: every regression date 1 .. n-1 of each
// contract in one launch (the features do not change from date to date when
// they are not fine-tuned); otherwise the date n-k-1 of backward iteration k.
cudaError_t launch_lsm_mlp_features(int k, bool all_dates, int max_steps, const LsmDev* c, int c_first, int c_end,
                                    const float* nets, float* feats, uint32_t* err, cudaStream_t stream);
// The binned path pass of backward iteration k (exercise at date n-k from the
// continuation table etab, discount, moments of date n-k-1) and the sliced
// Gram matrices of date n-k-1 that the solve sums.  Contracts [c_first,
// c_end) and their groups [g_first, g_end) (whole contracts; launches for
// disjoint ranges may run concurrently).
cudaError_t launch_lsm_mlp_binned(int precision, int k, int mode, const LsmDev* c, int c_first, int c_end,
                                  const uint32_t* group_contract, uint32_t g_first, uint32_t g_end, const void* store,
                                  double* cf, const int* snap_ok, const float* feats, const float* etab,
                                  unsigned long long* mom_part, float* gram_part, Welford* final_part,
                                  cudaStream_t stream);

size_t mlp_train_smem_bytes();
size_t mlp_infer_smem_bytes();
cudaError_t mlp_prepare();  // opts the kernels into their dynamic shared memory
// The first training of contracts [c_first, c_end) on their latest regression
// date n-1 (Adam, cfg.steps_first steps; its samples drawn by regenerating
// the sampled paths, so it needs neither the path store nor the terminal
// step) and, with fixed features (cfg.steps == 0), every date's feature table.
// pre_s / pre_cf: cfg.steps_first x 128 doubles per contract.
cudaError_t launch_lsm_mlp_first_training(int precision, const LsmDev* c, int c_first, int c_end, int max_steps,
                                          float* nets, float* snaps, int* snap_ok, int* adam_t, float* feats,
                                          double* pre_s, double* pre_cf, const MlpConfig& cfg, uint32_t* err,
                                          cudaStream_t stream);
// One backward iteration k: exercise at date n-k, discount, and (train =
// true) the Gram matrix and output-layer fit of date n-k-1 on node tables; at
// k = 0 the fit first waits for `trained` (recorded after
// launch_lsm_mlp_first_training).  train = false replays given networks path
// by path (lsm_mlp_pass).  Buffers: gram_part
// n x kNodeSlices x kGramPacked floats, feats (sum of n_steps + 1) x kNodes x
// 64 floats (rows as the snapshots), etab n x kNodes floats, mom_part groups x
// kMoments x kNodes.
// Contracts [c_first, c_end), groups [g_first, g_end), as launch_lsm_mlp_binned.
cudaError_t launch_lsm_mlp_iteration(int precision, int k, bool train, const LsmDev* c, int c_first, int c_end,
                                     int max_steps, const uint32_t* group_contract, uint32_t g_first, uint32_t g_end,
                                     const void* store,
                                     double* cf, float* nets, float* snaps, int* snap_ok, int* adam_t,
                                     float* gram_part, float* feats, float* etab, unsigned long long* mom_part,
                                     const MlpConfig& cfg, Welford* final_part, cudaEvent_t trained, uint32_t* err,
                                     cudaStream_t stream);
cudaError_t launch_mlp_grad(const float* params, const float* x0, const float* x1, const float* y, const float* w,
                            int n, float* grad, float* loss, uint32_t* err, cudaStream_t stream);
cudaError_t launch_mlp_forward(const float* params, const float* x0, const float* x1, int n, float* out,
                               uint32_t* err, cudaStream_t stream);
cudaError_t launch_umma_selftest(const float* A, const float* B, float* D, uint32_t* err, cudaStream_t stream);

}  // namespace mcdg
