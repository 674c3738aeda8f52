// lsm_mlp_dev.hpp -- launch interface of the learned-regression kernels.
#pragma once

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

size_t mlp_train_smem_bytes();
size_t mlp_infer_smem_bytes();
cudaError_t mlp_prepare();  // opts the kernels into their dynamic shared memory
// One backward iteration k: exercise at date n-k with that date's network,
// discount, and (train = true) the Gram matrix and output-layer fit of date
// n-k-1; at k = 0 the features are first trained on that date.  feat_cache
// (128 B per path, or null) carries each date's BF16 features to the next
// iteration's exercise decisions when the features are not fine-tuned.
cudaError_t launch_lsm_mlp_iteration(int precision, int k, bool train, const LsmDev* c, int n_contracts,
                                     const uint32_t* group_contract, uint32_t total_groups, const void* store,
                                     double* cf, float* nets, float* snaps, int* snap_ok, int* adam_t,
                                     float* gram_part, double* gram_sum, void* feat_cache, const MlpConfig& cfg,
                                     Welford* final_part, uint32_t* err, cudaStream_t stream);
cudaError_t launch_mlp_grad(const float* params, const float* x0, const float* x1, const float* y, const float* w,
                            int n, float* grad, float* loss, uint32_t* err, cudaStream_t stream);
cudaError_t launch_mlp_forward(const float* params, const float* x0, const float* x1, int n, float* out,
                               uint32_t* err, cudaStream_t stream);
cudaError_t launch_umma_selftest(const float* A, const float* B, float* D, uint32_t* err, cudaStream_t stream);

}  // namespace mcdg
