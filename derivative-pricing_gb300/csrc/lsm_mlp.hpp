// lsm_mlp.hpp -- learned continuation values for Longstaff-Schwartz.
#pragma once

#include <cstddef>

#include "context.hpp"
#include "mcd_gpu.h"

namespace mcdg {

// Prices a batch of American contracts with an MLP continuation-value
// regression in place of the Laguerre QR fit (see lsm_mlp.cu).
int lsm_mlp_batch(Ctx& ctx, const mcd_lsm_contract* cs, size_t n, int precision,
                  mcd_lsm_result* results);

}  // namespace mcdg
