// Forwarding header: the reference's mcd/core/rng_simd.hpp resolves to the
// GPU shim (kHasNeon is false there: the draws come from the GPU).
#pragma once
#include "../../../mcd_shim.hpp"
