// Forwarding header: the reference's mcd/core/sobol.hpp resolves to the GPU
// shim (its kSobolMaxDimensions is the GPU engine's 256-dimension table).
#pragma once
#include "../../../mcd_shim.hpp"
