// Forwarding header: the reference's mcd/core/types.hpp resolves to the GPU shim, so
// reference code that includes it builds unchanged against libmcd_shim.so.
#pragma once
#include "../../../mcd_shim.hpp"
