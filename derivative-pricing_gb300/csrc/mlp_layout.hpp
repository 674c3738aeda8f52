// mlp_layout.hpp -- parameter layout of the continuation network (host and device).
#pragma once

namespace mcdg {
namespace mlp {

constexpr int kHidden = 64;
constexpr int kTile = 128;  // samples per tensor-core tile (MMA M)
// Parameter offsets (floats).
constexpr int kW1 = 0;      // [64][2]
constexpr int kB1 = 128;    // [64]
constexpr int kW2 = 192;    // [64 out][64 in]
constexpr int kB2 = 4288;   // [64]
constexpr int kW3 = 4352;   // [64]
constexpr int kB3 = 4416;   // [1]
constexpr int kParams = 4417;
constexpr int kParamStride = 4480;  // padded per-network stride

}  // namespace mlp
}  // namespace mcdg
