// mlp.cuh -- the 2 -> 64 -> 64 -> 1 continuation-value network (GELU), its
// parameter layout and the device pieces shared by training and inference.
//
// Inputs: x0 = 4 (S/K - 1) (moneyness), x1 = tau/T (time to expiry).
// Output: continuation value / K.  Master parameters are FP32; the 64x64
// layer runs on the tensor cores with BF16 operands (weights and
// activations) and FP32 accumulation; layers 1 and 3 and the GELUs run on the
// CUDA cores in FP32.  GELU is the tanh form
//     gelu(z) = z/2 (1 + tanh(c (z + 0.044715 z^3))),  c = sqrt(2/pi),
// with tanh.approx.f32.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mlp_layout.hpp"

namespace mcdg {
namespace mlp {

constexpr float kGeluC = 0.7978845608028654f;

__device__ __forceinline__ float tanh_approx(float x) {
    float r;
    asm("tanh.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// gelu(z); t receives the tanh value for the derivative.
// Evaluated as u = z (c + c 0.044715 z^2), h = z/2, gelu = h + h t: five
// FP32 operations and one MUFU tanh.
__device__ __forceinline__ float gelu(float z, float& t) {
    constexpr float kC3 = kGeluC * 0.044715f;
    t = tanh_approx(z * __fmaf_rn(z * z, kC3, kGeluC));
    const float h = 0.5f * z;
    return __fmaf_rn(h, t, h);
}

__device__ __forceinline__ float gelu_grad(float z, float t) {
    const float du = kGeluC * __fmaf_rn(3.0f * 0.044715f, z * z, 1.0f);
    return __fmaf_rn(0.5f * z * (1.0f - t * t), du, 0.5f * (1.0f + t));
}

}  // namespace mlp
}  // namespace mcdg
