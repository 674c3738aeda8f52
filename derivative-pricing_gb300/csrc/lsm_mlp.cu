// lsm_mlp.cu -- learned continuation values for Longstaff-Schwartz.
//
// In place of the Laguerre least-squares fit of src/pricers/lsm.cpp:88-108,
// the regression basis is *learned*: a 2 -> 64 -> 64 -> 1 GELU network
// (mlp.cuh) of (4 (S/K - 1), tau/T) is trained with Adam on in-the-money paths
// from the simulator (target: time value = (discounted cash flow - exercise
// value)/K), and its 64 last-layer features plus a bias become the regression
// basis.  At every exercise date the output layer is then fitted exactly, by
// ridge least squares over *all* in-the-money paths of that date (like the
// reference's QR fit, but on 65 learned functions instead of 4 Laguerre
// ones); exercise where the predicted time value is negative.
//
// Kernels (BF16 operands K-major in shared memory, FP32 accumulators in
// tensor memory; umma.cuh):
//   lsm_mlp_train   one CTA per contract: Adam steps on 128-sample tiles.  Per
//                   step the 64x64 layer runs three tcgen05 MMA groups --
//                   forward Z2 = H1 W2^T (4 x K16), input gradient dH1 = dZ2 W2
//                   (4 x K16), weight gradient dW2 = dZ2^T H1 (8 x K16, M padded
//                   to 128 with zero rows) -- and the CUDA cores do layers 1 and
//                   3, the GELUs and the fixed-order reductions.
//   lsm_mlp_nodes, lsm_mlp_binned, lsm_mlp_gram_slices (lsm_mlp_nodes.cu)
//                   the fit of every date on node tables: the network at 512
//                   values of ln(S/K) on the tensor core, paths binned with
//                   exact integer moments, the Gram matrix of
//                   [features | 1 | target] from the moments.
//   lsm_mlp_pass    one CTA per group of chunks: replays of given networks
//                   (terminal step included) with the network evaluated
//                   path by path (Z2 = H1 W2^T on the tensor core).
//   lsm_mlp_solve   one CTA per contract: scaled ridge Cholesky solve (65 x 65,
//                   FP32 factor, FP64-residual refinement) for the output
//                   layer of that date, then the date's continuation table
//                   at the nodes for the next iteration's exercise test.
//   mlp_grad_kernel / mlp_forward_kernel / umma_selftest_kernel   checks.
//
// Every mbarrier wait is bounded (umma.cuh); on a timeout the kernel records
// an error code, waits once more (bounded) for its MMAs, frees its tensor
// memory and returns.
//
// nvcc-flags: --fmad=false
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "cp_async.cuh"
#include "device_common.cuh"
#include "lsm.hpp"
#include "lsm_mlp_dev.hpp"
#include "mlp.cuh"
#include "umma.cuh"

namespace mcdg {

using namespace mlp;

namespace {

constexpr uint32_t kIdesc = umma::idesc_bf16(128, 64);
constexpr int kRow = 65;  // scratch row stride in floats (65: bank-conflict free)
constexpr int kTrainThreads = 256;  // two threads per sample of a 128-sample tile

struct __align__(1024) TrainSmem {
    __nv_bfloat16 h1[128 * 64];     // A [sample][in]    K = 64
    __nv_bfloat16 h1t[64 * 128];    // B [in][sample]    K = 128
    __nv_bfloat16 dz2[128 * 64];    // A [sample][out]   K = 64
    __nv_bfloat16 dz2t[128 * 128];  // A [out][sample]   K = 128, rows 64..127 zero
    __nv_bfloat16 w2[64 * 64];      // B [out][in]       K = 64
    __nv_bfloat16 w2t[64 * 64];     // B [in][out]       K = 64
    float scratch[128 * kRow];      // per-sample FP32 rows (padded: conflict-free)
    float p[kParamStride];          // master parameters
    float m[kParamStride];          // Adam first moment
    float v[kParamStride];          // Adam second moment
    float g[384];                   // reduced gradients: W1 0..127, b1 128..191, b2 192..255, W3 256..319, b3 320
    float x0[128], x1[128], y[128], w[128], dy[128];
    uint64_t mbar;
    uint32_t tmem_base;
    float loss;
};

struct __align__(1024) InferSmem {
    __nv_bfloat16 h1[128 * 64];
    __nv_bfloat16 w2[64 * 64];
    float p[kParamStride];
    uint64_t mbar;
    uint32_t tmem_base;
};

__device__ __forceinline__ __nv_bfloat16* at(__nv_bfloat16* base, int r, int k, int kcols) {
    return reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(base) + umma::kmajor_offset(r, k, kcols));
}

__device__ __forceinline__ uint64_t desc(const void* p, uint32_t sbo, int kstep) {
    return umma::smem_desc(umma::smem_u32(p) + static_cast<uint32_t>(kstep) * 256u, 128u, sbo);
}

// Refreshes the BF16 copies of W2 (row `r` of W2 and column `r` of W2^T).
__device__ __forceinline__ void refresh_w2_row(TrainSmem& S, int r) {
    for (int j = 0; j < 64; j += 2) {
        const __nv_bfloat162 pr = __floats2bfloat162_rn(S.p[kW2 + r * 64 + j], S.p[kW2 + r * 64 + j + 1]);
        *reinterpret_cast<__nv_bfloat162*>(at(S.w2, r, j, 64)) = pr;
        *at(S.w2t, j, r, 64) = pr.x;
        *at(S.w2t, j + 1, r, 64) = pr.y;
    }
}

// Adam with the bias corrections passed as reciprocals (ic1 = 1 / (1 - 0.9^t),
// ic2 = 1 / (1 - 0.999^t)).
__device__ __forceinline__ float adam(float& p, float& m, float& v, float g, float lr, float ic1, float ic2) {
    m = 0.9f * m + 0.1f * g;
    v = 0.999f * v + 0.001f * g * g;
    const float mh = m * ic1, vh = v * ic2;
    p -= lr * mh / (sqrtf(vh) + 1e-8f);
    return p;
}

// One forward/backward pass over the 128-sample tile staged in S.x0/x1/y/w
// (n_eff = number of samples with weight > 0), then (optionally) an Adam
// update.  grad_out, when given, receives the full gradient in parameter
// layout.  Returns false on an MMA timeout.  kTrainThreads threads: thread s
// serves sample s mod 128 and hidden units 32 h .. 32 h + 31 (h = s / 128);
// warp w reads the tensor-memory lanes 32 (w mod 4) .. + 31 (its samples).
__device__ bool train_step(TrainSmem& S, uint32_t tm, uint32_t& phase, int n_eff, bool update, float lr,
                           int t_adam, float* grad_out, uint32_t* err) {
    const int s = threadIdx.x;
    const int warp = s >> 5;
    const int q = s & 127, half = s >> 7;
    const int lanes = 32 * (warp & 3);
    const int j0 = 32 * half;
    const float inv_n = 1.0f / static_cast<float>(n_eff > 0 ? n_eff : 1);
    // ---- layer 1 (CUDA cores) -> H1 (BF16, both layouts)
    {
        const float x0 = S.x0[q], x1 = S.x1[q];
        for (int j = j0; j < j0 + 32; j += 2) {
            float t;
            const float za = __fmaf_rn(S.p[kW1 + 2 * j], x0, __fmaf_rn(S.p[kW1 + 2 * j + 1], x1, S.p[kB1 + j]));
            const float zb = __fmaf_rn(S.p[kW1 + 2 * j + 2], x0, __fmaf_rn(S.p[kW1 + 2 * j + 3], x1, S.p[kB1 + j + 1]));
            const __nv_bfloat162 hp = __floats2bfloat162_rn(gelu(za, t), gelu(zb, t));
            *reinterpret_cast<__nv_bfloat162*>(at(S.h1, q, j, 64)) = hp;
            *at(S.h1t, j, q, 128) = hp.x;
            *at(S.h1t, j + 1, q, 128) = hp.y;
        }
    }
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    if (s == 0) {
        umma::fence_after_sync();
        for (int kk = 0; kk < 4; ++kk)
            umma::mma_bf16(tm, desc(S.h1, 1024, kk), desc(S.w2, 1024, kk), kIdesc, kk > 0);
        umma::mma_commit(&S.mbar);
    }
    const bool ok2 = __syncthreads_and(umma::mbar_wait(&S.mbar, phase, err, 2));
    if (!ok2) return false;
    phase ^= 1u;
    umma::fence_after_sync();
    // ---- layer 2 epilogue, layer 3 (each half's partial sum), loss
    float yh = half == 0 ? S.p[kB3] : 0.0f;
    for (int c = 2 * half; c < 2 * half + 2; ++c) {
        float zz[16];
        umma::tmem_ld16(umma::tmem_addr(tm, lanes, c * 16), zz);
        for (int u = 0; u < 16; ++u) {
            const int j = c * 16 + u;
            float t;
            const float h = gelu(zz[u] + S.p[kB2 + j], t);
            yh = __fmaf_rn(S.p[kW3 + j], h, yh);
            S.scratch[q * kRow + j] = h;
        }
    }
    if (half == 1) S.scratch[q * kRow + 64] = yh;  // column 64 of a scratch row is padding
    __syncthreads();
    float diff = 0.0f;
    if (half == 0) {
        diff = (yh + S.scratch[q * kRow + 64]) - S.y[q];
        S.dy[q] = S.w[q] > 0.0f ? 2.0f * diff * inv_n : 0.0f;
    }
    __syncthreads();
    const float dy = S.dy[q];
    // column sums over the 128 samples: four interleaved partial sums per
    // thread, added in a fixed order (short dependency chains)
    if (s < 64) {
        float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 4
        for (int r = 0; r < 128; r += 4)
#pragma unroll
            for (int u = 0; u < 4; ++u) a[u] = __fmaf_rn(S.dy[r + u], S.scratch[(r + u) * kRow + s], a[u]);
        S.g[256 + s] = (a[0] + a[1]) + (a[2] + a[3]);  // dW3
    } else if (s < 96) {  // db3: one warp
        const int l = s & 31;
        float a = (S.dy[l] + S.dy[l + 32]) + (S.dy[l + 64] + S.dy[l + 96]);
#pragma unroll
        for (int w = 16; w >= 1; w >>= 1) a += __shfl_xor_sync(0xffffffffu, a, w);
        if (l == 0) S.g[320] = a;
    }
    __syncthreads();
    // ---- back through GELU to dZ2 (BF16, both layouts) and its FP32 rows
    for (int c = 2 * half; c < 2 * half + 2; ++c) {
        float zz[16];
        umma::tmem_ld16(umma::tmem_addr(tm, lanes, c * 16), zz);
        for (int u = 0; u < 16; u += 2) {
            const int j = c * 16 + u;
            float ta, tb;
            const float za = zz[u] + S.p[kB2 + j], zb = zz[u + 1] + S.p[kB2 + j + 1];
            gelu(za, ta);
            gelu(zb, tb);
            const float da = dy * S.p[kW3 + j] * gelu_grad(za, ta);
            const float db = dy * S.p[kW3 + j + 1] * gelu_grad(zb, tb);
            S.scratch[q * kRow + j] = da;
            S.scratch[q * kRow + j + 1] = db;
            const __nv_bfloat162 dp = __floats2bfloat162_rn(da, db);
            *reinterpret_cast<__nv_bfloat162*>(at(S.dz2, q, j, 64)) = dp;
            *at(S.dz2t, j, q, 128) = dp.x;
            *at(S.dz2t, j + 1, q, 128) = dp.y;
        }
    }
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    if (s == 0) {
        umma::fence_after_sync();
        for (int kk = 0; kk < 4; ++kk)  // dH1 = dZ2 W2
            umma::mma_bf16(tm + 64, desc(S.dz2, 1024, kk), desc(S.w2t, 1024, kk), kIdesc, kk > 0);
        for (int kk = 0; kk < 8; ++kk)  // dW2 = dZ2^T H1 (rows 64..127 of A are zero)
            umma::mma_bf16(tm + 128, desc(S.dz2t, 2048, kk), desc(S.h1t, 2048, kk), kIdesc, kk > 0);
        umma::mma_commit(&S.mbar);
    }
    if (s < 64) {  // db2 while the tensor core runs
        float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 4
        for (int r = 0; r < 128; r += 4)
#pragma unroll
            for (int u = 0; u < 4; ++u) a[u] += S.scratch[(r + u) * kRow + s];
        S.g[192 + s] = (a[0] + a[1]) + (a[2] + a[3]);
    }
    const bool ok3 = __syncthreads_and(umma::mbar_wait(&S.mbar, phase, err, 3));
    if (!ok3) return false;
    phase ^= 1u;
    umma::fence_after_sync();
    __syncthreads();
    // ---- dH1 -> dZ1 (through GELU), FP32 rows
    {
        const float x0 = S.x0[q], x1 = S.x1[q];
        for (int c = 2 * half; c < 2 * half + 2; ++c) {
            float dd[16];
            umma::tmem_ld16(umma::tmem_addr(tm, lanes, 64 + c * 16), dd);
            for (int u = 0; u < 16; ++u) {
                const int j = c * 16 + u;
                float t;
                const float z = __fmaf_rn(S.p[kW1 + 2 * j], x0, __fmaf_rn(S.p[kW1 + 2 * j + 1], x1, S.p[kB1 + j]));
                gelu(z, t);
                S.scratch[q * kRow + j] = dd[u] * gelu_grad(z, t);
            }
        }
    }
    __syncthreads();
    if (s < 192) {  // db1, dW1[.][0], dW1[.][1]: one sum per thread
        const int j = s & 63, kind = s >> 6;
        const float* xs = kind == 1 ? S.x0 : S.x1;
        float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 4
        for (int r = 0; r < 128; r += 4)
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const float d = S.scratch[(r + u) * kRow + j];
                a[u] = kind == 0 ? a[u] + d : __fmaf_rn(d, xs[r + u], a[u]);
            }
        const float sum = (a[0] + a[1]) + (a[2] + a[3]);
        if (kind == 0) S.g[128 + j] = sum;
        else S.g[2 * j + kind - 1] = sum;
    }
    const float c1 = 1.0f / (1.0f - powf(0.9f, static_cast<float>(t_adam)));
    const float c2 = 1.0f / (1.0f - powf(0.999f, static_cast<float>(t_adam)));
    // ---- dW2 rows from tensor memory (lanes 0..63 = output neurons, readable
    // by warps 0, 1, 4 and 5; each takes 32 of the 64 columns), staged in shared
    // memory so that every thread shares the 4096 Adam updates: the FP32 copy
    // goes into the first half of dz2t (rows 0..63 of dZ2^T, whose MMA has
    // completed; the next step rewrites them)
    float* stage = reinterpret_cast<float*>(S.dz2t);
    if ((warp & 3) < 2) {
        const int r = lanes + (s & 31);  // output neuron
        for (int c = 2 * half; c < 2 * half + 2; ++c) {
            float dw[16];
            umma::tmem_ld16(umma::tmem_addr(tm, lanes, 128 + c * 16), dw);
#pragma unroll
            for (int u = 0; u < 16; ++u) stage[r * 64 + ((c * 16 + u) ^ (r & 31))] = dw[u];  // XOR swizzle
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    // consecutive threads take consecutive parameters: the parameter and moment
    // arrays are read and written without bank conflicts
    for (int i = s; i < 64 * 64; i += kTrainThreads) {
        const int row = i >> 6, col = i & 63;
        const float g = stage[row * 64 + (col ^ (row & 31))];
        const int idx = kW2 + i;
        if (grad_out) grad_out[idx] = g;
        if (update) adam(S.p[idx], S.m[idx], S.v[idx], g, lr, c1, c2);
    }
    // ---- the small parameters
    for (int u = s; u < 321; u += kTrainThreads) {
        int idx;
        if (u < 128) idx = kW1 + u;
        else if (u < 192) idx = kB1 + (u - 128);
        else if (u < 256) idx = kB2 + (u - 192);
        else if (u < 320) idx = kW3 + (u - 256);
        else idx = kB3;
        if (grad_out) grad_out[idx] = S.g[u];
        if (update) adam(S.p[idx], S.m[idx], S.v[idx], S.g[u], lr, c1, c2);
    }
    __syncthreads();
    if (update && s < 64) refresh_w2_row(S, s);
    // loss of the tile (before the update)
    if (half == 0) S.scratch[q] = S.w[q] > 0.0f ? diff * diff * inv_n : 0.0f;  // scratch rows are free again
    __syncthreads();
    if (s < 32) {
        float l = (S.scratch[s] + S.scratch[s + 32]) + (S.scratch[s + 64] + S.scratch[s + 96]);
#pragma unroll
        for (int w = 16; w >= 1; w >>= 1) l += __shfl_xor_sync(0xffffffffu, l, w);
        if (s == 0) S.loss = l;
    }
    __syncthreads();
    return true;
}

__device__ void train_setup(TrainSmem& S) {
    const int s = threadIdx.x;
    if (s == 0) umma::mbar_init(&S.mbar, 1);
    // dZ2^T rows 64..127 stay zero (M padding of the weight-gradient MMA)
    for (int i = s; i < 128 * 128 / 2; i += kTrainThreads) reinterpret_cast<uint32_t*>(S.dz2t)[i] = 0u;
    if ((s >> 5) == 0) umma::tmem_alloc(&S.tmem_base, 256);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
}

__device__ void train_teardown(TrainSmem& S, uint32_t phase, bool ok, uint32_t* err) {
    if (!ok) {
        // bounded second wait for any MMA still in flight, then release TMEM
        umma::mbar_wait(&S.mbar, phase, err, 4);
    }
    umma::fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) umma::tmem_dealloc(S.tmem_base, 256);
}

// Deterministic initial weights: He-scaled normals from Philox (stream 7).
__device__ void init_params(float* p, uint64_t seed) {
    const PhiloxKeys k = philox_keys(seed ^ 0x6a09e667f3bcc909ull);
    for (int i = threadIdx.x; i < kParamStride; i += blockDim.x) {
        float scale = 0.0f;
        if (i < kB1) scale = 1.0f;                 // W1: fan-in 2
        else if (i >= kW2 && i < kB2) scale = 0.1767767f;  // W2: sqrt(2/64)
        else if (i >= kW3 && i < kB3) scale = 0.125f;      // W3
        float val = 0.0f;
        if (scale != 0.0f) {
            const PhiloxPath pp = philox_path(static_cast<uint64_t>(i), 7u, k);
            val = scale * normal_from_bits_f32(philox_word0(pp, 0u, k));
        }
        p[i] = val;
    }
}

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

// Cash flows: FP64 on the FP64 path, FP32 (in the same buffer) on the FP32
// path, as the QR kernels keep them (lsm.cu).
template <int PREC>
__device__ __forceinline__ double cf_load(const double* cf, uint64_t idx) {
    if (PREC == 0) return cf[idx];
    return static_cast<double>(reinterpret_cast<const float*>(cf)[idx]);
}
template <int PREC>
__device__ __forceinline__ void cf_store(double* cf, uint64_t idx, double v) {
    if (PREC == 0) cf[idx] = v;
    else reinterpret_cast<float*>(cf)[idx] = static_cast<float>(v);
}

template <int PREC>
__device__ __forceinline__ double path_s(const void* store, uint64_t idx) {
    if (PREC == 0) return static_cast<const double*>(store)[idx];
    return static_cast<double>(static_cast<const float*>(store)[idx]);
}

// The path behind sample s (of 128) of training step st at a date.
__device__ __forceinline__ uint64_t train_sample_path(const LsmDev& c, int date, int st, int s) {
    const uint32_t h = mix32(static_cast<uint32_t>(c.seed) * 0x9E3779B1u ^
                             mix32((static_cast<uint32_t>(date) << 20) ^ (static_cast<uint32_t>(st) << 7) ^ s));
    return static_cast<uint64_t>(h) % c.path_count;
}

// ---------------------------------------------------------------------------
// Training samples of the first (latest) regression date, drawn without the
// path store: sample s of step st is path i of the contract, regenerated from
// its Philox stream up to date n with the forward simulation's arithmetic
// (gbm_log_step_f32 / gbm_step_f64), so its spot at date n-1 and its terminal
// cash flow (the payoff at date n, discounted once, rounded as the cash-flow
// store holds it) equal what the stores will hold bit for bit.  The training
// then needs neither the forward simulation nor the terminal step and runs
// alongside them.  CTAs per contract over the steps (grid-stride), one thread
// per sample; 2 KB of device memory per step and contract.
// ---------------------------------------------------------------------------
template <int PREC>
__global__ void __launch_bounds__(128)
    lsm_mlp_train_samples(const LsmDev* __restrict__ cs, int c_first, int n_contracts, int steps,
                          double* __restrict__ pre_s, double* __restrict__ pre_cf) {
    const int ci = c_first + static_cast<int>(blockIdx.x), s = threadIdx.x;
    if (ci >= n_contracts) return;
    const LsmDev c = cs[ci];
    const int n = c.n_steps;
    if (n - 1 < 1 || c.path_count == 0) return;  // no regression date, as the trainer
    for (int st = static_cast<int>(blockIdx.y); st < steps; st += static_cast<int>(gridDim.y)) {
        const uint64_t i = train_sample_path(c, n - 1, st, s);
        const PhiloxKeys key = philox_keys(c.seed);
        const PhiloxPath pp = philox_path(i, 0u, key);
        double s_prev = 0.0, s_last = 0.0;
        if (PREC == 0) {
            double sp = c.spot;
            for (int d = 0; d < n; ++d) {
                const double z = normal_from_bits_f64(philox_word0(pp, static_cast<uint32_t>(d), key));
                sp = gbm_step_f64(sp, z, c.drift, c.vs);
                if (d == n - 2) s_prev = sp;
            }
            s_last = sp;
        } else {
            const float mu = static_cast<float>(c.drift), sg = static_cast<float>(c.vs), s0 = static_cast<float>(c.spot);
            float x = 0.0f;
            for (int d = 0; d < n; ++d) {
                const float z = normal_from_bits_f32(philox_word0(pp, static_cast<uint32_t>(d), key));
                x = gbm_log_step_f32(x, z, mu, sg);
                if (d == n - 2) s_prev = static_cast<double>(gbm_spot_f32(s0, x));
            }
            s_last = static_cast<double>(gbm_spot_f32(s0, x));
        }
        // the terminal step's cash flow, in the path precision as the binned pass
        // computes it at k = 0 (lsm_mlp_binned: payoff, then one discount)
        double v;
        if (PREC == 0) {
            const double phi = c.type == 0 ? 1.0 : -1.0;
            const double x = phi * (s_last - c.strike);
            v = (x > 0.0 ? x : 0.0) * c.disc;
        } else {
            const float x = c.phi_f * (static_cast<float>(s_last) - c.strike_f);
            v = static_cast<double>((x > 0.0f ? x : 0.0f) * c.disc_f);
        }
        const size_t idx = (static_cast<size_t>(ci) * steps + st) * 128 + s;
        pre_s[idx] = s_prev;
        pre_cf[idx] = v;
    }
}

// ---------------------------------------------------------------------------
// per-contract trainer for date n - k - 1
// ---------------------------------------------------------------------------
template <int PREC>
__global__ void __launch_bounds__(kTrainThreads, 1)
    lsm_mlp_train(int k, const LsmDev* __restrict__ cs, int c_first, int n_contracts, const void* __restrict__ store,
                  const double* __restrict__ cf, float* __restrict__ nets, float* __restrict__ snaps,
                  int* __restrict__ snap_ok, int* __restrict__ adam_t, MlpConfig cfg,
                  const double* __restrict__ pre_s, const double* __restrict__ pre_cf, uint32_t* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
    const int ci = c_first + static_cast<int>(blockIdx.x);
    if (ci >= n_contracts) return;
    const LsmDev c = cs[ci];
    const int n = c.n_steps;
    const int date = n - k - 1;
    if (date < 1 || c.path_count == 0) return;  // nothing to sample (the host rejects 0 paths)
    const int s = threadIdx.x;
    float* net = nets + static_cast<size_t>(ci) * 3 * kParamStride;
    if (k == 0) {
        init_params(S.p, c.seed);
        for (int i = s; i < kParamStride; i += kTrainThreads) {
            S.m[i] = 0.0f;
            S.v[i] = 0.0f;
        }
    } else {
        for (int i = s; i < kParamStride; i += kTrainThreads) {
            S.p[i] = net[i];
            S.m[i] = net[kParamStride + i];
            S.v[i] = net[2 * kParamStride + i];
        }
    }
    train_setup(S);
    if (s < 64) refresh_w2_row(S, s);
    __syncthreads();
    const uint32_t tm = S.tmem_base;
    uint32_t phase = 0;
    int t = k == 0 ? 0 : adam_t[ci];
    const int steps = k == 0 ? cfg.steps_first : cfg.steps;
    const float lr = k == 0 ? cfg.lr_first : cfg.lr;
    const double inv_k = 1.0 / c.strike;
    const float x1 = static_cast<float>(n - date) / static_cast<float>(n);
    bool ok = true;
    // this thread's sample of step st: the path's spot at the date and its cash
    // flow, drawn beforehand (lsm_mlp_train_samples) or read from the stores
    const bool drawn = k == 0 && pre_s != nullptr;
    auto sample = [&](int st, double& sv, double& cfv) {
        if (drawn) {
            const size_t idx = (static_cast<size_t>(ci) * steps + st) * 128 + s;
            sv = pre_s[idx];
            cfv = pre_cf[idx];
            return;
        }
        const uint64_t i = train_sample_path(c, date, st, s);
        sv = path_s<PREC>(store, c.s_offset + static_cast<uint64_t>(date - 1) * c.path_count + i);
        cfv = cf_load<PREC>(cf, c.cf_offset + i);
    };
    double sv_next = 0.0, cf_next = 0.0;
    if (steps > 0 && s < 128) sample(0, sv_next, cf_next);
    const bool sampler = s < 128;  // thread s < 128 draws sample s of each tile
    for (int st = 0; st < steps && ok; ++st) {
        const double sv = sv_next, cfv = cf_next;
        // the next step's loads, in flight during this step
        if (sampler && st + 1 < steps) sample(st + 1, sv_next, cf_next);
        const double ex = (c.type == 0 ? 1.0 : -1.0) * (sv - c.strike);
        const bool itm = sampler && ex > 0.0;
        if (sampler) {
            S.x0[s] = static_cast<float>(4.0 * (sv * inv_k - 1.0));
            S.x1[s] = x1;
            // Target: time value (continuation minus exercise value) over K.  The
            // decision only needs its sign, and it is an order of magnitude
            // smaller than the continuation value itself, so the network's
            // relative error costs far fewer wrong decisions.
            S.y[s] = itm ? static_cast<float>((cfv - ex) * inv_k) : 0.0f;
            S.w[s] = itm ? 1.0f : 0.0f;
        }
        const int n_eff = __syncthreads_count(itm);
        ++t;
        ok = train_step(S, tm, phase, n_eff, true, lr, t, nullptr, err);
    }
    // persist the network (features and output layer) for the next dates
    for (int i = s; i < kParamStride; i += kTrainThreads) {
        net[i] = S.p[i];
        net[kParamStride + i] = S.m[i];
        net[2 * kParamStride + i] = S.v[i];
    }
    if (s == 0) adam_t[ci] = t;
    train_teardown(S, phase, ok, err);
}

// ---------------------------------------------------------------------------
// Per-path step over a group of chunks: exercise at date e with the network of
// that date evaluated path by path (layer 1 on the CUDA cores, Z2 = H1 W2^T on
// the tensor core), discount, and the cash-flow update or, at e = 1, the final
// Welford partial.  Replays given networks (mcd_lsm_reprice_mlp), terminal
// step (k = 0: no exercise) included; the fit itself, terminal step included,
// runs on node tables (lsm_mlp_nodes.cu).
// ---------------------------------------------------------------------------
constexpr int kGramDim = 66;  // 64 features, bias, target

struct __align__(1024) PassSmem {
    __nv_bfloat16 h1d[128 * 64];    // network input tile (S at date e)
    __nv_bfloat16 w2d[64 * 64];
    float pd[kParamStride - 4096];  // network without W2: W1 b1 | b2 W3 b3
    uint64_t mbar;
    uint32_t tmem_base;
};

// Copies a network into shared memory: the small parameters as FP32 (W2's
// slot removed) and W2 as the BF16 K-major MMA operand.
__device__ void load_net(const float* __restrict__ net, float* small, __nv_bfloat16* w2) {
    const int s = threadIdx.x;
    for (int i = s; i < kW2; i += 128) small[i] = net[i];
    for (int i = s; i < kParams - kB2; i += 128) small[kW2 + i] = net[kB2 + i];
    for (int i = s; i < 64 * 32; i += 128) {  // W2 [out][in] read in order (coalesced), pairs to BF16
        const int r = i >> 5, j = 2 * (i & 31);
        const float2 w = *reinterpret_cast<const float2*>(net + kW2 + r * 64 + j);
        *reinterpret_cast<__nv_bfloat162*>(at(w2, r, j, 64)) = __floats2bfloat162_rn(w.x, w.y);
    }
}

// Small-parameter offsets inside PassSmem::pd.
constexpr int sW1 = kW1, sB1 = kB1, sB2 = kW2, sW3 = kW2 + (kW3 - kB2), sB3 = kW2 + (kB3 - kB2);

__device__ __forceinline__ void layer1_row(const float* small, float x0, float x1, __nv_bfloat16* h1, int s) {
    for (int j = 0; j < 64; j += 2) {
        float t;
        const float za = __fmaf_rn(small[sW1 + 2 * j], x0, __fmaf_rn(small[sW1 + 2 * j + 1], x1, small[sB1 + j]));
        const float zb = __fmaf_rn(small[sW1 + 2 * j + 2], x0, __fmaf_rn(small[sW1 + 2 * j + 3], x1, small[sB1 + j + 1]));
        *reinterpret_cast<__nv_bfloat162*>(at(h1, s, j, 64)) = __floats2bfloat162_rn(gelu(za, t), gelu(zb, t));
    }
}

template <int PREC>
__global__ void __launch_bounds__(128)
    lsm_mlp_pass(int k, const LsmDev* __restrict__ cs, const uint32_t* __restrict__ group_contract,
                 uint32_t g_first, uint32_t total_groups, const void* __restrict__ store, double* __restrict__ cf,
                 const float* __restrict__ snaps, const int* __restrict__ snap_ok, Welford* __restrict__ final_part,
                 uint32_t* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    PassSmem& S = *reinterpret_cast<PassSmem*>(smem_raw);
    __shared__ Welford swf[4];
    const uint32_t g = g_first + blockIdx.x;
    if (g >= total_groups) return;
    const uint32_t ci = group_contract[g];
    const LsmDev c = cs[ci];
    const int n = c.n_steps;
    const int e = n - k;
    if (e < 1) return;
    const bool init = k == 0;
    const bool last = e == 1;
    const bool exercise = k > 0 && e <= n - 1 && snap_ok[c.reg_offset + e] == 1;
    const int s = threadIdx.x, warp = s >> 5;
    const double phi = c.type == 0 ? 1.0 : -1.0;
    const double inv_k = 1.0 / c.strike;
    if (exercise) {
        load_net(snaps + (static_cast<size_t>(c.reg_offset) + e) * kParamStride, S.pd, S.w2d);
        if (s == 0) umma::mbar_init(&S.mbar, 1);
        if (warp == 0) umma::tmem_alloc(&S.tmem_base, 64);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
    }
    const uint32_t tm = exercise ? S.tmem_base : 0u;
    uint32_t phase = 0;
    bool ok = true;
    const float x1e = static_cast<float>(n - e) / static_cast<float>(n);
    const uint32_t gl = g - c.group_begin;
    const uint32_t chunk0 = gl * c.group_chunks;
    const uint32_t chunk1 = min(c.n_chunks, chunk0 + c.group_chunks);
    Welford w{0ull, 0.0, 0.0};
    for (uint32_t ch = chunk0; ch < chunk1; ++ch) {
        for (int tile = 0; tile < kLsmChunk / 128; ++tile) {
            const uint64_t i = static_cast<uint64_t>(ch) * kLsmChunk + tile * 128 + s;
            const bool live = i < c.path_count;
            double v = 0.0, ex_e = 0.0;
            if (live) {
                if (init) {
                    const double sT = path_s<PREC>(store, c.s_offset + static_cast<uint64_t>(n - 1) * c.path_count + i);
                    const double x = phi * (sT - c.strike);
                    v = x > 0.0 ? x : 0.0;
                } else {
                    v = cf_load<PREC>(cf, c.cf_offset + i);
                }
            }
            if (exercise) {
                float x0 = 0.0f;
                if (live) {
                    const double se = path_s<PREC>(store, c.s_offset + static_cast<uint64_t>(e - 1) * c.path_count + i);
                    const double xx = phi * (se - c.strike);
                    ex_e = xx > 0.0 ? xx : 0.0;
                    x0 = static_cast<float>(4.0 * (se * inv_k - 1.0));
                }
                layer1_row(S.pd, x0, x1e, S.h1d, s);
                umma::fence_smem_to_async();
                umma::fence_before_sync();
                __syncthreads();
                if (s == 0) {
                    umma::fence_after_sync();
                    for (int kk = 0; kk < 4; ++kk)
                        umma::mma_bf16(tm, desc(S.h1d, 1024, kk), desc(S.w2d, 1024, kk), kIdesc, kk > 0);
                    umma::mma_commit(&S.mbar);
                }
                ok = __syncthreads_and(ok && umma::mbar_wait(&S.mbar, phase, err, 11));
                phase ^= 1u;
                umma::fence_after_sync();
                float yhat = S.pd[sB3];
                for (int cc = 0; cc < 4; ++cc) {
                    float zz[16];
                    umma::tmem_ld16(umma::tmem_addr(tm, 32 * warp, cc * 16), zz);
                    for (int q = 0; q < 16; ++q) {
                        float t;
                        yhat = __fmaf_rn(S.pd[sW3 + cc * 16 + q], gelu(zz[q] + S.pd[sB2 + cc * 16 + q], t), yhat);
                    }
                }
                // predicted time value < 0: exercise
                if (live && ok && ex_e > 0.0 && yhat < 0.0f) v = ex_e;
                umma::fence_before_sync();
                __syncthreads();  // the input tile and the accumulator are reused by the next tile
            }
            if (live) {
                v *= c.disc;
                if (last) welford_add(w, v);
                else cf_store<PREC>(cf, c.cf_offset + i, v);
            }
        }
        if (last) {  // one final partial per chunk, fixed tree
            Welford r = welford_warp_reduce(w);
            if ((s & 31) == 0) swf[warp] = r;
            __syncthreads();
            if (s == 0) final_part[c.chunk_begin + ch] = welford_merge(welford_merge(swf[0], swf[1]), welford_merge(swf[2], swf[3]));
            __syncthreads();
            w = Welford{0ull, 0.0, 0.0};
        }
    }
    if (exercise) {
        if (!ok) umma::mbar_wait(&S.mbar, phase, err, 13);
        umma::fence_before_sync();
        __syncthreads();
        if (warp == 0) umma::tmem_dealloc(tm, 64);
    }
}

// ---------------------------------------------------------------------------
// output layer of date d = n - k - 1: ridge least squares on the Gram matrix
//
// The 64 GELU features are smooth functions of one state variable and are
// strongly collinear, and the Gram matrix is accumulated in FP32, so it is
// only positive semi-definite to a small fraction of its diagonal.  The
// regressors are therefore scaled to unit diagonal and a ridge of kRidge is
// added in those units; a pivot that still falls below half the ridge drops
// its regressor (coefficient 0) instead of failing the date.
//
// FP64 is slow on this part, so the solve works in FP32 and in pairs of FP32
// values (hi + lo, about 48 bits):
//   1. the bin slices' partials are summed in order into pairs (error-free
//      two-sums) and standardised as pairs;
//   2. one sweep of 65 steps, one barrier each, factors the FP32 matrix
//      A = L L^T (right-looking Cholesky) and at the same time applies the
//      same row operations to the identity, which leaves W = L^-1: both live
//      in registers as 4 x 4 blocks of their lower triangles, one block per
//      thread (153 + 153 blocks of the 68 x 68 padded matrices), and each
//      step broadcasts the pivot column of A and the pivot row of W through
//      shared memory;
//   3. x = W^T W b, then two steps of iterative refinement with residuals
//      b - A x in pairs (x kept as a pair): two matrix-vector products per
//      solve instead of two triangular substitutions of 65 dependent steps.
//
// snap_ok of the date: 1 = fitted, 2 = fewer than 4 in-the-money paths (no
// exercise at this date, as src/pricers/lsm.cpp does), 0 = failed.
// ---------------------------------------------------------------------------
constexpr float kRidge = 1e-3f;
constexpr int kM = kGramDim - 1;           // 65 regressors (64 features + bias)
constexpr int kNB = 17;                    // 4 x 4 blocks per side
constexpr int kPad = 4 * kNB;              // 68: the system padded with identity rows
constexpr int kTriBlocks = kNB * (kNB + 1) / 2;  // 153 blocks of a lower triangle
constexpr int kWBase = 160;                // first thread of the W role (a warp boundary)
constexpr int kSolveThreads = 320;         // A role 0..152, W role 160..312
constexpr size_t kSolveFeatBytes = sizeof(float) * kNodes * 64;  // the solve's copy of a feature table
static_assert(kTriBlocks <= kWBase && kWBase + kTriBlocks <= kSolveThreads && kWBase % 32 == 0, "solve roles");
static_assert(4 * kM <= kSolveThreads && kPad <= kSolveThreads, "four residual threads per row");

__device__ __forceinline__ int packed_index(int r, int q) {  // r <= q
    return r * kGramDim - r * (r - 1) / 2 + (q - r);
}
__device__ __forceinline__ int sym_index(int r, int q) { return r <= q ? packed_index(r, q) : packed_index(q, r); }

// pairs of floats: s + e = a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {  // |a| >= |b|
    s = a + b;
    e = b - (s - a);
}
// (h, l) + (bh, bl), renormalised
__device__ __forceinline__ void pair_add(float& h, float& l, float bh, float bl) {
    float s, e;
    two_sum(h, bh, s, e);
    e += l + bl;
    fast_two_sum(s, e, h, l);
}
// (h, l) * f for a float f
__device__ __forceinline__ void pair_scale(float h, float l, float f, float& oh, float& ol) {
    const float p = h * f;
    const float e = __fmaf_rn(h, f, -p) + l * f;
    fast_two_sum(p, e, oh, ol);
}

// Arrays read or written as float4 first: each is a multiple of 16 bytes.
struct __align__(16) SolveSmem {
    float panelA[2][kPad][4];                // pivot block column of A, double-buffered by block step
    float panelW[2][4][kPad];                // pivot block row of W, double-buffered by block step
    float lpan[kPad][4];                     // the factor's pivot columns of the block step, by row
    float ld4[4][4], inv4[4];                // the diagonal block's factor (strictly lower) and reciprocal pivots
    float part[kNB][kPad];                   // partial sums of the matrix-vector products
    float vb[kPad], vr[kPad];                // right-hand side (hi), residual
    float vz[kPad], vx[kPad];                // W v, W^T W v
    float xh[kPad], xl[kPad];                // the solution, a pair
    float bl[kPad];                          // low part of the right-hand side
    float sc[kPad];                          // scale of each regressor (1 / sqrt of its diagonal)
    float coef[kPad];                        // fitted W3, b3
    int drop[kPad];
    float gh[kGramPacked], gl[kGramPacked];  // the Gram matrix (then standardised), pairs; column 65 = rhs
    int bad;
    int few;
};
static_assert(kPad % 4 == 0, "float4 rows");

// Lower-triangular block t (row-major over the triangle) -> block row and column.
__device__ __forceinline__ void tri_block(int t, int& R, int& C) {
    R = 0;
    while ((R + 1) * (R + 2) / 2 <= t) ++R;
    C = t - R * (R + 1) / 2;
}

// The 4 x 4 diagonal block D of the pivot panel, factored: the strictly lower
// factor Ld and the reciprocal pivots inv (0 for a dropped pivot), with the
// same operations in the same order as one pivot at a time.
__device__ __forceinline__ void diag_factor(float (&a)[4][4], float (&Ld)[4][4], float (&inv)[4]) {
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
        const float dj = a[jj][jj];
        inv[jj] = dj >= 0.5f * kRidge ? rsqrtf(dj) : 0.0f;
#pragma unroll
        for (int i = jj + 1; i < 4; ++i) Ld[i][jj] = a[i][jj] * inv[jj];
#pragma unroll
        for (int i = jj + 1; i < 4; ++i)
#pragma unroll
            for (int c = jj + 1; c <= i; ++c) a[i][c] = __fmaf_rn(-Ld[i][jj], Ld[c][jj], a[i][c]);
    }
}

__device__ __forceinline__ void load_rows(const float (*rows)[4], int r0, float (&x)[4][4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float4 v = *reinterpret_cast<const float4*>(rows[r0 + i]);
        x[i][0] = v.x;
        x[i][1] = v.y;
        x[i][2] = v.z;
        x[i][3] = v.w;
    }
}

// Block step J of the sweep: pivots 4 J .. 4 J + 3.  The owners of block
// column J of A and of block row J of W published them (the panels) before
// the first barrier; one thread per row then factors the panel's diagonal
// block and derives its row of the factor's four pivot columns; after the
// second barrier every thread applies the rank-4 update to its block of A
// (C > J) or the four row operations to its block of W, and the owners of the
// next panels publish them.  Same operations, in the same order, as four
// steps of one pivot each.
__device__ __forceinline__ void chol_block(SolveSmem& S, int J, bool role_a, bool role_w, int R, int C,
                                           float (&m)[4][4], int s) {
    const int buf = J & 1;
    __syncthreads();
    if (s < kPad) {
        float dg[4][4], Ld[4][4] = {}, inv[4];
        load_rows(S.panelA[buf], 4 * J, dg);
        diag_factor(dg, Ld, inv);
        if (s == 0) {
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
                S.drop[4 * J + jj] = inv[jj] == 0.0f ? 1 : 0;
                S.inv4[jj] = inv[jj];
#pragma unroll
                for (int i = 0; i < 4; ++i) S.ld4[i][jj] = Ld[i][jj];
            }
        }
        if (s >= 4 * J + 4) {  // row s of the factor's pivot columns
            const float4 v = *reinterpret_cast<const float4*>(S.panelA[buf][s]);
            float p[4] = {v.x, v.y, v.z, v.w}, l[4];
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
                l[jj] = p[jj] * inv[jj];
#pragma unroll
                for (int c = jj + 1; c < 4; ++c) p[c] = __fmaf_rn(-l[jj], Ld[c][jj], p[c]);
            }
            *reinterpret_cast<float4*>(S.lpan[s]) = make_float4(l[0], l[1], l[2], l[3]);
        }
    }
    __syncthreads();
    if (role_a && C > J) {
        float lr[4][4], lc[4][4];
        load_rows(S.lpan, 4 * R, lr);
        load_rows(S.lpan, 4 * C, lc);
#pragma unroll
        for (int jj = 0; jj < 4; ++jj)
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int c = 0; c < 4; ++c) m[i][c] = __fmaf_rn(-lr[i][jj], lc[c][jj], m[i][c]);
    }
    if (role_w && R >= J && C <= J) {
        // block (J, C) of W after the four pivots
        float y[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float4 v = *reinterpret_cast<const float4*>(&S.panelW[buf][i][4 * C]);
            y[i][0] = v.x;
            y[i][1] = v.y;
            y[i][2] = v.z;
            y[i][3] = v.w;
        }
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            const float iv = S.inv4[jj];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                y[jj][c] = y[jj][c] * iv;
#pragma unroll
                for (int i = jj + 1; i < 4; ++i) y[i][c] = __fmaf_rn(-S.ld4[i][jj], y[jj][c], y[i][c]);
            }
        }
        if (R == J) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int c = 0; c < 4; ++c) m[i][c] = y[i][c];
        } else {
            float lr[4][4];
            load_rows(S.lpan, 4 * R, lr);
#pragma unroll
            for (int jj = 0; jj < 4; ++jj)
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int c = 0; c < 4; ++c) m[i][c] = __fmaf_rn(-lr[i][jj], y[jj][c], m[i][c]);
        }
    }
    // publish the next panels (every owner, updated or not)
    if (J + 1 < kNB) {
        if (role_a && C == J + 1)
#pragma unroll
            for (int i = 0; i < 4; ++i)
                *reinterpret_cast<float4*>(S.panelA[buf ^ 1][4 * R + i]) = make_float4(m[i][0], m[i][1], m[i][2], m[i][3]);
        if (role_w && R == J + 1)
#pragma unroll
            for (int i = 0; i < 4; ++i)
                *reinterpret_cast<float4*>(&S.panelW[buf ^ 1][i][4 * C]) = make_float4(m[i][0], m[i][1], m[i][2], m[i][3]);
    }
}

// out = W v (transpose = false) or W^T v (transpose = true), W in the W role's
// registers; the partial sums are added in a fixed order.
__device__ __forceinline__ void w_matvec(SolveSmem& S, bool role_w, int R, int C, const float (&m)[4][4], const float* v,
                                         float* out, bool transpose, int s) {
    if (role_w) {
        if (!transpose) {
            const float4 x = *reinterpret_cast<const float4*>(&v[4 * C]);
            float p[4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
                p[i] = __fmaf_rn(m[i][3], x.w, __fmaf_rn(m[i][2], x.z, __fmaf_rn(m[i][1], x.y, m[i][0] * x.x)));
            *reinterpret_cast<float4*>(&S.part[C][4 * R]) = make_float4(p[0], p[1], p[2], p[3]);
        } else {
            const float4 x = *reinterpret_cast<const float4*>(&v[4 * R]);
            float p[4];
#pragma unroll
            for (int c = 0; c < 4; ++c)
                p[c] = __fmaf_rn(m[3][c], x.w, __fmaf_rn(m[2][c], x.z, __fmaf_rn(m[1][c], x.y, m[0][c] * x.x)));
            *reinterpret_cast<float4*>(&S.part[R][4 * C]) = make_float4(p[0], p[1], p[2], p[3]);
        }
    }
    __syncthreads();
    if (s < kPad) {
        const int blk = s >> 2;
        float acc = 0.0f;
        if (!transpose) {
            for (int c = 0; c <= blk; ++c) acc += S.part[c][s];
        } else {
            for (int r = blk; r < kNB; ++r) acc += S.part[r][s];
        }
        out[s] = acc;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kSolveThreads)
    lsm_mlp_solve(int k, const LsmDev* __restrict__ cs, int c_first, int n_contracts, const float* __restrict__ gram_part,
                  const float* __restrict__ feats, float* __restrict__ nets, float* __restrict__ snaps,
                  int* __restrict__ snap_ok, float* __restrict__ etab) {
    __shared__ SolveSmem S;
    extern __shared__ __align__(16) float s_feat[];  // the date's feature table (kSolveFeatBytes, dynamic)
    const int ci = c_first + static_cast<int>(blockIdx.x);
    if (ci >= n_contracts) return;
    const LsmDev c = cs[ci];
    const int d = c.n_steps - k - 1;
    if (d < 1) return;
    const int s = threadIdx.x;
    // The date's feature table, for the continuation table at the end, copied
    // in while the fit runs: row i's 16-byte piece q at piece q ^ (i mod 8)
    // (the rows are 256 bytes apart; the XOR keeps eight rows' reads on
    // different banks).
    {
        const float* F = feats + (static_cast<size_t>(c.reg_offset) + d) * kNodes * 64;
        for (int u = s; u < kNodes * 16; u += kSolveThreads) {
            const int row = u >> 4, piece = u & 15;
            cp_async16(s_feat + row * 64 + 4 * (piece ^ (row & 7)), F + static_cast<size_t>(row) * 64 + 4 * piece);
        }
        cp_async_commit();
    }
    // The snapshot of date d: the current network (its output layer is
    // replaced by the fit below).
    float* net = nets + static_cast<size_t>(ci) * 3 * kParamStride;
    float* snap = snaps + (static_cast<size_t>(c.reg_offset) + d) * kParamStride;
    static_assert(kParamStride % 4 == 0 && kB3 == kW3 + 64, "snapshot layout");
    for (int i = s; i < kParamStride / 4; i += kSolveThreads)
        reinterpret_cast<float4*>(snap)[i] = reinterpret_cast<const float4*>(net)[i];
    // 1. the bin slices' partials, summed in order into pairs
    {
        const float* part = gram_part + static_cast<size_t>(ci) * kNodeSlices * kGramPacked;
        constexpr int kIters = (kGramPacked + kSolveThreads - 1) / kSolveThreads;
        float v[kIters][kNodeSlices];  // every load first, in flight together
#pragma unroll
        for (int u = 0; u < kIters; ++u) {
            const int p = s + u * kSolveThreads;
#pragma unroll
            for (int sl = 0; sl < kNodeSlices; ++sl)
                v[u][sl] = p < kGramPacked ? part[static_cast<size_t>(sl) * kGramPacked + p] : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < kIters; ++u) {
            const int p = s + u * kSolveThreads;
            float h = v[u][0], l = 0.0f;
#pragma unroll
            for (int sl = 1; sl < kNodeSlices; ++sl) {
                float e;
                two_sum(h, v[u][sl], h, e);
                l += e;
            }
            if (p < kGramPacked) fast_two_sum(h, l, S.gh[p], S.gl[p]);
        }
    }
    if (s == 0) S.bad = 0;
    __syncthreads();
    if (s == 0) S.few = !(S.gh[packed_index(64, 64)] + S.gl[packed_index(64, 64)] >= 4.0f) ? 1 : 0;
    if (s < kPad) {
        const float a = s < kM ? S.gh[packed_index(s, s)] : 0.0f;
        S.sc[s] = s < kM ? (a > 0.0f ? rsqrtf(a) : 0.0f) : (s == kM ? 1.0f : 0.0f);  // the rhs column keeps scale 1
    }
    __syncthreads();
    if (S.few) {
        if (s == 0) snap_ok[c.reg_offset + d] = 2;
        cp_async_wait_all();  // no copy outlives the CTA
        return;
    }
    // standardised pairs G_rq sc_r sc_q, plus the ridge on the diagonal (whose
    // standardised value is 1 to the rounding of sc, or 0 for a regressor that
    // is zero on every path)
    const float ridge_lo = static_cast<float>(1e-3 - static_cast<double>(kRidge));
    for (int e = s; e < kGramDim * kGramDim; e += kSolveThreads) {
        const int r = e / kGramDim, q = e - r * kGramDim;
        if (r > q) continue;
        const int p = packed_index(r, q);
        float h, l, th, tl;
        pair_scale(S.gh[p], S.gl[p], S.sc[r], th, tl);
        pair_scale(th, tl, S.sc[q], h, l);
        if (r == q && r < kM) pair_add(h, l, kRidge, ridge_lo);
        S.gh[p] = h;
        S.gl[p] = l;
    }
    __syncthreads();
    // 2. roles and blocks; the right-hand side; the first pivot column and row
    const bool role_a = s < kTriBlocks;
    const bool role_w = s >= kWBase && s < kWBase + kTriBlocks;
    int R = 0, C = 0;
    tri_block(role_a ? s : (role_w ? s - kWBase : 0), R, C);
    float m[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int r = 4 * R + i, cc = 4 * C + q;
            float v = 0.0f;
            if (role_a) v = (r < kM && cc < kM) ? S.gh[sym_index(r, cc)] : (r == cc ? 1.0f : 0.0f);
            else if (role_w) v = r == cc ? 1.0f : 0.0f;
            m[i][q] = v;
        }
    if (s < kPad) {
        S.vb[s] = s < kM ? S.gh[packed_index(s, kM)] : 0.0f;
        S.bl[s] = s < kM ? S.gl[packed_index(s, kM)] : 0.0f;
    }
    if (role_a && C == 0)
#pragma unroll
        for (int i = 0; i < 4; ++i)
            *reinterpret_cast<float4*>(S.panelA[0][4 * R + i]) = make_float4(m[i][0], m[i][1], m[i][2], m[i][3]);
    if (role_w && R == 0)
#pragma unroll
        for (int i = 0; i < 4; ++i)
            *reinterpret_cast<float4*>(&S.panelW[0][i][4 * C]) = make_float4(m[i][0], m[i][1], m[i][2], m[i][3]);
    // the sweep: Cholesky of A and W = L^-1, 17 block steps of 4 pivots (the
    // last three pivots are the padding's, 1 each)
    for (int J = 0; J < kNB; ++J) chol_block(S, J, role_a, role_w, R, C, m, s);
    __syncthreads();
    // 3. x = W^T W b, then two refinement steps with residuals in pairs
    w_matvec(S, role_w, R, C, m, S.vb, S.vz, false, s);
    w_matvec(S, role_w, R, C, m, S.vz, S.vx, true, s);
    if (s < kPad) {
        S.xh[s] = s < kM ? S.vx[s] : 0.0f;
        S.xl[s] = 0.0f;
    }
    __syncthreads();
    for (int it = 0; it < 2; ++it) {
        // residual of row i = s / 4 from 4 threads (columns j = s mod 4 + 4 t), added in a fixed order
        const int i = s >> 2, sub = s & 3;
        float rh = 0.0f, rl = 0.0f;
        if (i < kM) {
            float qh = 0.0f, ql = 0.0f;  // a second chain: columns sub + 8 t and sub + 4 + 8 t
            for (int jj = sub; jj < kM; jj += 8) {
                {
                    const int p = sym_index(i, jj);
                    const float ah = S.gh[p], al = S.gl[p], xh = S.xh[jj], xl = S.xl[jj];
                    const float ph = ah * xh;
                    const float pe = __fmaf_rn(ah, xh, -ph) + (ah * xl + al * xh);
                    pair_add(rh, rl, ph, pe);
                }
                if (jj + 4 < kM) {
                    const int p = sym_index(i, jj + 4);
                    const float ah = S.gh[p], al = S.gl[p], xh = S.xh[jj + 4], xl = S.xl[jj + 4];
                    const float ph = ah * xh;
                    const float pe = __fmaf_rn(ah, xh, -ph) + (ah * xl + al * xh);
                    pair_add(qh, ql, ph, pe);
                }
            }
            pair_add(rh, rl, qh, ql);
        }
#pragma unroll
        for (int w = 1; w <= 2; w <<= 1) {  // lanes 4i .. 4i+3 of one warp
            const float oh = __shfl_xor_sync(0xffffffffu, rh, w), ol = __shfl_xor_sync(0xffffffffu, rl, w);
            if (sub & w) {
                float th = oh, tl = ol;
                pair_add(th, tl, rh, rl);
                rh = th;
                rl = tl;
            } else {
                pair_add(rh, rl, oh, ol);
            }
        }
        if (sub == 0 && i < kM) {  // r_i = b_i - (A x)_i
            float h = S.vb[i], l = S.bl[i];
            pair_add(h, l, -rh, -rl);
            S.vr[i] = h;
        }
        if (s >= kM && s < kPad) S.vr[s] = 0.0f;
        __syncthreads();
        w_matvec(S, role_w, R, C, m, S.vr, S.vz, false, s);
        w_matvec(S, role_w, R, C, m, S.vz, S.vx, true, s);
        if (s < kM) {
            float h = S.xh[s], l = S.xl[s];
            pair_add(h, l, S.vx[s], 0.0f);
            S.xh[s] = h;
            S.xl[s] = l;
        }
        __syncthreads();
    }
    if (s < kM) {
        const float b = S.drop[s] ? 0.0f : __fmaf_rn(S.xl[s], S.sc[s], S.xh[s] * S.sc[s]);
        S.coef[s] = b;
        if (!(fabsf(b) <= 1e30f)) atomicOr(&S.bad, 1);  // also catches NaN
    }
    cp_async_wait_all();
    __syncthreads();  // the snapshot copy and the feature table are complete
    // fitted output layer of date d (W3 then b3) into the snapshot
    const bool ok = S.bad == 0;
    if (ok && s <= 64) {
        const float val = S.coef[s];
        snap[kW3 + s] = val;
        net[kW3 + s] = val;  // fine-tuning continues from the fit
    }
    if (s == 0) snap_ok[c.reg_offset + d] = ok ? 1 : 0;
    if (!ok) return;
    // The continuation table of date d for the exercise test at d (the next
    // backward iteration): E_i = b3 + W3 . F_i at every node, from the
    // feature table this fit used.
    const float b3 = S.coef[64];
    for (int i = s; i < kNodes; i += kSolveThreads) {
        const float* row = s_feat + i * 64;
        float y = b3;
#pragma unroll 4
        for (int q = 0; q < 16; ++q) {
            const float4 f = *reinterpret_cast<const float4*>(row + 4 * (q ^ (i & 7)));
            y = __fmaf_rn(S.coef[4 * q], f.x, y);
            y = __fmaf_rn(S.coef[4 * q + 1], f.y, y);
            y = __fmaf_rn(S.coef[4 * q + 2], f.z, y);
            y = __fmaf_rn(S.coef[4 * q + 3], f.w, y);
        }
        etab[static_cast<size_t>(ci) * kNodes + i] = y;
    }
}

// ---------------------------------------------------------------------------
// checks: one gradient step, inference, a single GEMM
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTrainThreads, 1)
    mlp_grad_kernel(const float* __restrict__ params, const float* __restrict__ x0, const float* __restrict__ x1,
                    const float* __restrict__ y, const float* __restrict__ wt, int n, float* __restrict__ grad,
                    float* __restrict__ loss, uint32_t* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
    const int s = threadIdx.x;
    for (int i = s; i < kParamStride; i += kTrainThreads) {
        S.p[i] = i < kParams ? params[i] : 0.0f;
        S.m[i] = 0.0f;
        S.v[i] = 0.0f;
    }
    train_setup(S);
    if (s < 64) refresh_w2_row(S, s);
    const bool live = s < n && s < 128;
    if (s < 128) {
        S.x0[s] = live ? x0[s] : 0.0f;
        S.x1[s] = live ? x1[s] : 0.0f;
        S.y[s] = live ? y[s] : 0.0f;
        S.w[s] = live ? wt[s] : 0.0f;
    }
    const int n_eff = __syncthreads_count(live && wt[s] > 0.0f);
    uint32_t phase = 0;
    const bool ok = train_step(S, S.tmem_base, phase, n_eff, false, 0.0f, 1, grad, err);
    if (s == 0) *loss = S.loss;
    train_teardown(S, phase, ok, err);
}

__global__ void __launch_bounds__(128)
    mlp_forward_kernel(const float* __restrict__ params, const float* __restrict__ x0, const float* __restrict__ x1,
                       int n, float* __restrict__ out, uint32_t* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    InferSmem& S = *reinterpret_cast<InferSmem*>(smem_raw);
    const int s = threadIdx.x, warp = s >> 5;
    for (int i = s; i < kParamStride; i += 128) S.p[i] = i < kParams ? params[i] : 0.0f;
    __syncthreads();
    if (s < 64)
        for (int j = 0; j < 64; j += 2)
            *reinterpret_cast<__nv_bfloat162*>(at(S.w2, s, j, 64)) =
                __floats2bfloat162_rn(S.p[kW2 + s * 64 + j], S.p[kW2 + s * 64 + j + 1]);
    if (s == 0) umma::mbar_init(&S.mbar, 1);
    if (warp == 0) umma::tmem_alloc(&S.tmem_base, 64);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tm = S.tmem_base;
    uint32_t phase = 0;
    bool ok = true;
    const int tiles = (n + 127) / 128;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int i = tile * 128 + s;
        const float a = i < n ? x0[i] : 0.0f, b = i < n ? x1[i] : 0.0f;
        for (int j = 0; j < 64; j += 2) {
            float t;
            const float za = __fmaf_rn(S.p[kW1 + 2 * j], a, __fmaf_rn(S.p[kW1 + 2 * j + 1], b, S.p[kB1 + j]));
            const float zb = __fmaf_rn(S.p[kW1 + 2 * j + 2], a, __fmaf_rn(S.p[kW1 + 2 * j + 3], b, S.p[kB1 + j + 1]));
            *reinterpret_cast<__nv_bfloat162*>(at(S.h1, s, j, 64)) = __floats2bfloat162_rn(gelu(za, t), gelu(zb, t));
        }
        umma::fence_smem_to_async();
        umma::fence_before_sync();
        __syncthreads();
        if (s == 0) {
            umma::fence_after_sync();
            for (int kk = 0; kk < 4; ++kk)
                umma::mma_bf16(tm, desc(S.h1, 1024, kk), desc(S.w2, 1024, kk), kIdesc, kk > 0);
            umma::mma_commit(&S.mbar);
        }
        ok = __syncthreads_and(ok && umma::mbar_wait(&S.mbar, phase, err, 7));
        phase ^= 1u;
        umma::fence_after_sync();
        float yhat = S.p[kB3];
        for (int cc = 0; cc < 4; ++cc) {
            float zz[16];
            umma::tmem_ld16(umma::tmem_addr(tm, 32 * warp, cc * 16), zz);
            for (int q = 0; q < 16; ++q) {
                float t;
                yhat = __fmaf_rn(S.p[kW3 + cc * 16 + q], gelu(zz[q] + S.p[kB2 + cc * 16 + q], t), yhat);
            }
        }
        if (i < n) out[i] = ok ? yhat : 0.0f;
        umma::fence_before_sync();
        __syncthreads();
    }
    if (!ok) umma::mbar_wait(&S.mbar, phase, err, 8);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tm, 64);
}

// D (128 x 64) = A (128 x 64) B^T (B: 64 x 64), BF16 inputs, FP32 accumulate.
__global__ void __launch_bounds__(128, 1)
    umma_selftest_kernel(const float* __restrict__ A, const float* __restrict__ B, float* __restrict__ D,
                         uint32_t* __restrict__ err) {
    __shared__ __align__(1024) __nv_bfloat16 a_s[128 * 64];
    __shared__ __align__(1024) __nv_bfloat16 b_s[64 * 64];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    const int s = threadIdx.x, warp = s >> 5;
    for (int k = 0; k < 64; ++k) *at(a_s, s, k, 64) = __float2bfloat16_rn(A[s * 64 + k]);
    if (s < 64)
        for (int k = 0; k < 64; ++k) *at(b_s, s, k, 64) = __float2bfloat16_rn(B[s * 64 + k]);
    if (s == 0) umma::mbar_init(&mbar, 1);
    if (warp == 0) umma::tmem_alloc(&tbase, 64);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tm = tbase;
    if (s == 0) {
        for (int kk = 0; kk < 4; ++kk) umma::mma_bf16(tm, desc(a_s, 1024, kk), desc(b_s, 1024, kk), kIdesc, kk > 0);
        umma::mma_commit(&mbar);
    }
    const bool ok = __syncthreads_and(umma::mbar_wait(&mbar, 0, err, 9));
    umma::fence_after_sync();
    if (ok) {
        for (int c = 0; c < 4; ++c) {
            float v[16];
            umma::tmem_ld16(umma::tmem_addr(tm, 32 * warp, c * 16), v);
            for (int q = 0; q < 16; ++q) D[s * 64 + c * 16 + q] = v[q];
        }
    } else {
        umma::mbar_wait(&mbar, 0, err, 10);
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tm, 64);
}

template <typename K>
cudaError_t set_smem(K kernel, size_t bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}

}  // namespace

size_t mlp_train_smem_bytes() { return sizeof(TrainSmem); }
size_t mlp_infer_smem_bytes() { return sizeof(InferSmem); }

cudaError_t mlp_prepare() {
    cudaError_t e = set_smem(lsm_mlp_train<0>, sizeof(TrainSmem));
    if (e == cudaSuccess) e = set_smem(lsm_mlp_train<1>, sizeof(TrainSmem));
    if (e == cudaSuccess) e = set_smem(mlp_grad_kernel, sizeof(TrainSmem));
    if (e == cudaSuccess) e = set_smem(lsm_mlp_pass<0>, sizeof(PassSmem));
    if (e == cudaSuccess) e = set_smem(lsm_mlp_pass<1>, sizeof(PassSmem));
    if (e == cudaSuccess) e = set_smem(mlp_forward_kernel, sizeof(InferSmem));
    if (e == cudaSuccess) e = set_smem(lsm_mlp_solve, kSolveFeatBytes);
    return e;
}

cudaError_t launch_lsm_mlp_first_training(int precision, const LsmDev* c, int c_first, int c_end, int max_steps,
                                          float* nets, float* snaps, int* snap_ok, int* adam_t, float* feats,
                                          double* pre_s, double* pre_cf, const MlpConfig& cfg, uint32_t* err,
                                          cudaStream_t stream) {
    cudaGetLastError();
    if (c_end <= c_first) return cudaSuccess;
    const int n_contracts = c_end - c_first;
    if (cfg.steps_first > 0) {
        const dim3 grid(static_cast<unsigned>(n_contracts), static_cast<unsigned>(std::min(cfg.steps_first, 1024)));
        if (precision == 0)
            lsm_mlp_train_samples<0><<<grid, 128, 0, stream>>>(c, c_first, c_end, cfg.steps_first, pre_s, pre_cf);
        else
            lsm_mlp_train_samples<1><<<grid, 128, 0, stream>>>(c, c_first, c_end, cfg.steps_first, pre_s, pre_cf);
    }
    // the trainer reads no store at k = 0 when the samples are given
    if (precision == 0)
        lsm_mlp_train<0><<<n_contracts, kTrainThreads, sizeof(TrainSmem), stream>>>(
            0, c, c_first, c_end, nullptr, nullptr, nets, snaps, snap_ok, adam_t, cfg, pre_s, pre_cf, err);
    else
        lsm_mlp_train<1><<<n_contracts, kTrainThreads, sizeof(TrainSmem), stream>>>(
            0, c, c_first, c_end, nullptr, nullptr, nets, snaps, snap_ok, adam_t, cfg, pre_s, pre_cf, err);
    cudaError_t e = cudaGetLastError();
    // fixed features: every date's table at once
    if (e == cudaSuccess && cfg.steps == 0) e = launch_lsm_mlp_features(0, true, max_steps, c, c_first, c_end, nets, feats, err, stream);
    return e;
}

cudaError_t launch_lsm_mlp_iteration(int precision, int k, bool train, const LsmDev* c, int c_first, int c_end,
                                     int max_steps, const uint32_t* group_contract, uint32_t g_first, uint32_t g_end,
                                     const void* store,
                                     double* cf, float* nets, float* snaps, int* snap_ok, int* adam_t,
                                     float* gram_part, float* feats, float* etab, unsigned long long* mom_part,
                                     const MlpConfig& cfg, Welford* final_part, cudaEvent_t trained, uint32_t* err,
                                     cudaStream_t stream) {
    cudaGetLastError();
    if (g_end <= g_first || c_end <= c_first) return cudaSuccess;
    const uint32_t n_groups = g_end - g_first;
    const int n_contracts = c_end - c_first;
    const size_t pass_smem = sizeof(PassSmem);
    auto step = [&]() {  // the per-path network: terminal step, and replays of given networks
        if (precision == 0)
            lsm_mlp_pass<0><<<n_groups, 128, pass_smem, stream>>>(k, c, group_contract, g_first, g_end, store, cf,
                                                                      snaps, snap_ok, final_part, err);
        else
            lsm_mlp_pass<1><<<n_groups, 128, pass_smem, stream>>>(k, c, group_contract, g_first, g_end, store, cf,
                                                                      snaps, snap_ok, final_part, err);
    };
    auto trainer = [&]() {  // fine-tuning at a later date (k > 0): samples from the stores
        if (precision == 0)
            lsm_mlp_train<0><<<n_contracts, kTrainThreads, sizeof(TrainSmem), stream>>>(
                k, c, c_first, c_end, store, cf, nets, snaps, snap_ok, adam_t, cfg, nullptr, nullptr, err);
        else
            lsm_mlp_train<1><<<n_contracts, kTrainThreads, sizeof(TrainSmem), stream>>>(
                k, c, c_first, c_end, store, cf, nets, snaps, snap_ok, adam_t, cfg, nullptr, nullptr, err);
    };
    if (!train) {
        step();
        return cudaGetLastError();
    }
    int mode = kStep | kGram;  // exercise at date e, discount, regression data of date e-1
    const bool fine_tune = cfg.steps > 0;
    cudaError_t e = cudaSuccess;
    if (k == 0) {
        // The binned pass does the terminal step (payoff at date n, one
        // discount) along with the moments of date n-1.  The first training
        // (and, with fixed features, every date's feature table) ran on
        // another stream (launch_lsm_mlp_first_training).
        e = cudaStreamWaitEvent(stream, trained, 0);
    }
    // fine-tuned features: the table of date e-1 from the network as tuned so far
    if (e == cudaSuccess && fine_tune) e = launch_lsm_mlp_features(k, false, max_steps, c, c_first, c_end, nets, feats, err, stream);
    if (e == cudaSuccess)
        e = launch_lsm_mlp_binned(precision, k, mode, c, c_first, c_end, group_contract, g_first, g_end, store, cf,
                                  snap_ok, feats, etab, mom_part, gram_part, final_part, stream);
    if (e != cudaSuccess) return e;
    lsm_mlp_solve<<<n_contracts, kSolveThreads, kSolveFeatBytes, stream>>>(k, c, c_first, c_end, gram_part, feats, nets,
                                                                            snaps, snap_ok, etab);
    if (k > 0 && fine_tune) trainer();  // optional fine-tuning of the features
    return cudaGetLastError();
}

cudaError_t launch_mlp_grad(const float* params, const float* x0, const float* x1, const float* y, const float* w,
                            int n, float* grad, float* loss, uint32_t* err, cudaStream_t stream) {
    cudaGetLastError();
    mlp_grad_kernel<<<1, kTrainThreads, sizeof(TrainSmem), stream>>>(params, x0, x1, y, w, n, grad, loss, err);
    return cudaGetLastError();
}

cudaError_t launch_mlp_forward(const float* params, const float* x0, const float* x1, int n, float* out,
                               uint32_t* err, cudaStream_t stream) {
    cudaGetLastError();
    const int tiles = (n + 127) / 128;
    const int grid = tiles < 1024 ? (tiles > 0 ? tiles : 1) : 1024;
    mlp_forward_kernel<<<grid, 128, sizeof(InferSmem), stream>>>(params, x0, x1, n, out, err);
    return cudaGetLastError();
}

cudaError_t launch_umma_selftest(const float* A, const float* B, float* D, uint32_t* err, cudaStream_t stream) {
    cudaGetLastError();
    umma_selftest_kernel<<<1, 128, 0, stream>>>(A, B, D, err);
    return cudaGetLastError();
}

}  // namespace mcdg
