// lsm_mlp_nodes.cu -- the learned regression on node tables.
//
// At an exercise date the continuation network (lsm_mlp.cu, mlp.cuh) sees
// x0 = 4 (S/K - 1) and a time input that is one value per date, so each of its
// 64 last-layer features is a function of u = ln(S/K) alone at that date.
// Rather than evaluating the 2 -> 64 -> 64 network once per in-the-money path
// and date, each (contract, date) evaluates it at kNodes = 512 equally spaced
// values of u over the in-the-money side of the date's distribution (node_grid,
// lsm_mlp_dev.hpp) and every path uses the linear interpolation of those
// nodes, f(u) = (1 - t) F_i + t F_{i+1} with u in bin i at fraction t:
//
//   lsm_mlp_nodes        one CTA per (contract, 128-node tile, date): the
//                        feature table F of a date: layer 1 on the CUDA
//                        cores, Z2 = H1 W2^T on the tensor core (tcgen05,
//                        BF16 operands, FP32 accumulator in tensor memory),
//                        GELU.  With fixed features every date's table is
//                        built in one launch after the training; with
//                        fine-tuned features, one date per backward
//                        iteration.  (The continuation table of a date, E_i =
//                        b3 + W3 . F_i, is written by the solve that fits W3.)
//   lsm_mlp_binned       one CTA per group of chunks: exercise at date e where
//                        the interpolated continuation value is negative (at
//                        k = 0 the terminal payoff instead), discount,
//                        cash-flow update, and for the paths in the money at
//                        date e-1 the per-bin moments n, sum t, sum t^2, sum y,
//                        sum t y (y = time value / K) as exact integers (t to
//                        16 bits, y to 24 bits of its bound), added as 32-bit
//                        limbs with nine shared-memory atomics per path and
//                        folded into 64-bit sums every 32 chunks: the sums do
//                        not depend on the order of the additions, so the
//                        result is deterministic.
//   lsm_mlp_gram_slices  kNodeSlices CTAs per contract: the Gram matrix of
//                        [f | 1 | y] over the paths from the moments,
//                        G = sum over bins of (1-t)^2 F_i F_i^T + t(1-t)
//                        (F_i F_{i+1}^T + F_{i+1} F_i^T) + t^2 F_{i+1} F_{i+1}^T
//                        (and the right-hand side likewise), one partial per
//                        64 bins; lsm_mlp_solve sums them in order.
//
// The least-squares fit over the interpolated features is exact (no path is
// left out and no feature rounded to BF16 on its way to the Gram matrix); the
// interpolation moves a feature by ~h^2 f''/8 (h = 1/511 of the grid), far
// below the BF16 rounding of the network's own hidden layer.  Every mbarrier
// wait is bounded (umma.cuh).
//
// nvcc-flags: --fmad=false
#include <cuda_bf16.h>
#include <cuda_runtime.h>

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

constexpr int kGramDim = 66;   // 64 features, constant, target
constexpr int kFStride = 68;   // feature-table row stride in shared memory (16-byte rows)
constexpr int kBinsPerSlice = kNodes / kNodeSlices;
constexpr uint32_t kNodeIdesc = umma::idesc_bf16(128, 64);
static_assert(kNodes % 128 == 0 && kNodes % kNodeSlices == 0, "node tiles");

__device__ __forceinline__ __nv_bfloat16* at(__nv_bfloat16* base, int r, int k, int kcols) {
    return reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(base) + umma::kmajor_offset(r, k, kcols));
}

__device__ __forceinline__ uint64_t desc(const void* p, uint32_t sbo, int kstep) {
    return umma::smem_desc(umma::smem_u32(p) + static_cast<uint32_t>(kstep) * 256u, 128u, sbo);
}

__device__ __forceinline__ int packed_index(int r, int q) {  // r <= q
    return r * kGramDim - r * (r - 1) / 2 + (q - r);
}

// Bin and fraction of u on a grid: u below the first node or above the last
// uses the end bin (t clamped to [0, 1]).
__device__ __forceinline__ void locate(const NodeGrid& g, float u, int& i, float& t) {
    float x = (u - g.lo) * g.inv_h;
    x = fminf(fmaxf(x, 0.0f), static_cast<float>(kNodes - 1));
    i = min(static_cast<int>(x), kNodes - 2);
    t = fminf(x - static_cast<float>(i), 1.0f);
}

// ---------------------------------------------------------------------------
// Node tables: continuation values of date e and features of date e-1.
// ---------------------------------------------------------------------------
struct __align__(1024) NodeSmem {
    __nv_bfloat16 h1[128 * 64];  // A: [node][hidden 1], K-major, K = 64
    __nv_bfloat16 w2[64 * 64];   // B: [hidden 2][hidden 1], K-major
    __align__(16) float w0[64];  // W1[j][0]
    __align__(16) float c1[64];  // fma(W1[j][1], x1, b1[j]) at the date's time input
    float b2[64];
    float w3[64];
    NodeGrid grid;
    uint64_t mbar;
    uint32_t tmem_base;
};

// Layer 1 of one node with the date's time input folded into c:
// z[j] = fma(W1[j][0], x0, c[j]); four hidden units per 8-byte store.
__device__ __forceinline__ void layer1_node(const float* w0, const float* c, float x0, __nv_bfloat16* h1, int s) {
#pragma unroll 4
    for (int j = 0; j < 64; j += 4) {
        const float4 w = *reinterpret_cast<const float4*>(w0 + j);
        const float4 b = *reinterpret_cast<const float4*>(c + j);
        float t;
        const __nv_bfloat162 lo = __floats2bfloat162_rn(gelu(__fmaf_rn(w.x, x0, b.x), t), gelu(__fmaf_rn(w.y, x0, b.y), t));
        const __nv_bfloat162 hi = __floats2bfloat162_rn(gelu(__fmaf_rn(w.z, x0, b.z), t), gelu(__fmaf_rn(w.w, x0, b.w), t));
        uint2 v;
        v.x = *reinterpret_cast<const uint32_t*>(&lo);
        v.y = *reinterpret_cast<const uint32_t*>(&hi);
        *reinterpret_cast<uint2*>(at(h1, s, j, 64)) = v;  // units j..j+3: one 8-byte run (j % 8 is 0 or 4)
    }
}

__global__ void __launch_bounds__(128)
    lsm_mlp_nodes(int k, int all_dates, const LsmDev* __restrict__ cs, int c_first, int n_contracts,
                  const float* __restrict__ nets, float* __restrict__ feats, uint32_t* __restrict__ err) {
    __shared__ NodeSmem S;
    const int ci = c_first + static_cast<int>(blockIdx.x);
    if (ci >= n_contracts) return;
    const LsmDev c = cs[ci];
    const int n = c.n_steps;
    // the date: every regression date 1 .. n-1 (blockIdx.z + 1), or the one
    // of backward iteration k
    const int d = all_dates ? static_cast<int>(blockIdx.z) + 1 : n - k - 1;
    if (d < 1 || d > n - 1) return;
    const int tile = static_cast<int>(blockIdx.y);
    const int s = threadIdx.x, warp = s >> 5;
    float* F = feats + (static_cast<size_t>(c.reg_offset) + d) * kNodes * 64;
    const float* net = nets + static_cast<size_t>(ci) * 3 * kParamStride;
    const float x1 = static_cast<float>(n - d) / static_cast<float>(n);
    if (s < 64) {
        S.w0[s] = net[kW1 + 2 * s];
        S.c1[s] = __fmaf_rn(net[kW1 + 2 * s + 1], x1, net[kB1 + s]);
        S.b2[s] = net[kB2 + s];
    }
    for (int i = s; i < 64 * 32; i += 128) {  // W2 [out][in] read in order (coalesced), pairs to BF16
        const int r = i >> 5, j = 2 * (i & 31);
        const float2 w = *reinterpret_cast<const float2*>(net + kW2 + r * 64 + j);
        *reinterpret_cast<__nv_bfloat162*>(at(S.w2, r, j, 64)) = __floats2bfloat162_rn(w.x, w.y);
    }
    if (s == 0) {
        umma::mbar_init(&S.mbar, 1);
        S.grid = node_grid(c, d);  // FP64 library calls: once per CTA
    }
    if (warp == 0) umma::tmem_alloc(&S.tmem_base, 64);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tm = S.tmem_base;
    const NodeGrid g = S.grid;
    // one 128-node tile: layer 1 on the CUDA cores, Z2 = H1 W2^T on the tensor core, GELU
    const int i = tile * 128 + s;
    const float u = __fmaf_rn(static_cast<float>(i), g.h, g.lo);
    const float x0 = 4.0f * (expf(u) - 1.0f);
    layer1_node(S.w0, S.c1, x0, S.h1, s);
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    if (s == 0) {
        umma::fence_after_sync();
        for (int kk = 0; kk < 4; ++kk)
            umma::mma_bf16(tm, desc(S.h1, 1024, kk), desc(S.w2, 1024, kk), kNodeIdesc, kk > 0);
        umma::mma_commit(&S.mbar);
    }
    const bool ok = __syncthreads_and(umma::mbar_wait(&S.mbar, 0u, err, 41));
    if (ok) {
        umma::fence_after_sync();
        float4* dst = reinterpret_cast<float4*>(F + static_cast<size_t>(i) * 64);
        for (int cc = 0; cc < 4; ++cc) {
            float zz[16];
            umma::tmem_ld16(umma::tmem_addr(tm, 32 * warp, cc * 16), zz);
#pragma unroll
            for (int q = 0; q < 16; q += 4) {
                float t;
                float4 v;
                v.x = gelu(zz[q] + S.b2[cc * 16 + q], t);
                v.y = gelu(zz[q + 1] + S.b2[cc * 16 + q + 1], t);
                v.z = gelu(zz[q + 2] + S.b2[cc * 16 + q + 2], t);
                v.w = gelu(zz[q + 3] + S.b2[cc * 16 + q + 3], t);
                dst[(cc * 16 + q) / 4] = v;
            }
        }
    } else {
        umma::mbar_wait(&S.mbar, 0u, err, 42);  // the MMA that timed out, once more (bounded)
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tm, 64);
}

// ---------------------------------------------------------------------------
// Binned path pass.
// ---------------------------------------------------------------------------
constexpr int kBinThreads = 256;  // five CTAs per SM (48 registers): latency-bound on the shared-memory atomics
static_assert(kNodes == 2 * kBinThreads, "two bins per thread when the moments are folded");

// The moments are accumulated with 32-bit shared-memory atomics (the native
// ones; a 64-bit shared atomic add is several times slower) in limbs of at
// most 16 bits per path, over epochs of at most kEpochChunks chunks, so no
// limb sum can exceed 2^32: with tq in [0, 2^16], yb = yq + 2^24 in [0, 2^25]
// and P = tq yb in [0, 2^41] the limbs are
//   0: 1            1: tq
//   2: tq^2 mod 2^16    3: tq^2 / 2^16     (tq^2 <= 2^32)
//   4: yb mod 2^16      5: yb / 2^16
//   6: P mod 2^16       7: P / 2^16 mod 2^16   8: P / 2^32
// After each epoch the limbs are recombined exactly into the four 64-bit
// moments (n 2^40 + sum tq, sum tq^2, sum yq, sum tq yq, the last two modulo
// 2^64 as two's complement), which therefore equal the sums of the per-path
// 64-bit terms bit for bit.
constexpr int kLimbs = 9;
constexpr uint32_t kEpochChunks = 32;
static_assert(static_cast<uint64_t>(kEpochChunks) * kLsmChunk * 65536ull < (1ull << 32),
              "limb sums of one epoch fit 32 bits");

template <int PREC>
__global__ void __launch_bounds__(kBinThreads, 5)
    lsm_mlp_binned(int k, int mode, const LsmDev* __restrict__ cs, const uint32_t* __restrict__ group_contract,
                   uint32_t g_first, uint32_t total_groups, const void* __restrict__ store, double* __restrict__ cf,
                   const int* __restrict__ snap_ok, const float* __restrict__ etab,
                   unsigned long long* __restrict__ mom_part, Welford* __restrict__ final_part) {
    __shared__ float2 tab[kNodes];                             // continuation table of date e: value, slope to the next node
    __shared__ uint32_t lim[kLimbs][kNodes];                   // limbs of the moments of date e-1, bin by bin
    __shared__ unsigned long long mom[kMoments][kNodes];       // the moments, epochs folded so far
    __shared__ Welford swf[kBinThreads / 32];
    __shared__ Sum64 s64[kBinThreads / 32];
    __shared__ NodeGrid s_grid[2];                             // dates e and e-1
    const uint32_t g = g_first + blockIdx.x;
    if (g >= total_groups) return;
    const uint32_t ci = group_contract[g];
    const LsmDev c = cs[ci];
    const int n = c.n_steps;
    const int e = n - k;
    if (e < 1) return;
    const bool step = (mode & kStep) != 0;
    const bool init = step && k == 0;
    const bool last = step && e == 1;
    const bool exercise = step && k > 0 && e <= n - 1 && snap_ok[c.reg_offset + e] == 1;
    const bool gram = (mode & kGram) != 0 && e - 1 >= 1;
    if (!step && !gram) return;
    const int s = threadIdx.x, warp = s >> 5;
    // Per-path arithmetic in the path precision (FP64 on the FP64 path, FP32 on
    // the FP32 path); bins, fractions and targets in FP32.
    using T = typename std::conditional<PREC == 0, double, float>::type;
    const T phi = PREC == 0 ? T(c.type == 0 ? 1.0 : -1.0) : T(c.phi_f);
    const T strike = PREC == 0 ? T(c.strike) : T(c.strike_f);
    const T inv_k = PREC == 0 ? T(1.0 / c.strike) : T(c.inv_strike_f);
    const T disc = PREC == 0 ? T(c.disc) : T(c.disc_f);
    const float inv_kf = c.inv_strike_f;
    const T* S_path = static_cast<const T*>(store) + c.s_offset;
    T* cft = reinterpret_cast<T*>(cf) + c.cf_offset;
    if (s == 0) {  // FP64 library calls: once per CTA
        s_grid[0] = exercise ? node_grid(c, e) : NodeGrid{0.0f, 0.0f, 0.0f, 1.0f};
        s_grid[1] = gram ? node_grid(c, e - 1) : NodeGrid{0.0f, 0.0f, 0.0f, 1.0f};
    }
    if (exercise)
        for (int i = s; i < kNodes; i += kBinThreads) {
            const float* row = etab + static_cast<size_t>(ci) * kNodes;
            const float v = row[i];
            tab[i] = make_float2(v, i + 1 < kNodes ? row[i + 1] - v : 0.0f);
        }
    if (gram) {
        for (int i = s; i < kLimbs * kNodes; i += kBinThreads) (&lim[0][0])[i] = 0u;
        for (int i = s; i < kMoments * kNodes; i += kBinThreads) (&mom[0][0])[i] = 0ull;
    }
    __syncthreads();
    const NodeGrid ge = s_grid[0], gd = s_grid[1];
    const float yq_scale = static_cast<float>(kYScale) / gd.y_bound;
    const uint32_t gl = g - c.group_begin;
    const uint32_t chunk0 = gl * c.group_chunks;
    const uint32_t chunk1 = min(c.n_chunks, chunk0 + c.group_chunks);
    Welford w{0ull, 0.0, 0.0};
    Sum32 fin{0u, 0.0f, 0.0f, 0.0f, 0.0f};  // FP32 path: the last date's payoffs
    // the limbs of the epoch just ended, recombined into mom and cleared
    // (thread s folds bins s and s + kBinThreads)
    auto fold_epoch = [&]() {
        __syncthreads();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int b = s + h * kBinThreads;
            unsigned long long l[kLimbs];
#pragma unroll
            for (int q = 0; q < kLimbs; ++q) {
                l[q] = lim[q][b];
                lim[q][b] = 0u;
            }
            const unsigned long long st = l[1];
            mom[0][b] += (l[0] << kCountShift) + st;
            mom[1][b] += l[2] + (l[3] << 16);
            mom[2][b] += l[4] + (l[5] << 16) - (l[0] << 24);
            mom[3][b] += l[6] + (l[7] << 16) + (l[8] << 32) - (st << 24);
        }
        __syncthreads();
    };
    constexpr int kPer = kLsmChunk / kBinThreads;  // paths per thread and chunk
    for (uint32_t ch = chunk0; ch < chunk1; ++ch) {
        if (gram && ch > chunk0 && (ch - chunk0) % kEpochChunks == 0) fold_epoch();
        // every path load of this thread's kPer paths first (independent, in flight
        // together), from the chunk's column bases at fixed offsets
        const uint64_t p0 = static_cast<uint64_t>(ch) * kLsmChunk + s;  // this thread's first path
        const uint64_t rem = c.path_count - static_cast<uint64_t>(ch) * kLsmChunk;  // paths in the chunk and after
        T* cf_c = cft + p0;
        const T* v_c = init ? S_path + static_cast<uint64_t>(n - 1) * c.path_count + p0 : cf_c;
        const T* e_c = S_path + static_cast<uint64_t>(exercise ? e - 1 : 0) * c.path_count + p0;
        const T* d_c = S_path + static_cast<uint64_t>(gram ? e - 2 : 0) * c.path_count + p0;
        T vv[kPer], se[kPer], sd[kPer];
        bool live[kPer];
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            live[q] = static_cast<uint64_t>(q * kBinThreads + s) < rem;
            vv[q] = se[q] = sd[q] = T(0);
            if (live[q]) {
                vv[q] = v_c[q * kBinThreads];
                if (exercise) se[q] = e_c[q * kBinThreads];
                if (gram) sd[q] = d_c[q * kBinThreads];
            }
        }
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            if (!live[q]) continue;
            T v = vv[q];
            if (init) {
                const T x = phi * (v - strike);
                v = x > T(0) ? x : T(0);
            }
            if (exercise) {
                const T xx = phi * (se[q] - strike);
                if (xx > T(0)) {
                    int b;
                    float t;
                    locate(ge, __logf(static_cast<float>(se[q]) * inv_kf), b, t);
                    const float2 nb = tab[b];
                    const float cont = __fmaf_rn(t, nb.y, nb.x);
                    if (cont < 0.0f) v = xx;  // predicted time value < 0: exercise
                }
            }
            if (step) {
                v *= disc;
                if (last) {
                    if constexpr (PREC == 0) {
                        welford_add(w, v);
                    } else {
                        sum32_add(fin, v);
                    }
                } else {
                    cf_c[q * kBinThreads] = v;
                }
            }
            if (gram) {
                const T xx = phi * (sd[q] - strike);
                if (xx > T(0)) {
                    int b;
                    float t;
                    locate(gd, __logf(static_cast<float>(sd[q]) * inv_kf), b, t);
                    const float y = static_cast<float>((v - xx) * inv_k);
                    // 32-bit conversions (a 64-bit one would run on the FP64 unit), widened by
                    // integer products: tq in [0, 2^16], |yq| <= 2^24
                    const int tq = __float2int_rn(t * static_cast<float>(kTScale));
                    // (the float clamp keeps yq in range, NaN included: fmaxf returns the bound)
                    const int yq = __float2int_rn(fminf(fmaxf(y * yq_scale, -16777216.0f), 16777216.0f));
                    const uint32_t ut = static_cast<uint32_t>(tq);           // [0, 2^16]
                    const uint32_t yb = static_cast<uint32_t>(yq + 16777216);  // [0, 2^25]
                    const unsigned long long tt = static_cast<unsigned long long>(ut) * ut;
                    const unsigned long long pp = static_cast<unsigned long long>(ut) * yb;
                    atomicAdd(&lim[0][b], 1u);
                    atomicAdd(&lim[1][b], ut);
                    atomicAdd(&lim[2][b], static_cast<uint32_t>(tt) & 0xFFFFu);
                    atomicAdd(&lim[3][b], static_cast<uint32_t>(tt >> 16));
                    atomicAdd(&lim[4][b], yb & 0xFFFFu);
                    atomicAdd(&lim[5][b], yb >> 16);
                    atomicAdd(&lim[6][b], static_cast<uint32_t>(pp) & 0xFFFFu);
                    atomicAdd(&lim[7][b], static_cast<uint32_t>(pp >> 16) & 0xFFFFu);
                    atomicAdd(&lim[8][b], static_cast<uint32_t>(pp >> 32));
                }
            }
        }
        if (last) {  // one final partial per chunk, fixed tree
            if constexpr (PREC == 0) {
                Welford r = welford_warp_reduce(w);
                if ((s & 31) == 0) swf[warp] = r;
                __syncthreads();
                if (s == 0) {
                    Welford m = swf[0];
                    for (int q = 1; q < kBinThreads / 32; ++q) m = welford_merge(m, swf[q]);
                    final_part[c.chunk_begin + ch] = m;
                }
                w = Welford{0ull, 0.0, 0.0};
            } else {
                const Sum32 r = sum32_warp_reduce(fin);
                if ((s & 31) == 0) s64[warp] = sum32_wide(r);
                __syncthreads();
                if (s == 0) final_part[c.chunk_begin + ch] = sum64_fold<kBinThreads / 32>(s64);
                fin = Sum32{0u, 0.0f, 0.0f, 0.0f, 0.0f};
            }
            __syncthreads();
        }
    }
    if (gram) {
        fold_epoch();
        unsigned long long* out = mom_part + static_cast<size_t>(g) * kMoments * kNodes;
        for (int i = s; i < kMoments * kNodes; i += kBinThreads) out[i] = (&mom[0][0])[i];
    }
}

// ---------------------------------------------------------------------------
// Gram matrix of [f | 1 | y] from the bin moments, 128 bins per CTA.  Blocks of 4 x 4 entries of the upper triangle (one per thread);
// per bin, with A = Saa F_i + Sab F_{i+1} and B = Sab F_i + Sbb F_{i+1} on the
// block's rows, the block gains A F_i^T + B F_{i+1}^T on its columns.
// ---------------------------------------------------------------------------
constexpr int kGramThreads = 256;
constexpr int kBlocks = kFStride / 4;                         // 17 blocks of 4 indices (65 used)
constexpr int kBlockTasks = kBlocks * (kBlocks + 1) / 2;      // upper-triangular blocks
static_assert(kBlockTasks + kBlocks <= kGramThreads, "one task per thread");

__global__ void __launch_bounds__(kGramThreads)
    lsm_mlp_gram_slices(int k, const LsmDev* __restrict__ cs, int c_first, int n_contracts,
                        const unsigned long long* __restrict__ mom_part, const float* __restrict__ feats,
                        float* __restrict__ gram_part) {
    __shared__ __align__(16) float F[kBinsPerSlice + 1][kFStride];
    __shared__ float wgt[5][kBinsPerSlice];  // Saa, Sab, Sbb, Say, Sby of each bin
    __shared__ unsigned long long msum[5][kBinsPerSlice];  // n, sum t, sum t^2, sum y, sum t y
    __shared__ double s_yb;
    const int ci = c_first + static_cast<int>(blockIdx.x), slice = blockIdx.y;
    if (ci >= n_contracts) return;
    const LsmDev c = cs[ci];
    const int d = c.n_steps - k - 1;
    if (d < 1) return;
    const int s = threadIdx.x;
    const int row0 = slice * kBinsPerSlice;
    // feature rows row0 .. row0 + kBinsPerSlice, with the constant 1 in column 64:
    // the table's pieces copied in while the moments are summed
    {
        const float* src = feats + (static_cast<size_t>(c.reg_offset) + d) * kNodes * 64;
        for (int idx = s; idx < (kBinsPerSlice + 1) * (kFStride / 4); idx += kGramThreads) {
            const int r = idx / (kFStride / 4), q4 = idx % (kFStride / 4);
            if (row0 + r < kNodes && q4 < 16) {
                cp_async16(&F[r][4 * q4], src + static_cast<size_t>(row0 + r) * 64 + 4 * q4);
            } else {
                const float one = row0 + r < kNodes ? 1.0f : 0.0f;
                *reinterpret_cast<float4*>(&F[r][4 * q4]) = make_float4(one, 0.0f, 0.0f, 0.0f);
            }
        }
        cp_async_commit();
    }
    if (s == 0) s_yb = static_cast<double>(node_grid(c, d).y_bound);  // FP64 library calls: once per CTA
    {
        // The groups' moments of the slice's bins, summed with loads in flight:
        // thread s takes bin s mod 64 and word s / 64 of every group (word 0
        // holds n 2^40 + sum t, split per group).
        static_assert(kBinsPerSlice * kMoments == kGramThreads, "one (bin, word) per thread");
        const int bl = s % kBinsPerSlice, q = s / kBinsPerSlice;
        const int b = row0 + bl;
        unsigned long long a0 = 0ull, a1 = 0ull;
        if (b <= kNodes - 2) {
            const unsigned long long* p = mom_part + (static_cast<size_t>(c.group_begin) * kMoments + q) * kNodes + b;
            constexpr uint32_t kBatch = 8;
            for (uint32_t g0 = 0; g0 < c.n_groups; g0 += kBatch) {
                unsigned long long v[kBatch];
#pragma unroll
                for (uint32_t u = 0; u < kBatch; ++u)
                    v[u] = g0 + u < c.n_groups ? p[static_cast<size_t>(g0 + u) * kMoments * kNodes] : 0ull;
#pragma unroll
                for (uint32_t u = 0; u < kBatch; ++u) {
                    if (q == 0) {
                        a0 += v[u] >> kCountShift;
                        a1 += v[u] & ((1ull << kCountShift) - 1ull);
                    } else {
                        a0 += v[u];
                    }
                }
            }
        }
        if (q == 0) {
            msum[0][bl] = a0;
            msum[1][bl] = a1;
        } else {
            msum[q + 1][bl] = a0;
        }
    }
    __syncthreads();
    if (s < kBinsPerSlice) {
        const int b = row0 + s;
        float w[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        if (b <= kNodes - 2) {
            // n, sum t, sum t^2, sum y, sum t y
            const unsigned long long m[5] = {msum[0][s], msum[1][s], msum[2][s], msum[3][s], msum[4][s]};
            const double yb = s_yb;
            const double cnt = static_cast<double>(m[0]);
            const double st = static_cast<double>(m[1]) / kTScale;
            const double stt = static_cast<double>(m[2]) / (kTScale * kTScale);
            const double sy = static_cast<double>(static_cast<long long>(m[3])) * (yb / kYScale);
            const double sty = static_cast<double>(static_cast<long long>(m[4])) * (yb / (kTScale * kYScale));
            w[0] = static_cast<float>(cnt - 2.0 * st + stt);  // sum (1-t)^2
            w[1] = static_cast<float>(st - stt);              // sum t (1-t)
            w[2] = static_cast<float>(stt);                   // sum t^2
            w[3] = static_cast<float>(sy - sty);              // sum (1-t) y
            w[4] = static_cast<float>(sty);                   // sum t y
        }
#pragma unroll
        for (int q = 0; q < 5; ++q) wgt[q][s] = w[q];
    }
    cp_async_wait_all();
    __syncthreads();
    float* out = gram_part + (static_cast<size_t>(ci) * kNodeSlices + slice) * kGramPacked;
    if (s < kBlockTasks) {
        int bi = 0, rem = s;  // s -> (bi, bj), bi <= bj, row-major over the upper triangle
        while (rem >= kBlocks - bi) {
            rem -= kBlocks - bi;
            ++bi;
        }
        const int bj = bi + rem;
        float acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = 0.0f;
        float4 R = *reinterpret_cast<const float4*>(&F[0][4 * bi]);
        float4 Q = *reinterpret_cast<const float4*>(&F[0][4 * bj]);
        for (int j = 0; j < kBinsPerSlice; ++j) {
            const float4 Rn = *reinterpret_cast<const float4*>(&F[j + 1][4 * bi]);
            const float4 Qn = *reinterpret_cast<const float4*>(&F[j + 1][4 * bj]);
            const float saa = wgt[0][j], sab = wgt[1][j], sbb = wgt[2][j];
            const float r[4] = {R.x, R.y, R.z, R.w}, rn[4] = {Rn.x, Rn.y, Rn.z, Rn.w};
            const float q[4] = {Q.x, Q.y, Q.z, Q.w}, qn[4] = {Qn.x, Qn.y, Qn.z, Qn.w};
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const float A = __fmaf_rn(saa, r[a], sab * rn[a]);
                const float B = __fmaf_rn(sab, r[a], sbb * rn[a]);
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] = __fmaf_rn(A, q[b], __fmaf_rn(B, qn[b], acc[a][b]));
            }
            R = Rn;
            Q = Qn;
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int r = 4 * bi + a, q = 4 * bj + b;
                if (r <= q && q <= 64) out[packed_index(r, q)] = acc[a][b];
            }
    } else if (s < kBlockTasks + kBlocks) {  // right-hand side: column 65 on rows 4 bi .. 4 bi + 3
        const int bi = s - kBlockTasks;
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        float4 R = *reinterpret_cast<const float4*>(&F[0][4 * bi]);
        for (int j = 0; j < kBinsPerSlice; ++j) {
            const float4 Rn = *reinterpret_cast<const float4*>(&F[j + 1][4 * bi]);
            const float say = wgt[3][j], sby = wgt[4][j];
            acc[0] = __fmaf_rn(say, R.x, __fmaf_rn(sby, Rn.x, acc[0]));
            acc[1] = __fmaf_rn(say, R.y, __fmaf_rn(sby, Rn.y, acc[1]));
            acc[2] = __fmaf_rn(say, R.z, __fmaf_rn(sby, Rn.z, acc[2]));
            acc[3] = __fmaf_rn(say, R.w, __fmaf_rn(sby, Rn.w, acc[3]));
            R = Rn;
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
            if (4 * bi + a <= 64) out[packed_index(4 * bi + a, 65)] = acc[a];
    } else if (s == kBlockTasks + kBlocks) {
        out[packed_index(65, 65)] = 0.0f;  // sum y^2: not used by the fit
    }
}

}  // namespace

cudaError_t launch_lsm_mlp_features(int k, bool all_dates, int max_steps, const LsmDev* c, int c_first, int c_end,
                                    const float* nets, float* feats, uint32_t* err, cudaStream_t stream) {
    cudaGetLastError();
    if (c_end <= c_first || (all_dates && max_steps < 2)) return cudaSuccess;
    const dim3 grid(static_cast<unsigned>(c_end - c_first), kNodes / 128, all_dates ? static_cast<unsigned>(max_steps - 1) : 1u);
    lsm_mlp_nodes<<<grid, 128, 0, stream>>>(k, all_dates ? 1 : 0, c, c_first, c_end, nets, feats, err);
    return cudaGetLastError();
}

cudaError_t launch_lsm_mlp_binned(int precision, int k, int mode, const LsmDev* c, int c_first, int c_end,
                                  const uint32_t* group_contract, uint32_t g_first, uint32_t g_end, const void* store,
                                  double* cf, const int* snap_ok, const float* feats, const float* etab,
                                  unsigned long long* mom_part, float* gram_part, Welford* final_part,
                                  cudaStream_t stream) {
    cudaGetLastError();
    if (c_end <= c_first || g_end <= g_first) return cudaSuccess;
    const int n_contracts = c_end - c_first;
    const uint32_t n_groups = g_end - g_first;
    if (precision == 0)
        lsm_mlp_binned<0><<<n_groups, kBinThreads, 0, stream>>>(k, mode, c, group_contract, g_first, g_end, store, cf,
                                                                     snap_ok, etab, mom_part, final_part);
    else
        lsm_mlp_binned<1><<<n_groups, kBinThreads, 0, stream>>>(k, mode, c, group_contract, g_first, g_end, store, cf,
                                                                     snap_ok, etab, mom_part, final_part);
    if (mode & kGram)
        lsm_mlp_gram_slices<<<dim3(n_contracts, kNodeSlices), kGramThreads, 0, stream>>>(k, c, c_first, c_end, mom_part,
                                                                                         feats, gram_part);
    return cudaGetLastError();
}

}  // namespace mcdg
