// lsm_frozen.cu -- replay of a frozen Longstaff-Schwartz exercise policy,
// streamed: no path storage, one pass, several scenarios per path.
//
// Reference: reprice_against_frozen_policy (src/pricers/lsm.cpp:151-213)
// simulates the paths, seeds the cash flows with the terminal intrinsic and
// walks dates n-1..1 backwards: discount, then exercise where the frozen
// coefficients say so.  With the coefficients fixed, the cash flow a path ends
// with is the exercise value at the EARLIEST date whose test passes (later
// overwrites are earlier dates), or the terminal intrinsic, multiplied by the
// one-date discount once per date before it.  So a path can be priced
// forwards, stopping at its first exercise: the same multiplications in the
// same order give the same bits, and nothing is stored.  Frozen-boundary
// Greeks need the same replay at bumped inputs on the same draws (the
// reference's tests/lsm_test.cpp:138-185 calls the replay at S +/- h): each
// thread carries every scenario's state along one path, sharing the draws.
//
// Work layout, reductions and per-chunk partials are those of the backward
// pass's last date (lsm.cu): chunks of 1024 paths, 256 threads, a fixed
// reduction tree per chunk (FP64 Welford on the FP64 path, compensated FP32
// sums up to the warp on the FP32 path), chunks merged in order per contract
// -- the base scenario reproduces the fitted price bit for bit.
//
// nvcc-flags: --fmad=false
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "lsm.hpp"

namespace mcdg {

namespace {

__device__ __forceinline__ double intrinsic(double s, double k, int type) {
    const double x = (type == 0 ? 1.0 : -1.0) * (s - k);
    return (x < 0.0) ? 0.0 : x;
}

// Weighted Laguerre basis (src/pricers/lsm.cpp:21-25), FP64, and the FP32
// path's version; both as in the backward pass, so decisions agree with it.
__device__ __forceinline__ double continuation64(double s, double strike, const double g[4]) {
    const double x = s / strike;
    const double e = exp(-x / 2.0);
    double cont = 0.0;
    cont += g[0] * e;
    cont += g[1] * (e * (1.0 - x));
    cont += g[2] * (e * (1.0 - 2.0 * x + 0.5 * x * x));
    cont += g[3] * (e * (1.0 - 3.0 * x + 1.5 * x * x - x * x * x / 6.0));
    return cont;
}

// Scenarios by volatility: {base, spot+h, spot-h} share the base's GBM step
// constants (and so its growth factors), vol+h and vol-h have their own.
template <int NS>
constexpr int kGroups = NS == 1 ? 1 : 3;
__device__ __forceinline__ constexpr int group_of(int q) { return q < 3 ? 0 : q - 2; }
__device__ __forceinline__ constexpr int group_lead(int gi) { return gi == 0 ? 0 : gi + 2; }
template <int NS>
__device__ __forceinline__ bool group_live(const bool (&live)[NS], int gi) {
    bool any = false;
#pragma unroll
    for (int q = 0; q < NS; ++q) any = any || (group_of(q) == gi && live[q]);
    return any;
}

// One path, NS scenarios: cash flow of each scenario, discounted to t = 0.
template <int NS>
__device__ void replay64(const LsmDev& c, const FrozenDev& f, const LsmReg* __restrict__ rg, const PhiloxPath& pp,
                         const PhiloxKeys& k, double (&v)[NS]) {
    double s[NS];
    int stop[NS];
    bool live[NS];
#pragma unroll
    for (int q = 0; q < NS; ++q) {
        s[q] = f.sc[q].spot;
        stop[q] = c.n_steps;
        live[q] = true;
        v[q] = 0.0;
    }
    int n_live = NS;
    for (int d = 0; d < c.n_steps && n_live > 0; ++d) {
        const double z = normal_from_bits_f64(philox_word0(pp, static_cast<uint32_t>(d), k));
        const int date = d + 1;
        const bool test = date < c.n_steps && rg[date].has == 1;
        double g[4] = {0.0, 0.0, 0.0, 0.0};
        if (test) {
            g[0] = rg[date].gamma[0];
            g[1] = rg[date].gamma[1];
            g[2] = rg[date].gamma[2];
            g[3] = rg[date].gamma[3];
        }
        // one growth factor per volatility group (src/models/gbm.cpp:7-12):
        // the spot scenarios share the base's, bit for bit
        double gr[kGroups<NS>];
#pragma unroll
        for (int gi = 0; gi < kGroups<NS>; ++gi) {
            gr[gi] = 1.0;
            if (group_live<NS>(live, gi))
                gr[gi] = exp(f.sc[group_lead(gi)].drift + f.sc[group_lead(gi)].vs * z);
        }
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            if (!live[q]) continue;
            s[q] = s[q] * gr[group_of(q)];
            if (test) {
                const double ex = intrinsic(s[q], c.strike, c.type);
                if (ex > 0.0 && ex > continuation64(s[q], c.strike, g)) {
                    v[q] = ex;
                    stop[q] = date;
                    live[q] = false;
                    --n_live;
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < NS; ++q) {
        if (live[q]) v[q] = intrinsic(s[q], c.strike, c.type);
        for (int t = 0; t < stop[q]; ++t) v[q] *= c.disc;
    }
}

template <int NS>
__device__ void replay32(const LsmDev& c, const FrozenDev& f, const LsmReg* __restrict__ rg, const PhiloxPath& pp,
                         const PhiloxKeys& k, float (&v)[NS]) {
    float x[kGroups<NS>], s[NS];
    int stop[NS];
    bool live[NS];
#pragma unroll
    for (int gi = 0; gi < kGroups<NS>; ++gi) x[gi] = 0.0f;
#pragma unroll
    for (int q = 0; q < NS; ++q) {
        s[q] = f.sc[q].spot_f;
        stop[q] = c.n_steps;
        live[q] = true;
        v[q] = 0.0f;
    }
    const float phi = c.phi_f, strike = c.strike_f, inv_k = c.inv_strike_f;
    int n_live = NS;
    for (int d = 0; d < c.n_steps && n_live > 0; ++d) {
        const float z = normal_from_bits_f32(philox_word0(pp, static_cast<uint32_t>(d), k));
        const int date = d + 1;
        const bool test = date < c.n_steps && rg[date].has == 1;
        float g[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (test) {
            g[0] = rg[date].poly_f[0];
            g[1] = rg[date].poly_f[1];
            g[2] = rg[date].poly_f[2];
            g[3] = rg[date].poly_f[3];
        }
        // the FP32 forward pass's log-space step (lsm.cu, lsm_forward), one
        // log path per volatility group
        float e[kGroups<NS>];
#pragma unroll
        for (int gi = 0; gi < kGroups<NS>; ++gi) {
            e[gi] = 1.0f;
            if (group_live<NS>(live, gi)) {
                const FrozenScenario& g0 = f.sc[group_lead(gi)];
                x[gi] = __fmaf_rn(g0.sg_f, z, x[gi] + g0.mu_f);
                e[gi] = __expf(x[gi]);
            }
        }
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            if (!live[q]) continue;
            s[q] = f.sc[q].spot_f * e[group_of(q)];
            if (test) {
                const float ex = phi * (s[q] - strike);
                if (ex > 0.0f && ex > continuation_poly32(s[q], inv_k, g)) {
                    v[q] = ex;
                    stop[q] = date;
                    live[q] = false;
                    --n_live;
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < NS; ++q) {
        if (live[q]) v[q] = fmaxf(phi * (s[q] - strike), 0.0f);
        for (int t = 0; t < stop[q]; ++t) v[q] *= c.disc_f;
    }
}

// Per chunk: NS scenario averages (and, for the five-scenario form, the
// per-path central differences of delta, gamma and vega) as Welford partials.
// The FP32 five-scenario form runs 384 threads per SM at most 85 registers
// each (measured 1.3x faster than 512 threads at 106 registers on the 20-put
// grid: paths that exercise early leave the pass latency-bound).
template <int PREC, int NS>
__global__ void __launch_bounds__(kLsmThreads, ((PREC == 1 && NS > 1) ? 3 : 2) * (256 / kLsmThreads))
    lsm_frozen_stream(const LsmDev* __restrict__ cs, const FrozenDev* __restrict__ fz,
                      const uint32_t* __restrict__ chunk_contract, uint32_t total_chunks,
                      const LsmReg* __restrict__ reg, Welford* __restrict__ part) {
    constexpr int NW = NS == 1 ? 1 : kFrozenOutputs;
    __shared__ Welford swf[kLsmThreads / 32][NW];
    __shared__ Sum64 s64[NW][kLsmThreads / 32];
    const uint32_t chunk = blockIdx.x;
    if (chunk >= total_chunks) return;
    const uint32_t ci = chunk_contract[chunk];
    const LsmDev c = cs[ci];
    const FrozenDev& f = fz[ci];
    const LsmReg* rg = reg + c.reg_offset;
    const PhiloxKeys k = philox_keys(c.seed);
    const uint32_t local = chunk - c.chunk_begin;
    if constexpr (PREC == 0) {
        Welford w[NW];
#pragma unroll
        for (int q = 0; q < NW; ++q) w[q] = Welford{0ull, 0.0, 0.0};
        for (int j = 0; j < kLsmChunk / kLsmThreads; ++j) {
            const uint64_t i = static_cast<uint64_t>(local) * kLsmChunk + j * kLsmThreads + threadIdx.x;
            if (i >= c.path_count) break;
            double v[NS];
            replay64<NS>(c, f, rg, philox_path(i, 0u, k), k, v);
#pragma unroll
            for (int q = 0; q < NS; ++q) welford_add(w[q], v[q]);
            if constexpr (NS == kFrozenScenarios) {
                welford_add(w[5], (v[1] - v[2]) * f.inv_2hs);
                welford_add(w[6], ((v[1] - v[0]) - (v[0] - v[2])) * f.inv_hs2);
                welford_add(w[7], (v[3] - v[4]) * f.inv_2hv);
            }
        }
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            const Welford r = welford_warp_reduce(w[q]);
            if ((threadIdx.x & 31) == 0) swf[threadIdx.x >> 5][q] = r;
        }
        __syncthreads();
        if (threadIdx.x < NW) {
            const int q = threadIdx.x;
            Welford m = swf[0][q];
            for (int wi = 1; wi < kLsmThreads / 32; ++wi) m = welford_merge(m, swf[wi][q]);
            part[static_cast<uint64_t>(chunk) * NW + q] = m;
        }
    } else {
        // FP32 cash flows; compensated FP32 sums per thread and over the
        // warp tree (Sum32, as the backward pass's last date, so the base
        // scenario keeps its bits), FP64 from the warp sums on.
        Sum32 acc[NW];
#pragma unroll
        for (int q = 0; q < NW; ++q) acc[q] = Sum32{0u, 0.0f, 0.0f, 0.0f, 0.0f};
        for (int j = 0; j < kLsmChunk / kLsmThreads; ++j) {
            const uint64_t i = static_cast<uint64_t>(local) * kLsmChunk + j * kLsmThreads + threadIdx.x;
            if (i >= c.path_count) break;
            float v[NS];
            replay32<NS>(c, f, rg, philox_path(i, 0u, k), k, v);
#pragma unroll
            for (int q = 0; q < NS; ++q) sum32_add(acc[q], v[q]);
            if constexpr (NS == kFrozenScenarios) {
                sum32_add(acc[5], (v[1] - v[2]) * f.inv_2hs_f);
                sum32_add(acc[6], ((v[1] - v[0]) - (v[0] - v[2])) * f.inv_hs2_f);
                sum32_add(acc[7], (v[3] - v[4]) * f.inv_2hv_f);
            }
        }
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            const Sum32 r = sum32_warp_reduce(acc[q]);
            if ((threadIdx.x & 31) == 0) s64[q][threadIdx.x >> 5] = sum32_wide(r);
        }
        __syncthreads();
        if (threadIdx.x < NW)
            part[static_cast<uint64_t>(chunk) * NW + threadIdx.x] = sum64_fold<kLsmThreads / 32>(s64[threadIdx.x]);
    }
}

// Per (contract, output): chunk partials merged in chunk order (lane-strided,
// then the fixed warp tree, as lsm_finish), mean, standard error, count.
__global__ void lsm_frozen_finish(const LsmDev* __restrict__ cs, int n_contracts, int nw,
                                  const Welford* __restrict__ part, double* __restrict__ out) {
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wid >= n_contracts * nw) return;
    const int ci = wid / nw, q = wid % nw;
    const LsmDev c = cs[ci];
    Welford w{0ull, 0.0, 0.0};
    for (uint32_t ch = lane; ch < c.n_chunks; ch += 32)
        w = welford_merge(w, part[static_cast<uint64_t>(c.chunk_begin + ch) * nw + q]);
    w = welford_warp_reduce(w);
    if (lane != 0) return;
    const double var = w.count < 2 ? 0.0 : w.m2 / static_cast<double>(w.count - 1);
    double* o = out + (static_cast<size_t>(ci) * nw + q) * 3;
    o[0] = w.mean;
    o[1] = w.count == 0 ? 0.0 : sqrt(var / static_cast<double>(w.count));
    o[2] = static_cast<double>(w.count);
}

}  // namespace

cudaError_t launch_lsm_frozen(int precision, int n_scenarios, const LsmDev* c, const FrozenDev* f,
                              int n_contracts, const uint32_t* chunk_contract, uint32_t total_chunks,
                              const LsmReg* reg, Welford* partials, double* out, cudaStream_t stream) {
    cudaGetLastError();
    if (n_scenarios != 1 && n_scenarios != kFrozenScenarios) return cudaErrorInvalidValue;
    if (total_chunks) {
        const bool five = n_scenarios == kFrozenScenarios;
        if (precision == 0) {
            if (five) lsm_frozen_stream<0, kFrozenScenarios><<<total_chunks, kLsmThreads, 0, stream>>>(c, f, chunk_contract, total_chunks, reg, partials);
            else lsm_frozen_stream<0, 1><<<total_chunks, kLsmThreads, 0, stream>>>(c, f, chunk_contract, total_chunks, reg, partials);
        } else {
            if (five) lsm_frozen_stream<1, kFrozenScenarios><<<total_chunks, kLsmThreads, 0, stream>>>(c, f, chunk_contract, total_chunks, reg, partials);
            else lsm_frozen_stream<1, 1><<<total_chunks, kLsmThreads, 0, stream>>>(c, f, chunk_contract, total_chunks, reg, partials);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    const int nw = n_scenarios == 1 ? 1 : kFrozenOutputs;
    const int warps = n_contracts * nw;
    lsm_frozen_finish<<<(warps * 32 + 127) / 128, 128, 0, stream>>>(c, n_contracts, nw, partials, out);
    return cudaGetLastError();
}

}  // namespace mcdg
