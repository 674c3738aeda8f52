// gbm_paths.cu -- the batched GBM path engine (European, digital, Asian,
// barrier, lookback) as one persistent kernel per precision.
//
// Work decomposition.  Every contract's paths are cut into fixed slabs of
// kSlabPaths = 4096 paths; one (contract, slab) pair is one work item.  The
// host orders contracts longest-first and passes the running item count per
// contract (item_prefix).  A CTA of 128 threads claims items from a ticket
// counter (one atomicAdd per item, no waiting) until the list is exhausted.
// Inside a slab, thread t simulates paths slab*4096 + j*128 + t for
// j = 0..31, so the Philox counters of a warp are consecutive path indices.
//
// Determinism.  A slab's Welford triple depends only on the slab: per-thread
// accumulation in j order, then a fixed warp shuffle tree and a fixed 4-warp
// tree.  The merge kernel folds a contract's slabs in slab order with a fixed
// warp tree.  Grid size and kernel variant (register budget) only decide who
// computes an item, never the arithmetic, so results are bitwise identical
// across launch shapes.
//
// Reference semantics restated per kind (src/pricers/monte_carlo.cpp):
//   terminal products :135-149, path-dependent loop :154-177, Brownian-bridge
//   barrier :184-230, control-variate Asian :275-302, antithetic pairing
//   :73-79; payoffs include/mcd/payoffs/{european,digital,asian,barrier,
//   lookback}.hpp.
// nvcc-flags: --fmad=false
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "engine.hpp"

namespace mcdg {

namespace {

__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }

// ===========================================================================
// FP64: the reference's arithmetic (multiplicative steps, FP64 payoffs).
// ===========================================================================
__device__ __forceinline__ double draw64(const PhiloxPath& pp, uint32_t step, const PhiloxKeys& k,
                                         bool neg) {
    const double z = normal_from_bits_f64(philox_word0(pp, step, k));
    return neg ? -z : z;
}

template <int KIND>
__device__ double sample64(const DevContract& c, const PhiloxKeys& k, uint64_t path, bool neg) {
    const double phi = c.type == 0 ? 1.0 : -1.0;
    const PhiloxPath pp = philox_path(path, 0u, k);
    if constexpr (KIND == kEuropean || KIND == kDigital) {
        const double z = draw64(pp, 0u, k, neg);
        const double s = c.spot * exp(c.drift + c.vs * z);
        if constexpr (KIND == kEuropean) {
            return c.discount * dmax(phi * (s - c.strike), 0.0);
        } else {
            const bool itm = phi * (s - c.strike) > 0.0;
            return c.discount * (itm ? (c.asset ? s : c.cash) : 0.0);
        }
    } else if constexpr (KIND == kBarrierBridge) {
        const PhiloxPath pu = philox_path(path, 1u, k);
        double s = c.spot;
        bool breached = false;
        for (int step = 0; step < c.n_steps; ++step) {
            const double z = draw64(pp, static_cast<uint32_t>(step), k, neg);
            const double s_next = s * exp(c.drift + c.vs * z);
            const bool crossed = c.up ? s_next >= c.barrier : s_next <= c.barrier;
            breached = breached || crossed;
            if (!breached) {
                const double log_s = log(s);
                const double log_s_next = log(s_next);
                const double p_cross = exp(-2.0 * (c.log_barrier - log_s) *
                                           (c.log_barrier - log_s_next) / c.bb_denom);
                const double u = uniform_open01_f64(philox_word0(pu, static_cast<uint32_t>(step), k));
                breached = u < p_cross;
            }
            s = s_next;
        }
        const double vanilla = dmax(phi * (s - c.strike), 0.0);
        const bool pays = c.out ? !breached : breached;
        return c.discount * (pays ? vanilla : c.rebate);
    } else {
        double s = c.spot;
        double sum = 0.0, log_sum = 0.0, last = c.spot;
        double rmax = c.spot, rmin = c.spot;
        bool breached = false;
        for (int step = 0; step < c.n_steps; ++step) {
            const double z = draw64(pp, static_cast<uint32_t>(step), k, neg);
            s = s * exp(c.drift + c.vs * z);
            if constexpr (KIND == kAsianArith) {
                sum += s;
            } else if constexpr (KIND == kAsianGeo) {
                log_sum += log(s);
            } else if constexpr (KIND == kAsianCv) {
                sum += s;
                log_sum += log(s);
            } else if constexpr (KIND == kBarrier) {
                const bool crossed = c.up ? s >= c.barrier : s <= c.barrier;
                breached = breached || crossed;
            } else {
                rmax = dmax(rmax, s);
                rmin = dmin(rmin, s);
            }
            last = s;
        }
        const double n = static_cast<double>(c.n_steps);
        if constexpr (KIND == kAsianArith || KIND == kAsianGeo) {
            const double avg = KIND == kAsianArith ? sum / n : exp(log_sum / n);
            const double ref = c.floating ? (last - avg) : (avg - c.strike);
            return c.discount * dmax(phi * ref, 0.0);
        } else if constexpr (KIND == kAsianCv) {
            const double a = sum / n;
            const double g = exp(log_sum / n);
            const double arithmetic_payoff = c.discount * dmax(phi * (a - c.strike), 0.0);
            const double geometric_payoff = c.discount * dmax(phi * (g - c.strike), 0.0);
            return arithmetic_payoff - (geometric_payoff - c.kv_anchor);
        } else if constexpr (KIND == kBarrier) {
            const double vanilla = dmax(phi * (last - c.strike), 0.0);
            const bool pays = c.out ? !breached : breached;
            return c.discount * (pays ? vanilla : c.rebate);
        } else if constexpr (KIND == kLookbackFixed) {
            return c.discount * (c.type == 0 ? dmax(rmax - c.strike, 0.0) : dmax(c.strike - rmin, 0.0));
        } else {
            return c.discount * (c.type == 0 ? (last - rmin) : (rmax - last));
        }
    }
}

template <int KIND>
__device__ Welford slab64(const DevContract& c, const PhiloxKeys& k, uint64_t base) {
    Welford w{0ull, 0.0, 0.0};
    for (int j = 0; j < kPathsPerThread; ++j) {
        const uint64_t path = base + static_cast<uint64_t>(j * kSlabThreads) + threadIdx.x;
        if (path >= c.path_count) break;
        double sample = sample64<KIND>(c, k, path, false);
        if (c.antithetic) {
            const double sample2 = sample64<KIND>(c, k, path, true);
            sample = 0.5 * (sample + sample2);
        }
        welford_add(w, sample);
    }
    return w;
}

// ===========================================================================
// FP32: log-space paths x = ln(S/S0), FP32 payoffs, FP64 accumulation.
// ===========================================================================
__device__ __forceinline__ float draw32(const PhiloxPath& pp, uint32_t step, const PhiloxKeys& k,
                                        bool neg) {
    const float z = normal_from_bits_f32(philox_word0(pp, step, k));
    return neg ? -z : z;
}

// Path-dependent products (Asians, discrete barrier, lookbacks), NP paths
// (or antithetic halves) at once: their draws are independent dependency
// chains, so interleaving them gives every warp NP-fold instruction-level
// parallelism.  Each path's arithmetic is the single-path one, so the samples
// do not depend on NP.
template <int KIND, int NP>
__device__ __forceinline__ void path_dependent32(const DevContract& c, const PhiloxKeys& k,
                                                 const PhiloxPath (&pp)[NP], const bool (&neg)[NP],
                                                 double (&out)[NP]) {
    const float phi = c.type == 0 ? 1.0f : -1.0f;
    const float mu = static_cast<float>(c.drift);
    const float sg = static_cast<float>(c.vs);
    const float s0 = static_cast<float>(c.spot);
    const float strike = static_cast<float>(c.strike);
    const float lnh = static_cast<float>(c.log_h_rel);
    float x[NP], acc[NP], acc2[NP], xmax[NP], xmin[NP];  // log path, sum of S/S0, sum of x, extrema
    bool breached[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        x[p] = acc[p] = acc2[p] = xmax[p] = xmin[p] = 0.0f;
        breached[p] = false;
    }
    for (int step = 0; step < c.n_steps; ++step) {
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            const float z = draw32(pp[p], static_cast<uint32_t>(step), k, neg[p]);
            x[p] = __fmaf_rn(sg, z, x[p] + mu);
            if constexpr (KIND == kAsianArith) {
                acc[p] += __expf(x[p]);
            } else if constexpr (KIND == kAsianGeo) {
                acc2[p] += x[p];
            } else if constexpr (KIND == kAsianCv) {
                acc[p] += __expf(x[p]);
                acc2[p] += x[p];
            } else if constexpr (KIND == kBarrier) {
                const bool crossed = c.up ? x[p] >= lnh : x[p] <= lnh;
                breached[p] = breached[p] || crossed;
            } else {
                xmax[p] = fmaxf(xmax[p], x[p]);
                xmin[p] = fminf(xmin[p], x[p]);
            }
        }
    }
    const float inv_n = 1.0f / static_cast<float>(c.n_steps);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const float last = s0 * __expf(x[p]);
        if constexpr (KIND == kAsianArith || KIND == kAsianGeo) {
            const float avg = KIND == kAsianArith ? s0 * (acc[p] * inv_n) : s0 * __expf(acc2[p] * inv_n);
            const float ref = c.floating ? (last - avg) : (avg - strike);
            out[p] = c.discount * static_cast<double>(fmaxf(phi * ref, 0.0f));
        } else if constexpr (KIND == kAsianCv) {
            const float a = s0 * (acc[p] * inv_n);
            const float g = s0 * __expf(acc2[p] * inv_n);
            const double ap = c.discount * static_cast<double>(fmaxf(phi * (a - strike), 0.0f));
            const double gp = c.discount * static_cast<double>(fmaxf(phi * (g - strike), 0.0f));
            out[p] = ap - (gp - c.kv_anchor);
        } else if constexpr (KIND == kBarrier) {
            const float vanilla = fmaxf(phi * (last - strike), 0.0f);
            const bool pays = c.out ? !breached[p] : breached[p];
            out[p] = c.discount * static_cast<double>(pays ? vanilla : static_cast<float>(c.rebate));
        } else if constexpr (KIND == kLookbackFixed) {
            const float v = c.type == 0 ? fmaxf(s0 * __expf(xmax[p]) - strike, 0.0f)
                                        : fmaxf(strike - s0 * __expf(xmin[p]), 0.0f);
            out[p] = c.discount * static_cast<double>(v);
        } else {
            const float v = c.type == 0 ? (last - s0 * __expf(xmin[p])) : (s0 * __expf(xmax[p]) - last);
            out[p] = c.discount * static_cast<double>(v);
        }
    }
}

// Returns the discounted sample in FP64 (the payoff itself is FP32).
template <int KIND>
__device__ double sample32(const DevContract& c, const PhiloxKeys& k, uint64_t path, bool neg) {
    const float phi = c.type == 0 ? 1.0f : -1.0f;
    const float mu = static_cast<float>(c.drift);
    const float sg = static_cast<float>(c.vs);
    const float s0 = static_cast<float>(c.spot);
    const float strike = static_cast<float>(c.strike);
    const PhiloxPath pp = philox_path(path, 0u, k);
    if constexpr (KIND == kEuropean || KIND == kDigital) {
        const float z = draw32(pp, 0u, k, neg);
        const float s = s0 * __expf(__fmaf_rn(sg, z, mu));
        float payoff;
        if constexpr (KIND == kEuropean) {
            payoff = fmaxf(phi * (s - strike), 0.0f);
        } else {
            const bool itm = phi * (s - strike) > 0.0f;
            payoff = itm ? (c.asset ? s : static_cast<float>(c.cash)) : 0.0f;
        }
        return c.discount * static_cast<double>(payoff);
    } else if constexpr (KIND == kBarrierBridge) {
        const PhiloxPath pu = philox_path(path, 1u, k);
        const float lnh = static_cast<float>(c.log_h_rel);
        const float inv_denom = static_cast<float>(-2.0 / c.bb_denom);
        float x = 0.0f;
        bool breached = false;
        for (int step = 0; step < c.n_steps; ++step) {
            const float z = draw32(pp, static_cast<uint32_t>(step), k, neg);
            const float x_next = __fmaf_rn(sg, z, x + mu);
            const bool crossed = c.up ? x_next >= lnh : x_next <= lnh;
            breached = breached || crossed;
            if (!breached) {
                const float p_cross = __expf(inv_denom * (lnh - x) * (lnh - x_next));
                const float u = uniform_from_bits_f32(philox_word0(pu, static_cast<uint32_t>(step), k));
                breached = u < p_cross;
            }
            x = x_next;
        }
        const float s = s0 * __expf(x);
        const float vanilla = fmaxf(phi * (s - strike), 0.0f);
        const bool pays = c.out ? !breached : breached;
        return c.discount * static_cast<double>(pays ? vanilla : static_cast<float>(c.rebate));
    } else {
        const PhiloxPath pps[1] = {pp};
        const bool negs[1] = {neg};
        double out[1];
        path_dependent32<KIND, 1>(c, k, pps, negs, out);
        return out[0];
    }
}

template <int KIND>
__device__ Welford slab32(const DevContract& c, const PhiloxKeys& k, uint64_t base) {
    unsigned count = 0;
    double s1 = 0.0, s2 = 0.0;
    constexpr bool kPathDependent = KIND != kEuropean && KIND != kDigital && KIND != kBarrierBridge;
    if constexpr (kPathDependent) {
        if (c.antithetic) {  // the two halves of an antithetic sample share their draws
            for (int j = 0; j < kPathsPerThread; ++j) {
                const uint64_t path = base + static_cast<uint64_t>(j * kSlabThreads) + threadIdx.x;
                if (path >= c.path_count) break;
                const PhiloxPath pp = philox_path(path, 0u, k);
                const PhiloxPath pps[2] = {pp, pp};
                const bool negs[2] = {false, true};
                double out[2];
                path_dependent32<KIND, 2>(c, k, pps, negs, out);
                const double sample = 0.5 * (out[0] + out[1]);
                ++count;
                s1 += sample;
                s2 = fma(sample, sample, s2);
            }
        } else {  // two paths at a time, in path order
            for (int j = 0; j < kPathsPerThread; j += 2) {
                const uint64_t path = base + static_cast<uint64_t>(j * kSlabThreads) + threadIdx.x;
                if (path >= c.path_count) break;
                const uint64_t path2 = path + kSlabThreads;
                double out[2];
                if (path2 < c.path_count) {
                    const PhiloxPath pps[2] = {philox_path(path, 0u, k), philox_path(path2, 0u, k)};
                    const bool negs[2] = {false, false};
                    path_dependent32<KIND, 2>(c, k, pps, negs, out);
                } else {
                    const PhiloxPath pps[1] = {philox_path(path, 0u, k)};
                    const bool negs[1] = {false};
                    double one[1];
                    path_dependent32<KIND, 1>(c, k, pps, negs, one);
                    out[0] = one[0];
                }
                const int n_here = path2 < c.path_count ? 2 : 1;
                for (int p = 0; p < n_here; ++p) {
                    ++count;
                    s1 += out[p];
                    s2 = fma(out[p], out[p], s2);
                }
            }
        }
        return welford_from_sums(count, s1, s2);
    }
    for (int j = 0; j < kPathsPerThread; ++j) {
        const uint64_t path = base + static_cast<uint64_t>(j * kSlabThreads) + threadIdx.x;
        if (path >= c.path_count) break;
        double sample = sample32<KIND>(c, k, path, false);
        if (c.antithetic) {
            const double sample2 = sample32<KIND>(c, k, path, true);
            sample = 0.5 * (sample + sample2);
        }
        ++count;
        s1 += sample;
        s2 = fma(sample, sample, s2);
    }
    return welford_from_sums(count, s1, s2);
}

template <int PREC>
__device__ Welford run_slab(const DevContract& c, uint64_t base) {
    const PhiloxKeys k = philox_keys(c.seed);
#define MCD_KIND_CASE(K)                                                  \
    case K:                                                               \
        return PREC == 0 ? slab64<K>(c, k, base) : slab32<K>(c, k, base);
    switch (c.kind) {
        MCD_KIND_CASE(kEuropean)
        MCD_KIND_CASE(kDigital)
        MCD_KIND_CASE(kAsianArith)
        MCD_KIND_CASE(kAsianGeo)
        MCD_KIND_CASE(kAsianCv)
        MCD_KIND_CASE(kBarrier)
        MCD_KIND_CASE(kBarrierBridge)
        MCD_KIND_CASE(kLookbackFixed)
        default:
            return PREC == 0 ? slab64<kLookbackFloating>(c, k, base)
                             : slab32<kLookbackFloating>(c, k, base);
    }
#undef MCD_KIND_CASE
}

template <int PREC, int MINB>
__global__ void __launch_bounds__(kSlabThreads, MINB)
    path_kernel(const DevContract* __restrict__ contracts, int n_contracts,
                const uint32_t* __restrict__ item_prefix, uint32_t* __restrict__ ticket,
                Welford* __restrict__ partials, uint32_t* __restrict__ error_flag) {
    __shared__ uint32_t s_item, s_total;
    __shared__ Welford s_warp[kSlabThreads / 32];
    __shared__ DevContract s_contract;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    // The batch's item count is the prefix's last entry (read from memory, so
    // a captured launch serves every path count of the same contract count).
    if (threadIdx.x == 0) s_total = item_prefix[n_contracts];
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(ticket, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= s_total) return;
        // Largest contract index c with item_prefix[c] <= item (empty
        // contracts share their successor's prefix and are skipped).
        int lo = 0, hi = n_contracts;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (item_prefix[mid] <= item) lo = mid; else hi = mid;
        }
        static_assert(sizeof(DevContract) % 4 == 0 && sizeof(DevContract) / 4 <= kSlabThreads,
                      "contract staging assumes one word per thread");
        if (threadIdx.x < sizeof(DevContract) / 4)
            reinterpret_cast<uint32_t*>(&s_contract)[threadIdx.x] =
                reinterpret_cast<const uint32_t*>(&contracts[lo])[threadIdx.x];
        __syncthreads();
        const DevContract& c = s_contract;
        const uint32_t slab = item - item_prefix[lo];
        if (slab >= c.n_slabs) {  // planning invariant broken: record, skip the item
            if (threadIdx.x == 0) atomicOr(error_flag, 1u);
            __syncthreads();
            continue;
        }
        Welford w = run_slab<PREC>(c, static_cast<uint64_t>(slab) * kSlabPaths);
        w = welford_warp_reduce(w);
        if (lane == 0) s_warp[warp] = w;
        __syncthreads();
        if (threadIdx.x == 0) {
            partials[item] = welford_merge(welford_merge(s_warp[0], s_warp[1]),
                                           welford_merge(s_warp[2], s_warp[3]));
        }
        __syncthreads();
    }
}

struct DevMcResult {
    double price;
    double standard_error;
    unsigned long long path_count;
};

// One warp per contract: lanes fold slabs lane, lane+32, ... in slab order,
// then a fixed shuffle tree; results go to the caller's positions.
__global__ void merge_kernel(const DevContract* __restrict__ contracts, int n_contracts,
                             const uint32_t* __restrict__ item_prefix,
                             const Welford* __restrict__ partials, DevMcResult* __restrict__ results) {
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp_global >= n_contracts) return;
    const uint32_t begin = item_prefix[warp_global];
    const uint32_t count = contracts[warp_global].n_slabs;
    Welford w{0ull, 0.0, 0.0};
    for (uint32_t s = lane; s < count; s += 32) w = welford_merge(w, partials[begin + s]);
    w = welford_warp_reduce(w);
    if (lane == 0) {
        DevMcResult r;
        r.price = w.mean;
        const double var = w.count < 2 ? 0.0 : w.m2 / static_cast<double>(w.count - 1);
        r.standard_error = w.count == 0 ? 0.0 : sqrt(var / static_cast<double>(w.count));
        r.path_count = w.count;
        results[contracts[warp_global].orig_index] = r;
    }
}

// ---- parity kernels ----------------------------------------------------------
__global__ void philox_kernel(const uint4* __restrict__ counters, const uint2* __restrict__ keys,
                              size_t n, uint4* __restrict__ out) {
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint2 k = keys[i];
    out[i] = philox4x32_10(counters[i], k.x, k.y);
}

__global__ void draws_kernel(uint64_t seed, uint64_t path_begin, uint64_t n_paths,
                             uint32_t draw_begin, uint32_t n_draws, int stream_id, int precision,
                             double* __restrict__ out) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n_paths * n_draws) return;
    const uint64_t p = i / n_draws;
    const uint32_t d = static_cast<uint32_t>(i % n_draws);
    const PhiloxKeys k = philox_keys(seed);
    const PhiloxPath pp = philox_path(path_begin + p, static_cast<uint32_t>(stream_id), k);
    const uint32_t bits = philox_word0(pp, draw_begin + d, k);
    double v;
    if (stream_id == 0) {
        v = precision == 0 ? normal_from_bits_f64(bits) : static_cast<double>(normal_from_bits_f32(bits));
    } else {
        v = precision == 0 ? uniform_open01_f64(bits) : static_cast<double>(uniform_from_bits_f32(bits));
    }
    out[i] = v;
}

template <int PREC, int MINB>
cudaError_t launch_one(int grid, const DevContract* c, int n, const uint32_t* prefix, uint32_t* ticket,
                       Welford* partials, uint32_t* err, cudaStream_t stream) {
    cudaGetLastError();  // report this launch only
    path_kernel<PREC, MINB><<<grid, kSlabThreads, 0, stream>>>(c, n, prefix, ticket, partials, err);
    return cudaGetLastError();
}

template <int PREC>
cudaError_t launch_prec(int variant, int grid, const DevContract* c, int n, const uint32_t* prefix,
                        uint32_t* ticket, Welford* partials, uint32_t* err, cudaStream_t stream) {
    switch (variant) {
        case 0: return launch_one<PREC, 4>(grid, c, n, prefix, ticket, partials, err, stream);
        case 1: return launch_one<PREC, 8>(grid, c, n, prefix, ticket, partials, err, stream);
        case 2: return launch_one<PREC, 12>(grid, c, n, prefix, ticket, partials, err, stream);
        case 3: return launch_one<PREC, 16>(grid, c, n, prefix, ticket, partials, err, stream);
        default: return launch_one<PREC, 6>(grid, c, n, prefix, ticket, partials, err, stream);
    }
}

template <int PREC>
cudaError_t occupancy_prec(int variant, int* blocks) {
    switch (variant) {
        case 0: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, path_kernel<PREC, 4>, kSlabThreads, 0);
        case 1: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, path_kernel<PREC, 8>, kSlabThreads, 0);
        case 2: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, path_kernel<PREC, 12>, kSlabThreads, 0);
        case 3: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, path_kernel<PREC, 16>, kSlabThreads, 0);
        default: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, path_kernel<PREC, 6>, kSlabThreads, 0);
    }
}

// Digest of a word array: sum over i of splitmix64's finaliser (Steele, Lea
// and Flood, OOPSLA 2014) applied to word_i + (i + 1) * golden-ratio constant.
// Integer sums do not depend on the order of the additions, so the digest is
// the same for any grid; one CTA suffices for a contract list.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void __launch_bounds__(256) words_digest_kernel(const uint64_t* __restrict__ words, size_t n,
                                                           uint64_t* __restrict__ out) {
    __shared__ uint64_t part[8];
    uint64_t acc = 0;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) acc += mix64(words[i] + (i + 1) * 0x9E3779B97F4A7C15ull);
    for (int off = 16; off >= 1; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t total = 0;
        for (int w = 0; w < 8; ++w) total += part[w];
        *out = total;
    }
}

}  // namespace

cudaError_t launch_words_digest(const uint64_t* words, size_t n_words, uint64_t* out, cudaStream_t stream) {
    cudaGetLastError();
    words_digest_kernel<<<1, 256, 0, stream>>>(words, n_words, out);
    return cudaGetLastError();
}

cudaError_t launch_path_kernel(int precision, int variant, int grid, const DevContract* contracts,
                               int n_contracts, const uint32_t* item_prefix, uint32_t* ticket,
                               Welford* partials, uint32_t* error_flag, cudaStream_t stream) {
    if (precision == 0)
        return launch_prec<0>(variant, grid, contracts, n_contracts, item_prefix, ticket, partials,
                              error_flag, stream);
    return launch_prec<1>(variant, grid, contracts, n_contracts, item_prefix, ticket, partials,
                          error_flag, stream);
}

cudaError_t path_kernel_occupancy(int precision, int variant, int* blocks_per_sm) {
    return precision == 0 ? occupancy_prec<0>(variant, blocks_per_sm)
                          : occupancy_prec<1>(variant, blocks_per_sm);
}

cudaError_t launch_merge_kernel(const DevContract* contracts, int n_contracts,
                                const uint32_t* item_prefix, const Welford* partials,
                                void* results, cudaStream_t stream) {
    const int threads = 256;
    const int blocks = (n_contracts * 32 + threads - 1) / threads;
    if (blocks == 0) return cudaSuccess;
    cudaGetLastError();
    merge_kernel<<<blocks, threads, 0, stream>>>(contracts, n_contracts, item_prefix, partials,
                                                 static_cast<DevMcResult*>(results));
    return cudaGetLastError();
}

cudaError_t launch_philox_kernel(const uint32_t* counters, const uint32_t* keys, size_t n,
                                 uint32_t* out, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    const int threads = 256;
    const unsigned blocks = static_cast<unsigned>((n + threads - 1) / threads);
    cudaGetLastError();
    philox_kernel<<<blocks, threads, 0, stream>>>(reinterpret_cast<const uint4*>(counters),
                                                  reinterpret_cast<const uint2*>(keys), n,
                                                  reinterpret_cast<uint4*>(out));
    return cudaGetLastError();
}

cudaError_t launch_draws_kernel(uint64_t seed, uint64_t path_begin, uint64_t n_paths,
                                uint32_t draw_begin, uint32_t n_draws, int stream_id,
                                int precision, double* out, cudaStream_t stream) {
    const uint64_t total = n_paths * n_draws;
    if (total == 0) return cudaSuccess;
    const int threads = 256;
    const unsigned blocks = static_cast<unsigned>((total + threads - 1) / threads);
    cudaGetLastError();
    draws_kernel<<<blocks, threads, 0, stream>>>(seed, path_begin, n_paths, draw_begin, n_draws,
                                                 stream_id, precision, out);
    return cudaGetLastError();
}

}  // namespace mcdg
