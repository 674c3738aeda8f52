// qmc.cu -- Sobol quasi-Monte Carlo pricing of a batch of GBM contracts with
// Brownian-bridge paths, as one persistent kernel per precision.
//
// Reference semantics: src/core/sobol.cpp:83-97 (Gray-code point, indices
// 1..N as in src/pricers/qmc.cpp:20-25), src/models/brownian_bridge_path.cpp
// :20-77 (bisection bridge: terminal point from dimension 0, then breadth-
// first midpoints, dimension = draw number), src/pricers/qmc.cpp:15-57
// (European: one dimension and the exact terminal spot; Asian: dims =
// monitoring points, price = mean of discounted payoffs, no standard error).
// The same bridge paths also price the other batch products (geometric Asian,
// discrete barrier, lookback), which the reference prices by Monte Carlo only.
//
// Work decomposition, slab reduction and merge are the path engine's
// (gbm_paths.cu): (contract, 4096-path slab) items claimed from a ticket,
// fixed trees, so results do not depend on the launch shape.
//
// Per path, the bridge program (qmc.hpp) is walked in depth-first pre-order:
// each node takes its Sobol coordinate (XOR of the direction numbers of the
// set bits of the Gray code), the inverse normal, and the bridge update from
// the two ancestor values it sits between; spots are folded into the payoff
// aggregates at once (sum, log-sum, extrema, barrier test, terminal spot), so
// no path array is kept: one value per tree depth.
//
// nvcc-flags: --fmad=false
#include <cuda_runtime.h>

#include <type_traits>

#include "device_common.cuh"
#include "engine.hpp"
#include "qmc.hpp"

namespace mcdg {

namespace {

__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }

// Sobol coordinate bits of `dim` for Gray code `gray` (sobol.cpp:87-94;
// directions[dim * 32 + b] is the reference's v[b + 1]).
__device__ __forceinline__ uint32_t sobol_x(const uint32_t* __restrict__ dirs, uint32_t dim, uint32_t gray) {
    const uint32_t* v = dirs + dim * kSobolBits;
    uint32_t x = 0;
    while (gray != 0u) {
        const int b = __ffs(gray) - 1;
        x ^= __ldg(v + b);
        gray &= gray - 1u;
    }
    return x;
}

// Sobol coordinates of a warp's 32 consecutive indices.  Path p has index
// I = p + 1; a warp's paths are B .. B+31 with B a multiple of 32, so
// I = B' + low with B' in {B, B + 32} (B + 32 for the last lane only) and
// low < 32, and gray(B' + low) = gray(B') ^ gray(low).  The coordinate is
// linear in the Gray-code bits over GF(2): x(I) = X(B') ^ Y(low).  X is
// computed once per warp and dimension (lanes share the dimensions) into
// shared memory; Y depends on the lane and dimension only and is a table
// (kSobolDims x 32, uploaded with the directions).  A draw is then one XOR
// of two loads instead of a loop over the set bits of the index.
struct SobolLane {
    const uint32_t* x;  // this warp's X for this lane's B' (indexed by dimension)
    const uint32_t* y;  // Y table column of this lane (stride 32)
    __device__ __forceinline__ uint32_t operator()(uint32_t dim) const { return x[dim] ^ __ldg(y + dim * 32u); }
};

constexpr int kSxStride = kSobolDims + 1;  // +1 word: the last lane's row sits in another bank

// Bridge coefficients of one contract in program order, FP64 kernel.
struct QmcTables64 {
    BridgeNode node[kSobolDims];
    double a[kSobolDims], sd[kSobolDims], drift[kSobolDims];
};

// FP32 kernel: one 16-byte record per node, read with one shared-memory load
// (the same address across the warp): the FP32 coefficients and the node's
// Sobol dimension and slots packed into the last word.
struct QmcTables32 {
    float4 node[kSobolDims];  // {a, sd, drift, bits(meta)}
};
constexpr uint32_t kMetaRoot = 1u << 20;  // the terminal point (no ancestors)
__device__ __forceinline__ uint32_t meta_dim(uint32_t m) { return m & 0xFFu; }
__device__ __forceinline__ uint32_t meta_left(uint32_t m) { return (m >> 8) & 0xFu; }
__device__ __forceinline__ uint32_t meta_right(uint32_t m) { return (m >> 12) & 0xFu; }
__device__ __forceinline__ uint32_t meta_out(uint32_t m) { return (m >> 16) & 0xFu; }

template <int PREC>
using QmcTables = typename std::conditional<PREC == 0, QmcTables64, QmcTables32>::type;

// Bridge coefficients of one contract in program order, with the reference's
// operations (brownian_bridge_path.cpp:29-31, :52-62, :71-74): t_i = i T / n.
template <int PREC>
__device__ void fill_tables(const DevContract& c, const DevQmc& q, const BridgeNode* __restrict__ programs,
                            QmcTables<PREC>& S) {
    const int n = c.n_steps;
    const double nd = static_cast<double>(n);
    auto t_of = [&](int i) { return static_cast<double>(i) * q.time / nd; };
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const BridgeNode b = programs[q.prog_offset + e];
        const double tm = t_of(b.t_mid + 1);
        const bool root = b.t_left < 0 && b.t_right < 0;
        double a, sd;
        if (root) {
            a = 0.0;
            sd = sqrt(t_of(n));
        } else {
            const double tl = b.t_left < 0 ? 0.0 : t_of(b.t_left + 1);
            const double tr = t_of(b.t_right + 1);
            a = (tm - tl) / (tr - tl);
            sd = sqrt((tm - tl) * (tr - tm) / (tr - tl));
        }
        const double drift = q.drift_rate * tm;
        if constexpr (PREC == 0) {
            S.node[e] = b;
            S.a[e] = a;
            S.sd[e] = sd;
            S.drift[e] = drift;
        } else {
            const uint32_t meta = static_cast<uint32_t>(b.dim) | (static_cast<uint32_t>(b.slot_left) << 8) |
                                  (static_cast<uint32_t>(b.slot_right) << 12) |
                                  (static_cast<uint32_t>(b.slot_out) << 16) | (root ? kMetaRoot : 0u);
            S.node[e] = make_float4(static_cast<float>(a), static_cast<float>(sd), static_cast<float>(drift),
                                    __uint_as_float(meta));
        }
    }
}

template <int KIND>
__device__ double sample_qmc64(const DevContract& c, const DevQmc& q, const QmcTables64& S, const SobolLane& sob) {
    const double phi = c.type == 0 ? 1.0 : -1.0;
    if constexpr (KIND == kEuropean || KIND == kDigital) {  // qmc.cpp:20-27
        const double z = inv_normal_cdf_f64(static_cast<double>(sob(0u)) * (1.0 / 4294967296.0));
        const double s = c.spot * exp(c.drift + c.vs * z);
        if constexpr (KIND == kEuropean) {
            return c.discount * dmax(phi * (s - c.strike), 0.0);
        } else {
            const bool itm = phi * (s - c.strike) > 0.0;
            return c.discount * (itm ? (c.asset ? s : c.cash) : 0.0);
        }
    } else {
        const int n = c.n_steps;
        double w[kBridgeSlots];
        w[0] = 0.0;
        double sum = 0.0, lsum = 0.0, last = c.spot, hi = c.spot, lo = c.spot;
        bool breached = false;
        for (int e = 0; e < n; ++e) {
            const BridgeNode& b = S.node[e];
            const double z = inv_normal_cdf_f64(static_cast<double>(sob(b.dim)) * (1.0 / 4294967296.0));
            double val;
            if (b.t_left < 0 && b.t_right < 0) {
                val = S.sd[e] * z;
            } else {
                const double wl = w[b.slot_left], wr = w[b.slot_right];
                val = wl + S.a[e] * (wr - wl) + S.sd[e] * z;
            }
            w[b.slot_out] = val;
            const double s = c.spot * exp(S.drift[e] + q.vol * val);
            if (b.t_mid == n - 1) last = s;
            if constexpr (KIND == kAsianArith) {
                sum += s;
            } else if constexpr (KIND == kAsianGeo) {
                lsum += log(s);
            } else if constexpr (KIND == kBarrier) {
                breached = breached || (c.up ? s >= c.barrier : s <= c.barrier);
            } else {
                hi = dmax(hi, s);
                lo = dmin(lo, s);
            }
        }
        const double nd = static_cast<double>(n);
        if constexpr (KIND == kAsianArith || KIND == kAsianGeo) {  // qmc.cpp:44-53
            const double avg = KIND == kAsianArith ? sum / nd : exp(lsum / nd);
            const double ref = c.floating ? (last - avg) : (avg - c.strike);
            return c.discount * dmax(phi * ref, 0.0);
        } else if constexpr (KIND == kBarrier) {
            const double vanilla = dmax(phi * (last - c.strike), 0.0);
            const bool pays = c.out ? !breached : breached;
            return c.discount * (pays ? vanilla : c.rebate);
        } else if constexpr (KIND == kLookbackFixed) {
            return c.discount * (c.type == 0 ? dmax(hi - c.strike, 0.0) : dmax(c.strike - lo, 0.0));
        } else {
            return c.discount * (c.type == 0 ? (last - lo) : (hi - last));
        }
    }
}

// FP32: log-space spots x = ln(S/S0), FP32 payoff, FP64 accumulation.  The
// bridge values live in shared memory, one column per thread (w[slot * 128]):
// a node's slots are known only at run time, so a register array would be
// spilled to local memory.
template <int KIND>
__device__ double sample_qmc32(const DevContract& c, const DevQmc& q, const QmcTables32& S, const SobolLane& sob,
                               float* __restrict__ w) {
    const float phi = c.type == 0 ? 1.0f : -1.0f;
    const float s0 = static_cast<float>(c.spot);
    const float strike = static_cast<float>(c.strike);
    if constexpr (KIND == kEuropean || KIND == kDigital) {
        const float z = normal_from_sobol_f32(sob(0u));
        const float s = s0 * __expf(__fmaf_rn(static_cast<float>(c.vs), z, static_cast<float>(c.drift)));
        float payoff;
        if constexpr (KIND == kEuropean) {
            payoff = fmaxf(phi * (s - strike), 0.0f);
        } else {
            const bool itm = phi * (s - strike) > 0.0f;
            payoff = itm ? (c.asset ? s : static_cast<float>(c.cash)) : 0.0f;
        }
        return c.discount * static_cast<double>(payoff);
    } else {
        const int n = c.n_steps;
        const float vol = static_cast<float>(q.vol);
        const float lnh = static_cast<float>(c.log_h_rel);
        w[0] = 0.0f;
        float acc = 0.0f, acc2 = 0.0f, xlast = 0.0f, xmax = 0.0f, xmin = 0.0f;
        bool breached = false;
        for (int e = 0; e < n; ++e) {
            const float4 nd = S.node[e];
            const uint32_t meta = __float_as_uint(nd.w);
            const float z = normal_from_sobol_f32(sob(meta_dim(meta)));
            float val;
            const bool root = (meta & kMetaRoot) != 0u;
            if (root) {
                val = nd.y * z;
            } else {
                const float wl = w[meta_left(meta) * kSlabThreads], wr = w[meta_right(meta) * kSlabThreads];
                val = __fmaf_rn(nd.y, z, __fmaf_rn(nd.x, wr - wl, wl));
            }
            w[meta_out(meta) * kSlabThreads] = val;
            const float x = __fmaf_rn(vol, val, nd.z);
            if (root) xlast = x;  // the terminal point is the bridge's root
            if constexpr (KIND == kAsianArith) {
                acc += __expf(x);
            } else if constexpr (KIND == kAsianGeo) {
                acc2 += x;
            } else if constexpr (KIND == kBarrier) {
                breached = breached || (c.up ? x >= lnh : x <= lnh);
            } else {
                xmax = fmaxf(xmax, x);
                xmin = fminf(xmin, x);
            }
        }
        const float inv_n = 1.0f / static_cast<float>(n);
        const float last = s0 * __expf(xlast);
        if constexpr (KIND == kAsianArith || KIND == kAsianGeo) {
            const float avg = KIND == kAsianArith ? s0 * (acc * inv_n) : s0 * __expf(acc2 * inv_n);
            const float ref = c.floating ? (last - avg) : (avg - strike);
            return c.discount * static_cast<double>(fmaxf(phi * ref, 0.0f));
        } else if constexpr (KIND == kBarrier) {
            const float vanilla = fmaxf(phi * (last - strike), 0.0f);
            const bool pays = c.out ? !breached : breached;
            return c.discount * static_cast<double>(pays ? vanilla : static_cast<float>(c.rebate));
        } else if constexpr (KIND == kLookbackFixed) {
            const float v = c.type == 0 ? fmaxf(s0 * __expf(xmax) - strike, 0.0f)
                                        : fmaxf(strike - s0 * __expf(xmin), 0.0f);
            return c.discount * static_cast<double>(v);
        } else {
            const float v = c.type == 0 ? (last - s0 * __expf(xmin)) : (s0 * __expf(xmax) - last);
            return c.discount * static_cast<double>(v);
        }
    }
}

template <int PREC, int KIND>
__device__ Welford slab_qmc(const DevContract& c, const DevQmc& q, const QmcTables<PREC>& S,
                            const uint32_t* __restrict__ dirs, const uint32_t* __restrict__ ytab, uint32_t* sx,
                            float* bridge_w, uint64_t base) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t ndims = (KIND == kEuropean || KIND == kDigital) ? 1u : static_cast<uint32_t>(c.n_steps);
    uint32_t* xw = sx + warp * 2 * kSxStride;
    const SobolLane sob{xw + (lane == 31 ? kSxStride : 0), ytab + lane};
    Welford w{0ull, 0.0, 0.0};
    unsigned count = 0;
    double s1 = 0.0, s2 = 0.0;
    for (int j = 0; j < kPathsPerThread; ++j) {
        const uint64_t b0 = base + static_cast<uint64_t>(j * kSlabThreads) + 32u * warp;  // this warp's first path
        if (b0 >= c.path_count) break;  // uniform per warp
        // X for index bases B = b0 (lanes 0..30) and B + 32 (lane 31), dimensions spread over the lanes
        const uint32_t g0 = static_cast<uint32_t>(b0 ^ (b0 >> 1));
        const uint32_t g1 = static_cast<uint32_t>((b0 + 32) ^ ((b0 + 32) >> 1));
        __syncwarp();
        for (uint32_t d = lane; d < ndims; d += 32) {
            xw[d] = sobol_x(dirs, d, g0);
            xw[kSxStride + d] = sobol_x(dirs, d, g1);
        }
        __syncwarp();
        const uint64_t path = b0 + lane;
        if (path >= c.path_count) continue;
        if constexpr (PREC == 0) {
            welford_add(w, sample_qmc64<KIND>(c, q, S, sob));
        } else {
            const double v = sample_qmc32<KIND>(c, q, S, sob, bridge_w + threadIdx.x);
            ++count;
            s1 += v;
            s2 = fma(v, v, s2);
        }
    }
    if constexpr (PREC == 1) w = welford_from_sums(count, s1, s2);
    return w;
}

template <int PREC>
__device__ Welford run_qmc_slab(const DevContract& c, const DevQmc& q, const QmcTables<PREC>& S,
                                const uint32_t* __restrict__ dirs, const uint32_t* __restrict__ ytab, uint32_t* sx,
                                float* bridge_w, uint64_t base) {
    switch (c.kind) {
        case kEuropean: return slab_qmc<PREC, kEuropean>(c, q, S, dirs, ytab, sx, bridge_w, base);
        case kDigital: return slab_qmc<PREC, kDigital>(c, q, S, dirs, ytab, sx, bridge_w, base);
        case kAsianArith: return slab_qmc<PREC, kAsianArith>(c, q, S, dirs, ytab, sx, bridge_w, base);
        case kAsianGeo: return slab_qmc<PREC, kAsianGeo>(c, q, S, dirs, ytab, sx, bridge_w, base);
        case kBarrier: return slab_qmc<PREC, kBarrier>(c, q, S, dirs, ytab, sx, bridge_w, base);
        case kLookbackFixed: return slab_qmc<PREC, kLookbackFixed>(c, q, S, dirs, ytab, sx, bridge_w, base);
        default: return slab_qmc<PREC, kLookbackFloating>(c, q, S, dirs, ytab, sx, bridge_w, base);
    }
}

template <int PREC>
__global__ void __launch_bounds__(kSlabThreads)
    qmc_kernel(const DevContract* __restrict__ contracts, const DevQmc* __restrict__ qmc, int n_contracts,
               const uint32_t* __restrict__ item_prefix, uint32_t total_items,
               const BridgeNode* __restrict__ programs, const uint32_t* __restrict__ dirs,
               uint32_t* __restrict__ ticket, Welford* __restrict__ partials, uint32_t* __restrict__ error_flag) {
    const uint32_t* ytab = dirs + kSobolDims * kSobolBits;  // Y table follows the directions
    __shared__ uint32_t s_sx[(kSlabThreads / 32) * 2 * kSxStride];
    __shared__ uint32_t s_item;
    __shared__ Welford s_warp[kSlabThreads / 32];
    __shared__ DevContract s_c;
    __shared__ DevQmc s_q;
    __shared__ QmcTables<PREC> S;
    __shared__ float s_bridge[PREC == 0 ? 1 : kBridgeSlots * kSlabThreads];  // FP32 bridge values, per thread
    __shared__ int s_loaded;  // sorted index of the contract whose tables are in S
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_loaded = -1;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(ticket, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= total_items) return;
        int lo = 0, hi = n_contracts;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (item_prefix[mid] <= item) lo = mid; else hi = mid;
        }
        const bool reload = s_loaded != lo;
        __syncthreads();
        if (reload) {
            for (int i = threadIdx.x; i < static_cast<int>(sizeof(DevContract) / 4); i += kSlabThreads)
                reinterpret_cast<uint32_t*>(&s_c)[i] = reinterpret_cast<const uint32_t*>(&contracts[lo])[i];
            for (int i = threadIdx.x; i < static_cast<int>(sizeof(DevQmc) / 4); i += kSlabThreads)
                reinterpret_cast<uint32_t*>(&s_q)[i] = reinterpret_cast<const uint32_t*>(&qmc[lo])[i];
            __syncthreads();
            if (s_c.kind != kEuropean && s_c.kind != kDigital) {
                if (s_c.n_steps > kSobolDims) {  // planning invariant broken
                    if (threadIdx.x == 0) atomicOr(error_flag, 2u);
                    continue;
                }
                fill_tables<PREC>(s_c, s_q, programs, S);
            }
            if (threadIdx.x == 0) s_loaded = lo;
            __syncthreads();
        }
        const uint32_t slab = item - item_prefix[lo];
        if (slab >= s_c.n_slabs) {
            if (threadIdx.x == 0) atomicOr(error_flag, 1u);
            continue;
        }
        Welford w = run_qmc_slab<PREC>(s_c, s_q, S, dirs, ytab, s_sx, s_bridge, static_cast<uint64_t>(slab) * kSlabPaths);
        w = welford_warp_reduce(w);
        if (lane == 0) s_warp[warp] = w;
        __syncthreads();
        if (threadIdx.x == 0)
            partials[item] = welford_merge(welford_merge(s_warp[0], s_warp[1]), welford_merge(s_warp[2], s_warp[3]));
    }
}

__global__ void sobol_points_kernel(const uint32_t* __restrict__ dirs, uint32_t dim0, uint32_t n_dims,
                                    uint64_t index0, uint64_t n_idx, double* __restrict__ out) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n_idx * n_dims) return;
    const uint64_t index = index0 + i / n_dims;
    const uint32_t d = dim0 + static_cast<uint32_t>(i % n_dims);
    const uint32_t gray = static_cast<uint32_t>(index ^ (index >> 1));
    out[i] = index == 0 ? 0.0 : static_cast<double>(sobol_x(dirs, d, gray)) * (1.0 / 4294967296.0);
}

}  // namespace

cudaError_t launch_qmc_kernel(int precision, int grid, const DevContract* contracts, const DevQmc* qmc,
                              int n_contracts, const uint32_t* item_prefix, uint32_t total_items,
                              const BridgeNode* programs, const uint32_t* directions, uint32_t* ticket,
                              Welford* partials, uint32_t* error_flag, cudaStream_t stream) {
    cudaGetLastError();
    if (precision == 0)
        qmc_kernel<0><<<grid, kSlabThreads, 0, stream>>>(contracts, qmc, n_contracts, item_prefix, total_items,
                                                         programs, directions, ticket, partials, error_flag);
    else
        qmc_kernel<1><<<grid, kSlabThreads, 0, stream>>>(contracts, qmc, n_contracts, item_prefix, total_items,
                                                         programs, directions, ticket, partials, error_flag);
    return cudaGetLastError();
}

cudaError_t qmc_kernel_occupancy(int precision, int* blocks) {
    return precision == 0 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, qmc_kernel<0>, kSlabThreads, 0)
                          : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, qmc_kernel<1>, kSlabThreads, 0);
}

cudaError_t launch_sobol_points(const uint32_t* directions, uint32_t dim0, uint32_t n_dims, uint64_t index0,
                                uint64_t n_idx, double* out, cudaStream_t stream) {
    cudaGetLastError();
    const uint64_t total = n_idx * n_dims;
    if (total == 0) return cudaSuccess;
    const uint64_t blocks = (total + 255) / 256;
    sobol_points_kernel<<<static_cast<unsigned>(blocks), 256, 0, stream>>>(directions, dim0, n_dims, index0, n_idx,
                                                                           out);
    return cudaGetLastError();
}

}  // namespace mcdg
