// heston.cu -- Heston QE paths priced against many strikes in one pass.
//
// Reference: heston_qe_european (src/pricers/heston.cpp:120-156) with the
// Andersen QE variance step (:91-116, psi_c = 1.5) and the K0..K4 log-spot
// update (gamma1 = gamma2 = 1/2, :125-129).  Each (path, step) consumes the
// stream-0 normal for the spot and the stream-1 uniform for the variance,
// both keyed (seed, path, step) exactly as the reference.
//
// The reference prices one strike per call; calling it for K strikes with one
// seed re-simulates identical paths K times (common random numbers).  Here a
// path is simulated once and its terminal spot is paid out against all K
// strikes, which gives the same K results (to rounding) for 1/K of the
// simulation work.
//
// Work items are (parameter set, 4096-path slab).  A CTA of 128 threads
// simulates one path per thread per round (32 rounds per slab), stages the
// terminal values in shared memory, then pays them out: thread t serves
// strike t % K over the paths of group t / K (G = 128 / K groups), so every
// thread is busy when K <= 128; for 128 < K <= 256, thread t serves strikes t
// and t + 128 over all paths.  Accumulation is per thread in FP64 (FP64 path:
// Welford; FP32 path: FP32 payoffs summed per round with Kahan compensation,
// then added in FP64), and the groups and slabs are merged in fixed order.
//
// nvcc-flags: --fmad=false
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "heston.hpp"

namespace mcdg {

namespace {

__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }

// FP64 QE variance step in the reference's operation order (heston.cpp:91-116).
__device__ __forceinline__ double qe_step64(double v, const HestonSet& h, uint32_t ubits) {
    const double e = h.e;
    const double m = h.theta + (v - h.theta) * e;
    const double s2 = v * h.xi * h.xi * e / h.kappa * (1.0 - e) + h.s2_const;
    const double psi = s2 / (m * m);
    const double raw_uniform = uniform_open01_f64(ubits);
    if (psi <= 1.5) {
        const double inv_psi = 1.0 / psi;
        const double b2 = 2.0 * inv_psi - 1.0 + sqrt(2.0 * inv_psi) * sqrt(2.0 * inv_psi - 1.0);
        const double a = m / (1.0 + b2);
        const double z_v = inv_normal_cdf_f64(raw_uniform);
        const double b = sqrt(b2);
        return a * (b + z_v) * (b + z_v);
    }
    const double p = (psi - 1.0) / (psi + 1.0);
    const double beta = (1.0 - p) / m;
    if (raw_uniform <= p) return 0.0;
    return log((1.0 - p) / (1.0 - raw_uniform)) / beta;
}

// FP32 QE step: same scheme, FP32 arithmetic, 1-u formed from the bits.
__device__ __forceinline__ float qe_step32(float v, const HestonSet32& h, uint32_t ubits) {
    const float m = __fmaf_rn(v - h.theta, h.e, h.theta);
    const float s2 = __fmaf_rn(v, h.s2_lin, h.s2_const);
    const float psi = s2 * fast_rcp(m * m);
    if (psi <= 1.5f) {
        const float inv_psi = fast_rcp(psi);
        const float two = 2.0f * inv_psi;
        const float b2 = two - 1.0f + fast_sqrt(two) * fast_sqrt(two - 1.0f);
        const float a = m * fast_rcp(1.0f + b2);
        const float z_v = normal_from_bits_f32(ubits);
        const float bz = fast_sqrt(b2) + z_v;
        return a * bz * bz;
    }
    const float p = (psi - 1.0f) * fast_rcp(psi + 1.0f);
    const float u = uniform_from_bits_f32(ubits);
    if (u <= p) return 0.0f;
    // 1 - u = (~bits + 0.5) / 2^32, exact relative precision near u = 1
    const float one_minus_u = __fmaf_rn(__uint2float_rn(~ubits), 2.3283064365386963e-10f,
                                        1.1641532182693481e-10f);
    const float beta = (1.0f - p) * fast_rcp(m);
    return __logf((1.0f - p) * fast_rcp(one_minus_u)) * fast_rcp(beta);
}

struct KahanF {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

// FP32: two paths per thread in flight, so a larger register budget (6 CTAs
// of 128 threads per SM) than the FP64 kernel's (8).
template <int PREC>
__global__ void __launch_bounds__(128, PREC == 1 ? 6 : 8)
    heston_kernel(const HestonSet* __restrict__ sets, int n_sets, const double* __restrict__ strikes,
                  int n_strikes, int type, uint32_t items_per_set, uint32_t total_items,
                  uint32_t* __restrict__ ticket, Welford* __restrict__ partials) {
    __shared__ uint32_t s_item;
    __shared__ double s_terminal64[128];
    __shared__ float s_terminal32[128], s_terminal32b[128];
    __shared__ Welford s_acc[256];
    __shared__ HestonSet s_set;
    const int t = threadIdx.x;
    const int groups = n_strikes <= 128 ? 128 / n_strikes : 1;
    const int my_group = n_strikes <= 128 ? t / n_strikes : 0;
    const int k0 = n_strikes <= 128 ? t % n_strikes : t;
    const bool serves0 = (n_strikes <= 128) ? (my_group < groups) : (k0 < n_strikes);
    const bool serves1 = n_strikes > 128 && (t + 128) < n_strikes;
    const double phi = type == 0 ? 1.0 : -1.0;
    for (;;) {
        if (t == 0) s_item = atomicAdd(ticket, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= total_items) return;
        const int set = static_cast<int>(item / items_per_set);
        const uint32_t slab = item % items_per_set;
        static_assert(sizeof(HestonSet) % 4 == 0 && sizeof(HestonSet) / 4 <= 128, "one word per thread");
        if (t < static_cast<int>(sizeof(HestonSet) / 4))
            reinterpret_cast<uint32_t*>(&s_set)[t] = reinterpret_cast<const uint32_t*>(&sets[set])[t];
        __syncthreads();
        const HestonSet& h = s_set;
        const PhiloxKeys k = philox_keys(h.seed);
        const double strike0 = serves0 ? strikes[k0] : 0.0;
        const double strike1 = serves1 ? strikes[t + 128] : 0.0;
        Welford w0{0ull, 0.0, 0.0}, w1{0ull, 0.0, 0.0};
        unsigned cnt0 = 0, cnt1 = 0;
        double a0 = 0.0, q0 = 0.0, a1 = 0.0, q1 = 0.0;
        HestonSet32 h32;
        if (PREC == 1) h32 = make_set32(h);
        if constexpr (PREC == 0) {
            for (int j = 0; j < 32; ++j) {
                const uint64_t path = static_cast<uint64_t>(slab) * 4096 + static_cast<uint64_t>(j * 128 + t);
                if (path < h.path_count) {
                    const PhiloxPath ps = philox_path(path, 0u, k);
                    const PhiloxPath pv = philox_path(path, 1u, k);
                    double v = h.v0;
                    double log_s = h.log_s0;
                    for (int step = 0; step < h.n_steps; ++step) {
                        const uint32_t d = static_cast<uint32_t>(step);
                        const double z_s = normal_from_bits_f64(philox_word0(ps, d, k));
                        const double v_next = qe_step64(v, h, philox_word0(pv, d, k));
                        const double diffusion_var = dmax(h.k3 * v + h.k4 * v_next, 0.0);
                        log_s += h.drift + h.k0 + h.k1 * v + h.k2 * v_next + sqrt(diffusion_var) * z_s;
                        v = v_next;
                    }
                    s_terminal64[t] = exp(log_s);
                }
                __syncthreads();
                // Pay out the round's paths (paths of this round beyond path_count are skipped).
                const uint64_t round_base = static_cast<uint64_t>(slab) * 4096 + static_cast<uint64_t>(j * 128);
                const uint64_t left = round_base >= h.path_count ? 0 : h.path_count - round_base;
                const int round_live = left > 128 ? 128 : static_cast<int>(left);
                for (int p = my_group; p < round_live; p += groups) {
                    const double s_t = s_terminal64[p];
                    if (serves0) welford_add(w0, h.discount * dmax(phi * (s_t - strike0), 0.0));
                    if (serves1) welford_add(w1, h.discount * dmax(phi * (s_t - strike1), 0.0));
                }
                __syncthreads();
            }
        } else {
            // Two rounds per pass: each thread simulates the paths of rounds j
            // and j + 1 together (independent dependency chains), then both
            // rounds are paid out in order, so the sums are those of one round
            // at a time.
            const float fphi = static_cast<float>(phi);
            const float fk0 = static_cast<float>(strike0), fk1 = static_cast<float>(strike1);
            auto payout = [&](int j, const float* terminal) {
                const uint64_t round_base = static_cast<uint64_t>(slab) * 4096 + static_cast<uint64_t>(j * 128);
                const uint64_t left = round_base >= h.path_count ? 0 : h.path_count - round_base;
                const int round_live = left > 128 ? 128 : static_cast<int>(left);
                KahanF s0a, s0b, s1a, s1b;
                unsigned n_here = 0;
                for (int p = my_group; p < round_live; p += groups) {
                    const float s_t = terminal[p];
                    const float y0 = fmaxf(fphi * (s_t - fk0), 0.0f);
                    s0a.add(y0);
                    s0b.add(y0 * y0);
                    if (serves1) {
                        const float y1 = fmaxf(fphi * (s_t - fk1), 0.0f);
                        s1a.add(y1);
                        s1b.add(y1 * y1);
                    }
                    ++n_here;
                }
                if (serves0) {
                    cnt0 += n_here;
                    a0 += static_cast<double>(s0a.s) + static_cast<double>(-s0a.c);
                    q0 += static_cast<double>(s0b.s) + static_cast<double>(-s0b.c);
                }
                if (serves1) {
                    cnt1 += n_here;
                    a1 += static_cast<double>(s1a.s) + static_cast<double>(-s1a.c);
                    q1 += static_cast<double>(s1b.s) + static_cast<double>(-s1b.c);
                }
            };
            for (int j = 0; j < 32; j += 2) {
                const uint64_t path_a = static_cast<uint64_t>(slab) * 4096 + static_cast<uint64_t>(j * 128 + t);
                const uint64_t path_b = path_a + 128;
                if (path_a < h.path_count) {  // path_b exists only if path_a does
                    const bool live_b = path_b < h.path_count;
                    const PhiloxPath psa = philox_path(path_a, 0u, k), pva = philox_path(path_a, 1u, k);
                    const PhiloxPath psb = philox_path(path_b, 0u, k), pvb = philox_path(path_b, 1u, k);
                    float va = h32.v0, vb = h32.v0;
                    float xa = 0.0f, xb = 0.0f;  // ln(S/S0)
                    for (int step = 0; step < h.n_steps; ++step) {
                        const uint32_t d = static_cast<uint32_t>(step);
                        const float za = normal_from_bits_f32(philox_word0(psa, d, k));
                        const float zb = normal_from_bits_f32(philox_word0(psb, d, k));
                        const float va_next = qe_step32(va, h32, philox_word0(pva, d, k));
                        const float vb_next = qe_step32(vb, h32, philox_word0(pvb, d, k));
                        const float dva = fmaxf(__fmaf_rn(h32.k3, va, h32.k4 * va_next), 0.0f);
                        const float dvb = fmaxf(__fmaf_rn(h32.k3, vb, h32.k4 * vb_next), 0.0f);
                        const float ia = __fmaf_rn(h32.k1, va, __fmaf_rn(h32.k2, va_next, h32.c0));
                        const float ib = __fmaf_rn(h32.k1, vb, __fmaf_rn(h32.k2, vb_next, h32.c0));
                        xa = __fmaf_rn(fast_sqrt(dva), za, xa + ia);
                        xb = __fmaf_rn(fast_sqrt(dvb), zb, xb + ib);
                        va = va_next;
                        vb = vb_next;
                    }
                    s_terminal32[t] = h32.s0 * __expf(xa);
                    if (live_b) s_terminal32b[t] = h32.s0 * __expf(xb);
                }
                __syncthreads();
                payout(j, s_terminal32);
                payout(j + 1, s_terminal32b);
                __syncthreads();
            }
        }
        if (PREC == 1) {
            // discount applied once: mean scales by D, M2 by D^2
            const double d = h.discount;
            w0 = welford_from_sums(cnt0, a0 * d, q0 * d * d);
            w1 = welford_from_sums(cnt1, a1 * d, q1 * d * d);
        }
        // Merge the groups of each strike in group order (fixed tree).
        if (serves0) s_acc[n_strikes <= 128 ? my_group * n_strikes + k0 : k0] = w0;
        if (serves1) s_acc[t + 128] = w1;
        __syncthreads();
        if (n_strikes <= 128) {
            if (t < n_strikes) {
                Welford m = s_acc[t];
                for (int g = 1; g < groups; ++g) m = welford_merge(m, s_acc[g * n_strikes + t]);
                partials[static_cast<size_t>(item) * n_strikes + t] = m;
            }
        } else {
            for (int kk = t; kk < n_strikes; kk += 128)
                partials[static_cast<size_t>(item) * n_strikes + kk] = s_acc[kk];
        }
        __syncthreads();
    }
}

// One warp per (set, strike): fold the set's slabs in slab order, fixed tree.
__global__ void heston_merge_kernel(const HestonSet* __restrict__ sets, int n_sets, int n_strikes,
                                    uint32_t items_per_set, const Welford* __restrict__ partials,
                                    double* __restrict__ out /* n_sets*n_strikes x {price, se, count} */) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n_sets * n_strikes) return;
    const int set = w / n_strikes, kk = w % n_strikes;
    const uint32_t n_slabs = sets[set].n_slabs;
    Welford acc{0ull, 0.0, 0.0};
    for (uint32_t s = lane; s < n_slabs; s += 32)
        acc = welford_merge(acc, partials[(static_cast<size_t>(set) * items_per_set + s) * n_strikes + kk]);
    acc = welford_warp_reduce(acc);
    if (lane == 0) {
        const double var = acc.count < 2 ? 0.0 : acc.m2 / static_cast<double>(acc.count - 1);
        out[3 * static_cast<size_t>(w) + 0] = acc.mean;
        out[3 * static_cast<size_t>(w) + 1] = acc.count == 0 ? 0.0 : sqrt(var / static_cast<double>(acc.count));
        reinterpret_cast<unsigned long long*>(out)[3 * static_cast<size_t>(w) + 2] = acc.count;
    }
}

}  // namespace

cudaError_t launch_heston(int precision, int grid, const HestonSet* sets, int n_sets,
                          const double* strikes, int n_strikes, int type, uint32_t items_per_set,
                          uint32_t* ticket, Welford* partials, double* out, cudaStream_t stream) {
    const uint32_t total = items_per_set * static_cast<uint32_t>(n_sets);
    cudaGetLastError();
    if (total > 0) {
        if (precision == 0)
            heston_kernel<0><<<grid, 128, 0, stream>>>(sets, n_sets, strikes, n_strikes, type,
                                                       items_per_set, total, ticket, partials);
        else
            heston_kernel<1><<<grid, 128, 0, stream>>>(sets, n_sets, strikes, n_strikes, type,
                                                       items_per_set, total, ticket, partials);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    const int warps = n_sets * n_strikes;
    heston_merge_kernel<<<(warps * 32 + 255) / 256, 256, 0, stream>>>(sets, n_sets, n_strikes,
                                                                       items_per_set, partials, out);
    return cudaGetLastError();
}

cudaError_t heston_occupancy(int precision, int* blocks) {
    return precision == 0
               ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, heston_kernel<0>, 128, 0)
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, heston_kernel<1>, 128, 0);
}

}  // namespace mcdg
