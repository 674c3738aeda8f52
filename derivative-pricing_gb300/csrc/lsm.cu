// lsm.cu -- batched Longstaff-Schwartz American pricing (QR regression).
//
// Reference: monte_carlo_lsm_american (src/pricers/lsm.cpp:62-149; the frozen
// replay of :151-213 is the streaming kernel of lsm_frozen.cu): forward-simulated
// GBM paths, cash flows seeded with the terminal intrinsic, backward over dates
// n-1..1 (discount
// the cash flows, regress them on the weighted Laguerre basis of S/K over the
// in-the-money paths -- skipped below 4 such paths --, exercise where
// intrinsic > continuation), a final discount, Welford, and the inception check.
//
// Layout.  Every contract's paths live in HBM for the whole backward pass,
// date-major (S[d-1][i], coalesced per date for the forward stores and the
// backward column reads), FP32 or FP64; cash flows are FP64.  Paths are cut
// into fixed chunks of 1024 (the reduction unit); a chunk is one CTA of 256
// threads (4 paths per thread, stride 256).
//
// Backward pass.  All contracts of a batch step back in lockstep: iteration k
// handles date e = n_c - k of contract c.  Per iteration:
//   lsm_exercise  exercise at date e with that date's coefficients, discount,
//                 and either the Gram sums of date e-1 (pass A) or, when e = 1,
//                 the final Welford partial;
//   lsm_solve_a   per contract: fixed-order reduction, Cholesky G = R^T R,
//                 T = R^{-1};
//   lsm_gram_b    Gram sums and right-hand side in the preconditioned basis
//                 b' = b T (pass B);
//   lsm_solve_b   per contract: reduction, 4x4 Householder solve of
//                 G' beta' = h', gamma = T beta' (coefficients in the
//                 Laguerre basis, as the reference's policy stores them).
// This is Cholesky-QR2 applied to the least-squares problem: the first pass
// removes the conditioning (cond(X) reaches ~2e6 for these bases, cond(G)
// ~4e12), the second is solved at QR accuracy, so the coefficients agree with
// the reference's Householder QR to ~1e-10 relative and exercise decisions
// essentially never differ.  Every reduction tree is fixed by chunk index.
// Precision: the FP64 path is the reference's arithmetic throughout.  The
// FP32 path evaluates the basis, the exercise tests and the Gram products in
// FP32 (FP64 runs at a small fraction of the FP32 rate here), keeps the cash
// flows and continuation values in FP32 and accumulates the Gram products
// with compensated FP32 sums per chunk (per thread, then one warp per sum
// over the chunk's threads); the final payoffs are summed in compensated
// FP32 per thread and over the warp tree (Sum32); warp sums, chunk partials
// and the Cholesky-QR2 solves are FP64.  (The FP32 discount factor
// carries a relative error below 3e-8 per date, a bias under 2e-6 of the
// price after 50 dates.)
//
// nvcc-flags: --fmad=false
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "lsm.hpp"

namespace mcdg {

namespace {

__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }

__device__ __forceinline__ double intrinsic(double s, double k, int type) {
    return dmax((type == 0 ? 1.0 : -1.0) * (s - k), 0.0);
}

// Weighted Laguerre basis on x = S/K (src/pricers/lsm.cpp:21-25), the
// reference's expressions (FP64 path).
__device__ __forceinline__ void basis64(double s, double strike, double b[4]) {
    const double x = s / strike;
    const double e = exp(-x / 2.0);
    b[0] = e;
    b[1] = e * (1.0 - x);
    b[2] = e * (1.0 - 2.0 * x + 0.5 * x * x);
    b[3] = e * (1.0 - 3.0 * x + 1.5 * x * x - x * x * x / 6.0);
}

// FP32 path: the same basis evaluated in FP32.  FP64 arithmetic runs at a
// small fraction of the FP32 rate on this GPU, and with FP32 paths the basis
// carries FP32 inputs anyway; the regression is fitted to exactly this
// evaluated basis and the sums that need the range stay compensated (below).
__device__ __forceinline__ void basis32(float s, float inv_strike, float b[4]) {
    const float x = s * inv_strike;
    const float e = __expf(-0.5f * x);
    b[0] = e;
    b[1] = e * (1.0f - x);
    b[2] = e * __fmaf_rn(0.5f * x, x, __fmaf_rn(-2.0f, x, 1.0f));
    b[3] = e * __fmaf_rn(__fmaf_rn(-x / 6.0f, x, 1.5f * x), x, __fmaf_rn(-3.0f, x, 1.0f));
}

// Compensated FP32 accumulation (Knuth's TwoSum): hi + lo carries ~44 bits,
// enough for Gram sums of a chunk; chunk partials are then merged in FP64.
__device__ __forceinline__ void df_add(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float bp = s - hi;
    lo += (hi - (s - bp)) + (x - bp);
    hi = s;
}

// Fixed-shape block reduction of N compensated sums (256 threads): every
// thread's (hi, lo) pairs go to shared memory, then warp w folds sums w,
// w + 8, ...: lane l takes threads l, l + 32, ..., l + 224 in that order
// (compensated), then a compensated shuffle tree; the FP64 value hi + lo of
// each sum lands in res and, for thread 0, in out.
template <int N>
__device__ void block_sum_df(const float (&hi)[N], const float (&lo)[N], float2 (*scratch)[kLsmThreads],
                             double* res, double (&out)[N]) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int i = 0; i < N; ++i) scratch[i][t] = make_float2(hi[i], lo[i]);
    __syncthreads();
    for (int i = warp; i < N; i += kLsmThreads / 32) {
        float h = 0.0f, l = 0.0f;
#pragma unroll
        for (int u = 0; u < kLsmThreads / 32; ++u) {
            const float2 v = scratch[i][lane + 32 * u];
            df_add(h, l, v.x);
            l += v.y;
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            const float oh = __shfl_down_sync(0xffffffffu, h, off);
            const float ol = __shfl_down_sync(0xffffffffu, l, off);
            df_add(h, l, oh);
            l += ol;
        }
        if (lane == 0) res[i] = static_cast<double>(h) + static_cast<double>(l);
    }
    __syncthreads();
    if (t == 0) {
#pragma unroll
        for (int i = 0; i < N; ++i) out[i] = res[i];
    }
}

template <int PREC>
__device__ __forceinline__ double load_s(const void* store, uint64_t idx) {
    if (PREC == 0) return static_cast<const double*>(store)[idx];
    return static_cast<double>(static_cast<const float*>(store)[idx]);
}

// Fixed-shape block reduction of N doubles (256 threads): warp trees, then
// warp 0 folds the 8 warp results in order.  Result valid in thread 0.
template <int N>
__device__ void block_sum(double (&v)[N], double (*smem)[N]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        double x = v[i];
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
        v[i] = x;
    }
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < N; ++i) smem[warp][i] = v[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < N; ++i) {
            double x = smem[0][i];
            for (int w = 1; w < kLsmThreads / 32; ++w) x += smem[w][i];
            v[i] = x;
        }
    }
}

// ---------------------------------------------------------------------------
// forward simulation (src/pricers/lsm.cpp:35-58), date-major stores
// ---------------------------------------------------------------------------
template <int PREC>
__global__ void __launch_bounds__(kLsmThreads)
    lsm_forward(const LsmDev* __restrict__ cs, const uint32_t* __restrict__ chunk_contract,
                uint32_t total_chunks, void* __restrict__ store) {
    const uint32_t chunk = blockIdx.x;
    if (chunk >= total_chunks) return;
    const LsmDev c = cs[chunk_contract[chunk]];
    const uint32_t local = chunk - c.chunk_begin;
    const PhiloxKeys k = philox_keys(c.seed);
    const float mu = static_cast<float>(c.drift), sg = static_cast<float>(c.vs);
    const float s0 = static_cast<float>(c.spot);
    for (int j = 0; j < kLsmChunk / kLsmThreads; ++j) {
        const uint64_t i = static_cast<uint64_t>(local) * kLsmChunk + j * kLsmThreads + threadIdx.x;
        if (i >= c.path_count) break;
        const PhiloxPath pp = philox_path(i, 0u, k);
        if (PREC == 0) {
            double* S = static_cast<double*>(store) + c.s_offset;
            double s = c.spot;
            for (int d = 0; d < c.n_steps; ++d) {
                const double z = normal_from_bits_f64(philox_word0(pp, static_cast<uint32_t>(d), k));
                s = s * exp(c.drift + c.vs * z);
                S[static_cast<uint64_t>(d) * c.path_count + i] = s;
            }
        } else {
            // two paths per iteration when both exist: independent Philox
            // chains for instruction-level parallelism, the same values
            float* S = static_cast<float*>(store) + c.s_offset;
            const uint64_t i2 = i + kLsmThreads;
            if ((j & 1) == 0 && j + 1 < kLsmChunk / kLsmThreads && i2 < c.path_count) {
                const PhiloxPath pp2 = philox_path(i2, 0u, k);
                float x = 0.0f, x2 = 0.0f;
                for (int d = 0; d < c.n_steps; ++d) {
                    const float z = normal_from_bits_f32(philox_word0(pp, static_cast<uint32_t>(d), k));
                    const float z2 = normal_from_bits_f32(philox_word0(pp2, static_cast<uint32_t>(d), k));
                    x = __fmaf_rn(sg, z, x + mu);
                    x2 = __fmaf_rn(sg, z2, x2 + mu);
                    S[static_cast<uint64_t>(d) * c.path_count + i] = s0 * __expf(x);
                    S[static_cast<uint64_t>(d) * c.path_count + i2] = s0 * __expf(x2);
                }
                ++j;  // the partner path is done
                continue;
            }
            float x = 0.0f;
            for (int d = 0; d < c.n_steps; ++d) {
                const float z = normal_from_bits_f32(philox_word0(pp, static_cast<uint32_t>(d), k));
                x = __fmaf_rn(sg, z, x + mu);
                S[static_cast<uint64_t>(d) * c.path_count + i] = s0 * __expf(x);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// iteration k: exercise at date e, discount, pass A for date e-1 (or final)
// ---------------------------------------------------------------------------
template <int PREC>
__global__ void __launch_bounds__(kLsmThreads)
    lsm_exercise(int k, const LsmDev* __restrict__ cs,
                 const uint32_t* __restrict__ chunk_contract, uint32_t total_chunks,
                 const void* __restrict__ store, double* __restrict__ cf,
                 const LsmReg* __restrict__ reg, LsmPartial* __restrict__ part_a,
                 Welford* __restrict__ final_part) {
    __shared__ double smem[kLsmThreads / 32][11];
    __shared__ float2 scratch[11][kLsmThreads];  // FP32 path: the Gram sums' per-thread pairs
    __shared__ double sres[11];
    __shared__ Welford swf[kLsmThreads / 32];
    __shared__ Sum64 s64[kLsmThreads / 32];
    const uint32_t chunk = blockIdx.x;
    if (chunk >= total_chunks) return;
    const LsmDev c = cs[chunk_contract[chunk]];
    const int n = c.n_steps;
    const int e = n - k;
    if (e < 1) return;  // this contract has finished (uniform per CTA)
    const bool init = (k == 0);
    const bool last = (e == 1);
    const bool gram = !last;
    const LsmReg* re = (!init && e <= n - 1) ? &reg[c.reg_offset + e] : nullptr;
    const bool exercise = re != nullptr && re->has == 1;
    double g0 = 0, g1 = 0, g2 = 0, g3 = 0;
    if (exercise) {
        g0 = re->gamma[0];
        g1 = re->gamma[1];
        g2 = re->gamma[2];
        g3 = re->gamma[3];
    }
    const uint32_t local = chunk - c.chunk_begin;
    Welford w{0ull, 0.0, 0.0};
    if constexpr (PREC == 0) {
        double acc[11];
#pragma unroll
        for (int q = 0; q < 11; ++q) acc[q] = 0.0;
        for (int j = 0; j < kLsmChunk / kLsmThreads; ++j) {
            const uint64_t i = static_cast<uint64_t>(local) * kLsmChunk + j * kLsmThreads + threadIdx.x;
            if (i >= c.path_count) break;
            double v;
            if (init) {
                v = intrinsic(load_s<PREC>(store, c.s_offset + static_cast<uint64_t>(n - 1) * c.path_count + i),
                              c.strike, c.type);
            } else {
                v = cf[c.cf_offset + i];
                if (exercise) {
                    const double s = load_s<PREC>(store, c.s_offset + static_cast<uint64_t>(e - 1) * c.path_count + i);
                    const double ex = intrinsic(s, c.strike, c.type);
                    if (ex > 0.0) {
                        double b[4];
                        basis64(s, c.strike, b);
                        double cont = 0.0;
                        cont += g0 * b[0];
                        cont += g1 * b[1];
                        cont += g2 * b[2];
                        cont += g3 * b[3];
                        if (ex > cont) v = ex;
                    }
                }
            }
            v *= c.disc;
            if (last) {
                welford_add(w, v);
            } else {
                cf[c.cf_offset + i] = v;
                if (gram) {
                    const double s = load_s<PREC>(store, c.s_offset + static_cast<uint64_t>(e - 2) * c.path_count + i);
                    if (intrinsic(s, c.strike, c.type) > 0.0) {
                        double b[4];
                        basis64(s, c.strike, b);
                        acc[0] += 1.0;
                        acc[1] += b[0] * b[0];
                        acc[2] += b[0] * b[1];
                        acc[3] += b[0] * b[2];
                        acc[4] += b[0] * b[3];
                        acc[5] += b[1] * b[1];
                        acc[6] += b[1] * b[2];
                        acc[7] += b[1] * b[3];
                        acc[8] += b[2] * b[2];
                        acc[9] += b[2] * b[3];
                        acc[10] += b[3] * b[3];
                    }
                }
            }
        }
        if (gram) {
            block_sum<11>(acc, smem);
            if (threadIdx.x == 0) {
#pragma unroll
                for (int q = 0; q < 11; ++q) part_a[chunk].v[q] = acc[q];
            }
        }
    } else {
        // FP32 paths: FP32 cash flows (stored in the FP64 buffer's space),
        // basis, continuation value, exercise tests and Gram products; the
        // Gram sums and the final payoff sums up to the warp are
        // compensated FP32, everything above FP64.
        const float phi = c.phi_f, strike = c.strike_f, inv_kf = c.inv_strike_f, disc = c.disc_f;
        const float g0f = exercise ? re->gamma_f[0] : 0.0f, g1f = exercise ? re->gamma_f[1] : 0.0f,
                    g2f = exercise ? re->gamma_f[2] : 0.0f, g3f = exercise ? re->gamma_f[3] : 0.0f;
        const float* S = static_cast<const float*>(store) + c.s_offset;
        float* cff = reinterpret_cast<float*>(cf) + c.cf_offset;
        float hi[11], lo[11];
#pragma unroll
        for (int q = 0; q < 11; ++q) hi[q] = lo[q] = 0.0f;
        Sum32 fin{0u, 0.0f, 0.0f, 0.0f, 0.0f};  // final payoffs (last date)
        constexpr int kPer = kLsmChunk / kLsmThreads;
        // all loads of this thread's paths first (independent, in flight together)
        float vv[kPer], se[kPer], sd[kPer];
        bool live[kPer];
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint64_t i = static_cast<uint64_t>(local) * kLsmChunk + j * kLsmThreads + threadIdx.x;
            live[j] = i < c.path_count;
            vv[j] = 0.0f;
            se[j] = 0.0f;
            sd[j] = 0.0f;
            if (live[j]) {
                if (init) vv[j] = S[static_cast<uint64_t>(n - 1) * c.path_count + i];
                else vv[j] = cff[i];
                if (exercise) se[j] = S[static_cast<uint64_t>(e - 1) * c.path_count + i];
                if (gram) sd[j] = S[static_cast<uint64_t>(e - 2) * c.path_count + i];
            }
        }
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            if (!live[j]) continue;
            const uint64_t i = static_cast<uint64_t>(local) * kLsmChunk + j * kLsmThreads + threadIdx.x;
            float v = init ? fmaxf(phi * (vv[j] - strike), 0.0f) : vv[j];
            if (exercise) {
                const float ex = phi * (se[j] - strike);
                if (ex > 0.0f) {
                    float b[4];
                    basis32(se[j], inv_kf, b);
                    const float cont = __fmaf_rn(g3f, b[3], __fmaf_rn(g2f, b[2], __fmaf_rn(g1f, b[1], g0f * b[0])));
                    if (ex > cont) v = ex;
                }
            }
            v *= disc;
            if (last) {
                sum32_add(fin, v);
            } else {
                cff[i] = v;
                if (gram && phi * (sd[j] - strike) > 0.0f) {
                    float b[4];
                    basis32(sd[j], inv_kf, b);
                    df_add(hi[0], lo[0], 1.0f);
                    df_add(hi[1], lo[1], b[0] * b[0]);
                    df_add(hi[2], lo[2], b[0] * b[1]);
                    df_add(hi[3], lo[3], b[0] * b[2]);
                    df_add(hi[4], lo[4], b[0] * b[3]);
                    df_add(hi[5], lo[5], b[1] * b[1]);
                    df_add(hi[6], lo[6], b[1] * b[2]);
                    df_add(hi[7], lo[7], b[1] * b[3]);
                    df_add(hi[8], lo[8], b[2] * b[2]);
                    df_add(hi[9], lo[9], b[2] * b[3]);
                    df_add(hi[10], lo[10], b[3] * b[3]);
                }
            }
        }
        if (last) {
            const Sum32 r = sum32_warp_reduce(fin);
            if ((threadIdx.x & 31) == 0) s64[threadIdx.x >> 5] = sum32_wide(r);
        }
        if (gram) {
            double acc[11];
            block_sum_df<11>(hi, lo, scratch, sres, acc);
            if (threadIdx.x == 0) {
#pragma unroll
                for (int q = 0; q < 11; ++q) part_a[chunk].v[q] = acc[q];
            }
        }
    }
    if (last) {
        if constexpr (PREC == 0) {
            w = welford_warp_reduce(w);
            if ((threadIdx.x & 31) == 0) swf[threadIdx.x >> 5] = w;
            __syncthreads();
            if (threadIdx.x == 0) {
                Welford m = swf[0];
                for (int q = 1; q < kLsmThreads / 32; ++q) m = welford_merge(m, swf[q]);
                final_part[chunk] = m;
            }
        } else {
            __syncthreads();
            if (threadIdx.x == 0) final_part[chunk] = sum64_fold<kLsmThreads / 32>(s64);
        }
    }
}

// Upper-triangular index of (r, c), r <= c, in the packed 10-entry layout.
__device__ __forceinline__ int tri(int r, int col) {
    const int base[4] = {0, 4, 7, 9};
    return base[r] + (col - r);
}

// Per contract: fold pass-A partials in chunk order, Cholesky, T = R^{-1}.
__global__ void lsm_solve_a(int k, const LsmDev* __restrict__ cs, int n_contracts,
                            const LsmPartial* __restrict__ part_a, LsmReg* __restrict__ reg) {
    const int ci = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (ci >= n_contracts) return;
    const LsmDev c = cs[ci];
    const int date = c.n_steps - k - 1;  // regression date of this iteration
    if (date < 1) return;
    double s[11];
#pragma unroll
    for (int q = 0; q < 11; ++q) s[q] = 0.0;
    for (uint32_t ch = lane; ch < c.n_chunks; ch += 32)
#pragma unroll
        for (int q = 0; q < 11; ++q) s[q] += part_a[c.chunk_begin + ch].v[q];
#pragma unroll
    for (int q = 0; q < 11; ++q)
        for (int off = 16; off >= 1; off >>= 1) s[q] += __shfl_down_sync(0xffffffffu, s[q], off);
    if (lane != 0) return;
    LsmReg& r = reg[c.reg_offset + date];
    r.has = 0;
    r.degenerate = 0;
    if (s[0] < 4.0) {  // too few in-the-money paths (src/pricers/lsm.cpp:102-104)
        r.has = -1;
        return;
    }
    double G[4][4];
    for (int a = 0; a < 4; ++a)
        for (int b2 = a; b2 < 4; ++b2) G[a][b2] = G[b2][a] = s[1 + tri(a, b2)];
    double R[4][4] = {};
    // R only preconditions pass B, so when the Gram matrix of the raw basis
    // (condition up to ~1e13) is not numerically positive definite -- its
    // sums carry ~44 bits on the FP32 path -- the factorisation is retried
    // with a diagonal shift of 1e-10 of its trace (shifted Cholesky QR,
    // Fukaya, Kannan, Nakatsukasa, Zhang and Yamamoto, SIAM J. Sci. Comput.
    // 42 (2020)); pass B and the Householder solve then fit the unshifted
    // problem.  A date that factorises without the shift is unaffected.
    const double shift_step = 1e-10 * (G[0][0] + G[1][1] + G[2][2] + G[3][3]);
    bool ok = false;
    for (int attempt = 0; attempt < 2 && !ok; ++attempt) {
        const double shift = attempt == 0 ? 0.0 : shift_step;
        ok = true;
        for (int j = 0; j < 4 && ok; ++j) {
            double d = G[j][j] + shift;
            for (int p = 0; p < j; ++p) d -= R[p][j] * R[p][j];
            if (!(d > 0.0)) {
                ok = false;
                break;
            }
            R[j][j] = sqrt(d);
            for (int l = j + 1; l < 4; ++l) {
                double x = G[j][l];
                for (int p = 0; p < j; ++p) x -= R[p][j] * R[p][l];
                R[j][l] = x / R[j][j];
            }
        }
        if (ok && attempt == 1) r.degenerate = 2;  // factorised with the shift
    }
    double T[4][4] = {};
    if (ok) {
        for (int j = 3; j >= 0; --j) {
            T[j][j] = 1.0 / R[j][j];
            for (int l = j + 1; l < 4; ++l) {
                double x = 0.0;
                for (int p = j; p < l; ++p) x += T[j][p] * R[p][l];
                T[j][l] = -x / R[l][l];
            }
        }
    } else {
        for (int j = 0; j < 4; ++j) T[j][j] = 1.0;
        r.degenerate = 1;
    }
    for (int a = 0; a < 4; ++a)
        for (int b2 = a; b2 < 4; ++b2) {
            r.T[tri(a, b2)] = T[a][b2];
            r.T_f[tri(a, b2)] = static_cast<float>(T[a][b2]);
        }
}

// Pass B: Gram sums and right-hand side in the preconditioned basis b' = b T.
template <int PREC>
__global__ void __launch_bounds__(kLsmThreads)
    lsm_gram_b(int k, const LsmDev* __restrict__ cs, const uint32_t* __restrict__ chunk_contract,
               uint32_t total_chunks, const void* __restrict__ store, const double* __restrict__ cf,
               const LsmReg* __restrict__ reg, LsmPartial* __restrict__ part_b) {
    __shared__ double smem[kLsmThreads / 32][15];
    __shared__ float2 scratch[15][kLsmThreads];  // FP32 path: the sums' per-thread pairs
    __shared__ double sres[15];
    const uint32_t chunk = blockIdx.x;
    if (chunk >= total_chunks) return;
    const LsmDev c = cs[chunk_contract[chunk]];
    const int date = c.n_steps - k - 1;
    if (date < 1) return;
    const LsmReg& r = reg[c.reg_offset + date];
    if (r.has == -1) return;  // no regression at this date
    const uint32_t local = chunk - c.chunk_begin;
    double out[15];
    if constexpr (PREC == 0) {
        double T[10];
#pragma unroll
        for (int q = 0; q < 10; ++q) T[q] = r.T[q];
        double acc[15];
#pragma unroll
        for (int q = 0; q < 15; ++q) acc[q] = 0.0;
        for (int j = 0; j < kLsmChunk / kLsmThreads; ++j) {
            const uint64_t i = static_cast<uint64_t>(local) * kLsmChunk + j * kLsmThreads + threadIdx.x;
            if (i >= c.path_count) break;
            const double s = load_s<PREC>(store, c.s_offset + static_cast<uint64_t>(date - 1) * c.path_count + i);
            if (!(intrinsic(s, c.strike, c.type) > 0.0)) continue;
            double b[4];
            basis64(s, c.strike, b);
            // b'_l = sum_{j <= l} b_j T[j][l]
            double q0 = b[0] * T[0];
            double q1 = b[0] * T[1] + b[1] * T[4];
            double q2 = b[0] * T[2] + b[1] * T[5] + b[2] * T[7];
            double q3 = b[0] * T[3] + b[1] * T[6] + b[2] * T[8] + b[3] * T[9];
            const double y = cf[c.cf_offset + i];
            acc[0] += 1.0;
            acc[1] += q0 * q0;
            acc[2] += q0 * q1;
            acc[3] += q0 * q2;
            acc[4] += q0 * q3;
            acc[5] += q1 * q1;
            acc[6] += q1 * q2;
            acc[7] += q1 * q3;
            acc[8] += q2 * q2;
            acc[9] += q2 * q3;
            acc[10] += q3 * q3;
            acc[11] += q0 * y;
            acc[12] += q1 * y;
            acc[13] += q2 * y;
            acc[14] += q3 * y;
        }
        block_sum<15>(acc, smem);
#pragma unroll
        for (int q = 0; q < 15; ++q) out[q] = acc[q];
    } else {
        float T[10];
#pragma unroll
        for (int q = 0; q < 10; ++q) T[q] = r.T_f[q];
        const float phi = c.phi_f, strike = c.strike_f, inv_kf = c.inv_strike_f;
        const float* S = static_cast<const float*>(store) + c.s_offset;
        float hi[15], lo[15];
#pragma unroll
        for (int q = 0; q < 15; ++q) hi[q] = lo[q] = 0.0f;
        constexpr int kPer = kLsmChunk / kLsmThreads;
        float sv[kPer], yv[kPer];
        bool live[kPer];
        const float* cff = reinterpret_cast<const float*>(cf) + c.cf_offset;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint64_t i = static_cast<uint64_t>(local) * kLsmChunk + j * kLsmThreads + threadIdx.x;
            live[j] = i < c.path_count;
            sv[j] = live[j] ? S[static_cast<uint64_t>(date - 1) * c.path_count + i] : 0.0f;
            yv[j] = live[j] ? cff[i] : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            if (!live[j] || !(phi * (sv[j] - strike) > 0.0f)) continue;
            float b[4];
            basis32(sv[j], inv_kf, b);
            const float q0 = b[0] * T[0];
            const float q1 = __fmaf_rn(b[1], T[4], b[0] * T[1]);
            const float q2 = __fmaf_rn(b[2], T[7], __fmaf_rn(b[1], T[5], b[0] * T[2]));
            const float q3 = __fmaf_rn(b[3], T[9], __fmaf_rn(b[2], T[8], __fmaf_rn(b[1], T[6], b[0] * T[3])));
            const float y = yv[j];
            df_add(hi[0], lo[0], 1.0f);
            df_add(hi[1], lo[1], q0 * q0);
            df_add(hi[2], lo[2], q0 * q1);
            df_add(hi[3], lo[3], q0 * q2);
            df_add(hi[4], lo[4], q0 * q3);
            df_add(hi[5], lo[5], q1 * q1);
            df_add(hi[6], lo[6], q1 * q2);
            df_add(hi[7], lo[7], q1 * q3);
            df_add(hi[8], lo[8], q2 * q2);
            df_add(hi[9], lo[9], q2 * q3);
            df_add(hi[10], lo[10], q3 * q3);
            df_add(hi[11], lo[11], q0 * y);
            df_add(hi[12], lo[12], q1 * y);
            df_add(hi[13], lo[13], q2 * y);
            df_add(hi[14], lo[14], q3 * y);
        }
        block_sum_df<15>(hi, lo, scratch, sres, out);
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < 15; ++q) part_b[chunk].v[q] = out[q];
    }
}

// 4x4 Householder least squares (the reference's algorithm, src/core/linalg.cpp:7-71,
// on a square system): A is overwritten, y too.
__device__ void householder4(double A[4][4], double y[4], double beta[4]) {
    for (int kk = 0; kk < 4; ++kk) {
        double norm_sq = 0.0;
        for (int i = kk; i < 4; ++i) norm_sq += A[i][kk] * A[i][kk];
        const double norm = sqrt(norm_sq);
        if (norm == 0.0) continue;
        const double akk = A[kk][kk];
        const double alpha = akk >= 0.0 ? -norm : norm;
        double v[4] = {0, 0, 0, 0};
        v[kk] = akk - alpha;
        for (int i = kk + 1; i < 4; ++i) v[i] = A[i][kk];
        double vn = 0.0;
        for (int i = kk; i < 4; ++i) vn += v[i] * v[i];
        if (vn == 0.0) continue;
        for (int jj = kk; jj < 4; ++jj) {
            double dot = 0.0;
            for (int i = kk; i < 4; ++i) dot += v[i] * A[i][jj];
            const double f = 2.0 * dot / vn;
            for (int i = kk; i < 4; ++i) A[i][jj] -= f * v[i];
        }
        double dy = 0.0;
        for (int i = kk; i < 4; ++i) dy += v[i] * y[i];
        const double fy = 2.0 * dy / vn;
        for (int i = kk; i < 4; ++i) y[i] -= fy * v[i];
    }
    for (int i = 3; i >= 0; --i) {
        double sum = y[i];
        for (int jj = i + 1; jj < 4; ++jj) sum -= A[i][jj] * beta[jj];
        const double diag = A[i][i];
        beta[i] = diag != 0.0 ? sum / diag : 0.0;
    }
}

__global__ void lsm_solve_b(int k, const LsmDev* __restrict__ cs, int n_contracts,
                            const LsmPartial* __restrict__ part_b, LsmReg* __restrict__ reg) {
    const int ci = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (ci >= n_contracts) return;
    const LsmDev c = cs[ci];
    const int date = c.n_steps - k - 1;
    if (date < 1) return;
    LsmReg& r = reg[c.reg_offset + date];
    if (r.has == -1) return;
    double s[15];
#pragma unroll
    for (int q = 0; q < 15; ++q) s[q] = 0.0;
    for (uint32_t ch = lane; ch < c.n_chunks; ch += 32)
#pragma unroll
        for (int q = 0; q < 15; ++q) s[q] += part_b[c.chunk_begin + ch].v[q];
#pragma unroll
    for (int q = 0; q < 15; ++q)
        for (int off = 16; off >= 1; off >>= 1) s[q] += __shfl_down_sync(0xffffffffu, s[q], off);
    if (lane != 0) return;
    double G[4][4], y[4], beta[4] = {0, 0, 0, 0};
    for (int a = 0; a < 4; ++a)
        for (int b2 = a; b2 < 4; ++b2) G[a][b2] = G[b2][a] = s[1 + tri(a, b2)];
    for (int a = 0; a < 4; ++a) y[a] = s[11 + a];
    householder4(G, y, beta);
    // gamma = T beta
    for (int a = 0; a < 4; ++a) {
        double x = 0.0;
        for (int b2 = a; b2 < 4; ++b2) x += r.T[tri(a, b2)] * beta[b2];
        r.gamma[a] = x;
        r.gamma_f[a] = static_cast<float>(x);
    }
    r.has = 1;
}

__global__ void lsm_finish(const LsmDev* __restrict__ cs, int n_contracts,
                           const Welford* __restrict__ final_part, double* __restrict__ out) {
    const int ci = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (ci >= n_contracts) return;
    const LsmDev c = cs[ci];
    Welford w{0ull, 0.0, 0.0};
    for (uint32_t ch = lane; ch < c.n_chunks; ch += 32) w = welford_merge(w, final_part[c.chunk_begin + ch]);
    w = welford_warp_reduce(w);
    if (lane != 0) return;
    const double var = w.count < 2 ? 0.0 : w.m2 / static_cast<double>(w.count - 1);
    const double se = w.count == 0 ? 0.0 : sqrt(var / static_cast<double>(w.count));
    // inception decision (src/pricers/lsm.cpp:141-148)
    const bool ex0 = c.inception > w.mean;
    out[6 * ci + 0] = ex0 ? c.inception : w.mean;
    out[6 * ci + 1] = ex0 ? 0.0 : se;
    out[6 * ci + 2] = static_cast<double>(w.count);
    out[6 * ci + 3] = ex0 ? 1.0 : 0.0;
    out[6 * ci + 4] = w.mean;  // path average before the inception test
    out[6 * ci + 5] = se;
}

}  // namespace

cudaError_t launch_lsm_forward(int precision, const LsmDev* c, int n_contracts,
                               const uint32_t* chunk_contract, uint32_t total_chunks, void* s_store,
                               cudaStream_t stream) {
    (void)n_contracts;
    cudaGetLastError();
    if (total_chunks == 0) return cudaSuccess;
    if (precision == 0)
        lsm_forward<0><<<total_chunks, kLsmThreads, 0, stream>>>(c, chunk_contract, total_chunks, s_store);
    else
        lsm_forward<1><<<total_chunks, kLsmThreads, 0, stream>>>(c, chunk_contract, total_chunks, s_store);
    return cudaGetLastError();
}

cudaError_t launch_lsm_iteration(int precision, int k, const LsmDev* c, int n_contracts,
                                 const uint32_t* chunk_contract, uint32_t total_chunks, const void* s_store,
                                 double* cf, LsmReg* reg, LsmPartial* part_a, LsmPartial* part_b,
                                 Welford* final_part, cudaStream_t stream) {
    cudaGetLastError();
    if (total_chunks == 0) return cudaSuccess;
    const int solve_blocks = (n_contracts * 32 + 127) / 128;
    if (precision == 0)
        lsm_exercise<0><<<total_chunks, kLsmThreads, 0, stream>>>(k, c, chunk_contract, total_chunks, s_store, cf,
                                                                  reg, part_a, final_part);
    else
        lsm_exercise<1><<<total_chunks, kLsmThreads, 0, stream>>>(k, c, chunk_contract, total_chunks, s_store, cf,
                                                                  reg, part_a, final_part);
    lsm_solve_a<<<solve_blocks, 128, 0, stream>>>(k, c, n_contracts, part_a, reg);
    if (precision == 0)
        lsm_gram_b<0><<<total_chunks, kLsmThreads, 0, stream>>>(k, c, chunk_contract, total_chunks, s_store, cf, reg,
                                                                part_b);
    else
        lsm_gram_b<1><<<total_chunks, kLsmThreads, 0, stream>>>(k, c, chunk_contract, total_chunks, s_store, cf, reg,
                                                                part_b);
    lsm_solve_b<<<solve_blocks, 128, 0, stream>>>(k, c, n_contracts, part_b, reg);
    return cudaGetLastError();
}

cudaError_t launch_lsm_finish(const LsmDev* c, int n_contracts, const Welford* final_part,
                              double* out, cudaStream_t stream) {
    cudaGetLastError();
    lsm_finish<<<(n_contracts * 32 + 127) / 128, 128, 0, stream>>>(c, n_contracts, final_part, out);
    return cudaGetLastError();
}

}  // namespace mcdg
