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
// handles date e = n_c - k of contract c, in one pass over the date's columns
// (lsm_step): exercise at date e with that date's coefficients, discount, and
// either the regression sums of date e-1 -- Gram matrix and right-hand side
// in the basis b T_e, T_e being date e's preconditioner (adjacent dates'
// in-the-money populations are alike, so b T_e is already close to
// orthonormal on date e-1) -- or, when e = 1, the final Welford partial.  The
// last CTA of a contract to finish folds the chunk partials in chunk order
// and solves date e-1 (no separate launch; no CTA waits for another): the
// Cholesky factor R of the lagged Gram matrix gives date e-1's own
// preconditioner T = T_e R^{-1}; when that matrix is well conditioned the 4x4
// Householder solve of the preconditioned normal equations gives the
// coefficients at once.  Otherwise -- always on the first regression date,
// whose lag is the identity (cond of the raw Laguerre Gram matrix reaches
// ~4e12) -- lsm_refine makes a second pass in the basis b T and solves it:
// Cholesky-QR2 for that date.  Either way the coefficients agree with the
// reference's Householder QR to the limit set by the least-squares
// conditioning (its own algorithm moves them that much when the rows are
// reordered), and the fitted continuation values, hence the exercise
// decisions, coincide.  Every reduction tree is fixed by chunk index.
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

// Chunk reduction of plain FP32 per-thread sums (the FP32 step's sums in a
// well-conditioned basis): thread partials go to shared memory, warp w folds
// sums w, w + W, ... (W warps): lane l adds threads l, l + 32, ... in that
// order, then a shuffle tree; lane 0 widens the chunk's sum to FP64 in res.
// FP32 up to the chunk (1024 paths), FP64 above.
template <int N>
__device__ void block_sum_f32(const float (&v)[N], float (*scratch)[kLsmThreads], double* res) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int i = 0; i < N; ++i) scratch[i][t] = v[i];
    __syncthreads();
    for (int i = warp; i < N; i += kLsmThreads / 32) {
        float x = scratch[i][lane];
#pragma unroll
        for (int u = 1; u < kLsmThreads / 32; ++u) x += scratch[i][lane + 32 * u];
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
        if (lane == 0) res[i] = static_cast<double>(x);
    }
    __syncthreads();
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
                uint32_t chunk_first, uint32_t chunk_end, void* __restrict__ store) {
    const uint32_t chunk = chunk_first + blockIdx.x;
    if (chunk >= chunk_end) return;
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
                s = gbm_step_f64(s, z, c.drift, c.vs);
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
                float* out = S + i;  // date d's column, advanced by one column per date
                for (int d = 0; d < c.n_steps; ++d) {
                    const float z = normal_from_bits_f32(philox_word0(pp, static_cast<uint32_t>(d), k));
                    const float z2 = normal_from_bits_f32(philox_word0(pp2, static_cast<uint32_t>(d), k));
                    x = gbm_log_step_f32(x, z, mu, sg);
                    x2 = gbm_log_step_f32(x2, z2, mu, sg);
                    out[0] = gbm_spot_f32(s0, x);
                    out[kLsmThreads] = gbm_spot_f32(s0, x2);
                    out += c.path_count;
                }
                ++j;  // the partner path is done
                continue;
            }
            float x = 0.0f;
            for (int d = 0; d < c.n_steps; ++d) {
                const float z = normal_from_bits_f32(philox_word0(pp, static_cast<uint32_t>(d), k));
                x = gbm_log_step_f32(x, z, mu, sg);
                S[static_cast<uint64_t>(d) * c.path_count + i] = gbm_spot_f32(s0, x);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// per-date 4x4 algebra (FP64, one thread)
// ---------------------------------------------------------------------------
// Upper-triangular index of (r, c), r <= c, in the packed 10-entry layout.
__device__ __forceinline__ int tri(int r, int col) {
    const int base[4] = {0, 4, 7, 9};
    return base[r] + (col - r);
}

// Cholesky factor of G + shift I = R^T R (R upper); false when a pivot is
// not positive.
__device__ bool chol4(const double G[4][4], double shift, double R[4][4]) {
    for (int a = 0; a < 4; ++a)
        for (int b2 = 0; b2 < 4; ++b2) R[a][b2] = 0.0;
    for (int j = 0; j < 4; ++j) {
        double d = G[j][j] + shift;
        for (int p = 0; p < j; ++p) d -= R[p][j] * R[p][j];
        if (!(d > 0.0)) return false;
        R[j][j] = sqrt(d);
        for (int l = j + 1; l < 4; ++l) {
            double x = G[j][l];
            for (int p = 0; p < j; ++p) x -= R[p][j] * R[p][l];
            R[j][l] = x / R[j][j];
        }
    }
    return true;
}

// The same factorisation without divisions (FP64 division and square root
// are long software sequences on this GPU's FP64 pipe): one reciprocal square
// root per pivot, rinv[j] = 1 / R[j][j].
__device__ bool chol4_rsqrt(const double G[4][4], double R[4][4], double rinv[4]) {
    for (int a = 0; a < 4; ++a)
        for (int b2 = 0; b2 < 4; ++b2) R[a][b2] = 0.0;
    for (int j = 0; j < 4; ++j) {
        double d = G[j][j];
        for (int p = 0; p < j; ++p) d -= R[p][j] * R[p][j];
        if (!(d > 0.0)) return false;
        const double r = rsqrt(d);
        rinv[j] = r;
        R[j][j] = d * r;
        for (int l = j + 1; l < 4; ++l) {
            double x = G[j][l];
            for (int p = 0; p < j; ++p) x -= R[p][j] * R[p][l];
            R[j][l] = x * r;
        }
    }
    return true;
}

// T = R^{-1} from the pivots' reciprocals.
__device__ void inv_upper4_rinv(const double R[4][4], const double rinv[4], double T[4][4]) {
    for (int a = 0; a < 4; ++a)
        for (int b2 = 0; b2 < 4; ++b2) T[a][b2] = 0.0;
    for (int j = 3; j >= 0; --j) {
        T[j][j] = rinv[j];
        for (int l = j + 1; l < 4; ++l) {
            double x = 0.0;
            for (int p = j; p < l; ++p) x += T[j][p] * R[p][l];
            T[j][l] = -x * rinv[l];
        }
    }
}

// T = R^{-1} for upper-triangular R.
__device__ void inv_upper4(const double R[4][4], double T[4][4]) {
    for (int a = 0; a < 4; ++a)
        for (int b2 = 0; b2 < 4; ++b2) T[a][b2] = 0.0;
    for (int j = 3; j >= 0; --j) {
        T[j][j] = 1.0 / R[j][j];
        for (int l = j + 1; l < 4; ++l) {
            double x = 0.0;
            for (int p = j; p < l; ++p) x += T[j][p] * R[p][l];
            T[j][l] = -x / R[l][l];
        }
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

__device__ __forceinline__ void unpack_upper(const double* packed, double T[4][4]) {
    for (int a = 0; a < 4; ++a)
        for (int b2 = 0; b2 < 4; ++b2) T[a][b2] = b2 >= a ? packed[tri(a, b2)] : 0.0;
}

__device__ __forceinline__ void store_T(LsmReg& r, const double T[4][4]) {
    for (int a = 0; a < 4; ++a)
        for (int b2 = a; b2 < 4; ++b2) {
            r.T[tri(a, b2)] = T[a][b2];
            r.T_f[tri(a, b2)] = static_cast<float>(T[a][b2]);
        }
}

// Least squares on the preconditioned normal equations: s = (count, 10
// packed entries of G = P^T X^T X P, 4 entries of h = P^T X^T y) for the
// basis X P of preconditioner P (upper triangular).  Solves G beta = h by
// the 4x4 Householder QR and returns gamma = P beta, the coefficients in the
// Laguerre basis (the reference's policy layout).
__device__ void solve_preconditioned(const double s[15], const double P[4][4], double gamma[4]) {
    double G[4][4], y[4], beta[4] = {0, 0, 0, 0};
    for (int a = 0; a < 4; ++a)
        for (int b2 = a; b2 < 4; ++b2) G[a][b2] = G[b2][a] = s[1 + tri(a, b2)];
    for (int a = 0; a < 4; ++a) y[a] = s[11 + a];
    householder4(G, y, beta);
    for (int a = 0; a < 4; ++a) {
        double x = 0.0;
        for (int b2 = a; b2 < 4; ++b2) x += P[a][b2] * beta[b2];
        gamma[a] = x;
    }
}

// The regression of one date from its sums in the basis of the lagged
// preconditioner L (the next later date's T).  Cholesky of G' = R^T R gives
// this date's preconditioner T = L R^{-1} (so that T^T X^T X T = I).  When G'
// is well conditioned (cond bound ||R||_F^2 ||R^-1||_F^2 <= kappa_max) the
// date is solved here from the same factor, beta = R^{-1} R^{-T} h and
// gamma = L beta: has = 1.  Otherwise T is stored and the date is marked for
// a second pass in the basis X T (has = 2): that pass and its Householder
// solve are Cholesky-QR2.  The first regression date (L = I, the raw Laguerre
// Gram matrix, condition up to ~1e13) always takes it; where that raw matrix
// is not numerically positive definite (its FP32-path sums carry ~44 bits) the
// factorisation is retried with a diagonal shift of 1e-10 of the trace --
// shifted Cholesky QR (Fukaya, Kannan, Nakatsukasa, Zhang and Yamamoto, SIAM
// J. Sci. Comput. 42 (2020)) -- and the second pass fits the unshifted problem.
__device__ void solve_lagged(const double s[15], const double L[4][4], double kappa_max, LsmReg& r,
                             uint32_t* need_second_pass) {
    if (s[0] < 4.0) {  // too few in-the-money paths (src/pricers/lsm.cpp:102-104)
        r.has = -1;
        r.degenerate = 0;
        store_T(r, L);  // the lag passes through to the next earlier date
        return;
    }
    double G[4][4];
    for (int a = 0; a < 4; ++a)
        for (int b2 = a; b2 < 4; ++b2) G[a][b2] = G[b2][a] = s[1 + tri(a, b2)];
    double R[4][4], Ri[4][4], T[4][4], rinv[4];
    bool ok = chol4_rsqrt(G, R, rinv);
    double kappa = 1e300;
    if (ok) {
        inv_upper4_rinv(R, rinv, Ri);
        double fr = 0.0, fi = 0.0;
        for (int a = 0; a < 4; ++a)
            for (int b2 = a; b2 < 4; ++b2) {
                fr += R[a][b2] * R[a][b2];
                fi += Ri[a][b2] * Ri[a][b2];
            }
        kappa = fr * fi;
    }
    r.degenerate = 0;
    if (!ok) {
        const double shift = 1e-10 * (G[0][0] + G[1][1] + G[2][2] + G[3][3]);
        ok = chol4(G, shift, R);
        if (ok) inv_upper4(R, Ri);
        r.degenerate = ok ? 2 : 1;
    }
    if (ok) {
        for (int a = 0; a < 4; ++a)
            for (int b2 = 0; b2 < 4; ++b2) {
                double x = 0.0;
                for (int p = a; p <= b2; ++p) x += L[a][p] * Ri[p][b2];
                T[a][b2] = b2 >= a ? x : 0.0;
            }
    } else {
        for (int a = 0; a < 4; ++a)
            for (int b2 = 0; b2 < 4; ++b2) T[a][b2] = L[a][b2];
    }
    store_T(r, T);
    if (r.degenerate == 0 && kappa <= kappa_max) {
        double w[4], beta[4];
        for (int l = 0; l < 4; ++l) {  // w = R^{-T} h
            double x = 0.0;
            for (int p = 0; p <= l; ++p) x += Ri[p][l] * s[11 + p];
            w[l] = x;
        }
        for (int a = 0; a < 4; ++a) {  // beta = R^{-1} w
            double x = 0.0;
            for (int b2 = a; b2 < 4; ++b2) x += Ri[a][b2] * w[b2];
            beta[a] = x;
        }
        for (int a = 0; a < 4; ++a) {  // gamma = L beta
            double x = 0.0;
            for (int b2 = a; b2 < 4; ++b2) x += L[a][b2] * beta[b2];
            r.gamma[a] = x;
            r.gamma_f[a] = static_cast<float>(x);
        }
        laguerre_poly(r.gamma, r.poly_f);
        r.has = 1;
    } else {
        r.has = 2;
        atomicAdd(need_second_pass, 1u);
    }
}

// Fixed-order fold of a contract's chunk partials by the whole CTA: thread t
// takes chunks t, t + 256, ... in order, then the fixed block tree; the
// result is valid in thread 0.
template <int N>
__device__ void fold_partials(const LsmPartial* __restrict__ part, uint32_t begin, uint32_t count,
                              double (&v)[N], double (*smem)[N]) {
#pragma unroll
    for (int q = 0; q < N; ++q) v[q] = 0.0;
    for (uint32_t ch = threadIdx.x; ch < count; ch += kLsmThreads) {
        const double* p = part[begin + ch].v;
#pragma unroll
        for (int q = 0; q < N; ++q) v[q] += __ldcg(p + q);
    }
    block_sum<N>(v, smem);
}

// One arrival at a completion counter; true in the CTA that arrives last.
// The arriving CTA's writes (thread 0's) are fenced before the counter is
// bumped, the last arrival fences again before it reads the others', and
// resets the counter for the next launch.  No CTA waits on another.
__device__ __forceinline__ bool last_arrival(uint32_t* counter, uint32_t expected, int* s_flag) {
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t prev = atomicAdd(counter, 1u);
        const bool last = prev == expected - 1;
        if (last) *counter = 0u;
        *s_flag = last ? 1 : 0;
    }
    __syncthreads();
    const bool last = *s_flag != 0;
    if (last) __threadfence();
    return last;
}

// Publishes this CTA's chunk partial (thread 0 wrote part[chunk]) and climbs
// the two-level tree of the contract's sums: the last chunk of a group of
// LsmDev::fold_chunks chunks folds the group's partials in chunk order into
// the group partial, the last group of the contract folds the group partials
// in group order.  Every fold is short (a few dozen to a few hundred rows over
// the whole CTA), so the contract's totals are ready soon after its last
// chunk.  Returns true in the CTA holding the totals (valid in thread 0).
// counters: the group counter of group g at group_counters[2 g], the
// contract's at *contract_counter.
__device__ bool publish_and_fold(uint32_t chunk, const LsmDev& c, const LsmPartial* __restrict__ part,
                                 LsmPartial* __restrict__ gpart, uint32_t* group_counters,
                                 uint32_t* contract_counter, double (&tot)[15], double (*smem)[15],
                                 int* s_flag) {
    const uint32_t local = chunk - c.chunk_begin;
    const uint32_t g = local / c.fold_chunks;
    const uint32_t first = g * c.fold_chunks;
    const uint32_t count = min(c.fold_chunks, c.n_chunks - first);
    if (!last_arrival(&group_counters[2 * (c.fold_begin + g)], count, s_flag)) return false;
    fold_partials<15>(part, c.chunk_begin + first, count, tot, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < 15; ++q) gpart[c.fold_begin + g].v[q] = tot[q];
    }
    if (!last_arrival(contract_counter, c.n_folds, s_flag)) return false;
    fold_partials<15>(gpart, c.fold_begin, c.n_folds, tot, smem);
    return true;
}

// ---------------------------------------------------------------------------
// iteration k: exercise at date e, discount, and the regression sums of date
// e-1 in the lagged basis -- or, when e = 1, the final Welford partial.  The
// contract's last CTA folds the sums and solves date e-1.
// ---------------------------------------------------------------------------
// COMP (FP32 path): the sums are compensated FP32 per thread and chunk (the
// first iteration, whose basis is the raw Laguerre one); otherwise plain FP32
// per thread and chunk -- the lagged basis is close to orthonormal, where
// FP32 sums lose nothing the FP32 path data does not already carry.
template <int PREC, bool COMP>
__global__ void __launch_bounds__(kLsmThreads, PREC == 0 ? 1 : 8)
    lsm_step(int k, const LsmDev* __restrict__ cs, const uint32_t* __restrict__ chunk_contract,
             uint32_t chunk_first, uint32_t chunk_end, const void* __restrict__ store, double* __restrict__ cf,
             LsmReg* __restrict__ reg, LsmPartial* __restrict__ part, LsmPartial* __restrict__ gpart,
             Welford* __restrict__ final_part, uint32_t* __restrict__ counters,
             uint32_t* __restrict__ group_counters, uint32_t* __restrict__ need_second_pass, double kappa_max) {
    __shared__ double smem[kLsmThreads / 32][15];
    __shared__ float2 scratch[COMP ? 15 : 1][kLsmThreads];  // compensated sums' per-thread pairs
    __shared__ float pscratch[COMP ? 1 : 15][kLsmThreads];  // plain sums' per-thread values
    __shared__ double sres[15];
    __shared__ Welford swf[kLsmThreads / 32];
    __shared__ Sum64 s64[kLsmThreads / 32];
    __shared__ int s_last;
    const uint32_t chunk = chunk_first + blockIdx.x;
    if (chunk >= chunk_end) return;
    const uint32_t ci = chunk_contract[chunk];
    const LsmDev c = cs[ci];
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
    double out[15];
    if constexpr (PREC == 0) {
        // lagged preconditioner: date e's T (identity before the first regression)
        double T[10];
#pragma unroll
        for (int q = 0; q < 10; ++q) T[q] = init ? ((q == 0 || q == 4 || q == 7 || q == 9) ? 1.0 : 0.0) : re->T[q];
        double acc[15];
#pragma unroll
        for (int q = 0; q < 15; ++q) acc[q] = 0.0;
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
                const double s = load_s<PREC>(store, c.s_offset + static_cast<uint64_t>(e - 2) * c.path_count + i);
                if (intrinsic(s, c.strike, c.type) > 0.0) {
                    double b[4];
                    basis64(s, c.strike, b);
                    // b'_l = sum_{j <= l} b_j T[j][l]
                    const double q0 = b[0] * T[0];
                    const double q1 = b[0] * T[1] + b[1] * T[4];
                    const double q2 = b[0] * T[2] + b[1] * T[5] + b[2] * T[7];
                    const double q3 = b[0] * T[3] + b[1] * T[6] + b[2] * T[8] + b[3] * T[9];
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
                    acc[11] += q0 * v;
                    acc[12] += q1 * v;
                    acc[13] += q2 * v;
                    acc[14] += q3 * v;
                }
            }
        }
        if (gram) {
            block_sum<15>(acc, smem);
#pragma unroll
            for (int q = 0; q < 15; ++q) out[q] = acc[q];
        }
    } else {
        // FP32 paths: FP32 cash flows (stored in the FP64 buffer's space),
        // basis, continuation value, exercise tests and products; the sums
        // and the final payoff sums up to the warp are compensated FP32,
        // everything above FP64.
        const float phi = c.phi_f, strike = c.strike_f, inv_kf = c.inv_strike_f, disc = c.disc_f;
        float poly[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (exercise) {
#pragma unroll
            for (int q = 0; q < 4; ++q) poly[q] = re->poly_f[q];
        }
        float T[10];
#pragma unroll
        for (int q = 0; q < 10; ++q) T[q] = init ? ((q == 0 || q == 4 || q == 7 || q == 9) ? 1.0f : 0.0f) : re->T_f[q];
        const float* S = static_cast<const float*>(store) + c.s_offset;
        float* cff = reinterpret_cast<float*>(cf) + c.cf_offset;
        float hi[15], lo[15];
#pragma unroll
        for (int q = 0; q < 15; ++q) hi[q] = lo[q] = 0.0f;
        Sum32 fin{0u, 0.0f, 0.0f, 0.0f, 0.0f};  // final payoffs (last date)
        constexpr int kPer = kLsmChunk / kLsmThreads;
        // all loads of this thread's paths first (independent, in flight together);
        // the columns' thread bases once, 32-bit offsets within the chunk
        const uint64_t cb = static_cast<uint64_t>(local) * kLsmChunk;  // first path of the chunk
        const uint64_t i0 = cb + threadIdx.x;
        const uint32_t in_chunk = static_cast<uint32_t>(
            c.path_count - cb < static_cast<uint64_t>(kLsmChunk) ? c.path_count - cb : static_cast<uint64_t>(kLsmChunk));
        float* cf_t = cff + i0;
        const float* col_v = init ? S + static_cast<uint64_t>(n - 1) * c.path_count + i0 : cf_t;
        const float* col_e = S + static_cast<uint64_t>(exercise ? e - 1 : 0) * c.path_count + i0;
        const float* col_d = S + static_cast<uint64_t>(gram ? e - 2 : 0) * c.path_count + i0;
        float vv[kPer], se[kPer], sd[kPer];
        bool live[kPer];
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint32_t o = static_cast<uint32_t>(j * kLsmThreads);
            live[j] = o + threadIdx.x < in_chunk;
            vv[j] = 0.0f;
            se[j] = 0.0f;
            sd[j] = 0.0f;
            if (live[j]) {
                vv[j] = col_v[o];
                if (exercise) se[j] = col_e[o];
                if (gram) sd[j] = col_d[o];
            }
        }
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            if (!live[j]) continue;
            float v = init ? fmaxf(phi * (vv[j] - strike), 0.0f) : vv[j];
            if (exercise) {
                const float ex = phi * (se[j] - strike);
                if (ex > 0.0f && ex > continuation_poly32(se[j], inv_kf, poly)) v = ex;
            }
            v *= disc;
            if (last) {
                sum32_add(fin, v);
            } else {
                cf_t[j * kLsmThreads] = v;
                if (phi * (sd[j] - strike) > 0.0f) {
                    float b[4];
                    basis32(sd[j], inv_kf, b);
                    const float q0 = b[0] * T[0];
                    const float q1 = __fmaf_rn(b[1], T[4], b[0] * T[1]);
                    const float q2 = __fmaf_rn(b[2], T[7], __fmaf_rn(b[1], T[5], b[0] * T[2]));
                    const float q3 = __fmaf_rn(b[3], T[9], __fmaf_rn(b[2], T[8], __fmaf_rn(b[1], T[6], b[0] * T[3])));
                    if constexpr (!COMP) {
                        hi[0] += 1.0f;  // exact: a chunk holds fewer than 2^24 paths
                        hi[1] = __fmaf_rn(q0, q0, hi[1]);
                        hi[2] = __fmaf_rn(q0, q1, hi[2]);
                        hi[3] = __fmaf_rn(q0, q2, hi[3]);
                        hi[4] = __fmaf_rn(q0, q3, hi[4]);
                        hi[5] = __fmaf_rn(q1, q1, hi[5]);
                        hi[6] = __fmaf_rn(q1, q2, hi[6]);
                        hi[7] = __fmaf_rn(q1, q3, hi[7]);
                        hi[8] = __fmaf_rn(q2, q2, hi[8]);
                        hi[9] = __fmaf_rn(q2, q3, hi[9]);
                        hi[10] = __fmaf_rn(q3, q3, hi[10]);
                        hi[11] = __fmaf_rn(q0, v, hi[11]);
                        hi[12] = __fmaf_rn(q1, v, hi[12]);
                        hi[13] = __fmaf_rn(q2, v, hi[13]);
                        hi[14] = __fmaf_rn(q3, v, hi[14]);
                        continue;
                    }
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
                    df_add(hi[11], lo[11], q0 * v);
                    df_add(hi[12], lo[12], q1 * v);
                    df_add(hi[13], lo[13], q2 * v);
                    df_add(hi[14], lo[14], q3 * v);
                }
            }
        }
        if (last) {
            const Sum32 r = sum32_warp_reduce(fin);
            if ((threadIdx.x & 31) == 0) s64[threadIdx.x >> 5] = sum32_wide(r);
        }
        if (gram) {
            if constexpr (COMP) {
                block_sum_df<15>(hi, lo, scratch, sres, out);
            } else {
                block_sum_f32<15>(hi, pscratch, sres);
#pragma unroll
                for (int q = 0; q < 15; ++q) out[q] = sres[q];
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
        return;
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < 15; ++q) part[chunk].v[q] = out[q];
    }
    double tot[15];
    if (!publish_and_fold(chunk, c, part, gpart, group_counters, &counters[2 * ci], tot, smem, &s_last)) return;
    if (threadIdx.x == 0) {
        double L[4][4];
        if (init) {
            for (int a = 0; a < 4; ++a)
                for (int b2 = 0; b2 < 4; ++b2) L[a][b2] = a == b2 ? 1.0 : 0.0;
        } else {
            unpack_upper(re->T, L);
        }
        solve_lagged(tot, L, kappa_max, reg[c.reg_offset + e - 1], need_second_pass + k);
    }
}

// Second pass for the dates solve_lagged marked (has = 2): the sums in the
// basis of that date's own preconditioner T (compensated FP32 on the FP32
// path), then the contract's last chunk solves (has = 1).  A small
// persistent grid walks the chunks and skips those of other contracts.
template <int PREC>
__global__ void __launch_bounds__(kLsmThreads, PREC == 0 ? 1 : 4)
    lsm_refine(int k, const LsmDev* __restrict__ cs, const uint32_t* __restrict__ chunk_contract,
               uint32_t chunk_first, uint32_t chunk_end, const void* __restrict__ store, const double* __restrict__ cf,
               LsmReg* __restrict__ reg, LsmPartial* __restrict__ part, LsmPartial* __restrict__ gpart,
               uint32_t* __restrict__ counters, uint32_t* __restrict__ group_counters,
               const uint32_t* __restrict__ need_second_pass) {
    __shared__ double smem[kLsmThreads / 32][15];
    __shared__ float2 scratch[15][kLsmThreads];  // FP32 path: the sums' per-thread pairs
    __shared__ double sres[15];
    __shared__ int s_last;
    if (__ldcg(need_second_pass + k) == 0) return;  // no date of this iteration needs it
    for (uint32_t chunk = chunk_first + blockIdx.x; chunk < chunk_end; chunk += gridDim.x) {
    const uint32_t ci = chunk_contract[chunk];
    const LsmDev c = cs[ci];
    const int date = c.n_steps - k - 1;
    if (date < 1) continue;
    LsmReg& r = reg[c.reg_offset + date];
    if (r.has != 2) continue;  // solved by the first pass, or no regression at this date
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
            const double q0 = b[0] * T[0];
            const double q1 = b[0] * T[1] + b[1] * T[4];
            const double q2 = b[0] * T[2] + b[1] * T[5] + b[2] * T[7];
            const double q3 = b[0] * T[3] + b[1] * T[6] + b[2] * T[8] + b[3] * T[9];
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
        for (int q = 0; q < 15; ++q) part[chunk].v[q] = out[q];
    }
    double tot[15];
    if (publish_and_fold(chunk, c, part, gpart, group_counters + 1, &counters[2 * ci + 1], tot, smem, &s_last)) {
        if (threadIdx.x == 0) {
            double T[4][4], gamma[4];
            unpack_upper(r.T, T);
            solve_preconditioned(tot, T, gamma);
            for (int a = 0; a < 4; ++a) {
                r.gamma[a] = gamma[a];
                r.gamma_f[a] = static_cast<float>(gamma[a]);
            }
            laguerre_poly(r.gamma, r.poly_f);
            r.has = 1;
        }
    }
    __syncthreads();  // shared memory is reused by the next chunk
    }
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
                               const uint32_t* chunk_contract, uint32_t chunk_first, uint32_t chunk_count,
                               void* s_store, cudaStream_t stream) {
    (void)n_contracts;
    cudaGetLastError();
    if (chunk_count == 0) return cudaSuccess;
    const uint32_t end = chunk_first + chunk_count;
    if (precision == 0)
        lsm_forward<0><<<chunk_count, kLsmThreads, 0, stream>>>(c, chunk_contract, chunk_first, end, s_store);
    else
        lsm_forward<1><<<chunk_count, kLsmThreads, 0, stream>>>(c, chunk_contract, chunk_first, end, s_store);
    return cudaGetLastError();
}

cudaError_t launch_lsm_iteration(int precision, int k, const LsmDev* c, int n_contracts,
                                 const uint32_t* chunk_contract, uint32_t chunk_first, uint32_t chunk_count,
                                 uint32_t total_folds, const void* s_store, double* cf, LsmReg* reg,
                                 LsmPartial* part, LsmPartial* gpart, Welford* final_part, uint32_t* counters,
                                 cudaStream_t stream) {
    cudaGetLastError();
    if (chunk_count == 0) return cudaSuccess;
    const uint32_t end = chunk_first + chunk_count;
    // counters: 2 per contract (first pass, second pass), 2 per fold group, then
    // one word per iteration counting the dates marked for the second pass
    // (shared by concurrent chains: a chain's second pass reads it after its
    // own first pass, and only adds are made to it).
    uint32_t* group_counters = counters + 2 * static_cast<size_t>(n_contracts);
    uint32_t* need = group_counters + 2 * static_cast<size_t>(total_folds);
    // The second pass always runs after the first iteration (its lag is the
    // identity), on a CTA per chunk; later it is rare and runs on a small
    // persistent grid whose CTAs walk the chunks and skip those of contracts
    // whose date needs no second pass (all of them return at once when no
    // date does).
    const unsigned refine_grid = (k == 0 || chunk_count < kRefineGrid) ? chunk_count : kRefineGrid;
    // Condition bound below which a date is solved from its lagged sums: FP64
    // sums are good to ~1e-15, so 1e2 keeps the solve near FP64 accuracy; the
    // FP32 path's plain chunk sums are good to ~1e-8 relative once summed
    // over the chunks, and 1e3 keeps its coefficients inside the rounding the
    // FP32 basis values carry anyway.
    if (precision == 0) {
        if (k == 0)
            lsm_step<0, true><<<chunk_count, kLsmThreads, 0, stream>>>(
                k, c, chunk_contract, chunk_first, end, s_store, cf, reg, part, gpart, final_part, counters,
                group_counters, need, 1e2);
        else
            lsm_step<0, false><<<chunk_count, kLsmThreads, 0, stream>>>(
                k, c, chunk_contract, chunk_first, end, s_store, cf, reg, part, gpart, final_part, counters,
                group_counters, need, 1e2);
        lsm_refine<0><<<refine_grid, kLsmThreads, 0, stream>>>(k, c, chunk_contract, chunk_first, end, s_store, cf,
                                                               reg, part, gpart, counters, group_counters, need);
    } else {
        if (k == 0)
            lsm_step<1, true><<<chunk_count, kLsmThreads, 0, stream>>>(
                k, c, chunk_contract, chunk_first, end, s_store, cf, reg, part, gpart, final_part, counters,
                group_counters, need, 1e3);
        else
            lsm_step<1, false><<<chunk_count, kLsmThreads, 0, stream>>>(
                k, c, chunk_contract, chunk_first, end, s_store, cf, reg, part, gpart, final_part, counters,
                group_counters, need, 1e3);
        lsm_refine<1><<<refine_grid, kLsmThreads, 0, stream>>>(k, c, chunk_contract, chunk_first, end, s_store, cf,
                                                               reg, part, gpart, counters, group_counters, need);
    }
    return cudaGetLastError();
}

cudaError_t launch_lsm_finish(const LsmDev* c, int n_contracts, const Welford* final_part,
                              double* out, cudaStream_t stream) {
    cudaGetLastError();
    lsm_finish<<<(n_contracts * 32 + 127) / 128, 128, 0, stream>>>(c, n_contracts, final_part, out);
    return cudaGetLastError();
}

}  // namespace mcdg
