// device_common.cuh -- numerics shared by every kernel of the engine.
//
//  * Philox4x32-10 (Salmon et al. 2011) with the reference's counter layout
//    {path_lo, path_hi, draw, stream} and key {seed_lo, seed_hi}
//    (src/core/rng.cpp:9-13, :26-30, :41-57).  Only word 0 feeds a draw
//    (rng.cpp:64, :73), so the word-0 form lets the compiler drop the dead half
//    of the last round; the path-only half of round 0 is hoisted by callers.
//  * FP64 transform: (bits+0.5)/2^32 (rng.cpp:34-37), Acklam's rational inverse
//    CDF and one Halley step against erfc (src/core/normal.cpp:22-82).
//  * FP32 transform: the same u, formed as q = min(u, 1-u) from the bits (so the
//    tails keep full relative precision), mapped by this project's polynomial
//    fits in w = -ln(4q(1-q)) (Giles' change of variable for erfinv; the
//    coefficients come from csrc/fit_inverse_normal.py).
//  * Welford triples and the Chan-Golub-LeVeque merge
//    (include/mcd/core/stats.hpp:23-65).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "engine.hpp"

namespace mcdg {

constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

// Round keys of one seed, kept in registers for the life of a work item.
struct PhiloxKeys {
    uint32_t k0[10];
    uint32_t k1[10];
};

__device__ __forceinline__ PhiloxKeys philox_keys(uint64_t seed) {
    PhiloxKeys k;
    uint32_t a = static_cast<uint32_t>(seed), b = static_cast<uint32_t>(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        k.k0[r] = a;
        k.k1[r] = b;
        a += kPhiloxW0;
        b += kPhiloxW1;
    }
    return k;
}

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = static_cast<uint64_t>(kPhiloxM0) * c.x;
        const uint64_t p1 = static_cast<uint64_t>(kPhiloxM1) * c.z;
        c = make_uint4(static_cast<uint32_t>(p1 >> 32) ^ c.y ^ k0, static_cast<uint32_t>(p1),
                       static_cast<uint32_t>(p0 >> 32) ^ c.w ^ k1, static_cast<uint32_t>(p0));
        k0 += kPhiloxW0;
        k1 += kPhiloxW1;
    }
    return c;
}

// Path-constant part of round 0 (depends on path_lo and stream only).
struct PhiloxPath {
    uint32_t r0_w2;  // hi(M0*path_lo) ^ stream ^ k1[0]
    uint32_t r0_w3;  // lo(M0*path_lo)
    uint32_t path_hi;
};

__device__ __forceinline__ PhiloxPath philox_path(uint64_t path, uint32_t stream,
                                                  const PhiloxKeys& k) {
    const uint64_t p0 = static_cast<uint64_t>(kPhiloxM0) * static_cast<uint32_t>(path);
    PhiloxPath pp;
    pp.r0_w2 = static_cast<uint32_t>(p0 >> 32) ^ stream ^ k.k1[0];
    pp.r0_w3 = static_cast<uint32_t>(p0);
    pp.path_hi = static_cast<uint32_t>(path >> 32);
    return pp;
}

// Word 0 of philox4x32_10({path_lo, path_hi, draw, stream}, key).
__device__ __forceinline__ uint32_t philox_word0(const PhiloxPath& pp, uint32_t draw,
                                                 const PhiloxKeys& k) {
    // round 0 as one 32x32->64 product, rounds 1..9 as split halves: the mix
    // that measured fastest on the batch (the same bits either way)
    const uint64_t p1 = static_cast<uint64_t>(kPhiloxM1) * draw;
    uint32_t c0 = static_cast<uint32_t>(p1 >> 32) ^ pp.path_hi ^ k.k0[0];
    uint32_t c1 = static_cast<uint32_t>(p1);
    uint32_t c2 = pp.r0_w2;
    uint32_t c3 = pp.r0_w3;
#pragma unroll
    for (int r = 1; r < 10; ++r) {
        // high and low halves as separate 32-bit multiplies (the same bits
        // as one 32x32->64 product)
        const uint32_t n0 = __umulhi(kPhiloxM1, c2) ^ c1 ^ k.k0[r];
        const uint32_t n1 = kPhiloxM1 * c2;
        const uint32_t n2 = __umulhi(kPhiloxM0, c0) ^ c3 ^ k.k1[r];
        const uint32_t n3 = kPhiloxM0 * c0;
        c0 = n0;
        c1 = n1;
        c2 = n2;
        c3 = n3;
    }
    return c0;
}

// ---------------------------------------------------------------------------
// FP64 transform (src/core/rng.cpp:34-37, src/core/normal.cpp:22-82)
//
// Translation units including this header are compiled with --fmad=false:
// every fused multiply-add is written out (fma / __fmaf_rn), everything else
// rounds as written, like the reference's -ffp-contract=off build.  That
// fixes the arithmetic independently of register allocation, so every kernel
// variant computes the same bits.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double uniform_open01_f64(uint32_t bits) {
    return (static_cast<double>(bits) + 0.5) * (1.0 / 4294967296.0);
}

__device__ __forceinline__ double normal_cdf_f64(double x) {
    return 0.5 * erfc(-x / 1.41421356237309504880);
}

__device__ __forceinline__ double inv_normal_cdf_f64(double u) {
    const double low = 0.02425;
    const double high = 1.0 - low;
    double z;
    if (u < low || high < u) {
        const bool lower = u < low;
        const double q = sqrt(-2.0 * log(lower ? u : 1.0 - u));
        double num = fma(-7.784894002430293e-03, q, -3.223964580411365e-01);
        num = fma(num, q, -2.400758277161838e+00);
        num = fma(num, q, -2.549732539343734e+00);
        num = fma(num, q, 4.374664141464968e+00);
        num = fma(num, q, 2.938163982698783e+00);
        double den = fma(7.784695709041462e-03, q, 3.224671290700398e-01);
        den = fma(den, q, 2.445134137142996e+00);
        den = fma(den, q, 3.754408661907416e+00);
        den = fma(den, q, 1.0);
        const double r = num / den;
        z = lower ? r : -r;
    } else {
        const double t = u - 0.5;
        const double r = t * t;
        double num = fma(-3.969683028665376e+01, r, 2.209460984245205e+02);
        num = fma(num, r, -2.759285104469687e+02);
        num = fma(num, r, 1.383577518672690e+02);
        num = fma(num, r, -3.066479806614716e+01);
        num = fma(num, r, 2.506628277459239e+00) * t;
        double den = fma(-5.447609879822406e+01, r, 1.615858368580409e+02);
        den = fma(den, r, -1.556989798598866e+02);
        den = fma(den, r, 6.680131188771972e+01);
        den = fma(den, r, -1.328068155288572e+01);
        den = fma(den, r, 1.0);
        z = num / den;
    }
    const double error = normal_cdf_f64(z) - u;
    const double sqrt_2pi = 2.50662827463100050242;  // sqrt(2*pi)
    const double r = error * sqrt_2pi * exp(0.5 * z * z);
    z -= r / (1.0 + 0.5 * z * r);
    return z;
}

__device__ __forceinline__ double normal_from_bits_f64(uint32_t bits) {
    return inv_normal_cdf_f64(uniform_open01_f64(bits));
}

// ---------------------------------------------------------------------------
// FP32 transform
// ---------------------------------------------------------------------------
__device__ __forceinline__ float fast_sqrt(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float fast_rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Standard normal of the reference's u = (bits+0.5)/2^32, in FP32.
//
// q = min(u, 1-u) is formed from the bits (for bits >= 2^31 the mirror
// 1-u = (~bits + 0.5)/2^32), so the tails keep full relative precision.
// With x = 1 - 2q and w = -ln(4 q (1 - q)) = -ln(1 - x^2), Phi^-1(1 - q) =
// x P(w) for a P that is smooth in w (M. Giles' change of variable for erfinv,
// "Approximating the erfinv function", GPU Computing Gems Jade, 2011).  P is a
// polynomial of degree 8 in w - 2.5 for w < 5 (q > 0.0017, 99.66 % of the
// draws) and of degree 9 in sqrt(w) - 3 above (32-bit inputs give q >= 2^-33,
// so w <= 21.5); the coefficients are this project's own least-squares fits to
// the double-precision quantile (csrc/fit_inverse_normal.py), with relative fit
// errors of 9.4e-8 and 1.2e-7.  One MUFU log2, eight or nine FMAs and the
// product: about half the instructions of a rational with per-lane branch
// selects, which every warp would pay for both branches.  Only warps holding a
// tail draw (about one in ten) also run the second polynomial.
__device__ __forceinline__ float inv_normal_upper(float q) {  // Phi^-1(1 - q) >= 0, q in (0, 1/2]
    const float y = __fmaf_rn(-q, q, q);                                   // q (1 - q)
    const float w = __fmaf_rn(__log2f(y), -0.693147181f, -1.386294361f);   // -ln(4 y)
    const float x = __fmaf_rn(-2.0f, q, 1.0f);                             // 1 - 2q
    float p;
    if (w < 5.0f) {
        const float t = w - 2.5f;
        p = 4.035420447e-08f;
        p = __fmaf_rn(p, t, 4.861469141e-07f);
        p = __fmaf_rn(p, t, -4.990533717e-06f);
        p = __fmaf_rn(p, t, -6.218398536e-06f);
        p = __fmaf_rn(p, t, 3.091499728e-04f);
        p = __fmaf_rn(p, t, -1.773009095e-03f);
        p = __fmaf_rn(p, t, -5.908170540e-03f);
        p = __fmaf_rn(p, t, 3.488026592e-01f);
        p = __fmaf_rn(p, t, 2.123313567e+00f);
    } else {
        const float t = fast_sqrt(w) - 3.0f;
        p = 5.067717386e-05f;
        p = __fmaf_rn(p, t, -2.118356777e-04f);
        p = __fmaf_rn(p, t, -3.360669450e-05f);
        p = __fmaf_rn(p, t, 1.810359006e-03f);
        p = __fmaf_rn(p, t, -5.043195909e-03f);
        p = __fmaf_rn(p, t, 8.166690883e-03f);
        p = __fmaf_rn(p, t, -1.082257433e-02f);
        p = __fmaf_rn(p, t, 1.333906298e-02f);
        p = __fmaf_rn(p, t, 1.416583983e+00f);
        p = __fmaf_rn(p, t, 4.006434684e+00f);
    }
    return p * x;
}

__device__ __forceinline__ float normal_from_bits_f32(uint32_t bits) {
    const bool upper = (bits >> 31) != 0u;
    const uint32_t m = upper ? ~bits : bits;
    const float q = __fmaf_rn(__uint2float_rn(m), 2.3283064365386963e-10f, 1.1641532182693481e-10f);
    const float z = inv_normal_upper(q);
    return upper ? z : -z;
}

// Standard normal of a Sobol coordinate u = x / 2^32 (x > 0), in FP32: the
// mirror 1 - u = (2^32 - x) / 2^32 is formed exactly from the bits.
__device__ __forceinline__ float normal_from_sobol_f32(uint32_t x) {
    const bool upper = x > 0x80000000u;
    const uint32_t m = upper ? (0u - x) : x;
    const float z = inv_normal_upper(__uint2float_rn(m) * 2.3283064365386963e-10f);
    return upper ? z : -z;
}

// Uniform (bits+0.5)/2^32 in FP32 (for comparisons against probabilities).
__device__ __forceinline__ float uniform_from_bits_f32(uint32_t bits) {
    return __fmaf_rn(__uint2float_rn(bits), 2.3283064365386963e-10f, 1.1641532182693481e-10f);
}

// ---------------------------------------------------------------------------
// Welford triples (include/mcd/core/stats.hpp:23-65)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void welford_add(Welford& w, double value) {
    ++w.count;
    const double delta = value - w.mean;
    w.mean += delta / static_cast<double>(w.count);
    const double delta2 = value - w.mean;
    w.m2 += delta * delta2;
}

__host__ __device__ __forceinline__ Welford welford_merge(const Welford& a, const Welford& b) {
    if (b.count == 0) return a;
    if (a.count == 0) return b;
    const unsigned long long n = a.count + b.count;
    const double delta = b.mean - a.mean;
    const double w = static_cast<double>(b.count) / static_cast<double>(n);
    Welford r;
    r.count = n;
    r.mean = a.mean + delta * w;
    r.m2 = a.m2 + b.m2 +
           delta * delta * static_cast<double>(a.count) * static_cast<double>(b.count) /
               static_cast<double>(n);
    return r;
}

__device__ __forceinline__ Welford welford_shfl_down(const Welford& w, int offset) {
    Welford o;
    o.count = __shfl_down_sync(0xffffffffu, w.count, offset);
    o.mean = __shfl_down_sync(0xffffffffu, w.mean, offset);
    o.m2 = __shfl_down_sync(0xffffffffu, w.m2, offset);
    return o;
}

// Fixed-shape warp tree: lane i merges lane i+off (off = 16, 8, 4, 2, 1); the
// result is valid in lane 0.  Deterministic because lane positions are fixed.
__device__ __forceinline__ Welford welford_warp_reduce(Welford w) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const Welford o = welford_shfl_down(w, off);
        w = welford_merge(w, o);
    }
    return w;
}

// (count, sum, sum of squares) -> Welford triple for one thread's samples.
__device__ __forceinline__ Welford welford_from_sums(unsigned count, double s1, double s2) {
    Welford w;
    w.count = count;
    if (count == 0) {
        w.mean = 0.0;
        w.m2 = 0.0;
        return w;
    }
    w.mean = s1 / static_cast<double>(count);
    const double m2 = s2 - s1 * w.mean;
    w.m2 = m2 > 0.0 ? m2 : 0.0;
    return w;
}

// Payoff sums of the FP32 Longstaff-Schwartz kernels, whose threads price
// only a few cash flows each: compensated FP32 sums (Knuth's TwoSum; hi + lo
// carries ~2^-44 relative) of the values and of their squares (each square's
// rounding error recovered exactly by an FMA), added up per thread and over
// the warp tree in FP32, converted to FP64 once per warp and folded in FP64
// above that.  Converting, adding or Welford-merging every cash flow in FP64
// would occupy the FP64 pipe, a small fraction of the FP32 rate on this GPU.
// Needs --fmad=false (TwoSum must not be contracted).
struct Sum32 {
    unsigned n;
    float hi, lo, qhi, qlo;
};
struct Sum64 {
    unsigned n;
    double s1, s2;
};

__device__ __forceinline__ void two_sum_add(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float bp = s - hi;
    lo += (hi - (s - bp)) + (x - bp);
    hi = s;
}

__device__ __forceinline__ void sum32_add(Sum32& a, float v) {
    ++a.n;
    two_sum_add(a.hi, a.lo, v);
    const float p = v * v;
    two_sum_add(a.qhi, a.qlo, p);
    a.qlo += __fmaf_rn(v, v, -p);
}

__device__ __forceinline__ Sum32 sum32_warp_reduce(Sum32 a) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const unsigned n = __shfl_down_sync(0xffffffffu, a.n, off);
        const float hi = __shfl_down_sync(0xffffffffu, a.hi, off);
        const float lo = __shfl_down_sync(0xffffffffu, a.lo, off);
        const float qhi = __shfl_down_sync(0xffffffffu, a.qhi, off);
        const float qlo = __shfl_down_sync(0xffffffffu, a.qlo, off);
        a.n += n;
        two_sum_add(a.hi, a.lo, hi);
        a.lo += lo;
        two_sum_add(a.qhi, a.qlo, qhi);
        a.qlo += qlo;
    }
    return a;
}

__device__ __forceinline__ Sum64 sum32_wide(const Sum32& a) {
    return Sum64{a.n, static_cast<double>(a.hi) + static_cast<double>(a.lo),
                 static_cast<double>(a.qhi) + static_cast<double>(a.qlo)};
}

// Warp sums folded in warp order (one thread), as a Welford triple.
template <int W>
__device__ __forceinline__ Welford sum64_fold(const Sum64* s) {
    unsigned n = 0;
    double s1 = 0.0, s2 = 0.0;
    for (int w = 0; w < W; ++w) {
        n += s[w].n;
        s1 += s[w].s1;
        s2 += s[w].s2;
    }
    return welford_from_sums(n, s1, s2);
}

}  // namespace mcdg
