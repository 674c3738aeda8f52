/*
 * mcd_oracle.c -- CPU oracle for the mcd Monte Carlo hot path (test
 * infrastructure only; see mcd_oracle.h).  Compiled with -std=c11
 * -ffp-contract=off so every floating-point expression rounds exactly as the
 * reference's ISO C++20 build does (CMakeLists.txt:9-11, :60-62).
 *
 * Every function names the reference file:line it restates.  Expression order
 * is kept where it decides the rounding (that is what makes the restatement
 * bit-identical to the reference built from source).
 */
#define _GNU_SOURCE
#include "mcd_oracle.h"

#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define PI_D 3.14159265358979323846
#define SQRT2_D 1.41421356237309504880
#define SQRT3_D 1.73205080756887729353
#define INV_SQRTPI_D 0.56418958354775628695

/* std::max / std::min semantics (return the first argument on ties). */
static inline double maxd(double a, double b) { return (a < b) ? b : a; }
static inline double mind(double a, double b) { return (b < a) ? b : a; }
static inline double sgn(int type) { return type == 0 ? 1.0 : -1.0; }

/* ------------------------------------------------------------------------ */
/* Philox4x32-10: src/core/rng.cpp:9-13 (constants), :26-30 (round),        */
/* :32 (key bump), :41-47 (10 rounds).                                      */
/* ------------------------------------------------------------------------ */
void orc_philox4x32_10(const uint32_t counter[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = counter[0], c1 = counter[1], c2 = counter[2], c3 = counter[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 0; round < 10; ++round) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n1 = (uint32_t)p1;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        const uint32_t n3 = (uint32_t)p0;
        c0 = n0;
        c1 = n1;
        c2 = n2;
        c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* src/core/rng.cpp:34-37 */
double orc_uniform_open01(uint32_t bits) { return ((double)bits + 0.5) / 4294967296.0; }

/* ---- normal.cpp: pdf :8-11, cdf :13-15, Acklam :22-66, Halley :70-82 ---- */
double orc_normal_pdf(double x) {
    const double inv_sqrt_2pi = INV_SQRTPI_D / SQRT2_D;
    return inv_sqrt_2pi * exp(-0.5 * x * x);
}

double orc_normal_cdf(double x) { return 0.5 * erfc(-x / SQRT2_D); }

static const double kA1 = -3.969683028665376e+01, kA2 = 2.209460984245205e+02,
                    kA3 = -2.759285104469687e+02, kA4 = 1.383577518672690e+02,
                    kA5 = -3.066479806614716e+01, kA6 = 2.506628277459239e+00;
static const double kB1 = -5.447609879822406e+01, kB2 = 1.615858368580409e+02,
                    kB3 = -1.556989798598866e+02, kB4 = 6.680131188771972e+01,
                    kB5 = -1.328068155288572e+01;
static const double kC1 = -7.784894002430293e-03, kC2 = -3.223964580411365e-01,
                    kC3 = -2.400758277161838e+00, kC4 = -2.549732539343734e+00,
                    kC5 = 4.374664141464968e+00, kC6 = 2.938163982698783e+00;
static const double kD1 = 7.784695709041462e-03, kD2 = 3.224671290700398e-01,
                    kD3 = 2.445134137142996e+00, kD4 = 3.754408661907416e+00;

double orc_inv_normal_cdf(double u) {
    const double low = 0.02425;
    const double high = 1.0 - low;
    double z;
    if (u < low || high < u) {
        const int lower = u < low;
        const double q = sqrt(-2.0 * log(lower ? u : 1.0 - u));
        const double num = (((((kC1 * q + kC2) * q + kC3) * q + kC4) * q + kC5) * q + kC6);
        const double den = ((((kD1 * q + kD2) * q + kD3) * q + kD4) * q + 1.0);
        const double r = num / den;
        z = lower ? r : -r;
    } else {
        const double t = u - 0.5;
        const double r = t * t;
        const double num = (((((kA1 * r + kA2) * r + kA3) * r + kA4) * r + kA5) * r + kA6) * t;
        const double den = (((((kB1 * r + kB2) * r + kB3) * r + kB4) * r + kB5) * r + 1.0);
        z = num / den;
    }
    const double error = orc_normal_cdf(z) - u;
    const double sqrt_2pi = sqrt(2.0 * PI_D);
    const double r = error * sqrt_2pi * exp(0.5 * z * z);
    z -= r / (1.0 + 0.5 * z * r);
    return z;
}

/* src/core/rng.cpp:59-66 (stream 0) and :68-74 (stream 1); counter layout
 * {path_lo, path_hi, draw, stream}, key {seed_lo, seed_hi} (:49-57). */
double orc_normal_variate(uint64_t seed, uint64_t path, uint32_t draw) {
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    const uint32_t ctr[4] = {(uint32_t)path, (uint32_t)(path >> 32), draw, 0u};
    uint32_t out[4];
    orc_philox4x32_10(ctr, key, out);
    return orc_inv_normal_cdf(orc_uniform_open01(out[0]));
}

double orc_uniform_variate(uint64_t seed, uint64_t path, uint32_t draw) {
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    const uint32_t ctr[4] = {(uint32_t)path, (uint32_t)(path >> 32), draw, 1u};
    uint32_t out[4];
    orc_philox4x32_10(ctr, key, out);
    return orc_uniform_open01(out[0]);
}

/* ---- Welford: include/mcd/core/stats.hpp:23-65 ------------------------- */
void orc_welford_add(orc_welford* w, double value) {
    ++w->count;
    const double delta = value - w->mean;
    w->mean += delta / (double)w->count;
    const double delta2 = value - w->mean;
    w->m2 += delta * delta2;
}

void orc_welford_merge(orc_welford* w, const orc_welford* o) {
    if (o->count == 0) return;
    if (w->count == 0) {
        *w = *o;
        return;
    }
    const uint64_t n = w->count + o->count;
    const double delta = o->mean - w->mean;
    const double other_weight = (double)o->count / (double)n;
    const double new_mean = w->mean + delta * other_weight;
    const double new_m2 =
        w->m2 + o->m2 + delta * delta * (double)w->count * (double)o->count / (double)n;
    w->count = n;
    w->mean = new_mean;
    w->m2 = new_m2;
}

double orc_welford_variance(const orc_welford* w) {
    return w->count < 2 ? 0.0 : w->m2 / (double)(w->count - 1);
}

double orc_welford_se(const orc_welford* w) {
    return w->count == 0 ? 0.0 : sqrt(orc_welford_variance(w) / (double)w->count);
}

/* src/core/thread_pool.cpp:9-18 */
void orc_chunk_bounds(unsigned chunk, uint64_t total, unsigned chunk_count, uint64_t* begin,
                      uint64_t* end) {
    const uint64_t base = total / chunk_count;
    const uint64_t rem = total % chunk_count;
    const uint64_t b = (uint64_t)chunk * base + ((uint64_t)chunk < rem ? (uint64_t)chunk : rem);
    *begin = b;
    *end = b + base + ((uint64_t)chunk < rem ? 1u : 0u);
}

/* src/core/thread_pool.cpp:41-44 */
unsigned orc_default_chunk_count(void) {
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (unsigned)n : 1u;
}

/* ---- a fixed-item parallel loop over pthreads (host baseline only) ------ */
typedef void (*orc_item_fn)(void* ctx, unsigned item);
typedef struct {
    orc_item_fn fn;
    void* ctx;
    unsigned n_items;
    atomic_uint next;
} orc_pool_job;

static void* orc_pool_worker(void* arg) {
    orc_pool_job* job = (orc_pool_job*)arg;
    unsigned item;
    while ((item = atomic_fetch_add(&job->next, 1u)) < job->n_items) job->fn(job->ctx, item);
    return NULL;
}

static void orc_parallel_for(unsigned n_items, unsigned num_threads, orc_item_fn fn, void* ctx) {
    if (num_threads <= 1 || n_items <= 1) {
        for (unsigned i = 0; i < n_items; ++i) fn(ctx, i);
        return;
    }
    if (num_threads > n_items) num_threads = n_items;
    orc_pool_job job;
    job.fn = fn;
    job.ctx = ctx;
    job.n_items = n_items;
    atomic_init(&job.next, 0u);
    pthread_t* threads = (pthread_t*)malloc(sizeof(pthread_t) * num_threads);
    unsigned started = 0;
    for (unsigned t = 1; t < num_threads; ++t)
        if (pthread_create(&threads[started], NULL, orc_pool_worker, &job) == 0) ++started;
    orc_pool_worker(&job);
    for (unsigned t = 0; t < started; ++t) pthread_join(threads[t], NULL);
    free(threads);
}

/* ------------------------------------------------------------------------ */
/* GBM exact step: src/models/gbm.cpp:7-12                                  */
/* ------------------------------------------------------------------------ */
static inline double gbm_terminal_spot(double spot, double rate, double q, double vol, double time,
                                       double z) {
    const double drift = (rate - q - 0.5 * vol * vol) * time;
    const double diffusion = vol * sqrt(time) * z;
    return spot * exp(drift + diffusion);
}

/* ---- product description used by the generic engine ---------------------- */
enum { P_EUROPEAN = 0, P_DIGITAL = 1, P_ASIAN = 2, P_BARRIER = 3, P_LOOKBACK = 4,
       P_ASIAN_CV = 5, P_BARRIER_BB = 6 };

typedef struct {
    int product, type, direction, knock, strike_style, average_style, digital_style, n;
    double spot, strike, barrier, rebate, rate, q, vol, time, cash;
    double dt, discount, log_barrier, kv_anchor;
    uint64_t seed;
} orc_product;

/* include/mcd/payoffs/european.hpp:19-22 and digital.hpp:16-23 */
static inline double terminal_payoff(const orc_product* p, double s) {
    const double phi = sgn(p->type);
    if (p->product == P_EUROPEAN) return maxd(phi * (s - p->strike), 0.0);
    const int itm = phi * (s - p->strike) > 0.0;
    if (!itm) return 0.0;
    return p->digital_style == 0 ? p->cash : s;
}

/* monte_carlo.cpp:135-149 (terminal), :154-177 (path dependent),
 * :184-230 (Brownian-bridge barrier), :275-302 (control-variate Asian). */
static double run_one_path(const orc_product* p, uint64_t path, int negate) {
    if (p->product == P_EUROPEAN || p->product == P_DIGITAL) {
        const double z = orc_normal_variate(p->seed, path, 0);
        return p->discount *
               terminal_payoff(p, gbm_terminal_spot(p->spot, p->rate, p->q, p->vol, p->time,
                                                    negate ? -z : z));
    }
    if (p->product == P_BARRIER_BB) {
        double s = p->spot;
        int breached = 0;
        for (int step = 0; step < p->n; ++step) {
            const uint32_t st = (uint32_t)step;
            const double z = orc_normal_variate(p->seed, path, st);
            const double s_next = gbm_terminal_spot(s, p->rate, p->q, p->vol, p->dt, negate ? -z : z);
            const int crossed = p->direction == 0 ? s_next >= p->barrier : s_next <= p->barrier;
            breached = breached || crossed;
            if (!breached) {
                const double log_s = log(s);
                const double log_s_next = log(s_next);
                const double p_cross = exp(-2.0 * (p->log_barrier - log_s) *
                                           (p->log_barrier - log_s_next) / (p->vol * p->vol * p->dt));
                const double u = orc_uniform_variate(p->seed, path, st);
                breached = u < p_cross;
            }
            s = s_next;
        }
        const double phi = sgn(p->type);
        const double vanilla = maxd(phi * (s - p->strike), 0.0);
        const int pays_vanilla = p->knock == 1 ? !breached : breached;
        return p->discount * (pays_vanilla ? vanilla : p->rebate);
    }
    /* path-dependent payoffs: asian.hpp:14-65, barrier.hpp:14-38,
     * lookback.hpp:13-57 (extremum seeded with S0). */
    double s = p->spot;
    double sum = 0.0, log_sum = 0.0, last = 0.0;
    unsigned count = 0;
    int breached = 0;
    double rmax = p->spot, rmin = p->spot;
    if (p->product == P_LOOKBACK && p->strike_style == 1) last = p->spot;
    for (int step = 0; step < p->n; ++step) {
        const double z = orc_normal_variate(p->seed, path, (uint32_t)step);
        s = gbm_terminal_spot(s, p->rate, p->q, p->vol, p->dt, negate ? -z : z);
        switch (p->product) {
        case P_ASIAN:
            if (p->average_style == 0) sum += s; else log_sum += log(s);
            last = s;
            ++count;
            break;
        case P_ASIAN_CV:
            sum += s;
            log_sum += log(s);
            last = s;
            ++count;
            break;
        case P_BARRIER: {
            const int crossed = p->direction == 0 ? s >= p->barrier : s <= p->barrier;
            breached = breached || crossed;
            last = s;
            break;
        }
        default: /* lookback */
            rmax = maxd(rmax, s);
            rmin = mind(rmin, s);
            last = s;
            break;
        }
    }
    const double phi = sgn(p->type);
    switch (p->product) {
    case P_ASIAN: {
        const double average =
            p->average_style == 0 ? sum / (double)count : exp(log_sum / (double)count);
        const double ref = p->strike_style == 0 ? (average - p->strike) : (last - average);
        return p->discount * maxd(phi * ref, 0.0);
    }
    case P_ASIAN_CV: {
        const double a_avg = sum / (double)count;
        const double a_ref = p->strike_style == 0 ? (a_avg - p->strike) : (last - a_avg);
        const double g_avg = exp(log_sum / (double)count);
        const double g_ref = p->strike_style == 0 ? (g_avg - p->strike) : (last - g_avg);
        const double arithmetic_payoff = p->discount * maxd(phi * a_ref, 0.0);
        const double geometric_payoff = p->discount * maxd(phi * g_ref, 0.0);
        return arithmetic_payoff - (geometric_payoff - p->kv_anchor);
    }
    case P_BARRIER: {
        const double vanilla = maxd(phi * (last - p->strike), 0.0);
        const int pays_vanilla = p->knock == 1 ? !breached : breached;
        return p->discount * (pays_vanilla ? vanilla : p->rebate);
    }
    default:
        if (p->strike_style == 0)
            return p->discount * (p->type == 0 ? maxd(rmax - p->strike, 0.0)
                                               : maxd(p->strike - rmin, 0.0));
        return p->discount * (p->type == 0 ? (last - rmin) : (rmax - last));
    }
}

/* accumulate_paths + run_chunked_and_merge: monte_carlo.cpp:42-92 */
typedef struct {
    const orc_product* p;
    int antithetic;
    uint64_t path_count;
    unsigned chunk_count;
    orc_welford* per_chunk;
} orc_chunk_job;

static void orc_chunk_task(void* ctx, unsigned chunk) {
    orc_chunk_job* job = (orc_chunk_job*)ctx;
    uint64_t begin, end;
    orc_chunk_bounds(chunk, job->path_count, job->chunk_count, &begin, &end);
    orc_welford local = {0, 0.0, 0.0};
    for (uint64_t i = begin; i < end; ++i) {
        double sample = run_one_path(job->p, i, 0);
        if (job->antithetic) {
            const double sample2 = run_one_path(job->p, i, 1);
            sample = 0.5 * (sample + sample2);
        }
        orc_welford_add(&local, sample);
    }
    job->per_chunk[chunk] = local;
}

static orc_mc_result orc_run_product(const orc_product* p, uint64_t path_count,
                                     const orc_options* options) {
    orc_options def = {0, 0, 0, 1, 0};
    if (!options) options = &def;
    const unsigned chunks = options->chunk_count ? options->chunk_count : orc_default_chunk_count();
    orc_chunk_job job;
    job.p = p;
    job.antithetic = options->antithetic;
    job.path_count = path_count;
    job.chunk_count = chunks;
    job.per_chunk = (orc_welford*)calloc(chunks, sizeof(orc_welford));
    orc_parallel_for(chunks, options->num_threads, orc_chunk_task, &job);
    orc_welford merged = {0, 0.0, 0.0};
    for (unsigned i = 0; i < chunks; ++i) orc_welford_merge(&merged, &job.per_chunk[i]);
    free(job.per_chunk);
    orc_mc_result r;
    r.price = merged.mean;
    r.standard_error = orc_welford_se(&merged);
    r.path_count = merged.count;
    return r;
}

static void product_init(orc_product* p, double spot, double strike, double rate, double q,
                         double vol, double time, int type, uint64_t seed) {
    memset(p, 0, sizeof(*p));
    p->spot = spot;
    p->strike = strike;
    p->rate = rate;
    p->q = q;
    p->vol = vol;
    p->time = time;
    p->type = type;
    p->seed = seed;
    p->discount = exp(-rate * time);
}

orc_mc_result orc_mc_european(double spot, double strike, double rate, double carry_yield,
                              double vol, double time, int type, uint64_t path_count,
                              uint64_t seed, const orc_options* options) {
    orc_product p;
    product_init(&p, spot, strike, rate, carry_yield, vol, time, type, seed);
    p.product = P_EUROPEAN;
    return orc_run_product(&p, path_count, options);
}

orc_mc_result orc_mc_digital(double spot, double strike, double rate, double carry_yield,
                             double vol, double time, int type, int digital_style,
                             double cash_amount, uint64_t path_count, uint64_t seed,
                             const orc_options* options) {
    orc_product p;
    product_init(&p, spot, strike, rate, carry_yield, vol, time, type, seed);
    p.product = P_DIGITAL;
    p.digital_style = digital_style;
    p.cash = cash_amount;
    return orc_run_product(&p, path_count, options);
}

orc_mc_result orc_mc_asian(double spot, double strike, double rate, double carry_yield,
                           double vol, double time, int type, int strike_style,
                           int average_style, int monitoring_points, uint64_t path_count,
                           uint64_t seed, const orc_options* options) {
    orc_product p;
    product_init(&p, spot, strike, rate, carry_yield, vol, time, type, seed);
    p.product = P_ASIAN;
    p.strike_style = strike_style;
    p.average_style = average_style;
    p.n = monitoring_points;
    p.dt = time / (double)monitoring_points;
    /* monte_carlo.cpp:276: the control variate applies only to fixed-strike
     * arithmetic Asians, anchored at kemna_vorst (analytic.cpp:51-59). */
    if (average_style == 0 && options && options->control_variate && strike_style == 0) {
        p.product = P_ASIAN_CV;
        p.kv_anchor = orc_kemna_vorst(spot, strike, rate, carry_yield, vol, time, type);
    }
    return orc_run_product(&p, path_count, options);
}

orc_mc_result orc_mc_barrier(double spot, double strike, double barrier, double rate,
                             double carry_yield, double vol, double time, int type,
                             int direction, int knock, double rebate, int monitoring_points,
                             uint64_t path_count, uint64_t seed, const orc_options* options) {
    orc_product p;
    product_init(&p, spot, strike, rate, carry_yield, vol, time, type, seed);
    p.product = (options && options->brownian_bridge) ? P_BARRIER_BB : P_BARRIER;
    p.barrier = barrier;
    p.rebate = rebate;
    p.direction = direction;
    p.knock = knock;
    p.n = monitoring_points;
    p.dt = time / (double)monitoring_points;
    p.log_barrier = log(barrier);
    return orc_run_product(&p, path_count, options);
}

orc_mc_result orc_mc_lookback(double spot, double strike, double rate, double carry_yield,
                              double vol, double time, int type, int strike_style,
                              int monitoring_points, uint64_t path_count, uint64_t seed,
                              const orc_options* options) {
    orc_product p;
    product_init(&p, spot, strike, rate, carry_yield, vol, time, type, seed);
    p.product = P_LOOKBACK;
    p.strike_style = strike_style;
    p.n = monitoring_points;
    p.dt = time / (double)monitoring_points;
    return orc_run_product(&p, path_count, options);
}

/* ------------------------------------------------------------------------ */
/* Sobol: src/core/sobol.cpp:22-30 (polynomials), :40-68 (Bratley-Fox       */
/* direction numbers, m_i = 1), :83-97 (Gray-code point).  Dimensions 0..6  */
/* are the reference's table; dimensions 7.. continue with every further    */
/* primitive polynomial in ascending (degree, interior mask) order, using   */
/* the same m_i = 1 initialisation (the reference caps at 7, sobol.hpp:14). */
/* ------------------------------------------------------------------------ */
static const unsigned kRefDeg[7] = {0, 1, 2, 3, 4, 5, 6};
static const uint32_t kRefMask[7] = {0u, 0u, 1u, 1u, 1u, 2u, 1u};

/* x has order 2^s - 1 modulo p(x) = x^s + a_1 x^{s-1} + ... + a_{s-1} x + 1. */
static int is_primitive(unsigned s, uint32_t interior) {
    uint32_t poly = (1u << s) | 1u; /* bit k = coefficient of x^k */
    for (unsigned j = 1; j < s; ++j)
        if ((interior >> (j - 1)) & 1u) poly |= 1u << (s - j);
    const uint32_t period = (1u << s) - 1u;
    uint32_t r = 1u; /* x^0 */
    for (uint32_t k = 1; k <= period; ++k) {
        r <<= 1;
        if (r & (1u << s)) r ^= poly;
        if (r == 1u) return k == period;
    }
    return 0;
}

static unsigned g_poly_deg[ORC_SOBOL_MAX_DIMS];
static uint32_t g_poly_mask[ORC_SOBOL_MAX_DIMS];
static pthread_once_t g_poly_once = PTHREAD_ONCE_INIT;

static void build_polynomials(void) {
    unsigned d = 0;
    for (; d < 7; ++d) {
        g_poly_deg[d] = kRefDeg[d];
        g_poly_mask[d] = kRefMask[d];
    }
    for (unsigned s = 1; d < ORC_SOBOL_MAX_DIMS && s < 20; ++s) {
        for (uint32_t m = 0; d < ORC_SOBOL_MAX_DIMS && m < (s > 1 ? (1u << (s - 1)) : 1u); ++m) {
            int used = 0;
            for (unsigned k = 1; k < 7; ++k)
                if (kRefDeg[k] == s && kRefMask[k] == m) used = 1;
            if (used || !is_primitive(s, m)) continue;
            g_poly_deg[d] = s;
            g_poly_mask[d] = m;
            ++d;
        }
    }
}

int orc_sobol_polynomial(unsigned dimension, unsigned* degree, uint32_t* interior) {
    if (dimension >= ORC_SOBOL_MAX_DIMS) return -1;
    pthread_once(&g_poly_once, build_polynomials);
    *degree = g_poly_deg[dimension];
    *interior = g_poly_mask[dimension];
    return 0;
}

void orc_sobol_directions(unsigned dimension, uint32_t v[33]) {
    unsigned s;
    uint32_t mask;
    uint32_t m[33];
    memset(m, 0, sizeof(m));
    memset(v, 0, sizeof(uint32_t) * 33);
    if (orc_sobol_polynomial(dimension, &s, &mask) != 0) return;
    if (s == 0) {
        for (unsigned k = 1; k <= 32; ++k) m[k] = 1;
    } else {
        for (unsigned k = 1; k <= s && k <= 32; ++k) m[k] = 1;
        for (unsigned k = s + 1; k <= 32; ++k) {
            uint32_t mk = m[k - s] ^ (m[k - s] << s);
            for (unsigned j = 1; j < s; ++j)
                if ((mask >> (j - 1)) & 1u) mk ^= (m[k - j] << j);
            m[k] = mk;
        }
    }
    for (unsigned k = 1; k <= 32; ++k) v[k] = m[k] << (32 - k);
}

uint32_t orc_sobol_bits(unsigned dimension, uint64_t index) {
    uint32_t v[33];
    orc_sobol_directions(dimension, v);
    const uint64_t gray = index ^ (index >> 1);
    uint32_t x = 0;
    for (unsigned b = 0; b < 32; ++b)
        if ((gray >> b) & 1u) x ^= v[b + 1];
    return x;
}

double orc_sobol_point(unsigned dimension, uint64_t index) {
    if (index == 0) return 0.0;
    return (double)orc_sobol_bits(dimension, index) / (double)((uint64_t)1 << 32);
}

/* src/models/brownian_bridge_path.cpp:20-77 (BFS bisection; normals[0] is the
 * terminal point). */
void orc_brownian_bridge_gbm_path(double spot, double rate, double carry_yield, double vol,
                                  double time, int n, const double* normals, double* spots) {
    double* t = (double*)malloc(sizeof(double) * (size_t)(n + 1));
    double* w = (double*)calloc((size_t)n, sizeof(double));
    for (int i = 0; i <= n; ++i) t[i] = (double)i * time / (double)n;
    w[n - 1] = sqrt(t[n]) * normals[0];
    if (n > 1) {
        int* ql = (int*)malloc(sizeof(int) * (size_t)(2 * n + 1));
        int* qr = (int*)malloc(sizeof(int) * (size_t)(2 * n + 1));
        size_t head = 0, tail = 0;
        ql[tail] = -1;
        qr[tail] = n - 1;
        ++tail;
        int draw = 1;
        while (head < tail && draw < n) {
            const int left = ql[head], right = qr[head];
            ++head;
            if (right - left <= 1) continue;
            const int mid = (left + right) / 2;
            const double t_left = left == -1 ? 0.0 : t[left + 1];
            const double w_left = left == -1 ? 0.0 : w[left];
            const double t_right = t[right + 1];
            const double w_right = w[right];
            const double t_mid = t[mid + 1];
            const double mean = w_left + (t_mid - t_left) / (t_right - t_left) * (w_right - w_left);
            const double variance = (t_mid - t_left) * (t_right - t_mid) / (t_right - t_left);
            w[mid] = mean + sqrt(variance) * normals[draw];
            ++draw;
            ql[tail] = left;
            qr[tail] = mid;
            ++tail;
            ql[tail] = mid;
            qr[tail] = right;
            ++tail;
        }
        free(ql);
        free(qr);
    }
    const double drift_rate = rate - carry_yield - 0.5 * vol * vol;
    for (int i = 0; i < n; ++i) {
        const double drift = drift_rate * t[i + 1];
        spots[i] = spot * exp(drift + vol * w[i]);
    }
    free(t);
    free(w);
}

/* src/pricers/qmc.cpp:15-30 */
double orc_qmc_sobol_european(double spot, double strike, double rate, double carry_yield,
                              double vol, double time, int type, uint64_t path_count) {
    const double discount = exp(-rate * time);
    const double phi = sgn(type);
    double sum = 0.0;
    for (uint64_t index = 1; index <= path_count; ++index) {
        const double u = orc_sobol_point(0, index);
        const double z = orc_inv_normal_cdf(u);
        sum += discount * maxd(phi * (gbm_terminal_spot(spot, rate, carry_yield, vol, time, z) - strike), 0.0);
    }
    return sum / (double)path_count;
}

/* src/pricers/qmc.cpp:32-57 (arithmetic average; dims = monitoring points). */
double orc_qmc_sobol_asian(double spot, double strike, double rate, double carry_yield,
                           double vol, double time, int type, int strike_style,
                           int monitoring_points, uint64_t path_count) {
    const double discount = exp(-rate * time);
    const int n = monitoring_points;
    const double phi = sgn(type);
    double* normals = (double*)malloc(sizeof(double) * (size_t)n);
    double* spots = (double*)malloc(sizeof(double) * (size_t)n);
    uint32_t(*v)[33] = malloc(sizeof(uint32_t[33]) * (size_t)n);
    for (int d = 0; d < n; ++d) orc_sobol_directions((unsigned)d, v[d]);
    double sum = 0.0;
    for (uint64_t index = 1; index <= path_count; ++index) {
        const uint64_t gray = index ^ (index >> 1);
        for (int d = 0; d < n; ++d) {
            uint32_t x = 0;
            for (unsigned b = 0; b < 32; ++b)
                if ((gray >> b) & 1u) x ^= v[d][b + 1];
            const double u = (double)x / (double)((uint64_t)1 << 32);
            normals[d] = orc_inv_normal_cdf(u);
        }
        orc_brownian_bridge_gbm_path(spot, rate, carry_yield, vol, time, n, normals, spots);
        double s_sum = 0.0, last = 0.0;
        unsigned count = 0;
        for (int i = 0; i < n; ++i) {
            s_sum += spots[i];
            last = spots[i];
            ++count;
        }
        const double average = s_sum / (double)count;
        const double ref = strike_style == 0 ? (average - strike) : (last - average);
        sum += discount * maxd(phi * ref, 0.0);
    }
    free(normals);
    free(spots);
    free(v);
    return sum / (double)path_count;
}

/* ------------------------------------------------------------------------ */
/* Longstaff-Schwartz: src/pricers/lsm.cpp                                  */
/* ------------------------------------------------------------------------ */
/* lsm.cpp:21-25 */
void orc_laguerre_basis(double x, double out[4]) {
    const double e = exp(-x / 2.0);
    out[0] = e;
    out[1] = e * (1.0 - x);
    out[2] = e * (1.0 - 2.0 * x + 0.5 * x * x);
    out[3] = e * (1.0 - 3.0 * x + 1.5 * x * x - x * x * x / 6.0);
}

static inline double intrinsic(double s, double k, int type) {
    return maxd(sgn(type) * (s - k), 0.0);
}

/* src/core/linalg.cpp:7-71 */
void orc_householder_least_squares(double* a, int rows, int cols, double* y, double* beta) {
    double* v = (double*)malloc(sizeof(double) * (size_t)rows);
    for (int k = 0; k < cols; ++k) {
        double norm_sq = 0.0;
        for (int i = k; i < rows; ++i) {
            const double x = a[(size_t)i * cols + k];
            norm_sq += x * x;
        }
        const double norm = sqrt(norm_sq);
        if (norm == 0.0) continue;
        const double akk = a[(size_t)k * cols + k];
        const double alpha = akk >= 0.0 ? -norm : norm;
        const int len = rows - k;
        v[0] = akk - alpha;
        for (int i = k + 1; i < rows; ++i) v[i - k] = a[(size_t)i * cols + k];
        double v_norm_sq = 0.0;
        for (int i = 0; i < len; ++i) v_norm_sq += v[i] * v[i];
        if (v_norm_sq == 0.0) continue;
        for (int j = k; j < cols; ++j) {
            double dot = 0.0;
            for (int i = k; i < rows; ++i) dot += v[i - k] * a[(size_t)i * cols + j];
            const double factor = 2.0 * dot / v_norm_sq;
            for (int i = k; i < rows; ++i) a[(size_t)i * cols + j] -= factor * v[i - k];
        }
        double dot_y = 0.0;
        for (int i = k; i < rows; ++i) dot_y += v[i - k] * y[i];
        const double factor_y = 2.0 * dot_y / v_norm_sq;
        for (int i = k; i < rows; ++i) y[i] -= factor_y * v[i - k];
    }
    for (int i = cols - 1; i >= 0; --i) {
        double sum = y[i];
        for (int j = i + 1; j < cols; ++j) sum -= a[(size_t)i * cols + j] * beta[j];
        const double diag = a[(size_t)i * cols + i];
        beta[i] = diag != 0.0 ? sum / diag : 0.0;
    }
    free(v);
}

/* lsm.cpp:35-58: row-major path_count x (n+1) FP64 paths. */
static double* simulate_paths(double spot, double rate, double q, double vol, double time, int n,
                              uint64_t path_count, uint64_t seed) {
    const double dt = time / (double)n;
    const size_t stride = (size_t)n + 1;
    double* paths = (double*)malloc(sizeof(double) * (size_t)path_count * stride);
    for (uint64_t i = 0; i < path_count; ++i) {
        double s = spot;
        const size_t row = (size_t)i * stride;
        paths[row] = s;
        for (int step = 0; step < n; ++step) {
            const double z = orc_normal_variate(seed, i, (uint32_t)step);
            s = gbm_terminal_spot(s, rate, q, vol, dt, z);
            paths[row + (size_t)step + 1] = s;
        }
    }
    return paths;
}

/* lsm.cpp:62-149 */
orc_mc_result orc_lsm_american(double spot, double strike, double rate, double carry_yield,
                               double vol, double time, int type, int monitoring_points,
                               uint64_t path_count, uint64_t seed, double* coefficients,
                               uint8_t* has_coeffs, int* exercise_at_inception) {
    const int n = monitoring_points;
    const double dt = time / (double)n;
    const double disc = exp(-rate * dt);
    const size_t stride = (size_t)n + 1;
    double* paths = simulate_paths(spot, rate, carry_yield, vol, time, n, path_count, seed);
    double* cashflow = (double*)malloc(sizeof(double) * (size_t)path_count);
    double* design = (double*)malloc(sizeof(double) * (size_t)path_count * 4);
    double* targets = (double*)malloc(sizeof(double) * (size_t)path_count);
    uint64_t* itm = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)path_count);
    if (coefficients) memset(coefficients, 0, sizeof(double) * stride * 4);
    if (has_coeffs) memset(has_coeffs, 0, stride);
    for (uint64_t i = 0; i < path_count; ++i)
        cashflow[i] = intrinsic(paths[(size_t)i * stride + (size_t)n], strike, type);
    for (int step = n - 1; step >= 1; --step) {
        for (uint64_t i = 0; i < path_count; ++i) cashflow[i] *= disc;
        uint64_t m = 0;
        for (uint64_t i = 0; i < path_count; ++i) {
            const double s = paths[(size_t)i * stride + (size_t)step];
            if (intrinsic(s, strike, type) > 0.0) {
                orc_laguerre_basis(s / strike, &design[m * 4]);
                targets[m] = cashflow[i];
                itm[m] = i;
                ++m;
            }
        }
        if (m < 4) continue;
        double beta[4] = {0, 0, 0, 0};
        orc_householder_least_squares(design, (int)m, 4, targets, beta);
        if (coefficients) memcpy(&coefficients[(size_t)step * 4], beta, sizeof(beta));
        if (has_coeffs) has_coeffs[step] = 1;
        for (uint64_t j = 0; j < m; ++j) {
            const uint64_t i = itm[j];
            const double s = paths[(size_t)i * stride + (size_t)step];
            double basis[4];
            orc_laguerre_basis(s / strike, basis);
            double continuation = 0.0;
            for (int b = 0; b < 4; ++b) continuation += beta[b] * basis[b];
            const double exercise_value = intrinsic(s, strike, type);
            if (exercise_value > continuation) cashflow[i] = exercise_value;
        }
    }
    for (uint64_t i = 0; i < path_count; ++i) cashflow[i] *= disc;
    orc_welford acc = {0, 0.0, 0.0};
    for (uint64_t i = 0; i < path_count; ++i) orc_welford_add(&acc, cashflow[i]);
    free(paths);
    free(cashflow);
    free(design);
    free(targets);
    free(itm);
    orc_mc_result r;
    r.path_count = path_count;
    const double inception = intrinsic(spot, strike, type);
    if (inception > acc.mean) {
        if (exercise_at_inception) *exercise_at_inception = 1;
        r.price = inception;
        r.standard_error = 0.0;
        return r;
    }
    if (exercise_at_inception) *exercise_at_inception = 0;
    r.price = acc.mean;
    r.standard_error = orc_welford_se(&acc);
    return r;
}

/* lsm.cpp:151-213 */
double orc_lsm_reprice_frozen(double spot, double strike, double rate, double carry_yield,
                              double vol, double time, int type, int monitoring_points,
                              uint64_t path_count, uint64_t seed, const double* coefficients,
                              const uint8_t* has_coeffs, int exercise_at_inception) {
    const int n = monitoring_points;
    const double dt = time / (double)n;
    const double disc = exp(-rate * dt);
    const size_t stride = (size_t)n + 1;
    double* paths = simulate_paths(spot, rate, carry_yield, vol, time, n, path_count, seed);
    double* cashflow = (double*)malloc(sizeof(double) * (size_t)path_count);
    for (uint64_t i = 0; i < path_count; ++i)
        cashflow[i] = intrinsic(paths[(size_t)i * stride + (size_t)n], strike, type);
    for (int step = n - 1; step >= 1; --step) {
        for (uint64_t i = 0; i < path_count; ++i) cashflow[i] *= disc;
        if (!has_coeffs[step]) continue;
        const double* beta = &coefficients[(size_t)step * 4];
        for (uint64_t i = 0; i < path_count; ++i) {
            const double s = paths[(size_t)i * stride + (size_t)step];
            const double exercise_value = intrinsic(s, strike, type);
            if (exercise_value <= 0.0) continue;
            double basis[4];
            orc_laguerre_basis(s / strike, basis);
            double continuation = 0.0;
            for (int b = 0; b < 4; ++b) continuation += beta[b] * basis[b];
            if (exercise_value > continuation) cashflow[i] = exercise_value;
        }
    }
    for (uint64_t i = 0; i < path_count; ++i) cashflow[i] *= disc;
    orc_welford acc = {0, 0.0, 0.0};
    for (uint64_t i = 0; i < path_count; ++i) orc_welford_add(&acc, cashflow[i]);
    free(paths);
    free(cashflow);
    if (exercise_at_inception) return intrinsic(spot, strike, type);
    return acc.mean;
}

/* ------------------------------------------------------------------------ */
/* Heston: src/pricers/heston.cpp                                           */
/* ------------------------------------------------------------------------ */
/* heston.cpp:91-116 */
static double qe_variance_step(double v_t, double kappa, double theta, double xi, double dt,
                               double raw_uniform) {
    const double psi_critical = 1.5;
    const double e = exp(-kappa * dt);
    const double m = theta + (v_t - theta) * e;
    const double s2 = v_t * xi * xi * e / kappa * (1.0 - e) +
                      theta * xi * xi / (2.0 * kappa) * (1.0 - e) * (1.0 - e);
    const double psi = s2 / (m * m);
    if (psi <= psi_critical) {
        const double inv_psi = 1.0 / psi;
        const double b2 = 2.0 * inv_psi - 1.0 + sqrt(2.0 * inv_psi) * sqrt(2.0 * inv_psi - 1.0);
        const double a = m / (1.0 + b2);
        const double z_v = orc_inv_normal_cdf(raw_uniform);
        const double b = sqrt(b2);
        return a * (b + z_v) * (b + z_v);
    }
    const double p = (psi - 1.0) / (psi + 1.0);
    const double beta = (1.0 - p) / m;
    if (raw_uniform <= p) return 0.0;
    return log((1.0 - p) / (1.0 - raw_uniform)) / beta;
}

/* heston.cpp:120-156 */
orc_mc_result orc_heston_qe_european(const orc_heston_params* p, double strike, int type,
                                     int monitoring_points, uint64_t path_count, uint64_t seed) {
    const double dt = p->time / (double)monitoring_points;
    const double drift = (p->rate - p->carry_yield) * dt;
    const double k0 = -p->rho * p->kappa * p->theta * dt / p->xi;
    const double k1 = 0.5 * dt * (p->kappa * p->rho / p->xi - 0.5) - p->rho / p->xi;
    const double k2 = 0.5 * dt * (p->kappa * p->rho / p->xi - 0.5) + p->rho / p->xi;
    const double k3 = 0.5 * dt * (1.0 - p->rho * p->rho);
    const double k4 = k3;
    const double discount = exp(-p->rate * p->time);
    const double phi = sgn(type);
    const double log_s0 = log(p->spot);
    orc_welford acc = {0, 0.0, 0.0};
    for (uint64_t i = 0; i < path_count; ++i) {
        double v = p->v0;
        double log_s = log_s0;
        for (int step = 0; step < monitoring_points; ++step) {
            const uint32_t d = (uint32_t)step;
            const double z_s = orc_normal_variate(seed, i, d);
            const double raw_uniform = orc_uniform_variate(seed, i, d);
            const double v_next = qe_variance_step(v, p->kappa, p->theta, p->xi, dt, raw_uniform);
            const double diffusion_var = maxd(k3 * v + k4 * v_next, 0.0);
            log_s += drift + k0 + k1 * v + k2 * v_next + sqrt(diffusion_var) * z_s;
            v = v_next;
        }
        const double s_t = exp(log_s);
        const double payoff = maxd(phi * (s_t - strike), 0.0);
        orc_welford_add(&acc, discount * payoff);
    }
    orc_mc_result r;
    r.price = acc.mean;
    r.standard_error = orc_welford_se(&acc);
    r.path_count = acc.count;
    return r;
}

/* Gauss-Legendre: src/core/gauss_legendre.cpp:9-69 */
static void legendre(int n, double x, double* p_n, double* p_nm1) {
    double p_prev = 1.0, p_curr = x;
    if (n == 0) {
        *p_n = 1.0;
        *p_nm1 = 0.0;
        return;
    }
    for (int k = 2; k <= n; ++k) {
        const double p_next =
            ((2.0 * (double)k - 1.0) * x * p_curr - ((double)k - 1.0) * p_prev) / (double)k;
        p_prev = p_curr;
        p_curr = p_next;
    }
    *p_n = p_curr;
    *p_nm1 = p_prev;
}

static void gauss_legendre_rule(int order, double* nodes, double* weights) {
    const int half = (order + 1) / 2;
    for (int i = 0; i < half; ++i) {
        double x = cos(PI_D * ((double)i + 0.75) / ((double)order + 0.5));
        double p_prime = 0.0;
        for (int iter = 0; iter < 100; ++iter) {
            double pn, pnm1;
            legendre(order, x, &pn, &pnm1);
            p_prime = (double)order * (x * pn - pnm1) / (x * x - 1.0);
            const double dx = pn / p_prime;
            x -= dx;
            if (fabs(dx) < 1e-15) break;
        }
        const double weight = 2.0 / ((1.0 - x * x) * p_prime * p_prime);
        nodes[i] = -x;
        nodes[order - 1 - i] = x;
        weights[i] = weight;
        weights[order - 1 - i] = weight;
    }
}

/* heston.cpp:26-40 ("Little Trap" characteristic function) */
static double complex heston_cf(const orc_heston_params* p, double complex u) {
    const double complex i = I;
    const double complex rho_xi_iu = p->rho * p->xi * i * u;
    const double complex bmr = p->kappa - rho_xi_iu;
    const double complex d = csqrt(bmr * bmr + p->xi * p->xi * (i * u + u * u));
    const double complex c = (bmr - d) / (bmr + d);
    const double complex exp_neg_dt = cexp(-d * p->time);
    const double complex big_c =
        i * u * (p->rate - p->carry_yield) * p->time +
        (p->kappa * p->theta / (p->xi * p->xi)) *
            ((bmr - d) * p->time - 2.0 * clog((1.0 - c * exp_neg_dt) / (1.0 - c)));
    const double complex big_d =
        (bmr - d) / (p->xi * p->xi) * (1.0 - exp_neg_dt) / (1.0 - c * exp_neg_dt);
    return cexp(big_c + big_d * p->v0);
}

/* heston.cpp:48-82 (128-point Gauss-Legendre on [0, 200]) */
double orc_heston_semi_analytic(const orc_heston_params* p, double strike, int type) {
    enum { ORDER = 128 };
    double nodes[ORDER], weights[ORDER];
    gauss_legendre_rule(ORDER, nodes, weights);
    const double complex i = I;
    const double log_moneyness = log(strike / p->spot);
    const double complex phi_neg_i = heston_cf(p, CMPLX(0.0, -1.0));
    const double a = 0.0, b = 200.0;
    const double half_width = 0.5 * (b - a), midpoint = 0.5 * (a + b);
    double sum1 = 0.0, sum2 = 0.0;
    for (int k = 0; k < ORDER; ++k) {
        const double u = midpoint + half_width * nodes[k];
        const double complex phi_u_minus_i = heston_cf(p, CMPLX(u, -1.0));
        const double complex v1 =
            cexp(-i * u * log_moneyness) * (phi_u_minus_i / phi_neg_i) / (i * u);
        sum1 += weights[k] * creal(v1);
        const double complex phi_u = heston_cf(p, CMPLX(u, 0.0));
        const double complex v2 = cexp(-i * u * log_moneyness) * phi_u / (i * u);
        sum2 += weights[k] * creal(v2);
    }
    const double p1 = 0.5 + half_width * sum1 / PI_D;
    const double p2 = 0.5 + half_width * sum2 / PI_D;
    const double dq = exp(-p->carry_yield * p->time);
    const double dr = exp(-p->rate * p->time);
    const double call = p->spot * dq * p1 - strike * dr * p2;
    if (type == 0) return call;
    return call - p->spot * dq + strike * dr;
}

/* ------------------------------------------------------------------------ */
/* Greeks                                                                   */
/* ------------------------------------------------------------------------ */
/* src/greeks/finite_difference.cpp:23-38 */
orc_bumps orc_default_bump_sizes(double spot, double vol, double time) {
    orc_bumps b;
    b.spot = maxd(spot * 0.01, 1e-4);
    b.vol = maxd(vol * 0.01, 1e-4);
    b.rate = 0.01;
    b.time = maxd(time * 0.01, 1e-4);
    return b;
}

/* finite_difference.cpp:40-65 (nine CRN re-prices, single-threaded). */
orc_european_greeks orc_fd_european(double spot, double strike, double rate, double carry_yield,
                                    double vol, double time, int type, uint64_t path_count,
                                    uint64_t seed, orc_bumps bumps, unsigned chunk_count) {
    orc_options o = {0, 0, 0, 1, chunk_count};
#define PR(s, r, q, v, t) orc_mc_european(s, strike, r, q, v, t, type, path_count, seed, &o).price
    const double v0 = PR(spot, rate, carry_yield, vol, time);
    const double su = PR(spot + bumps.spot, rate, carry_yield, vol, time);
    const double sd = PR(spot - bumps.spot, rate, carry_yield, vol, time);
    const double vu = PR(spot, rate, carry_yield, vol + bumps.vol, time);
    const double vd = PR(spot, rate, carry_yield, vol - bumps.vol, time);
    const double ru = PR(spot, rate + bumps.rate, carry_yield, vol, time);
    const double rd = PR(spot, rate - bumps.rate, carry_yield, vol, time);
    const double tu = PR(spot, rate, carry_yield, vol, time + bumps.time);
    const double td = PR(spot, rate, carry_yield, vol, time - bumps.time);
#undef PR
    orc_european_greeks g;
    g.delta = (su - sd) / (2.0 * bumps.spot);
    g.gamma = (su - 2.0 * v0 + sd) / (bumps.spot * bumps.spot);
    g.vega = (vu - vd) / (2.0 * bumps.vol);
    g.theta = -(tu - td) / (2.0 * bumps.time);
    g.rho = (ru - rd) / (2.0 * bumps.rate);
    return g;
}

static orc_greek finish_greek(const orc_welford* w) {
    orc_greek g;
    g.value = w->mean;
    g.standard_error = orc_welford_se(w);
    return g;
}

/* likelihood_ratio.cpp:33-73 */
static orc_lr_greeks lr_terminal(const orc_product* p, uint64_t path_count) {
    const double discount = exp(-p->rate * p->time);
    const double sqrt_t = sqrt(p->time);
    const double mu = p->rate - p->q - 0.5 * p->vol * p->vol;
    orc_welford d = {0}, g = {0}, v = {0}, th = {0}, rh = {0};
    for (uint64_t i = 0; i < path_count; ++i) {
        const double z = orc_normal_variate(p->seed, i, 0);
        const double s_t = gbm_terminal_spot(p->spot, p->rate, p->q, p->vol, p->time, z);
        const double h = discount * terminal_payoff(p, s_t);
        const double delta_score = z / (p->spot * p->vol * sqrt_t);
        const double gamma_score =
            (z * z - p->vol * sqrt_t * z - 1.0) / (p->spot * p->spot * p->vol * p->vol * p->time);
        const double vega_score = (z * z - 1.0) / p->vol - sqrt_t * z;
        const double rho_raw = sqrt_t * z / p->vol;
        const double theta_raw = (z * z - 1.0) / (2.0 * p->time) + mu * z / (p->vol * sqrt_t);
        orc_welford_add(&d, h * delta_score);
        orc_welford_add(&g, h * gamma_score);
        orc_welford_add(&v, h * vega_score);
        orc_welford_add(&rh, h * (rho_raw - p->time));
        orc_welford_add(&th, h * (p->rate - theta_raw));
    }
    orc_lr_greeks r;
    r.delta = finish_greek(&d);
    r.gamma = finish_greek(&g);
    r.vega = finish_greek(&v);
    r.rho = finish_greek(&rh);
    r.theta = finish_greek(&th);
    r.has_theta = 1;
    return r;
}

orc_lr_greeks orc_lr_european(double spot, double strike, double rate, double carry_yield,
                              double vol, double time, int type, uint64_t path_count,
                              uint64_t seed) {
    orc_product p;
    product_init(&p, spot, strike, rate, carry_yield, vol, time, type, seed);
    p.product = P_EUROPEAN;
    return lr_terminal(&p, path_count);
}

orc_lr_greeks orc_lr_digital(double spot, double strike, double rate, double carry_yield,
                             double vol, double time, int type, int digital_style,
                             double cash_amount, uint64_t path_count, uint64_t seed) {
    orc_product p;
    product_init(&p, spot, strike, rate, carry_yield, vol, time, type, seed);
    p.product = P_DIGITAL;
    p.digital_style = digital_style;
    p.cash = cash_amount;
    return lr_terminal(&p, path_count);
}

/* likelihood_ratio.cpp:105-154 */
orc_lr_greeks orc_lr_barrier(double spot, double strike, double barrier, double rate,
                             double carry_yield, double vol, double time, int type,
                             int direction, int knock, double rebate, int monitoring_points,
                             uint64_t path_count, uint64_t seed) {
    const double dt = time / (double)monitoring_points;
    const double sqrt_dt = sqrt(dt);
    const double discount = exp(-rate * time);
    orc_welford d = {0}, g = {0}, v = {0}, rh = {0};
    for (uint64_t i = 0; i < path_count; ++i) {
        double s = spot, z1 = 0.0, vega_sum = 0.0, rho_sum = 0.0, last = 0.0;
        int breached = 0;
        for (int step = 0; step < monitoring_points; ++step) {
            const double z = orc_normal_variate(seed, i, (uint32_t)step);
            if (step == 0) z1 = z;
            vega_sum += (z * z - 1.0) / vol - sqrt_dt * z;
            rho_sum += sqrt_dt * z / vol;
            s = gbm_terminal_spot(s, rate, carry_yield, vol, dt, z);
            const int crossed = direction == 0 ? s >= barrier : s <= barrier;
            breached = breached || crossed;
            last = s;
        }
        const double phi = sgn(type);
        const double vanilla = maxd(phi * (last - strike), 0.0);
        const int pays = knock == 1 ? !breached : breached;
        const double h = discount * (pays ? vanilla : rebate);
        const double delta_score = z1 / (spot * vol * sqrt_dt);
        const double gamma_score = (z1 * z1 - vol * sqrt_dt * z1 - 1.0) / (spot * spot * vol * vol * dt);
        orc_welford_add(&d, h * delta_score);
        orc_welford_add(&g, h * gamma_score);
        orc_welford_add(&v, h * vega_sum);
        orc_welford_add(&rh, h * (rho_sum - time));
    }
    orc_lr_greeks r;
    memset(&r, 0, sizeof(r));
    r.delta = finish_greek(&d);
    r.gamma = finish_greek(&g);
    r.vega = finish_greek(&v);
    r.rho = finish_greek(&rh);
    r.has_theta = 0;
    return r;
}

/* pathwise.cpp:28-55 */
orc_pathwise_greeks orc_pathwise_european(double spot, double strike, double rate,
                                          double carry_yield, double vol, double time, int type,
                                          uint64_t path_count, uint64_t seed) {
    const double discount = exp(-rate * time);
    const double sqrt_t = sqrt(time);
    const double phi = sgn(type);
    orc_welford d = {0}, v = {0}, rh = {0};
    for (uint64_t i = 0; i < path_count; ++i) {
        const double z = orc_normal_variate(seed, i, 0);
        const double s_t = gbm_terminal_spot(spot, rate, carry_yield, vol, time, z);
        const int itm = phi * (s_t - strike) > 0.0;
        const double slope = itm ? phi : 0.0;
        const double h = discount * maxd(phi * (s_t - strike), 0.0);
        const double ds_dspot = s_t / spot;
        const double ds_dvol = s_t * (sqrt_t * z - vol * time);
        const double ds_drate = s_t * time;
        orc_welford_add(&d, discount * slope * ds_dspot);
        orc_welford_add(&v, discount * slope * ds_dvol);
        orc_welford_add(&rh, discount * slope * ds_drate - time * h);
    }
    orc_pathwise_greeks r;
    r.delta = finish_greek(&d);
    r.vega = finish_greek(&v);
    r.rho = finish_greek(&rh);
    return r;
}

/* pathwise.cpp:64-147 */
orc_pathwise_greeks orc_pathwise_asian(double spot, double strike, double rate,
                                       double carry_yield, double vol, double time, int type,
                                       int strike_style, int average_style,
                                       int monitoring_points, uint64_t path_count,
                                       uint64_t seed) {
    const double dt = time / (double)monitoring_points;
    const double sqrt_dt = sqrt(dt);
    const double discount = exp(-rate * time);
    const double phi = sgn(type);
    const double n = (double)monitoring_points;
    orc_welford d = {0}, v = {0}, rh = {0};
    for (uint64_t p = 0; p < path_count; ++p) {
        double s = spot, cum_z = 0.0, sum_s = 0.0, log_sum = 0.0;
        double sum_s_dvol = 0.0, sum_dlns_dvol = 0.0, sum_s_drate = 0.0, sum_dlns_drate = 0.0;
        double last_s_dvol = 0.0, last_s_drate = 0.0;
        for (int step = 0; step < monitoring_points; ++step) {
            const double z = orc_normal_variate(seed, p, (uint32_t)step);
            cum_z += z;
            s = gbm_terminal_spot(s, rate, carry_yield, vol, dt, z);
            const double i = (double)(step + 1);
            const double dlns_dvol = -vol * i * dt + sqrt_dt * cum_z;
            const double dlns_drate = i * dt;
            const double ds_dvol = s * dlns_dvol;
            const double ds_drate = s * dlns_drate;
            sum_s += s;
            log_sum += log(s);
            sum_s_dvol += ds_dvol;
            sum_dlns_dvol += dlns_dvol;
            sum_s_drate += ds_drate;
            sum_dlns_drate += dlns_drate;
            last_s_dvol = ds_dvol;
            last_s_drate = ds_drate;
        }
        const double avg = average_style == 0 ? sum_s / n : exp(log_sum / n);
        const double d_avg_dspot = avg / spot;
        const double d_avg_dvol = average_style == 0 ? sum_s_dvol / n : avg * (sum_dlns_dvol / n);
        const double d_avg_drate = average_style == 0 ? sum_s_drate / n : avg * (sum_dlns_drate / n);
        const double d_slast_dspot = s / spot;
        const double ref = strike_style == 0 ? (avg - strike) : (s - avg);
        const int itm = phi * ref > 0.0;
        const double slope = itm ? phi : 0.0;
        const double h = discount * maxd(phi * ref, 0.0);
        double delta_raw, vega_raw, rate_raw;
        if (strike_style == 0) {
            delta_raw = slope * d_avg_dspot;
            vega_raw = slope * d_avg_dvol;
            rate_raw = slope * d_avg_drate;
        } else {
            delta_raw = slope * (d_slast_dspot - d_avg_dspot);
            vega_raw = slope * (last_s_dvol - d_avg_dvol);
            rate_raw = slope * (last_s_drate - d_avg_drate);
        }
        orc_welford_add(&d, discount * delta_raw);
        orc_welford_add(&v, discount * vega_raw);
        orc_welford_add(&rh, discount * rate_raw - time * h);
    }
    orc_pathwise_greeks r;
    r.delta = finish_greek(&d);
    r.vega = finish_greek(&v);
    r.rho = finish_greek(&rh);
    return r;
}

/* ------------------------------------------------------------------------ */
/* Analytic oracles: src/pricers/analytic.cpp                               */
/* ------------------------------------------------------------------------ */
/* analytic.cpp:20-38 */
double orc_bsm(double spot, double strike, double rate, double carry_yield, double vol,
               double time, int type) {
    const double b = rate - carry_yield;
    const double sqrt_t = sqrt(time);
    const double d1 = (log(spot / strike) + (b + 0.5 * vol * vol) * time) / (vol * sqrt_t);
    const double d2 = d1 - vol * sqrt_t;
    const double phi = sgn(type);
    const double df_carry = exp(-carry_yield * time);
    const double df_rate = exp(-rate * time);
    return phi * spot * df_carry * orc_normal_cdf(phi * d1) -
           phi * strike * df_rate * orc_normal_cdf(phi * d2);
}

/* analytic.cpp:51-59 */
double orc_kemna_vorst(double spot, double strike, double rate, double carry_yield, double vol,
                       double time, int type) {
    const double sigma_g = vol / SQRT3_D;
    const double b_g = 0.5 * (rate - carry_yield - vol * vol / 6.0);
    const double q_eff = rate - b_g;
    return orc_bsm(spot, strike, rate, q_eff, sigma_g, time, type);
}

/* analytic.cpp:61-132 */
double orc_reiner_rubinstein(double spot, double strike, double barrier, double rate,
                             double carry_yield, double vol, double time, int type,
                             int direction, int knock, double rebate) {
    const double b = rate - carry_yield;
    const double sqrt_t = sqrt(time);
    const double mu = (b - 0.5 * vol * vol) / (vol * vol);
    const double lambda = sqrt(mu * mu + 2.0 * rate / (vol * vol));
    const double phi = sgn(type);
    const double eta = direction == 1 ? 1.0 : -1.0;
    const double x1 = log(spot / strike) / (vol * sqrt_t) + (1.0 + mu) * vol * sqrt_t;
    const double x2 = log(spot / barrier) / (vol * sqrt_t) + (1.0 + mu) * vol * sqrt_t;
    const double y1 = log(barrier * barrier / (spot * strike)) / (vol * sqrt_t) + (1.0 + mu) * vol * sqrt_t;
    const double y2 = log(barrier / spot) / (vol * sqrt_t) + (1.0 + mu) * vol * sqrt_t;
    const double z = log(barrier / spot) / (vol * sqrt_t) + lambda * vol * sqrt_t;
    const double df_carry = exp((b - rate) * time);
    const double df_rate = exp(-rate * time);
    const double hs_2mu1 = pow(barrier / spot, 2.0 * (mu + 1.0));
    const double hs_2mu = pow(barrier / spot, 2.0 * mu);
    const double A = phi * spot * df_carry * orc_normal_cdf(phi * x1) -
                     phi * strike * df_rate * orc_normal_cdf(phi * x1 - phi * vol * sqrt_t);
    const double B = phi * spot * df_carry * orc_normal_cdf(phi * x2) -
                     phi * strike * df_rate * orc_normal_cdf(phi * x2 - phi * vol * sqrt_t);
    const double C = phi * spot * df_carry * hs_2mu1 * orc_normal_cdf(eta * y1) -
                     phi * strike * df_rate * hs_2mu * orc_normal_cdf(eta * y1 - eta * vol * sqrt_t);
    const double D = phi * spot * df_carry * hs_2mu1 * orc_normal_cdf(eta * y2) -
                     phi * strike * df_rate * hs_2mu * orc_normal_cdf(eta * y2 - eta * vol * sqrt_t);
    const double E = rebate * df_rate *
                     (orc_normal_cdf(eta * x2 - eta * vol * sqrt_t) -
                      hs_2mu * orc_normal_cdf(eta * y2 - eta * vol * sqrt_t));
    const double F = rebate * (pow(barrier / spot, mu + lambda) * orc_normal_cdf(eta * z) +
                               pow(barrier / spot, mu - lambda) *
                                   orc_normal_cdf(eta * z - 2.0 * eta * lambda * vol * sqrt_t));
    const int above = strike > barrier;
    if (knock == 0) {
        if (direction == 1) {
            if (type == 0) return above ? (C + E) : (A - B + D + E);
            return above ? (B - C + D + E) : (A + E);
        }
        if (type == 0) return above ? (A + E) : (B - C + D + E);
        return above ? (A - B + D + E) : (C + E);
    }
    if (direction == 1) {
        if (type == 0) return above ? (A - C + F) : (B - D + F);
        return above ? (A - B + C - D + F) : F;
    }
    if (type == 0) return above ? F : (A - B + C - D + F);
    return above ? (B - D + F) : (A - C + F);
}

/* analytic.cpp:145-190 (lookback core terms and fixed strike) */
static void lookback_core(double spot, double reference, double rate, double q, double vol,
                          double time, double* lambda, double* d1, double* std_dev) {
    *lambda = 2.0 * (rate - q) / (vol * vol);
    *std_dev = vol * sqrt(time);
    *d1 = log(spot / reference) / *std_dev + 0.5 * (*lambda + 1.0) * *std_dev;
}

static double lookback_fixed_ab(double spot, double reference, double rate, double q, double vol,
                                double time, double eta) {
    double lambda, d1, std_dev;
    lookback_core(spot, reference, rate, q, vol, time, &lambda, &d1, &std_dev);
    const double n1 = orc_normal_cdf(eta * d1);
    const double n2 = orc_normal_cdf(eta * (d1 - std_dev));
    const double n3 = orc_normal_cdf(eta * (d1 - lambda * std_dev));
    const double n4 = orc_normal_cdf(eta * d1);
    const double pow_ratio = pow(spot / reference, -lambda);
    const double df_carry = exp(-q * time);
    const double df_rate = exp(-rate * time);
    return eta * (spot * df_carry * n1 - reference * df_rate * n2 -
                  spot * df_rate * (pow_ratio * n3 - df_carry * n4 / df_rate) / lambda);
}

double orc_lookback_fixed(double spot, double strike, double rate, double carry_yield,
                          double vol, double time, int type) {
    const double extremum = spot;
    const double eta = type == 0 ? 1.0 : -1.0;
    const int guaranteed = type == 0 ? strike <= extremum : strike >= extremum;
    if (guaranteed)
        return lookback_fixed_ab(spot, extremum, rate, carry_yield, vol, time, eta) +
               eta * exp(-rate * time) * (extremum - strike);
    return lookback_fixed_ab(spot, strike, rate, carry_yield, vol, time, eta);
}

/* analytic.cpp:192-208 */
double orc_lookback_floating(double spot, double rate, double carry_yield, double vol,
                             double time, int type) {
    const double extremum = spot;
    const double eta = type == 0 ? 1.0 : -1.0;
    double lambda, d1, std_dev;
    lookback_core(spot, extremum, rate, carry_yield, vol, time, &lambda, &d1, &std_dev);
    const double n1 = orc_normal_cdf(eta * d1);
    const double n2 = orc_normal_cdf(eta * (d1 - std_dev));
    const double n3 = orc_normal_cdf(eta * (-d1 + lambda * std_dev));
    const double n4 = orc_normal_cdf(eta * -d1);
    const double pow_ratio = pow(spot / extremum, -lambda);
    const double df_carry = exp(-carry_yield * time);
    const double df_rate = exp(-rate * time);
    return eta * ((spot * df_carry * n1 - extremum * df_rate * n2) +
                  spot * df_rate * (pow_ratio * n3 - df_carry * n4 / df_rate) / lambda);
}

/* analytic.cpp:210-218 */
double orc_digital_analytic(double spot, double strike, double rate, double carry_yield,
                            double vol, double time, int type, int style, double cash_amount) {
    const double b = rate - carry_yield;
    const double sqrt_t = sqrt(time);
    const double d1 = (log(spot / strike) + (b + 0.5 * vol * vol) * time) / (vol * sqrt_t);
    const double d2 = d1 - vol * sqrt_t;
    const double phi = sgn(type);
    if (style == 0) return cash_amount * exp(-rate * time) * orc_normal_cdf(phi * d2);
    return spot * exp(-carry_yield * time) * orc_normal_cdf(phi * d1);
}

/* src/pricers/binomial.cpp:41-72 */
double orc_crr_binomial_american(double spot, double strike, double rate, double carry_yield,
                                 double vol, double time, int steps, int type) {
    const double dt = time / (double)steps;
    const double u = exp(vol * sqrt(dt));
    const double d = 1.0 / u;
    const double growth = exp((rate - carry_yield) * dt);
    const double pi = (growth - d) / (u - d);
    const double discount = exp(-rate * dt);
    const double phi = sgn(type);
    double* values = (double*)malloc(sizeof(double) * (size_t)(steps + 1));
    for (int i = 0; i <= steps; ++i) {
        const double up = (double)i;
        const double down = (double)steps - up;
        const double st = spot * pow(u, up) * pow(d, down);
        values[i] = maxd(phi * (st - strike), 0.0);
    }
    for (int level = steps - 1; level >= 0; --level) {
        for (int i = 0; i <= level; ++i) {
            const double cont = discount * (pi * values[i + 1] + (1.0 - pi) * values[i]);
            const double up = (double)i;
            const double down = (double)level - up;
            const double node = spot * pow(u, up) * pow(d, down);
            const double ex = maxd(phi * (node - strike), 0.0);
            values[i] = maxd(cont, ex);
        }
    }
    const double r = values[0];
    free(values);
    return r;
}

/* ------------------------------------------------------------------------ */
/* Batch helpers (CPU baseline)                                             */
/* ------------------------------------------------------------------------ */
void orc_price_batch(const orc_contract* c, int n, unsigned num_threads, unsigned chunk_count,
                     orc_mc_result* out) {
    for (int i = 0; i < n; ++i) {
        orc_options o = {c[i].antithetic, c[i].control_variate, c[i].brownian_bridge,
                         num_threads, chunk_count};
        switch (c[i].product) {
        case 0:
            out[i] = orc_mc_european(c[i].spot, c[i].strike, c[i].rate, c[i].carry_yield, c[i].vol,
                                     c[i].time, c[i].type, c[i].path_count, c[i].seed, &o);
            break;
        case 1:
            out[i] = orc_mc_digital(c[i].spot, c[i].strike, c[i].rate, c[i].carry_yield, c[i].vol,
                                    c[i].time, c[i].type, c[i].digital_style, c[i].cash_amount,
                                    c[i].path_count, c[i].seed, &o);
            break;
        case 2:
            out[i] = orc_mc_asian(c[i].spot, c[i].strike, c[i].rate, c[i].carry_yield, c[i].vol,
                                  c[i].time, c[i].type, c[i].strike_style, c[i].average_style,
                                  c[i].monitoring_points, c[i].path_count, c[i].seed, &o);
            break;
        case 3:
            out[i] = orc_mc_barrier(c[i].spot, c[i].strike, c[i].barrier, c[i].rate,
                                    c[i].carry_yield, c[i].vol, c[i].time, c[i].type,
                                    c[i].direction, c[i].knock, c[i].rebate,
                                    c[i].monitoring_points, c[i].path_count, c[i].seed, &o);
            break;
        default:
            out[i] = orc_mc_lookback(c[i].spot, c[i].strike, c[i].rate, c[i].carry_yield,
                                     c[i].vol, c[i].time, c[i].type, c[i].strike_style,
                                     c[i].monitoring_points, c[i].path_count, c[i].seed, &o);
            break;
        }
    }
}

typedef struct {
    const orc_heston_params* sets;
    const double* strikes;
    int n_strikes, type, steps;
    uint64_t paths, seed;
    orc_mc_result* out;
} orc_heston_job;

static void orc_heston_task(void* ctx, unsigned item) {
    orc_heston_job* j = (orc_heston_job*)ctx;
    const unsigned set = item / (unsigned)j->n_strikes, k = item % (unsigned)j->n_strikes;
    j->out[item] = orc_heston_qe_european(&j->sets[set], j->strikes[k], j->type, j->steps, j->paths,
                                          j->seed);
}

void orc_heston_batch(const orc_heston_params* sets, int n_sets, const double* strikes,
                      int n_strikes, int type, int monitoring_points, uint64_t path_count,
                      uint64_t seed, unsigned num_threads, orc_mc_result* out) {
    orc_heston_job j = {sets, strikes, n_strikes, type, monitoring_points, path_count, seed, out};
    orc_parallel_for((unsigned)(n_sets * n_strikes), num_threads, orc_heston_task, &j);
}

typedef struct {
    const double* params;
    int steps;
    uint64_t paths, seed;
    orc_mc_result* out;
} orc_lsm_job;

static void orc_lsm_task(void* ctx, unsigned item) {
    orc_lsm_job* j = (orc_lsm_job*)ctx;
    const double* p = &j->params[(size_t)item * 7];
    j->out[item] = orc_lsm_american(p[0], p[1], p[2], p[3], p[4], p[5], (int)p[6], j->steps, j->paths,
                                    j->seed, NULL, NULL, NULL);
}

void orc_lsm_batch(const double* params, int n, int monitoring_points, uint64_t path_count,
                   uint64_t seed, unsigned num_threads, orc_mc_result* out) {
    orc_lsm_job j = {params, monitoring_points, path_count, seed, out};
    orc_parallel_for((unsigned)n, num_threads, orc_lsm_task, &j);
}
