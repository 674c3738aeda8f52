// request.cpp -- the JSON request handler behind the reference's JSON CLI
// (apps/mcd_cli/main.cpp:229-538) and its AWS Lambda request layer
// (infra/lambda/request.py:225-477), on the GPU engine.  One flat JSON object
// in, one out: the result, or {"error": message}.  Same products, request
// kinds, field names, validation and response fields (price, standard_error,
// ci_95_low/high = price -/+ 1.959963985 SE, path_count, seed,
// elapsed_seconds, paths_per_second; QMC without SE plus a note; LR Greeks
// with <greek>_se).
//
// Two dialects, as the reference has two front ends of one schema:
//   CLI     the CLI's validation messages;
//   Lambda  the Lambda layer's: its messages, a cap on path_count, binomial
//           steps in 1..20,000, and the "antithetic" / "control_variate"
//           toggles of European and Asian price requests.
//
// Additions, in new fields only:
//   "precision": "fp64" (default: the reference's arithmetic) or "fp32";
//   "request": "batch"         many contracts in one launch (mcd_price_batch);
//   "request": "batch_greeks"  price and CRN finite-difference, pathwise and
//                              likelihood-ratio Greeks of many contracts in one
//                              launch (mcd_greeks_batch; "spot_bump",
//                              "vol_bump" relative, default 1e-4).
// In a batch request every contract field may be a scalar (shared) or an
// array (one entry per contract, all arrays of one length); the response
// holds arrays in the same order.
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "json.hpp"
#include "mcd_gpu.h"
#include "mcd_shim.hpp"

namespace {

using mcd::OptionType;
using mcdjson::Object;
using mcdjson::Value;
namespace pricers = mcd::pricers;
namespace greeks = mcd::greeks;

constexpr double kMaxExactInteger = 9007199254740992.0;  // 2^53: seeds and counts travel as JSON numbers
constexpr double kZ975 = 1.959963985;

struct Dialect {
    bool lambda = false;
    std::uint64_t max_path_count = 0;  // 0: no cap
};
thread_local Dialect g_dialect;  // of the request being handled on this thread

template <typename F>
auto timed(F&& f) {
    const auto start = std::chrono::steady_clock::now();
    auto v = f();
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    return std::make_pair(std::move(v), s);
}

const Value& require(const Object& o, const char* key) {
    const Value* v = mcdjson::find(o, key);
    if (!v) throw std::runtime_error(std::string("missing required field '") + key + "'");
    return *v;
}

double as_number(const Value& v, const char* key) {
    if (v.type != Value::Type::Number) throw std::runtime_error(std::string("field '") + key + "' must be a number");
    return v.num;
}

const std::string& as_string(const Value& v, const char* key) {
    if (v.type != Value::Type::String) throw std::runtime_error(std::string("field '") + key + "' must be a string");
    return v.str;
}

double req_num(const Object& o, const char* key) { return as_number(require(o, key), key); }
double opt_num(const Object& o, const char* key, double def) {
    const Value* v = mcdjson::find(o, key);
    return v ? as_number(*v, key) : def;
}
std::string req_str(const Object& o, const char* key) { return as_string(require(o, key), key); }
std::string opt_str(const Object& o, const char* key, const std::string& def) {
    const Value* v = mcdjson::find(o, key);
    return v ? as_string(*v, key) : def;
}

std::uint64_t count_of(double d, const char* key) {
    if (d < 0.0 || d != std::floor(d) || d > kMaxExactInteger)
        throw std::runtime_error(std::string("field '") + key +
                                 (g_dialect.lambda ? "' must be a non-negative integer no larger than 2^53"
                                                   : "' must be a non-negative integer no larger than 2^53 "
                                                     "(exactly representable as a JSON number)"));
    return static_cast<std::uint64_t>(d);
}
std::uint64_t req_count(const Object& o, const char* key) { return count_of(req_num(o, key), key); }

// path_count, with the Lambda layer's cost cap (infra/lambda/request.py:63-70)
std::uint64_t req_paths(const Object& o) {
    const std::uint64_t n = req_count(o, "path_count");
    if (g_dialect.max_path_count && n > g_dialect.max_path_count) {
        std::string cap = std::to_string(g_dialect.max_path_count);
        for (int i = static_cast<int>(cap.size()) - 3; i > 0; i -= 3) cap.insert(static_cast<size_t>(i), ",");
        throw std::runtime_error("'path_count' must not exceed " + cap +
                                 " on this demo endpoint (CLAUDE.md sec.6 Phase 7 cost guardrail) -- run the full "
                                 "engine locally for larger studies");
    }
    return n;
}

int int_of(double d, const char* key) {
    if (d != std::floor(d) || d < -2147483648.0 || d > 2147483647.0)
        throw std::runtime_error(std::string("field '") + key + "' must be an integer");
    return static_cast<int>(d);
}
int req_int(const Object& o, const char* key) { return int_of(req_num(o, key), key); }

OptionType option_type(const std::string& s) {
    if (s == "call") return OptionType::Call;
    if (s == "put") return OptionType::Put;
    throw std::runtime_error("'type' must be 'call' or 'put'");
}
mcd::BarrierDirection direction(const std::string& s) {
    if (s == "up") return mcd::BarrierDirection::Up;
    if (s == "down") return mcd::BarrierDirection::Down;
    throw std::runtime_error("'direction' must be 'up' or 'down'");
}
mcd::BarrierKnock knock(const std::string& s) {
    if (s == "in") return mcd::BarrierKnock::In;
    if (s == "out") return mcd::BarrierKnock::Out;
    throw std::runtime_error("'knock' must be 'in' or 'out'");
}
mcd::StrikeStyle strike_style(const std::string& s, const char* key = "strike_style") {
    if (s == "fixed") return mcd::StrikeStyle::Fixed;
    if (s == "floating") return mcd::StrikeStyle::Floating;
    if (g_dialect.lambda) throw std::runtime_error(std::string("'") + key + "' must be 'fixed' or 'floating'");
    throw std::runtime_error("'strike_style'/'style' must be 'fixed' or 'floating'");
}

// The Lambda layer's variance-reduction toggles (infra/lambda/request.py:232-241).
pricers::McOptions lambda_options(const Object& req) {
    pricers::McOptions o;
    if (!g_dialect.lambda) return o;
    const Value* a = mcdjson::find(req, "antithetic");
    const Value* c = mcdjson::find(req, "control_variate");
    auto truthy = [](const Value* v) {
        if (!v) return false;
        if (v->type == Value::Type::Bool) return v->b;
        if (v->type == Value::Type::Number) return v->num != 0.0;
        if (v->type == Value::Type::String) return !v->str.empty();
        return false;
    };
    o.antithetic = truthy(a);
    o.control_variate = truthy(c);
    return o;
}
mcd::AverageStyle average_style(const std::string& s) {
    if (s == "arithmetic") return mcd::AverageStyle::Arithmetic;
    if (s == "geometric") return mcd::AverageStyle::Geometric;
    throw std::runtime_error("'average_style' must be 'arithmetic' or 'geometric'");
}
mcd::DigitalStyle digital_style(const std::string& s) {
    if (s == "cash_or_nothing") return mcd::DigitalStyle::CashOrNothing;
    if (s == "asset_or_nothing") return mcd::DigitalStyle::AssetOrNothing;
    throw std::runtime_error("'digital_style' must be 'cash_or_nothing' or 'asset_or_nothing'");
}

Object mc_json(double price, double se, std::uint64_t paths, std::uint64_t seed, double elapsed) {
    Object out;
    out.emplace_back("price", Value::number(price));
    out.emplace_back("standard_error", Value::number(se));
    out.emplace_back("ci_95_low", Value::number(price - kZ975 * se));
    out.emplace_back("ci_95_high", Value::number(price + kZ975 * se));
    out.emplace_back("path_count", Value::number(static_cast<double>(paths)));
    out.emplace_back("seed", Value::number(static_cast<double>(seed)));
    out.emplace_back("elapsed_seconds", Value::number(elapsed));
    out.emplace_back("paths_per_second", Value::number(elapsed > 0.0 ? static_cast<double>(paths) / elapsed : 0.0));
    return out;
}

Object analytic_json(double price, double elapsed) {
    Object out;
    out.emplace_back("price", Value::number(price));
    out.emplace_back("elapsed_seconds", Value::number(elapsed));
    return out;
}

Object qmc_json(double price, std::uint64_t paths, double elapsed) {
    Object out;
    out.emplace_back("price", Value::number(price));
    out.emplace_back("path_count", Value::number(static_cast<double>(paths)));
    out.emplace_back("elapsed_seconds", Value::number(elapsed));
    out.emplace_back("paths_per_second", Value::number(elapsed > 0.0 ? static_cast<double>(paths) / elapsed : 0.0));
    out.emplace_back("note", Value::string(g_dialect.lambda
                                               ? "Sobol QMC is deterministic: no standard_error/confidence interval "
                                                 "is reported. See docs/design/10-sobol-qmc.md sec.6."
                                               : "Sobol QMC is deterministic: no standard_error/confidence interval "
                                                 "is reported."));
    return out;
}

template <typename G>
void add_greek(Object& out, const char* name, const G& g) {
    out.emplace_back(name, Value::number(g.value));
    out.emplace_back(std::string(name) + "_se", Value::number(g.standard_error));
}

Object lr_json(const greeks::LrGreeks& g, double elapsed) {
    Object out;
    add_greek(out, "delta", g.delta);
    add_greek(out, "gamma", g.gamma);
    add_greek(out, "vega", g.vega);
    add_greek(out, "rho", g.rho);
    if (g.theta) add_greek(out, "theta", *g.theta);
    out.emplace_back("elapsed_seconds", Value::number(elapsed));
    return out;
}

Object pathwise_json(const greeks::PathwiseGreeks& g, double elapsed) {
    Object out;
    add_greek(out, "delta", g.delta);
    add_greek(out, "vega", g.vega);
    add_greek(out, "rho", g.rho);
    out.emplace_back("elapsed_seconds", Value::number(elapsed));
    return out;
}

// ---- batch requests -----------------------------------------------------------
struct Batch {
    const Object& req;
    size_t n = 1;
    explicit Batch(const Object& r) : req(r) {
        size_t len = 0;
        for (const auto& kv : req) {
            if (kv.second.type != Value::Type::Array) continue;
            if (kv.second.items.empty()) throw std::runtime_error("field '" + kv.first + "' is an empty array");
            if (len && kv.second.items.size() != len)
                throw std::runtime_error("batch arrays must all have the same length ('" + kv.first + "')");
            len = kv.second.items.size();
        }
        n = len ? len : 1;
    }
    const Value* at(const char* key, size_t i) const {
        const Value* v = mcdjson::find(req, key);
        if (!v) return nullptr;
        return v->type == Value::Type::Array ? &v->items[i] : v;
    }
    double num(const char* key, size_t i) const {
        const Value* v = at(key, i);
        if (!v) throw std::runtime_error(std::string("missing required field '") + key + "'");
        return as_number(*v, key);
    }
    double num(const char* key, size_t i, double def) const {
        const Value* v = at(key, i);
        return v ? as_number(*v, key) : def;
    }
    std::string str(const char* key, size_t i) const {
        const Value* v = at(key, i);
        if (!v) throw std::runtime_error(std::string("missing required field '") + key + "'");
        return as_string(*v, key);
    }
    bool flag(const char* key, size_t i) const {
        const Value* v = at(key, i);
        if (!v) return false;
        if (v->type != Value::Type::Bool) throw std::runtime_error(std::string("field '") + key + "' must be a boolean");
        return v->b;
    }
};

mcd_contract batch_contract(const Batch& b, size_t i) {
    mcd_contract c;
    std::memset(&c, 0, sizeof c);
    const std::string product = b.str("product", i);
    if (product == "european") c.product = MCD_PRODUCT_EUROPEAN;
    else if (product == "digital") c.product = MCD_PRODUCT_DIGITAL;
    else if (product == "asian") c.product = MCD_PRODUCT_ASIAN;
    else if (product == "barrier") c.product = MCD_PRODUCT_BARRIER;
    else if (product == "lookback") c.product = MCD_PRODUCT_LOOKBACK;
    else throw std::runtime_error("batch: unsupported 'product': '" + product + "'");
    c.type = option_type(b.str("type", i)) == OptionType::Call ? MCD_CALL : MCD_PUT;
    c.spot = b.num("spot", i);
    c.strike = c.product == MCD_PRODUCT_LOOKBACK ? b.num("strike", i, 0.0) : b.num("strike", i);
    c.rate = b.num("rate", i);
    c.carry_yield = b.num("carry_yield", i);
    c.vol = b.num("vol", i);
    c.time = b.num("time", i);
    c.path_count = count_of(b.num("path_count", i), "path_count");
    c.seed = count_of(b.num("seed", i), "seed");
    c.monitoring_points = 1;
    c.cash_amount = 1.0;
    if (c.product == MCD_PRODUCT_DIGITAL) {
        c.digital_style = digital_style(b.str("digital_style", i)) == mcd::DigitalStyle::CashOrNothing ? 0 : 1;
        c.cash_amount = b.num("cash_amount", i, 1.0);
    }
    if (c.product >= MCD_PRODUCT_ASIAN) c.monitoring_points = int_of(b.num("monitoring_points", i), "monitoring_points");
    if (c.product == MCD_PRODUCT_ASIAN) {
        c.strike_style = strike_style(b.str("strike_style", i)) == mcd::StrikeStyle::Fixed ? 0 : 1;
        c.average_style = average_style(b.str("average_style", i)) == mcd::AverageStyle::Arithmetic ? 0 : 1;
    }
    if (c.product == MCD_PRODUCT_LOOKBACK) c.strike_style = strike_style(b.str("style", i)) == mcd::StrikeStyle::Fixed ? 0 : 1;
    if (c.product == MCD_PRODUCT_BARRIER) {
        c.barrier = b.num("barrier", i);
        c.direction = direction(b.str("direction", i)) == mcd::BarrierDirection::Up ? MCD_UP : MCD_DOWN;
        c.knock = knock(b.str("knock", i)) == mcd::BarrierKnock::In ? MCD_IN : MCD_OUT;
        c.rebate = b.num("rebate", i, 0.0);
    }
    c.antithetic = b.flag("antithetic", i);
    c.control_variate = b.flag("control_variate", i);
    c.brownian_bridge = b.flag("brownian_bridge", i);
    return c;
}

mcd_ctx* shared_ctx() {
    static mcd_ctx* ctx = [] {
        mcd_ctx* c = nullptr;
        if (mcd_create(0, &c) != MCD_OK) throw std::runtime_error(std::string("mcd_create: ") + mcd_last_error(nullptr));
        return c;
    }();
    return ctx;
}

Value array_of(const std::vector<double>& v) {
    std::vector<Value> items;
    items.reserve(v.size());
    for (double x : v) items.push_back(Value::number(x));
    return Value::array(std::move(items));
}

Object handle_batch(const Object& req, bool with_greeks, int precision) {
    const Batch b(req);
    std::vector<mcd_contract> cs(b.n);
    for (size_t i = 0; i < b.n; ++i) cs[i] = batch_contract(b, i);
    mcd_ctx* ctx = shared_ctx();
    double total_paths = 0.0;
    for (const auto& c : cs) total_paths += static_cast<double>(c.path_count);
    Object out;
    out.emplace_back("count", Value::number(static_cast<double>(b.n)));
    if (!with_greeks) {
        std::vector<mcd_mc_result> r(b.n);
        auto [rc, elapsed] = timed([&] { return mcd_price_batch(ctx, cs.data(), cs.size(), precision, r.data()); });
        if (rc != MCD_OK) throw std::runtime_error(mcd_last_error(ctx));
        std::vector<double> price, se, lo, hi, paths, seeds;
        for (size_t i = 0; i < b.n; ++i) {
            price.push_back(r[i].price);
            se.push_back(r[i].standard_error);
            lo.push_back(r[i].price - kZ975 * r[i].standard_error);
            hi.push_back(r[i].price + kZ975 * r[i].standard_error);
            paths.push_back(static_cast<double>(r[i].path_count));
            seeds.push_back(static_cast<double>(cs[i].seed));
        }
        out.emplace_back("price", array_of(price));
        out.emplace_back("standard_error", array_of(se));
        out.emplace_back("ci_95_low", array_of(lo));
        out.emplace_back("ci_95_high", array_of(hi));
        out.emplace_back("path_count", array_of(paths));
        out.emplace_back("seed", array_of(seeds));
        out.emplace_back("elapsed_seconds", Value::number(elapsed));
        out.emplace_back("paths_per_second", Value::number(elapsed > 0.0 ? total_paths / elapsed : 0.0));
        return out;
    }
    const double spot_bump = opt_num(req, "spot_bump", 1e-4), vol_bump = opt_num(req, "vol_bump", 1e-4);
    std::vector<mcd_greeks_result> r(b.n);
    auto [rc, elapsed] = timed(
        [&] { return mcd_greeks_batch(ctx, cs.data(), cs.size(), spot_bump, vol_bump, precision, r.data()); });
    if (rc != MCD_OK) throw std::runtime_error(mcd_last_error(ctx));
    static const char* names[12] = {"price", "fd_delta", "fd_gamma", "fd_vega", "pathwise_delta", "pathwise_vega",
                                    "pathwise_rho", "lr_delta", "lr_gamma", "lr_vega", "lr_rho", "lr_theta"};
    for (int q = 0; q < 12; ++q) {
        std::vector<Value> val, se;
        for (size_t i = 0; i < b.n; ++i) {
            const mcd_greek& g = (&r[i].price)[q];
            const bool defined = (r[i].defined >> q) & 1u;
            val.push_back(defined ? Value::number(g.value) : Value::null());
            se.push_back(defined ? Value::number(g.standard_error) : Value::null());
        }
        out.emplace_back(names[q], Value::array(std::move(val)));
        out.emplace_back(std::string(names[q]) + "_se", Value::array(std::move(se)));
    }
    out.emplace_back("elapsed_seconds", Value::number(elapsed));
    out.emplace_back("paths_per_second", Value::number(elapsed > 0.0 ? total_paths / elapsed : 0.0));
    return out;
}

// ---- single requests (main.cpp:229-538) ---------------------------------------------
Object handle(const Object& req) {
    const std::string kind = opt_str(req, "request", "price");
    const std::string prec = opt_str(req, "precision", "fp64");
    if (prec != "fp64" && prec != "fp32") throw std::runtime_error("'precision' must be 'fp64' or 'fp32'");
    mcd::gpu::set_precision(prec == "fp32" ? mcd::gpu::Precision::FP32 : mcd::gpu::Precision::FP64);
    if (kind == "batch" || kind == "batch_greeks") return handle_batch(req, kind == "batch_greeks", prec == "fp32" ? 1 : 0);

    const std::string product = req_str(req, "product");
    if (product == "forward") {
        const double spot = req_num(req, "spot"), rate = req_num(req, "rate"), q = req_num(req, "carry_yield"),
                     t = req_num(req, "time");
        auto [v, s] = timed([&] { return pricers::forward_price(spot, rate, q, t); });
        return analytic_json(v, s);
    }
    if (product == "binomial_european" || product == "binomial_american") {
        const double spot = req_num(req, "spot"), k = req_num(req, "strike"), rate = req_num(req, "rate"),
                     q = req_num(req, "carry_yield"), vol = req_num(req, "vol"), t = req_num(req, "time");
        const OptionType type = option_type(req_str(req, "type"));
        const int steps = req_int(req, "steps");
        if (g_dialect.lambda && (steps < 1 || steps > 20000))
            throw std::runtime_error("'steps' must be between 1 and 20,000 on this demo endpoint");
        if (product == "binomial_american") {
            auto [v, s] = timed([&] { return pricers::crr_binomial_american(spot, k, rate, q, vol, t, steps, type); });
            return analytic_json(v, s);
        }
        auto [v, s] = timed([&] { return pricers::crr_binomial(spot, k, rate, q, vol, t, steps, type); });
        Object out = analytic_json(v.price, s);
        out.emplace_back("risk_neutral_probability", Value::number(v.risk_neutral_probability));
        out.emplace_back("up_factor", Value::number(v.up_factor));
        out.emplace_back("down_factor", Value::number(v.down_factor));
        return out;
    }
    if (product == "european") {
        const double spot = req_num(req, "spot"), k = req_num(req, "strike"), rate = req_num(req, "rate"),
                     q = req_num(req, "carry_yield"), vol = req_num(req, "vol"), t = req_num(req, "time");
        const OptionType type = option_type(req_str(req, "type"));
        if (kind == "greeks") {
            const auto n = req_paths(req);
            const auto seed = req_count(req, "seed");
            const auto bumps = greeks::default_bump_sizes(spot, vol, t);
            auto [g, s] = timed([&] { return greeks::finite_difference_european(spot, k, rate, q, vol, t, type, n, seed, bumps); });
            Object out;
            out.emplace_back("delta", Value::number(g.delta));
            out.emplace_back("gamma", Value::number(g.gamma));
            out.emplace_back("vega", Value::number(g.vega));
            out.emplace_back("theta", Value::number(g.theta));
            out.emplace_back("rho", Value::number(g.rho));
            out.emplace_back("elapsed_seconds", Value::number(s));
            return out;
        }
        if (kind == "lr_greeks") {
            const auto n = req_paths(req);
            const auto seed = req_count(req, "seed");
            auto [g, s] = timed([&] { return greeks::likelihood_ratio_european(spot, k, rate, q, vol, t, type, n, seed); });
            return lr_json(g, s);
        }
        if (kind == "pathwise_greeks") {
            const auto n = req_paths(req);
            const auto seed = req_count(req, "seed");
            auto [g, s] = timed([&] { return greeks::pathwise_european(spot, k, rate, q, vol, t, type, n, seed); });
            return pathwise_json(g, s);
        }
        if (kind == "qmc_sobol") {
            const auto n = req_paths(req);
            auto [r, s] = timed([&] { return pricers::qmc_sobol_european(spot, k, rate, q, vol, t, type, n); });
            return qmc_json(r.price, n, s);
        }
        const auto n = req_paths(req);
        const auto seed = req_count(req, "seed");
        const pricers::McOptions opts = lambda_options(req);
        auto [r, s] = timed([&] { return pricers::monte_carlo_european(spot, k, rate, q, vol, t, type, n, seed, opts); });
        Object out = mc_json(r.price, r.standard_error, r.path_count, seed, s);
        out.emplace_back("simd_enabled", Value::boolean(false));  // the NEON CPU path is not used
        return out;
    }
    if (product == "digital") {
        const double spot = req_num(req, "spot"), k = req_num(req, "strike"), rate = req_num(req, "rate"),
                     q = req_num(req, "carry_yield"), vol = req_num(req, "vol"), t = req_num(req, "time");
        const OptionType type = option_type(req_str(req, "type"));
        const auto style = digital_style(req_str(req, "digital_style"));
        const double cash = opt_num(req, "cash_amount", 1.0);
        const auto n = req_paths(req);
        const auto seed = req_count(req, "seed");
        if (kind == "lr_greeks") {
            auto [g, s] = timed([&] { return greeks::likelihood_ratio_digital(spot, k, rate, q, vol, t, type, style, cash, n, seed); });
            return lr_json(g, s);
        }
        auto [r, s] = timed([&] { return pricers::monte_carlo_digital(spot, k, rate, q, vol, t, type, style, cash, n, seed); });
        Object out = mc_json(r.price, r.standard_error, r.path_count, seed, s);
        out.emplace_back("simd_enabled", Value::boolean(false));
        return out;
    }
    if (product == "asian") {
        const double spot = req_num(req, "spot"), k = req_num(req, "strike"), rate = req_num(req, "rate"),
                     q = req_num(req, "carry_yield"), vol = req_num(req, "vol"), t = req_num(req, "time");
        const OptionType type = option_type(req_str(req, "type"));
        const auto ss = strike_style(req_str(req, "strike_style"));
        const auto as = average_style(req_str(req, "average_style"));
        const int m = req_int(req, "monitoring_points");
        const auto n = req_paths(req);
        if (kind == "qmc_sobol") {
            if (as != mcd::AverageStyle::Arithmetic)
                throw std::runtime_error(g_dialect.lambda ? "'qmc_sobol' asian only supports 'arithmetic' average_style "
                                                            "(docs/design/10-sobol-qmc.md sec.4)"
                                                          : "'qmc_sobol' asian only supports 'arithmetic' average_style");
            if (m < 1 || m > static_cast<int>(mcd::kSobolMaxDimensions))
                throw std::runtime_error("'monitoring_points' for 'qmc_sobol' asian must be between 1 and " +
                                         std::to_string(mcd::kSobolMaxDimensions) +
                                         (g_dialect.lambda ? " (docs/design/10-sobol-qmc.md sec.2/4: the "
                                                             "from-scratch-verified Sobol dimension budget)"
                                                           : ""));
            auto [r, s] = timed([&] { return pricers::qmc_sobol_asian(spot, k, rate, q, vol, t, type, ss, m, n); });
            return qmc_json(r.price, n, s);
        }
        const auto seed = req_count(req, "seed");
        if (kind == "pathwise_greeks") {
            auto [g, s] = timed([&] { return greeks::pathwise_asian(spot, k, rate, q, vol, t, type, ss, as, m, n, seed); });
            return pathwise_json(g, s);
        }
        const pricers::McOptions opts = lambda_options(req);
        auto [r, s] = timed([&] { return pricers::monte_carlo_asian(spot, k, rate, q, vol, t, type, ss, as, m, n, seed, opts); });
        return mc_json(r.price, r.standard_error, r.path_count, seed, s);
    }
    if (product == "barrier") {
        const double spot = req_num(req, "spot"), k = req_num(req, "strike"), h = req_num(req, "barrier"),
                     rate = req_num(req, "rate"), q = req_num(req, "carry_yield"), vol = req_num(req, "vol"),
                     t = req_num(req, "time");
        const OptionType type = option_type(req_str(req, "type"));
        const auto dir = direction(req_str(req, "direction"));
        const auto kn = knock(req_str(req, "knock"));
        const double rebate = opt_num(req, "rebate", 0.0);
        const int m = req_int(req, "monitoring_points");
        const auto n = req_paths(req);
        const auto seed = req_count(req, "seed");
        if (kind == "lr_greeks") {
            auto [g, s] = timed([&] { return greeks::likelihood_ratio_barrier(spot, k, h, rate, q, vol, t, type, dir, kn, rebate, m, n, seed); });
            return lr_json(g, s);
        }
        auto [r, s] = timed([&] { return pricers::monte_carlo_barrier(spot, k, h, rate, q, vol, t, type, dir, kn, rebate, m, n, seed); });
        return mc_json(r.price, r.standard_error, r.path_count, seed, s);
    }
    if (product == "lookback") {
        const double spot = req_num(req, "spot"), k = opt_num(req, "strike", 0.0), rate = req_num(req, "rate"),
                     q = req_num(req, "carry_yield"), vol = req_num(req, "vol"), t = req_num(req, "time");
        const OptionType type = option_type(req_str(req, "type"));
        const auto st = strike_style(req_str(req, "style"), "style");
        const int m = req_int(req, "monitoring_points");
        const auto n = req_paths(req);
        const auto seed = req_count(req, "seed");
        auto [r, s] = timed([&] { return pricers::monte_carlo_lookback(spot, k, rate, q, vol, t, type, st, m, n, seed); });
        return mc_json(r.price, r.standard_error, r.path_count, seed, s);
    }
    if (product == "american") {
        const double spot = req_num(req, "spot"), k = req_num(req, "strike"), rate = req_num(req, "rate"),
                     q = req_num(req, "carry_yield"), vol = req_num(req, "vol"), t = req_num(req, "time");
        const OptionType type = option_type(req_str(req, "type"));
        const int m = req_int(req, "monitoring_points");
        const auto n = req_paths(req);
        const auto seed = req_count(req, "seed");
        auto [r, s] = timed([&] { return pricers::monte_carlo_lsm_american(spot, k, rate, q, vol, t, type, m, n, seed); });
        return mc_json(r.price, r.standard_error, n, seed, s);
    }
    if (product == "heston") {
        const mcd::models::HestonParams p{req_num(req, "spot"), req_num(req, "rate"), req_num(req, "carry_yield"),
                                          req_num(req, "v0"),   req_num(req, "kappa"), req_num(req, "theta"),
                                          req_num(req, "xi"),   req_num(req, "rho"),   req_num(req, "time")};
        const double k = req_num(req, "strike");
        const OptionType type = option_type(req_str(req, "type"));
        if (kind == "semi_analytic") {
            auto [v, s] = timed([&] { return pricers::heston_semi_analytic(p, k, type); });
            return analytic_json(v, s);
        }
        const int m = req_int(req, "monitoring_points");
        const auto n = req_paths(req);
        const auto seed = req_count(req, "seed");
        auto [r, s] = timed([&] { return pricers::heston_qe_european(p, k, type, m, n, seed); });
        return mc_json(r.price, r.standard_error, r.path_count, seed, s);
    }
    throw std::runtime_error("unknown 'product': '" + product + "'");
}

}  // namespace

extern "C" char* mcd_shim_handle_request(const char* request, int dialect, uint64_t max_path_count, int* status) {
    g_dialect = Dialect{dialect == MCD_SHIM_DIALECT_LAMBDA, dialect == MCD_SHIM_DIALECT_LAMBDA ? max_path_count : 0};
    std::string body;
    int st = MCD_SHIM_OK;
    try {
        const Object req = mcdjson::parse_object(request ? request : "");
        // the CLI prints 10 significant digits; the Lambda layer returns
        // Python floats, i.e. every double exactly
        body = mcdjson::serialize(handle(req), g_dialect.lambda ? 17 : 10);
    } catch (const mcd::gpu::Error& e) {  // the device failed, not the request
        st = MCD_SHIM_INTERNAL_ERROR;
        Object err;
        err.emplace_back("error", Value::string(e.what()));
        body = mcdjson::serialize(err);
    } catch (const std::exception& e) {
        st = MCD_SHIM_REQUEST_ERROR;
        Object err;
        err.emplace_back("error", Value::string(e.what()));
        body = mcdjson::serialize(err);
    } catch (...) {  // nothing may unwind through the C boundary
        st = MCD_SHIM_INTERNAL_ERROR;
        body = "{\"error\":\"internal error\"}";
    }
    if (status) *status = st;
    char* out = static_cast<char*>(std::malloc(body.size() + 1));
    if (out) std::memcpy(out, body.c_str(), body.size() + 1);
    return out;
}

extern "C" void mcd_shim_free(char* p) { std::free(p); }
