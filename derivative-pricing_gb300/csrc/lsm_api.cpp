// lsm_api.cpp -- C ABI for the batched Longstaff-Schwartz engine (lsm.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "context.hpp"
#include "mlp_layout.hpp"
#include "lsm.hpp"
#include "lsm_mlp_dev.hpp"
#include "mcd_gpu.h"

using namespace mcdg;

namespace {

// Extension slots of Ctx::ext used by this module (Heston uses 0..3).
enum { kDev = 4, kChunkMap = 5, kStore = 6, kCf = 7, kReg = 8, kPartA = 9, kPartB = 10,
       kFinal = 11, kOut = 12, kNets = 13, kSnaps = 14, kSnapOk = 15, kAdamT = 16, kErr = 17,
       kGroupMap = 18, kGramPart = 19, kFeats = 20, kMomPart = 35, kFzDev = 36, kFzPart = 37,
       kFzOut = 38, kETab = 39, kCounters = 40, kPreS = 41, kPreCf = 42 };  // kPartB: group partials

// Concurrent chains of the backward pass (at most Ctx::kAuxStreams + 1):
// QR regression, learned regression.
constexpr int kLsmChains = 2;
constexpr int kLsmChainsLearned = 2;
constexpr double kLsmFirstChainShare = 0.5;
static_assert(kLsmChains <= Ctx::kAuxStreams + 1 && kLsmChainsLearned <= Ctx::kAuxStreams + 1,
              "one stream per chain");

struct LsmPlan {
    std::vector<LsmDev> dev;
    std::vector<uint32_t> chunk_contract;
    std::vector<uint32_t> group_contract;  // learned regression: group -> contract
    uint64_t store_elems = 0, cf_elems = 0, reg_rows = 0;
    uint32_t total_chunks = 0, total_groups = 0, total_folds = 0;
    int max_steps = 0;
};

int plan_lsm(Ctx& ctx, const mcd_lsm_contract* cs, size_t n, LsmPlan& p) {
    p = LsmPlan{};
    p.dev.resize(n);
    for (size_t i = 0; i < n; ++i) {
        const mcd_lsm_contract& c = cs[i];
        const double v[] = {c.spot, c.strike, c.rate, c.carry_yield, c.vol, c.time};
        for (double x : v)
            if (!std::isfinite(x)) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "lsm contract " + std::to_string(i) + ": non-finite parameter");
        if (!(c.spot > 0) || !(c.strike > 0) || !(c.vol > 0) || !(c.time > 0))
            return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "lsm contract " + std::to_string(i) + ": spot, strike, vol, time must be > 0");
        if (c.type != 0 && c.type != 1) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "type must be 0 (call) or 1 (put)");
        if (c.monitoring_points < 1 || c.monitoring_points > 100000)
            return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "monitoring_points must be 1..100000");
        if (c.path_count > (1ull << 40)) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "path_count too large");
        LsmDev& d = p.dev[i];
        std::memset(&d, 0, sizeof d);
        const double dt = c.time / static_cast<double>(c.monitoring_points);
        d.spot = c.spot;
        d.strike = c.strike;
        d.disc = std::exp(-c.rate * dt);
        d.drift = (c.rate - c.carry_yield - 0.5 * c.vol * c.vol) * dt;
        d.vs = c.vol * std::sqrt(dt);
        const double phi = c.type == 0 ? 1.0 : -1.0;
        const double x = phi * (c.spot - c.strike);
        d.inception = x > 0.0 ? x : 0.0;
        d.strike_f = static_cast<float>(c.strike);
        d.inv_strike_f = static_cast<float>(1.0 / c.strike);
        d.disc_f = static_cast<float>(d.disc);
        d.phi_f = c.type == 0 ? 1.0f : -1.0f;
        d.seed = c.seed;
        d.path_count = c.path_count;
        d.n_steps = c.monitoring_points;
        d.type = c.type;
        d.s_offset = p.store_elems;
        d.cf_offset = p.cf_elems;
        d.reg_offset = static_cast<uint32_t>(p.reg_rows);
        const uint64_t chunks = (c.path_count + kLsmChunk - 1) / kLsmChunk;
        if (p.total_chunks + chunks > 0x7FFFFFFFull) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "batch too large");
        d.chunk_begin = p.total_chunks;
        d.n_chunks = static_cast<uint32_t>(chunks);
        for (uint64_t q = 0; q < chunks; ++q) p.chunk_contract.push_back(static_cast<uint32_t>(i));
        p.total_chunks += static_cast<uint32_t>(chunks);
        p.store_elems += static_cast<uint64_t>(c.monitoring_points) * c.path_count;
        p.cf_elems += c.path_count;
        p.reg_rows += static_cast<uint64_t>(c.monitoring_points) + 1;
        // learned regression: at most kLsmMaxGroups CTAs per contract, each
        // of at least kLsmMinGroupChunks chunks (a CTA's set-up -- clearing
        // and writing out its bin moments -- is then a small share of its
        // work); the moments are exact integers, so the price does not depend
        // on the split
        const uint64_t per_group =
            std::max<uint64_t>((chunks + kLsmMaxGroups - 1) / kLsmMaxGroups, kLsmMinGroupChunks);
        const uint32_t groups = static_cast<uint32_t>((chunks + per_group - 1) / per_group);
        d.group_chunks = static_cast<uint32_t>(per_group);
        d.group_begin = p.total_groups;
        d.n_groups = groups;
        for (uint32_t g = 0; g < groups; ++g) p.group_contract.push_back(static_cast<uint32_t>(i));
        p.total_groups += groups;
        // QR regression: the chunk sums are folded in groups of at least
        // kLsmMinFoldChunks chunks (at most kLsmMaxFolds per contract), then
        // the groups (lsm.cu, publish_and_fold)
        const uint64_t per_fold =
            std::max<uint64_t>((chunks + kLsmMaxFolds - 1) / kLsmMaxFolds, kLsmMinFoldChunks);
        const uint32_t folds = static_cast<uint32_t>((chunks + per_fold - 1) / per_fold);
        d.fold_chunks = static_cast<uint32_t>(per_fold);
        d.fold_begin = p.total_folds;
        d.n_folds = folds;
        p.total_folds += folds;
        p.max_steps = std::max(p.max_steps, c.monitoring_points);
    }
    return MCD_OK;
}

// Runs a planned batch with stored paths.  mlp = false: Laguerre QR
// regression, fitted (the table stays in kReg).  mlp = true: learned
// regression, fitted, or (frozen) replaying the networks in frozen_nets, one
// kParamStride block per (contract, date) row.  Frozen QR policies are
// replayed by the streaming kernel instead (frozen_run).
int upload_and_run(Ctx& ctx, const LsmPlan& p, int precision, bool frozen, std::vector<double>& out,
                   bool mlp = false, const std::vector<float>* frozen_nets = nullptr,
                   const std::vector<int>* frozen_ok = nullptr) {
    const size_t n = p.dev.size();
    const size_t elem = precision == 0 ? sizeof(double) : sizeof(float);
    if (mlp && !frozen)  // training samples paths; the bin moments of one CTA are exact up to 2^23 paths
        for (const LsmDev& d : p.dev) {
            if (d.path_count == 0)
                return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "learned regression: path_count must be >= 1");
            if (static_cast<uint64_t>(d.group_chunks) * kLsmChunk > (1ull << 23))
                return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "learned regression: path_count must be <= 2^31");
        }
    int rc = ctx.reserve(ctx.ext[kDev], sizeof(LsmDev) * n, "lsm contracts");
    if (!rc) rc = ctx.reserve(ctx.ext[kChunkMap], sizeof(uint32_t) * std::max<size_t>(p.total_chunks, 1), "lsm chunk map");
    if (!rc) rc = ctx.reserve(ctx.ext[kStore], elem * std::max<uint64_t>(p.store_elems, 1), "lsm path store");
    if (!rc) rc = ctx.reserve(ctx.ext[kCf], sizeof(double) * std::max<uint64_t>(p.cf_elems, 1), "lsm cash flows");
    if (!rc) rc = ctx.reserve(ctx.ext[kReg], sizeof(LsmReg) * p.reg_rows, "lsm regression table");
    if (!rc) rc = ctx.reserve(ctx.ext[kPartA], sizeof(LsmPartial) * std::max<size_t>(p.total_chunks, 1), "lsm partials");
    if (!rc) rc = ctx.reserve(ctx.ext[kPartB], sizeof(LsmPartial) * std::max<size_t>(p.total_folds, 1), "lsm group partials");
    if (!rc) rc = ctx.reserve(ctx.ext[kFinal], sizeof(Welford) * std::max<size_t>(p.total_chunks, 1), "lsm final partials");
    if (!rc) rc = ctx.reserve(ctx.ext[kOut], sizeof(double) * 6 * n, "lsm results");
    const size_t n_counters = 2 * n + 2 * static_cast<size_t>(p.total_folds) + static_cast<size_t>(p.max_steps) + 1;
    if (!rc) rc = ctx.reserve(ctx.ext[kCounters], sizeof(uint32_t) * n_counters, "lsm chunk counters");
    if (!rc && mlp) {
        rc = ctx.reserve(ctx.ext[kNets], sizeof(float) * 3 * mlp::kParamStride * n, "mlp networks");
        if (!rc) rc = ctx.reserve(ctx.ext[kSnaps], sizeof(float) * mlp::kParamStride * p.reg_rows, "mlp snapshots");
        if (!rc) rc = ctx.reserve(ctx.ext[kSnapOk], sizeof(int) * p.reg_rows, "mlp snapshot flags");
        if (!rc) rc = ctx.reserve(ctx.ext[kAdamT], sizeof(int) * n, "mlp adam steps");
        const size_t pre = static_cast<size_t>(std::max(ctx.mlp_steps_first, 1)) * 128 * n;
        if (!rc && !frozen) rc = ctx.reserve(ctx.ext[kPreS], sizeof(double) * pre, "mlp training samples");
        if (!rc && !frozen) rc = ctx.reserve(ctx.ext[kPreCf], sizeof(double) * pre, "mlp training cash flows");
        if (!rc) rc = ctx.reserve(ctx.ext[kErr], 256, "mlp error word");
        if (!rc) rc = ctx.reserve(ctx.ext[kGroupMap], sizeof(uint32_t) * std::max<uint32_t>(p.total_groups, 1), "mlp group map");
        if (!rc) rc = ctx.reserve(ctx.ext[kGramPart], sizeof(float) * kGramPacked * kNodeSlices * n, "mlp gram partials");
        if (!rc) rc = ctx.reserve(ctx.ext[kFeats], sizeof(float) * 64 * kNodes * p.reg_rows, "mlp feature tables");
        if (!rc) rc = ctx.reserve(ctx.ext[kETab], sizeof(float) * kNodes * n, "mlp continuation tables");
        if (!rc)
            rc = ctx.reserve(ctx.ext[kMomPart], sizeof(unsigned long long) * kMoments * kNodes *
                                                     std::max<uint32_t>(p.total_groups, 1), "mlp bin moments");
        if (!rc) {
            cudaError_t pe = mlp_prepare();
            if (pe != cudaSuccess) rc = ctx.cuda_fail(pe, "mlp shared memory opt-in");
        }
    }
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(ctx.ext[kDev].ptr, p.dev.data(), sizeof(LsmDev) * n, cudaMemcpyHostToDevice, ctx.stream);
    if (e == cudaSuccess && p.total_chunks)
        e = cudaMemcpyAsync(ctx.ext[kChunkMap].ptr, p.chunk_contract.data(), sizeof(uint32_t) * p.total_chunks,
                            cudaMemcpyHostToDevice, ctx.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx.ext[kReg].ptr, 0, sizeof(LsmReg) * p.reg_rows, ctx.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx.ext[kCounters].ptr, 0, sizeof(uint32_t) * n_counters, ctx.stream);
    if (e == cudaSuccess && mlp) {
        e = cudaMemsetAsync(ctx.ext[kErr].ptr, 0, 256, ctx.stream);
        if (e == cudaSuccess && p.total_groups)
            e = cudaMemcpyAsync(ctx.ext[kGroupMap].ptr, p.group_contract.data(), sizeof(uint32_t) * p.total_groups,
                                cudaMemcpyHostToDevice, ctx.stream);
        if (e == cudaSuccess) {
            if (frozen_nets && frozen_ok) {
                e = cudaMemcpyAsync(ctx.ext[kSnaps].ptr, frozen_nets->data(), sizeof(float) * frozen_nets->size(),
                                    cudaMemcpyHostToDevice, ctx.stream);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(ctx.ext[kSnapOk].ptr, frozen_ok->data(), sizeof(int) * frozen_ok->size(),
                                        cudaMemcpyHostToDevice, ctx.stream);
            } else {
                e = cudaMemsetAsync(ctx.ext[kSnapOk].ptr, 0, sizeof(int) * p.reg_rows, ctx.stream);
            }
        }
    }
    if (e != cudaSuccess) return ctx.cuda_fail(e, "lsm upload");
    const MlpConfig cfg{ctx.mlp_steps_first, ctx.mlp_steps, ctx.mlp_lr_first, ctx.mlp_lr};

    // Capture forward pass + every backward iteration + finish into one graph.
    // The contracts run as up to kLsmChains independent chains (contiguous
    // ranges of about equal chunk counts), each captured on its own stream: a
    // date ends with a tail of little parallelism -- the QR pass's last chunk
    // folds and per-contract solve, the learned fit's Gram slices and
    // per-contract solve -- and another chain's work fills the GPU meanwhile.
    // Chains share no data but the QR second-pass counters (see
    // launch_lsm_iteration) and the learned kernels' error word; a price does
    // not depend on the number of chains.
    struct Chain {
        uint32_t chunk_first = 0, chunk_count = 0, g_first = 0, g_end = 0;
        int c_first = 0, c_end = 0, max_steps = 0;
    };
    std::vector<Chain> chains;
    {
        int rc2 = ctx.ensure_aux();
        if (rc2) return rc2;
        const int want = static_cast<int>(std::min<size_t>(n, static_cast<size_t>(mlp ? kLsmChainsLearned : kLsmChains)));
        size_t ci = 0;
        for (int j = 0; j < want && ci < n; ++j) {
            // chain 0 starts first (the others' forward simulations follow its
            // own) and takes kLsmFirstChainShare of the chunks; the rest split
            // the remainder evenly
            const double bound = want == 1 ? 1.0
                                            : kLsmFirstChainShare + (1.0 - kLsmFirstChainShare) * j / (want - 1);
            const uint64_t target = static_cast<uint64_t>(static_cast<double>(p.total_chunks) * bound);
            Chain ch;
            ch.chunk_first = p.dev[ci].chunk_begin;
            ch.g_first = ch.g_end = p.dev[ci].group_begin;
            ch.c_first = ch.c_end = static_cast<int>(ci);
            while (ci < n && (j == want - 1 || ch.chunk_first + ch.chunk_count < target || ch.chunk_count == 0)) {
                ch.chunk_count += p.dev[ci].n_chunks;
                ch.g_end = p.dev[ci].group_begin + p.dev[ci].n_groups;
                ch.max_steps = std::max(ch.max_steps, p.dev[ci].n_steps);
                ch.c_end = static_cast<int>(++ci);
            }
            chains.push_back(ch);
        }
    }
    cudaGetLastError();
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "lsm begin capture");
    const LsmDev* d_dev = static_cast<const LsmDev*>(ctx.ext[kDev].ptr);
    const uint32_t* d_map = static_cast<const uint32_t*>(ctx.ext[kChunkMap].ptr);
    // The chains start one after another: chain j+1's forward simulation
    // (which fills the GPU) follows chain j's, and so overlaps chain j's first
    // backward steps -- for the learned regression, its training, which runs
    // one CTA per contract.
    cudaError_t le = cudaSuccess;
    // The learned regression's first training runs beside each chain's
    // forward simulation, on a stream of its own (aux_stream[chains - 1 + j]
    // for chain j); the chain's first fit waits for it (ev_train[j]).
    const bool side_training = mlp && !frozen;
    static_assert(2 * kLsmChainsLearned - 1 <= Ctx::kAuxStreams, "a training stream per learned chain");
    if (side_training) {
        le = cudaEventRecord(ctx.ev_fork, ctx.stream);
        for (size_t j = 0; j < chains.size() && le == cudaSuccess; ++j) {
            const Chain& ch = chains[j];
            cudaStream_t ts = ctx.aux_stream[chains.size() - 1 + j];
            le = cudaStreamWaitEvent(ts, ctx.ev_fork, 0);
            if (le == cudaSuccess)
                le = launch_lsm_mlp_first_training(precision, d_dev, ch.c_first, ch.c_end, ch.max_steps,
                                                   static_cast<float*>(ctx.ext[kNets].ptr),
                                                   static_cast<float*>(ctx.ext[kSnaps].ptr),
                                                   static_cast<int*>(ctx.ext[kSnapOk].ptr),
                                                   static_cast<int*>(ctx.ext[kAdamT].ptr),
                                                   static_cast<float*>(ctx.ext[kFeats].ptr),
                                                   static_cast<double*>(ctx.ext[kPreS].ptr),
                                                   static_cast<double*>(ctx.ext[kPreCf].ptr), cfg,
                                                   static_cast<uint32_t*>(ctx.ext[kErr].ptr), ts);
            if (le == cudaSuccess) le = cudaEventRecord(ctx.ev_train[j], ts);
        }
    }
    for (size_t j = 0; j < chains.size() && le == cudaSuccess; ++j) {
        const Chain& ch = chains[j];
        cudaStream_t cs = j == 0 ? ctx.stream : ctx.aux_stream[j - 1];
        if (j > 0) le = cudaStreamWaitEvent(cs, ctx.ev_stage[j - 1], 0);
        if (le == cudaSuccess)
            le = launch_lsm_forward(precision, d_dev, static_cast<int>(n), d_map, ch.chunk_first, ch.chunk_count,
                                    ctx.ext[kStore].ptr, cs);
        if (le == cudaSuccess && j + 1 < chains.size()) le = cudaEventRecord(ctx.ev_stage[j], cs);
        for (int k = 0; k < ch.max_steps && le == cudaSuccess; ++k) {
            if (mlp)
                le = launch_lsm_mlp_iteration(precision, k, !frozen, d_dev, ch.c_first, ch.c_end, ch.max_steps,
                                              static_cast<const uint32_t*>(ctx.ext[kGroupMap].ptr), ch.g_first,
                                              ch.g_end, ctx.ext[kStore].ptr, static_cast<double*>(ctx.ext[kCf].ptr),
                                              static_cast<float*>(ctx.ext[kNets].ptr),
                                              static_cast<float*>(ctx.ext[kSnaps].ptr),
                                              static_cast<int*>(ctx.ext[kSnapOk].ptr),
                                              static_cast<int*>(ctx.ext[kAdamT].ptr),
                                              static_cast<float*>(ctx.ext[kGramPart].ptr),
                                              static_cast<float*>(ctx.ext[kFeats].ptr),
                                              static_cast<float*>(ctx.ext[kETab].ptr),
                                              static_cast<unsigned long long*>(ctx.ext[kMomPart].ptr), cfg,
                                              static_cast<Welford*>(ctx.ext[kFinal].ptr),
                                              side_training ? ctx.ev_train[j] : nullptr,
                                              static_cast<uint32_t*>(ctx.ext[kErr].ptr), cs);
            else
                le = launch_lsm_iteration(precision, k, d_dev, static_cast<int>(n), d_map, ch.chunk_first,
                                          ch.chunk_count, p.total_folds, ctx.ext[kStore].ptr,
                                          static_cast<double*>(ctx.ext[kCf].ptr),
                                          static_cast<LsmReg*>(ctx.ext[kReg].ptr),
                                          static_cast<LsmPartial*>(ctx.ext[kPartA].ptr),
                                          static_cast<LsmPartial*>(ctx.ext[kPartB].ptr),
                                          static_cast<Welford*>(ctx.ext[kFinal].ptr),
                                          static_cast<uint32_t*>(ctx.ext[kCounters].ptr), cs);
        }
        if (j > 0 && le == cudaSuccess) le = cudaEventRecord(ctx.ev_join[j - 1], cs);
    }
    for (size_t j = 1; j < chains.size() && le == cudaSuccess; ++j)
        le = cudaStreamWaitEvent(ctx.stream, ctx.ev_join[j - 1], 0);
    if (le == cudaSuccess)
        le = launch_lsm_finish(d_dev, static_cast<int>(n), static_cast<const Welford*>(ctx.ext[kFinal].ptr),
                               static_cast<double*>(ctx.ext[kOut].ptr), ctx.stream);
    e = cudaStreamEndCapture(ctx.stream, &graph);
    if (le != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return ctx.cuda_fail(le, "lsm capture");
    }
    if (e != cudaSuccess) return ctx.cuda_fail(e, "lsm end capture");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "lsm instantiate");
    int pair = -1;
    rc = ctx.record_start(ctx.stream, &pair);
    if (!rc) {
        e = cudaGraphLaunch(exec, ctx.stream);
        if (e != cudaSuccess) rc = ctx.cuda_fail(e, "lsm graph launch");
    }
    if (!rc) rc = ctx.record_stop(ctx.stream, pair);
    out.assign(6 * n, 0.0);
    if (!rc) {
        e = cudaMemcpyAsync(out.data(), ctx.ext[kOut].ptr, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, ctx.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx.stream);
        if (e != cudaSuccess) rc = ctx.cuda_fail(e, "lsm execution");
    }
    cudaGraphExecDestroy(exec);
    ctx.collect_timing(false);
    if (!rc && mlp) {
        uint32_t werr = 0;
        e = cudaMemcpy(&werr, ctx.ext[kErr].ptr, sizeof werr, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return ctx.cuda_fail(e, "mlp error word");
        if (werr != 0)
            return ctx.fail(MCD_ERR_TIMEOUT, "tensor-core wait gave up (code " + std::to_string(werr) + ")");
    }
    return rc;
}

int lsm_batch(Ctx& ctx, const mcd_lsm_contract* cs, size_t n, int precision, int regression,
              mcd_lsm_result* results, std::vector<LsmReg>* reg_out) {
    if (precision != 0 && precision != 1) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    if (regression != MCD_LSM_QR && regression != MCD_LSM_MLP)
        return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "regression must be MCD_LSM_QR or MCD_LSM_MLP");
    if (n == 0) return MCD_OK;
    if (!cs || !results) return ctx.fail(MCD_ERR_INVALID_ARGUMENT, "null array");
    LsmPlan p;
    int rc = plan_lsm(ctx, cs, n, p);
    if (rc) return rc;
    std::vector<double> out;
    const bool mlp = regression == MCD_LSM_MLP;
    rc = upload_and_run(ctx, p, precision, false, out, mlp);
    if (rc) return rc;
    std::vector<int> ok;
    if (mlp) {
        ok.resize(p.reg_rows);
        cudaError_t e = cudaMemcpy(ok.data(), ctx.ext[kSnapOk].ptr, sizeof(int) * p.reg_rows, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return ctx.cuda_fail(e, "mlp snapshot flags");
        ctx.mlp_reg_offset.resize(n);
        ctx.mlp_steps_of.resize(n);
        for (size_t i = 0; i < n; ++i) {
            ctx.mlp_reg_offset[i] = p.dev[i].reg_offset;
            ctx.mlp_steps_of[i] = p.dev[i].n_steps;
        }
    }
    std::vector<size_t> fallback;
    for (size_t i = 0; i < n; ++i) {
        results[i].price = out[6 * i];
        results[i].standard_error = out[6 * i + 1];
        results[i].path_count = static_cast<uint64_t>(out[6 * i + 2]);
        results[i].exercise_at_inception = out[6 * i + 3] != 0.0 ? 1 : 0;
        results[i].reserved = 0;
        if (mlp) {
            // A date whose training ended with non-finite weights: the network
            // is not trusted and the contract is priced by the QR regression.
            const int nd = p.dev[i].n_steps;
            for (int d = 1; d < nd; ++d)
                if (ok[p.dev[i].reg_offset + d] == 0) {
                    fallback.push_back(i);
                    break;
                }
        }
    }
    for (size_t i : fallback) {
        mcd_lsm_result r{};
        rc = lsm_batch(ctx, &cs[i], 1, precision, MCD_LSM_QR, &r, nullptr);
        if (rc) return rc;
        r.reserved = 1;  // priced by the QR fallback
        results[i] = r;
    }
    if (reg_out && !mlp) {
        reg_out->resize(p.reg_rows);
        cudaError_t e = cudaMemcpy(reg_out->data(), ctx.ext[kReg].ptr, sizeof(LsmReg) * p.reg_rows,
                                   cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return ctx.cuda_fail(e, "lsm policy copy");
    }
    return MCD_OK;
}

// One scenario's inputs: the GBM step constants of `vol` in the order of
// plan_lsm (src/models/gbm.cpp:8-10), plus the FP32 kernel's copies.
FrozenScenario scenario(double spot, const mcd_lsm_contract& c, double vol) {
    const double dt = c.time / static_cast<double>(c.monitoring_points);
    FrozenScenario s{};
    s.spot = spot;
    s.drift = (c.rate - c.carry_yield - 0.5 * vol * vol) * dt;
    s.vs = vol * std::sqrt(dt);
    s.spot_f = static_cast<float>(spot);
    s.mu_f = static_cast<float>(s.drift);
    s.sg_f = static_cast<float>(s.vs);
    return s;
}

// Scenarios base, spot +/- hs, vol +/- hv (hs = hv = 0: the base alone).
// The kernel shares the base's growth factors with the two spot scenarios,
// so those must keep the base volatility.
FrozenDev frozen_dev(const mcd_lsm_contract& c, double hs, double hv) {
    FrozenDev f{};
    f.sc[0] = scenario(c.spot, c, c.vol);
    f.sc[1] = scenario(c.spot + hs, c, c.vol);
    f.sc[2] = scenario(c.spot - hs, c, c.vol);
    f.sc[3] = scenario(c.spot, c, c.vol + hv);
    f.sc[4] = scenario(c.spot, c, c.vol - hv);
    f.inv_2hs = hs > 0.0 ? 0.5 / hs : 0.0;
    f.inv_hs2 = hs > 0.0 ? 1.0 / (hs * hs) : 0.0;
    f.inv_2hv = hv > 0.0 ? 0.5 / hv : 0.0;
    f.inv_2hs_f = static_cast<float>(f.inv_2hs);
    f.inv_hs2_f = static_cast<float>(f.inv_hs2);
    f.inv_2hv_f = static_cast<float>(f.inv_2hv);
    return f;
}

// Streams the planned contracts against the regression table in kReg
// (uploaded from `reg` when given, else left there by a fit on this
// context).  out: n x outputs x {mean, se, count}.
int frozen_run(Ctx& ctx, const LsmPlan& p, const std::vector<FrozenDev>& fz, int precision, int n_scenarios,
               const std::vector<LsmReg>* reg, std::vector<double>& out) {
    const size_t n = p.dev.size();
    const int nw = n_scenarios == 1 ? 1 : kFrozenOutputs;
    int rc = ctx.reserve(ctx.ext[kDev], sizeof(LsmDev) * n, "lsm contracts");
    if (!rc) rc = ctx.reserve(ctx.ext[kChunkMap], sizeof(uint32_t) * std::max<size_t>(p.total_chunks, 1), "lsm chunk map");
    if (!rc) rc = ctx.reserve(ctx.ext[kReg], sizeof(LsmReg) * p.reg_rows, "lsm regression table");
    if (!rc) rc = ctx.reserve(ctx.ext[kFzDev], sizeof(FrozenDev) * n, "frozen scenarios");
    if (!rc) rc = ctx.reserve(ctx.ext[kFzPart], sizeof(Welford) * nw * std::max<size_t>(p.total_chunks, 1), "frozen partials");
    if (!rc) rc = ctx.reserve(ctx.ext[kFzOut], sizeof(double) * 3 * nw * n, "frozen results");
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(ctx.ext[kDev].ptr, p.dev.data(), sizeof(LsmDev) * n, cudaMemcpyHostToDevice, ctx.stream);
    if (e == cudaSuccess && p.total_chunks)
        e = cudaMemcpyAsync(ctx.ext[kChunkMap].ptr, p.chunk_contract.data(), sizeof(uint32_t) * p.total_chunks,
                            cudaMemcpyHostToDevice, ctx.stream);
    if (e == cudaSuccess && reg)
        e = cudaMemcpyAsync(ctx.ext[kReg].ptr, reg->data(), sizeof(LsmReg) * p.reg_rows, cudaMemcpyHostToDevice,
                            ctx.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx.ext[kFzDev].ptr, fz.data(), sizeof(FrozenDev) * n, cudaMemcpyHostToDevice, ctx.stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "frozen upload");
    int pair = -1;
    rc = ctx.record_start(ctx.stream, &pair);
    if (rc) return rc;
    e = launch_lsm_frozen(precision, n_scenarios, static_cast<const LsmDev*>(ctx.ext[kDev].ptr),
                          static_cast<const FrozenDev*>(ctx.ext[kFzDev].ptr), static_cast<int>(n),
                          static_cast<const uint32_t*>(ctx.ext[kChunkMap].ptr), p.total_chunks,
                          static_cast<const LsmReg*>(ctx.ext[kReg].ptr), static_cast<Welford*>(ctx.ext[kFzPart].ptr),
                          static_cast<double*>(ctx.ext[kFzOut].ptr), ctx.stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "frozen launch");
    rc = ctx.record_stop(ctx.stream, pair);
    if (rc) return rc;
    out.assign(static_cast<size_t>(3) * nw * n, 0.0);
    e = cudaMemcpyAsync(out.data(), ctx.ext[kFzOut].ptr, sizeof(double) * out.size(), cudaMemcpyDeviceToHost, ctx.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx.stream);
    if (e != cudaSuccess) return ctx.cuda_fail(e, "frozen execution");
    ctx.collect_timing(false);
    return MCD_OK;
}

// The policy table of one contract from the ABI's coefficient layout.
std::vector<LsmReg> policy_table(const LsmPlan& p, int monitoring_points, const double* coefficients,
                                 const uint8_t* has) {
    std::vector<LsmReg> reg(p.reg_rows);
    std::memset(reg.data(), 0, sizeof(LsmReg) * reg.size());
    for (int d = 1; d < monitoring_points; ++d) {
        if (!has[d]) continue;
        reg[d].has = 1;
        for (int b = 0; b < 4; ++b) {
            reg[d].gamma[b] = coefficients[4 * d + b];
            reg[d].gamma_f[b] = static_cast<float>(coefficients[4 * d + b]);
        }
        laguerre_poly(reg[d].gamma, reg[d].poly_f);
    }
    return reg;
}

double intrinsic_host(double s, double k, int type) {
    const double x = (type == 0 ? 1.0 : -1.0) * (s - k);
    return x > 0.0 ? x : 0.0;
}

// Greeks of contract i from the five-scenario results (frozen inception
// decision applied as src/pricers/lsm.cpp:206-212 does per replay).
void assemble_greeks(const mcd_lsm_contract& c, double hs, double hv, bool inception, const double* r,
                     mcd_american_greeks& g) {
    double price[kFrozenScenarios];
    const double spots[kFrozenScenarios] = {c.spot, c.spot + hs, c.spot - hs, c.spot, c.spot};
    for (int q = 0; q < kFrozenScenarios; ++q)
        price[q] = inception ? intrinsic_host(spots[q], c.strike, c.type) : r[3 * q];
    std::memset(&g, 0, sizeof g);
    g.price = {price[0], inception ? 0.0 : r[1]};
    g.delta = {(price[1] - price[2]) / (2.0 * hs), inception ? 0.0 : r[3 * 5 + 1]};
    g.gamma = {(price[1] - 2.0 * price[0] + price[2]) / (hs * hs), inception ? 0.0 : r[3 * 6 + 1]};
    g.vega = {(price[3] - price[4]) / (2.0 * hv), inception ? 0.0 : r[3 * 7 + 1]};
    for (int q = 0; q < 4; ++q) g.scenario[q] = price[q + 1];
    g.spot_bump = hs;
    g.vol_bump = hv;
    g.path_count = static_cast<uint64_t>(r[2]);
    g.exercise_at_inception = inception ? 1 : 0;
}

}  // namespace

extern "C" {

int mcd_lsm_american(mcd_ctx* handle, double spot, double strike, double rate, double carry_yield,
                     double vol, double time, int type, int monitoring_points,
                     uint64_t path_count, uint64_t seed, int precision, int regression,
                     mcd_lsm_result* out, double* coefficients, uint8_t* has_coefficients) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (!out) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "out must not be NULL");
    const mcd_lsm_contract c{spot, strike, rate, carry_yield, vol, time, type, monitoring_points,
                             path_count, seed};
    std::vector<LsmReg> reg;
    const bool want_policy = coefficients || has_coefficients;
    const int rc = lsm_batch(*ctx, &c, 1, precision, regression, out,
                             (want_policy && regression == MCD_LSM_QR) ? &reg : nullptr);
    if (rc) return rc;
    if (want_policy && regression == MCD_LSM_QR) {
        for (int d = 0; d <= monitoring_points; ++d) {
            const bool has = reg[d].has == 1;
            if (has_coefficients) has_coefficients[d] = has ? 1 : 0;
            if (coefficients)
                for (int b = 0; b < 4; ++b) coefficients[4 * d + b] = has ? reg[d].gamma[b] : 0.0;
        }
    }
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_lsm_reprice_frozen(mcd_ctx* handle, double spot, double strike, double rate,
                           double carry_yield, double vol, double time, int type,
                           int monitoring_points, uint64_t path_count, uint64_t seed,
                           const double* coefficients, const uint8_t* has_coefficients,
                           int exercise_at_inception, int precision, double* price) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (!coefficients || !has_coefficients || !price) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "null argument");
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    const mcd_lsm_contract c{spot, strike, rate, carry_yield, vol, time, type, monitoring_points,
                             path_count, seed};
    LsmPlan p;
    int rc = plan_lsm(*ctx, &c, 1, p);
    if (rc) return rc;
    const std::vector<LsmReg> reg = policy_table(p, monitoring_points, coefficients, has_coefficients);
    const std::vector<FrozenDev> fz{frozen_dev(c, 0.0, 0.0)};
    std::vector<double> out;
    rc = frozen_run(*ctx, p, fz, precision, 1, &reg, out);
    if (rc) return rc;
    // Frozen inception decision (src/pricers/lsm.cpp:206-212): the base run's
    // choice is replayed; otherwise the price is the path average itself.
    *price = exercise_at_inception ? intrinsic_host(spot, strike, type) : out[0];
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_lsm_frozen_greeks(mcd_ctx* handle, double spot, double strike, double rate, double carry_yield,
                          double vol, double time, int type, int monitoring_points, uint64_t path_count,
                          uint64_t seed, const double* coefficients, const uint8_t* has_coefficients,
                          int exercise_at_inception, double spot_bump, double vol_bump, int precision,
                          mcd_american_greeks* out) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (!coefficients || !has_coefficients || !out) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "null argument");
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    if (!(spot_bump > 0.0 && spot_bump < spot) || !(vol_bump > 0.0 && vol_bump < vol))
        return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "bumps must satisfy 0 < spot_bump < spot and 0 < vol_bump < vol");
    const mcd_lsm_contract c{spot, strike, rate, carry_yield, vol, time, type, monitoring_points,
                             path_count, seed};
    LsmPlan p;
    int rc = plan_lsm(*ctx, &c, 1, p);
    if (rc) return rc;
    const std::vector<LsmReg> reg = policy_table(p, monitoring_points, coefficients, has_coefficients);
    const std::vector<FrozenDev> fz{frozen_dev(c, spot_bump, vol_bump)};
    std::vector<double> res;
    rc = frozen_run(*ctx, p, fz, precision, kFrozenScenarios, &reg, res);
    if (rc) return rc;
    assemble_greeks(c, spot_bump, vol_bump, exercise_at_inception != 0, res.data(), *out);
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_lsm_greeks_batch(mcd_ctx* handle, const mcd_lsm_contract* contracts, size_t n, double spot_bump_rel,
                         double vol_bump_rel, int precision, mcd_american_greeks* results) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    if (!(spot_bump_rel > 0.0 && spot_bump_rel < 1.0) || !(vol_bump_rel > 0.0 && vol_bump_rel < 1.0))
        return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "relative bumps must lie in (0, 1)");
    if (n == 0) return MCD_OK;
    if (!contracts || !results) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "null array");
    LsmPlan p;
    int rc = plan_lsm(*ctx, contracts, n, p);
    if (rc) return rc;
    // fit every policy (stored paths, QR); the table stays on the device
    std::vector<double> fit;
    rc = upload_and_run(*ctx, p, precision, false, fit);
    if (rc) return rc;
    std::vector<FrozenDev> fz(n);
    for (size_t i = 0; i < n; ++i)
        fz[i] = frozen_dev(contracts[i], spot_bump_rel * contracts[i].spot, vol_bump_rel * contracts[i].vol);
    std::vector<double> res;
    rc = frozen_run(*ctx, p, fz, precision, kFrozenScenarios, nullptr, res);
    if (rc) return rc;
    for (size_t i = 0; i < n; ++i)
        assemble_greeks(contracts[i], spot_bump_rel * contracts[i].spot, vol_bump_rel * contracts[i].vol,
                        fit[6 * i + 3] != 0.0, res.data() + 3 * kFrozenOutputs * i, results[i]);
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_lsm_batch(mcd_ctx* handle, const mcd_lsm_contract* contracts, size_t n, int precision,
                  int regression, mcd_lsm_result* results) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    return lsm_batch(*ctx, contracts, n, precision, regression, results, nullptr);
} catch (...) {
    return abi_exception(handle);
}

int mcd_lsm_set_mlp_config(mcd_ctx* handle, int steps_first, int steps, double lr_first, double lr) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (steps_first < 0 || steps < 0 || steps_first > 1000000 || steps > 1000000 || !(lr_first > 0) || !(lr > 0))
        return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "steps must be 0..1e6 and learning rates > 0");
    ctx->mlp_steps_first = steps_first;
    ctx->mlp_steps = steps;
    ctx->mlp_lr_first = static_cast<float>(lr_first);
    ctx->mlp_lr = static_cast<float>(lr);
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_lsm_mlp_policy(mcd_ctx* handle, size_t contract, float* weights, uint8_t* has) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (contract >= ctx->mlp_reg_offset.size()) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "no such contract in the last learned run");
    const uint32_t off = ctx->mlp_reg_offset[contract];
    const int nd = ctx->mlp_steps_of[contract];
    std::vector<float> buf(static_cast<size_t>(nd + 1) * mlp::kParamStride);
    std::vector<int> ok(nd + 1);
    cudaError_t e = cudaMemcpy(buf.data(), static_cast<float*>(ctx->ext[kSnaps].ptr) + static_cast<size_t>(off) * mlp::kParamStride,
                               sizeof(float) * buf.size(), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(ok.data(), static_cast<int*>(ctx->ext[kSnapOk].ptr) + off, sizeof(int) * ok.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "mlp policy copy");
    for (int d = 0; d <= nd; ++d) {
        if (has) has[d] = ok[d] == 1 ? 1 : 0;
        if (weights)
            for (int q = 0; q < mlp::kParams; ++q)
                weights[static_cast<size_t>(d) * mlp::kParams + q] = ok[d] == 1 ? buf[static_cast<size_t>(d) * mlp::kParamStride + q] : 0.0f;
    }
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_lsm_reprice_mlp(mcd_ctx* handle, double spot, double strike, double rate, double carry_yield,
                        double vol, double time, int type, int monitoring_points, uint64_t path_count,
                        uint64_t seed, const float* weights, const uint8_t* has, int precision,
                        mcd_lsm_result* out) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (!weights || !has || !out) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "null argument");
    if (precision != 0 && precision != 1) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (FP32)");
    const mcd_lsm_contract c{spot, strike, rate, carry_yield, vol, time, type, monitoring_points, path_count, seed};
    LsmPlan p;
    int rc = plan_lsm(*ctx, &c, 1, p);
    if (rc) return rc;
    std::vector<float> nets(p.reg_rows * mlp::kParamStride, 0.0f);
    std::vector<int> ok(p.reg_rows, 0);
    for (int d = 1; d < monitoring_points; ++d) {
        if (!has[d]) continue;
        ok[d] = 1;
        for (int q = 0; q < mlp::kParams; ++q)
            nets[static_cast<size_t>(d) * mlp::kParamStride + q] = weights[static_cast<size_t>(d) * mlp::kParams + q];
    }
    std::vector<double> res;
    rc = upload_and_run(*ctx, p, precision, true, res, true, &nets, &ok);
    if (rc) return rc;
    out->price = res[0];
    out->standard_error = res[1];
    out->path_count = static_cast<uint64_t>(res[2]);
    out->exercise_at_inception = res[3] != 0.0 ? 1 : 0;
    out->reserved = 0;
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_umma_selftest(mcd_ctx* handle, const float* a, const float* b, float* d) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (!a || !b || !d) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "null argument");
    int rc = ctx->reserve(ctx->ext[kErr], 256, "error word");
    if (!rc) rc = ctx->reserve(ctx->d_scratch2, sizeof(float) * (128 * 64 * 2 + 64 * 64), "selftest buffers");
    if (rc) return rc;
    float* da = static_cast<float*>(ctx->d_scratch2.ptr);
    float* db = da + 128 * 64;
    float* dd = db + 64 * 64;
    uint32_t werr = 0;
    cudaError_t e = cudaMemcpyAsync(da, a, sizeof(float) * 128 * 64, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(db, b, sizeof(float) * 64 * 64, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->ext[kErr].ptr, 0, 256, ctx->stream);
    if (e == cudaSuccess) e = launch_umma_selftest(da, db, dd, static_cast<uint32_t*>(ctx->ext[kErr].ptr), ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, dd, sizeof(float) * 128 * 64, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&werr, ctx->ext[kErr].ptr, sizeof werr, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "umma selftest");
    if (werr) return ctx->fail(MCD_ERR_TIMEOUT, "tensor-core wait gave up");
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_mlp_gradients(mcd_ctx* handle, const float* params, const float* x0, const float* x1, const float* y,
                      const float* w, int n, float* grad, float* loss) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (n < 1 || n > 128) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "n must be 1..128");
    if (!params || !x0 || !x1 || !y || !w || !grad || !loss) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "null argument");
    int rc = ctx->reserve(ctx->ext[kErr], 256, "error word");
    const size_t floats = mlp::kParamStride * 2 + 128 * 4 + 4;
    if (!rc) rc = ctx->reserve(ctx->d_scratch2, sizeof(float) * floats, "gradient buffers");
    if (rc) return rc;
    cudaError_t e = mlp_prepare();
    if (e != cudaSuccess) return ctx->cuda_fail(e, "mlp shared memory opt-in");
    float* dp = static_cast<float*>(ctx->d_scratch2.ptr);
    float* dg = dp + mlp::kParamStride;
    float* dx0 = dg + mlp::kParamStride;
    float* dx1 = dx0 + 128;
    float* dy = dx1 + 128;
    float* dw = dy + 128;
    float* dl = dw + 128;
    uint32_t werr = 0;
    e = cudaMemcpyAsync(dp, params, sizeof(float) * mlp::kParams, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx0, x0, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx1, x1, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dy, y, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dw, w, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->ext[kErr].ptr, 0, 256, ctx->stream);
    if (e == cudaSuccess)
        e = launch_mlp_grad(dp, dx0, dx1, dy, dw, n, dg, dl, static_cast<uint32_t*>(ctx->ext[kErr].ptr), ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(grad, dg, sizeof(float) * mlp::kParams, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(loss, dl, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&werr, ctx->ext[kErr].ptr, sizeof werr, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "mlp gradients");
    if (werr) return ctx->fail(MCD_ERR_TIMEOUT, "tensor-core wait gave up");
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

int mcd_mlp_forward(mcd_ctx* handle, const float* params, const float* x0, const float* x1, size_t n, float* out) try {
    MCD_CTX_OR_FAIL(handle, ctx);
    if (n == 0) return MCD_OK;
    if (n > (1u << 26)) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "at most 2^26 inputs per call");
    if (!params || !x0 || !x1 || !out) return ctx->fail(MCD_ERR_INVALID_ARGUMENT, "null argument");
    int rc = ctx->reserve(ctx->ext[kErr], 256, "error word");
    if (!rc) rc = ctx->reserve(ctx->d_scratch2, sizeof(float) * (mlp::kParamStride + 3 * n), "forward buffers");
    if (rc) return rc;
    cudaError_t e = mlp_prepare();
    if (e != cudaSuccess) return ctx->cuda_fail(e, "mlp shared memory opt-in");
    float* dp = static_cast<float*>(ctx->d_scratch2.ptr);
    float* dx0 = dp + mlp::kParamStride;
    float* dx1 = dx0 + n;
    float* dout = dx1 + n;
    uint32_t werr = 0;
    e = cudaMemcpyAsync(dp, params, sizeof(float) * mlp::kParams, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx0, x0, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx1, x1, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->ext[kErr].ptr, 0, 256, ctx->stream);
    if (e == cudaSuccess)
        e = launch_mlp_forward(dp, dx0, dx1, static_cast<int>(n), dout, static_cast<uint32_t*>(ctx->ext[kErr].ptr), ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&werr, ctx->ext[kErr].ptr, sizeof werr, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "mlp forward");
    if (werr) return ctx->fail(MCD_ERR_TIMEOUT, "tensor-core wait gave up");
    return MCD_OK;
} catch (...) {
    return abi_exception(handle);
}

}  // extern "C"
