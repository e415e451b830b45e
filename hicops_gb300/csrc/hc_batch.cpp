// Batched search support: CUDA-graph replay of the whole query pipeline and
// the autotuner that picks the search launch shape (block size, scorecard
// tile, postings lists in flight per warp, resident CTAs, schedule).
#include <algorithm>
#include <cstring>
#include <vector>

#include "hc_internal.h"

namespace hc {

static bool same_key(const GraphKey &a, const GraphKey &b) { return std::memcmp(&a, &b, sizeof(a)) == 0; }

// Replays the context's graph for `key`, capturing it first (through `body`
// on the capture stream) when the key differs from the captured one.
template <class Body>
static int replay(hc_ctx *ctx, const GraphKey &key, cudaStream_t st, Body body)
{
    if (!ctx->graph_exec || !same_key(key, ctx->graph_key))
    {
        if (ctx->graph_exec)
        {
            cudaGraphExecDestroy(ctx->graph_exec);
            ctx->graph_exec = nullptr;
        }
        if (!ctx->cap_stream) HC_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking));
        // with profiling on, the stage events are captured as external
        // event-record nodes (the graph key includes the profiling switch)
        HC_CUDA(ctx, cudaStreamBeginCapture(ctx->cap_stream, cudaStreamCaptureModeRelaxed));
        int rc = body(ctx->cap_stream);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(ctx->cap_stream, &g);
        if (rc)
        {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        HC_CUDA(ctx, e);
        e = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
        cudaGraphDestroy(g);
        HC_CUDA(ctx, e);
        ctx->graph_key = key;
        ctx->graph_launches = ctx->last_launches;
    }
    HC_CUDA(ctx, cudaGraphLaunch(ctx->graph_exec, st));
    ctx->last_launches = ctx->graph_launches;
    return HC_SUCCESS;
}

static GraphKey make_key(const hc_ctx *ctx, const uint32_t *d_idx, const uint32_t *d_moz, const uint32_t *d_intensity,
                         const float *d_precurse, const double *d_dM, uint32_t nspec, uint32_t npeaks,
                         hc_result *d_out, uint32_t *d_hist)
{
    GraphKey key{};
    key.idx = d_idx;
    key.moz = d_moz;
    key.inten = d_intensity;
    key.prec = d_precurse;
    key.dM = d_dM;
    key.out = d_out;
    key.hist = d_hist;
    key.nspec = nspec;
    key.npeaks = npeaks;
    key.tuning = ctx->tuning;
    key.profiling = ctx->profiling ? 1u : 0u;
    return key;
}

}  // namespace hc

using namespace hc;

extern "C" {

int hc_dslim_query_graph(hc_ctx *ctx, const uint32_t *d_idx, const uint32_t *d_moz, const uint32_t *d_intensity,
                         const float *d_precurse, const double *d_dM, uint32_t nspec, uint32_t npeaks,
                         hc_result *d_out, uint32_t *d_hist, void *stream)
{
    if (!ctx) return HC_ERR_INVLD_PTR;
    if (nspec && (!d_idx || !d_moz || !d_intensity || !d_precurse || !d_out || !d_hist))
        return set_error(ctx, HC_ERR_INVLD_PTR, "null device buffer");
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    const GraphKey key = make_key(ctx, d_idx, d_moz, d_intensity, d_precurse, d_dM, nspec, npeaks, d_out, d_hist);
    // everything that allocates or copies synchronously happens before capture
    int rc = prepare_query(ctx, nspec);
    if (rc) return rc;
    rc = replay(ctx, key, st, [&](cudaStream_t cs) {
        return query_device(ctx, d_idx, d_moz, d_intensity, d_precurse, d_dM, nspec, npeaks, d_out, d_hist, cs);
    });
    ctx->last_learned = false;
    return rc;
}

int hc_dslim_query_learned(hc_ctx *ctx, hc_mlp *mlp, const uint32_t *d_idx, const uint32_t *d_moz,
                           const uint32_t *d_intensity, const float *d_precurse, const double *d_dM, uint32_t nspec,
                           uint32_t npeaks, hc_result *d_out, uint32_t *d_hist, float *d_learned_log10e,
                           void *stream)
{
    if (!ctx || !mlp) return HC_ERR_INVLD_PTR;
    if (nspec && (!d_idx || !d_moz || !d_intensity || !d_precurse || !d_out || !d_hist))
        return set_error(ctx, HC_ERR_INVLD_PTR, "null device buffer");
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    GraphKey key = make_key(ctx, d_idx, d_moz, d_intensity, d_precurse, d_dM, nspec, npeaks, d_out, d_hist);
    key.mlp = mlp;
    key.learned = d_learned_log10e;
    learned_gate(mlp, &key.gate_resid, &key.gate_radius);
    int rc = prepare_query(ctx, nspec);
    if (rc) return rc;
    if ((rc = learned_prepare(mlp, nspec))) return rc;
    rc = replay(ctx, key, st, [&](cudaStream_t cs) {
        int r = query_device(ctx, d_idx, d_moz, d_intensity, d_precurse, d_dM, nspec, npeaks, d_out, d_hist, cs,
                             false);
        if (r) return r;
        int launches = ctx->last_launches;
        r = learned_pipeline(mlp, d_hist, d_out, nspec, d_learned_log10e, cs, &launches);
        ctx->last_launches = launches;
        return r;
    });
    ctx->last_learned = true;
    return rc;
}

int hc_tune(hc_ctx *ctx, const uint32_t *d_idx, const uint32_t *d_moz, const uint32_t *d_intensity,
            const float *d_precurse, const double *d_dM, uint32_t nspec, uint32_t npeaks, hc_result *d_out,
            uint32_t *d_hist, hc_tuning *best, float *best_ms)
{
    if (!ctx) return HC_ERR_INVLD_PTR;
    if (nspec == 0) return set_error(ctx, HC_ERR_NOT_ENOUGH_DATA, "empty tuning sample");
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    const hc_tuning saved = ctx->tuning;
    // stage 1: schedule x CTAs per SM x block size x chunks in flight, each with
    // the largest scorecard tile that fits (small windows in the same launch)
    std::vector<hc_tuning> cand;
    for (uint32_t sched : {0u, 2u})
        for (uint32_t cps : {1u, 2u})
            for (uint32_t thr : {256u, 512u, 1024u})
                for (uint32_t g : {2u, 4u, 8u})
                {
                    if (g >= 4 && thr > 512) continue;
                    hc_tuning t{};
                    t.threads = thr;
                    t.pairs_per_warp = g;
                    t.ctas_per_sm = cps;
                    t.schedule = sched;
                    t.defer_cap = saved.defer_cap;
                    // two resident CTAs share the SM's shared memory
                    t.tile = max_tile_for(ctx, ctx->p.dF, cps, thr);
                    if (t.tile < kRowG) continue;
                    cand.push_back(t);
                }
    cudaEvent_t e0, e1;
    HC_CUDA(ctx, cudaEventCreate(&e0));
    HC_CUDA(ctx, cudaEventCreate(&e1));
    const bool prof = ctx->profiling;
    ctx->profiling = false;
    int rc = HC_SUCCESS;
    std::vector<std::pair<float, hc_tuning>> timed;
    auto run = [&](const hc_tuning &t) {
        if (hc_ctx_set_tuning(ctx, &t) != HC_SUCCESS) return;
        rc = query_device(ctx, d_idx, d_moz, d_intensity, d_precurse, d_dM, nspec, npeaks, d_out, d_hist, st);
        if (rc) return;
        float ms[2];
        for (int r = 0; r < 2 && !rc; r++)
        {
            cudaEventRecord(e0, st);
            rc = query_device(ctx, d_idx, d_moz, d_intensity, d_precurse, d_dM, nspec, npeaks, d_out, d_hist, st);
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&ms[r], e0, e1);
        }
        if (!rc) timed.emplace_back(std::min(ms[0], ms[1]), t);
    };
    for (const hc_tuning &t : cand)
    {
        run(t);
        if (rc) break;
    }
    // stage 2: smaller scorecard tiles (fewer candidates per tile, more room for
    // the shared lists) for the three fastest shapes
    if (!rc)
    {
        std::sort(timed.begin(), timed.end(), [](const auto &a, const auto &b) { return a.first < b.first; });
        const size_t top = std::min<size_t>(3, timed.size());
        std::vector<hc_tuning> more;
        for (size_t k = 0; k < top; k++)
            for (uint32_t cut : {1u, 2u, 4u})
            {
                hc_tuning t = timed[k].second;
                if (t.tile <= cut * kRowG) continue;
                t.tile -= cut * kRowG;
                more.push_back(t);
            }
        for (const hc_tuning &t : more)
        {
            run(t);
            if (rc) break;
        }
    }
    // stage 3: the fastest longest-first shape with the small-window spectra
    // in a launch of their own, for a few split points
    if (!rc)
    {
        const auto best2 = std::min_element(timed.begin(), timed.end(), [](const auto &a, const auto &b) {
            if ((a.second.schedule == 2) != (b.second.schedule == 2)) return a.second.schedule == 2;
            return a.first < b.first;
        });
        if (best2 != timed.end() && best2->second.schedule == 2)
        {
            const hc_tuning base = best2->second;
            for (uint32_t lg : {12u, 15u, 18u})
            {
                hc_tuning t = base;
                t.small_log2 = lg;
                run(t);
                if (rc) break;
            }
        }
    }
    ctx->profiling = prof;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc || timed.empty())
    {
        ctx->tuning = saved;
        return rc ? rc : set_error(ctx, HC_ERR_INVLD_PARAM, "no launch shape could be timed");
    }
    const auto bestp = *std::min_element(timed.begin(), timed.end(),
                                         [](const auto &a, const auto &b) { return a.first < b.first; });
    ctx->tuning = bestp.second;
    if (best) *best = bestp.second;
    if (best_ms) *best_ms = bestp.first;
    return HC_SUCCESS;
}

int hc_ctx_set_phase_timing(hc_ctx *ctx, int on)
{
    if (!ctx) return HC_ERR_INVLD_PTR;
    cudaSetDevice(ctx->device);
    if (on && !ctx->d_phase)
    {
        HC_CUDA(ctx, cudaMalloc((void **)&ctx->d_phase, 8 * 16));
        HC_CUDA(ctx, cudaMemset(ctx->d_phase, 0, 8 * 16));
    }
    if (!on && ctx->d_phase)
    {
        cudaFree(ctx->d_phase);
        ctx->d_phase = nullptr;
    }
    return HC_SUCCESS;
}

int hc_phase_cycles(hc_ctx *ctx, uint64_t out[10])
{
    if (!ctx || !out) return HC_ERR_INVLD_PTR;
    if (!ctx->d_phase) return set_error(ctx, HC_ERR_INVLD_PARAM, "phase timing is off");
    HC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    HC_CUDA(ctx, cudaDeviceSynchronize());
    HC_CUDA(ctx, cudaMemcpy(out, ctx->d_phase, 8 * 10, cudaMemcpyDeviceToHost));
    HC_CUDA(ctx, cudaMemset(ctx->d_phase, 0, 8 * 16));
    return HC_SUCCESS;
}

}  // extern "C"
