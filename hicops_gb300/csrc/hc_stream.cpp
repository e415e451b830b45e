// Streaming query over a large host batch (the batch loop of
// DSLIM_SearchManager, source/core/dslim_query.cpp:160-420, where an I/O
// thread fills QCHUNK-sized batches that DSLIM_QuerySpectrum searches one after
// another). Here sub-batches alternate between two staging slots: while the
// device searches sub-batch b, the host packs sub-batch b+1 into pinned memory
// and its copies run on a copy stream; results come back on the same copy
// stream once the search event of their sub-batch has fired.
//
// The slots (pinned host and device buffers, the copy stream, events) belong
// to the context and are kept between calls; a call grows them only when its
// sub-batches need more room than an earlier call's did.
#include <algorithm>
#include <cstring>
#include <vector>

#include "hc_internal.h"

namespace hc {

namespace {

struct Slot
{
    // pinned host staging
    uint32_t *h_idx = nullptr, *h_moz = nullptr, *h_int = nullptr, *h_hist = nullptr;
    float *h_prec = nullptr, *h_learned = nullptr;
    double *h_dM = nullptr;
    hc_result *h_out = nullptr;
    // device buffers
    uint32_t *d_idx = nullptr, *d_moz = nullptr, *d_int = nullptr, *d_hist = nullptr;
    float *d_prec = nullptr, *d_learned = nullptr;
    double *d_dM = nullptr;
    hc_result *d_out = nullptr;
    cudaEvent_t ev_in = nullptr, ev_done = nullptr, ev_out = nullptr;
    int64_t s0 = -1;  // first spectrum of the sub-batch in flight (-1: none)
    uint32_t n = 0;
};

void free_slot(Slot &s)
{
    cudaFreeHost(s.h_idx);
    cudaFreeHost(s.h_moz);
    cudaFreeHost(s.h_int);
    cudaFreeHost(s.h_hist);
    cudaFreeHost(s.h_prec);
    cudaFreeHost(s.h_learned);
    cudaFreeHost(s.h_dM);
    cudaFreeHost(s.h_out);
    cudaFree(s.d_idx);
    cudaFree(s.d_moz);
    cudaFree(s.d_int);
    cudaFree(s.d_hist);
    cudaFree(s.d_prec);
    cudaFree(s.d_learned);
    cudaFree(s.d_dM);
    cudaFree(s.d_out);
    if (s.ev_in) cudaEventDestroy(s.ev_in);
    if (s.ev_done) cudaEventDestroy(s.ev_done);
    if (s.ev_out) cudaEventDestroy(s.ev_out);
    s = Slot();
}

template <class T>
cudaError_t hpin(T **p, size_t n) { return cudaMallocHost((void **)p, sizeof(T) * (n ? n : 1)); }
template <class T>
cudaError_t dmem(T **p, size_t n) { return cudaMalloc((void **)p, sizeof(T) * (n ? n : 1)); }

}  // namespace

struct StreamStage
{
    Slot slot[2];
    cudaStream_t cs = nullptr;  // copy stream
    // what the slots hold room for
    uint32_t batch = 0, peaks = 0;
    bool dM = false, hist = false, learned = false;
};

void free_stream_stage(StreamStage *st)
{
    if (!st) return;
    for (Slot &s : st->slot) free_slot(s);
    if (st->cs) cudaStreamDestroy(st->cs);
    delete st;
}

// Makes the context's slots hold sub-batches of `batch` spectra and `peaks`
// peaks with the optional buffers asked for; reallocates only when they do not.
static int ensure_stage(hc_ctx *ctx, uint32_t batch, uint32_t peaks, bool dM, bool hist, bool learned)
{
    StreamStage *&g = ctx->stage;
    if (g && g->batch >= batch && g->peaks >= peaks && (g->dM || !dM) && (g->hist || !hist) &&
        (g->learned || !learned))
        return HC_SUCCESS;
    StreamStage want;
    if (g)
    {
        want.batch = g->batch;
        want.peaks = g->peaks;
        want.dM = g->dM;
        want.hist = g->hist;
        want.learned = g->learned;
        free_stream_stage(g);
        g = nullptr;
    }
    StreamStage *n = new StreamStage();
    n->batch = std::max(want.batch, batch);
    n->peaks = std::max(want.peaks, peaks);
    n->dM = want.dM || dM;
    n->hist = want.hist || hist;
    n->learned = want.learned || learned;
    cudaError_t e = cudaStreamCreateWithFlags(&n->cs, cudaStreamNonBlocking);
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    const size_t B = n->batch, P = n->peaks;
    for (Slot &s : n->slot)
    {
        chk(hpin(&s.h_idx, B + 1));
        chk(hpin(&s.h_moz, P));
        chk(hpin(&s.h_int, P));
        chk(hpin(&s.h_prec, B));
        chk(hpin(&s.h_out, B));
        chk(dmem(&s.d_idx, B + 1));
        chk(dmem(&s.d_moz, P + 4));
        chk(dmem(&s.d_int, P + 4));
        chk(dmem(&s.d_prec, B));
        chk(dmem(&s.d_out, B));
        chk(dmem(&s.d_hist, B * HC_HIST_BINS));
        if (n->dM)
        {
            chk(hpin(&s.h_dM, B));
            chk(dmem(&s.d_dM, B));
        }
        if (n->hist) chk(hpin(&s.h_hist, B * HC_HIST_BINS));
        if (n->learned)
        {
            chk(hpin(&s.h_learned, B));
            chk(dmem(&s.d_learned, B));
        }
        chk(cudaEventCreateWithFlags(&s.ev_in, cudaEventDisableTiming));
        chk(cudaEventCreateWithFlags(&s.ev_done, cudaEventDisableTiming));
        chk(cudaEventCreateWithFlags(&s.ev_out, cudaEventDisableTiming));
    }
    if (e != cudaSuccess)
    {
        free_stream_stage(n);
        return set_error(ctx, HC_ERR_BAD_MEM_ALLOC, std::string("stream staging: ") + cudaGetErrorString(e));
    }
    g = n;
    return HC_SUCCESS;
}

}  // namespace hc

extern "C" int hc_dslim_query_stream(hc_ctx *ctx, const uint32_t *idx, const uint32_t *moz, const uint32_t *intensity,
                                     const float *precurse, const double *dM_per_spec, uint32_t nspec,
                                     uint32_t batch, hc_mlp *mlp, hc_result *out, uint32_t *hist,
                                     float *learned_log10e)
{
    using namespace hc;
    if (!ctx) return HC_ERR_INVLD_PTR;
    if (nspec == 0) return HC_SUCCESS;
    if (!idx || !moz || !intensity || !precurse || !out) return HC_ERR_INVLD_PTR;
    if (batch == 0) return set_error(ctx, HC_ERR_INVLD_SIZE, "hc_dslim_query_stream: batch of 0 spectra");
    for (uint32_t i = 0; i < nspec; i++)
        if (idx[i + 1] < idx[i]) return set_error(ctx, HC_ERR_INVLD_SIZE, "idx not monotone");
    HC_CUDA(ctx, cudaSetDevice(ctx->device));
    batch = std::min(batch, nspec);
    const uint32_t nb = (nspec + batch - 1) / batch;
    uint32_t maxpk = 0;
    for (uint32_t b = 0; b < nb; b++)
    {
        const uint32_t s0 = b * batch, s1 = std::min(nspec, s0 + batch);
        maxpk = std::max(maxpk, idx[s1] - idx[s0]);
    }
    const bool want_learned = mlp && learned_log10e;
    int rc = ensure_stage(ctx, batch, maxpk, dM_per_spec != nullptr, hist != nullptr, want_learned);
    if (rc) return rc;
    if ((rc = prepare_query(ctx, batch))) return rc;
    if (mlp && (rc = learned_prepare(mlp, batch))) return rc;
    StreamStage &g = *ctx->stage;
    Slot *slot = g.slot;
    cudaStream_t cs = g.cs;
    auto fail = [&](int code, const char *what) {
        if (rc == HC_SUCCESS) rc = set_error(ctx, code, what);
        return rc;
    };
    // results of a finished sub-batch: pinned staging -> the caller's arrays
    auto drain = [&](Slot &s) {
        if (s.s0 < 0) return;
        if (cudaEventSynchronize(s.ev_out) != cudaSuccess) fail(HC_ERR_CUDA, "stream copy-out");
        if (rc == HC_SUCCESS)
        {
            std::memcpy(out + s.s0, s.h_out, sizeof(hc_result) * s.n);
            if (hist) std::memcpy(hist + (size_t)s.s0 * HC_HIST_BINS, s.h_hist, 4ull * HC_HIST_BINS * s.n);
            if (want_learned) std::memcpy(learned_log10e + s.s0, s.h_learned, 4ull * s.n);
        }
        s.s0 = -1;
    };
    for (uint32_t b = 0; b < nb && rc == HC_SUCCESS; b++)
    {
        Slot &s = slot[b & 1];
        drain(s);  // the slot's previous sub-batch (b - 2) is done with its buffers
        if (rc) break;
        const uint32_t s0 = b * batch, s1 = std::min(nspec, s0 + batch), n = s1 - s0;
        const uint32_t p0 = idx[s0], np = idx[s1] - p0;
        for (uint32_t i = 0; i <= n; i++) s.h_idx[i] = idx[s0 + i] - p0;
        std::memcpy(s.h_moz, moz + p0, 4ull * np);
        std::memcpy(s.h_int, intensity + p0, 4ull * np);
        std::memcpy(s.h_prec, precurse + s0, 4ull * n);
        if (dM_per_spec) std::memcpy(s.h_dM, dM_per_spec + s0, 8ull * n);
        cudaError_t e = cudaMemcpyAsync(s.d_idx, s.h_idx, 4ull * (n + 1), cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess && np) e = cudaMemcpyAsync(s.d_moz, s.h_moz, 4ull * np, cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess && np) e = cudaMemcpyAsync(s.d_int, s.h_int, 4ull * np, cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess) e = cudaMemcpyAsync(s.d_prec, s.h_prec, 4ull * n, cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess && dM_per_spec)
            e = cudaMemcpyAsync(s.d_dM, s.h_dM, 8ull * n, cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess) e = cudaEventRecord(s.ev_in, cs);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, s.ev_in, 0);
        if (e != cudaSuccess)
        {
            fail(HC_ERR_CUDA, cudaGetErrorString(e));
            break;
        }
        int q = query_device(ctx, s.d_idx, s.d_moz, s.d_int, s.d_prec, dM_per_spec ? s.d_dM : nullptr, n, np,
                             s.d_out, s.d_hist, ctx->stream, mlp == nullptr);
        if (q == HC_SUCCESS && mlp)
            q = learned_pipeline(mlp, s.d_hist, s.d_out, n, want_learned ? s.d_learned : nullptr, ctx->stream,
                                 nullptr);
        if (q != HC_SUCCESS)
        {
            rc = q;
            break;
        }
        e = cudaEventRecord(s.ev_done, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, s.ev_done, 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(s.h_out, s.d_out, sizeof(hc_result) * n, cudaMemcpyDeviceToHost, cs);
        if (e == cudaSuccess && hist)
            e = cudaMemcpyAsync(s.h_hist, s.d_hist, 4ull * HC_HIST_BINS * n, cudaMemcpyDeviceToHost, cs);
        if (e == cudaSuccess && want_learned)
            e = cudaMemcpyAsync(s.h_learned, s.d_learned, 4ull * n, cudaMemcpyDeviceToHost, cs);
        if (e == cudaSuccess) e = cudaEventRecord(s.ev_out, cs);
        if (e != cudaSuccess)
        {
            fail(HC_ERR_CUDA, cudaGetErrorString(e));
            break;
        }
        s.s0 = s0;
        s.n = n;
    }
    // the last one or two sub-batches, in order
    if (slot[0].s0 >= 0 && slot[1].s0 >= 0 && slot[1].s0 < slot[0].s0)
    {
        drain(slot[1]);
        drain(slot[0]);
    }
    else
    {
        drain(slot[0]);
        drain(slot[1]);
    }
    cudaStreamSynchronize(ctx->stream);
    cudaStreamSynchronize(cs);
    slot[0].s0 = slot[1].s0 = -1;
    return rc;
}
