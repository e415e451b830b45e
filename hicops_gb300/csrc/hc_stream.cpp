// Streaming query over a large host batch (the batch loop of
// DSLIM_SearchManager, source/core/dslim_query.cpp:160-420, where an I/O
// thread fills QCHUNK-sized batches that DSLIM_QuerySpectrum searches one after
// another). Here sub-batches alternate between two staging slots: while the
// device searches sub-batch b, the host packs sub-batch b+1 into pinned memory
// and its copies run on a copy stream; results come back on the same copy
// stream once the search event of their sub-batch has fired.
#include <algorithm>
#include <cstring>
#include <vector>

#include "hc_internal.h"

namespace {

struct Slot
{
    // pinned host staging
    uint32_t *h_idx = nullptr, *h_moz = nullptr, *h_int = nullptr, *h_hist = nullptr;
    float *h_prec = nullptr, *h_learned = nullptr;
    double *h_dM = nullptr;
    hc_result *h_out = nullptr;
    // device buffers
    uint32_t *d_idx = nullptr, *d_moz = nullptr, *d_int = nullptr, *d_hist = nullptr, *d_nfb = nullptr;
    float *d_prec = nullptr, *d_X = nullptr, *d_scr = nullptr, *d_learned = nullptr;
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
    cudaFree(s.d_nfb);
    cudaFree(s.d_prec);
    cudaFree(s.d_X);
    cudaFree(s.d_scr);
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

extern "C" int hc_dslim_query_stream(hc_ctx *ctx, const uint32_t *idx, const uint32_t *moz, const uint32_t *intensity,
                                     const float *precurse, const double *dM_per_spec, uint32_t nspec,
                                     uint32_t batch, hc_mlp *mlp, float thresh, hc_result *out, uint32_t *hist,
                                     float *learned_log10e)
{
    using namespace hc;
    if (!ctx) return HC_ERR_INVLD_PTR;
    if (nspec == 0) return HC_SUCCESS;
    if (!idx || !moz || !intensity || !precurse || !out) return HC_ERR_INVLD_PTR;
    if (batch == 0) return set_error(ctx, HC_ERR_INVLD_SIZE, "hc_dslim_query_stream: batch of 0 spectra");
    for (uint32_t i = 0; i < nspec; i++)
        if (idx[i + 1] < idx[i]) return set_error(ctx, HC_ERR_INVLD_SIZE, "idx not monotone");
    cudaSetDevice(ctx->device);
    batch = std::min(batch, nspec);
    const uint32_t nb = (nspec + batch - 1) / batch;
    uint32_t maxpk = 0;
    for (uint32_t b = 0; b < nb; b++)
    {
        const uint32_t s0 = b * batch, s1 = std::min(nspec, s0 + batch);
        maxpk = std::max(maxpk, idx[s1] - idx[s0]);
    }

    Slot slot[2];
    cudaStream_t cs = nullptr;
    int rc = HC_SUCCESS;
    auto fail = [&](int code, const char *what) {
        if (rc == HC_SUCCESS) rc = set_error(ctx, code, what);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return fail(HC_ERR_CUDA, "copy stream");
    for (Slot &s : slot)
    {
        cudaError_t e = cudaSuccess;
        auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
        chk(hpin(&s.h_idx, batch + 1));
        chk(hpin(&s.h_moz, maxpk));
        chk(hpin(&s.h_int, maxpk));
        chk(hpin(&s.h_prec, batch));
        chk(hpin(&s.h_out, batch));
        if (dM_per_spec) chk(hpin(&s.h_dM, batch));
        if (hist) chk(hpin(&s.h_hist, (size_t)batch * HC_HIST_BINS));
        if (mlp && learned_log10e) chk(hpin(&s.h_learned, batch));
        chk(dmem(&s.d_idx, batch + 1));
        chk(dmem(&s.d_moz, maxpk + 4));
        chk(dmem(&s.d_int, maxpk + 4));
        chk(dmem(&s.d_prec, batch));
        chk(dmem(&s.d_out, batch));
        chk(dmem(&s.d_hist, (size_t)batch * HC_HIST_BINS));
        if (dM_per_spec) chk(dmem(&s.d_dM, batch));
        if (mlp)
        {
            chk(dmem(&s.d_X, (size_t)batch * 256));
            chk(dmem(&s.d_scr, (size_t)batch * 3));
            chk(dmem(&s.d_learned, batch));
            chk(dmem(&s.d_nfb, 1));
        }
        chk(cudaEventCreateWithFlags(&s.ev_in, cudaEventDisableTiming));
        chk(cudaEventCreateWithFlags(&s.ev_done, cudaEventDisableTiming));
        chk(cudaEventCreateWithFlags(&s.ev_out, cudaEventDisableTiming));
        if (e != cudaSuccess)
        {
            fail(HC_ERR_BAD_MEM_ALLOC, cudaGetErrorString(e));
            break;
        }
    }
    // results of a finished sub-batch: pinned staging -> the caller's arrays
    auto drain = [&](Slot &s) {
        if (s.s0 < 0) return;
        if (cudaEventSynchronize(s.ev_out) != cudaSuccess) fail(HC_ERR_CUDA, "stream copy-out");
        if (rc == HC_SUCCESS)
        {
            std::memcpy(out + s.s0, s.h_out, sizeof(hc_result) * s.n);
            if (hist) std::memcpy(hist + (size_t)s.s0 * HC_HIST_BINS, s.h_hist, 4ull * HC_HIST_BINS * s.n);
            if (s.h_learned) std::memcpy(learned_log10e + s.s0, s.h_learned, 4ull * s.n);
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
        int q = query_device(ctx, s.d_idx, s.d_moz, s.d_int, s.d_prec, s.d_dM, n, np, s.d_out, s.d_hist,
                             ctx->stream);
        if (q == HC_SUCCESS && mlp)
        {
            q = hc_mlp_features(ctx, s.d_hist, s.d_out, n, s.d_X, ctx->stream);
            if (q == HC_SUCCESS)
                q = hc_mlp_evalues(mlp, s.d_X, s.d_out, n, thresh, s.d_learned, s.d_nfb, s.d_scr, ctx->stream);
        }
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
        if (e == cudaSuccess && s.h_learned)
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
    if (slot[0].s0 >= 0 && slot[1].s0 >= 0 && slot[1].s0 < slot[0].s0) std::swap(slot[0], slot[1]);
    drain(slot[0]);
    drain(slot[1]);
    cudaStreamSynchronize(ctx->stream);
    cudaStreamSynchronize(cs);
    for (Slot &s : slot) free_slot(s);
    cudaStreamDestroy(cs);
    return rc;
}
