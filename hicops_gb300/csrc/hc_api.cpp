// C ABI of hicops_gb300 (include/hicops_gb300.h): context management, index
// construction/loading/export, and the host- and device-buffer query calls.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <thread>
#include <string>
#include <vector>

#include "hc_internal.h"

namespace hc {

int set_error(hc_ctx *ctx, int code, const std::string &msg)
{
    if (ctx) ctx->last_error = msg;
    return code;
}

int cuda_check(hc_ctx *ctx, cudaError_t e, const char *what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return set_error(ctx, e == cudaErrorMemoryAllocation ? HC_ERR_BAD_MEM_ALLOC : HC_ERR_CUDA, m);
}

void free_len(LenHost &lh)
{
    cudaFree(lh.d_mass);
    cudaFree(lh.d_seqid);
    cudaFree(lh.d_sites);
    cudaFree(lh.d_modnum);
    cudaFree(lh.d_seqs);
    cudaFree(lh.d_bA);
    cudaFree(lh.d_qA);
    cudaFree(lh.d_qp);
    cudaFree(lh.d_qion);
    cudaFree(lh.d_qAs);
    cudaFree(lh.d_qps);
    cudaFree(lh.d_cls);
    cudaFree(lh.d_rows);
    const uint32_t L = lh.L;
    lh = LenHost();
    lh.L = L;
}

static int check_params(const hc_params *p)
{
    if (!p) return HC_ERR_INVLD_PTR;
    if (p->min_len < 2 || p->max_len < p->min_len || p->max_len - p->min_len + 1 > HC_MAX_LENGTHS ||
        p->max_len > 62)
        return HC_ERR_INVLD_PARAM;
    if (p->maxz < 1 || p->maxz > (uint32_t)kMaxZ || p->scale == 0 || p->max_mass <= p->min_mass)
        return HC_ERR_INVLD_PARAM;
    if ((uint64_t)p->max_mass * p->scale >= 0x7FFFFFFFull) return HC_ERR_INVLD_PARAM;
    if (p->nmods > HC_MAX_MODS || p->topmatches > 63) return HC_ERR_INVLD_PARAM;
    if (p->dF > 16) return HC_ERR_INVLD_PARAM;  // (2dF+1) bins per peak kept in shared memory (hc_query.cu kMaxDF)
    return HC_SUCCESS;
}

static LenHost *find_len(hc_ctx *ctx, uint32_t L)
{
    if (L < ctx->p.min_len || L > ctx->p.max_len) return nullptr;
    return &ctx->lens[L - ctx->p.min_len];
}

}  // namespace hc

using namespace hc;

extern "C" {

int hc_version(void) { return 10000; }

const char *hc_status_string(int s)
{
    switch (s)
    {
    case HC_SUCCESS: return "success";
    case HC_ERR_INVLD_MEMORY: return "invalid memory";
    case HC_ERR_INVLD_PARAM: return "invalid parameter";
    case HC_ERR_INVLD_INDEX: return "invalid index";
    case HC_ERR_INVLD_SIZE: return "invalid size";
    case HC_ERR_BAD_MEM_ALLOC: return "allocation failed";
    case HC_ERR_INVLD_PTR: return "invalid pointer";
    case HC_ERR_INVLD_MOD: return "invalid modification";
    case HC_ERR_NOT_ENOUGH_DATA: return "not enough data";
    case HC_ERR_FILE_NOT_FOUND: return "file not found";
    case HC_ERR_FILE_ERROR: return "file error";
    case HC_ERR_CUDA: return "CUDA error";
    case HC_ERR_TIMEOUT: return "work still running at the deadline";
    case HC_ERR_NO_DEVICE: return "no usable CUDA device";
    default: return "unknown status";
    }
}

int hc_ctx_create(int device, const hc_params *p, hc_ctx **out)
{
    if (!out) return HC_ERR_INVLD_PTR;
    *out = nullptr;
    int rc = check_params(p);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return HC_ERR_NO_DEVICE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return HC_ERR_NO_DEVICE;
    if (prop.major < 10) return HC_ERR_NO_DEVICE;  // built for sm_103a only
    hc_ctx *ctx = new hc_ctx();
    ctx->device = device;
    ctx->p = *p;
    ctx->sm_count = prop.multiProcessorCount;
    ctx->smem_optin = prop.sharedMemPerBlockOptin;
    ctx->smem_sm = prop.sharedMemPerMultiprocessor;
    ctx->smem_reserved = prop.reservedSharedMemPerBlock;
    if (cudaSetDevice(device) != cudaSuccess) { delete ctx; return HC_ERR_NO_DEVICE; }
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
    {
        delete ctx;
        return HC_ERR_CUDA;
    }
    make_ion_tables(ctx->p, &ctx->tables);
    ctx->class_of.assign(kCodes, (uint8_t)kClassNone);
    QueryConst qc;
    make_query_const(&qc);
    {
        std::vector<double> lt(kLog10Tab);
        make_log10_table(lt.data(), kLog10Tab);
        if (cudaMalloc((void **)&ctx->d_log10, sizeof(double) * kLog10Tab) != cudaSuccess ||
            cudaMemcpy(ctx->d_log10, lt.data(), sizeof(double) * kLog10Tab, cudaMemcpyHostToDevice) != cudaSuccess)
        {
            hc_ctx_destroy(ctx);
            return HC_ERR_BAD_MEM_ALLOC;
        }
        qc.log10_tab = ctx->d_log10;
    }
    if (cudaMalloc((void **)&ctx->d_tables, sizeof(IonTables)) != cudaSuccess ||
        cudaMalloc((void **)&ctx->d_qconst, sizeof(QueryConst)) != cudaSuccess ||
        cudaMemcpy(ctx->d_tables, &ctx->tables, sizeof(IonTables), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(ctx->d_qconst, &qc, sizeof(QueryConst), cudaMemcpyHostToDevice) != cudaSuccess)
    {
        hc_ctx_destroy(ctx);
        return HC_ERR_BAD_MEM_ALLOC;
    }
    const uint32_t nlen = p->max_len - p->min_len + 1;
    ctx->lens.resize(nlen);
    for (uint32_t i = 0; i < nlen; i++) ctx->lens[i].L = p->min_len + i;
    // default launch shape: one 1024-thread CTA per SM, 2 postings chunks in
    // flight per lane, the largest scorecard tile that leaves the SM 60 KB of L1
    ctx->tuning.threads = 1024;
    ctx->tuning.tile = max_tile(ctx, p->dF, 1024);
    ctx->tuning.ctas_per_sm = 1;
    ctx->tuning.pairs_per_warp = 2;
    ctx->tuning.schedule = 0;
    ctx->tuning.defer_cap = HC_DEFER_MAX;
    ctx->tuning.small_log2 = 0;
    *out = ctx;
    return HC_SUCCESS;
}

int hc_ctx_destroy(hc_ctx *ctx)
{
    if (!ctx) return HC_ERR_INVLD_PTR;
    cudaSetDevice(ctx->device);
    for (auto &lh : ctx->lens) free_len(lh);
    cudaFree(ctx->d_lens);
    cudaFree(ctx->d_tables);
    cudaFree(ctx->d_classes);
    cudaFree(ctx->d_class_of);
    cudaFree(ctx->d_qconst);
    cudaFree(ctx->qs.d_win);
    cudaFree(ctx->qs.d_wide);
    cudaFree(ctx->qs.d_work);
    cudaFree(ctx->qs.d_order);
    cudaFree(ctx->qs.d_fitstart);
    cudaFree(ctx->d_phase);
    cudaFree(ctx->d_log10);
    cudaFree(ctx->qs.d_in);
    cudaFree(ctx->qs.d_outbuf);
    for (auto &e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->cap_stream) cudaStreamDestroy(ctx->cap_stream);
    free_stream_stage(ctx->stage);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return HC_SUCCESS;
}

const char *hc_last_error(const hc_ctx *ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int hc_ctx_set_tuning(hc_ctx *ctx, const hc_tuning *t)
{
    if (!ctx || !t) return HC_ERR_INVLD_PTR;
    if (t->threads < 64 || t->threads > 1024 || (t->threads & 31) || t->tile < kRowG || (t->tile % kRowG) ||
        t->tile > 32768 ||
        t->ctas_per_sm < 1 || t->ctas_per_sm > 8 ||
        (t->pairs_per_warp != 1 && t->pairs_per_warp != 2 && t->pairs_per_warp != 4 && t->pairs_per_warp != 8) ||
        t->schedule > 2 || t->defer_cap > HC_DEFER_MAX || t->small_log2 > 40)
        return set_error(ctx, HC_ERR_INVLD_PARAM, "bad tuning");
    const size_t need = search_smem(t->tile, ctx->p.dF, false, t->threads);
    if (t->ctas_per_sm * (need + ctx->smem_reserved) > ctx->smem_sm || need > ctx->smem_optin)
        return set_error(ctx, HC_ERR_INVLD_PARAM, "tile does not fit in shared memory");
    ctx->tuning = *t;
    return HC_SUCCESS;
}

int hc_ctx_get_tuning(const hc_ctx *ctx, hc_tuning *t)
{
    if (!ctx || !t) return HC_ERR_INVLD_PTR;
    *t = ctx->tuning;
    return HC_SUCCESS;
}

int hc_ctx_wait(hc_ctx *ctx, void *stream, double timeout_s)
{
    if (!ctx) return HC_ERR_INVLD_PTR;
    HC_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    const auto t0 = std::chrono::steady_clock::now();
    for (;;)
    {
        const cudaError_t e = cudaStreamQuery(st);
        if (e == cudaSuccess) return HC_SUCCESS;
        if (e != cudaErrorNotReady) return cuda_check(ctx, e, "hc_ctx_wait");
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_s >= 0.0 && dt >= timeout_s)
            return set_error(ctx, HC_ERR_TIMEOUT, "hc_ctx_wait: work still running at the deadline");
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

int64_t hc_make_entries(const hc_params *p, uint32_t L, const uint8_t *seqs, uint32_t npep, hc_entry *out,
                        int64_t cap)
{
    if (!p || (!seqs && npep)) return HC_ERR_INVLD_PTR;
    if (L < 2 || L > 62) return HC_ERR_INVLD_PARAM;
    return make_entries(*p, L, seqs, npep, out, out ? cap : 0);
}

static int upload_seqs(hc_ctx *ctx, LenHost &lh, const uint8_t *seqs, uint32_t npep)
{
    for (size_t i = 0; i < (size_t)npep * lh.L; i++)
        if (seqs[i] < 'A' || seqs[i] > 'Z') return set_error(ctx, HC_ERR_INVLD_PARAM, "residue outside A-Z");
    HC_CUDA(ctx, cudaMalloc((void **)&lh.d_seqs, (size_t)npep * lh.L + 1));
    HC_CUDA(ctx, cudaMemcpy(lh.d_seqs, seqs, (size_t)npep * lh.L, cudaMemcpyHostToDevice));
    lh.npep = npep;
    return HC_SUCCESS;
}

int hc_dslim_construct(hc_ctx *ctx, uint32_t L, const uint8_t *seqs, uint32_t npep, const hc_entry *order,
                       uint32_t norder)
{
    if (!ctx || (!seqs && npep)) return HC_ERR_INVLD_PTR;
    LenHost *lh = find_len(ctx, L);
    if (!lh) return set_error(ctx, HC_ERR_INVLD_PARAM, "length outside [min_len, max_len]");
    cudaSetDevice(ctx->device);
    free_len(*lh);
    int rc = upload_seqs(ctx, *lh, seqs, npep);
    if (rc) return rc;
    if (!order) return build_length_device(ctx, *lh, nullptr, true);  // entries enumerated on the device
    for (uint32_t i = 0; i < norder; i++)
        if (order[i].seqid >= npep) return set_error(ctx, HC_ERR_INVLD_INDEX, "entry seqid out of range");
    if (norder >= (1u << 24)) return set_error(ctx, HC_ERR_INVLD_SIZE, "more than 2^24 entries in one length");
    lh->n = norder;
    return build_length_device(ctx, *lh, order, false);
}

int hc_dslim_load(hc_ctx *ctx, uint32_t L, const uint8_t *seqs, uint32_t npep, const hc_entry *entries,
                  uint32_t n, const uint32_t *bA, const uint32_t *iA)
{
    if (!ctx || (!seqs && npep) || (!entries && n) || !bA || (!iA && n)) return HC_ERR_INVLD_PTR;
    LenHost *lh = find_len(ctx, L);
    if (!lh) return set_error(ctx, HC_ERR_INVLD_PARAM, "length outside [min_len, max_len]");
    if (n >= (1u << 24)) return set_error(ctx, HC_ERR_INVLD_SIZE, "more than 2^24 entries in one length");
    cudaSetDevice(ctx->device);
    free_len(*lh);
    int rc = upload_seqs(ctx, *lh, seqs, npep);
    if (rc) return rc;
    const uint32_t speclen = 2 * ctx->p.maxz * (L - 1);
    const uint64_t M = (uint64_t)n * speclen;
    const uint32_t nb = ctx->p.max_mass * ctx->p.scale;
    // the postings count must match the bucket array (the check of dslim.cpp:119-124)
    if (bA[nb] != M) return set_error(ctx, HC_ERR_INVLD_SIZE, "bA[max] != entries * speclen");
    for (uint32_t b = 0; b < nb; b++)
        if (bA[b] > bA[b + 1]) return set_error(ctx, HC_ERR_INVLD_INDEX, "bA not monotone");
    for (uint64_t i = 0; i < M; i++)
        if (iA[i] >= M) return set_error(ctx, HC_ERR_INVLD_INDEX, "iA entry out of range");
    // ids ascend inside every bucket (DSLIM_Optimize, dslim.cpp:452-482)
    for (uint32_t b = 0; b < nb; b++)
        for (uint32_t i = bA[b] + 1; i < bA[b + 1]; i++)
            if (iA[i] <= iA[i - 1]) return set_error(ctx, HC_ERR_INVLD_INDEX, "iA not ascending inside a bucket");
    for (uint32_t i = 0; i < n; i++)
        if (entries[i].seqid >= npep) return set_error(ctx, HC_ERR_INVLD_INDEX, "entry seqid out of range");
    lh->n = n;
    std::vector<float> m(n);
    std::vector<uint32_t> s(n), mo(n);
    std::vector<uint64_t> si(n);
    for (uint32_t i = 0; i < n; i++)
    {
        m[i] = entries[i].mass;
        s[i] = entries[i].seqid;
        si[i] = entries[i].sites;
        mo[i] = entries[i].modnum;
    }
    HC_CUDA(ctx, cudaMalloc((void **)&lh->d_mass, 4ull * n + 4));
    HC_CUDA(ctx, cudaMalloc((void **)&lh->d_seqid, 4ull * n + 4));
    HC_CUDA(ctx, cudaMalloc((void **)&lh->d_modnum, 4ull * n + 4));
    HC_CUDA(ctx, cudaMalloc((void **)&lh->d_sites, 8ull * n + 8));
    HC_CUDA(ctx, cudaMalloc((void **)&lh->d_bA, 4ull * (nb + 1)));
    HC_CUDA(ctx, cudaMemcpy(lh->d_mass, m.data(), 4ull * n, cudaMemcpyHostToDevice));
    HC_CUDA(ctx, cudaMemcpy(lh->d_seqid, s.data(), 4ull * n, cudaMemcpyHostToDevice));
    HC_CUDA(ctx, cudaMemcpy(lh->d_modnum, mo.data(), 4ull * n, cudaMemcpyHostToDevice));
    HC_CUDA(ctx, cudaMemcpy(lh->d_sites, si.data(), 8ull * n, cudaMemcpyHostToDevice));
    HC_CUDA(ctx, cudaMemcpy(lh->d_bA, bA, 4ull * (nb + 1), cudaMemcpyHostToDevice));
    uint32_t *d_ids = nullptr;
    HC_CUDA(ctx, cudaMalloc((void **)&d_ids, 4 * M + 4));
    HC_CUDA(ctx, cudaMemcpy(d_ids, iA, 4 * M, cudaMemcpyHostToDevice));
    lh->npost = M;
    const int rq = build_query_postings(ctx, *lh, M ? d_ids : nullptr);
    cudaFree(d_ids);
    if (rq) return rq;
    lh->built = true;
    ctx->lens_dirty = true;
    return HC_SUCCESS;
}

int hc_dslim_info(hc_ctx *ctx, uint32_t L, uint32_t *n_entries, uint64_t *n_postings)
{
    if (!ctx) return HC_ERR_INVLD_PTR;
    LenHost *lh = find_len(ctx, L);
    if (!lh) return HC_ERR_INVLD_PARAM;
    if (n_entries) *n_entries = lh->built ? lh->n : 0;
    if (n_postings) *n_postings = lh->built ? lh->npost : 0;
    return HC_SUCCESS;
}

int hc_dslim_export(hc_ctx *ctx, uint32_t L, hc_entry *entries, uint32_t *bA, uint32_t *iA)
{
    if (!ctx) return HC_ERR_INVLD_PTR;
    LenHost *lh = find_len(ctx, L);
    if (!lh || !lh->built) return set_error(ctx, HC_ERR_INVLD_INDEX, "length not built");
    cudaSetDevice(ctx->device);
    const uint32_t n = lh->n, nb = ctx->p.max_mass * ctx->p.scale;
    if (entries)
    {
        std::vector<float> m(n);
        std::vector<uint32_t> s(n), mo(n);
        std::vector<uint64_t> si(n);
        HC_CUDA(ctx, cudaMemcpy(m.data(), lh->d_mass, 4ull * n, cudaMemcpyDeviceToHost));
        HC_CUDA(ctx, cudaMemcpy(s.data(), lh->d_seqid, 4ull * n, cudaMemcpyDeviceToHost));
        HC_CUDA(ctx, cudaMemcpy(mo.data(), lh->d_modnum, 4ull * n, cudaMemcpyDeviceToHost));
        HC_CUDA(ctx, cudaMemcpy(si.data(), lh->d_sites, 8ull * n, cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < n; i++) entries[i] = hc_entry{m[i], s[i], si[i], mo[i], 0};
    }
    if (bA) HC_CUDA(ctx, cudaMemcpy(bA, lh->d_bA, 4ull * (nb + 1), cudaMemcpyDeviceToHost));
    if (iA && lh->npost)
    {
        uint32_t *d_ids = nullptr;
        HC_CUDA(ctx, cudaMalloc((void **)&d_ids, 4 * lh->npost));
        const int rc = export_ids(ctx, *lh, d_ids);
        if (rc == HC_SUCCESS) HC_CUDA(ctx, cudaMemcpy(iA, d_ids, 4 * lh->npost, cudaMemcpyDeviceToHost));
        cudaFree(d_ids);
        if (rc) return rc;
    }
    return HC_SUCCESS;
}

int hc_dslim_query_device(hc_ctx *ctx, const uint32_t *d_idx, const uint32_t *d_moz, const uint32_t *d_intensity,
                          const float *d_precurse, const double *d_dM, uint32_t nspec, uint32_t npeaks,
                          hc_result *d_out, uint32_t *d_hist, void *stream)
{
    if (!ctx) return HC_ERR_INVLD_PTR;
    if (nspec && (!d_idx || !d_moz || !d_intensity || !d_precurse || !d_out || !d_hist))
        return set_error(ctx, HC_ERR_INVLD_PTR, "null device buffer");
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    return query_device(ctx, d_idx, d_moz, d_intensity, d_precurse, d_dM, nspec, npeaks, d_out, d_hist, st);
}

int hc_dslim_query(hc_ctx *ctx, const uint32_t *idx, const uint32_t *moz, const uint32_t *intensity,
                   const float *precurse, const double *dM_per_spec, uint32_t nspec, hc_result *out,
                   uint32_t *hist)
{
    if (!ctx) return HC_ERR_INVLD_PTR;
    if (nspec == 0) return HC_SUCCESS;
    if (!idx || !moz || !intensity || !precurse || !out) return HC_ERR_INVLD_PTR;
    cudaSetDevice(ctx->device);
    const uint32_t npk = idx[nspec] - idx[0];
    for (uint32_t i = 0; i < nspec; i++)
        if (idx[i + 1] < idx[i]) return set_error(ctx, HC_ERR_INVLD_SIZE, "idx not monotone");
    // one staging buffer: idx | moz | int | prec | dM | out | hist
    const size_t b_idx = 4ull * (nspec + 1), b_pk = 4ull * npk, b_prec = 4ull * nspec;
    const size_t b_dM = dM_per_spec ? 8ull * nspec : 0, b_out = sizeof(hc_result) * nspec;
    const size_t b_hist = 4ull * HC_HIST_BINS * nspec;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t need = al(b_idx) + 2 * al(b_pk) + al(b_prec) + al(b_dM) + al(b_out) + al(b_hist);
    if (ctx->qs.in_cap < need)
    {
        cudaFree(ctx->qs.d_in);
        ctx->qs.d_in = nullptr;
        ctx->qs.in_cap = 0;
        HC_CUDA(ctx, cudaMalloc(&ctx->qs.d_in, need));
        ctx->qs.in_cap = need;
    }
    char *b = (char *)ctx->qs.d_in;
    uint32_t *d_idx = (uint32_t *)b; b += al(b_idx);
    uint32_t *d_moz = (uint32_t *)b; b += al(b_pk);
    uint32_t *d_int = (uint32_t *)b; b += al(b_pk);
    float *d_prec = (float *)b; b += al(b_prec);
    double *d_dM = dM_per_spec ? (double *)b : nullptr; b += al(b_dM);
    hc_result *d_out = (hc_result *)b; b += al(b_out);
    uint32_t *d_hist = (uint32_t *)b;
    cudaStream_t st = ctx->stream;
    std::vector<uint32_t> idx0(nspec + 1);
    for (uint32_t i = 0; i <= nspec; i++) idx0[i] = idx[i] - idx[0];
    HC_CUDA(ctx, cudaMemcpyAsync(d_idx, idx0.data(), b_idx, cudaMemcpyHostToDevice, st));
    HC_CUDA(ctx, cudaMemcpyAsync(d_moz, moz + idx[0], b_pk, cudaMemcpyHostToDevice, st));
    HC_CUDA(ctx, cudaMemcpyAsync(d_int, intensity + idx[0], b_pk, cudaMemcpyHostToDevice, st));
    HC_CUDA(ctx, cudaMemcpyAsync(d_prec, precurse, b_prec, cudaMemcpyHostToDevice, st));
    if (d_dM) HC_CUDA(ctx, cudaMemcpyAsync(d_dM, dM_per_spec, b_dM, cudaMemcpyHostToDevice, st));
    int rc = query_device(ctx, d_idx, d_moz, d_int, d_prec, d_dM, nspec, npk, d_out, d_hist, st);
    if (rc) return rc;
    HC_CUDA(ctx, cudaMemcpyAsync(out, d_out, b_out, cudaMemcpyDeviceToHost, st));
    if (hist) HC_CUDA(ctx, cudaMemcpyAsync(hist, d_hist, b_hist, cudaMemcpyDeviceToHost, st));
    HC_CUDA(ctx, cudaStreamSynchronize(st));
    return HC_SUCCESS;
}

int hc_last_launch_count(const hc_ctx *ctx) { return ctx ? ctx->last_launches : -1; }

uint64_t hc_check_division(uint32_t d, uint32_t xmax)
{
    if (d < 2) return 1;
    uint32_t m, sh;
    division_magic(d, &m, &sh);
    uint64_t bad = 0;
    for (uint32_t x = 0; x < xmax; x++)
        if ((uint32_t)(((uint64_t)x * m) >> 32) >> sh != x / d) bad++;
    return bad;
}

int hc_ctx_set_profiling(hc_ctx *ctx, int on)
{
    if (!ctx) return HC_ERR_INVLD_PTR;
    cudaSetDevice(ctx->device);
    if (on && !ctx->ev[0])
        for (auto &e : ctx->ev) HC_CUDA(ctx, cudaEventCreate(&e));
    ctx->profiling = on != 0;
    return HC_SUCCESS;
}

int hc_last_stage_times(hc_ctx *ctx, float *ms, int *nstages)
{
    if (!ctx || !ms || !nstages) return HC_ERR_INVLD_PTR;
    if (!ctx->profiling || !ctx->ev[0]) return set_error(ctx, HC_ERR_INVLD_PARAM, "profiling is off");
    const bool learned = ctx->last_learned;
    HC_CUDA(ctx, cudaEventSynchronize(ctx->ev[learned ? 5 : 4]));
    for (int i = 0; i < 4; i++) HC_CUDA(ctx, cudaEventElapsedTime(&ms[i], ctx->ev[i], ctx->ev[i + 1]));
    ms[4] = 0.0f;
    if (learned) HC_CUDA(ctx, cudaEventElapsedTime(&ms[4], ctx->ev[4], ctx->ev[5]));
    *nstages = learned ? 5 : 4;
    return HC_SUCCESS;
}

int hc_last_kernel_times(hc_ctx *ctx, float *ms_windows, float *ms_search, float *ms_wide, float *ms_tailfit)
{
    if (!ctx) return HC_ERR_INVLD_PTR;
    if (!ctx->profiling || !ctx->ev[0]) return set_error(ctx, HC_ERR_INVLD_PARAM, "profiling is off");
    HC_CUDA(ctx, cudaEventSynchronize(ctx->ev[4]));
    float t[4];
    for (int i = 0; i < 4; i++) HC_CUDA(ctx, cudaEventElapsedTime(&t[i], ctx->ev[i], ctx->ev[i + 1]));
    if (ms_windows) *ms_windows = t[0];
    if (ms_search) *ms_search = t[1];
    if (ms_wide) *ms_wide = t[2];
    if (ms_tailfit) *ms_tailfit = t[3];
    return HC_SUCCESS;
}

}  // extern "C"
