// Allocation-free DSLIM query: the same search as hc_dslim_query_device, for
// callers that cannot allocate device memory while they search. A search
// service that hands all free device memory to its own pool at start-up (so
// that spectra batches of any size fit) cannot let a library cudaMalloc on
// the request path: the call would fail, or would synchronise the device and
// stall the other streams of the process. Such callers build the index and
// create the context beforehand (both allocate) and then search through this
// entry point, which only launches kernels.
//
// The per-query scratch (precursor windows, overflow list, work counters,
// longest-first order, tail-fit bins, length table) lives in one file-scope
// device array of fixed size, so a call is limited to kNoAllocMaxSpectra
// spectra. Every GPU that loads the library holds the array until the
// process exits. All calls on a device share it and it keeps the last call's
// contents: calls that overlap on the GPU (different streams, or different
// contexts on the same device) race and must be serialised by the caller.
//
// Set-up. The first call in a CUDA context (normally a device's primary
// context) looks up the array's device address in that context
// (cudaGetSymbolAddress) and loads every kernel the search can launch, so
// that no later call loads code (with lazy module loading, the default, a
// kernel's first launch would load it and allocate device memory for it).
// Make that first call before any stream capture. The address and the
// loaded kernels belong to the context, so the cache is keyed by the
// context current at the call, not by the device ordinal. The work
// counters, which must start at zero, are cleared by every call on its own
// stream; every other scratch word is written before it is read.
#include <cstring>
#include <mutex>

#include "hc_internal.h"

namespace hc {
namespace {

constexpr uint32_t kNoAllocMaxSpectra = 16384;
constexpr size_t kAlign = 256;
constexpr size_t al(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }
constexpr size_t kWinOff = 0;
constexpr size_t kWideOff = kWinOff + al(sizeof(int2) * (size_t)kNoAllocMaxSpectra * HC_MAX_LENGTHS);
constexpr size_t kWorkOff = kWideOff + al(4ull * (kNoAllocMaxSpectra + 4));
constexpr size_t kOrderOff = kWorkOff + al(4ull * kWorkWords);
constexpr size_t kFitOff = kOrderOff + al(8ull * kNoAllocMaxSpectra);
constexpr size_t kLensOff = kFitOff + al(4ull * kNoAllocMaxSpectra);
constexpr size_t kScratchBytes = kLensOff + al(sizeof(LenDev) * HC_MAX_LENGTHS);  // about 8.5 MB

// The scratch itself. Host code must not use the symbol as an address: its
// device address comes from cudaGetSymbolAddress, once per CUDA context.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;

// One set-up per CUDA context: its handle and the array's address in it.
struct CtxSlot
{
    void *cu_ctx;
    unsigned char *addr;
};
constexpr int kMaxCtx = 64;
CtxSlot g_slot[kMaxCtx] = {};
int g_nslot = 0;

// cuCtxGetCurrent from the driver, looked up once through the runtime (the
// library does not link the driver library itself)
using CtxGetCurrent = int (*)(void **);
CtxGetCurrent ctx_get_current()
{
    static CtxGetCurrent fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<CtxGetCurrent>(f);
    }();
    return fn;
}

// The array's address in the current context, setting the context up on
// its first call. Caller holds g_mu and has made the context's device current.
int scratch_address(hc_ctx *ctx, unsigned char **out)
{
    // a runtime call first, so that the device's primary context is current
    // when the caller has not made another one current
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_check(ctx, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    void *cur = nullptr;
    const CtxGetCurrent get = ctx_get_current();
    if (!get || get(&cur) != 0 || !cur)
        return set_error(ctx, HC_ERR_CUDA, "hc_dslim_query_noalloc: no current CUDA context");
    for (int i = 0; i < g_nslot; i++)
        if (g_slot[i].cu_ctx == cur)
        {
            *out = g_slot[i].addr;
            return HC_SUCCESS;
        }
    if (g_nslot == kMaxCtx) return set_error(ctx, HC_ERR_INVLD_SIZE, "hc_dslim_query_noalloc: too many CUDA contexts");
    const int rc = preload_query_kernels(ctx);
    if (rc) return rc;
    g_slot[g_nslot++] = CtxSlot{cur, static_cast<unsigned char *>(p)};
    *out = static_cast<unsigned char *>(p);
    return HC_SUCCESS;
}

}  // namespace
}  // namespace hc

using namespace hc;

extern "C" int hc_dslim_query_noalloc(hc_ctx *ctx, const uint32_t *d_idx, const uint32_t *d_moz,
                                      const uint32_t *d_intensity, const float *d_precurse, const double *d_dM,
                                      uint32_t nspec, uint32_t npeaks, hc_result *d_out, uint32_t *d_hist,
                                      void *stream)
{
    (void)npeaks;
    if (!ctx) return HC_ERR_INVLD_PTR;
    if (nspec > kNoAllocMaxSpectra)
        return set_error(ctx, HC_ERR_INVLD_SIZE, "hc_dslim_query_noalloc: more than 16384 spectra in one call");
    if (ctx->lens.size() > HC_MAX_LENGTHS)
        return set_error(ctx, HC_ERR_INVLD_SIZE, "hc_dslim_query_noalloc: too many peptide lengths");
    if (nspec && (!d_idx || !d_moz || !d_intensity || !d_precurse || !d_out || !d_hist))
        return set_error(ctx, HC_ERR_INVLD_PTR, "null device buffer");
    HC_CUDA(ctx, cudaSetDevice(ctx->device));
    unsigned char *base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        const int rc = scratch_address(ctx, &base);
        if (rc) return rc;
    }
    ScratchPtrs s;
    s.win = reinterpret_cast<int2 *>(base + kWinOff);
    s.wide = reinterpret_cast<uint32_t *>(base + kWideOff);
    s.work = reinterpret_cast<uint32_t *>(base + kWorkOff);
    s.order = reinterpret_cast<uint32_t *>(base + kOrderOff);
    s.fitstart = reinterpret_cast<int32_t *>(base + kFitOff);
    s.lens = reinterpret_cast<LenDev *>(base + kLensOff);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    return launch_query_scratch(ctx, d_idx, d_moz, d_intensity, d_precurse, d_dM, nspec, d_out, d_hist, s, st);
}
