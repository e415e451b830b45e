// Allocation-free DSLIM query: the same search as hc_dslim_query_device, for
// callers that cannot allocate device memory while they search. A search
// service that hands all free device memory to its own pool at start-up (so
// that spectra batches of any size fit) cannot let a library cudaMalloc on
// the request path: the call would fail, or would synchronise the device and
// stall the other streams of the process. Such callers build the index and
// create the context beforehand (both allocate) and then search through this
// entry point, which only copies the small length table and launches kernels.
//
// The per-query scratch (precursor windows, overflow list, work counters,
// longest-first order, tail-fit bins, length table) lives in one file-scope
// device array of fixed size, so a call is limited to kNoAllocMaxSpectra
// spectra. Every GPU that loads the library holds the array until the
// process exits. All calls on a device share it and it keeps the last call's
// contents: calls that overlap on the GPU (different streams, or different
// contexts on the same device) race and must be serialised by the caller.
// The first call on a device does the set-up: it looks up the array's device
// address with that device current (cudaGetSymbolAddress, which may load the
// module), so make it before any stream capture. The work counters, which
// must start at zero, are cleared by every call on its own stream; every
// other scratch word is written before it is read.
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
constexpr size_t kOrderOff = kWorkOff + al(4ull * (4 + 2 * 64));
constexpr size_t kFitOff = kOrderOff + al(8ull * kNoAllocMaxSpectra);
constexpr size_t kLensOff = kFitOff + al(4ull * kNoAllocMaxSpectra);
constexpr size_t kScratchBytes = kLensOff + al(sizeof(LenDev) * HC_MAX_LENGTHS);  // about 8.5 MB

// The scratch itself. Host code must not use the symbol as an address: its
// device address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
unsigned char *g_addr[256] = {};  // device address of g_noalloc_scratch, per device ordinal

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
    if (ctx->lens.size() > HC_MAX_LENGTHS || ctx->device < 0 || ctx->device >= 256)
        return set_error(ctx, HC_ERR_INVLD_SIZE, "hc_dslim_query_noalloc: too many peptide lengths");
    if (nspec && (!d_idx || !d_moz || !d_intensity || !d_precurse || !d_out || !d_hist))
        return set_error(ctx, HC_ERR_INVLD_PTR, "null device buffer");
    HC_CUDA(ctx, cudaSetDevice(ctx->device));
    unsigned char *base = nullptr;
    {
        // set-up on the first call on this device, with the device current
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[ctx->device])
        {
            void *p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return cuda_check(ctx, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
            g_addr[ctx->device] = static_cast<unsigned char *>(p);
        }
        base = g_addr[ctx->device];
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
