// MS2 ingestion. The host reads an MS2 text file the way the reference's
// MSQuery::initialize / readspectrum do (source/core/msquery.cpp:88-178,
// 300-505) and keeps the raw peaks; hc_ms2_extract then hands out batches the
// way MSQuery::extractbatch does (msquery.cpp:239-297), with the peak picking
// of MSQuery::pickpeaks (msquery.cpp:509-569) on the device, one thread per
// spectrum: sort the peaks by intensity with the reference's quicksort
// (KeyVal_Parallel_Internal, source/core/include/keyval.h:48-104: Hoare
// partition around the middle key, which fixes the order of equal
// intensities), set the top peak to base_int, scale the next QALEN-1 by
// base_int / top (truncated to integers) and keep the highest ones that
// reach min_int. A second kernel prefix-sums the kept counts and a third
// copies the kept peaks into the CSR batch.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "hc_internal.h"

struct hc_ms2
{
    int device = 0;
    std::vector<uint64_t> off;  // raw peaks of spectrum s: [off[s], off[s+1])
    std::vector<uint32_t> mz, intn;
    std::vector<double> prec, rtime;
    std::vector<uint32_t> z;  // the reference keeps the charge unsigned (msquery.hpp _Spectrum::Z)
    uint32_t maxslen = 0;
    // device scratch, grown on demand
    uint64_t *d_off = nullptr;
    uint32_t *d_mz = nullptr, *d_int = nullptr, *d_idx = nullptr, *d_omz = nullptr, *d_oint = nullptr;
    size_t cap_spec = 0, cap_raw = 0;
};

namespace hc {
namespace {

constexpr int kSortStack = 128;  // the smaller side is sorted first: at most 2*32 levels

// KeyVal_Parallel_Internal (keyval.h:48-104) without recursion: its two
// recursive calls cover disjoint ranges, so the order they run in does not
// change the result. Pushing the larger side first bounds the stack.
__device__ bool key_sort(uint32_t *key, uint32_t *val, int n)
{
    if (n < 2) return true;
    int stack[kSortStack];
    int sp = 0;
    stack[sp++] = 0;
    stack[sp++] = n - 1;
    while (sp > 0)
    {
        const int right = stack[--sp], left = stack[--sp];
        int i = left, j = right;
        const uint32_t pivot = key[(left + right) / 2];
        while (i <= j)
        {
            while (key[i] < pivot) i++;
            while (key[j] > pivot) j--;
            if (i <= j)
            {
                const uint32_t k = key[i], v = val[i];
                key[i] = key[j];
                val[i] = val[j];
                key[j] = k;
                val[j] = v;
                i++;
                j--;
            }
        }
        if (sp + 4 > kSortStack) return false;
        const bool lo = left < j, hi = i < right;
        if (j - left > right - i)
        {
            if (lo) { stack[sp++] = left; stack[sp++] = j; }
            if (hi) { stack[sp++] = i; stack[sp++] = right; }
        }
        else
        {
            if (hi) { stack[sp++] = i; stack[sp++] = right; }
            if (lo) { stack[sp++] = left; stack[sp++] = j; }
        }
    }
    return true;
}

// Spectra [0, nspec) of the batch; raw offsets relative to off[0].
__global__ void k_pick(const uint64_t *__restrict__ off, uint32_t *__restrict__ mz, uint32_t *__restrict__ intn,
                       uint32_t nspec, uint32_t base_int, uint32_t min_int, uint32_t *__restrict__ count)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nspec) return;
    const uint64_t o = off[s] - off[0];
    const int n = (int)(off[s + 1] - off[s]);
    uint32_t *it = intn + o, *ms = mz + o;
    if (!key_sort(it, ms, n))
    {
        count[s] = 0xFFFFFFFFu;  // cannot happen with the stack bound above; reported as an error
        return;
    }
    uint32_t keep = 0;
    if (n > 0)
    {
        const uint32_t top = it[n - 1];
        const double factor = (double)base_int / (double)top;
        it[n - 1] = base_int;
        keep = 1;
        for (int j = n - 2; j >= n - (int)HC_QALEN && j >= 0; j--)
        {
            // an all-zero spectrum scales 0 * inf = NaN, which converts to 0
            it[j] = top ? (uint32_t)((double)it[j] * factor) : 0u;
            if (it[j] >= min_int) keep++;
        }
    }
    count[s] = keep;
}

// In-place inclusive prefix sum of the kept counts in one block: on entry
// idx[1..n] holds the counts, on exit idx[s] is where spectrum s starts.
// Sets idx[n+1] = 1 when a sort reported failure.
__global__ void k_scan(uint32_t *__restrict__ idx, uint32_t n)
{
    __shared__ uint32_t warp_sum[32];
    __shared__ uint32_t carry;
    __shared__ uint32_t bad;
    const uint32_t t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (t == 0)
    {
        carry = 0;
        bad = 0;
        idx[0] = 0;
    }
    __syncthreads();
    for (uint32_t base = 0; base < n; base += blockDim.x)
    {
        const uint32_t s = base + t;
        uint32_t v = s < n ? idx[s + 1] : 0u;
        if (v == 0xFFFFFFFFu)
        {
            bad = 1;
            v = 0;
        }
        uint32_t x = v;
        for (int d = 1; d < 32; d <<= 1)
        {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
            if (lane >= (uint32_t)d) x += y;
        }
        if (lane == 31) warp_sum[w] = x;
        __syncthreads();
        if (w == 0)
        {
            uint32_t ws = lane < (blockDim.x >> 5) ? warp_sum[lane] : 0u;
            for (int d = 1; d < 32; d <<= 1)
            {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, ws, d);
                if (lane >= (uint32_t)d) ws += y;
            }
            warp_sum[lane] = ws;
        }
        __syncthreads();
        const uint32_t incl = carry + (w ? warp_sum[w - 1] : 0u) + x;
        if (s < n) idx[s + 1] = incl;
        __syncthreads();
        if (t == blockDim.x - 1) carry = incl;
        __syncthreads();
    }
    if (t == 0) idx[n + 1] = bad;
}

// the kept peaks (the last k of each sorted spectrum) into the CSR batch,
// one warp per spectrum
__global__ void k_pick_copy(const uint64_t *__restrict__ off, const uint32_t *__restrict__ mz,
                            const uint32_t *__restrict__ intn, uint32_t nspec, const uint32_t *__restrict__ idx,
                            uint32_t *__restrict__ omz, uint32_t *__restrict__ oint)
{
    const uint32_t s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= nspec) return;
    const uint32_t k = idx[s + 1] - idx[s];
    const uint64_t src = off[s + 1] - off[0] - k;
    for (uint32_t t = threadIdx.x & 31; t < k; t += 32)
    {
        omz[idx[s] + t] = mz[src + t];
        oint[idx[s] + t] = intn[src + t];
    }
}

// strtok_r: next token delimited by runs of any byte in `delim`
const char *next_tok(const char *&p, const char *delim, size_t &len)
{
    while (*p && std::strchr(delim, *p)) p++;
    if (!*p) return nullptr;
    const char *b = p;
    while (*p && !std::strchr(delim, *p)) p++;
    len = (size_t)(p - b);
    return b;
}

std::string tok_or(const char *b, size_t len, const char *dflt) { return b ? std::string(b, len) : std::string(dflt); }

// std::getline: the '\n' is dropped, a '\r' before it stays
bool read_line(FILE *f, std::string &line)
{
    line.clear();
    char buf[4096];
    bool any = false;
    while (std::fgets(buf, sizeof(buf), f))
    {
        any = true;
        const size_t n = std::strlen(buf);
        if (n && buf[n - 1] == '\n')
        {
            line.append(buf, n - 1);
            return true;
        }
        line.append(buf, n);
    }
    return any;
}

void free_scratch(hc_ms2 *m)
{
    cudaFree(m->d_off);
    cudaFree(m->d_mz);
    cudaFree(m->d_int);
    cudaFree(m->d_idx);
    cudaFree(m->d_omz);
    cudaFree(m->d_oint);
    m->d_off = nullptr;
    m->d_mz = m->d_int = m->d_idx = m->d_omz = m->d_oint = nullptr;
    m->cap_spec = m->cap_raw = 0;
}

}  // namespace
}  // namespace hc

using namespace hc;

extern "C" int hc_ms2_open(hc_ctx *ctx, const char *path, hc_ms2 **out, uint32_t *nspec, uint32_t *maxslen)
{
    if (!ctx || !path || !out) return HC_ERR_INVLD_PTR;
    *out = nullptr;
    FILE *f = std::fopen(path, "rb");
    if (!f) return set_error(ctx, HC_ERR_FILE_ERROR, std::string("cannot open ") + path);
    hc_ms2 *m = new hc_ms2();
    m->device = ctx->device;
    const double scale = (double)ctx->p.scale;
    // MSQuery keeps Z, precursor and retention time in one spectrum_t that is
    // overwritten line by line, so a spectrum without those lines inherits them
    uint32_t z = 0;
    double prec = 0.0, rt = 0.0;
    bool started = false;
    uint32_t cur = 0;
    std::string line;
    m->off.push_back(0);
    auto close_spectrum = [&]() {
        m->prec.push_back(prec);
        m->z.push_back(z);
        m->rtime.push_back(rt);
        m->off.push_back(m->mz.size());
        if (cur > m->maxslen) m->maxslen = cur;
        cur = 0;
    };
    while (read_line(f, line))
    {
        if (line.empty() || line[0] == 'H' || line[0] == 'D') continue;
        const char *p = line.c_str();
        size_t len = 0;
        if (line[0] == 'Z')
        {
            next_tok(p, " \t", len);
            const char *a = next_tok(p, " \t", len);
            z = (uint32_t)std::atoi(tok_or(a, len, "1").c_str());
            const char *b = next_tok(p, " \t", len);
            prec = std::atof(tok_or(b, len, "0.01").c_str());
        }
        else if (line[0] == 'I')
        {
            next_tok(p, " \t", len);
            const char *a = next_tok(p, " \t", len);
            if (a && std::string(a, len) == "RTime")
            {
                const char *b = next_tok(p, " \t", len);
                rt = std::atof(tok_or(b, len, "0.00").c_str());
            }
        }
        else if (line[0] == 'S')
        {
            if (started) close_spectrum();
            started = true;
        }
        else
        {
            // a peak: tokens split on ' ' only (msquery.cpp:388-404, 478-498)
            const char *dflt = m->prec.empty() ? "0.01" : "0.0";
            const char *a = next_tok(p, " ", len);
            const double mzv = std::atof(tok_or(a, len, dflt).c_str());
            const char *b = next_tok(p, " ", len);
            const double iv = std::atof(tok_or(b, len, dflt).c_str());
            m->mz.push_back((uint32_t)(mzv * scale));
            m->intn.push_back((uint32_t)(iv * 1000));
            cur++;
        }
    }
    const bool rerr = std::ferror(f) != 0;
    std::fclose(f);
    if (started) close_spectrum();
    if (rerr)
    {
        delete m;
        return set_error(ctx, HC_ERR_FILE_ERROR, std::string("read failed: ") + path);
    }
    if (m->mz.empty())
    {
        // MSQuery::initialize: no peak line at all (msquery.cpp:143-147)
        delete m;
        return set_error(ctx, HC_ERR_INVLD_SIZE, std::string("no peaks in ") + path);
    }
    if (m->mz.size() >= 0xFFFFFFFFull || m->off.size() > 0xFFFFFFFFull)
    {
        delete m;
        return set_error(ctx, HC_ERR_INVLD_SIZE, "MS2 file holds 2^32 peaks or more");
    }
    *out = m;
    if (nspec) *nspec = (uint32_t)m->prec.size();
    if (maxslen) *maxslen = m->maxslen;
    return HC_SUCCESS;
}

extern "C" int hc_ms2_close(hc_ms2 *m)
{
    if (!m) return HC_SUCCESS;
    cudaSetDevice(m->device);
    free_scratch(m);
    delete m;
    return HC_SUCCESS;
}

extern "C" int hc_ms2_extract(hc_ctx *ctx, hc_ms2 *m, uint32_t first, uint32_t count, uint32_t *idx, uint32_t *moz,
                              uint32_t *intensity, float *precurse, int32_t *charges, float *rtimes, uint32_t *nout,
                              uint64_t *npeaks)
{
    if (!ctx || !m || !idx) return HC_ERR_INVLD_PTR;
    const uint32_t total = (uint32_t)m->prec.size();
    if (first > total) return set_error(ctx, HC_ERR_INVLD_SIZE, "hc_ms2_extract: first spectrum past the end");
    const uint32_t n = count < total - first ? count : total - first;  // extractbatch clamps (msquery.cpp:254-258)
    if (nout) *nout = n;
    if (npeaks) *npeaks = 0;
    for (uint32_t k = 0; k < n; k++)
    {
        const uint32_t s = first + k;
        const uint32_t zu = m->z[s];
        if (precurse) precurse[k] = (float)m->prec[s];
        if (charges) charges[k] = (int32_t)(1u > zu ? 1u : zu);                  // MAX(1, Z), unsigned compare
        if (rtimes) rtimes[k] = (float)(0.0 > m->rtime[s] ? 0.0 : m->rtime[s]);  // MAX(0.0, rtime)
    }
    idx[0] = 0;
    if (n == 0) return HC_SUCCESS;
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    const uint64_t r0 = m->off[first], r1 = m->off[first + n];
    const size_t nraw = (size_t)(r1 - r0);
    cudaError_t e = cudaSuccess;
    if (m->cap_spec < n || m->cap_raw < nraw + 1)
    {
        free_scratch(m);
        const size_t cs = n, cr = nraw + 1;
        e = cudaMalloc((void **)&m->d_off, 8ull * (cs + 1));
        if (e == cudaSuccess) e = cudaMalloc((void **)&m->d_idx, 4ull * (cs + 2));
        if (e == cudaSuccess) e = cudaMalloc((void **)&m->d_mz, 4ull * cr);
        if (e == cudaSuccess) e = cudaMalloc((void **)&m->d_int, 4ull * cr);
        if (e == cudaSuccess) e = cudaMalloc((void **)&m->d_omz, 4ull * cr);
        if (e == cudaSuccess) e = cudaMalloc((void **)&m->d_oint, 4ull * cr);
        if (e != cudaSuccess)
        {
            free_scratch(m);
            return set_error(ctx, HC_ERR_BAD_MEM_ALLOC, cudaGetErrorString(e));
        }
        m->cap_spec = cs;
        m->cap_raw = cr;
    }
    uint32_t bad = 0;
    e = cudaMemcpyAsync(m->d_off, m->off.data() + first, 8ull * (n + 1), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nraw)
        e = cudaMemcpyAsync(m->d_mz, m->mz.data() + r0, 4ull * nraw, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nraw)
        e = cudaMemcpyAsync(m->d_int, m->intn.data() + r0, 4ull * nraw, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
    {
        k_pick<<<(n + 127) / 128, 128, 0, st>>>(m->d_off, m->d_mz, m->d_int, n, (uint32_t)ctx->p.base_int,
                                               (uint32_t)ctx->p.min_int, m->d_idx + 1);
        k_scan<<<1, 1024, 0, st>>>(m->d_idx, n);
        k_pick_copy<<<(n + 7) / 8, 256, 0, st>>>(m->d_off, m->d_mz, m->d_int, n, m->d_idx, m->d_omz, m->d_oint);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(idx, m->d_idx, 4ull * (n + 1), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, m->d_idx + n + 1, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_error(ctx, HC_ERR_CUDA, cudaGetErrorString(e));
    if (bad) return set_error(ctx, HC_ERR_CUDA, "hc_ms2_extract: peak sort stack exhausted");
    const uint32_t kept = idx[n];
    if (kept && moz) e = cudaMemcpyAsync(moz, m->d_omz, 4ull * kept, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && kept && intensity)
        e = cudaMemcpyAsync(intensity, m->d_oint, 4ull * kept, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_error(ctx, HC_ERR_CUDA, cudaGetErrorString(e));
    if (npeaks) *npeaks = kept;
    return HC_SUCCESS;
}
