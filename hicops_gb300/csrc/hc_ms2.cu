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
#include <algorithm>
#include <string>
#include <thread>
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

// One line of the file: [p, e), cut at its first NUL byte as the reference's
// strtok on c_str() cuts it. The '\n' is not part of it; a '\r' before it is
// (std::getline keeps it).
struct Line
{
    const char *p, *e;
};

// strtok_r on a line: the next token after runs of ' ' (and '\t' if `tab`)
bool next_tok(const char *&p, const char *e, bool tab, const char *&tb, const char *&te)
{
    while (p < e && (*p == ' ' || (tab && *p == '\t'))) p++;
    if (p >= e) return false;
    tb = p;
    while (p < e && *p != ' ' && !(tab && *p == '\t')) p++;
    te = p;
    return true;
}

// atof / atoi of a token (the token is copied so the conversion cannot read past it)
double tok_atof(const char *tb, const char *te, double dflt, bool have)
{
    if (!have) return dflt;
    char buf[64];
    const size_t n = (size_t)(te - tb);
    if (n < sizeof(buf))
    {
        std::memcpy(buf, tb, n);
        buf[n] = 0;
        return std::atof(buf);
    }
    return std::atof(std::string(tb, n).c_str());
}

int tok_atoi(const char *tb, const char *te, int dflt, bool have)
{
    if (!have) return dflt;
    char buf[64];
    const size_t n = (size_t)(te - tb);
    if (n < sizeof(buf))
    {
        std::memcpy(buf, tb, n);
        buf[n] = 0;
        return std::atoi(buf);
    }
    return std::atoi(std::string(tb, n).c_str());
}

// The spectra of one stretch of the file. Every stretch but the first starts
// at an 'S' line; the first holds the file's first 'S' line. A spectrum's
// charge / precursor (a 'Z' line) and retention time (an 'I RTime' line) are
// recorded only when one of its lines sets them: the others inherit the
// previous spectrum's values, which are known once the stretches are joined.
struct Stretch
{
    std::vector<uint8_t> zset, rset;
    std::vector<uint32_t> z;
    std::vector<double> prec, rt;
    std::vector<uint64_t> npk;
    std::vector<uint32_t> mz, intn;
    uint64_t peak_lines = 0;
};

void parse_stretch(const char *b, const char *e, bool first, double scale, Stretch &out)
{
    bool started = false;
    uint8_t zs = 0, rs = 0;
    uint32_t z = 0;
    double prec = 0.0, rt = 0.0;
    uint64_t cur = 0;
    auto close = [&]() {
        out.zset.push_back(zs);
        out.rset.push_back(rs);
        out.z.push_back(z);
        out.prec.push_back(prec);
        out.rt.push_back(rt);
        out.npk.push_back(cur);
        zs = rs = 0;
        cur = 0;
    };
    const char *p = b;
    while (p < e)
    {
        const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(e - p)));
        const char *le = nl ? nl : e;
        Line ln{p, le};
        p = nl ? nl + 1 : e;
        if (ln.p == ln.e) continue;  // empty line
        const char c = *ln.p;
        const char *zero = static_cast<const char *>(std::memchr(ln.p, 0, (size_t)(ln.e - ln.p)));
        const char *ee = zero ? zero : ln.e;
        const char *q = ln.p, *tb = nullptr, *te = nullptr;
        if (c == 'H' || c == 'D') continue;
        if (c == 'Z')
        {
            next_tok(q, ee, true, tb, te);
            bool h = next_tok(q, ee, true, tb, te);
            z = (uint32_t)tok_atoi(tb, te, 1, h);
            h = next_tok(q, ee, true, tb, te);
            prec = tok_atof(tb, te, 0.01, h);
            zs = 1;
        }
        else if (c == 'I')
        {
            next_tok(q, ee, true, tb, te);
            if (next_tok(q, ee, true, tb, te) && te - tb == 5 && std::memcmp(tb, "RTime", 5) == 0)
            {
                const bool h = next_tok(q, ee, true, tb, te);
                rt = tok_atof(tb, te, 0.00, h);
                rs = 1;
            }
        }
        else if (c == 'S')
        {
            if (started) close();
            started = true;
        }
        else
        {
            // a peak: tokens split on ' ' only (msquery.cpp:388-404, 478-498); a
            // missing token reads "0.01" in the file's first spectrum, "0.0" after
            const double dflt = (first && out.npk.empty()) ? 0.01 : 0.0;
            bool h = next_tok(q, ee, false, tb, te);
            const double mzv = tok_atof(tb, te, dflt, h);
            h = next_tok(q, ee, false, tb, te);
            const double iv = tok_atof(tb, te, dflt, h);
            out.mz.push_back((uint32_t)(mzv * scale));
            out.intn.push_back((uint32_t)(iv * 1000));
            cur++;
            out.peak_lines++;
        }
    }
    if (started) close();
}

// position of the next line start at or after p that begins with 'S' (or e)
const char *next_s_line(const char *base, const char *p, const char *e)
{
    if (p > base && p[-1] != '\n')
    {
        const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(e - p)));
        if (!nl) return e;
        p = nl + 1;
    }
    while (p < e)
    {
        if (*p == 'S') return p;
        const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(e - p)));
        if (!nl) return e;
        p = nl + 1;
    }
    return e;
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

extern "C" int hc_ms2_read(const char *path, uint32_t scale_u, hc_ms2 **out, uint32_t *nspec, uint32_t *maxslen)
{
    if (!path || !out) return HC_ERR_INVLD_PTR;
    *out = nullptr;
    FILE *f = std::fopen(path, "rb");
    if (!f) return HC_ERR_FILE_ERROR;
    std::vector<char> buf;
    bool rerr = std::fseek(f, 0, SEEK_END) != 0;
    const long fsz = rerr ? -1 : std::ftell(f);
    rerr = rerr || fsz < 0 || std::fseek(f, 0, SEEK_SET) != 0;
    if (!rerr)
    {
        buf.resize((size_t)fsz + 1);
        rerr = std::fread(buf.data(), 1, (size_t)fsz, f) != (size_t)fsz;
        buf[(size_t)fsz] = 0;
    }
    std::fclose(f);
    if (rerr) return HC_ERR_FILE_ERROR;
    const char *base = buf.data(), *end = base + (buf.size() - 1);
    const double scale = (double)scale_u;

    // stretches: the first runs from the file start through its first 'S'
    // line; the others start at 'S' lines, about equal in size
    const char *s0 = next_s_line(base, base, end);
    const unsigned hw = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    const size_t span = (size_t)(end - s0);
    const unsigned nt = s0 < end ? (unsigned)std::max<size_t>(1, std::min<size_t>(hw, span / (1u << 20) + 1)) : 1u;
    std::vector<const char *> cut{base};
    for (unsigned k = 1; k < nt; k++)
    {
        const char *c = next_s_line(base, s0 + 1 + span * k / nt, end);
        if (c > cut.back() && c < end) cut.push_back(c);
    }
    cut.push_back(end);
    const size_t ns_ = cut.size() - 1;
    std::vector<Stretch> parts(ns_);
    {
        std::vector<std::thread> th;
        for (size_t k = 1; k < ns_; k++)
            th.emplace_back([&, k]() { parse_stretch(cut[k], cut[k + 1], false, scale, parts[k]); });
        parse_stretch(cut[0], cut[1], true, scale, parts[0]);
        for (auto &t : th) t.join();
    }

    // join: inherit charge / precursor / retention time in file order (the
    // reference's spectrum_t starts zeroed, msquery.cpp:27-42)
    hc_ms2 *m = new hc_ms2();
    uint64_t peak_lines = 0, nsp = 0, npk = 0;
    for (const Stretch &st : parts)
    {
        peak_lines += st.peak_lines;
        nsp += st.npk.size();
        npk += st.mz.size();
    }
    m->off.reserve(nsp + 1);
    m->prec.reserve(nsp);
    m->z.reserve(nsp);
    m->rtime.reserve(nsp);
    m->mz.reserve(npk);
    m->intn.reserve(npk);
    m->off.push_back(0);
    uint32_t cz = 0;
    double cprec = 0.0, crt = 0.0;
    for (const Stretch &st : parts)
    {
        for (size_t i = 0; i < st.npk.size(); i++)
        {
            if (st.zset[i])
            {
                cz = st.z[i];
                cprec = st.prec[i];
            }
            if (st.rset[i]) crt = st.rt[i];
            m->z.push_back(cz);
            m->prec.push_back(cprec);
            m->rtime.push_back(crt);
            m->off.push_back(m->off.back() + st.npk[i]);
            if (st.npk[i] > m->maxslen) m->maxslen = (uint32_t)std::min<uint64_t>(st.npk[i], 0xFFFFFFFFu);
        }
        // peaks of a stretch without an 'S' line (only possible with no 'S' at all) belong to no spectrum
        const uint64_t used = m->off.back() - m->mz.size();
        m->mz.insert(m->mz.end(), st.mz.begin(), st.mz.begin() + (ptrdiff_t)used);
        m->intn.insert(m->intn.end(), st.intn.begin(), st.intn.begin() + (ptrdiff_t)used);
    }
    // MSQuery::initialize: no peak line at all is ERR_INVLD_SIZE (msquery.cpp:143-147)
    if (peak_lines == 0 || m->mz.size() >= 0xFFFFFFFFull || m->off.size() > 0xFFFFFFFFull)
    {
        delete m;
        return HC_ERR_INVLD_SIZE;
    }
    *out = m;
    if (nspec) *nspec = (uint32_t)m->prec.size();
    if (maxslen) *maxslen = m->maxslen;
    return HC_SUCCESS;
}

extern "C" int hc_ms2_open(hc_ctx *ctx, const char *path, hc_ms2 **out, uint32_t *nspec, uint32_t *maxslen)
{
    if (!ctx || !path || !out) return HC_ERR_INVLD_PTR;
    const int rc = hc_ms2_read(path, ctx->p.scale, out, nspec, maxslen);
    if (rc == HC_ERR_FILE_ERROR) return set_error(ctx, rc, std::string("cannot read ") + path);
    if (rc == HC_ERR_INVLD_SIZE) return set_error(ctx, rc, std::string("no peaks (or 2^32 or more) in ") + path);
    return rc;
}

extern "C" int hc_ms2_raw(const hc_ms2 *m, uint32_t first, uint32_t count, uint64_t *off, uint32_t *mz,
                          uint32_t *intensity, double *prec, uint32_t *z, double *rtime)
{
    if (!m || !off) return HC_ERR_INVLD_PTR;
    const uint64_t total = m->prec.size();
    if ((uint64_t)first + count > total) return HC_ERR_INVLD_SIZE;
    const uint64_t a = m->off[first];
    for (uint32_t k = 0; k <= count; k++) off[k] = m->off[first + k] - a;
    const uint64_t n = m->off[first + count] - a;
    if (mz && n) std::memcpy(mz, m->mz.data() + a, 4 * n);
    if (intensity && n) std::memcpy(intensity, m->intn.data() + a, 4 * n);
    for (uint32_t k = 0; k < count; k++)
    {
        if (prec) prec[k] = m->prec[first + k];
        if (z) z[k] = m->z[first + k];
        if (rtime) rtime[k] = m->rtime[first + k];
    }
    return HC_SUCCESS;
}

extern "C" int hc_ms2_close(hc_ms2 *m)
{
    if (!m) return HC_SUCCESS;
    if (m->cap_spec)  // a reader that never extracted made no CUDA call
    {
        cudaSetDevice(m->device);
        free_scratch(m);
    }
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
    if (m->cap_spec && m->device != ctx->device)  // scratch of another device
    {
        cudaSetDevice(m->device);
        free_scratch(m);
    }
    cudaSetDevice(ctx->device);
    m->device = ctx->device;
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
