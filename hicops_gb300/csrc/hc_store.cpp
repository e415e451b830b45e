// On-disk index: the built lengths of a context written to one file and read
// back without rebuilding (the reference rebuilds its index on every run;
// hicops.cpp:174-260 calls LBE_Initialize / DSLIM_Construct per length).
//
// Layout (little-endian, as the device holds it):
//   "HCDSLIM2" | u64 params hash | u32 number of lengths
//   per length: u32 L, npep, n, entry shift of the postings (3) | u64 npost |
//               u32 nb | u64 qtotal
//               seqs u8[npep*L] | mass f32[n] | seqid u32[n] | sites u64[n] |
//               modnum u32[n] | bA u32[nb+1] | qA u32[nb+1] | qp u32[qtotal] |
//               ions u16[qtotal]
// The row tables are rebuilt on load (they are derived from qA/qp).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hc_internal.h"

namespace {

constexpr char kMagic[8] = {'H', 'C', 'D', 'S', 'L', 'I', 'M', '2'};

// FNV-1a over every parameter that changes the index's contents
uint64_t index_hash(const hc_params &p)
{
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const void *v, size_t n) {
        const unsigned char *b = static_cast<const unsigned char *>(v);
        for (size_t i = 0; i < n; i++)
        {
            h ^= b[i];
            h *= 1099511628211ull;
        }
    };
    const uint32_t u[] = {p.min_len, p.max_len, p.maxz, p.scale, p.min_mass, p.max_mass, p.nmods, p.vmods_per_pep};
    mix(u, sizeof(u));
    for (uint32_t m = 0; m < p.nmods && m < HC_MAX_MODS; m++)
    {
        mix(&p.mod_mass[m], 4);
        mix(p.mod_res[m], 4);
        mix(&p.mod_per_pep[m], 4);
    }
    return h;
}

struct File
{
    FILE *f = nullptr;
    ~File()
    {
        if (f) std::fclose(f);
    }
};

// device array <-> file through a bounded host buffer
bool put_dev(FILE *f, const void *d, size_t bytes, std::vector<char> &buf)
{
    const char *src = static_cast<const char *>(d);
    for (size_t off = 0; off < bytes; off += buf.size())
    {
        const size_t n = std::min(buf.size(), bytes - off);
        if (cudaMemcpy(buf.data(), src + off, n, cudaMemcpyDeviceToHost) != cudaSuccess) return false;
        if (std::fwrite(buf.data(), 1, n, f) != n) return false;
    }
    return true;
}

bool get_dev(FILE *f, void *d, size_t bytes, std::vector<char> &buf)
{
    char *dst = static_cast<char *>(d);
    for (size_t off = 0; off < bytes; off += buf.size())
    {
        const size_t n = std::min(buf.size(), bytes - off);
        if (std::fread(buf.data(), 1, n, f) != n) return false;
        if (cudaMemcpy(dst + off, buf.data(), n, cudaMemcpyHostToDevice) != cudaSuccess) return false;
    }
    return true;
}

template <class T>
bool put(FILE *f, const T &v) { return std::fwrite(&v, sizeof(T), 1, f) == 1; }
template <class T>
bool get(FILE *f, T &v) { return std::fread(&v, sizeof(T), 1, f) == 1; }

}  // namespace

using namespace hc;

extern "C" int hc_dslim_save(hc_ctx *ctx, const char *path)
{
    if (!ctx || !path) return HC_ERR_INVLD_PTR;
    cudaSetDevice(ctx->device);
    File fh;
    fh.f = std::fopen(path, "wb");
    if (!fh.f) return set_error(ctx, HC_ERR_FILE_NOT_FOUND, std::string("cannot create ") + path);
    FILE *f = fh.f;
    const uint32_t nb = ctx->p.max_mass * ctx->p.scale;
    uint32_t nbuilt = 0;
    for (const LenHost &lh : ctx->lens) nbuilt += lh.built ? 1u : 0u;
    bool ok = std::fwrite(kMagic, 1, 8, f) == 8 && put(f, index_hash(ctx->p)) && put(f, nbuilt);
    std::vector<char> buf(64u << 20);
    for (const LenHost &lh : ctx->lens)
    {
        if (!ok) break;
        if (!lh.built) continue;
        uint32_t qtotal32 = 0;
        if (cudaMemcpy(&qtotal32, lh.d_qA + nb, 4, cudaMemcpyDeviceToHost) != cudaSuccess) ok = false;
        const uint64_t qtotal = qtotal32;
        ok = ok && put(f, lh.L) && put(f, lh.npep) && put(f, lh.n) && put(f, kQpEntryShift) && put(f, lh.npost) &&
             put(f, nb) && put(f, qtotal);
        ok = ok && put_dev(f, lh.d_seqs, (size_t)lh.npep * lh.L, buf);
        ok = ok && put_dev(f, lh.d_mass, 4ull * lh.n, buf) && put_dev(f, lh.d_seqid, 4ull * lh.n, buf);
        ok = ok && put_dev(f, lh.d_sites, 8ull * lh.n, buf) && put_dev(f, lh.d_modnum, 4ull * lh.n, buf);
        ok = ok && put_dev(f, lh.d_bA, 4ull * (nb + 1), buf) && put_dev(f, lh.d_qA, 4ull * (nb + 1), buf);
        ok = ok && put_dev(f, lh.d_qp, 4ull * qtotal, buf) && put_dev(f, lh.d_qion, 2ull * qtotal, buf);
    }
    if (!ok || std::fflush(f) != 0) return set_error(ctx, HC_ERR_FILE_ERROR, std::string("write failed: ") + path);
    return HC_SUCCESS;
}

extern "C" int hc_dslim_restore(hc_ctx *ctx, const char *path)
{
    if (!ctx || !path) return HC_ERR_INVLD_PTR;
    cudaSetDevice(ctx->device);
    File fh;
    fh.f = std::fopen(path, "rb");
    if (!fh.f) return set_error(ctx, HC_ERR_FILE_NOT_FOUND, std::string("cannot open ") + path);
    FILE *f = fh.f;
    char magic[8];
    uint64_t hash = 0;
    uint32_t nbuilt = 0;
    if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kMagic, 8) != 0 || !get(f, hash) || !get(f, nbuilt))
        return set_error(ctx, HC_ERR_FILE_ERROR, std::string("not an index file: ") + path);
    if (hash != index_hash(ctx->p))
        return set_error(ctx, HC_ERR_INVLD_PARAM, "index file was built with other index parameters");
    const uint32_t nb_ctx = ctx->p.max_mass * ctx->p.scale;
    std::vector<char> buf(64u << 20);
    for (uint32_t k = 0; k < nbuilt; k++)
    {
        uint32_t L = 0, npep = 0, n = 0, shift = 0, nb = 0;
        uint64_t npost = 0, qtotal = 0;
        if (!(get(f, L) && get(f, npep) && get(f, n) && get(f, shift) && get(f, npost) && get(f, nb) && get(f, qtotal)))
            return set_error(ctx, HC_ERR_FILE_ERROR, "truncated index file");
        if (L < ctx->p.min_len || L > ctx->p.max_len || nb != nb_ctx || qtotal >= 0xFFFFFFFFull ||
            shift != kQpEntryShift)
            return set_error(ctx, HC_ERR_FILE_ERROR, "index file does not match this context");
        LenHost &lh = ctx->lens[L - ctx->p.min_len];
        free_len(lh);
        lh.npep = npep;
        lh.n = n;
        lh.npost = npost;
        cudaError_t e = cudaMalloc((void **)&lh.d_seqs, (size_t)npep * L + 1);
        if (e == cudaSuccess) e = cudaMalloc((void **)&lh.d_mass, 4ull * n + 4);
        if (e == cudaSuccess) e = cudaMalloc((void **)&lh.d_seqid, 4ull * n + 4);
        if (e == cudaSuccess) e = cudaMalloc((void **)&lh.d_sites, 8ull * n + 8);
        if (e == cudaSuccess) e = cudaMalloc((void **)&lh.d_modnum, 4ull * n + 4);
        if (e == cudaSuccess) e = cudaMalloc((void **)&lh.d_bA, 4ull * (nb + 1));
        if (e == cudaSuccess) e = cudaMalloc((void **)&lh.d_qA, 4ull * (nb + 1));
        if (e == cudaSuccess) e = cudaMalloc((void **)&lh.d_qp, 4ull * (qtotal + kIaPad));
        if (e == cudaSuccess) e = cudaMemset(lh.d_qp + qtotal, 0xFF, 4ull * kIaPad);
        if (e == cudaSuccess) e = cudaMalloc((void **)&lh.d_qion, 2ull * (qtotal + kIaPad));
        if (e != cudaSuccess)
        {
            free_len(lh);
            return set_error(ctx, HC_ERR_BAD_MEM_ALLOC, cudaGetErrorString(e));
        }
        bool ok = get_dev(f, lh.d_seqs, (size_t)npep * L, buf);
        ok = ok && get_dev(f, lh.d_mass, 4ull * n, buf) && get_dev(f, lh.d_seqid, 4ull * n, buf);
        ok = ok && get_dev(f, lh.d_sites, 8ull * n, buf) && get_dev(f, lh.d_modnum, 4ull * n, buf);
        ok = ok && get_dev(f, lh.d_bA, 4ull * (nb + 1), buf) && get_dev(f, lh.d_qA, 4ull * (nb + 1), buf);
        ok = ok && get_dev(f, lh.d_qp, 4ull * qtotal, buf) && get_dev(f, lh.d_qion, 2ull * qtotal, buf);
        if (!ok)
        {
            free_len(lh);
            return set_error(ctx, HC_ERR_FILE_ERROR, "truncated index file");
        }
        lh.L = L;
        int rc = check_query_postings(ctx, lh, qtotal);
        if (rc == HC_SUCCESS && n)
        {
            // entries name peptides of this length only
            std::vector<uint32_t> sid(n);
            if (cudaMemcpy(sid.data(), lh.d_seqid, 4ull * n, cudaMemcpyDeviceToHost) != cudaSuccess)
                rc = set_error(ctx, HC_ERR_CUDA, "index file: reading entries back");
            else if (*std::max_element(sid.begin(), sid.end()) >= npep)
                rc = set_error(ctx, HC_ERR_FILE_ERROR, "index file: entry names a missing peptide");
        }
        if (rc == HC_SUCCESS) rc = build_rows(ctx, lh);
        if (rc)
        {
            free_len(lh);
            return rc;
        }
        lh.built = true;
        ctx->lens_dirty = true;
    }
    return HC_SUCCESS;
}
