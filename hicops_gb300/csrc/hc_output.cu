// PSM output in the reference's TSV format (DFile_PrintScore,
// source/core/dslim_fileout.cpp:112-152, header at 68-72): one row per
// reported spectrum with the top hit's peptide sequence and mass gathered on
// the device, numbers printed the way std::to_string prints them ("%f" for
// float and double, decimal for integers).
#include <cstdio>
#include <string>
#include <vector>

#include "hc_internal.h"

namespace hc {
namespace {

constexpr uint32_t kSeqCap = 64;  // bytes per gathered sequence (peptide lengths stay below it)

// Per reported spectrum i: the top hit (length index, entry) -> entry mass and
// the peptide's residues (zero-terminated).
__global__ void k_psm_rows(const LenDev *__restrict__ lens, const int2 *__restrict__ hits, uint32_t n,
                           float *__restrict__ mass, char *__restrict__ seq)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int2 h = hits[i];
    const LenDev d = lens[h.x];
    const uint32_t sid = d.seqid[h.y];
    mass[i] = d.mass[h.y];
    char *o = seq + (size_t)i * kSeqCap;
    const uint8_t *s = d.seqs + (size_t)sid * d.L;
    for (uint32_t k = 0; k < d.L && k + 1 < kSeqCap; k++) o[k] = (char)s[k];
    o[d.L < kSeqCap ? d.L : kSeqCap - 1] = 0;
}

}  // namespace
}  // namespace hc

using namespace hc;

extern "C" int hc_write_psms(hc_ctx *ctx, const char *path, const char *file_label, uint32_t spec_base,
                             const hc_result *res, uint32_t nspec, const float *precurse, const int32_t *charges,
                             const float *rtimes, int append)
{
    if (!ctx || !path || (nspec && (!res || !precurse))) return HC_ERR_INVLD_PTR;
    cudaSetDevice(ctx->device);
    std::vector<int2> hits;
    std::vector<uint32_t> rows;
    const uint32_t nlen = (uint32_t)ctx->lens.size();
    for (uint32_t i = 0; i < nspec; i++)
    {
        const hc_result &r = res[i];
        if (!r.reported) continue;  // the reference prints only these (dslim_query.cpp:800-812)
        if (r.idxoffset < 0 || (uint32_t)r.idxoffset >= nlen || r.psid < 0 ||
            (uint32_t)r.psid >= ctx->lens[r.idxoffset].n)
            return set_error(ctx, HC_ERR_INVLD_PARAM, "hc_write_psms: result does not belong to this index");
        hits.push_back(make_int2(r.idxoffset, r.psid));
        rows.push_back(i);
    }
    const uint32_t n = (uint32_t)hits.size();
    std::vector<float> mass(n);
    std::vector<char> seq((size_t)n * kSeqCap);
    if (n)
    {
        int rc = sync_lengths(ctx);
        if (rc) return rc;
        int2 *d_hits = nullptr;
        float *d_mass = nullptr;
        char *d_seq = nullptr;
        cudaError_t e = cudaMalloc((void **)&d_hits, sizeof(int2) * n);
        if (e == cudaSuccess) e = cudaMalloc((void **)&d_mass, 4ull * n);
        if (e == cudaSuccess) e = cudaMalloc((void **)&d_seq, (size_t)n * kSeqCap);
        if (e == cudaSuccess) e = cudaMemcpy(d_hits, hits.data(), sizeof(int2) * n, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
        {
            k_psm_rows<<<(n + 127) / 128, 128, 0, ctx->stream>>>(ctx->d_lens, d_hits, n, d_mass, d_seq);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpy(mass.data(), d_mass, 4ull * n, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(seq.data(), d_seq, (size_t)n * kSeqCap, cudaMemcpyDeviceToHost);
        cudaFree(d_hits);
        cudaFree(d_mass);
        cudaFree(d_seq);
        if (e != cudaSuccess) return set_error(ctx, HC_ERR_CUDA, cudaGetErrorString(e));
    }
    FILE *f = std::fopen(path, append ? "a" : "w");
    if (!f) return set_error(ctx, HC_ERR_FILE_NOT_FOUND, std::string("cannot open ") + path);
    if (!append)
        std::fputs("file\tscan_num\tprec_mass\tcharge\tretention_time\tpeptide\tmatched_ions\ttotal_ions\t"
                   "calc_pep_mass\tmass_diff\tmod_info\thyperscore\texpectscore\tnum_hits\n", f);
    const char *label = file_label ? file_label : "";
    for (uint32_t k = 0; k < n; k++)
    {
        const uint32_t i = rows[k];
        const hc_result &r = res[i];
        const float pm = precurse[i];
        const float md = pm - mass[k];  // float difference, as the reference computes it
        std::fprintf(f, "%s\t%u\t%f\t%d\t%f\t%s\t%u\t%u\t%f\t%f\t\t%f\t%f\t%u\n", label, spec_base + i + 1,
                     (double)pm, charges ? charges[i] : 0, (double)(rtimes ? rtimes[i] : 0.0f),
                     seq.data() + (size_t)k * kSeqCap, (unsigned)r.sharedions, (unsigned)r.totalions,
                     (double)mass[k], (double)md, (double)r.hyperscore, r.evalue, r.cpsms);
    }
    const bool bad = std::ferror(f) != 0;
    std::fclose(f);
    if (bad) return set_error(ctx, HC_ERR_FILE_ERROR, std::string("write failed: ") + path);
    return HC_SUCCESS;
}
