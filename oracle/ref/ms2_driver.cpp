/*
 * Runs the reference MS2 reader and peak picker, unmodified, on one MS2 file
 * (TEST INFRASTRUCTURE: pins the CPU restatement in oracle/ms2.py and makes
 * golden vectors for the device path).
 *
 *   ms2_driver <file.ms2> <scale> <base_int> <min_int> <out.bin>
 *
 * MSQuery::initialize (source/core/msquery.cpp:88-178) then
 * MSQuery::extractbatch (msquery.cpp:239-297) batch after batch of QCHUNK
 * spectra, as the reference's query loop drives it. out.bin:
 *   i32 status | u32 nspec | u32 npeaks | u32 idx[nspec+1] | u32 moz[npeaks] |
 *   u32 intensity[npeaks] | f32 precurse[nspec] | i32 charges[nspec] |
 *   f32 rtimes[nspec]
 */
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "msquery.hpp"

gParams params;

int main(int argc, char **argv)
{
    if (argc != 6)
    {
        std::fprintf(stderr, "usage: %s file.ms2 scale base_int min_int out.bin\n", argv[0]);
        return 2;
    }
    params.scale = (uint_t)std::strtoul(argv[2], nullptr, 10);
    params.base_int = (int_t)std::strtol(argv[3], nullptr, 10);
    params.min_int = (int_t)std::strtol(argv[4], nullptr, 10);

    std::vector<uint32_t> idx(1, 0), moz, inten;
    std::vector<float> prec, rt;
    std::vector<int32_t> z;

    MSQuery q;
    string_t fname(argv[1]);
    int32_t status = q.initialize(&fname, 0);
    if (status == SLM_SUCCESS)
    {
        Queries b;
        b.init();
        int_t rem = (int_t)q.getQAcount();
        while (rem > 0 && status == SLM_SUCCESS)
        {
            b.reset();
            status = q.extractbatch(QCHUNK, &b, rem);
            const uint32_t base = idx.back();
            for (int_t s = 0; s < b.numSpecs; s++)
            {
                idx.push_back(base + b.idx[s + 1]);
                prec.push_back(b.precurse[s]);
                z.push_back(b.charges[s]);
                rt.push_back(b.rtimes[s]);
            }
            moz.insert(moz.end(), b.moz, b.moz + b.idx[b.numSpecs]);
            inten.insert(inten.end(), b.intensity, b.intensity + b.idx[b.numSpecs]);
        }
        b.deinit();
    }

    FILE *f = std::fopen(argv[5], "wb");
    if (!f) return 3;
    const uint32_t nspec = (uint32_t)prec.size(), npeaks = (uint32_t)moz.size();
    std::fwrite(&status, 4, 1, f);
    std::fwrite(&nspec, 4, 1, f);
    std::fwrite(&npeaks, 4, 1, f);
    std::fwrite(idx.data(), 4, idx.size(), f);
    std::fwrite(moz.data(), 4, moz.size(), f);
    std::fwrite(inten.data(), 4, inten.size(), f);
    std::fwrite(prec.data(), 4, prec.size(), f);
    std::fwrite(z.data(), 4, z.size(), f);
    std::fwrite(rt.data(), 4, rt.size(), f);
    std::fclose(f);
    return 0;
}
