/*
 * Driver that runs the unmodified reference DSLIM index build and query
 * (TEST INFRASTRUCTURE: produces golden vectors; never part of the product).
 *
 * Sequence follows the reference's own driver, source/app/hicops.cpp:184-308:
 *   UTILS_InitializeModInfo, MODS_Initialize, then per peptide length
 *   LBE_CountPeps -> LBE_CreatePartitions -> LBE_Initialize -> LBE_Distribute
 *   -> DSLIM_Construct; then DSLIM_DeallocateSpecArr and
 *   DSLIM_InitializeScorecard; then DSLIM_QuerySpectrum per batch of at most
 *   QCHUNK spectra (source/core/dslim_query.cpp:311-381 does the batching).
 *
 * usage: ref_driver <params.txt> <dbdir> <queries.bin> <outdir> [--dump-index]
 *
 * params.txt holds "key value" lines for the gParams fields
 * (source/core/include/slm_dsts.h:359-418) plus "mod <residues> <mass> <per_pep>".
 * queries.bin: u32 nspec, u32 npeaks, u32 idx[nspec+1], u32 moz[npeaks],
 *              u32 intensity[npeaks], f32 precurse[nspec], i32 charge[nspec],
 *              f32 rtime[nspec].
 */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "dslim.h"
#include "lbe.h"
#include "mods.h"
#include "scheduler.h"
#include "expeRT.h"
#include "ref_record.h"

extern gParams params;
extern Scheduler *SchedHandle;
extern expeRT *ePtrs;
extern ref_record_t *g_records;
extern int g_nrecords;

static std::vector<char> slurp(const std::string &path)
{
    std::ifstream f(path, std::ios::binary);
    return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

template <class T>
static void dump(const std::string &path, const T *p, size_t n)
{
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { perror(path.c_str()); exit(3); }
    fwrite(p, sizeof(T), n, f);
    fclose(f);
}

int main(int argc, char **argv)
{
    if (argc < 5)
    {
        fprintf(stderr, "usage: %s params.txt dbdir queries.bin outdir [--dump-index]\n", argv[0]);
        return 2;
    }
    const std::string dbdir = argv[2], outdir = argv[4];
    const bool dump_index = (argc > 5 && std::string(argv[5]) == "--dump-index");

    /* ---- params ---- */
    std::ifstream pf(argv[1]);
    std::string line;
    int nmods = 0;
    while (std::getline(pf, line))
    {
        std::istringstream ss(line);
        std::string k;
        ss >> k;
        if (k == "threads") ss >> params.threads;
        else if (k == "min_len") ss >> params.min_len;
        else if (k == "max_len") ss >> params.max_len;
        else if (k == "maxz") ss >> params.maxz;
        else if (k == "topmatches") ss >> params.topmatches;
        else if (k == "scale") ss >> params.scale;
        else if (k == "min_shp") ss >> params.min_shp;
        else if (k == "min_cpsm") ss >> params.min_cpsm;
        else if (k == "spadmem") ss >> params.spadmem;
        else if (k == "min_mass") ss >> params.min_mass;
        else if (k == "max_mass") ss >> params.max_mass;
        else if (k == "dF") ss >> params.dF;
        else if (k == "base_int") ss >> params.base_int;
        else if (k == "min_int") ss >> params.min_int;
        else if (k == "dM") ss >> params.dM;
        else if (k == "res") ss >> params.res;
        else if (k == "expect_max") ss >> params.expect_max;
        else if (k == "vmods_per_pep") ss >> params.vModInfo.vmods_per_pep;
        else if (k == "mod")
        {
            std::string res;
            double mass;
            int per;
            ss >> res >> mass >> per;
            SLM_varAA &v = params.vModInfo.vmods[nmods];
            for (size_t i = 0; i < 4; i++) v.residues[i] = i < res.size() ? res[i] : '\0';
            /* same conversion as source/app/hicops.cpp:661 */
            v.modMass = (uint_t)(mass * params.scale);
            v.aa_per_peptide = per;
            nmods++;
        }
    }
    params.vModInfo.num_vars = nmods;
    params.nodes = 1;
    params.myid = 0;
    params.maxprepthds = 1;
    if (nmods == 0)
        params.modconditions = "0 M 0";
    else
    {
        /* string built as in source/app/hicops.cpp:631-664 */
        params.modconditions = std::to_string(params.vModInfo.vmods_per_pep);
        for (int m = 0; m < nmods; m++)
        {
            params.modconditions += " " + std::string(params.vModInfo.vmods[m].residues,
                                                      strnlen(params.vModInfo.vmods[m].residues, 4));
            params.modconditions += " " + std::to_string(params.vModInfo.vmods[m].aa_per_peptide);
        }
    }

    /* ---- index ---- */
    const uint_t nlen = params.max_len - params.min_len + 1;
    Index *idx = new Index[nlen];
    status_t st = UTILS_InitializeModInfo(&params.vModInfo);
    if (st == SLM_SUCCESS) st = MODS_Initialize();

    auto t0 = std::chrono::steady_clock::now();
    double t_construct = 0;
    for (uint_t L = params.min_len; L <= params.max_len && st == SLM_SUCCESS; L++)
    {
        Index *ix = idx + (L - params.min_len);
        ix->pepIndex.peplen = L;
        std::string f = dbdir + "/" + std::to_string(L) + ".peps";
        st = LBE_CountPeps((char_t *)f.c_str(), ix, L);
        if (st == SLM_SUCCESS) st = LBE_CreatePartitions(ix);
        if (st == SLM_SUCCESS) st = LBE_Initialize(ix);
        if (st == SLM_SUCCESS) st = LBE_Distribute(ix);
        if (st == SLM_SUCCESS)
        {
            if (ix->nChunks != 1)
            {
                fprintf(stderr, "length %u: nChunks=%u (raise spadmem)\n", L, ix->nChunks);
                return 4;
            }
            auto c0 = std::chrono::steady_clock::now();
            st = DSLIM_Construct(ix);
            t_construct += std::chrono::duration<double>(std::chrono::steady_clock::now() - c0).count();
        }
        if (st != SLM_SUCCESS)
        {
            fprintf(stderr, "index build failed at length %u: %d\n", L, st);
            return 5;
        }
        /* entries in the reference's final (sorted) order */
        const uint_t n = ix->lcltotCnt;
        std::vector<float> mass(n);
        std::vector<uint32_t> seqid(n), modnum(n);
        std::vector<uint64_t> sites(n);
        for (uint_t i = 0; i < n; i++)
        {
            mass[i] = ix->pepEntries[i].Mass;
            seqid[i] = ix->pepEntries[i].seqID;
            modnum[i] = ix->pepEntries[i].sites.modNum;
            sites[i] = ix->pepEntries[i].sites.sites;
        }
        const std::string p = outdir + "/len" + std::to_string(L);
        uint32_t counts[2] = {n, ix->pepCount};
        dump(p + "_count.bin", counts, 2);
        dump(p + "_mass.bin", mass.data(), n);
        dump(p + "_seqid.bin", seqid.data(), n);
        dump(p + "_modnum.bin", modnum.data(), n);
        dump(p + "_sites.bin", sites.data(), n);
        if (dump_index)
        {
            const size_t speclen = (L - 1) * params.maxz * iSERIES;
            dump(p + "_bA.bin", ix->ionIndex[0].bA, (size_t)params.max_mass * params.scale + 1);
            dump(p + "_iA.bin", ix->ionIndex[0].iA, (size_t)n * speclen);
        }
    }
    DSLIM_DeallocateSpecArr();
    st = DSLIM_InitializeScorecard(idx, nlen);
    double t_index = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

    /* ---- queries ---- */
    std::vector<char> qb = slurp(argv[3]);
    const uint32_t *hdr = (const uint32_t *)qb.data();
    const uint32_t nspec = hdr[0], npk = hdr[1];
    const uint32_t *qidx = hdr + 2;
    const uint32_t *qmoz = qidx + nspec + 1;
    const uint32_t *qint = qmoz + npk;
    const float *qprec = (const float *)(qint + npk);
    const int32_t *qchg = (const int32_t *)(qprec + nspec);
    const float *qrt = (const float *)(qchg + nspec);

    std::vector<ref_record_t> recs(nspec);
    memset(recs.data(), 0, sizeof(ref_record_t) * nspec);
    g_records = recs.data();
    g_nrecords = (int)nspec;

    SchedHandle = new Scheduler(0);
    ePtrs = new expeRT[params.threads];

    Queries q;
    q.init();
    double t_query = 0;
    for (uint32_t s0 = 0; s0 < nspec && st == SLM_SUCCESS; s0 += QCHUNK)
    {
        const uint32_t n = std::min<uint32_t>(QCHUNK, nspec - s0);
        const uint32_t base = qidx[s0];
        for (uint32_t i = 0; i <= n; i++) q.idx[i] = qidx[s0 + i] - base;
        const uint32_t np = qidx[s0 + n] - base;
        memcpy(q.moz, qmoz + base, np * 4);
        memcpy(q.intensity, qint + base, np * 4);
        memcpy(q.precurse, qprec + s0, n * 4);
        memcpy(q.charges, qchg + s0, n * 4);
        memcpy(q.rtimes, qrt + s0, n * 4);
        q.numSpecs = n;
        q.numPeaks = np;
        q.batchNum = s0 / QCHUNK;
        auto c0 = std::chrono::steady_clock::now();
        st = DSLIM_QuerySpectrum(&q, idx, nlen);
        t_query += std::chrono::duration<double>(std::chrono::steady_clock::now() - c0).count();
    }
    if (st != SLM_SUCCESS)
    {
        fprintf(stderr, "query failed: %d\n", st);
        return 6;
    }
    dump(outdir + "/results.bin", recs.data(), nspec);
    FILE *tf = fopen((outdir + "/timing.txt").c_str(), "w");
    fprintf(tf, "threads %u\nindex_s %.6f\nconstruct_s %.6f\nquery_s %.6f\nnspec %u\n",
            params.threads, t_index, t_construct, t_query, nspec);
    fclose(tf);
    return 0;
}
