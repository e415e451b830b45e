/*
 * Link-time shims for building the reference HiCOPS DSLIM path as a CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY. This file is compiled together with the
 * unmodified reference translation units (dslim.cpp, dslim_query.cpp,
 * expeRT.cpp, utils.cpp, lbe_internal.cpp, mods.cpp, ...) by
 * oracle/ref/Makefile into oracle/_ref/. Nothing in the product links it.
 *
 * What it provides, and why:
 *  - the global `gParams params` and `queryfiles` that the reference defines in
 *    source/app/hicops.cpp (that TU is not built: it includes an empty
 *    submodule, source/app/hicops.hpp:24);
 *  - no-op bodies for the MS2 reader (source/core/msquery.cpp and
 *    source/core/ms2prep.cpp need MPI). Queries are fed as in-memory CSR
 *    batches, so the reader is never called;
 *  - DFile_* (source/core/include/dslim_fileout.h:27-31) replaced by a
 *    recorder: DFile_PrintScore is called from OpenMP workers once per
 *    reported spectrum (source/core/dslim_query.cpp:815) *before*
 *    res.reset() (:821), so the worker's Results (histogram, mu, beta) are
 *    still readable here.
 */
#include "dslim.h"
#include "dslim_fileout.h"
#include "msquery.hpp"
#include "ms2prep.hpp"
#include "ref_record.h"

gParams params;
std::vector<string_t> queryfiles;

extern BYICount *Score;

ref_record_t *g_records = nullptr;
int g_nrecords = 0;

/* ---- MS2 reader stubs (never reached with in-memory batches) ---- */
MSQuery::MSQuery() : currPtr(0), running_count(0), curr_chunk(0), qfile(nullptr),
                     qfileIndex(0), m_isinit(false) {}
MSQuery::~MSQuery() {}
uint_t MSQuery::getQAcount() { return 0; }
status_t MSQuery::extractbatch(uint_t, Queries *, int_t &) { return SLM_SUCCESS; }
status_t MSQuery::DeinitQueryFile() { return SLM_SUCCESS; }
BOOL MSQuery::isDeInit() { return true; }
uint_t MSQuery::getQfileIndex() { return 0; }
uint_t &MSQuery::Curr_chunk() { return curr_chunk; }

namespace hcp { namespace ms2 {
status_t initialize(lwqueue<MSQuery *> **, int_t &, int_t &) { return SLM_SUCCESS; }
void deinitialize() {}
} }

/* ---- result recorder in place of the TSV writer ---- */
status_t DFile_InitFiles() { return SLM_SUCCESS; }
status_t DFile_DeinitFiles() { return SLM_SUCCESS; }
status_t DFile_PrintPartials(uint_t, Results *) { return SLM_SUCCESS; }

status_t DFile_PrintScore(Index *index, uint_t specid, float_t pmass, hCell *psm,
                          double_t e_x, uint_t npsms)
{
    (void)pmass;
    if (g_records == nullptr || (int)specid >= g_nrecords)
        return SLM_SUCCESS;

    const int thno = omp_get_thread_num();
    const Results &res = Score[thno].res;
    const Index &li = index[psm->idxoffset];
    const pepEntry &pe = li.pepEntries[psm->psid];

    ref_record_t &r = g_records[specid];
    r.reported = 1;
    r.psid = psm->psid;
    r.idxoffset = psm->idxoffset;
    r.sharedions = psm->sharedions;
    r.totalions = psm->totalions;
    r.hyperscore = psm->hyperscore;
    r.e_x = e_x;
    r.npsms = (int)npsms;
    r.mu = res.mu;
    r.beta = res.beta;
    r.minhyp = res.minhypscore;
    r.nexthyp = res.nexthypscore;
    r.maxhyp = res.maxhypscore;
    r.seqid = pe.seqID;
    r.modnum = pe.sites.modNum;
    r.sites = pe.sites.sites;
    r.pepmass = pe.Mass;
    for (int b = 0; b < REF_HIST_BINS; b++)
        r.hist[b] = (unsigned)res.survival[b];
    return SLM_SUCCESS;
}
