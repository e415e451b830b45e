// hicops_dslim_shim.cpp — the binding a maintainer compiles into the HiCOPS
// reference in place of the DSLIM bodies (source/core/dslim.cpp and
// dslim_query.cpp): the reference's own function names and types
// (source/core/include/dslim.h:49, 53, 184), forwarding to the C ABI of
// include/hicops_gb300.h. Compile against the reference's headers
// (source/core/include plus its generated config.hpp / common.hpp) and link
// with -lhicops_gb300. DFile_PrintScore (dslim_fileout.h:29) and the global
// gParams `params` are the reference's own; this file only calls them.
#include <cstddef>
#include <cstring>
#include <vector>

#include "dslim.h"
#include "dslim_fileout.h"
#include "hicops_gb300.h"

extern gParams params;

// pepEntry (slm_dsts.h:146-282: float, uint, then modAA {ull sites; uint
// modNum}) and hc_entry share one 24-byte layout, so the reference's sorted
// entries pass through without a copy.
#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Winvalid-offsetof"
static_assert(sizeof(pepEntry) == sizeof(hc_entry), "pepEntry and hc_entry differ in size");
static_assert(offsetof(pepEntry, Mass) == offsetof(hc_entry, mass), "pepEntry::Mass");
static_assert(offsetof(pepEntry, seqID) == offsetof(hc_entry, seqid), "pepEntry::seqID");
static_assert(offsetof(pepEntry, sites) + offsetof(modAA, sites) == offsetof(hc_entry, sites), "modAA::sites");
static_assert(offsetof(pepEntry, sites) + offsetof(modAA, modNum) == offsetof(hc_entry, modnum), "modAA::modNum");
#pragma GCC diagnostic pop
static_assert(sizeof(((Queries *)0)->idx[0]) == sizeof(uint32_t), "Queries::idx");
static_assert(sizeof(((Queries *)0)->moz[0]) == sizeof(uint32_t), "Queries::moz");
static_assert(sizeof(((Queries *)0)->intensity[0]) == sizeof(uint32_t), "Queries::intensity");
static_assert(sizeof(((Queries *)0)->precurse[0]) == sizeof(float), "Queries::precurse");
static_assert(sizeof(((SLM_varAA *)0)->residues) == sizeof(((hc_params *)0)->mod_res[0]), "SLM_varAA::residues");

static hc_ctx *g_ctx = nullptr;
static int_t g_spectrum_id = 0;  // the reference's spectrumID (dslim_query.cpp:53, 828)

// gParams (slm_dsts.h:359-418) -> hc_params
static hc_params to_hc(const gParams &p)
{
    hc_params h;
    std::memset(&h, 0, sizeof(h));
    h.min_len = p.min_len;
    h.max_len = p.max_len;
    h.maxz = p.maxz;
    h.topmatches = p.topmatches;
    h.scale = p.scale;
    h.min_shp = p.min_shp;
    h.min_cpsm = p.min_cpsm;
    h.min_mass = p.min_mass;
    h.max_mass = p.max_mass;
    h.dF = p.dF;
    h.base_int = p.base_int;
    h.min_int = p.min_int;
    h.dM = p.dM;
    h.expect_max = p.expect_max;
    h.nmods = p.vModInfo.num_vars;
    h.vmods_per_pep = p.vModInfo.vmods_per_pep;
    for (uint32_t m = 0; m < h.nmods && m < HC_MAX_MODS; m++)
    {
        h.mod_mass[m] = p.vModInfo.vmods[m].modMass;
        std::memcpy(h.mod_res[m], p.vModInfo.vmods[m].residues, sizeof(h.mod_res[m]));
        h.mod_per_pep[m] = p.vModInfo.vmods[m].aa_per_peptide;
    }
    h.threads = p.threads;
    return h;
}

static status_t ensure_ctx()
{
    if (g_ctx) return SLM_SUCCESS;
    const hc_params h = to_hc(params);
    return hc_ctx_create(0, &h, &g_ctx);
}

// dslim.h:49 — one peptide length's index, in the entry order LBE_Initialize
// sorted (lbe_internal.cpp:184-187), built on the device.
status_t DSLIM_Construct(Index *index)
{
    if (!index) return ERR_INVLD_PTR;
    status_t st = ensure_ctx();
    if (st != SLM_SUCCESS) return st;
    return hc_dslim_construct(g_ctx, index->pepIndex.peplen, reinterpret_cast<const uint8_t *>(index->pepIndex.seqs),
                              index->lclpepCnt, reinterpret_cast<const hc_entry *>(index->pepEntries),
                              index->lcltotCnt);
}

// dslim.h:53 — the scorecards, heaps and histograms are device scratch of the context
status_t DSLIM_InitializeScorecard(Index *, uint_t) { return ensure_ctx(); }

// dslim.h:184 — one batch; DFile_PrintScore is called for every spectrum the
// reference would print (cpsms >= min_cpsm and e(x) < expect_max,
// dslim_query.cpp:773-816), from this thread, in spectrum order.
status_t DSLIM_QuerySpectrum(Queries *ss, Index *index, uint_t)
{
    if (!ss || !index || !g_ctx) return ERR_INVLD_PTR;
    const uint32_t n = ss->numSpecs > 0 ? (uint32_t)ss->numSpecs : 0u;
    std::vector<hc_result> out(n);
    status_t st = hc_dslim_query(g_ctx, ss->idx, ss->moz, ss->intensity, ss->precurse, nullptr, n, out.data(),
                                 nullptr);
    if (st != SLM_SUCCESS) return st;
    for (uint32_t q = 0; q < n && st == SLM_SUCCESS; q++)
    {
        const hc_result &r = out[q];
        if (!r.reported) continue;
        hCell psm;
        psm.idxoffset = (ushort_t)r.idxoffset;
        psm.psid = r.psid;
        psm.sharedions = r.sharedions;
        psm.totalions = r.totalions;
        psm.hyperscore = r.hyperscore;
        psm.pmass = ss->precurse[q];
        psm.pchg = ss->charges ? ss->charges[q] : 0;
        psm.rtime = ss->rtimes ? ss->rtimes[q] : 0.0f;
        psm.fileIndex = (ushort_t)ss->fileNum;
        st = DFile_PrintScore(index, g_spectrum_id + q, ss->precurse[q], &psm, r.evalue, r.cpsms);
    }
    g_spectrum_id += (int_t)n;
    return st;
}

// dslim.cpp:657-691 (DSLIM_DeallocateIonIndex and the rest of DSLIM_Deinitialize)
status_t DSLIM_Deinitialize()
{
    if (g_ctx) hc_ctx_destroy(g_ctx);
    g_ctx = nullptr;
    return SLM_SUCCESS;
}
